// engine_pf1.cu -- kernels for the binary PhaseField without optional terms
// (the lean variant of engine_pf.cu; register-allocated on its own).
#include "kernels.cuh"

MG_DEFINE_LAUNCHERS(mg::K_PF1, pf1)
