// engine_pf.cu -- kernels instantiated for one potential kind (compiled
// separately so the build runs in parallel and each kernel is register-
// allocated for its own potential only).
#include "kernels.cuh"

MG_DEFINE_LAUNCHERS(mg::K_PF, pf)
