// minim.h -- source-compatible front door of the GB300 engine: the State /
// Potential / Minimiser API of the minim library, with LjNd, PhaseField,
// PhaseFieldUnstructured and BarAndHinge evaluated and minimised on the GPU.
#ifndef MINIM_GB300_MINIM_H
#define MINIM_GB300_MINIM_H

#include "Communicator.h"
#include "Minimiser.h"
#include "Potential.h"
#include "State.h"
#include "minimisers/Anneal.h"
#include "minimisers/Fire.h"
#include "minimisers/GradDescent.h"
#include "minimisers/Lbfgs.h"
#include "potentials/BarAndHinge.h"
#include "potentials/LjNd.h"
#include "potentials/PhaseField.h"
#include "potentials/PhaseFieldUnstructured.h"
#include "utils/mpi.h"
#include "utils/print.h"
#include "utils/vec.h"

#endif
