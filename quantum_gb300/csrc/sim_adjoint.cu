// Interpreter simulation kernel, adjoint mode.
#define TFQG_SIM_MODE kModeAdjoint
#define TFQG_SIM_NAME adjoint
#include "sim_mode.cuh"
