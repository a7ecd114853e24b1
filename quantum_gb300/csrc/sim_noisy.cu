// Interpreter simulation kernel, noisy mode.
#define TFQG_SIM_MODE kModeNoisy
#define TFQG_SIM_NAME noisy
#include "sim_mode.cuh"
