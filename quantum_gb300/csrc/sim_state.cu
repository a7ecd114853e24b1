// Interpreter simulation kernel, state mode.
#define TFQG_SIM_MODE kModeState
#define TFQG_SIM_NAME state
#include "sim_mode.cuh"
