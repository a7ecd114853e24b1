// Interpreter simulation kernel, expect mode.
#define TFQG_SIM_MODE kModeExpect
#define TFQG_SIM_NAME expect
#include "sim_mode.cuh"
