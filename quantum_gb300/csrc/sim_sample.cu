// Interpreter simulation kernel, sample mode.
#define TFQG_SIM_MODE kModeSample
#define TFQG_SIM_NAME sample
#include "sim_mode.cuh"
