// Kernels for field model 4 (see inst_body.cuh).
#define RAPT_MODEL 4
#include "inst_body.cuh"
