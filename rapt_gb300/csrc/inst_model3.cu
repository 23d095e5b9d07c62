// Kernels for field model 3 (see inst_body.cuh).
#define RAPT_MODEL 3
#include "inst_body.cuh"
