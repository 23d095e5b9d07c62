// Kernels for field model 1 (see inst_body.cuh).
#define RAPT_MODEL 1
#include "inst_body.cuh"
