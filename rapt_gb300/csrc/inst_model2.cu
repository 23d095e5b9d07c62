// Kernels for field model 2 (see inst_body.cuh).
#define RAPT_MODEL 2
#include "inst_body.cuh"
