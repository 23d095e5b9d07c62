// Kernels for field model 8 (see inst_body.cuh).
#define RAPT_MODEL 8
#include "inst_body.cuh"
