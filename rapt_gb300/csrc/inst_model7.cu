// Kernels for field model 7 (see inst_body.cuh).
#define RAPT_MODEL 7
#include "inst_body.cuh"
