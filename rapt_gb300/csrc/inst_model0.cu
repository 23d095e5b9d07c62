// Kernels for field model 0 (see inst_body.cuh).
#define RAPT_MODEL 0
#include "inst_body.cuh"
