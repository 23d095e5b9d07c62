// Kernels for field model 6 (see inst_body.cuh).
#define RAPT_MODEL 6
#include "inst_body.cuh"
