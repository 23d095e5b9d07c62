// Kernels for field model 5 (see inst_body.cuh).
#define RAPT_MODEL 5
#include "inst_body.cuh"
