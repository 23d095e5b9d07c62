// launch.h -- host-side table of per-model kernel launchers.
#pragma once
#include <cuda_runtime.h>
#include "common.cuh"

namespace rapt {

struct LaunchArgs {
  DevEnsemble E;
  KParams P;
  Scratch* S;
  int grid, block;
  cudaStream_t stream;
};

using LaunchFn = cudaError_t (*)(const LaunchArgs&);
using OccFn = int (*)(int block);
using FieldEvalFn = cudaError_t (*)(const FieldP& f, int what, int64_t n, const double* tpos, double* out,
                                    cudaStream_t s);
using RhsEvalFn = cudaError_t (*)(const KParams& P, int mode, int64_t n, const double* state, const double* mass,
                                  const double* charge, const double* v, double* out, cudaStream_t s);
using AdaptiveInitFn = cudaError_t (*)(const DevEnsemble& E, const KParams& P, cudaStream_t s);

struct ModelTable {
  LaunchFn particle[2];  // [tableau]
  LaunchFn gc[2];
  OccFn occ_particle[2];
  OccFn occ_gc[2];
  LaunchFn particle32, gc32;  // FP32-stage form (DOP853 / DOPRI5)
  OccFn occ_particle32, occ_gc32;
  FieldEvalFn field_eval;
  RhsEvalFn rhs_eval;
  AdaptiveInitFn adaptive_init;
};

void register_model_0(ModelTable*);
void register_model_1(ModelTable*);
void register_model_2(ModelTable*);
void register_model_3(ModelTable*);
void register_model_4(ModelTable*);
void register_model_5(ModelTable*);
void register_model_6(ModelTable*);
void register_model_7(ModelTable*);

}  // namespace rapt
