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
using BcStartFn = cudaError_t (*)(const FieldP& f, double flres, int64_t n, const double* st, const double* cst,
                                  double delta, double bctimestep, double* plan, int32_t* status, int32_t* flag,
                                  double* scratch, long long stride, int cap, cudaStream_t s);
using BcIntervalFn = cudaError_t (*)(const FieldP& f, const KParams& P, int64_t n, double* st, const double* cst,
                                     const double* plan, double d, int64_t j, double* rows, int max_rows,
                                     int32_t* nrows, int32_t* status, int64_t* counters, int32_t* flag,
                                     double* scratch, long long stride, int cap, cudaStream_t s);
using BcEvalFn = cudaError_t (*)(const FieldP& f, double flres, int what, int64_t n, const double* tpos,
                                 const double* Bm, double d, const double* cst, double* out, double* scratch,
                                 long long stride, int cap, cudaStream_t s);
using BounceFn = cudaError_t (*)(const FieldP& f, double flres, int64_t n, const double* in, double* out,
                                 double* scratch, long long stride, int cap, cudaStream_t s);

struct ModelTable {
  LaunchFn particle[2];  // [tableau]
  LaunchFn gc[2];
  OccFn occ_particle[2];
  OccFn occ_gc[2];
  LaunchFn particle32, gc32;  // FP32-stage form (DOP853 / DOPRI5)
  OccFn occ_particle32, occ_gc32;
  // guiding-centre DOPRI5 kernels with the step learner: [0] plain, [1] sample
  // collection, [2] MLP proposals; FP64 and FP32-stage forms
  LaunchFn gc_lrn[3], gc32_lrn[3];
  OccFn occ_gc_lrn[3], occ_gc32_lrn[3];
  FieldEvalFn field_eval;
  RhsEvalFn rhs_eval;
  AdaptiveInitFn adaptive_init;
  BounceFn bounce_period;
  LaunchFn gc_dense;  // DOPRI5 guiding centres with dense output (rapt_config.dense_output)
  OccFn occ_gc_dense;
  BcStartFn bc_start;        // BounceCenter.advance: cadence and row count
  BcIntervalFn bc_interval;  // BounceCenter.advance: one output interval of every tracer
  BcEvalFn bc_eval;          // second invariant, its gradient, the bounce-averaged drift
};

// MLP kernels (mlp.cu); packed BF16 weights take kMlpPackedWords u32
constexpr int kMlpPackedWords = 64 * 8 + 64 * 32 + 8 * 32 + 64 * 32 + 64 * 4 + 8 * 32 * 2 + 8 * 32 * 8 + 32 * 8 +
                                 32 * 16 + 32 * 16 + 32 * 2;
cudaError_t mlp_pack(const float* p, uint32_t* w, cudaStream_t s);
// training gradient: at most kMlpTrainMaxBlocks blocks, each writing a partial
// gradient of kMlpGaccWords floats and two loss doubles to the workspaces
constexpr int kMlpTrainMaxBlocks = 1024;
constexpr int kMlpGaccWords = (RAPT_MLP_NTRAIN + 31) / 32 * 32;
cudaError_t mlp_grad(const float* samples, int64_t nsamp, int64_t batch, int random, uint64_t seed, int64_t step,
                     float switch_weight, const uint32_t* w, const float* p, float* grad, double* loss, float* partial,
                     double* lpart, cudaStream_t s);
// canonical order of n samples (a 64-bit hash of each sample's words, sorted):
// the kernels append samples in an order set by atomics; after this the order
// depends only on the set of samples. tmp: mlp_sort_tmp_bytes(n) bytes.
size_t mlp_sort_tmp_bytes(int64_t n);
cudaError_t mlp_samples_sort(float* samples, int64_t n, void* tmp, size_t tmp_bytes, cudaStream_t s);
cudaError_t mlp_adam(float* p, float* m, float* v, const float* g, float lr, int64_t t, cudaStream_t s);
cudaError_t mlp_forward(const uint32_t* w, const float* p, const float* feat, int64_t n, float* out, int num_sms,
                        cudaStream_t s);

void register_model_0(ModelTable*);
void register_model_1(ModelTable*);
void register_model_2(ModelTable*);
void register_model_3(ModelTable*);
void register_model_4(ModelTable*);
void register_model_5(ModelTable*);
void register_model_6(ModelTable*);
void register_model_7(ModelTable*);
void register_model_8(ModelTable*);

}  // namespace rapt
