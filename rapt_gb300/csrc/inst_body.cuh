// inst_body.cuh -- instantiates every kernel for one field model. Included by
// inst_model<k>.cu with RAPT_MODEL defined, so the models compile in parallel.
#include "bc_kernels.cuh"
#include "dense_kernels.cuh"
#include "eval_kernels.cuh"
#include "fp32_kernels.cuh"
#include "launch.h"

#define RAPT_CAT2(a, b) a##b
#define RAPT_CAT(a, b) RAPT_CAT2(a, b)

namespace rapt {
namespace {
constexpr int kM = RAPT_MODEL;

template <int TAB>
cudaError_t launch_particle(const LaunchArgs& a) {
  k_particle<kM, TAB><<<a.grid, a.block, 0, a.stream>>>(a.E, a.P, a.S);
  return cudaGetLastError();
}
template <int TAB>
cudaError_t launch_gc(const LaunchArgs& a) {
  k_gc<kM, TAB><<<a.grid, a.block, 0, a.stream>>>(a.E, a.P, a.S);
  return cudaGetLastError();
}
template <int TAB>
int occ_particle(int block) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_particle<kM, TAB>, block, 0);
  return nb;
}
template <int TAB>
int occ_gc(int block) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gc<kM, TAB>, block, 0);
  return nb;
}
cudaError_t launch_gc_dense(const LaunchArgs& a) {
  k_gc_dense<kM><<<a.grid, a.block, 0, a.stream>>>(a.E, a.P, a.S);
  return cudaGetLastError();
}
int occ_gc_dense(int block) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gc_dense<kM>, block, 0);
  return nb;
}
cudaError_t launch_particle32(const LaunchArgs& a) {
  k_particle32<kM><<<a.grid, a.block, 0, a.stream>>>(a.E, a.P, a.S);
  return cudaGetLastError();
}
cudaError_t launch_gc32(const LaunchArgs& a) {
  k_gc32<kM><<<a.grid, a.block, 0, a.stream>>>(a.E, a.P, a.S);
  return cudaGetLastError();
}
int occ_particle32(int block) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_particle32<kM>, block, 0);
  return nb;
}
int occ_gc32(int block) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gc32<kM>, block, 0);
  return nb;
}
// guiding-centre kernels with the step learner; dynamic shared memory per warp
// (the occupancy is taken without collection; a collecting launch needs more
// shared memory per block, and its surplus blocks start as others finish)
template <int LRN>
size_t lrn_smem(int block, bool collect) {
  return (size_t)(block / 32) * StepLearner<LRN>::warp_words(collect) * sizeof(uint32_t);
}
template <int LRN>
cudaError_t launch_gc_lrn(const LaunchArgs& a) {
  k_gc<kM, 0, LRN><<<a.grid, a.block, lrn_smem<LRN>(a.block, a.P.collect != 0), a.stream>>>(a.E, a.P, a.S);
  return cudaGetLastError();
}
template <int LRN>
cudaError_t launch_gc32_lrn(const LaunchArgs& a) {
  k_gc32<kM, LRN><<<a.grid, a.block, lrn_smem<LRN>(a.block, a.P.collect != 0), a.stream>>>(a.E, a.P, a.S);
  return cudaGetLastError();
}
template <int LRN>
int occ_gc_lrn(int block) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gc<kM, 0, LRN>, block, lrn_smem<LRN>(block, false));
  return nb;
}
template <int LRN>
int occ_gc32_lrn(int block) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_gc32<kM, LRN>, block, lrn_smem<LRN>(block, false));
  return nb;
}
cudaError_t field_eval(const FieldP& f, int what, int64_t n, const double* tpos, double* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_field_eval<kM><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(f, what, n, tpos, out);
  return cudaGetLastError();
}
cudaError_t rhs_eval(const KParams& P, int mode, int64_t n, const double* state, const double* mass,
                     const double* charge, const double* v, double* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (P.form == RAPT_FORM_FP32 || P.form == RAPT_FORM_LEARNED_FP32)
    k_rhs_eval32<kM><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(P, mode, n, state, mass, charge, out);
  else
    k_rhs_eval<kM><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(P, mode, n, state, mass, charge, v, out);
  return cudaGetLastError();
}
cudaError_t bounce_period(const FieldP& f, double flres, int64_t n, const double* in, double* out, double* scratch,
                          long long stride, int cap, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_bounce_period<kM><<<(unsigned)((n + 63) / 64), 64, 0, s>>>(f, flres, n, in, out, scratch, stride, cap);
  return cudaGetLastError();
}
cudaError_t bc_start(const FieldP& f, double flres, int64_t n, const double* st, const double* cst, double delta,
                     double bctimestep, double* plan, int32_t* status, int32_t* flag, double* scratch,
                     long long stride, int cap, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_bc_start<kM><<<(unsigned)((n + 63) / 64), 64, 0, s>>>(f, flres, n, st, cst, delta, bctimestep, plan, status,
                                                          flag, scratch, stride, cap);
  return cudaGetLastError();
}
cudaError_t bc_interval(const FieldP& f, const KParams& P, int64_t n, double* st, const double* cst,
                        const double* plan, double d, int64_t j, double* rows, int max_rows, int32_t* nrows,
                        int32_t* status, int64_t* counters, int32_t* flag, double* scratch, long long stride,
                        int cap, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_bc_interval<kM><<<(unsigned)((n + 63) / 64), 64, 0, s>>>(f, P, n, st, cst, plan, d, j, rows, max_rows, nrows,
                                                             status, counters, flag, scratch, stride, cap);
  return cudaGetLastError();
}
cudaError_t bc_eval(const FieldP& f, double flres, int what, int64_t n, const double* tpos, const double* Bm,
                    double d, const double* cst, double* out, double* scratch, long long stride, int cap,
                    cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_bc_eval<kM><<<(unsigned)((n + 63) / 64), 64, 0, s>>>(f, flres, what, n, tpos, Bm, d, cst, out, scratch, stride,
                                                         cap);
  return cudaGetLastError();
}
cudaError_t adaptive_init(const DevEnsemble& E, const KParams& P, cudaStream_t s) {
  if (E.n <= 0) return cudaSuccess;
  k_adaptive_init<kM><<<(unsigned)((E.n + 127) / 128), 128, 0, s>>>(E, P);
  return cudaGetLastError();
}
}  // namespace

void RAPT_CAT(register_model_, RAPT_MODEL)(ModelTable* t) {
  t->particle[0] = launch_particle<0>;
  t->particle[1] = launch_particle<1>;
  t->gc[0] = launch_gc<0>;
  t->gc[1] = launch_gc<1>;
  t->occ_particle[0] = occ_particle<0>;
  t->occ_particle[1] = occ_particle<1>;
  t->occ_gc[0] = occ_gc<0>;
  t->occ_gc[1] = occ_gc<1>;
  t->particle32 = launch_particle32;
  t->gc32 = launch_gc32;
  t->occ_particle32 = occ_particle32;
  t->occ_gc32 = occ_gc32;
  t->gc_lrn[0] = launch_gc<0>;
  t->gc_lrn[1] = launch_gc_lrn<1>;
  t->gc_lrn[2] = launch_gc_lrn<2>;
  t->occ_gc_lrn[0] = occ_gc<0>;
  t->occ_gc_lrn[1] = occ_gc_lrn<1>;
  t->occ_gc_lrn[2] = occ_gc_lrn<2>;
  t->gc32_lrn[0] = launch_gc32;
  t->gc32_lrn[1] = launch_gc32_lrn<1>;
  t->gc32_lrn[2] = launch_gc32_lrn<2>;
  t->occ_gc32_lrn[0] = occ_gc32;
  t->occ_gc32_lrn[1] = occ_gc32_lrn<1>;
  t->occ_gc32_lrn[2] = occ_gc32_lrn<2>;
  t->field_eval = field_eval;
  t->rhs_eval = rhs_eval;
  t->adaptive_init = adaptive_init;
  t->bounce_period = bounce_period;
  t->gc_dense = launch_gc_dense;
  t->occ_gc_dense = occ_gc_dense;
  t->bc_start = bc_start;
  t->bc_interval = bc_interval;
  t->bc_eval = bc_eval;
}
}  // namespace rapt
