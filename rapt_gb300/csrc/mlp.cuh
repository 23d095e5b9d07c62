// mlp.cuh -- the step-size / switch MLP: 16 (14 used) -> 64 -> 64 -> 2, ReLU,
// BF16 weights and activations, FP32 accumulation on the tensor cores
// (mma.sync.m16n8k16.bf16; one warp handles 32 samples at a time).
//
// Fragment layouts of mma.m16n8k16 (PTX ISA), g = lane / 4, q = lane % 4:
//   A (16x16, row): a0 = A[g][2q..2q+1], a1 = A[g+8][2q..], a2 = A[g][2q+8..], a3 = A[g+8][2q+8..]
//   B (16x8, col):  b0 = B[2q..2q+1][g], b1 = B[2q+8..2q+9][g]
//   C (16x8):       c0,c1 = C[g][2q..2q+1], c2,c3 = C[g+8][2q..2q+1]
// Activations go through shared memory as BF16 so that few registers stay
// live inside the tracer kernels that call the network once per RK step.
//
// Output 0 is the log correction of the plain controller's next step size,
// output 1 the logit of "the next adiabaticity check fails" (Adaptive switch).
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "common.cuh"

namespace rapt {

constexpr int kMlpIn = 16;
constexpr int kSampleStride = 18;  // 16 features, step target, switch label (-1: none)
// FP32 parameter vector (offsets in floats); W?T are [out][in]
constexpr int kOffW1 = 0;                      // W1T [64][16]
constexpr int kOffB1 = kOffW1 + 64 * 16;
constexpr int kOffW2 = kOffB1 + 64;            // W2T [64][64]
constexpr int kOffB2 = kOffW2 + 64 * 64;
constexpr int kOffW3 = kOffB2 + 64;            // W3T [8][64], rows 2..7 stay zero
constexpr int kOffB3 = kOffW3 + 8 * 64;
constexpr int kMlpTrainable = kOffB3 + 8;      // 5768 weights and biases
constexpr int kOffXmu = kMlpTrainable;         // feature mean [16]
constexpr int kOffXsig = kOffXmu + 16;         // feature scale [16]
constexpr int kOffYmu = kOffXsig + 16;         // target mean [8]
constexpr int kOffYsig = kOffYmu + 8;          // target scale [8]
constexpr int kMlpParams = kOffYsig + 8;       // 5816 floats
static_assert(kMlpParams == RAPT_MLP_NPARAMS && kMlpTrainable == RAPT_MLP_NTRAIN, "MLP layout");
// packed BF16 weights (one u32 = two bf16), offsets in u32
constexpr int kPW1 = 0;                        // W1T [64][8]
constexpr int kPW2 = kPW1 + 64 * 8;            // W2T [64][32]
constexpr int kPW3 = kPW2 + 64 * 32;           // W3T [8][32]
constexpr int kPW2N = kPW3 + 8 * 32;           // W2  [64 in][32]: B operand of the backward pass
constexpr int kPW3N = kPW2N + 64 * 32;         // W3  [64 in][4]
// inference fragments: each lane's mma B fragments and bias pairs stored
// contiguously, so that one call loads them with a few vector loads
constexpr int kPF1 = kPW3N + 64 * 4;           // W1: [8 n-tiles][32 lanes][2]
constexpr int kPF2 = kPF1 + 8 * 32 * 2;        // W2: [8 n-tiles][32 lanes][8] (4 k-steps x 2)
constexpr int kPF3 = kPF2 + 8 * 32 * 8;        // W3: [32 lanes][8] (4 k-steps x 2)
constexpr int kPB1 = kPF3 + 32 * 8;            // b1: [32 lanes][16] (8 n-tiles x 2), float bits
constexpr int kPB2 = kPB1 + 32 * 16;           // b2: [32 lanes][16]
constexpr int kPB3 = kPB2 + 32 * 16;           // b3: [32 lanes][2]
constexpr int kMlpPacked = kPB3 + 32 * 2;

extern __shared__ __align__(16) uint32_t rapt_dyn_smem[];

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ float bf16_lo(uint32_t u) { return __uint_as_float(u << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t u) { return __uint_as_float(u & 0xffff0000u); }

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment (m-tile t, k-step s) of a row-major BF16 matrix stored as u32 [rows][K2].
__device__ __forceinline__ void load_a(const uint32_t* M, int K2, int t, int s, int g, int q, uint32_t* a) {
  const int r0 = 16 * t + g, r1 = r0 + 8, c = 8 * s + q;
  a[0] = M[r0 * K2 + c];
  a[1] = M[r1 * K2 + c];
  a[2] = M[r0 * K2 + c + 4];
  a[3] = M[r1 * K2 + c + 4];
}
// B fragment (n-tile j, k-step s) of a K x N matrix stored column-major, u32 [N][K2].
__device__ __forceinline__ void load_b(const uint32_t* BT, int K2, int j, int s, int g, int q, uint32_t* b) {
  const int r = 8 * j + g, c = 8 * s + q;
  b[0] = BT[r * K2 + c];
  b[1] = BT[r * K2 + c + 4];
}

// Dense layer out = ReLU(in @ W + b) for 32 rows: in u32 [32][K/2], W as W^T
// u32 [N][K/2]; writes BF16 out u32 [32][N/2].
template <int K, int N>
__device__ __forceinline__ void dense_relu(const uint32_t* in, const uint32_t* WT, const float* bias, uint32_t* out,
                                           int g, int q) {
#pragma unroll
  for (int j = 0; j < N / 8; ++j) {
    float c[2][4];
    const float b0 = bias[8 * j + 2 * q], b1 = bias[8 * j + 2 * q + 1];
#pragma unroll
    for (int t = 0; t < 2; ++t) { c[t][0] = c[t][2] = b0; c[t][1] = c[t][3] = b1; }
#pragma unroll
    for (int s = 0; s < K / 16; ++s) {
      uint32_t b[2];
      load_b(WT, K / 2, j, s, g, q, b);
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        uint32_t a[4];
        load_a(in, K / 2, t, s, g, q, a);
        mma_bf16(c[t], a, b);
      }
    }
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      out[(16 * t + g) * (N / 2) + 4 * j + q] = pack_bf16x2(fmaxf(c[t][0], 0.f), fmaxf(c[t][1], 0.f));
      out[(16 * t + g + 8) * (N / 2) + 4 * j + q] = pack_bf16x2(fmaxf(c[t][2], 0.f), fmaxf(c[t][3], 0.f));
    }
  }
}

// Output layer (8 columns, two used): this lane's sample's two outputs (network units).
__device__ __forceinline__ void dense_out(const uint32_t* in, const uint32_t* WT, const float* bias, int g, int q,
                                          int lane, float* y) {
  float c[2][4];
  const float b0 = bias[2 * q], b1 = bias[2 * q + 1];
#pragma unroll
  for (int t = 0; t < 2; ++t) { c[t][0] = c[t][2] = b0; c[t][1] = c[t][3] = b1; }
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    uint32_t b[2];
    load_b(WT, 32, 0, s, g, q, b);
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      uint32_t a[4];
      load_a(in, 32, t, s, g, q, a);
      mma_bf16(c[t], a, b);
    }
  }
  // sample 16 t + rr sits on lane 4 (rr % 8), columns 0..1, in c[t][0..1] (rr < 8) or c[t][2..3]
  const int rr = lane & 15, src = 4 * (rr & 7);
  float v[2][4];
#pragma unroll
  for (int tt = 0; tt < 2; ++tt)
#pragma unroll
    for (int i = 0; i < 4; ++i) v[tt][i] = __shfl_sync(kFull, c[tt][i], src);
  const bool hi_t = lane >= 16, hi_r = rr >= 8;
  y[0] = hi_t ? (hi_r ? v[1][2] : v[1][0]) : (hi_r ? v[0][2] : v[0][0]);
  y[1] = hi_t ? (hi_r ? v[1][3] : v[1][1]) : (hi_r ? v[0][3] : v[0][1]);
}

// One normalised feature, (v - mu) / sig, with the approximate FP32 quotient
// (__fdividef, 2 ulp): features enter the network in BF16 (8 bits), and
// training and inference normalise with this same function.
__device__ __forceinline__ float norm_feature(float v, float mu, float sig) { return __fdividef(v - mu, sig); }

// Normalise 16 raw features and write them as BF16 row `lane` of X (u32 [32][8]).
__device__ __forceinline__ void stage_features(const float* p, const float* f, uint32_t* X, int lane) {
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float a = norm_feature(f[2 * i], p[kOffXmu + 2 * i], p[kOffXsig + 2 * i]);
    const float b = norm_feature(f[2 * i + 1], p[kOffXmu + 2 * i + 1], p[kOffXsig + 2 * i + 1]);
    X[lane * 8 + i] = pack_bf16x2(a, b);
  }
}

// Two ReLU-layer C fragments (n-tiles 2s, 2s+1 of a 16-row tile) packed as the
// BF16 A fragment of the next layer's k-step s: a0 = tile 2s rows g, a1 = tile
// 2s rows g+8, a2/a3 = tile 2s+1 (the C and A layouts of m16n8k16 line up).
__device__ __forceinline__ void relu_pack_a(const float* c0, const float* c1, uint32_t* a) {
  a[0] = pack_bf16x2(fmaxf(c0[0], 0.f), fmaxf(c0[1], 0.f));
  a[1] = pack_bf16x2(fmaxf(c0[2], 0.f), fmaxf(c0[3], 0.f));
  a[2] = pack_bf16x2(fmaxf(c1[0], 0.f), fmaxf(c1[1], 0.f));
  a[3] = pack_bf16x2(fmaxf(c1[2], 0.f), fmaxf(c1[3], 0.f));
}

// Per-warp shared memory of inference (u32): the staged inputs X [32][8].
constexpr int kWarpSmemInfer = 32 * 8;

// Whole-warp inference on the staged X rows, one 16-row tile at a time, with
// the hidden activations kept in registers as A fragments (H1) or consumed
// as soon as a pair of n-tiles is complete (H2); the BF16 roundings are those
// of storing H1 and H2. Weights and biases come from the per-lane fragment
// layout (kPF*, kPB*) in vector loads. Every lane gets its row's two outputs
// in target units. All 32 lanes must call it (mma.sync).
__device__ __forceinline__ void mlp_forward_staged(const uint32_t* __restrict__ w, const float* __restrict__ p,
                                                   const uint32_t* X, float* out) {
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  const uint2* F1 = reinterpret_cast<const uint2*>(w + kPF1) + lane;          // + 32 j
  const uint4* F2 = reinterpret_cast<const uint4*>(w + kPF2) + 2 * lane;      // + 64 j
  const uint4* F3 = reinterpret_cast<const uint4*>(w + kPF3) + 2 * lane;
  const float4* B1 = reinterpret_cast<const float4*>(w + kPB1) + 4 * lane;
  const float4* B2 = reinterpret_cast<const float4*>(w + kPB2) + 4 * lane;
  const float2 b3 = __ldg(reinterpret_cast<const float2*>(w + kPB3) + lane);
  __syncwarp();
  // sample 16 t + rr sits on lane 4 (rr % 8), columns 0..1, in c3[0..1] (rr < 8)
  // or c3[2..3] of tile t; the tile loop is rolled to keep the code small
  const int rr = lane & 15, src = 4 * (rr & 7);
  const bool hi_r = rr >= 8;
  float y0 = 0.f, y1 = 0.f;
#pragma unroll 1
  for (int t = 0; t < 2; ++t) {
    float c3[4];
    uint32_t xa[4];
    load_a(X, 8, t, 0, g, q, xa);
    uint32_t h1[4][4];  // layer-2 A fragments, k-steps 0..3
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const float4 bb = __ldg(B1 + s);  // biases of n-tiles 2s, 2s+1
      float c[2][4] = {{bb.x, bb.y, bb.x, bb.y}, {bb.z, bb.w, bb.z, bb.w}};
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {
        const uint2 bf = __ldg(F1 + 32 * (2 * s + jj));
        const uint32_t b[2] = {bf.x, bf.y};
        mma_bf16(c[jj], xa, b);
      }
      relu_pack_a(c[0], c[1], h1[s]);
    }
    c3[0] = c3[2] = b3.x;
    c3[1] = c3[3] = b3.y;
#pragma unroll
    for (int s3 = 0; s3 < 4; ++s3) {
      const float4 bb = __ldg(B2 + s3);
      float c2[2][4] = {{bb.x, bb.y, bb.x, bb.y}, {bb.z, bb.w, bb.z, bb.w}};
#pragma unroll
      for (int jj = 0; jj < 2; ++jj) {
        const int j = 2 * s3 + jj;
        const uint4 f0 = __ldg(F2 + 64 * j), f1 = __ldg(F2 + 64 * j + 1);
        const uint32_t bk[4][2] = {{f0.x, f0.y}, {f0.z, f0.w}, {f1.x, f1.y}, {f1.z, f1.w}};
#pragma unroll
        for (int s = 0; s < 4; ++s) mma_bf16(c2[jj], h1[s], bk[s]);
      }
      const uint4 f3 = __ldg(F3 + (s3 >> 1));
      const uint32_t bw[2] = {(s3 & 1) ? f3.z : f3.x, (s3 & 1) ? f3.w : f3.y};
      uint32_t a3[4];
      relu_pack_a(c2[0], c2[1], a3);
      mma_bf16(c3, a3, bw);
    }
    const float v0 = __shfl_sync(kFull, c3[0], src), v1 = __shfl_sync(kFull, c3[1], src);
    const float v2 = __shfl_sync(kFull, c3[2], src), v3 = __shfl_sync(kFull, c3[3], src);
    if ((lane >> 4) == t) {
      y0 = hi_r ? v2 : v0;
      y1 = hi_r ? v3 : v1;
    }
  }
  __syncwarp();
  out[0] = y0 * p[kOffYsig] + p[kOffYmu];
  out[1] = y1 * p[kOffYsig + 1] + p[kOffYmu + 1];
}

// Fraction of the output interval [xend - hmax, xend] done at time rt (a
// learner feature; FP32 quotient).
__device__ __forceinline__ float interval_progress(double xend, double rt, double hmax) {
  return 1.f - __fdividef((float)(xend - rt), (float)hmax);
}

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// ---------------------------------------------------------------- step learner
// The training target is the step h* = h (1 / err)^(1/5) that would have put the
// error estimate (order 5) exactly at the acceptance threshold; the host scales
// the proposals down by a margin calibrated on held-out samples.
constexpr float kLearnRho = 1.0f;
constexpr double kMe = 9.10938291e-31;

// Hook of the tracer kernels. LRN = 0: plain (all no-ops), 1: collect training
// samples from the plain controller, 2: MLP step proposals.
template <int LRN>
struct StepLearner {
  // shared memory per warp: inference buffers (LRN 2), then raw feature rows of
  // the samples being collected
  static constexpr int kRawOff = LRN == 2 ? kWarpSmemInfer : 0;
  // words per warp of a launch: the raw rows only when samples are collected
  __host__ __device__ static constexpr int warp_words(bool collect) {
    return LRN == 0 ? 0 : kRawOff + ((LRN == 1 || collect) ? 32 * 16 : 0);
  }
  float c_mass, c_energy, c_sign, c_pitch;  // per-tracer feature constants
  float rlast;                              // this lane's latest correction from the network (1: none yet)
  float rcap;                               // cap on the correction of the pending step
  unsigned wit;                             // loop iterations of the warp (warp-uniform)
  double hctl;                              // learned: the controller's proposal for the pending step
  bool pend_apply;                          // learned: the pending step came from the staged accept
  double hbase;                             // collect: the controller's step after the sampled step
  double hcont;                             // learned: the step wanted before the interval-end clip
  bool want, pend, pend_sw, have_prop;
  uint32_t* sm;

  __device__ __forceinline__ void init(const KParams& P) {
    want = pend = pend_sw = have_prop = pend_apply = false;
    rlast = 1.f;
    wit = 0;
    sm = LRN ? rapt_dyn_smem + (threadIdx.x >> 5) * warp_words(P.collect != 0) : nullptr;
  }
  // Per-tracer constants; vs is the speed, pitch scale converts ppar to cos(pitch).
  __device__ __forceinline__ void load(double mass, double charge, double vs, double ppar_unit) {
    want = pend = pend_sw = have_prop = pend_apply = false;
    rlast = 1.f;
    if constexpr (LRN != 0) {
      const double gam = 1.0 / sqrt(1.0 - (vs / kC) * (vs / kC));
      c_mass = log10f((float)(mass / kMe));
      c_energy = log10f(fmaxf((float)(gam - 1.0), 1e-12f));
      c_sign = charge > 0 ? 1.f : -1.f;
      c_pitch = (float)(ppar_unit / (gam * mass * vs));
    }
  }
  // The step h is about to be clipped to end the output interval.
  __device__ __forceinline__ void before_clip(double h) {
    if constexpr (LRN == 2) hcont = h;
  }
  // After an accepted step of size h (err, previous err, the controller's next
  // step hnew) ending at position pos with parallel momentum ppar. A step that
  // ended an output interval gives no sample; the learned form continues the
  // next interval with the step wanted before the clip (in place of HINIT).
  // The learned form scales hnew by the lane's latest correction from the
  // network (capped at hmax and, after a rejection, at the last accepted step)
  // and stages this step's features for the warp's next network call (infer).
  // `allow` switches the proposals off (the plain controller takes over) for
  // the rest of an output interval that has seen many rejections. A step that
  // ends an interval whose row gets an adiabaticity check (`row_check`) stages
  // its features for a switch-labelled sample (on_row).
  __device__ __forceinline__ void on_accept(const KParams& P, int64_t idx, long long nacc, double h, double err,
                                            double errprev, double& hnew, double hmax, bool last, bool rej_before,
                                            bool allow, bool row_check, float x, float y, float z, float ppar,
                                            double vs, float progress) {
    if constexpr (LRN == 0) return;
    bool coll = false, coll_sw = false;
    if (last) {
      if constexpr (LRN == 2) {
        hnew = hcont;
        have_prop = true;
      }
      coll_sw = (LRN == 1 || P.collect) && row_check;
      if (!coll_sw) return;
    } else {
      coll = (LRN == 1 || P.collect) &&
             (mix64((uint64_t)idx * 0x100000001b3ull + (uint64_t)nacc) & P.samp_mask) == 0;
    }
    const bool inf = LRN == 2 && allow && !last;
    const double hprop = hnew;  // the controller's proposal
    // step ratios in FP32 (approximate quotients): they are features and caps
    // of a correction factor, and an FP64 division costs ~10 instructions of
    // the FP64 pipe (1/64 of the FP32 rate). A step capped at hmax to within
    // FP32 rounding is still clipped to the interval end (hmax = the interval).
    const float fh = (float)fabs(h), fhn = (float)fabs(hnew), fhmax = (float)hmax;
    if constexpr (LRN == 2) {
      if (inf) {
        float cap = __fdividef(fhmax, fhn);
        if (rej_before) cap = fminf(cap, __fdividef(fh, fhn));
        hctl = hnew;
        rcap = cap;
        hnew *= (double)fminf(rlast, cap);
      }
    }
    if (!coll && !coll_sw && !inf) return;
    float f[16];
    const float r = sqrtf(x * x + y * y + z * z);
    const float ir = __fdividef(1.f, r);
    f[0] = __logf((float)(fabs(h) * vs) * ir);
    f[1] = __log10f(fmaxf((float)err, 1e-10f));
    f[2] = __log10f(fmaxf((float)errprev, 1e-10f));
    f[3] = __logf(__fdividef(fhn, fh));
    f[4] = 1.f;
    f[5] = c_sign;
    f[6] = c_mass;
    f[7] = c_energy;
    f[8] = ppar * c_pitch;
    f[9] = __logf(r * (float)(1.0 / kRe));
    f[10] = z * ir;
    f[11] = progress;
    f[12] = __fdividef(fhmax, fh);
    f[13] = rej_before ? 1.f : 0.f;
    f[14] = 0.f;
    f[15] = 0.f;
    const int lane = threadIdx.x & 31;
    if (coll || coll_sw) {
      float* row = reinterpret_cast<float*>(sm + kRawOff) + lane * 16;
#pragma unroll
      for (int i = 0; i < 16; ++i) row[i] = f[i];
      pend = coll;
      pend_sw = coll_sw;
      hbase = hprop;
    }
    if constexpr (LRN == 2) {
      if (inf) {
        stage_features(P.mlp_p, f, sm, lane);
        want = true;
        pend_apply = true;
      }
    }
  }
  // Collect: label the staged sample with the attempt that followed it.
  __device__ __forceinline__ void on_attempt(const KParams& P, double h, double err, bool clipped) {
    if constexpr (LRN == 2) pend_apply = false;  // the pending step has been attempted
    if constexpr (LRN != 0) {
      if (!pend) return;
      pend = false;
      if (clipped) return;
      const float y0 = __logf((float)fabs(h / hbase)) + 0.2f * __logf(kLearnRho / fmaxf((float)err, 1e-10f));
      const unsigned long long pos = atomicAdd(P.samp_count, 1ull);
      if (pos < (unsigned long long)P.samp_cap) {
        const float* row = reinterpret_cast<const float*>(sm + kRawOff) + (threadIdx.x & 31) * 16;
        float* dst = P.samp + pos * kSampleStride;
#pragma unroll
        for (int i = 0; i < 16; ++i) dst[i] = row[i];
        dst[16] = y0;
        dst[17] = -1.f;
      }
    }
  }
  // Collect: the adiabaticity check of the row that ended the interval labels
  // the staged sample (label 1: the tracer switches to particle mode); its step
  // target is NaN (no step follows the row in this interval).
  __device__ __forceinline__ void on_row(const KParams& P, bool switches) {
    if constexpr (LRN != 0) {
      if (!pend_sw) return;
      pend_sw = false;
      const unsigned long long pos = atomicAdd(P.samp_count, 1ull);
      if (pos < (unsigned long long)P.samp_cap) {
        const float* row = reinterpret_cast<const float*>(sm + kRawOff) + (threadIdx.x & 31) * 16;
        float* dst = P.samp + pos * kSampleStride;
#pragma unroll
        for (int i = 0; i < 16; ++i) dst[i] = row[i];
        dst[16] = __int_as_float(0x7fc00000);
        dst[17] = switches ? 1.f : 0.f;
      }
    }
  }
  // Learned: warp-collective inference, on every learn_every-th iteration of
  // the warp's loop, for the lanes that staged features since the last call.
  // It refreshes their correction; a lane whose pending step is the one
  // proposed at the accept that staged the features gets the fresh correction
  // on that step at once (from the controller's proposal, so corrections do
  // not compound), the others from their next accepted step on. One call
  // serves every lane that accepted a step in between, so its cost is spread
  // over learn_every iterations. Called by all 32 lanes at the top of the loop.
  __device__ __forceinline__ void infer(const KParams& P, double& h) {
    if constexpr (LRN == 2) {
      ++wit;
      if (wit % (unsigned)P.learn_every == 0u && __any_sync(kFull, want)) {
        float o[2];
        mlp_forward_staged(P.mlp_w, P.mlp_p, sm, o);
        if (want) {
          rlast = __expf(fminf(fmaxf(o[0], -3.f), 3.f)) * P.learn_scale;
          if (pend_apply) h = hctl * (double)fminf(rlast, rcap);
        }
        want = false;
      }
    }
  }
};

}  // namespace rapt
