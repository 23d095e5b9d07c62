// mlp.cu -- training and batch inference of the step-size / switch MLP on the
// tensor cores (mma.sync BF16, FP32 accumulation), plus Adam and weight packing.
//
// Loss per sample: 0.5 (o0 - t0)^2 on the normalised step target (where it is
// not NaN) plus switch_weight * BCE(sigmoid(o1), label) where a label exists
// (label >= 0); the batch loss is the mean. Backward pass per 32-sample chunk (one warp):
//   dO -> dW3, db3 (CUDA cores), dZ2 = (dO W3^T) * [H2 > 0] (BF16),
//   dW2 = H1^T dZ2, dH1 = dZ2 W2^T, dZ1 = dH1 * [H1 > 0], dW1 = X^T dZ1
// (mma.sync). Deterministic: one warp per block sums its chunks' weight
// gradients in shared memory in program order (each lane adds to its own
// addresses), writes the block's partial gradient, and k_mlp_reduce sums the
// partials over the blocks in a fixed order -- no floating-point atomics, so
// the same samples, seed and parameters give the same bits on every run.
#include <cub/device/device_radix_sort.cuh>

#include "mlp.cuh"
#include "launch.h"

namespace rapt {
namespace {

static_assert(kMlpPacked == kMlpPackedWords, "packed weight size");
static_assert(((kMlpTrainable + 31) / 32 * 32) == kMlpGaccWords, "partial gradient stride");
constexpr int kTrainWarps = 1;  // one warp per block: see the header
// per-warp shared memory (u32): X, XT, H1, H1T, H2, dZ2, dZ2T, dZ1T, dO
constexpr int kSX = 0, kSXT = 256, kSH1 = 512, kSH1T = 1536, kSH2 = 2560, kSDZ2 = 3584, kSDZ2T = 4608,
              kSDZ1T = 5632, kSDO = 6656, kWarpSmemTrain = 6720;
constexpr int kGaccWords = (kMlpTrainable + 31) / 32 * 32;
constexpr size_t kTrainSmemBytes = (size_t)(kGaccWords + kTrainWarps * kWarpSmemTrain) * 4;

struct TrainArgs {
  const float* samples;  // [nsamp][kSampleStride]
  int64_t nsamp;
  int64_t batch;         // samples in this gradient
  int random;            // 1: sample indices drawn by hash from (seed, step); 0: samples 0..batch-1
  uint64_t seed;
  int64_t step;
  float inv_batch, switch_weight;
  const uint32_t* w;
  const float* p;
  float* partial;        // [gridDim.x][kGaccWords] per-block gradient sums
  double* lpart;         // [gridDim.x][2] per-block (step, switch) loss sums (divided by batch)
};

__device__ __forceinline__ void st16(uint32_t* base, int idx16, uint32_t v16) {
  reinterpret_cast<unsigned short*>(base)[idx16] = (unsigned short)v16;
}

__global__ void __launch_bounds__(kTrainWarps * 32) k_mlp_train(TrainArgs a) {
  float* gacc = reinterpret_cast<float*>(rapt_dyn_smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  uint32_t* S = rapt_dyn_smem + kGaccWords + warp * kWarpSmemTrain;
  uint32_t *X = S + kSX, *XT = S + kSXT, *H1 = S + kSH1, *H1T = S + kSH1T, *H2 = S + kSH2;
  uint32_t *DZ2 = S + kSDZ2, *DZ2T = S + kSDZ2T, *DZ1T = S + kSDZ1T;
  float* DO = reinterpret_cast<float*>(S + kSDO);
  for (int i = threadIdx.x; i < kGaccWords; i += blockDim.x) gacc[i] = 0.f;
  __syncthreads();
  const float* p = a.p;
  double l0sum = 0, l1sum = 0;

  const int64_t nchunks = (a.batch + 31) / 32;
  for (int64_t c = (int64_t)blockIdx.x * kTrainWarps + warp; c < nchunks; c += (int64_t)gridDim.x * kTrainWarps) {
    const int64_t b = c * 32 + lane;
    const bool valid = b < a.batch;
    int64_t si = 0;
    if (valid) si = a.random ? (int64_t)(mix64(a.seed ^ mix64((uint64_t)(a.step * a.batch + b))) % (uint64_t)a.nsamp) : b;
    const float* smp = a.samples + si * kSampleStride;
    // ---- forward
    float xn[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) xn[i] = valid ? norm_feature(smp[i], p[kOffXmu + i], p[kOffXsig + i]) : 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const uint32_t u = pack_bf16x2(xn[2 * i], xn[2 * i + 1]);
      X[lane * 8 + i] = u;
      st16(XT, (2 * i) * 32 + lane, u & 0xffffu);
      st16(XT, (2 * i + 1) * 32 + lane, u >> 16);
    }
    __syncwarp();
    dense_relu<16, 64>(X, a.w + kPW1, p + kOffB1, H1, g, q);
    __syncwarp();
#pragma unroll 4
    for (int jj = 0; jj < 32; ++jj) {
      const int j = (jj + lane) & 31;
      const uint32_t u = H1[lane * 32 + j];
      st16(H1T, (2 * j) * 32 + lane, u & 0xffffu);
      st16(H1T, (2 * j + 1) * 32 + lane, u >> 16);
    }
    dense_relu<64, 64>(H1, a.w + kPW2, p + kOffB2, H2, g, q);
    __syncwarp();
    float o[2];
    dense_out(H2, a.w + kPW3, p + kOffB3, g, q, lane, o);
    // ---- loss and output gradient
    float d0 = 0.f, d1 = 0.f;
    if (valid) {
      const float tg = smp[16];  // NaN: no step target (switch-labelled sample)
      if (tg == tg) {
        const float tn = (tg - p[kOffYmu]) / p[kOffYsig];
        d0 = o[0] - tn;
        l0sum += 0.5 * (double)d0 * d0;
      }
      const float lab = smp[17];
      if (lab >= 0.f) {
        const float sg = 1.f / (1.f + __expf(-o[1]));
        d1 = a.switch_weight * (sg - lab);
        // BCE with logits: max(o,0) - o*lab + log(1 + exp(-|o|))
        l1sum += (double)a.switch_weight * (fmaxf(o[1], 0.f) - o[1] * lab + log1pf(__expf(-fabsf(o[1]))));
      }
    }
    d0 *= a.inv_batch;
    d1 *= a.inv_batch;
    DO[2 * lane] = d0;
    DO[2 * lane + 1] = d1;
    __syncwarp();
    // ---- dW3, db3: lane handles hidden units 2 lane, 2 lane + 1
    {
      float a00 = 0, a01 = 0, a10 = 0, a11 = 0;
#pragma unroll 4
      for (int s = 0; s < 32; ++s) {
        const uint32_t u = H2[s * 32 + lane];
        const float h0 = bf16_lo(u), h1 = bf16_hi(u), e0 = DO[2 * s], e1 = DO[2 * s + 1];
        a00 += h0 * e0; a01 += h0 * e1; a10 += h1 * e0; a11 += h1 * e1;
      }
      gacc[kOffW3 + 2 * lane] += a00;
      gacc[kOffW3 + 64 + 2 * lane] += a01;
      gacc[kOffW3 + 2 * lane + 1] += a10;
      gacc[kOffW3 + 64 + 2 * lane + 1] += a11;
      float s0 = d0, s1 = d1;
#pragma unroll
      for (int m = 16; m > 0; m >>= 1) {
        s0 += __shfl_xor_sync(kFull, s0, m);
        s1 += __shfl_xor_sync(kFull, s1, m);
      }
      if (lane == 0) { gacc[kOffB3] += s0; gacc[kOffB3 + 1] += s1; }
    }
    // ---- dZ2 = (dO W3^T) * [H2 > 0], lane = sample
    {
      const uint32_t* W3N = a.w + kPW3N;
#pragma unroll 4
      for (int jj = 0; jj < 32; ++jj) {
        const int j = (jj + lane) & 31;
        const uint32_t hu = H2[lane * 32 + j];
        const uint32_t wa = W3N[(2 * j) * 4], wb = W3N[(2 * j + 1) * 4];
        const float z0 = bf16_lo(hu) > 0.f ? d0 * bf16_lo(wa) + d1 * bf16_hi(wa) : 0.f;
        const float z1 = bf16_hi(hu) > 0.f ? d0 * bf16_lo(wb) + d1 * bf16_hi(wb) : 0.f;
        const uint32_t pk = pack_bf16x2(z0, z1);
        DZ2[lane * 32 + j] = pk;
        st16(DZ2T, (2 * j) * 32 + lane, pk & 0xffffu);
        st16(DZ2T, (2 * j + 1) * 32 + lane, pk >> 16);
      }
    }
    __syncwarp();
    // ---- db2: lane sums rows 2 lane, 2 lane + 1 of dZ2T over the 32 samples
    {
      float s0 = 0, s1 = 0;
#pragma unroll 4
      for (int ww = 0; ww < 16; ++ww) {
        const int w = (ww + lane) & 15;
        const uint32_t u0 = DZ2T[(2 * lane) * 16 + w], u1 = DZ2T[(2 * lane + 1) * 16 + w];
        s0 += bf16_lo(u0) + bf16_hi(u0);
        s1 += bf16_lo(u1) + bf16_hi(u1);
      }
      gacc[kOffB2 + 2 * lane] += s0;
      gacc[kOffB2 + 2 * lane + 1] += s1;
    }
    // ---- dW2[in m][out n] = sum_s H1[s][m] dZ2[s][n]; stored as W2T[n][m]
#pragma unroll 1
    for (int t = 0; t < 4; ++t) {
#pragma unroll 2
      for (int j = 0; j < 8; ++j) {
        float cc[4] = {0, 0, 0, 0};
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          uint32_t af[4], bf[2];
          load_a(H1T, 16, t, s, g, q, af);
          load_b(DZ2T, 16, j, s, g, q, bf);
          mma_bf16(cc, af, bf);
        }
        const int m0 = 16 * t + g, n0 = 8 * j + 2 * q;
        gacc[kOffW2 + n0 * 64 + m0] += cc[0];
        gacc[kOffW2 + (n0 + 1) * 64 + m0] += cc[1];
        gacc[kOffW2 + n0 * 64 + m0 + 8] += cc[2];
        gacc[kOffW2 + (n0 + 1) * 64 + m0 + 8] += cc[3];
      }
    }
    // ---- dZ1 = (dZ2 W2^T) * [H1 > 0] -> dZ1T [64 in][32 samples]
#pragma unroll 1
    for (int j = 0; j < 8; ++j) {
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        float cc[4] = {0, 0, 0, 0};
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          uint32_t af[4], bf[2];
          load_a(DZ2, 32, t, s, g, q, af);
          load_b(a.w + kPW2N, 32, j, s, g, q, bf);
          mma_bf16(cc, af, bf);
        }
        const int r0 = 16 * t + g, r1 = r0 + 8, n0 = 8 * j + 2 * q;
        const uint32_t m0 = H1[r0 * 32 + 4 * j + q], m1 = H1[r1 * 32 + 4 * j + q];
        const uint32_t p0 = pack_bf16x2(bf16_lo(m0) > 0.f ? cc[0] : 0.f, bf16_hi(m0) > 0.f ? cc[1] : 0.f);
        const uint32_t p1 = pack_bf16x2(bf16_lo(m1) > 0.f ? cc[2] : 0.f, bf16_hi(m1) > 0.f ? cc[3] : 0.f);
        st16(DZ1T, n0 * 32 + r0, p0 & 0xffffu);
        st16(DZ1T, (n0 + 1) * 32 + r0, p0 >> 16);
        st16(DZ1T, n0 * 32 + r1, p1 & 0xffffu);
        st16(DZ1T, (n0 + 1) * 32 + r1, p1 >> 16);
      }
    }
    __syncwarp();
    // ---- db1
    {
      float s0 = 0, s1 = 0;
#pragma unroll 4
      for (int ww = 0; ww < 16; ++ww) {
        const int w = (ww + lane) & 15;
        const uint32_t u0 = DZ1T[(2 * lane) * 16 + w], u1 = DZ1T[(2 * lane + 1) * 16 + w];
        s0 += bf16_lo(u0) + bf16_hi(u0);
        s1 += bf16_lo(u1) + bf16_hi(u1);
      }
      gacc[kOffB1 + 2 * lane] += s0;
      gacc[kOffB1 + 2 * lane + 1] += s1;
    }
    // ---- dW1[in m][out n] = sum_s X[s][m] dZ1[s][n]; stored as W1T[n][m]
#pragma unroll 2
    for (int j = 0; j < 8; ++j) {
      float cc[4] = {0, 0, 0, 0};
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        uint32_t af[4], bf[2];
        load_a(XT, 16, 0, s, g, q, af);
        load_b(DZ1T, 16, j, s, g, q, bf);
        mma_bf16(cc, af, bf);
      }
      const int n0 = 8 * j + 2 * q;
      gacc[kOffW1 + n0 * 16 + g] += cc[0];
      gacc[kOffW1 + (n0 + 1) * 16 + g] += cc[1];
      gacc[kOffW1 + n0 * 16 + g + 8] += cc[2];
      gacc[kOffW1 + (n0 + 1) * 16 + g + 8] += cc[3];
    }
    __syncwarp();
  }
  // loss: warp reduce (a fixed butterfly order)
#pragma unroll
  for (int m = 16; m > 0; m >>= 1) {
    l0sum += __shfl_xor_sync(kFull, l0sum, m);
    l1sum += __shfl_xor_sync(kFull, l1sum, m);
  }
  if (lane == 0) {
    a.lpart[2 * blockIdx.x] = l0sum * (double)a.inv_batch;
    a.lpart[2 * blockIdx.x + 1] = l1sum * (double)a.inv_batch;
  }
  __syncwarp();
  float* dst = a.partial + (size_t)blockIdx.x * kGaccWords;
  for (int i = threadIdx.x; i < kGaccWords; i += blockDim.x) dst[i] = gacc[i];
}

// grad[i] = sum over blocks of partial[b][i], blocks in order; thread 0 of
// block 0 adds the loss partials to loss[0..1] in order.
__global__ void k_mlp_reduce(const float* partial, const double* lpart, int nblocks, float* grad, double* loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kMlpTrainable) {
    float s = 0.f;
    for (int b = 0; b < nblocks; ++b) s += partial[(size_t)b * kGaccWords + i];
    grad[i] = s;
  }
  if (i == 0 && loss) {
    double l0 = 0, l1 = 0;
    for (int b = 0; b < nblocks; ++b) { l0 += lpart[2 * b]; l1 += lpart[2 * b + 1]; }
    loss[0] += l0;
    loss[1] += l1;
  }
}

// One packed u32 slot per thread.
__global__ void k_mlp_pack(const float* p, uint32_t* w) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= kMlpPacked) return;
  float lo, hi;
  if (s < kPW2) {
    const int o = s / 8, i2 = s % 8;
    lo = p[kOffW1 + o * 16 + 2 * i2]; hi = p[kOffW1 + o * 16 + 2 * i2 + 1];
  } else if (s < kPW3) {
    const int r = s - kPW2, o = r / 32, i2 = r % 32;
    lo = p[kOffW2 + o * 64 + 2 * i2]; hi = p[kOffW2 + o * 64 + 2 * i2 + 1];
  } else if (s < kPW2N) {
    const int r = s - kPW3, o = r / 32, i2 = r % 32;
    lo = p[kOffW3 + o * 64 + 2 * i2]; hi = p[kOffW3 + o * 64 + 2 * i2 + 1];
  } else if (s < kPW3N) {
    const int r = s - kPW2N, in = r / 32, o2 = r % 32;
    lo = p[kOffW2 + (2 * o2) * 64 + in]; hi = p[kOffW2 + (2 * o2 + 1) * 64 + in];
  } else if (s < kPF1) {
    const int r = s - kPW3N, in = r / 4, o2 = r % 4;
    lo = p[kOffW3 + (2 * o2) * 64 + in]; hi = p[kOffW3 + (2 * o2 + 1) * 64 + in];
  } else if (s < kPB1) {
    // B fragments of one lane (g = lane / 4, q = lane % 4): u32 column c of W?T row n
    int row, c, base, stride;
    if (s < kPF2) {         // W1: [j][lane][k], k-step 0
      const int r = s - kPF1, j = r / 64, lane = (r / 2) % 32, k = r % 2;
      row = 8 * j + lane / 4; c = lane % 4 + 4 * k; base = kOffW1; stride = 16;
    } else if (s < kPF3) {  // W2: [j][lane][2 s + half]
      const int r = s - kPF2, j = r / 256, lane = (r / 8) % 32, k = r % 8;
      row = 8 * j + lane / 4; c = 8 * (k / 2) + lane % 4 + 4 * (k % 2); base = kOffW2; stride = 64;
    } else {                // W3: [lane][2 s3 + half], n-tile 0
      const int r = s - kPF3, lane = r / 8, k = r % 8;
      row = lane / 4; c = 8 * (k / 2) + lane % 4 + 4 * (k % 2); base = kOffW3; stride = 64;
    }
    lo = p[base + row * stride + 2 * c]; hi = p[base + row * stride + 2 * c + 1];
  } else {
    // bias pairs of one lane, stored as float bits
    int idx;
    if (s < kPB2) { const int r = s - kPB1, lane = r / 16, k = r % 16; idx = kOffB1 + 8 * (k / 2) + 2 * (lane % 4) + k % 2; }
    else if (s < kPB3) { const int r = s - kPB2, lane = r / 16, k = r % 16; idx = kOffB2 + 8 * (k / 2) + 2 * (lane % 4) + k % 2; }
    else { const int r = s - kPB3, lane = r / 2, k = r % 2; idx = kOffB3 + 2 * (lane % 4) + k; }
    w[s] = __float_as_uint(p[idx]);
    return;
  }
  w[s] = pack_bf16x2(lo, hi);
}

// Adam on the trainable part of the parameter vector.
__global__ void k_mlp_adam(float* p, float* m, float* v, const float* g, float lr, float b1, float b2, float eps,
                           float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpTrainable) return;
  const float gi = g[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

__global__ void __launch_bounds__(128) k_mlp_forward(const uint32_t* w, const float* p, const float* feat, int64_t n,
                                                     float* out) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t* sm = rapt_dyn_smem + warp * kWarpSmemInfer;
  const int64_t nchunks = (n + 31) / 32;
  for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; c < nchunks;
       c += (int64_t)gridDim.x * (blockDim.x >> 5)) {
    const int64_t i = c * 32 + lane;
    float f[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) f[k] = i < n ? feat[i * 16 + k] : 0.f;
    stage_features(p, f, sm, lane);
    float o[2];
    mlp_forward_staged(w, p, sm, o);
    if (i < n) {
      out[2 * i] = o[0];
      out[2 * i + 1] = o[1];
    }
  }
}

// Sort key of a sample: a 64-bit hash of its 18 words (mix64 chained over the
// words); the value is the sample's index.
__global__ void k_sample_keys(const float* samples, int64_t n, unsigned long long* keys, uint32_t* idx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t* w = reinterpret_cast<const uint32_t*>(samples + i * kSampleStride);
  uint64_t h = 0x243f6a8885a308d3ull;
#pragma unroll
  for (int k = 0; k < kSampleStride; ++k) h = mix64(h ^ w[k]);
  keys[i] = h;
  idx[i] = (uint32_t)i;
}

__global__ void k_sample_gather(const float* src, const uint32_t* idx, int64_t n, float* dst) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * kSampleStride) return;
  const int64_t i = t / kSampleStride, k = t % kSampleStride;
  dst[t] = src[(int64_t)idx[i] * kSampleStride + k];
}

}  // namespace

// Workspace of mlp_samples_sort: keys in/out, indices in/out, the gathered
// copy, and CUB's radix-sort storage, each 256-byte aligned.
static size_t al256(size_t b) { return (b + 255) & ~size_t(255); }
static size_t cub_sort_bytes(int64_t n) {
  size_t b = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, b, (const unsigned long long*)nullptr, (unsigned long long*)nullptr,
                                  (const uint32_t*)nullptr, (uint32_t*)nullptr, (int)n);
  return b;
}
size_t mlp_sort_tmp_bytes(int64_t n) {
  return 2 * al256((size_t)n * 8) + 2 * al256((size_t)n * 4) + al256((size_t)n * kSampleStride * 4) +
         al256(cub_sort_bytes(n));
}

cudaError_t mlp_samples_sort(float* samples, int64_t n, void* tmp, size_t tmp_bytes, cudaStream_t s) {
  if (n <= 1) return cudaSuccess;
  if (n > 0x7fffffffLL || tmp_bytes < mlp_sort_tmp_bytes(n)) return cudaErrorInvalidValue;
  char* p = static_cast<char*>(tmp);
  auto take = [&](size_t b) { char* q = p; p += al256(b); return q; };
  auto* k0 = reinterpret_cast<unsigned long long*>(take((size_t)n * 8));
  auto* k1 = reinterpret_cast<unsigned long long*>(take((size_t)n * 8));
  auto* i0 = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  auto* i1 = reinterpret_cast<uint32_t*>(take((size_t)n * 4));
  auto* copy = reinterpret_cast<float*>(take((size_t)n * kSampleStride * 4));
  size_t cb = cub_sort_bytes(n);
  void* cubtmp = take(cb);
  k_sample_keys<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(samples, n, k0, i0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  e = cub::DeviceRadixSort::SortPairs(cubtmp, cb, k0, k1, i0, i1, (int)n, 0, 64, s);
  if (e != cudaSuccess) return e;
  const int64_t words = n * kSampleStride;
  k_sample_gather<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(samples, i1, n, copy);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(samples, copy, (size_t)words * 4, cudaMemcpyDeviceToDevice, s);
}

cudaError_t mlp_pack(const float* p, uint32_t* w, cudaStream_t s) {
  k_mlp_pack<<<(kMlpPacked + 255) / 256, 256, 0, s>>>(p, w);
  return cudaGetLastError();
}

cudaError_t mlp_grad(const float* samples, int64_t nsamp, int64_t batch, int random, uint64_t seed, int64_t step,
                     float switch_weight, const uint32_t* w, const float* p, float* grad, double* loss, float* partial,
                     double* lpart, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmemBytes);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  TrainArgs a{samples, nsamp, batch, random, seed, step, 1.f / (float)batch, switch_weight, w, p, partial, lpart};
  const int64_t chunks = (batch + 31) / 32;
  int64_t grid = (chunks + 1) / 2;  // two chunks per warp
  if (grid > kMlpTrainMaxBlocks) grid = kMlpTrainMaxBlocks;
  if (grid < 1) grid = 1;
  k_mlp_train<<<(unsigned)grid, kTrainWarps * 32, kTrainSmemBytes, s>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_mlp_reduce<<<(kMlpTrainable + 255) / 256, 256, 0, s>>>(partial, lpart, (int)grid, grad, loss);
  return cudaGetLastError();
}

cudaError_t mlp_adam(float* p, float* m, float* v, const float* g, float lr, int64_t t, cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - powf(b1, (float)t), bc2 = 1.f - powf(b2, (float)t);
  k_mlp_adam<<<(kMlpTrainable + 255) / 256, 256, 0, s>>>(p, m, v, g, lr, b1, b2, 1e-8f, bc1, bc2);
  return cudaGetLastError();
}

cudaError_t mlp_forward(const uint32_t* w, const float* p, const float* feat, int64_t n, float* out, int num_sms,
                        cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t chunks = (n + 31) / 32;
  int64_t grid = (chunks + 3) / 4;
  if (grid > 4 * num_sms) grid = 4 * num_sms;
  k_mlp_forward<<<(unsigned)grid, 128, 4 * kWarpSmemInfer * 4, s>>>(w, p, feat, n, out);
  return cudaGetLastError();
}

}  // namespace rapt
