// capi.cu -- the C ABI of librapt_gpu.so (declared in include/rapt_gpu.h).
//
// The context owns one CUDA stream, one device block holding every SoA array
// of the ensemble, and a small scratch block (work-queue heads and counters of
// the persistent kernels). rapt_advance() runs rounds of one launch per mode
// until no tracer is left pending (Adaptive alternates modes across rounds).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cub/device/device_radix_sort.cuh>

#include "launch.h"

using namespace rapt;

namespace {

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  bool field_set = false;
  FieldP field{};
  rapt_config cfg{};
  int num_sms = 0;
  int64_t n = 0;
  int max_rows = 0, max_sw = 0;
  void* block = nullptr;
  DevEnsemble E{};
  Scratch* scratch = nullptr;
  unsigned long long* h_pending = nullptr;  // pinned
  void* tmp = nullptr;
  size_t tmp_bytes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  ModelTable tab[RAPT_N_MODELS];
  // step-size MLP: one device block of parameters, Adam moments, gradient,
  // loss and packed weights; a separate sample buffer
  void* mlp_block = nullptr;
  float *mlp_p = nullptr, *mlp_m = nullptr, *mlp_v = nullptr, *mlp_g = nullptr;
  double* mlp_loss = nullptr;
  uint32_t* mlp_w = nullptr;
  // work-queue order (longest expected work first): sort keys and indices,
  // the step totals at the start of the last call, CUB's sort storage
  void* ord_block = nullptr;
  uint32_t *ord_key_in = nullptr, *ord_key_out = nullptr;
  int32_t *ord_idx_in = nullptr, *ord = nullptr;
  int64_t* ord_steps = nullptr;
  void* ord_tmp = nullptr;
  size_t ord_tmp_bytes = 0;
  float* mlp_partial = nullptr;  // [kMlpTrainMaxBlocks][kMlpGaccWords]
  double* mlp_lpart = nullptr;   // [kMlpTrainMaxBlocks][2]
  bool mlp_ready = false;
  int64_t mlp_t = 0;  // Adam step count
  double* fl_scratch = nullptr;  // field-line traces of the bounce-period cadence
  size_t fl_bytes = 0;
  float* samp = nullptr;
  unsigned long long* samp_count = nullptr;
  int64_t samp_cap = 0;
  uint64_t samp_mask = 0;
  // Grid field: axes and snapshots in one device block (rapt_grid_set)
  double* grid = nullptr;
  FieldP grid_desc{};  // only the g* pointers and sizes are used
};

int fail(Ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess) return fail(c, RAPT_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T>
T* carve(char*& p, size_t count) {
  T* r = reinterpret_cast<T*>(p);
  size_t bytes = count * sizeof(T);
  bytes = (bytes + 255) & ~size_t(255);
  p += bytes;
  return r;
}

size_t ensemble_bytes(int64_t n, int max_rows, int max_sw) {
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t N = (size_t)n;
  size_t b = 0;
  b += 2 * al(N);                                      // mode, seg_active
  b += al(N * max_rows) + al(N * max_sw);              // row_mode, sw_mode
  b += 5 * al(N * 4);                                  // status, flags, nrows, nswitch, nseg
  b += 22 * al(N * 8);                                 // doubles
  b += al(N * max_rows * 7 * 8) + al(N * max_sw * 8);  // rows, sw_time
  b += 3 * al(N * 8);                                  // int64 counters
  return b;
}

void build_field(int model, const double* params, int np, FieldP* f) {
  std::memset(f, 0, sizeof(*f));
  f->model = model;
  f->is_static = 1;
  f->gradstep = 1e-6;  // _Field.__init__, fields.py:38-41
  f->timestep = 1e-3;
  double* p = f->p;
  switch (model) {
    case RAPT_EARTH_DIPOLE: p[0] = kB0; f->gradstep = kRe * 1e-6; break;
    case RAPT_DOUBLE_DIPOLE: p[0] = kB0; p[1] = 20 * kRe; p[2] = 1; f->gradstep = kRe / 1000; break;
    case RAPT_UNIFORM_BZ: p[0] = 1; break;
    case RAPT_UNIFORM_CROSSED_EB: p[0] = 1; p[1] = 1; f->is_static = 0; break;
    case RAPT_VAR_EARTH_DIPOLE: p[0] = 0.1; p[1] = 10; f->gradstep = kRe / 1000; f->is_static = 0; break;
    case RAPT_PARABOLIC: p[0] = 10.0; p[1] = 1.0; p[2] = 0.2; break;
    case RAPT_HARRIS: p[0] = 20e-9; p[1] = 0.5 * kRe; p[2] = 2e-9; p[3] = 0.2e-3; f->is_static = 0; break;
    case RAPT_COMPRESSED_DIPOLE: p[0] = kB0; p[1] = 0.1; p[2] = 60.0; f->gradstep = kRe / 1000; f->is_static = 0; break;
    case RAPT_GRID: f->gradstep = 1e-3 * kRe; break;  // fields.py:578; static stays 1 (fields.py:41)
    default: break;
  }
  for (int i = 0; i < np && i < 8; ++i) p[i] = params[i];
  if (model == RAPT_HARRIS) f->gradstep = p[1] * 1e-4;
}

void attach_grid(const FieldP& g, FieldP* f) {
  f->gt = g.gt; f->gx = g.gx; f->gy = g.gy; f->gz = g.gz;
  f->gB = g.gB; f->gE = g.gE;
  f->nt = g.nt; f->nx = g.nx; f->ny = g.ny; f->nz = g.nz;
  for (int a = 0; a < 4; ++a) f->ginv[a] = g.ginv[a];
}

void finish_field(FieldP* f) {
  const double* p = f->p;
  f->inv2d = 1.0 / (2.0 * f->gradstep);
  switch (f->model) {
    case RAPT_EARTH_DIPOLE: f->c0 = -3.0 * p[0] * kRe3; break;
    case RAPT_DOUBLE_DIPOLE: f->c0 = -p[0] * kRe3; break;
    case RAPT_VAR_EARTH_DIPOLE: f->c0 = -kB0 * kRe3; f->c1 = 2.0 * kPi / p[1]; break;
    case RAPT_HARRIS: f->c0 = 1.0 / p[1]; break;
    case RAPT_COMPRESSED_DIPOLE:
      f->c0 = -p[0] * kRe3;
      f->c1 = 2.0 * kPi / p[2];
      f->c2 = p[0] * p[1] * f->c1 * kRe3;
      break;
    default: break;
  }
  // float-float constants of the FP32 form's field models (positions in Re)
  double k[4] = {0, 0, 0, 0};
  if (f->model == RAPT_EARTH_DIPOLE) k[0] = -3.0 * p[0];
  if (f->model == RAPT_DOUBLE_DIPOLE) { k[0] = -p[0]; k[1] = p[1] / kRe; k[2] = p[2]; }
  for (int i = 0; i < 4; ++i) {
    f->dh[i] = (float)k[i];
    f->dl[i] = (float)(k[i] - (double)f->dh[i]);
  }
  // the FP32 form's dipole stencil (fp32_form.cuh): positions in units of
  // L = 2^22 m, unit coefficient; c = -B0 (Re / L)^3 in both dipole models
  if (f->model == RAPT_EARTH_DIPOLE || f->model == RAPT_DOUBLE_DIPOLE) {
    const double L = 4194304.0;
    auto split = [](double v, float& h, float& l) { h = (float)v; l = (float)(v - (double)h); };
    f->sd = (float)(f->gradstep / L);
    const double step = (double)f->sd * L;  // the realised step (m)
    const double c = -p[0] * (kRe / L) * (kRe / L) * (kRe / L);
    split(fabs(c), f->cah, f->cal);
    split(fabs(c) / (2.0 * step), f->sgh, f->sgl);
    split((c < 0 ? -1.0 : 1.0) / (2.0 * step), f->sch, f->scl);
    if (f->model == RAPT_DOUBLE_DIPOLE) {
      split(p[1], f->sxh, f->sxl);
      split(p[2], f->skh, f->skl);
    }
  }
}

// trace points per direction of the bounce-period field-line trace; a thread's
// scratch is 8 * kFieldlineCap doubles (64 KB)
constexpr int kFieldlineCap = 1024;

KParams make_params(const Ctx* c, int kind) {
  KParams P{};
  P.f = c->field;
  const rapt_config& g = c->cfg;
  P.rtol = g.rtol; P.atol = g.atol; P.cycres = g.cyclotronresolution; P.gctimestep = g.gctimestep;
  P.epss = g.epss; P.epst = g.epst; P.rkf_tol = g.rkf_tol; P.rkf_hmin = g.rkf_hmin;
  P.enforce_eq = g.enforce_equatorial; P.tableau = g.tableau; P.gc_eom = g.gc_eom; P.nsteps = g.nsteps;
  P.kind = kind; P.form = g.form;
  P.budget = g.max_steps_per_launch > 0 ? g.max_steps_per_launch : (1LL << 62);
  P.max_rows = c->max_rows; P.max_sw = c->max_sw;
  P.max_segments = 100000;
  P.mlp_w = c->mlp_w;
  P.mlp_p = c->mlp_p;
  P.learn_scale = g.learned_scale > 0 ? (float)g.learned_scale : 1.0f;
  P.samp = c->samp;
  P.samp_count = c->samp_count;
  P.samp_cap = c->samp_cap;
  P.samp_mask = c->samp_mask;
  P.collect = g.collect;
  P.bounceres = g.bounceresolution;
  P.flres = g.fieldlineresolution;
  P.fl_scratch = nullptr;
  P.fl_cap = kFieldlineCap;
  P.fl_stride = 8LL * kFieldlineCap;
  P.learn_every = g.learned_every > 1 ? g.learned_every : 1;
  return P;
}

__global__ void k_prepare(DevEnsemble E, const double* delta, double delta_all, int kind) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= E.n) return;
  E.delta[k] = delta ? delta[k] : delta_all;
  E.flags[k] &= RAPT_FLAG_CHECK_ADIABATICITY;
  if (kind == RAPT_KIND_ADAPTIVE) E.flags[k] |= RAPT_FLAG_CHECK_ADIABATICITY;
  E.seg_active[k] = 0;
  E.nseg[k] = 0;
  E.status[k] = RAPT_ST_OK;
  E.t_int[k] = E.t_row[k];
}

__global__ void k_fill_defaults(DevEnsemble E, int have_tint, int have_tcur) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= E.n) return;
  if (!have_tint) E.t_int[k] = E.t_row[k];
  if (!have_tcur) E.tcur[k] = E.t_row[k];
}

// Dependent-chain FMA throughput kernels (8 independent chains per thread).
template <typename T>
__global__ void k_fma_peak(T* out, int iters, T seed) {
  T a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = seed + (T)(threadIdx.x + j);
  const T m = (T)0.9999999, b = (T)1e-7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = fma(a[j], m, b);
  }
  T s = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += a[j];
  if (s == (T)-1.2345) out[threadIdx.x] = s;
}

}  // namespace

extern "C" {

int rapt_abi_version(void) { return RAPT_GPU_ABI_VERSION; }

void rapt_config_default(rapt_config* g) {
  std::memset(g, 0, sizeof(*g));
  g->rtol = 1.49012e-8;  // rapt/__init__.py:21-34
  g->atol = 1.49012e-8;
  g->cyclotronresolution = 10;
  g->gctimestep = 0;
  g->epss = 5e-2;
  g->epst = 5e-2;
  g->nsteps = 500;
  g->rkf_tol = 1e-3;
  g->rkf_hmin = 1e-12;
  g->bounceresolution = 10;
  g->fieldlineresolution = 50;
}

int rapt_ctx_create(int device, void** out) {
  if (!out) return RAPT_ERR_INVALID;
  *out = nullptr;
  Ctx* c = new Ctx();
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete c; return RAPT_ERR_CUDA; }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&c->scratch, sizeof(Scratch)) != cudaSuccess ||
      cudaMallocHost(&c->h_pending, sizeof(unsigned long long)) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
    delete c;
    return RAPT_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  register_model_0(&c->tab[0]);
  register_model_1(&c->tab[1]);
  register_model_2(&c->tab[2]);
  register_model_3(&c->tab[3]);
  register_model_4(&c->tab[4]);
  register_model_5(&c->tab[5]);
  register_model_6(&c->tab[6]);
  register_model_7(&c->tab[7]);
  register_model_8(&c->tab[8]);
  rapt_config_default(&c->cfg);
  *out = c;
  return RAPT_OK;
}

void rapt_ctx_destroy(void* ctx) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->block);
  cudaFree(c->ord_block);
  cudaFree(c->scratch);
  cudaFree(c->tmp);
  cudaFree(c->mlp_block);
  cudaFree(c->fl_scratch);
  cudaFree(c->samp_count);  // base of the sample allocation
  cudaFree(c->grid);
  cudaFreeHost(c->h_pending);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char* rapt_last_error(const void* ctx) {
  const Ctx* c = static_cast<const Ctx*>(ctx);
  return c ? c->err.c_str() : "null context";
}

int rapt_field_set(void* ctx, int model, const double* params, int nparams) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  if (model < 0 || model >= RAPT_N_MODELS)
    return fail(c, RAPT_ERR_UNSUPPORTED, "field model %d has no device implementation", model);
  if (nparams < 0 || nparams > 8 || (nparams > 0 && !params)) return fail(c, RAPT_ERR_INVALID, "bad field params");
  if (model == RAPT_GRID && !c->grid) return fail(c, RAPT_ERR_STATE, "no grid data: call rapt_grid_set");
  build_field(model, params, nparams, &c->field);
  if (model == RAPT_GRID) attach_grid(c->grid_desc, &c->field);
  if (model == RAPT_DOUBLE_DIPOLE && !(c->field.p[2] >= 1))
    return fail(c, RAPT_ERR_INVALID, "DoubleDipole imagestrength must be >= 1 (fields.py:340)");
  finish_field(&c->field);
  c->field_set = true;
  return RAPT_OK;
}

int rapt_field_set_steps(void* ctx, double gradientstepsize, double timederivstepsize) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  if (!c->field_set) return fail(c, RAPT_ERR_STATE, "no field set");
  if (!(gradientstepsize > 0) || !(timederivstepsize > 0)) return fail(c, RAPT_ERR_INVALID, "step sizes must be > 0");
  c->field.gradstep = gradientstepsize;
  c->field.timestep = timederivstepsize;
  finish_field(&c->field);
  return RAPT_OK;
}

int rapt_field_set_static(void* ctx, int is_static) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  if (!c->field_set) return fail(c, RAPT_ERR_STATE, "no field set");
  c->field.is_static = is_static ? 1 : 0;
  return RAPT_OK;
}

static bool ascending(const double* a, int n) {
  for (int i = 0; i < n; ++i)
    if (!std::isfinite(a[i]) || (i > 0 && !(a[i] > a[i - 1]))) return false;
  return true;
}

int rapt_grid_set(void* ctx, int32_t nt, const double* t, int32_t nx, const double* x, int32_t ny, const double* y,
                  int32_t nz, const double* z, const double* B, const double* E) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  if (nt < 1 || nx < 2 || ny < 2 || nz < 2 || !t || !x || !y || !z || !B)
    return fail(c, RAPT_ERR_INVALID, "grid: need nt >= 1 snapshots, >= 2 points per axis, axes and B");
  if (!ascending(t, nt) || !ascending(x, nx) || !ascending(y, ny) || !ascending(z, nz))
    return fail(c, RAPT_ERR_INVALID, "grid: times and axes must be finite and strictly ascending");
  const size_t nodes = (size_t)nt * (size_t)nx * (size_t)ny * (size_t)nz;
  if (nodes > ((size_t)1 << 36)) return fail(c, RAPT_ERR_INVALID, "grid: too many nodes");
  const size_t naxis = (size_t)nt + nx + ny + nz;
  const size_t words = naxis + 3 * nodes * (E ? 2 : 1);
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (c->grid) {
    CK(cudaFree(c->grid));
    c->grid = nullptr;
    if (c->field_set && c->field.model == RAPT_GRID) c->field_set = false;
  }
  double* d = nullptr;
  if (cudaMalloc(&d, words * sizeof(double)) != cudaSuccess)
    return fail(c, RAPT_ERR_NOMEM, "grid: cannot allocate %zu bytes", words * sizeof(double));
  c->grid = d;
  // [B | E | t | x | y | z]: the snapshot arrays first keep them 256-byte aligned
  double* dB = d;
  double* dE = E ? d + 3 * nodes : nullptr;
  double* da = d + 3 * nodes * (E ? 2 : 1);
  CK(cudaMemcpy(dB, B, 3 * nodes * sizeof(double), cudaMemcpyHostToDevice));
  if (E) CK(cudaMemcpy(dE, E, 3 * nodes * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(da, t, nt * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(da + nt, x, nx * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(da + nt + nx, y, ny * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(da + nt + nx + ny, z, nz * sizeof(double), cudaMemcpyHostToDevice));
  FieldP& g = c->grid_desc;
  g.gB = dB; g.gE = dE;
  g.gt = da; g.gx = da + nt; g.gy = da + nt + nx; g.gz = da + nt + nx + ny;
  g.nt = nt; g.nx = nx; g.ny = ny; g.nz = nz;
  // cell guesses of uniform axes (checked on the device against the axis values)
  const double* ax[4] = {t, x, y, z};
  const int an[4] = {nt, nx, ny, nz};
  for (int a = 0; a < 4; ++a) g.ginv[a] = an[a] > 1 ? (an[a] - 1) / (ax[a][an[a] - 1] - ax[a][0]) : 0.0;
  build_field(RAPT_GRID, nullptr, 0, &c->field);
  attach_grid(g, &c->field);
  finish_field(&c->field);
  c->field_set = true;
  return RAPT_OK;
}

int rapt_config_set(void* ctx, const rapt_config* g) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || !g) return RAPT_ERR_INVALID;
  if (!(g->rtol >= 0) || !(g->atol >= 0) || g->nsteps <= 0 || !(g->cyclotronresolution > 0))
    return fail(c, RAPT_ERR_INVALID, "bad tolerances, nsteps or cyclotronresolution");
  if (g->tableau < 0 || g->tableau > 1) return fail(c, RAPT_ERR_INVALID, "tableau must be 0 or 1");
  if (g->gc_eom < 0 || g->gc_eom > 2) return fail(c, RAPT_ERR_INVALID, "gc_eom must be 0, 1 or 2");
  if (g->form < RAPT_FORM_PLAIN || g->form > RAPT_FORM_LEARNED_FP32)
    return fail(c, RAPT_ERR_UNSUPPORTED, "form %d not available", g->form);
  if ((g->form == RAPT_FORM_FP32 || g->form == RAPT_FORM_LEARNED_FP32) && (g->tableau != 0 || g->gc_eom != 0))
    return fail(c, RAPT_ERR_UNSUPPORTED, "the FP32 form runs DOP853/DOPRI5 with the Tao-Chan-Brizard equations");
  if ((g->form == RAPT_FORM_LEARNED || g->form == RAPT_FORM_LEARNED_FP32 || g->collect) && g->tableau != 0)
    return fail(c, RAPT_ERR_UNSUPPORTED, "the step learner drives the DOPRI5 controller (tableau 0)");
  if (!(g->learned_scale >= 0)) return fail(c, RAPT_ERR_INVALID, "learned_scale must be >= 0");
  if (g->learned_every < 0) return fail(c, RAPT_ERR_INVALID, "learned_every must be >= 0");
  if (!(g->gctimestep >= 0)) return fail(c, RAPT_ERR_INVALID, "GCtimestep must be >= 0");
  if (g->dense_output && (g->form != RAPT_FORM_PLAIN || g->tableau != 0 || g->collect))
    return fail(c, RAPT_ERR_UNSUPPORTED, "dense output runs the plain FP64 DOPRI5 guiding-centre kernel");
  if (g->gctimestep == 0 && !(g->bounceresolution > 0 && g->fieldlineresolution > 0))
    return fail(c, RAPT_ERR_INVALID, "bounceresolution and fieldlineresolution must be > 0");
  c->cfg = *g;
  return RAPT_OK;
}

int rapt_ensemble_alloc(void* ctx, int64_t n, int32_t max_rows, int32_t max_switch) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  if (n <= 0 || max_rows < 2 || max_switch < 0) return fail(c, RAPT_ERR_INVALID, "bad ensemble size");
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  cudaFree(c->block);
  c->block = nullptr;
  cudaFree(c->ord_block);
  c->ord_block = nullptr;
  c->n = 0;
  if (n > 0x7fffffffLL) return fail(c, RAPT_ERR_INVALID, "at most 2^31 - 1 tracers per ensemble");
  {
    // queue-order buffers: keys and indices in and out, step totals, sort storage
    const size_t N = (size_t)n;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    size_t cub_bytes = 0;
    CK(cub::DeviceRadixSort::SortPairsDescending(nullptr, cub_bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr,
                                                 (const int32_t*)nullptr, (int32_t*)nullptr, (int)n));
    const size_t ob = 4 * al(N * 4) + al(N * 8) + al(cub_bytes);
    if (cudaMalloc(&c->ord_block, ob) != cudaSuccess) {
      cudaGetLastError();
      return fail(c, RAPT_ERR_NOMEM, "cudaMalloc(%zu bytes) for the queue order failed", ob);
    }
    CK(cudaMemsetAsync(c->ord_block, 0, ob, c->stream));
    char* q = static_cast<char*>(c->ord_block);
    c->ord_key_in = carve<uint32_t>(q, N);
    c->ord_key_out = carve<uint32_t>(q, N);
    c->ord_idx_in = carve<int32_t>(q, N);
    c->ord = carve<int32_t>(q, N);
    c->ord_steps = carve<int64_t>(q, N);
    c->ord_tmp = q;
    c->ord_tmp_bytes = cub_bytes;
  }
  const size_t bytes = ensemble_bytes(n, max_rows, max_switch);
  if (cudaMalloc(&c->block, bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(c, RAPT_ERR_NOMEM, "cudaMalloc(%zu bytes) failed", bytes);
  }
  CK(cudaMemsetAsync(c->block, 0, bytes, c->stream));
  char* p = static_cast<char*>(c->block);
  DevEnsemble& E = c->E;
  const size_t N = (size_t)n;
  E.n = n;
  E.mode = carve<int8_t>(p, N);
  E.seg_active = carve<int8_t>(p, N);
  E.row_mode = carve<int8_t>(p, N * max_rows);
  E.sw_mode = carve<int8_t>(p, N * max_switch);
  E.status = carve<int32_t>(p, N);
  E.flags = carve<int32_t>(p, N);
  E.nrows = carve<int32_t>(p, N);
  E.nswitch = carve<int32_t>(p, N);
  E.nseg = carve<int32_t>(p, N);
  E.t_int = carve<double>(p, N);
  E.t_row = carve<double>(p, N);
  E.tcur = carve<double>(p, N);
  for (int i = 0; i < 6; ++i) E.s[i] = carve<double>(p, N);
  E.mu = carve<double>(p, N);
  E.v = carve<double>(p, N);
  E.mass = carve<double>(p, N);
  E.charge = carve<double>(p, N);
  E.delta = carve<double>(p, N);
  E.seg_stop = carve<double>(p, N);
  E.seg_dt = carve<double>(p, N);
  E.seg_gm = carve<double>(p, N);
  E.carry_h = carve<double>(p, N);
  E.carry_fac = carve<double>(p, N);
  E.carry_nst = carve<double>(p, N);
  E.rows = carve<double>(p, N * max_rows * 7);
  E.sw_time = carve<double>(p, N * max_switch);
  E.naccept = carve<int64_t>(p, N);
  E.nreject = carve<int64_t>(p, N);
  E.nfcn = carve<int64_t>(p, N);
  E.order = nullptr;  // index order until the first advance sorts the queue
  c->n = n;
  c->max_rows = max_rows;
  c->max_sw = max_switch;
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

int rapt_ensemble_upload(void* ctx, const rapt_host_state* h) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || !h) return RAPT_ERR_INVALID;
  if (c->n == 0) return fail(c, RAPT_ERR_STATE, "no ensemble allocated");
  if (h->n != c->n) return fail(c, RAPT_ERR_INVALID, "n %lld != allocated %lld", (long long)h->n, (long long)c->n);
  if (!h->mode || !h->t_row || !h->s[0] || !h->s[1] || !h->s[2] || !h->s[3] || !h->mass || !h->charge)
    return fail(c, RAPT_ERR_INVALID, "mode, t_row, s[0..3], mass and charge are required");
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)c->n;
  DevEnsemble& E = c->E;
  cudaStream_t s = c->stream;
  auto up = [&](void* d, const void* hp, size_t bytes) -> cudaError_t {
    if (hp) return cudaMemcpyAsync(d, hp, bytes, cudaMemcpyHostToDevice, s);
    return cudaMemsetAsync(d, 0, bytes, s);
  };
  CK(up(E.mode, h->mode, N));
  CK(up(E.status, h->status, N * 4));
  CK(up(E.flags, h->flags, N * 4));
  CK(up(E.t_row, h->t_row, N * 8));
  CK(up(E.t_int, h->t_int, N * 8));
  CK(up(E.tcur, h->tcur, N * 8));
  for (int i = 0; i < 6; ++i) CK(up(E.s[i], h->s[i], N * 8));
  CK(up(E.mu, h->mu, N * 8));
  CK(up(E.v, h->v, N * 8));
  CK(up(E.mass, h->mass, N * 8));
  CK(up(E.charge, h->charge, N * 8));
  CK(up(E.naccept, h->naccept, N * 8));
  CK(up(E.nreject, h->nreject, N * 8));
  CK(up(E.nfcn, h->nfcn, N * 8));
  CK(up(E.nswitch, h->nswitch, N * 4));
  CK(cudaMemsetAsync(E.nrows, 0, N * 4, s));
  k_fill_defaults<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(E, h->t_int != nullptr, h->tcur != nullptr);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  return RAPT_OK;
}

int rapt_ensemble_download(void* ctx, rapt_host_state* h) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || !h) return RAPT_ERR_INVALID;
  if (c->n == 0) return fail(c, RAPT_ERR_STATE, "no ensemble allocated");
  if (h->n != c->n) return fail(c, RAPT_ERR_INVALID, "n mismatch");
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)c->n;
  DevEnsemble& E = c->E;
  cudaStream_t s = c->stream;
  auto dn = [&](void* hp, const void* d, size_t bytes) -> cudaError_t {
    return hp ? cudaMemcpyAsync(hp, d, bytes, cudaMemcpyDeviceToHost, s) : cudaSuccess;
  };
  CK(dn(h->mode, E.mode, N));
  CK(dn(h->status, E.status, N * 4));
  CK(dn(h->flags, E.flags, N * 4));
  CK(dn(h->t_int, E.t_int, N * 8));
  CK(dn(h->t_row, E.t_row, N * 8));
  CK(dn(h->tcur, E.tcur, N * 8));
  for (int i = 0; i < 6; ++i) CK(dn(h->s[i], E.s[i], N * 8));
  CK(dn(h->mu, E.mu, N * 8));
  CK(dn(h->v, E.v, N * 8));
  CK(dn(h->mass, E.mass, N * 8));
  CK(dn(h->charge, E.charge, N * 8));
  CK(dn(h->naccept, E.naccept, N * 8));
  CK(dn(h->nreject, E.nreject, N * 8));
  CK(dn(h->nfcn, E.nfcn, N * 8));
  CK(dn(h->nswitch, E.nswitch, N * 4));
  CK(cudaStreamSynchronize(s));
  return RAPT_OK;
}

int rapt_rows_download(void* ctx, double* rows, int8_t* row_mode, int32_t* nrows, double* sw_time, int8_t* sw_mode,
                       int reset) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  if (c->n == 0) return fail(c, RAPT_ERR_STATE, "no ensemble allocated");
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)c->n;
  DevEnsemble& E = c->E;
  cudaStream_t s = c->stream;
  if (rows) CK(cudaMemcpyAsync(rows, E.rows, N * c->max_rows * 7 * 8, cudaMemcpyDeviceToHost, s));
  if (row_mode) CK(cudaMemcpyAsync(row_mode, E.row_mode, N * c->max_rows, cudaMemcpyDeviceToHost, s));
  if (nrows) CK(cudaMemcpyAsync(nrows, E.nrows, N * 4, cudaMemcpyDeviceToHost, s));
  if (sw_time && c->max_sw) CK(cudaMemcpyAsync(sw_time, E.sw_time, N * c->max_sw * 8, cudaMemcpyDeviceToHost, s));
  if (sw_mode && c->max_sw) CK(cudaMemcpyAsync(sw_mode, E.sw_mode, N * c->max_sw, cudaMemcpyDeviceToHost, s));
  if (reset) {
    CK(cudaMemsetAsync(E.nrows, 0, N * 4, s));
    CK(cudaMemsetAsync(E.nswitch, 0, N * 4, s));
  }
  CK(cudaStreamSynchronize(s));
  return RAPT_OK;
}

__global__ void k_clear_rows_full(DevEnsemble E) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < E.n && E.status[k] == RAPT_ST_ROWS_FULL) E.status[k] = RAPT_ST_OK;
}

static int advance_impl(Ctx* c, int kind, const double* delta, double delta_all, rapt_stats* stats, bool resume);

// The ensemble restricted to tracer k (every per-tracer array offset by k, n = 1).
static DevEnsemble ensemble_view(const DevEnsemble& E, int64_t k, int max_rows, int max_sw) {
  DevEnsemble V = E;
  V.n = 1;
  V.mode += k; V.status += k; V.flags += k; V.t_int += k; V.t_row += k; V.tcur += k;
  for (int i = 0; i < 6; ++i) V.s[i] += k;
  V.mu += k; V.v += k; V.mass += k; V.charge += k;
  V.naccept += k; V.nreject += k; V.nfcn += k; V.nswitch += k;
  V.delta += k; V.seg_stop += k; V.seg_dt += k; V.seg_gm += k; V.seg_active += k; V.nseg += k;
  V.carry_h += k; V.carry_fac += k; V.carry_nst += k;
  V.rows += (size_t)k * max_rows * 7;
  V.row_mode += (size_t)k * max_rows;
  V.nrows += k;
  V.sw_time += (size_t)k * max_sw;
  V.sw_mode += (size_t)k * max_sw;
  V.order = nullptr;
  return V;
}

int rapt_advance(void* ctx, int kind, const double* delta, double delta_all, rapt_stats* stats) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  return advance_impl(c, kind, delta, delta_all, stats, false);
}

int rapt_advance_resume(void* ctx, int kind, rapt_stats* stats) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  return advance_impl(c, kind, nullptr, 0.0, stats, true);
}

// Sort keys of the work queue: the RK attempts each tracer took in the previous
// call (its step totals minus those at the start of that call), or, where none
// are recorded (first call, state re-uploaded), an estimate from the state:
// 1000 v / |x|, the transit rate that sets a guiding centre's steps.
__global__ void k_order_keys(DevEnsemble E, int64_t* steps_prev, uint32_t* key, int32_t* idx) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= E.n) return;
  const int64_t tot = E.naccept[k] + E.nreject[k];
  const int64_t d = tot - steps_prev[k];
  steps_prev[k] = tot;
  uint32_t v;
  if (d > 0) {
    v = (uint32_t)min(d, (int64_t)0x7fffffff);
  } else {
    const double r = sqrt(E.s[0][k] * E.s[0][k] + E.s[1][k] * E.s[1][k] + E.s[2][k] * E.s[2][k]);
    double speed = E.v[k];
    if (E.mode[k] == RAPT_MODE_PARTICLE) {
      const double p2 = E.s[3][k] * E.s[3][k] + E.s[4][k] * E.s[4][k] + E.s[5][k] * E.s[5][k];
      speed = sqrt(p2) / sqrt(E.mass[k] * E.mass[k] + p2 / (kC * kC));
    }
    const double est = r > 0.0 ? 1000.0 * speed / r : 0.0;
    v = (est >= 0.0 && est < 2.0e9) ? (uint32_t)est : 2000000000u;
  }
  key[k] = v;
  idx[k] = (int32_t)k;
}

static int advance_impl(Ctx* c, int kind, const double* delta, double delta_all, rapt_stats* stats, bool resume) {
  if (!c->field_set) return fail(c, RAPT_ERR_STATE, "no field set");
  if (c->n == 0) return fail(c, RAPT_ERR_STATE, "no ensemble allocated");
  if (kind < RAPT_KIND_PARTICLE || kind > RAPT_KIND_ADAPTIVE) return fail(c, RAPT_ERR_INVALID, "bad kind");
  if (!resume && !delta && !std::isfinite(delta_all)) return fail(c, RAPT_ERR_INVALID, "delta must be finite");
  CK(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  DevEnsemble& E = c->E;
  const size_t N = (size_t)c->n;
  double* d_delta = nullptr;
  if (delta) {
    if (c->tmp_bytes < N * 8) {
      cudaFree(c->tmp);
      c->tmp = nullptr;
      c->tmp_bytes = 0;
      CK(cudaMalloc(&c->tmp, N * 8));
      c->tmp_bytes = N * 8;
    }
    d_delta = static_cast<double*>(c->tmp);
    CK(cudaMemcpyAsync(d_delta, delta, N * 8, cudaMemcpyHostToDevice, s));
  }
  KParams P = make_params(c, kind);
  const ModelTable& T = c->tab[c->field.model];
  const int tab = c->cfg.tableau;
  const int block = c->cfg.threads_per_block > 0 ? c->cfg.threads_per_block : 128;
  if (block % 32 != 0 || block > 128) return fail(c, RAPT_ERR_INVALID, "threads_per_block must be a multiple of 32, <= 128");
  const int form = c->cfg.form;
  const bool f32 = form == RAPT_FORM_FP32 || form == RAPT_FORM_LEARNED_FP32;
  const bool learned = form == RAPT_FORM_LEARNED || form == RAPT_FORM_LEARNED_FP32;
  const int lrn = learned ? 2 : (c->cfg.collect ? 1 : 0);
  if (learned && !c->mlp_ready) return fail(c, RAPT_ERR_STATE, "learned form without MLP parameters (rapt_mlp_set_params)");
  if (c->cfg.collect && !c->samp)
    return fail(c, RAPT_ERR_STATE, "collection without a sample buffer (rapt_mlp_samples_reserve)");
  // the step learner drives the guiding-centre kernels; particles run the plain controller
  int bps_p = f32 ? T.occ_particle32(block) : T.occ_particle[tab](block);
  const bool dense = c->cfg.dense_output != 0;
  if (dense && kind != RAPT_KIND_PARTICLE && c->max_rows < 18)
    return fail(c, RAPT_ERR_INVALID, "dense output needs max_rows >= 18 (a step may cover 17 output times)");
  int bps_g = dense ? T.occ_gc_dense(block)
                    : (tab != 0 ? T.occ_gc[tab](block) : (f32 ? T.occ_gc32_lrn[lrn](block) : T.occ_gc_lrn[lrn](block)));
  if (c->cfg.blocks_per_sm > 0) {
    bps_p = std::min(bps_p, c->cfg.blocks_per_sm);
    bps_g = std::min(bps_g, c->cfg.blocks_per_sm);
  }
  if (bps_p < 1 || bps_g < 1) return fail(c, RAPT_ERR_CUDA, "kernel does not fit on an SM");
  if (kind != RAPT_KIND_PARTICLE && c->cfg.gctimestep == 0) {
    // bounce-period cadence: one field-line scratch slot per guiding-centre thread
    const size_t threads = c->cfg.per_tracer_launches ? 32 : (size_t)c->num_sms * bps_g * block;
    const size_t bytes = threads * (size_t)P.fl_stride * sizeof(double);
    if (c->fl_bytes < bytes) {
      cudaFree(c->fl_scratch);
      c->fl_scratch = nullptr;
      c->fl_bytes = 0;
      if (cudaMalloc(&c->fl_scratch, bytes) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, RAPT_ERR_NOMEM, "cudaMalloc(%zu bytes) for field-line traces failed", bytes);
      }
      c->fl_bytes = bytes;
    }
    P.fl_scratch = c->fl_scratch;
  }

  CK(cudaEventRecord(c->ev0, s));
  if (resume) k_clear_rows_full<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(E);
  else k_prepare<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(E, d_delta, delta_all, kind);
  CK(cudaGetLastError());
  if (!resume && !c->cfg.per_tracer_launches) {
    // queue order for this call: longest expected work first (a resumed call
    // keeps the order of the call it continues)
    k_order_keys<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(E, c->ord_steps, c->ord_key_in, c->ord_idx_in);
    CK(cudaGetLastError());
    size_t tb = c->ord_tmp_bytes;
    CK(cub::DeviceRadixSort::SortPairsDescending(c->ord_tmp, tb, c->ord_key_in, c->ord_key_out, c->ord_idx_in,
                                                 c->ord, (int)c->n, 0, 32, s));
    E.order = c->ord;
  }
  CK(cudaMemsetAsync(c->scratch, 0, sizeof(Scratch), s));
  int64_t launches = 0, kl = 1;
  const int max_rounds = 1000000;
  int round = 0;
  // one round: reset the queue heads and the pending count, run the particle
  // kernel and the guiding-centre kernel over the ensemble view Ev
  auto enqueue_round = [&](const DevEnsemble& Ev, int grid_p, int grid_g, int blk) -> int {
    CK(cudaMemsetAsync(c->scratch, 0, 3 * sizeof(unsigned long long), s));  // queue[2], pending
    LaunchArgs a{Ev, P, c->scratch, 0, blk, s};
    if (kind != RAPT_KIND_GC) {
      a.grid = grid_p;
      CK(f32 ? T.particle32(a) : T.particle[tab](a));
      ++kl;
    }
    if (kind != RAPT_KIND_PARTICLE) {
      a.grid = grid_g;
      CK(dense ? T.gc_dense(a) : (tab != 0 ? T.gc[tab](a) : (f32 ? T.gc32_lrn[lrn](a) : T.gc_lrn[lrn](a))));
      ++kl;
    }
    return RAPT_OK;
  };
  auto read_pending = [&]() -> int {
    CK(cudaMemcpyAsync(c->h_pending, &c->scratch->pending, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    return RAPT_OK;
  };
  if (c->cfg.per_tracer_launches) {
    // the unbatched pattern: every tracer gets its own launches (one warp),
    // rounds repeated until it is done -- for comparison with the batched grid
    for (int64_t k = 0; k < c->n; ++k) {
      const DevEnsemble Ek = ensemble_view(E, k, c->max_rows, c->max_sw);
      for (round = 0; round < max_rounds; ++round) {
        int rc = enqueue_round(Ek, 1, 1, 32);
        if (rc) return rc;
        ++launches;
        rc = read_pending();
        if (rc) return rc;
        CK(cudaStreamSynchronize(s));
        if (*c->h_pending == 0) break;
      }
      if (round >= max_rounds) break;
    }
  } else if (c->cfg.use_graph) {
    // capture kGraphRounds rounds and the pending read-back once, replay until done
    constexpr int kGraphRounds = 4;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int rc = RAPT_OK;
    const int64_t kl0 = kl;
    for (int r = 0; r < kGraphRounds && rc == RAPT_OK; ++r)
      rc = enqueue_round(E, c->num_sms * bps_p, c->num_sms * bps_g, block);
    if (rc == RAPT_OK) rc = read_pending();
    cudaError_t ec = cudaStreamEndCapture(s, &graph);
    if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
    if (ec != cudaSuccess) return fail(c, RAPT_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ec));
    ec = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ec != cudaSuccess) return fail(c, RAPT_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ec));
    const int64_t per_replay = kl - kl0;
    kl = kl0;
    for (round = 0; round < max_rounds; round += kGraphRounds) {
      ec = cudaGraphLaunch(exec, s);
      if (ec == cudaSuccess) ec = cudaStreamSynchronize(s);
      if (ec != cudaSuccess) { cudaGraphExecDestroy(exec); return fail(c, RAPT_ERR_CUDA, "graph launch: %s", cudaGetErrorString(ec)); }
      launches += kGraphRounds;
      kl += per_replay;
      if (*c->h_pending == 0) break;
    }
    cudaGraphExecDestroy(exec);
  } else {
    for (; round < max_rounds; ++round) {
      int rc = enqueue_round(E, c->num_sms * bps_p, c->num_sms * bps_g, block);
      if (rc) return rc;
      ++launches;
      rc = read_pending();
      if (rc) return rc;
      CK(cudaStreamSynchronize(s));
      if (*c->h_pending == 0) break;
    }
  }
  CK(cudaEventRecord(c->ev1, s));
  Scratch hs;
  CK(cudaMemcpyAsync(&hs, c->scratch, sizeof(Scratch), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (stats) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    stats->accepted = (int64_t)hs.accepted;
    stats->rejected = (int64_t)hs.rejected;
    stats->rhs_evals = (int64_t)hs.rhs;
    stats->switches = (int64_t)hs.switches;
    stats->done = (int64_t)hs.done;
    stats->failed = (int64_t)hs.failed;
    stats->launches = launches;
    stats->kernel_launches = kl;
    stats->kernel_ms = ms;
  }
  if (round >= max_rounds) return fail(c, RAPT_ERR_STATE, "advance did not finish in %d rounds", max_rounds);
  return RAPT_OK;
}

int rapt_adaptive_init(void* ctx) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  if (!c->field_set || c->n == 0) return fail(c, RAPT_ERR_STATE, "field and ensemble required");
  CK(cudaSetDevice(c->device));
  const KParams P = make_params(c, RAPT_KIND_ADAPTIVE);
  CK(c->tab[c->field.model].adaptive_init(c->E, P, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

static int ensure_tmp(Ctx* c, size_t bytes) {
  if (c->tmp_bytes >= bytes) return RAPT_OK;
  cudaFree(c->tmp);
  c->tmp = nullptr;
  c->tmp_bytes = 0;
  CK(cudaMalloc(&c->tmp, bytes));
  c->tmp_bytes = bytes;
  return RAPT_OK;
}

int rapt_field_eval(void* ctx, int what, int64_t n, const double* tpos, double* out) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || n < 0 || (n > 0 && (!tpos || !out))) return RAPT_ERR_INVALID;
  if (!c->field_set) return fail(c, RAPT_ERR_STATE, "no field set");
  if (what < 0 || what > 10) return fail(c, RAPT_ERR_INVALID, "bad quantity %d", what);
  if (n == 0) return RAPT_OK;
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)n;
  int rc = ensure_tmp(c, N * 13 * 8);
  if (rc) return rc;
  double* d_in = static_cast<double*>(c->tmp);
  double* d_out = d_in + 4 * N;
  CK(cudaMemcpyAsync(d_in, tpos, N * 32, cudaMemcpyHostToDevice, c->stream));
  CK(c->tab[c->field.model].field_eval(c->field, what, n, d_in, d_out, c->stream));
  CK(cudaMemcpyAsync(out, d_out, N * 72, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

int rapt_rhs_eval(void* ctx, int mode, int64_t n, const double* state, const double* mass, const double* charge,
                  const double* v, double* out) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || n < 0 || (n > 0 && (!state || !mass || !charge || !out))) return RAPT_ERR_INVALID;
  if (!c->field_set) return fail(c, RAPT_ERR_STATE, "no field set");
  if (mode == RAPT_MODE_GC && !v) return fail(c, RAPT_ERR_INVALID, "GC needs v");
  if (n == 0) return RAPT_OK;
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)n;
  int rc = ensure_tmp(c, N * 17 * 8);
  if (rc) return rc;
  double* d = static_cast<double*>(c->tmp);
  double *d_state = d, *d_mass = d + 8 * N, *d_charge = d + 9 * N, *d_v = d + 10 * N, *d_out = d + 11 * N;
  CK(cudaMemcpyAsync(d_state, state, N * 64, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(d_mass, mass, N * 8, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(d_charge, charge, N * 8, cudaMemcpyHostToDevice, c->stream));
  if (v) CK(cudaMemcpyAsync(d_v, v, N * 8, cudaMemcpyHostToDevice, c->stream));
  else CK(cudaMemsetAsync(d_v, 0, N * 8, c->stream));
  const KParams P = make_params(c, RAPT_KIND_PARTICLE);
  CK(c->tab[c->field.model].rhs_eval(P, mode, n, d_state, d_mass, d_charge, d_v, d_out, c->stream));
  CK(cudaMemcpyAsync(out, d_out, N * 48, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

static int mlp_ensure(Ctx* c) {
  if (c->mlp_block) return RAPT_OK;
  const size_t fl = (size_t)RAPT_MLP_NPARAMS * 4;
  const size_t packed = ((size_t)kMlpPackedWords * 4 + 255) & ~size_t(255);
  // parameters, Adam moments, gradient, loss words, packed weights, then the
  // per-block gradient and loss partials of the deterministic reduction
  const size_t bytes = 4 * fl + 256 + packed + (size_t)kMlpTrainMaxBlocks * kMlpGaccWords * 4 +
                       (size_t)kMlpTrainMaxBlocks * 2 * 8;
  CK(cudaMalloc(&c->mlp_block, bytes));
  CK(cudaMemsetAsync(c->mlp_block, 0, bytes, c->stream));
  char* p = static_cast<char*>(c->mlp_block);
  c->mlp_p = reinterpret_cast<float*>(p);
  c->mlp_m = reinterpret_cast<float*>(p + fl);
  c->mlp_v = reinterpret_cast<float*>(p + 2 * fl);
  c->mlp_g = reinterpret_cast<float*>(p + 3 * fl);
  c->mlp_loss = reinterpret_cast<double*>(p + 4 * fl);
  c->mlp_w = reinterpret_cast<uint32_t*>(p + 4 * fl + 256);
  c->mlp_partial = reinterpret_cast<float*>(p + 4 * fl + 256 + packed);
  c->mlp_lpart = reinterpret_cast<double*>(p + 4 * fl + 256 + packed + (size_t)kMlpTrainMaxBlocks * kMlpGaccWords * 4);
  return RAPT_OK;
}

int rapt_mlp_set_params(void* ctx, const float* params, int32_t n) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || !params) return RAPT_ERR_INVALID;
  if (n != RAPT_MLP_NPARAMS) return fail(c, RAPT_ERR_INVALID, "expected %d parameters, got %d", RAPT_MLP_NPARAMS, n);
  for (int i = RAPT_MLP_NTRAIN + 16; i < RAPT_MLP_NTRAIN + 32; ++i)
    if (!(params[i] != 0.f) || !std::isfinite(params[i])) return fail(c, RAPT_ERR_INVALID, "feature scales must be finite and nonzero");
  if (!(params[RAPT_MLP_NTRAIN + 40] != 0.f) || !(params[RAPT_MLP_NTRAIN + 41] != 0.f))
    return fail(c, RAPT_ERR_INVALID, "target scales must be nonzero");
  CK(cudaSetDevice(c->device));
  int rc = mlp_ensure(c);
  if (rc) return rc;
  const size_t fl = (size_t)RAPT_MLP_NPARAMS * 4;
  CK(cudaMemcpyAsync(c->mlp_p, params, fl, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->mlp_m, 0, 2 * fl, c->stream));
  c->mlp_t = 0;
  CK(mlp_pack(c->mlp_p, c->mlp_w, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->mlp_ready = true;
  return RAPT_OK;
}

int rapt_mlp_get_params(void* ctx, float* params, int32_t n) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || !params) return RAPT_ERR_INVALID;
  if (n != RAPT_MLP_NPARAMS) return fail(c, RAPT_ERR_INVALID, "expected %d parameters, got %d", RAPT_MLP_NPARAMS, n);
  if (!c->mlp_ready) return fail(c, RAPT_ERR_STATE, "no MLP parameters set");
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(params, c->mlp_p, (size_t)n * 4, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

int rapt_mlp_forward(void* ctx, const float* features, int64_t n, float* out) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || n < 0 || (n > 0 && (!features || !out))) return RAPT_ERR_INVALID;
  if (!c->mlp_ready) return fail(c, RAPT_ERR_STATE, "no MLP parameters set");
  if (n == 0) return RAPT_OK;
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)n;
  int rc = ensure_tmp(c, N * 18 * 4);
  if (rc) return rc;
  float* d_in = static_cast<float*>(c->tmp);
  float* d_out = d_in + 16 * N;
  CK(cudaMemcpyAsync(d_in, features, N * 64, cudaMemcpyHostToDevice, c->stream));
  CK(mlp_forward(c->mlp_w, c->mlp_p, d_in, n, d_out, c->num_sms, c->stream));
  CK(cudaMemcpyAsync(out, d_out, N * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

int rapt_mlp_grad(void* ctx, const float* samples, int64_t n, float switch_weight, float* grad, double* loss) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || n <= 0 || !samples || !grad) return RAPT_ERR_INVALID;
  if (!c->mlp_ready) return fail(c, RAPT_ERR_STATE, "no MLP parameters set");
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)n;
  int rc = ensure_tmp(c, N * RAPT_MLP_SAMPLE * 4);
  if (rc) return rc;
  float* d_s = static_cast<float*>(c->tmp);
  CK(cudaMemcpyAsync(d_s, samples, N * RAPT_MLP_SAMPLE * 4, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->mlp_g, 0, (size_t)RAPT_MLP_NTRAIN * 4, c->stream));
  CK(cudaMemsetAsync(c->mlp_loss, 0, 16, c->stream));
  CK(mlp_grad(d_s, n, n, 0, 0, 0, switch_weight, c->mlp_w, c->mlp_p, c->mlp_g, c->mlp_loss, c->mlp_partial,
              c->mlp_lpart, c->stream));
  CK(cudaMemcpyAsync(grad, c->mlp_g, (size_t)RAPT_MLP_NTRAIN * 4, cudaMemcpyDeviceToHost, c->stream));
  double hl[2];
  CK(cudaMemcpyAsync(hl, c->mlp_loss, 16, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (loss) { loss[0] = hl[0]; loss[1] = hl[1]; }
  return RAPT_OK;
}

int rapt_mlp_samples_reserve(void* ctx, int64_t capacity, uint64_t mask) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || capacity <= 0) return RAPT_ERR_INVALID;
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (capacity != c->samp_cap) {
    cudaFree(c->samp_count);  // base of the sample allocation
    c->samp = nullptr;
    c->samp_cap = 0;
    c->samp_count = nullptr;
    const size_t bytes = 256 + (size_t)capacity * RAPT_MLP_SAMPLE * 4;
    void* b = nullptr;
    if (cudaMalloc(&b, bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(c, RAPT_ERR_NOMEM, "cudaMalloc(%zu bytes) for samples failed", bytes);
    }
    c->samp_count = static_cast<unsigned long long*>(b);
    c->samp = reinterpret_cast<float*>(static_cast<char*>(b) + 256);
    c->samp_cap = capacity;
  }
  c->samp_mask = mask;
  CK(cudaMemsetAsync(c->samp_count, 0, 8, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

static int samples_count(Ctx* c, int64_t* count) {
  unsigned long long k = 0;
  CK(cudaMemcpyAsync(&k, c->samp_count, 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *count = (int64_t)std::min<unsigned long long>(k, (unsigned long long)c->samp_cap);
  return RAPT_OK;
}

int rapt_mlp_samples_count(void* ctx, int64_t* count) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || !count) return RAPT_ERR_INVALID;
  if (!c->samp) { *count = 0; return RAPT_OK; }
  CK(cudaSetDevice(c->device));
  return samples_count(c, count);
}

int rapt_mlp_samples_download(void* ctx, float* out, int64_t first, int64_t n) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || first < 0 || n < 0 || (n > 0 && !out)) return RAPT_ERR_INVALID;
  if (!c->samp) return fail(c, RAPT_ERR_STATE, "no sample buffer");
  CK(cudaSetDevice(c->device));
  int64_t cnt = 0;
  int rc = samples_count(c, &cnt);
  if (rc) return rc;
  if (first + n > cnt) return fail(c, RAPT_ERR_INVALID, "samples [%lld, %lld) beyond the %lld held", (long long)first,
                                   (long long)(first + n), (long long)cnt);
  if (n == 0) return RAPT_OK;
  CK(cudaMemcpyAsync(out, c->samp + (size_t)first * RAPT_MLP_SAMPLE, (size_t)n * RAPT_MLP_SAMPLE * 4,
                     cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

int rapt_mlp_samples_upload(void* ctx, const float* samples, int64_t n) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || n <= 0 || !samples) return RAPT_ERR_INVALID;
  int rc = rapt_mlp_samples_reserve(ctx, std::max<int64_t>(n, c->samp_cap), c->samp_mask);
  if (rc) return rc;
  CK(cudaMemcpyAsync(c->samp, samples, (size_t)n * RAPT_MLP_SAMPLE * 4, cudaMemcpyHostToDevice, c->stream));
  const unsigned long long k = (unsigned long long)n;
  CK(cudaMemcpyAsync(c->samp_count, &k, 8, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

int rapt_mlp_samples_sort(void* ctx, int64_t first, int64_t n) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || first < 0 || n < 0) return RAPT_ERR_INVALID;
  if (!c->samp) return fail(c, RAPT_ERR_STATE, "no sample buffer");
  CK(cudaSetDevice(c->device));
  int64_t cnt = 0;
  int rc = samples_count(c, &cnt);
  if (rc) return rc;
  if (first + n > cnt) return fail(c, RAPT_ERR_INVALID, "samples [%lld, %lld) beyond the %lld held", (long long)first,
                                   (long long)(first + n), (long long)cnt);
  if (n > 0x7fffffffLL) return fail(c, RAPT_ERR_INVALID, "at most 2^31 - 1 samples per sort");
  if (n <= 1) return RAPT_OK;
  const size_t bytes = mlp_sort_tmp_bytes(n);
  void* tmp = nullptr;
  if (cudaMalloc(&tmp, bytes) != cudaSuccess) {
    cudaGetLastError();
    return fail(c, RAPT_ERR_NOMEM, "cudaMalloc(%zu bytes) for the sample sort failed", bytes);
  }
  const cudaError_t e = mlp_samples_sort(c->samp + (size_t)first * RAPT_MLP_SAMPLE, n, tmp, bytes, c->stream);
  const cudaError_t e2 = cudaStreamSynchronize(c->stream);
  cudaFree(tmp);
  if (e != cudaSuccess) return fail(c, RAPT_ERR_CUDA, "sample sort: %s", cudaGetErrorString(e));
  if (e2 != cudaSuccess) return fail(c, RAPT_ERR_CUDA, "sample sort: %s", cudaGetErrorString(e2));
  return RAPT_OK;
}

int rapt_mlp_train(void* ctx, int64_t steps, int32_t batch, float lr, float switch_weight, uint64_t seed,
                   double* loss) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || steps <= 0 || batch <= 0 || !(lr > 0) || !(switch_weight >= 0)) return RAPT_ERR_INVALID;
  if (!c->mlp_ready) return fail(c, RAPT_ERR_STATE, "no MLP parameters set");
  if (!c->samp) return fail(c, RAPT_ERR_STATE, "no samples");
  CK(cudaSetDevice(c->device));
  int64_t cnt = 0;
  int rc = samples_count(c, &cnt);
  if (rc) return rc;
  if (cnt <= 0) return fail(c, RAPT_ERR_STATE, "no samples");
  const int64_t tail = std::max<int64_t>(1, steps / 10);
  for (int64_t it = 0; it < steps; ++it) {
    if (it == steps - tail) CK(cudaMemsetAsync(c->mlp_loss, 0, 16, c->stream));
    CK(cudaMemsetAsync(c->mlp_g, 0, (size_t)RAPT_MLP_NTRAIN * 4, c->stream));
    CK(mlp_grad(c->samp, cnt, batch, 1, seed, c->mlp_t, switch_weight, c->mlp_w, c->mlp_p, c->mlp_g,
                it >= steps - tail ? c->mlp_loss : c->mlp_loss + 2, c->mlp_partial, c->mlp_lpart, c->stream));
    ++c->mlp_t;
    CK(mlp_adam(c->mlp_p, c->mlp_m, c->mlp_v, c->mlp_g, lr, c->mlp_t, c->stream));
    CK(mlp_pack(c->mlp_p, c->mlp_w, c->stream));
  }
  double hl[2];
  CK(cudaMemcpyAsync(hl, c->mlp_loss, 16, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  if (loss) { loss[0] = hl[0] / (double)tail; loss[1] = hl[1] / (double)tail; }
  return RAPT_OK;
}

int rapt_gc_bounce_period(void* ctx, int64_t n, const double* state, double* out) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || n < 0 || (n > 0 && (!state || !out))) return RAPT_ERR_INVALID;
  if (!c->field_set) return fail(c, RAPT_ERR_STATE, "no field set");
  if (n == 0) return RAPT_OK;
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)n;
  const long long stride = 8LL * kFieldlineCap;
  int rc = ensure_tmp(c, N * 8 * 8);
  if (rc) return rc;
  double* d_in = static_cast<double*>(c->tmp);
  double* d_out = d_in + 7 * N;
  // scratch for the traces: reuse the advance buffer when it is large enough
  const size_t need = N * (size_t)stride * sizeof(double);
  if (c->fl_bytes < need) {
    cudaFree(c->fl_scratch);
    c->fl_scratch = nullptr;
    c->fl_bytes = 0;
    if (cudaMalloc(&c->fl_scratch, need) != cudaSuccess) {
      cudaGetLastError();
      return fail(c, RAPT_ERR_NOMEM, "cudaMalloc(%zu bytes) for field-line traces failed", need);
    }
    c->fl_bytes = need;
  }
  CK(cudaMemcpyAsync(d_in, state, N * 7 * 8, cudaMemcpyHostToDevice, c->stream));
  CK(c->tab[c->field.model].bounce_period(c->field, c->cfg.fieldlineresolution, n, d_in, d_out, c->fl_scratch,
                                          stride, kFieldlineCap, c->stream));
  CK(cudaMemcpyAsync(out, d_out, N * 8, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return RAPT_OK;
}

// Per-thread field-line scratch for n concurrent traces (kFieldlineCap points per direction).
static int ensure_fl_scratch(Ctx* c, size_t n) {
  const size_t need = n * (size_t)(8LL * kFieldlineCap) * sizeof(double);
  if (c->fl_bytes >= need) return RAPT_OK;
  cudaFree(c->fl_scratch);
  c->fl_scratch = nullptr;
  c->fl_bytes = 0;
  if (cudaMalloc(&c->fl_scratch, need) != cudaSuccess) {
    cudaGetLastError();
    return fail(c, RAPT_ERR_NOMEM, "cudaMalloc(%zu bytes) for field-line traces failed", need);
  }
  c->fl_bytes = need;
  return RAPT_OK;
}

// BounceCenter passes. A first pass gives each thread a small trace slot
// (kBcCapSmall points per direction: 8 KB; the lines of the pitch angles where
// the reference's second-invariant integral runs have a few tens), 16,384
// tracers at a time, so that the slots (128 MiB) stay in L2; a tracer whose
// right-hand side met a non-finite value (a trace that did not fit, among
// others) is then rerun from its start with full slots (kFieldlineCap points,
// 64 KB), 2,048 at a time. The rerun reproduces a full-slot run exactly.
constexpr int kBcCapSmall = 128;
constexpr int64_t kBcChunkSmall = 16384, kBcChunkFull = 2048;

static int bc_pass(Ctx* c, int64_t n, double* state, const double* cst, double delta, double bctimestep,
                   double eyegradientstep, double* rows, int32_t max_rows, int32_t* nrows, int32_t* status,
                   int64_t* counters, int32_t* flagged, int cap, int64_t chunk_max) {
  const long long stride = 8LL * cap;
  const int64_t chunk = std::min<int64_t>(n, chunk_max);
  int rc = ensure_fl_scratch(c, (size_t)chunk * (size_t)cap / kFieldlineCap + 1);
  if (rc) return rc;
  KParams P = make_params(c, RAPT_KIND_GC);
  const ModelTable& T = c->tab[c->field.model];
  // device block per chunk: st 5 | cst 4 | plan 4 | counters 4 (int64) | status, nrows, flag (int32) | rows
  const size_t C = (size_t)chunk, R = (size_t)max_rows;
  rc = ensure_tmp(c, C * (17 * 8 + 4 * 4) + C * R * 4 * 8);
  if (rc) return rc;
  char* base = static_cast<char*>(c->tmp);
  double* d_st = reinterpret_cast<double*>(base);
  double* d_cst = d_st + 5 * C;
  double* d_plan = d_cst + 4 * C;
  int64_t* d_cnt = reinterpret_cast<int64_t*>(d_plan + 4 * C);
  int32_t* d_status = reinterpret_cast<int32_t*>(d_cnt + 4 * C);
  int32_t* d_nrows = d_status + C;
  int32_t* d_flag = d_nrows + C;
  double* d_rows = reinterpret_cast<double*>(d_flag + C + C);  // 17C doubles + 4C int32: 8-byte aligned
  std::vector<double> plan;
  for (int64_t k0 = 0; k0 < n; k0 += chunk) {
    const int64_t m = std::min(chunk, n - k0);
    const size_t M = (size_t)m;
    CK(cudaMemcpyAsync(d_st, state + 5 * k0, M * 5 * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_cst, cst + 4 * k0, M * 4 * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(d_cnt, 0, M * 4 * 8, c->stream));
    CK(cudaMemsetAsync(d_nrows, 0, M * 4, c->stream));
    CK(cudaMemsetAsync(d_flag, 0, M * 4, c->stream));
    CK(T.bc_start(c->field, c->cfg.fieldlineresolution, m, d_st, d_cst, delta, bctimestep, d_plan, d_status,
                  d_flag, c->fl_scratch, stride, cap, c->stream));
    plan.resize(M * 4);
    CK(cudaMemcpyAsync(plan.data(), d_plan, M * 4 * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    double kmax = 0.0;
    for (size_t i = 0; i < M; ++i) kmax = std::max(kmax, plan[4 * i + 2]);
    if (kmax > 1e7) return fail(c, RAPT_ERR_INVALID, "more than 1e7 rows per BounceCenter (delta / dt)");
    for (int64_t j = 0; j < (int64_t)kmax; ++j)
      CK(T.bc_interval(c->field, P, m, d_st, d_cst, d_plan, eyegradientstep, j, d_rows, max_rows, d_nrows, d_status,
                       d_cnt, d_flag, c->fl_scratch, stride, cap, c->stream));
    CK(cudaMemcpyAsync(state + 5 * k0, d_st, M * 5 * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(status + k0, d_status, M * 4, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(nrows + k0, d_nrows, M * 4, cudaMemcpyDeviceToHost, c->stream));
    if (flagged) CK(cudaMemcpyAsync(flagged + k0, d_flag, M * 4, cudaMemcpyDeviceToHost, c->stream));
    if (max_rows > 0)
      CK(cudaMemcpyAsync(rows + (size_t)k0 * R * 4, d_rows, M * R * 4 * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(counters + 4 * k0, d_cnt, M * 4 * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return RAPT_OK;
}

int rapt_bc_advance(void* ctx, int64_t n, double* state, const double* cst, double delta, double bctimestep,
                    double eyegradientstep, double* rows, int32_t max_rows, int32_t* nrows, int32_t* status,
                    int64_t* counters) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || n < 0 || (n > 0 && (!state || !cst || !nrows || !status)) || max_rows < 0 || (max_rows > 0 && !rows))
    return RAPT_ERR_INVALID;
  if (!c->field_set) return fail(c, RAPT_ERR_STATE, "no field set");
  if (!c->field.is_static)
    return fail(c, RAPT_ERR_UNSUPPORTED, "BounceCenter works with static fields only (BounceCenter.py:95-97)");
  if (!(bctimestep > 0) || !(eyegradientstep > 0) || !std::isfinite(delta))
    return fail(c, RAPT_ERR_INVALID, "bad BCtimestep, eyegradientstep or delta");
  if (n == 0) return RAPT_OK;
  CK(cudaSetDevice(c->device));
  const size_t N = (size_t)n, R = (size_t)max_rows;
  const std::vector<double> start(state, state + 5 * N);
  std::vector<int32_t> flagged(N, 0);
  std::vector<int64_t> cnt(4 * N, 0);
  int rc = bc_pass(c, n, state, cst, delta, bctimestep, eyegradientstep, rows, max_rows, nrows, status, cnt.data(),
                   flagged.data(), kBcCapSmall, kBcChunkSmall);
  if (rc) return rc;
  std::vector<int64_t> redo;
  for (size_t i = 0; i < N; ++i)
    if (flagged[i]) redo.push_back((int64_t)i);
  if (!redo.empty()) {
    const size_t m = redo.size();
    std::vector<double> st2(5 * m), cst2(4 * m), rows2(m * R * 4);
    std::vector<int32_t> nr2(m), status2(m);
    std::vector<int64_t> cnt2(4 * m);
    for (size_t a = 0; a < m; ++a) {
      std::memcpy(&st2[5 * a], &start[5 * redo[a]], 5 * 8);
      std::memcpy(&cst2[4 * a], cst + 4 * redo[a], 4 * 8);
    }
    rc = bc_pass(c, (int64_t)m, st2.data(), cst2.data(), delta, bctimestep, eyegradientstep,
                 R ? rows2.data() : nullptr, max_rows, nr2.data(), status2.data(), cnt2.data(), nullptr,
                 kFieldlineCap, kBcChunkFull);
    if (rc) return rc;
    for (size_t a = 0; a < m; ++a) {
      const size_t k = (size_t)redo[a];
      std::memcpy(state + 5 * k, &st2[5 * a], 5 * 8);
      if (R) std::memcpy(rows + k * R * 4, &rows2[a * R * 4], R * 4 * 8);
      nrows[k] = nr2[a];
      status[k] = status2[a];
      std::memcpy(&cnt[4 * k], &cnt2[4 * a], 4 * 8);
    }
  }
  if (counters) std::memcpy(counters, cnt.data(), 4 * N * 8);
  return RAPT_OK;
}

int rapt_bc_eval(void* ctx, int what, int64_t n, const double* tpos, const double* Bm, double eyegradientstep,
                 const double* cst, double* out) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c || what < 0 || what > 3 || n < 0 || (n > 0 && (!tpos || !Bm || !out || (what == 2 && !cst))))
    return RAPT_ERR_INVALID;
  if (!c->field_set) return fail(c, RAPT_ERR_STATE, "no field set");
  if (n == 0) return RAPT_OK;
  CK(cudaSetDevice(c->device));
  const long long stride = 8LL * kFieldlineCap;
  const int64_t chunk = std::min<int64_t>(n, kBcChunkFull);
  int rc = ensure_fl_scratch(c, (size_t)chunk);
  if (rc) return rc;
  const size_t C = (size_t)chunk;
  rc = ensure_tmp(c, C * 12 * 8);
  if (rc) return rc;
  double* d_tp = static_cast<double*>(c->tmp);
  double* d_bm = d_tp + 4 * C;
  double* d_cst = d_bm + C;
  double* d_out = d_cst + 4 * C;
  for (int64_t k0 = 0; k0 < n; k0 += chunk) {
    const int64_t m = std::min(chunk, n - k0);
    const size_t M = (size_t)m;
    CK(cudaMemcpyAsync(d_tp, tpos + 4 * k0, M * 4 * 8, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(d_bm, Bm + k0, M * 8, cudaMemcpyHostToDevice, c->stream));
    if (what == 2) CK(cudaMemcpyAsync(d_cst, cst + 4 * k0, M * 4 * 8, cudaMemcpyHostToDevice, c->stream));
    CK(c->tab[c->field.model].bc_eval(c->field, c->cfg.fieldlineresolution, what, m, d_tp, d_bm, eyegradientstep,
                                      d_cst, d_out, c->fl_scratch, stride, kFieldlineCap, c->stream));
    CK(cudaMemcpyAsync(out + 3 * k0, d_out, M * 3 * 8, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return RAPT_OK;
}

int rapt_host_register(void* p, uint64_t bytes) {
  if (!p || bytes == 0) return RAPT_ERR_INVALID;
  return cudaHostRegister(p, (size_t)bytes, cudaHostRegisterDefault) == cudaSuccess ? RAPT_OK : RAPT_ERR_CUDA;
}

int rapt_host_unregister(void* p) {
  if (!p) return RAPT_ERR_INVALID;
  return cudaHostUnregister(p) == cudaSuccess ? RAPT_OK : RAPT_ERR_CUDA;
}

int rapt_measure_peaks(void* ctx, double* fp64_tflops, double* fp32_tflops) {
  Ctx* c = static_cast<Ctx*>(ctx);
  if (!c) return RAPT_ERR_INVALID;
  CK(cudaSetDevice(c->device));
  int rc = ensure_tmp(c, 4096 * 8);
  if (rc) return rc;
  const int blocks = c->num_sms * 4, threads = 256;
  auto run = [&](auto tag, int iters, double* out_tflops) -> int {
    using T = decltype(tag);
    for (int rep = 0; rep < 2; ++rep) {
      CK(cudaEventRecord(c->ev0, c->stream));
      k_fma_peak<T><<<blocks, threads, 0, c->stream>>>(static_cast<T*>(c->tmp), iters, (T)1.0);
      CK(cudaGetLastError());
      CK(cudaEventRecord(c->ev1, c->stream));
      CK(cudaEventSynchronize(c->ev1));
    }
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
    *out_tflops = flops / (ms * 1e-3) / 1e12;
    return RAPT_OK;
  };
  double a = 0, b = 0;
  rc = run(double(0), 4096, &a);
  if (rc) return rc;
  rc = run(float(0), 65536, &b);
  if (rc) return rc;
  if (fp64_tflops) *fp64_tflops = a;
  if (fp32_tflops) *fp32_tflops = b;
  return RAPT_OK;
}

}  // extern "C"
