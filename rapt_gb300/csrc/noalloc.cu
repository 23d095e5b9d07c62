// noalloc.cu -- GuidingCenter.advance on caller-owned device memory, with no
// allocation of any kind.
//
// Some callers cannot call cudaMalloc: a host application that must not
// allocate after start-up (real-time loops), code that owns device memory
// through its own pool and must not create a second allocator, or code that
// runs between other work that must not be disturbed by an implicit device
// synchronisation (cudaMalloc/cudaFree can synchronise the device). For them,
// rapt_gc_advance_noalloc runs the persistent guiding-centre kernel on the
// caller's state arrays and keeps every other word the kernel needs -- the
// work-queue heads and counters, and the per-tracer advance bookkeeping -- in
// one file-scope __device__ array of fixed size (RAPT_NOALLOC_SCRATCH_BYTES).
// That array exists on every GPU that loads the library, until the process
// exits.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress (with that device current) and keeps it, together with
// the unique id of the device's context; a later call on a different context
// (after cudaDeviceReset) looks the address up again. Make the first call on a
// device before any stream capture on it. Every call reuses the same array and
// clears the parts that must start at zero, so calls whose work overlaps on the
// GPU (two host threads, or two streams, on the same device) race on it and
// must be serialised. The call is synchronous: it returns after the GPU work
// has completed.
//
// Only the configuration this path runs is accepted: the plain FP64 form, a
// fixed output cadence (GCtimestep > 0), no dense output and no sample
// collection; anything else returns RAPT_ERR_UNSUPPORTED rather than running
// something other than what was asked.
#include <cmath>
#include <cstring>
#include <mutex>

#include "launch.h"

using namespace rapt;

namespace {

constexpr int64_t kMax = RAPT_NOALLOC_MAX_TRACERS;
constexpr size_t al256(size_t b) { return (b + 255) & ~size_t(255); }

// Layout of the scratch array: the Scratch words, then per-tracer bookkeeping.
constexpr size_t kOffScratch = 0;
constexpr size_t kOffD = al256(sizeof(Scratch));             // 8 double arrays
constexpr size_t kOffI = kOffD + 8 * al256(kMax * 8);          // 3 int32 arrays
constexpr size_t kOffB = kOffI + 3 * al256(kMax * 4);          // 2 int8 arrays
constexpr size_t kBytes = kOffB + 2 * al256(kMax);
static_assert(kBytes <= RAPT_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the declared size");

// The scratch: fixed size, one per device, never allocated or freed.
static __device__ __align__(256) unsigned char g_noalloc_scratch[RAPT_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_addr[kMaxDevices] = {nullptr};
unsigned long long g_ctx_id[kMaxDevices] = {0};

// Unique id of the current CUDA context (cuCtxGetId, through the runtime's
// driver entry points so that the library needs no link to libcuda), or 0 when
// the driver does not provide it or no context is current.
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);
unsigned long long current_ctx_id() {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", reinterpret_cast<void**>(&get_current), 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      get_current = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", reinterpret_cast<void**>(&get_id), 12000,
                                         cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      get_id = nullptr;
    cudaGetLastError();
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (get_current && get_id && get_current(&ctx) == 0 && ctx && get_id(ctx, &id) == 0) return id;
  return 0;
}

// Device address of g_noalloc_scratch on `device` (which must be current):
// looked up once per device context. Without a context id (old driver) it is
// looked up on every call.
int scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return RAPT_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_mu);
  const unsigned long long id = current_ctx_id();
  if (!g_addr[device] || id == 0 || id != g_ctx_id[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return RAPT_ERR_CUDA;
    }
    g_addr[device] = p;
    g_ctx_id[device] = current_ctx_id();  // the lookup may have created the context
  }
  *out = static_cast<unsigned char*>(g_addr[device]);
  return RAPT_OK;
}

__global__ void k_noalloc_init(DevEnsemble E, double delta) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= E.n) return;
  E.mode[k] = RAPT_MODE_GC;
  E.flags[k] = 0;
  E.nswitch[k] = 0;
  E.nseg[k] = 0;
  E.seg_active[k] = 0;
  E.status[k] = RAPT_ST_OK;
  E.delta[k] = delta;
  E.t_int[k] = E.t_row[k];
  E.tcur[k] = E.t_row[k];
  E.s[4][k] = 0.0;
  E.s[5][k] = 0.0;
}

void register_model(int m, ModelTable* t) {
  switch (m) {
    case 0: register_model_0(t); break;
    case 1: register_model_1(t); break;
    case 2: register_model_2(t); break;
    case 3: register_model_3(t); break;
    case 4: register_model_4(t); break;
    case 5: register_model_5(t); break;
    case 6: register_model_6(t); break;
    default: register_model_7(t); break;
  }
}

// Same field construction as rapt_field_set (defaults of fields.py, then overrides).
void field_params(int model, const double* params, int np, FieldP* f) {
  std::memset(f, 0, sizeof(*f));
  f->model = model;
  f->is_static = 1;
  f->gradstep = 1e-6;
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
    default: p[0] = kB0; p[1] = 0.1; p[2] = 60.0; f->gradstep = kRe / 1000; f->is_static = 0; break;
  }
  for (int i = 0; i < np && i < 8; ++i) p[i] = params[i];
  if (model == RAPT_HARRIS) f->gradstep = p[1] * 1e-4;
  f->inv2d = 1.0 / (2.0 * f->gradstep);
  switch (model) {
    case RAPT_EARTH_DIPOLE: f->c0 = -3.0 * p[0] * kRe3; break;
    case RAPT_DOUBLE_DIPOLE: f->c0 = -p[0] * kRe3; break;
    case RAPT_VAR_EARTH_DIPOLE: f->c0 = -kB0 * kRe3; f->c1 = 2.0 * kPi / p[1]; break;
    case RAPT_HARRIS: f->c0 = 1.0 / p[1]; break;
    case RAPT_COMPRESSED_DIPOLE: f->c0 = -p[0] * kRe3; f->c1 = 2.0 * kPi / p[2]; f->c2 = p[0] * p[1] * f->c1 * kRe3; break;
    default: break;
  }
}

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int d) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    cudaSetDevice(d);
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace

extern "C" int rapt_gc_advance_noalloc(int device, int model, const double* params, int nparams,
                                       const rapt_config* cfg, const rapt_gc_device_state* st, double delta,
                                       void* stream, rapt_stats* stats) {
  if (!cfg || !st) return RAPT_ERR_INVALID;
  if (st->n < 0 || st->n > kMax) return RAPT_ERR_INVALID;  // more tracers than the scratch holds
  if (model < 0 || model >= RAPT_N_MODELS) return RAPT_ERR_UNSUPPORTED;
  if (model == RAPT_GRID) return RAPT_ERR_UNSUPPORTED;  // its data live in a context (rapt_grid_set)
  if (nparams < 0 || nparams > 8 || (nparams > 0 && !params)) return RAPT_ERR_INVALID;
  if (!std::isfinite(delta) || cfg->tableau < 0 || cfg->tableau > 1 || cfg->gc_eom < 0 || cfg->gc_eom > 2 ||
      cfg->nsteps <= 0 || st->max_rows < 2)
    return RAPT_ERR_INVALID;
  // the range checks of rapt_config_set
  if (!(cfg->rtol >= 0) || !(cfg->atol >= 0) || !(cfg->gctimestep >= 0) || !std::isfinite(cfg->gctimestep) ||
      !(cfg->epss >= 0) || !(cfg->epst >= 0) || cfg->max_steps_per_launch < 0 ||
      (cfg->tableau == 1 && !(cfg->rkf_tol > 0 && cfg->rkf_hmin >= 0)))
    return RAPT_ERR_INVALID;
  // what this path does not run: other forms, the bounce-period cadence
  // (GCtimestep == 0 needs per-thread field-line scratch), dense output and
  // sample collection
  if (cfg->form != RAPT_FORM_PLAIN || cfg->gctimestep == 0.0 || cfg->dense_output || cfg->collect)
    return RAPT_ERR_UNSUPPORTED;
  if (st->n == 0) return RAPT_OK;
  if (!st->t || !st->x || !st->y || !st->z || !st->ppar || !st->mu || !st->v || !st->mass || !st->charge ||
      !st->status || !st->naccept || !st->nreject || !st->nfcn || !st->rows || !st->row_mode || !st->nrows)
    return RAPT_ERR_INVALID;
  DeviceGuard guard(device);
  unsigned char* base = nullptr;
  int rc = scratch_address(device, &base);
  if (rc != RAPT_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // Device ensemble: the caller's arrays plus bookkeeping carved from the scratch.
  DevEnsemble E{};
  E.n = st->n;
  double* d = reinterpret_cast<double*>(base + kOffD);
  const size_t dstride = al256(kMax * 8) / 8;
  E.t_int = d + 0 * dstride;
  E.tcur = d + 1 * dstride;
  E.delta = d + 2 * dstride;
  E.seg_stop = d + 3 * dstride;
  E.seg_dt = d + 4 * dstride;
  E.seg_gm = d + 5 * dstride;
  E.s[4] = d + 6 * dstride;
  E.s[5] = d + 7 * dstride;
  int32_t* ip = reinterpret_cast<int32_t*>(base + kOffI);
  const size_t istride = al256(kMax * 4) / 4;
  E.flags = ip;
  E.nswitch = ip + istride;
  E.nseg = ip + 2 * istride;
  int8_t* bp = reinterpret_cast<int8_t*>(base + kOffB);
  E.mode = bp;
  E.seg_active = bp + al256(kMax);
  E.t_row = st->t;
  E.s[0] = st->x; E.s[1] = st->y; E.s[2] = st->z; E.s[3] = st->ppar;
  E.mu = const_cast<double*>(st->mu);
  E.v = const_cast<double*>(st->v);
  E.mass = const_cast<double*>(st->mass);
  E.charge = const_cast<double*>(st->charge);
  E.status = st->status;
  E.naccept = st->naccept;
  E.nreject = st->nreject;
  E.nfcn = st->nfcn;
  E.rows = st->rows;
  E.row_mode = st->row_mode;
  E.nrows = st->nrows;
  E.sw_time = nullptr;
  E.sw_mode = nullptr;
  Scratch* S = reinterpret_cast<Scratch*>(base + kOffScratch);

  KParams P{};
  field_params(model, params, nparams, &P.f);
  P.rtol = cfg->rtol; P.atol = cfg->atol; P.cycres = cfg->cyclotronresolution; P.gctimestep = cfg->gctimestep;
  P.epss = cfg->epss; P.epst = cfg->epst; P.rkf_tol = cfg->rkf_tol; P.rkf_hmin = cfg->rkf_hmin;
  P.enforce_eq = cfg->enforce_equatorial; P.tableau = cfg->tableau; P.gc_eom = cfg->gc_eom;
  P.nsteps = cfg->nsteps; P.kind = RAPT_KIND_GC; P.form = RAPT_FORM_PLAIN;
  P.budget = cfg->max_steps_per_launch > 0 ? cfg->max_steps_per_launch : (1LL << 62);
  P.max_rows = st->max_rows; P.max_sw = 0; P.max_segments = 1;

  ModelTable T{};
  register_model(model, &T);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return RAPT_ERR_CUDA;
  const int block = 128;
  const int bps = T.occ_gc[P.tableau](block);
  if (bps < 1) return RAPT_ERR_CUDA;

  k_noalloc_init<<<(unsigned)((E.n + 255) / 256), 256, 0, s>>>(E, delta);
  if (cudaGetLastError() != cudaSuccess) return RAPT_ERR_CUDA;
  if (cudaMemsetAsync(S, 0, sizeof(Scratch), s) != cudaSuccess) return RAPT_ERR_CUDA;
  if (cudaMemsetAsync(st->nrows, 0, (size_t)E.n * sizeof(int32_t), s) != cudaSuccess) return RAPT_ERR_CUDA;
  constexpr int64_t kMaxRounds = 1000000;
  int64_t rounds = 0;  // guiding-centre kernel launches
  unsigned long long pending = 1;
  while (pending != 0 && rounds < kMaxRounds) {
    if (cudaMemsetAsync(S, 0, 3 * sizeof(unsigned long long), s) != cudaSuccess) return RAPT_ERR_CUDA;
    LaunchArgs a{E, P, S, sms * bps, block, s};
    if (T.gc[P.tableau](a) != cudaSuccess) return RAPT_ERR_CUDA;
    ++rounds;
    if (cudaMemcpyAsync(&pending, &S->pending, sizeof(pending), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      return RAPT_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RAPT_ERR_CUDA;
  }
  if (stats) {
    Scratch hs;
    if (cudaMemcpyAsync(&hs, S, sizeof(Scratch), cudaMemcpyDeviceToHost, s) != cudaSuccess) return RAPT_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RAPT_ERR_CUDA;
    std::memset(stats, 0, sizeof(*stats));
    stats->accepted = (int64_t)hs.accepted;
    stats->rejected = (int64_t)hs.rejected;
    stats->rhs_evals = (int64_t)hs.rhs;
    stats->done = (int64_t)hs.done;
    stats->failed = (int64_t)hs.failed;
    stats->launches = rounds;
    stats->kernel_launches = rounds + 1;  // the guiding-centre rounds and the one bookkeeping kernel
  }
  // tracers still pending after the round cap: the advance did not finish
  if (pending != 0) return RAPT_ERR_STATE;
  return RAPT_OK;
}
