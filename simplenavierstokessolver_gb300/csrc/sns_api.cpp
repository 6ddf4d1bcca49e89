// Host side of libsns_gpu.so: the C ABI declared in include/sns_gpu.h.
//
// Everything computed here that feeds the kernels (grid metrics, Thomas
// factors, Poisson eigenvalues, FFT twiddles, RK scalars) uses the
// reference's expressions in its operation order; this file must be compiled
// without floating-point contraction (-ffp-contract=off), which the build
// recipe enforces.
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstddef>
#include <cstring>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "diag_internal.h"
#include "host_common.h"
#include "npy.h"
#include "sns_batch.h"
#include "sns_gpu.h"
#include "sns_internal.h"

namespace sns {

static std::atomic<long long> g_launches{0};
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
static std::atomic<long long> g_allocs{0};
void count_allocation() { g_allocs.fetch_add(1, std::memory_order_relaxed); }

static thread_local std::string g_error;

void record_error(const char *msg) { g_error = msg; }

static int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

#define SNS_CUDA(call)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess)                                                                   \
      return fail(SNS_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
  } while (0)

constexpr uint64_t kFluidMagic = 0x534e53464c554944ull;  // "SNSFLUID"
constexpr uint64_t kTempMagic = 0x534e5354454d5045ull;   // "SNSTEMPE"

static bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
static bool is_pow2_double(double v) {
  if (!(v > 0.0) || !std::isfinite(v)) return false;
  int e;
  return std::frexp(v, &e) == 0.5;
}

// ------------------------------------------------------------------- context
struct FluidExt;
struct TempExt;

// A reference-named call whose launch waits for a later call of the same
// substage, to share its launch: the explicit temperature update runs inside
// the next fluid_compute_potential's fused Poisson launch (as sns_run does),
// the velocity correction together with the next fluid_update_pressure. Every
// other entry point performs pending work first (flush_pending).
struct PendingTemp {
  TempExt *te = nullptr;  // set: an explicit temperature update not launched yet
  int rk = -1, out = -1;
  StageScalars s{};
  const double *ux_k = nullptr, *uy_k = nullptr;  // the velocity it reads
};
struct PendingCorr {
  FluidExt *fe = nullptr;  // set: a velocity correction not launched yet
  int rk = -1, impx = 0, impy = 0;
  StageScalars s{};
};

constexpr int kFacSlots = 8;  // factor upload slots: more than one substage's uploads

struct Context {
  const param_t *param = nullptr;
  int refs = 0;
  int nx = 0, ny = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t side = nullptr;  // temperature update overlapped with the Poisson solve
  cudaEvent_t ev_fwd = nullptr, ev_temp = nullptr;
  DevGrid g{};
  std::vector<void *> allocs;
  std::vector<double> dxf, dxc;  // host copies of the reference arrays (0-based)
  double *staging = nullptr;     // pinned, nx*ny doubles
  unsigned long long *red_host = nullptr;  // pinned, nx+1 words
  // factors for the implicit solves: device buffer, and a ring of pinned host
  // staging slots so that the uploads are asynchronous; a slot is rewritten
  // only after its previous upload completed (fac_ev)
  double *fac = nullptr;
  size_t fac_words = 0;
  double *fac_host = nullptr;  // [kFacSlots][fac_words], pinned
  cudaEvent_t fac_ev[kFacSlots] = {};
  unsigned fac_next = 0;        // next slot of the ring
  int fac_slot = 0;             // the slot being filled
  double *fac_stage = nullptr;  // its host words
  double *diag = nullptr;  // block partials of sns_diagnostics
  // fused Poisson (+ temperature) launches: flag words, on unless disabled
  // or unsupported for this size
  bool fused = true;
  bool fused_ready = false;
  // ux, uy on the device change with every bump of `version`; colmax holds
  // the max-|u| reduction of the state of version `red_version` (written by
  // the last substage of sns_run / sns_integrate), so param_decide_dt and the
  // next sns_run skip their reduction launch while nothing changed in between
  unsigned long long version = 1, red_version = 0;
  unsigned long long red_host_version = 0;  // state version whose reduction red_host holds
  PendingTemp ptemp;
  PendingCorr pcorr;
  FusedState fz;
  unsigned *fz_err_host = nullptr;  // pinned
  // the Poisson lines' solver: SNS_FORM_EXACT (the reference's
  // recurrence, identical results) or SNS_FORM_PARALLEL (partition
  // method with parallel cyclic reduction, held to the path's tolerance)
  int form = SNS_FORM_EXACT;
  ParFactors par{};
  bool par_ready = false;
  unsigned *par_err_host = nullptr;  // pinned
  // asynchronous checkpoint (sns_checkpoint): a device snapshot of ux, uy, p
  // and T taken on the solver's stream, its copy to pinned memory on ck_stream,
  // and a host thread that writes the files
  double *ck_dev = nullptr;
  double *ck_host = nullptr;
  cudaStream_t ck_stream = nullptr;
  cudaEvent_t ck_snap = nullptr, ck_done = nullptr;
  std::thread ck_thread;
  int ck_status = SNS_OK;
  std::string ck_error;
  // optional per-launch event timing (sns_profile)
  bool prof = false;
  std::vector<cudaEvent_t> prof_ev;  // two per slot
  std::vector<int> prof_kind;
  size_t prof_used = 0;
  double prof_ms[K_NUM_KINDS] = {};
  long long prof_n[K_NUM_KINDS] = {};
};

static void prof_collect(Context *c) {
  if (c->prof_used == 0) return;
  cudaStreamSynchronize(c->stream);
  for (size_t k = 0; k < c->prof_used; k++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->prof_ev[2 * k], c->prof_ev[2 * k + 1]) == cudaSuccess) {
      c->prof_ms[c->prof_kind[k]] += ms;
      c->prof_n[c->prof_kind[k]] += 1;
    }
  }
  c->prof_used = 0;
}

// brackets the launches of one kernel with events on the solver's stream
// when profiling is on; no work at all otherwise
struct Prof {
  Context *c;
  cudaStream_t st;
  long idx = -1;
  Prof(Context *c_, int kind, cudaStream_t s_ = nullptr) : c(c_), st(s_ ? s_ : c_->stream) {
    if (!c->prof) return;
    if (c->prof_used >= 2048) prof_collect(c);
    if (2 * (c->prof_used + 1) > c->prof_ev.size()) {
      cudaEvent_t a, b;
      if (cudaEventCreate(&a) != cudaSuccess) return;
      if (cudaEventCreate(&b) != cudaSuccess) {
        cudaEventDestroy(a);
        return;
      }
      c->prof_ev.push_back(a);
      c->prof_ev.push_back(b);
      c->prof_kind.push_back(0);
    }
    idx = (long)c->prof_used++;
    c->prof_kind[idx] = kind;
    cudaEventRecord(c->prof_ev[2 * idx], st);
  }
  ~Prof() {
    if (idx >= 0) cudaEventRecord(c->prof_ev[2 * idx + 1], st);
  }
};

// the plain kernels of the context's arithmetic form: sns::exact (the
// reference's roundings) or sns::contract (fused multiply-adds)
#define FORM(c, fn) ((c)->form == SNS_FORM_PARALLEL ? contract::fn : exact::fn)

static std::mutex g_mu;
static std::vector<Context *> g_contexts;

struct FluidExt {
  fluid_t pub;  // first member: fluid_t* and FluidExt* coincide
  uint64_t magic;
  Context *ctx;
  Fields f;
};

struct TempExt {
  temperature_t pub;
  uint64_t magic;
  Context *ctx;
  TempFields f;
  int cur;   // buffer holding the current temperature
  int snap;  // buffer the buoyancy refers to; -1 forcing off, -2 never computed
};

static FluidExt *as_fluid(const fluid_t *f) {
  auto *e = reinterpret_cast<FluidExt *>(const_cast<fluid_t *>(f));
  return (e && e->magic == kFluidMagic) ? e : nullptr;
}
static TempExt *as_temp(const temperature_t *t) {
  auto *e = reinterpret_cast<TempExt *>(const_cast<temperature_t *>(t));
  return (e && e->magic == kTempMagic) ? e : nullptr;
}

template <typename T>
static int dev_alloc(Context *c, T **p, size_t count) {
  void *ptr = nullptr;
  cudaError_t e = counted_malloc(&ptr, std::max<size_t>(count, 1) * sizeof(T));
  if (e != cudaSuccess) return fail(SNS_ERR_OOM, "cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
  c->allocs.push_back(ptr);
  *p = static_cast<T *>(ptr);
  return SNS_OK;
}

template <typename T>
static int upload(Context *c, const T **dst, const std::vector<T> &src) {
  T *p = nullptr;
  if (int rc = dev_alloc(c, &p, src.size())) return rc;
  SNS_CUDA(cudaMemcpy(p, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  *dst = p;
  return SNS_OK;
}

static void destroy_context(Context *c) {
  if (c->ck_thread.joinable()) c->ck_thread.join();
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->ck_host) cudaFreeHost(c->ck_host);
  if (c->ck_snap) cudaEventDestroy(c->ck_snap);
  if (c->ck_done) cudaEventDestroy(c->ck_done);
  if (c->ck_stream) cudaStreamDestroy(c->ck_stream);
  for (cudaEvent_t e : c->prof_ev) cudaEventDestroy(e);
  c->prof_ev.clear();
  for (void *p : c->allocs) cudaFree(p);
  c->allocs.clear();
  if (c->staging) cudaFreeHost(c->staging);
  if (c->red_host) cudaFreeHost(c->red_host);
  if (c->fz_err_host) cudaFreeHost(c->fz_err_host);
  if (c->par_err_host) cudaFreeHost(c->par_err_host);
  if (c->fac_host) cudaFreeHost(c->fac_host);
  for (cudaEvent_t e : c->fac_ev)
    if (e) cudaEventDestroy(e);
  if (c->ev_fwd) cudaEventDestroy(c->ev_fwd);
  if (c->ev_temp) cudaEventDestroy(c->ev_temp);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

static int build_context(Context *c, const param_t *param) {
  const int nx = param->itot, ny = param->jtot;
  c->param = param;
  c->nx = nx;
  c->ny = ny;
  // the side stream carries the temperature update beside the Poisson
  // kernels (off the critical path); the main stream's blocks are scheduled
  // first when both have work waiting
  int prio_least = 0, prio_greatest = 0;
  SNS_CUDA(cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest));
  SNS_CUDA(cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, prio_greatest));
  SNS_CUDA(cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_least));
  SNS_CUDA(cudaEventCreateWithFlags(&c->ev_fwd, cudaEventDisableTiming));
  SNS_CUDA(cudaEventCreateWithFlags(&c->ev_temp, cudaEventDisableTiming));
  c->dxf.assign(param->dxf, param->dxf + nx);
  c->dxc.assign(param->dxc, param->dxc + nx + 1);
  DevGrid &g = c->g;
  g.nx = nx;
  g.ny = ny;
  g.nh = ny / 2 + 1;
  g.jpitch = (g.nh + 15) / 16 * 16;
  g.dy = param->dy;
  bool rcp = is_pow2_double(param->dy);
  for (double v : c->dxf) rcp = rcp && is_pow2_double(v);
  for (double v : c->dxc) rcp = rcp && is_pow2_double(v);
  g.rcp = rcp;
  g.rdy = 1.0 / param->dy;
  const double *dxf = param->dxf, *dxc = param->dxc;
  auto DXF = [&](int i) { return dxf[i - 1]; };
  auto DXC = [&](int i) { return dxc[i - 1]; };
  std::vector<double> rdxf(nx), rdxc(nx + 1), dxi(nx + 1), ccm(nx), ccp(nx), cfm(nx), cfp(nx), pl(nx);
  for (int i = 1; i <= nx; i++) {
    rdxf[i - 1] = 1.0 / DXF(i);
    ccm[i - 1] = DXC(i) / (2. * DXF(i));      // src/temperature/update.c:44, update_velocity.c:242
    ccp[i - 1] = DXC(i + 1) / (2. * DXF(i));  // src/temperature/update.c:45, update_velocity.c:243
    if (i >= 2) {
      cfm[i - 1] = DXF(i - 1) / (2. * DXC(i));  // src/fluid/update_velocity.c:148
      cfp[i - 1] = DXF(i) / (2. * DXC(i));      // src/fluid/update_velocity.c:149
    }
    pl[i - 1] = 1. / DXC(i) / DXF(i);  // src/fluid/compute_potential.c:118
  }
  for (int i = 1; i <= nx + 1; i++) {
    rdxc[i - 1] = 1.0 / DXC(i);
    dxi[i - 1] = 1. / DXC(i);  // src/fluid/correct_velocity.c:13
  }
  {
    // the power-of-two products taken in integer arithmetic (velocity,
    // temperature and correction kernels, the Poisson forward elimination)
    auto p2 = [](double v) {
      int e;
      return is_pow2_double(v) && (std::frexp(v, &e), std::abs(e - 1) <= 64);
    };
    bool ok = rcp && p2(g.rdy);
    for (int i = 0; i < nx; i++) ok = ok && p2(rdxf[i]) && p2(ccm[i]) && p2(ccp[i]) && p2(pl[i]);
    for (int i = 0; i <= nx; i++) ok = ok && p2(rdxc[i]);
    for (int i = 1; i < nx; i++) ok = ok && p2(cfm[i]) && p2(cfp[i]);
    g.p2 = ok;
  }
  int rc = SNS_OK;
  if ((rc = upload(c, &g.dxf, c->dxf)) || (rc = upload(c, &g.dxc, c->dxc)) || (rc = upload(c, &g.rdxf, rdxf)) ||
      (rc = upload(c, &g.rdxc, rdxc)) || (rc = upload(c, &g.dxi, dxi)) || (rc = upload(c, &g.c_cm, ccm)) ||
      (rc = upload(c, &g.c_cp, ccp)) || (rc = upload(c, &g.c_fm, cfm)) || (rc = upload(c, &g.c_fp, cfp)) ||
      (rc = upload(c, &g.pl, pl)))
    return rc;
  // Poisson factors per mode J (src/fluid/compute_potential.c:109-127)
  const int nh = g.nh;
  const size_t jp = (size_t)g.jpitch;
  std::vector<double> pinv((size_t)nx * jp, 0.0), pup((size_t)nx * jp, 0.0), pd0(nh);
  {
    std::vector<double> l(nx), d(nx), u(nx), inv(nx), up(nx);
    const double dy = param->dy;
    for (int J = 0; J < nh; J++) {
      const double eig = poisson_eigenvalue(dy, ny, J);
      for (int i = 1; i <= nx; i++) {
        l[i - 1] = 1. / DXC(i) / DXF(i);
        u[i - 1] = 1. / DXC(i + 1) / DXF(i);
      }
      for (int i = 1; i <= nx; i++) d[i - 1] = -l[i - 1] - u[i - 1] + eig;
      d[0] += l[0];
      d[nx - 1] += u[nx - 1];
      factorize(nx, l.data(), d.data(), u.data(), inv.data(), up.data());
      pd0[J] = d[0];
      for (int x = 0; x < nx; x++) {
        pinv[(size_t)x * jp + J] = inv[x];
        pup[(size_t)x * jp + J] = up[x];
      }
    }
  }
  if ((rc = upload(c, &g.pinv, pinv)) || (rc = upload(c, &g.pup, pup)) || (rc = upload(c, &g.pd0, pd0)))
    return rc;
  const std::vector<double> tw = twiddle_table(ny);
  if ((rc = upload(c, &g.tw, tw))) return rc;
  fft_layout(ny, &g.fft_nst, &g.fft_first2);
  SNS_CUDA(counted_malloc_host(&c->staging, sizeof(double) * (size_t)nx * ny));
  SNS_CUDA(counted_malloc_host(&c->red_host, sizeof(unsigned long long) * (size_t)(nx + 1)));
  return SNS_OK;
}

static int check_inputs(const param_t *param, const parallel_t *parallel) {
  if (!param || !parallel) return fail(SNS_ERR_ARG, "param and parallel must not be NULL");
  if (parallel->mpisize != 1)
    return fail(SNS_ERR_UNSUPPORTED, "single-rank only (mpisize=%d); one GPU holds the whole domain", parallel->mpisize);
  if (param->itot < 2 || param->itot > 16384)
    return fail(SNS_ERR_UNSUPPORTED, "itot=%d outside [2, 16384]", param->itot);
  if (param->jtot < 2 || !is_pow2(param->jtot) || param->jtot > 16384)
    return fail(SNS_ERR_UNSUPPORTED, "jtot=%d must be a power of two in [2, 16384] (real FFT along y)", param->jtot);
  if (!param->dxf || !param->dxc) return fail(SNS_ERR_ARG, "param grid arrays are NULL");
  return SNS_OK;
}

static Context *acquire_context(const param_t *param) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (Context *c : g_contexts)
    if (c->param == param && c->nx == param->itot && c->ny == param->jtot) {
      c->refs++;
      return c;
    }
  Context *c = new Context();
  if (build_context(c, param) != SNS_OK) {
    std::string keep = g_error;
    destroy_context(c);
    g_error = keep;
    return nullptr;
  }
  c->refs = 1;
  g_contexts.push_back(c);
  return c;
}

static void release_context(Context *c) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (--c->refs > 0) return;
  g_contexts.erase(std::remove(g_contexts.begin(), g_contexts.end(), c), g_contexts.end());
  destroy_context(c);
}

// ------------------------------------------------- host boundary rules
// single-rank forms of src/fluid/boundary_conditions.c:6-55 and
// src/temperature/boundary_conditions.c:6-21 on reference-layout host arrays
static void host_bc_ux(int nx, int ny, double *ux) {
  auto UX = [&](int i, int j) -> double & { return ux[(size_t)j * (nx + 1) + (i - 1)]; };
  for (int i = 2; i <= nx; i++) {
    UX(i, 0) = UX(i, ny);
    UX(i, ny + 1) = UX(i, 1);
  }
  for (int j = 0; j <= ny + 1; j++) {
    UX(1, j) = 0.;
    UX(nx + 1, j) = 0.;
  }
}
static void host_bc_uy(int nx, int ny, double *uy) {
  auto UY = [&](int i, int j) -> double & { return uy[(size_t)j * (nx + 2) + i]; };
  for (int i = 1; i <= nx; i++) {
    UY(i, 0) = UY(i, ny);
    UY(i, ny + 1) = UY(i, 1);
  }
  for (int j = 0; j <= ny + 1; j++) {
    UY(0, j) = 0.;
    UY(nx + 1, j) = 0.;
  }
}
static void host_bc_p(int nx, int ny, double *p) {
  auto P = [&](int i, int j) -> double & { return p[(size_t)j * (nx + 2) + i]; };
  for (int i = 1; i <= nx; i++) {
    P(i, 0) = P(i, ny);
    P(i, ny + 1) = P(i, 1);
  }
  for (int j = 0; j <= ny + 1; j++) {
    P(0, j) = P(1, j);
    P(nx + 1, j) = P(nx, j);
  }
}
static void host_bc_temp(int nx, int ny, double *t) {
  auto T = [&](int i, int j) -> double & { return t[(size_t)j * (nx + 2) + i]; };
  for (int i = 1; i <= nx; i++) {
    T(i, 0) = T(i, ny);
    T(i, ny + 1) = T(i, 1);
  }
  for (int j = 1; j <= ny; j++) {
    T(0, j) = TEMP_XM;
    T(nx + 1, j) = TEMP_XP;
  }
}

// -------------------------------------------------- dense <-> reference layout
// The structures' host arrays are pinned, so one strided 2D DMA copy per
// field moves the dense interior (x fastest, ny rows) to or from a
// reference-layout array whose rows have `width` entries and whose interior
// column x sits at offset `off`. Callers synchronise once after all copies.
static int fetch(Context *c, const double *dev) {
  SNS_CUDA(cudaMemcpyAsync(c->staging, dev, sizeof(double) * (size_t)c->nx * c->ny, cudaMemcpyDeviceToHost,
                           c->stream));
  return SNS_OK;
}

static int download(Context *c, const double *dev, double *host, int width, int off, int first_x) {
  const int nx = c->nx, ny = c->ny;
  SNS_CUDA(cudaMemcpy2DAsync(host + width + off + first_x, sizeof(double) * width, dev + first_x,
                             sizeof(double) * nx, sizeof(double) * (nx - first_x), ny, cudaMemcpyDeviceToHost,
                             c->stream));
  return SNS_OK;
}

// ux (first_x = 1): the device keeps its wall column x = 0 at zero, it is never copied
static int upload_field(Context *c, double *dev, const double *host, int width, int off, int first_x) {
  const int nx = c->nx, ny = c->ny;
  SNS_CUDA(cudaMemcpy2DAsync(dev + first_x, sizeof(double) * nx, host + width + off + first_x,
                             sizeof(double) * width, sizeof(double) * (nx - first_x), ny, cudaMemcpyHostToDevice,
                             c->stream));
  return SNS_OK;
}

// sources: srcux* rows of itot-1 entries for i = 2..itot, srcuy*/srctemp* rows of itot
static int download_src(Context *c, const double *dev, double *host, int is_ux) {
  const int nx = c->nx, ny = c->ny;
  const int w = is_ux ? nx - 1 : nx, x0 = is_ux ? 1 : 0;
  SNS_CUDA(cudaMemcpy2DAsync(host, sizeof(double) * w, dev + x0, sizeof(double) * nx, sizeof(double) * w, ny,
                             cudaMemcpyDeviceToHost, c->stream));
  return SNS_OK;
}

static int upload_src(Context *c, double *dev, const double *host, int is_ux) {
  const int nx = c->nx, ny = c->ny;
  const int w = is_ux ? nx - 1 : nx, x0 = is_ux ? 1 : 0;
  SNS_CUDA(cudaMemcpy2DAsync(dev + x0, sizeof(double) * nx, host, sizeof(double) * w, sizeof(double) * w, ny,
                             cudaMemcpyHostToDevice, c->stream));
  return SNS_OK;
}

// The device alias of a pinned host array (nullptr when the array is not
// pinned, e.g. a caller replaced the pointer: the copies then go through DMA).
static double *dev_alias(const double *h) {
  void *d = nullptr;
  if (!h || cudaHostGetDevicePointer(&d, const_cast<double *>(h), 0) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return static_cast<double *>(d);
}

// one entry of a host -> device transfer list, as upload_src lays it out
static bool xfer_src(XferList &L, int nx, double *dev, const double *host, int is_ux) {
  const double *a = dev_alias(host);
  if (!a || L.n >= kXferMax) return false;
  const int w = is_ux ? nx - 1 : nx, x0 = is_ux ? 1 : 0;
  L.f[L.n++] = XferField{a, dev + x0, w, nx, w};
  return true;
}

// one entry of a device -> host transfer list, as download_src lays it out
static bool xfer_src_down(XferList &L, int nx, const double *dev, double *host, int is_ux) {
  double *a = dev_alias(host);
  if (!a || L.n >= kXferMax) return false;
  const int w = is_ux ? nx - 1 : nx, x0 = is_ux ? 1 : 0;
  L.f[L.n++] = XferField{dev + x0, a, nx, w, w};
  return true;
}

// a reference-layout host array moved whole by the linear copy kernel: needs
// the array pinned (a device alias) and 16-byte aligned
static bool lin_field(LinList &L, double *dev, double *host, int W, int kind) {
  double *a = dev_alias(host);
  if (!a || (reinterpret_cast<uintptr_t>(a) & 15u) || L.n >= kXferMax) return false;
  L.f[L.n++] = LinField{a, dev, W, kind};
  return true;
}

// pinned, zeroed host array (nullptr on failure)
static double *host_array(size_t n) {
  void *p = nullptr;
  if (counted_malloc_host(&p, std::max<size_t>(n, 1) * sizeof(double)) != cudaSuccess) return nullptr;
  std::memset(p, 0, std::max<size_t>(n, 1) * sizeof(double));
  return static_cast<double *>(p);
}

static void host_free(double *p) {
  if (p) cudaFreeHost(p);
}

// -------------------------------------------------------------- RK scalars
static StageScalars stage_scalars(const param_t *param, int rk) {
  StageScalars s{};
  const double alpha = param->rkcoefs[rk].alpha, beta = param->rkcoefs[rk].beta, gamma = param->rkcoefs[rk].gamma;
  const double dt = param->dt, Ra = param->Ra, Pr = param->Pr;
  s.adt = alpha * dt;
  s.bdt = beta * dt;
  s.gdt = gamma * dt;
  s.has_b = beta != 0.0;
  s.kappa = 1. / sqrt(Pr) / sqrt(Ra);  // src/temperature/update.c:65
  s.nu = sqrt(Pr) / sqrt(Ra);          // src/fluid/update_velocity.c:171
  s.rgdt = 1. / (gamma * dt);          // src/fluid/compute_potential.c:81
  s.rny = 1.0 / param->jtot;           // exact: jtot is a power of two
  const double Re = sqrt(Ra) / sqrt(Pr);  // src/fluid/update_pressure.c:19
  s.pcorr = -(gamma * dt) / (2. * Re);    // src/fluid/update_pressure.c:37
  return s;
}

// ------------------------------------------------- implicit-solve factors
// Factor buffer layout (doubles): [l | inv | up | zero-as-bytes] per system.
struct HostFactors {
  std::vector<double> l, inv, up;
  double d0 = 0;
};

// the reference's tridiagonal l, d, u of the Crank-Nicolson solve along x
// kind 0: temperature (src/temperature/update.c:141-149), n = itot
// kind 1: ux (src/fluid/update_velocity.c:249-264), n = itot+1 with identity end rows
// kind 2: uy (src/fluid/update_velocity.c:500-508), n = itot
static void x_tri(const param_t *param, int rk, int kind, std::vector<double> &l, std::vector<double> &d,
                  std::vector<double> &u) {
  const int nx = param->itot;
  const double *dxf = param->dxf, *dxc = param->dxc;
  auto DXF = [&](int i) { return dxf[i - 1]; };
  auto DXC = [&](int i) { return dxc[i - 1]; };
  const double gamma = param->rkcoefs[rk].gamma, dt = param->dt, Ra = param->Ra, Pr = param->Pr;
  const int n = kind == 1 ? nx + 1 : nx;
  l.assign(n, 0.);
  d.assign(n, 0.);
  u.assign(n, 0.);
  for (int i = 1; i <= n; i++) {
    if (kind == 1 && (i == 1 || i == nx + 1)) {
      l[i - 1] = 0.;
      u[i - 1] = 0.;
      d[i - 1] = 1.;
      continue;
    }
    double pf, cm, cp;
    if (kind == 0) {
      pf = (gamma * dt) / (2. * sqrt(Pr) * sqrt(Ra));
      cm = 1. / DXF(i) / DXC(i);
      cp = 1. / DXF(i) / DXC(i + 1);
    } else if (kind == 1) {
      pf = (gamma * dt * sqrt(Pr)) / (2. * sqrt(Ra));
      cm = 1. / DXC(i) / DXF(i - 1);
      cp = 1. / DXC(i) / DXF(i);
    } else {
      pf = (gamma * dt * sqrt(Pr)) / (2. * sqrt(Ra));
      cm = 1. / DXF(i) / DXC(i);
      cp = 1. / DXF(i) / DXC(i + 1);
    }
    const double c0 = -cm - cp;
    l[i - 1] = -pf * cm;
    u[i - 1] = -pf * cp;
    d[i - 1] = 1. - pf * c0;
  }
}

static void x_system(const param_t *param, int rk, int kind, HostFactors &hf) {
  std::vector<double> l, d, u;
  x_tri(param, rk, kind, l, d, u);
  const int n = (int)l.size();
  hf.l = l;
  hf.inv.assign(n, 0.);
  hf.up.assign(n, 0.);
  factorize(n, l.data(), d.data(), u.data(), hf.inv.data(), hf.up.data());
  hf.d0 = d[0];
}

// the reference's constant periodic y matrix: src/temperature/update.c:189-197
// (temperature, is_temp) or src/fluid/update_velocity.c:404-412 (velocity)
static void y_tri(const param_t *param, int rk, int is_temp, std::vector<double> &l, std::vector<double> &d,
                  std::vector<double> &u) {
  const int n = param->jtot;
  const double gamma = param->rkcoefs[rk].gamma, dt = param->dt, Ra = param->Ra, Pr = param->Pr, dy = param->dy;
  const double pf = is_temp ? (gamma * dt) / (2. * sqrt(Pr) * sqrt(Ra)) : (gamma * dt * sqrt(Pr)) / (2. * sqrt(Ra));
  l.assign(n, 0.);
  d.assign(n, 0.);
  u.assign(n, 0.);
  for (int j = 0; j < n; j++) {
    const double cm = 1. / dy / dy, cp = 1. / dy / dy;
    const double c0 = -cm - cp;
    l[j] = -pf * cm;
    u[j] = -pf * cp;
    d[j] = 1. - pf * c0;
  }
}

// src/linalg.c:52-108 on the y matrix of y_tri
static void y_system(const param_t *param, int rk, int is_temp, HostFactors &sub, std::vector<double> &q1,
                     double &l_last, double &u_last, double &den) {
  const int n = param->jtot;
  std::vector<double> l, d, u;
  y_tri(param, rk, is_temp, l, d, u);
  const int m = n - 1;
  sub.l.assign(l.begin(), l.begin() + m);
  sub.inv.assign(m, 0.);
  sub.up.assign(m, 0.);
  factorize(m, l.data(), d.data(), u.data(), sub.inv.data(), sub.up.data());
  sub.d0 = d[0];
  // second small system: RHS (-l[0], 0, ..., 0, -u[n-2]) (src/linalg.c:75-87), full Thomas
  q1.assign(m, 0.);
  for (int i = 0; i < m; i++) q1[i] = i == 0 ? -l[i] : i == m - 1 ? -u[i] : 0.;
  {
    std::vector<double> ll(l.begin(), l.begin() + m), dd(d.begin(), d.begin() + m), uu(u.begin(), u.begin() + m);
    uu[0] = uu[0] / dd[0];
    q1[0] = q1[0] / dd[0];
    for (int i = 1; i <= m - 1; i++) {
      double v = dd[i] - ll[i] * uu[i - 1];
      if (std::fabs(v) < DBL_EPSILON) {
        uu[i] = 0.;
        q1[i] = 0.;
      } else {
        v = 1. / v;
        uu[i] = v * uu[i];
        q1[i] = v * (q1[i] - ll[i] * q1[i - 1]);
      }
    }
    for (int i = m - 2; i >= 0; i--) q1[i] -= uu[i] * q1[i + 1];
  }
  l_last = l[n - 1];
  u_last = u[n - 1];
  den = (d[n - 1] + u[n - 1] * q1[0] + l[n - 1] * q1[n - 2]);
}

// copies n doubles at word offset `off` of the substage's pinned staging slot
// into the device factor buffer (stream-ordered, asynchronous)
static int stage_upload(Context *c, size_t off, const double *src, size_t n) {
  std::memcpy(c->fac_stage + off, src, n * sizeof(double));
  SNS_CUDA(cudaMemcpyAsync(c->fac + off, c->fac_stage + off, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return SNS_OK;
}

// copies factor arrays into the context's device buffer at word offset `off`
static int push_factors(Context *c, const HostFactors &hf, size_t off, LineFactors &lf) {
  const size_t n = hf.l.size();
  double *st = c->fac_stage + off;
  std::memcpy(st, hf.l.data(), n * sizeof(double));
  std::memcpy(st + n, hf.inv.data(), n * sizeof(double));  // 0 marks |pivot| < DBL_EPSILON rows
  std::memcpy(st + 2 * n, hf.up.data(), n * sizeof(double));
  SNS_CUDA(cudaMemcpyAsync(c->fac + off, st, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  lf.n = (int)n;
  lf.l = c->fac + off;
  lf.inv = c->fac + off + n;
  lf.up = c->fac + off + 2 * n;
  lf.d0 = hf.d0;
  return SNS_OK;
}

// factor layout: one x system at 0 and one y system at 4(nx+1) for the
// reference-named calls; three x systems (stride 3(nx+2)) and two y systems
// (stride 4 ny) after 9(nx+2) for the merged sweeps of the fused step
static size_t xset_off(const Context *c, int k) { return (size_t)k * 3 * (c->nx + 2); }
static size_t yset_off(const Context *c, int k) { return 9 * (size_t)(c->nx + 2) + (size_t)k * 4 * c->ny; }
// then the parallel form's line blocks: three x systems (temperature, ux,
// uy) and two y systems (temperature, velocity)
static size_t cnx_off(const Context *c, int k) {
  return std::max(4 * (size_t)(c->nx + 1) + 5 * (size_t)c->ny, yset_off(c, 2)) + 16 + (size_t)k * par_cn_stride(c->nx);
}
static size_t cny_off(const Context *c, int k) { return cnx_off(c, 3) + (size_t)k * par_cn_stride(c->ny); }

static int ensure_factor_buffer(Context *c) {
  const size_t need = cny_off(c, 2) + 16;
  if (c->fac_words >= need) return SNS_OK;
  if (int rc = dev_alloc(c, &c->fac, need)) return rc;
  if (c->fac_host) cudaFreeHost(c->fac_host);
  c->fac_host = nullptr;
  SNS_CUDA(counted_malloc_host(&c->fac_host, kFacSlots * need * sizeof(double)));
  for (cudaEvent_t &e : c->fac_ev)
    if (!e) SNS_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  c->fac_words = need;
  return SNS_OK;
}

// the next pinned staging slot of the ring, once its previous upload ran (in
// steady state long done: the ring spans more than a substage's uploads)
static int begin_factor_uploads(Context *c) {
  if (int rc = ensure_factor_buffer(c)) return rc;
  c->fac_slot = (int)(c->fac_next++ % kFacSlots);
  SNS_CUDA(cudaEventSynchronize(c->fac_ev[c->fac_slot]));
  c->fac_stage = c->fac_host + (size_t)c->fac_slot * c->fac_words;
  return SNS_OK;
}

static int end_factor_uploads(Context *c) {
  SNS_CUDA(cudaEventRecord(c->fac_ev[c->fac_slot], c->stream));
  return SNS_OK;
}

// ------------------------------------------ parallel form: Crank-Nicolson lines
// The Crank-Nicolson lines of the parallel form run the partition method
// (k_par_cn in plain_parallel.cu) where the line length allows it: results
// differ from the reference's Thomas recurrences (src/linalg.c:9-108) by
// rounding only.
static bool cn_parallel(const Context *c, int n) {
  return c->form == SNS_FORM_PARALLEL && parallel_cn_supported(n);
}

// the factor block of one line system: inv, g = a inv, up, v, w (rows
// interleaved), the PCR coefficients, then the interface rows' sub- and
// super-diagonals. a, d, c: the device line's rows; periodic: a_0 couples
// row 0 to row n-1 and c_{n-1} row n-1 to row 0 (otherwise both are dropped)
static void cn_block(int n, std::vector<double> a, const std::vector<double> &d, std::vector<double> c, bool periodic,
                     std::vector<double> &out) {
  if (!periodic) {
    a[0] = 0.0;
    c[n - 1] = 0.0;
  }
  const int m = n / kPartSeg;
  std::vector<double> blk(partition_stride(n));
  partition_factors_tri(n, a.data(), d.data(), c.data(), periodic, false, true, blk.data());
  out.assign(par_cn_stride(n), 0.0);
  std::copy(blk.begin(), blk.begin() + n, out.begin());  // inv
  for (int i = 0; i < n; i++) {
    const size_t o = (size_t)(i % m) * kPartSeg + i / m;
    out[n + o] = a[i] * blk[o];  // g
  }
  std::copy(blk.begin() + n, blk.end(), out.begin() + 2 * (size_t)n);  // up v w alpha beta rD
  double *ae = out.data() + par_cn_stride(n) - 2 * kPartSeg, *ce = ae + kPartSeg;
  for (int k = 0; k < kPartSeg; k++) {
    ae[k] = a[(size_t)k * m + m - 1];
    ce[k] = c[(size_t)k * m + m - 1];
  }
}

// the device rows x = 0..itot-1 of the x system of `kind` (x_tri); for ux
// row 0 is the wall's identity row and the other wall's row itot is not
// stored: both hold zero in the reference's solve, so their couplings to
// rows 1 and itot-1 drop out
static void cn_x_block(const param_t *param, int rk, int kind, std::vector<double> &out) {
  std::vector<double> l, d, u;
  x_tri(param, rk, kind, l, d, u);
  const int nx = param->itot;
  l.resize(nx);
  d.resize(nx);
  u.resize(nx);
  if (kind == 1) {
    l[1] = 0.0;
    u[nx - 1] = 0.0;
  }
  cn_block(nx, l, d, u, false, out);
}

static void cn_y_block(const param_t *param, int rk, int is_temp, std::vector<double> &out) {
  std::vector<double> l, d, u;
  y_tri(param, rk, is_temp, l, d, u);
  cn_block(param->jtot, l, d, u, true, out);
}

static ParCnArgs cn_x_args(const Context *c) {
  ParCnArgs a{};
  a.n = c->nx;
  a.lines = c->ny;
  a.es = 1;
  a.ls = c->nx;
  return a;
}

static ParCnArgs cn_y_args(const Context *c) {
  ParCnArgs a{};
  a.n = c->ny;
  a.lines = c->nx;
  a.es = c->nx;
  a.ls = 1;
  return a;
}

static int implicit_x(Context *c, const param_t *param, int rk, int kind, double *q) {
  if (cn_parallel(c, c->nx)) {
    std::vector<double> blk;
    cn_x_block(param, rk, kind, blk);
    if (int rc = begin_factor_uploads(c)) return rc;
    if (int rc = stage_upload(c, cnx_off(c, 0), blk.data(), blk.size())) return rc;
    if (int rc = end_factor_uploads(c)) return rc;
    ParCnArgs a = cn_x_args(c);
    a.f[0] = ParCnField{q, c->fac + cnx_off(c, 0), 0};
    a.nf = 1;
    Prof pf(c, K_SOLVE_X);
    SNS_CUDA(launch_par_cn(false, a, c->stream));
    return SNS_OK;
  }
  HostFactors hf;
  x_system(param, rk, kind, hf);
  LineFactors lf{};
  if (int rc = begin_factor_uploads(c)) return rc;
  if (int rc = push_factors(c, hf, 0, lf)) return rc;
  if (int rc = end_factor_uploads(c)) return rc;
  Prof pf(c, K_SOLVE_X);
  SNS_CUDA(FORM(c, launch_solve_x)(c->g, lf, kind == 1 ? 1 : 0, q, c->stream));
  return SNS_OK;
}

static int implicit_y(Context *c, const param_t *param, int rk, int is_temp, int first_col, double *q) {
  if (cn_parallel(c, c->ny)) {
    std::vector<double> blk;
    cn_y_block(param, rk, is_temp, blk);
    if (int rc = begin_factor_uploads(c)) return rc;
    if (int rc = stage_upload(c, cny_off(c, 0), blk.data(), blk.size())) return rc;
    if (int rc = end_factor_uploads(c)) return rc;
    ParCnArgs a = cn_y_args(c);
    a.f[0] = ParCnField{q, c->fac + cny_off(c, 0), first_col};
    a.nf = 1;
    Prof pf(c, K_SOLVE_Y);
    SNS_CUDA(launch_par_cn(true, a, c->stream));
    return SNS_OK;
  }
  HostFactors sub;
  std::vector<double> q1;
  PeriodicFactors pf{};
  y_system(param, rk, is_temp, sub, q1, pf.l_last, pf.u_last, pf.den);
  const size_t off = 4 * (size_t)(c->nx + 1);
  if (int rc = begin_factor_uploads(c)) return rc;
  if (int rc = push_factors(c, sub, off, pf.sub)) return rc;
  const size_t qoff = off + 4 * sub.l.size();
  if (int rc = stage_upload(c, qoff, q1.data(), q1.size())) return rc;
  if (int rc = end_factor_uploads(c)) return rc;
  pf.q1 = c->fac + qoff;
  Prof pr(c, K_SOLVE_Y);
  SNS_CUDA(FORM(c, launch_solve_y)(c->g, pf, first_col, q, c->stream));
  return SNS_OK;
}

static int ensure_implicit_buffers(FluidExt *fe) {
  Context *c = fe->ctx;
  const size_t n = (size_t)c->nx * c->ny;
  if (int rc = ensure_factor_buffer(c)) return rc;
  if (!fe->f.qx) {
    if (int rc = dev_alloc(c, &fe->f.qx, n)) return rc;
    if (int rc = dev_alloc(c, &fe->f.qy, n)) return rc;
  }
  return SNS_OK;
}

// ------------------------------------------------------------ operations
static int do_temp_update(const param_t *param, int rk, FluidExt *fe, TempExt *te) {
  Context *c = te->ctx;
  int out = 0;
  while (out == te->cur || out == te->snap) out++;
  const int impx = param->implicitx, impy = param->implicity;
  const StageScalars s = stage_scalars(param, rk);
  if (impx || impy) {
    if (int rc = ensure_factor_buffer(c)) return rc;
    if (!te->f.qt)
      if (int rc = dev_alloc(c, &te->f.qt, (size_t)c->nx * c->ny)) return rc;
  }
  {
    Prof pf(c, K_TEMP);
    SNS_CUDA(FORM(c, launch_temp_update)(c->g, s, impx, impy, te->f.t[te->cur], te->f.t[out], te->f.at, te->f.qt, fe->f.ux,
                                fe->f.uy, c->stream));
  }
  if (impx || impy) {
    if (impx)
      if (int rc = implicit_x(c, param, rk, 0, te->f.qt)) return rc;
    if (impy)
      if (int rc = implicit_y(c, param, rk, 1, 0, te->f.qt)) return rc;
    Prof pf(c, K_ADD_INC);
    SNS_CUDA(launch_add_increment(c->g, 0, te->f.t[te->cur], te->f.qt, te->f.t[out], c->stream));
  }
  te->cur = out;
  return SNS_OK;
}

static int do_velocity_update(const param_t *param, int rk, FluidExt *fe, const TempExt *te) {
  Context *c = fe->ctx;
  const int impx = param->implicitx, impy = param->implicity;
  const StageScalars s = stage_scalars(param, rk);
  if (impx || impy)
    if (int rc = ensure_implicit_buffers(fe)) return rc;
  const double *tf = (te && te->snap >= 0) ? te->f.t[te->snap] : nullptr;
  Fields &f = fe->f;
  {
    Prof pf(c, K_VEL);
    SNS_CUDA(FORM(c, launch_velocity_update)(c->g, s, impx, impy, f.ux, f.uy, f.p, tf, f.ux_alt, f.uy_alt, f.aux, f.auy,
                                    f.qx, f.qy, c->stream));
  }
  if (impx || impy) {
    if (impx) {
      if (int rc = implicit_x(c, param, rk, 1, f.qx)) return rc;
      if (int rc = implicit_x(c, param, rk, 2, f.qy)) return rc;
    }
    if (impy) {
      if (int rc = implicit_y(c, param, rk, 0, 1, f.qx)) return rc;
      if (int rc = implicit_y(c, param, rk, 0, 0, f.qy)) return rc;
    }
    Prof pf(c, K_ADD_INC);
    SNS_CUDA(launch_add_increment(c->g, 1, f.ux, f.qx, f.ux_alt, c->stream));
    SNS_CUDA(launch_add_increment(c->g, 0, f.uy, f.qy, f.uy_alt, c->stream));
  }
  std::swap(f.ux, f.ux_alt);
  std::swap(f.uy, f.uy_alt);
  return SNS_OK;
}

// The implicit-scheme substage updates of the fused step: temperature and
// velocity sources first, then the Crank-Nicolson sweeps of the three fields
// side by side (one launch per direction), then the increments. Each field
// goes through exactly the operations of do_temp_update / do_velocity_update
// on the same inputs (the velocity sources read the starting T, which the
// temperature increment does not touch); only independent launches merge.
static int implicit_updates(const param_t *param, int rk, FluidExt *fe, TempExt *te) {
  Context *c = fe->ctx;
  Fields &f = fe->f;
  const int impx = param->implicitx, impy = param->implicity;
  const bool with_t = param->with_temperature && te;
  const StageScalars s = stage_scalars(param, rk);
  if (int rc = ensure_implicit_buffers(fe)) return rc;
  int out = 0;
  if (with_t) {
    if (!te->f.qt)
      if (int rc = dev_alloc(c, &te->f.qt, (size_t)c->nx * c->ny)) return rc;
    while (out == te->cur || out == te->snap) out++;
    Prof pf(c, K_TEMP);
    SNS_CUDA(FORM(c, launch_temp_update)(c->g, s, impx, impy, te->f.t[te->cur], te->f.t[out], te->f.at, te->f.qt, f.ux, f.uy,
                                c->stream));
  }
  const double *tf = (te && te->snap >= 0) ? te->f.t[te->snap] : nullptr;
  {
    Prof pf(c, K_VEL);
    SNS_CUDA(FORM(c, launch_velocity_update)(c->g, s, impx, impy, f.ux, f.uy, f.p, tf, f.ux_alt, f.uy_alt, f.aux, f.auy, f.qx,
                                    f.qy, c->stream));
  }
  // fields: temperature (if coupled), ux, uy
  const int kinds[3] = {0, 1, 2};
  double *qs[3] = {with_t ? te->f.qt : nullptr, f.qx, f.qy};
  if (impx || impy)
    if (int rc = begin_factor_uploads(c)) return rc;
  if (impx && cn_parallel(c, c->nx)) {
    ParCnArgs a = cn_x_args(c);
    for (int k = with_t ? 0 : 1; k < 3; k++) {
      std::vector<double> blk;
      cn_x_block(param, rk, kinds[k], blk);
      if (int rc = stage_upload(c, cnx_off(c, k), blk.data(), blk.size())) return rc;
      a.f[a.nf++] = ParCnField{qs[k], c->fac + cnx_off(c, k), 0};
    }
    Prof pf(c, K_SOLVE_X);
    SNS_CUDA(launch_par_cn(false, a, c->stream));
  } else if (impx) {
    SolveXSet set{};
    for (int k = with_t ? 0 : 1; k < 3; k++) {
      HostFactors hf;
      x_system(param, rk, kinds[k], hf);
      if (int rc = push_factors(c, hf, xset_off(c, k), set.f[set.n])) return rc;
      set.mode[set.n] = kinds[k] == 1 ? 1 : 0;
      set.q[set.n] = qs[k];
      set.n++;
    }
    Prof pf(c, K_SOLVE_X);
    SNS_CUDA(FORM(c, launch_solve_x_set)(c->g, set, c->stream));
  }
  if (impy && cn_parallel(c, c->ny)) {
    ParCnArgs a = cn_y_args(c);
    for (int sys = with_t ? 0 : 1; sys < 2; sys++) {  // y systems: temperature, velocity
      std::vector<double> blk;
      cn_y_block(param, rk, sys == 0 ? 1 : 0, blk);
      if (int rc = stage_upload(c, cny_off(c, sys), blk.data(), blk.size())) return rc;
      const double *fac = c->fac + cny_off(c, sys);
      if (sys == 0) {
        a.f[a.nf++] = ParCnField{te->f.qt, fac, 0};
      } else {
        a.f[a.nf++] = ParCnField{f.qx, fac, 1};  // ux: columns 1..itot-1
        a.f[a.nf++] = ParCnField{f.qy, fac, 0};
      }
    }
    Prof pr(c, K_SOLVE_Y);
    SNS_CUDA(launch_par_cn(true, a, c->stream));
  } else if (impy) {
    SolveYSet set{};
    for (int sys = with_t ? 0 : 1; sys < 2; sys++) {  // y systems: temperature, velocity
      HostFactors sub;
      std::vector<double> q1;
      PeriodicFactors pf{};
      y_system(param, rk, sys == 0 ? 1 : 0, sub, q1, pf.l_last, pf.u_last, pf.den);
      const size_t off = yset_off(c, sys);
      if (int rc = push_factors(c, sub, off, pf.sub)) return rc;
      const size_t qoff = off + 3 * sub.l.size();
      if (int rc = stage_upload(c, qoff, q1.data(), q1.size())) return rc;
      pf.q1 = c->fac + qoff;
      if (sys == 0) {
        set.f[set.n] = pf;
        set.first_col[set.n] = 0;
        set.q[set.n++] = te->f.qt;
      } else {
        set.f[set.n] = pf;
        set.first_col[set.n] = 1;  // ux
        set.q[set.n++] = f.qx;
        set.f[set.n] = pf;
        set.first_col[set.n] = 0;  // uy
        set.q[set.n++] = f.qy;
      }
    }
    Prof pr(c, K_SOLVE_Y);
    SNS_CUDA(FORM(c, launch_solve_y_set)(c->g, set, c->stream));
  }
  if (impx || impy)
    if (int rc = end_factor_uploads(c)) return rc;
  {
    Prof pf(c, K_ADD_INC);
    if (with_t) SNS_CUDA(launch_add_increment(c->g, 0, te->f.t[te->cur], te->f.qt, te->f.t[out], c->stream));
    SNS_CUDA(launch_add_increment(c->g, 1, f.ux, f.qx, f.ux_alt, c->stream));
    SNS_CUDA(launch_add_increment(c->g, 0, f.uy, f.qy, f.uy_alt, c->stream));
  }
  if (with_t) te->cur = out;
  std::swap(f.ux, f.ux_alt);
  std::swap(f.uy, f.uy_alt);
  return SNS_OK;
}

static int poisson_forward(Context *c, const StageScalars &s, Fields &f) {
  Prof pf(c, K_POI_FWD);
  if (c->form == SNS_FORM_PARALLEL) {
    SNS_CUDA(launch_par_fwd(c->g, s, f.ux, f.uy, f.spec, c->stream));
  } else {
    SNS_CUDA(launch_poisson_fwd(c->g, s, f.ux, f.uy, f.spec, c->stream));
  }
  return SNS_OK;
}

static int poisson_rest(Context *c, const StageScalars &s, Fields &f) {
  if (c->form == SNS_FORM_PARALLEL) {
    {
      Prof pf(c, K_POI_PCR);
      SNS_CUDA(launch_par_tri(c->g, f.spec, c->par, c->stream));
      c->par.stale = 0;  // a test's stale wait applies to one launch
    }
    Prof pf(c, K_POI_BWD);
    SNS_CUDA(launch_par_bwd(c->g, s, f.spec, f.psi, c->stream));
    return SNS_OK;
  }
  {
    Prof pf(c, K_POI_TRI);
    SNS_CUDA(launch_poisson_tri(c->g, f.spec, c->stream));
  }
  {
    Prof pf(c, K_POI_BWD);
    SNS_CUDA(launch_poisson_bwd(c->g, s, f.spec, f.psi, c->stream));
  }
  return SNS_OK;
}

// Partition-method factors of the Poisson lines (host, once per context) for
// the parallel tridiagonal form. The form needs itot a multiple of 32 (one
// segment per lane) and the mean mode's last Thomas pivot to vanish, so that
// pinning that unknown to zero reproduces the reference's gauge of psi
// (src/linalg.c:36-38 zeroes the row): true on uniform grids, checked here.
static int parallel_prepare(Context *c) {
  if (c->par_ready) return SNS_OK;
  const int nx = c->nx, ny = c->ny, nh = c->g.nh;
  if (!parallel_tri_supported(nx, ny))
    return fail(SNS_ERR_UNSUPPORTED, "parallel tridiagonal form: itot=%d must be a multiple of 32 in [64, 14048]", nx);
  const double *dxf = c->dxf.data(), *dxc = c->dxc.data();
  std::vector<double> l_raw(nx), u_raw(nx), a(nx), cc(nx);
  for (int i = 1; i <= nx; i++) {
    l_raw[i - 1] = 1. / dxc[i - 1] / dxf[i - 1];  // src/fluid/compute_potential.c:118-119
    u_raw[i - 1] = 1. / dxc[i] / dxf[i - 1];
    a[i - 1] = i > 1 ? l_raw[i - 1] : 0.0;
    cc[i - 1] = i < nx ? u_raw[i - 1] : 0.0;
  }
  {
    // the mean mode's Thomas pivots: only the last one may vanish, and it must
    std::vector<double> d(nx), inv(nx), up(nx);
    for (int i = 0; i < nx; i++) d[i] = -l_raw[i] - u_raw[i] + poisson_eigenvalue(c->g.dy, ny, 0);
    d[0] += l_raw[0];
    d[nx - 1] += u_raw[nx - 1];
    factorize(nx, l_raw.data(), d.data(), u_raw.data(), inv.data(), up.data());
    bool ok = inv[nx - 1] == 0.0;
    for (int i = 1; i < nx - 1; i++) ok = ok && inv[i] != 0.0;
    if (!ok)
      return fail(SNS_ERR_UNSUPPORTED,
                  "parallel tridiagonal form: the mean mode's last pivot does not vanish on this grid "
                  "(the reference's gauge of psi cannot be pinned); use the Thomas form");
  }
  // per mode: inv, g = a inv, up, v, w (rows interleaved), then the PCR
  // coefficients; g takes the product by the sub-diagonal off the forward
  // elimination's dependent chain
  const size_t base = partition_stride(nx), stride = base + nx;
  const int m = nx / kPartSeg;
  std::vector<double> fac(stride * nh), blk(base), lo(nx), hi(nx);
  for (int x = 0; x < nx; x++) {
    lo[(size_t)(x % m) * kPartSeg + x / m] = a[x];
    hi[(size_t)(x % m) * kPartSeg + x / m] = cc[x];
  }
  for (int J = 0; J < nh; J++) {
    partition_factors(nx, a.data(), cc.data(), l_raw.data(), u_raw.data(), poisson_eigenvalue(c->g.dy, ny, J),
                      J == 0, true, blk.data());
    double *o = fac.data() + stride * J;
    std::copy(blk.begin(), blk.begin() + nx, o);                         // inv
    for (int i = 0; i < nx; i++) o[nx + i] = lo[i] * blk[i];            // g
    std::copy(blk.begin() + nx, blk.end(), o + 2 * (size_t)nx);         // up v w alpha beta rD
  }
  int rc = SNS_OK;
  if ((rc = upload(c, &c->par.fac, fac)) || (rc = upload(c, &c->par.lo, lo)) || (rc = upload(c, &c->par.hi, hi)))
    return rc;
  if ((rc = dev_alloc(c, &c->par.err, (size_t)1))) return rc;
  SNS_CUDA(cudaMemset(c->par.err, 0, sizeof(unsigned)));
  if (!c->par_err_host) SNS_CUDA(counted_malloc_host(&c->par_err_host, sizeof(unsigned)));
  *c->par_err_host = 0;
  c->par.stride = stride;
  c->par_ready = true;
  return SNS_OK;
}

// flag words of the fused launch, allocated and zeroed on first use
static int fused_prepare(Context *c) {
  if (c->fused_ready) return SNS_OK;
  int groups = 0, spans = 0;
  fused_layout(c->g, &groups, &spans);
  if (int rc = dev_alloc(c, &c->fz.fwd_done, (size_t)groups)) return rc;
  if (int rc = dev_alloc(c, &c->fz.bwd_cnt, (size_t)spans)) return rc;
  if (int rc = dev_alloc(c, &c->fz.err, (size_t)1)) return rc;
  SNS_CUDA(cudaMemsetAsync(c->fz.fwd_done, 0, sizeof(unsigned) * groups, c->stream));
  SNS_CUDA(cudaMemsetAsync(c->fz.bwd_cnt, 0, sizeof(unsigned long long) * spans, c->stream));
  SNS_CUDA(cudaMemsetAsync(c->fz.err, 0, sizeof(unsigned), c->stream));
  if (!c->fz_err_host) SNS_CUDA(counted_malloc_host(&c->fz_err_host, sizeof(unsigned)));
  *c->fz_err_host = 0;
  c->fz.epoch = 0;
  c->fused_ready = true;
  return SNS_OK;
}

// after a stream synchronisation: a fused launch whose wait gave up leaves
// its results undefined; report it, reset the flags and stop fusing. A
// parallel tridiagonal launch whose copy wait gave up left lines unsolved.
static int fused_check(Context *c) {
  if (c->par_ready && c->par_err_host && *c->par_err_host) {
    *c->par_err_host = 0;
    cudaMemsetAsync(c->par.err, 0, sizeof(unsigned), c->stream);
    return fail(SNS_ERR_STATE, "parallel tridiagonal launch: a copy wait gave up; results of that step are invalid");
  }
  if (!c->fused_ready || !c->fz_err_host || *c->fz_err_host == 0) return SNS_OK;
  const unsigned code = *c->fz_err_host;
  *c->fz_err_host = 0;
  c->fused = false;
  c->fused_ready = false;
  return fail(SNS_ERR_STATE, "fused Poisson launch: a %s wait gave up (code %u); results of that step are invalid",
              (code & 1) ? "sweep" : "worker", code);
}

static int fused_enqueue_err(Context *c) {
  if (c->fused_ready)
    SNS_CUDA(cudaMemcpyAsync(c->fz_err_host, c->fz.err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  if (c->par_ready)
    SNS_CUDA(cudaMemcpyAsync(c->par_err_host, c->par.err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  return SNS_OK;
}

// the Poisson solve as one fused launch when possible (temperature update
// folded in when t_out is given); *fused_out tells whether it ran. When it
// did not, nothing was launched and the caller runs the separate kernels.
static int try_fused(Context *c, const StageScalars &s, Fields &f, const double *t_in, double *t_out, double *at,
                       const double *ux_k, const double *uy_k, bool *fused_out) {
  *fused_out = false;
  if (c->fused && c->form == SNS_FORM_EXACT) {
    if (int rc = fused_prepare(c)) return rc;
    cudaError_t e;
    {
      Prof pf(c, K_POI_FUSED);
      e = launch_poisson_fused(c->g, s, f.ux, f.uy, f.spec, f.psi, t_in, t_out, at, ux_k, uy_k, c->fz, c->stream);
    }
    if (e == cudaSuccess) {
      *fused_out = true;
      return SNS_OK;
    }
    if (e != cudaErrorNotSupported && e != cudaErrorCooperativeLaunchTooLarge)
      return fail(SNS_ERR_CUDA, "fused Poisson launch: %s", cudaGetErrorString(e));
    cudaGetLastError();
    c->fused = false;  // this size cannot run fused here: three kernels from now on
  }
  return SNS_OK;
}

static int poisson(Context *c, const StageScalars &s, Fields &f) {
  bool fused = false;
  if (int rc = try_fused(c, s, f, nullptr, nullptr, nullptr, nullptr, nullptr, &fused)) return rc;
  if (fused) return SNS_OK;
  if (int rc = poisson_forward(c, s, f)) return rc;
  return poisson_rest(c, s, f);
}

// dt from the reduction results (src/param/decide_dt.c:11-101)
static void finish_decide_dt(param_t *param, const Context *c) {
  const double safe_factors[2] = {0.7, 0.9};
  const int nx = c->nx;
  const double Ra = param->Ra, Pr = param->Pr;
  const double diffusivity = fmax(sqrt(Pr) / sqrt(Ra), 1. / sqrt(Pr) / sqrt(Ra));
  const double lx = param->lx;
  const double *dxc = param->dxc;
  const double dy = param->dy;
  const double small = 1.e-8;
  double dt_adv = 5.e-2;
  // min_j DXC(i)/max(|ux(i,j)|, small) = DXC(i)/max(max_j |ux(i,j)|, small):
  // IEEE division is monotonic in the divisor, so this is the reference's value
  for (int i = 2; i <= nx; i++) {
    double m;
    std::memcpy(&m, &c->red_host[i - 1], sizeof m);
    const double vel = fmax(m, small);
    dt_adv = fmin(dt_adv, dxc[i - 1] / vel);
  }
  {
    double m;
    std::memcpy(&m, &c->red_host[nx], sizeof m);
    const double vel = fmax(m, small);
    dt_adv = fmin(dt_adv, dy / vel);
  }
  dt_adv *= safe_factors[0];
  double dx = lx;
  for (int i = 2; i <= nx; i++) dx = fmin(dx, dxc[i - 1]);
  double dt_dif_x = 0.25 / diffusivity * pow(dx, 2.);
  double dt_dif_y = 0.25 / diffusivity * pow(dy, 2.);
  dt_dif_x *= safe_factors[1];
  dt_dif_y *= safe_factors[1];
  double dt = 1.e-2;
  double optimal_wtime = DBL_MAX;
  int bx = -1, by = -1;
  for (int implicity = 0; implicity < 2; implicity++) {
    for (int implicitx = 0; implicitx < 2; implicitx++) {
      const double cand = implicitx ? implicity ? dt_adv : fmin(dt_adv, dt_dif_y)
                                    : implicity ? fmin(dt_adv, dt_dif_x) : fmin(dt_adv, fmin(dt_dif_x, dt_dif_y));
      const double niter = 1. / cand;
      const double wtime = param->expimp_wtimes[implicity][implicitx] * niter;
      if (wtime < optimal_wtime) {
        dt = cand;
        optimal_wtime = wtime;
        bx = implicitx;
        by = implicity;
      }
    }
  }
  param->implicitx = bx;
  param->implicity = by;
  param->dt = dt;
}

// word 0 of the reduction copied to the host: a NaN or infinity in ux, uy
// or p (set by the reduction kernels). The reference has no such check (its
// dt rule ignores NaN, src/param/decide_dt.c:38,46): the dt is decided as
// it would be, and the caller learns of the divergence from the status.
static int nonfinite_check(const Context *c, const param_t *param) {
  if (c->red_host[0] == 0) return SNS_OK;
  return fail(SNS_ERR_NONFINITE, "the velocity or pressure holds NaN or infinity (step %d, time %g)",
              param ? param->step : -1, param ? param->time : 0.0);
}

static int reduce_to_host(Context *c, Fields &f, bool launch) {
  // copied to the host at the end of the call that computed it
  if (!launch && c->red_host_version == c->version) return SNS_OK;
  if (launch) {
    SNS_CUDA(cudaMemsetAsync(f.colmax, 0, sizeof(unsigned long long) * (c->nx + 1), c->stream));
    Prof pf(c, K_UMAX);
    SNS_CUDA(launch_umax(c->g, f.ux, f.uy, f.colmax, f.uymax, c->stream));
  }
  SNS_CUDA(cudaMemcpyAsync(c->red_host, f.colmax, sizeof(unsigned long long) * (c->nx + 1), cudaMemcpyDeviceToHost,
                           c->stream));
  if (int rc = fused_enqueue_err(c)) return rc;
  SNS_CUDA(cudaStreamSynchronize(c->stream));
  if (int rc = fused_check(c)) return rc;
  c->red_host_version = c->version;
  return SNS_OK;
}

static bool same_scalars(const StageScalars &a, const StageScalars &b) {
  return a.adt == b.adt && a.bdt == b.bdt && a.gdt == b.gdt && a.has_b == b.has_b && a.kappa == b.kappa &&
         a.nu == b.nu && a.rgdt == b.rgdt && a.rny == b.rny && a.pcorr == b.pcorr;
}

// launches the deferred work of the reference-named calls (PendingTemp,
// PendingCorr) in call order: a temperature update is consumed before a
// correction can be deferred, so at most one of them waits
static int flush_pending(Context *c) {
  if (!c) return SNS_OK;
  if (TempExt *te = c->ptemp.te) {
    const PendingTemp pt = c->ptemp;
    c->ptemp = PendingTemp{};
    {
      Prof pf(c, K_TEMP);
      SNS_CUDA(FORM(c, launch_temp_update)(c->g, pt.s, 0, 0, te->f.t[te->cur], te->f.t[pt.out], te->f.at, nullptr, pt.ux_k,
                                  pt.uy_k, c->stream));
    }
    te->cur = pt.out;
  }
  if (FluidExt *fe = c->pcorr.fe) {
    const PendingCorr pc = c->pcorr;
    c->pcorr = PendingCorr{};
    Prof pf(c, K_CORR);
    SNS_CUDA(FORM(c, launch_correct)(c->g, pc.s, fe->f.psi, fe->f.ux, fe->f.uy, c->stream));
  }
  return SNS_OK;
}

static Context *ctx_of(const fluid_t *f, const temperature_t *t) {
  if (FluidExt *fe = f ? as_fluid(f) : nullptr) return fe->ctx;
  if (TempExt *te = t ? as_temp(t) : nullptr) return te->ctx;
  return nullptr;
}

}  // namespace sns

using namespace sns;

// =========================================================== C ABI
extern "C" {

const char *sns_last_error(void) { return g_error.c_str(); }
long long sns_kernel_launches(void) { return g_launches.load(); }
long long sns_allocations(void) { return g_allocs.load(); }

int sns_abi_layout(size_t *out, int n) {
  const size_t v[] = {sizeof(param_t),          offsetof(param_t, itot),    offsetof(param_t, dy),
                      offsetof(param_t, rkcoefs), offsetof(param_t, time),  offsetof(param_t, dt),
                      offsetof(param_t, step),  offsetof(param_t, expimp_wtimes), offsetof(param_t, timemax),
                      offsetof(param_t, log),   offsetof(param_t, stat),    sizeof(parallel_t),
                      sizeof(fluid_t),          offsetof(fluid_t, srcuyg),  sizeof(temperature_t),
                      sizeof(sns_case_desc),    offsetof(sns_case_desc, fixed_dt), offsetof(sns_case_desc, compensated)};
  const int m = (int)(sizeof v / sizeof v[0]);
  for (int k = 0; k < m && k < n; k++) out[k] = v[k];
  return m;
}

param_t *sns_param_create(int itot, int jtot, double ly, double stretch_in, double Ra, double Pr,
                          int with_temperature, int with_thermal_forcing) {
  if (itot < 2 || jtot < 2) {
    fail(SNS_ERR_ARG, "itot=%d jtot=%d", itot, jtot);
    return nullptr;
  }
  param_t *param = static_cast<param_t *>(calloc(1, sizeof(param_t)));
  if (!param) return nullptr;
  param->load_flow_field = false;
  param->with_temperature = with_temperature != 0;
  param->with_thermal_forcing = with_thermal_forcing != 0;
  param->timemax = 2.0e+2;
  param->wtimemax = 6.0e+2;
  param->itot = itot;
  param->jtot = jtot;
  param->lx = LX;
  param->ly = ly;
  param->stretch = stretch_in;
  param->Ra = Ra;
  param->Pr = Pr;
  // src/param/init.c:124-195
  param->xf = static_cast<double *>(calloc(itot + 1, sizeof(double)));
  param->xc = static_cast<double *>(calloc(itot + 2, sizeof(double)));
  param->dxf = static_cast<double *>(calloc(itot, sizeof(double)));
  param->dxc = static_cast<double *>(calloc(itot + 1, sizeof(double)));
  param->yf = static_cast<double *>(calloc(jtot + 1, sizeof(double)));
  param->yc = static_cast<double *>(calloc(jtot, sizeof(double)));
  make_grid(itot, jtot, param->lx, ly, stretch_in, param->xf, param->xc, param->dxf, param->dxc, param->yf, param->yc,
            &param->dy);
  // src/param/init.c:197-213
  param->rkcoefs[0].alpha = 32. / 60.;
  param->rkcoefs[0].beta = 0. / 60.;
  param->rkcoefs[1].alpha = 25. / 60.;
  param->rkcoefs[1].beta = -17. / 60.;
  param->rkcoefs[2].alpha = 45. / 60.;
  param->rkcoefs[2].beta = -25. / 60.;
  for (int rk = 0; rk < RKSTEPMAX; rk++) param->rkcoefs[rk].gamma = param->rkcoefs[rk].alpha + param->rkcoefs[rk].beta;
  param->expimp_wtimes[0][0] = 1.;
  param->expimp_wtimes[0][1] = 2.;
  param->expimp_wtimes[1][0] = 2.;
  param->expimp_wtimes[1][1] = 3.;
  return param;
}

int sns_param_destroy(param_t *param) {
  if (!param) return SNS_OK;
  free(param->xf);
  free(param->xc);
  free(param->dxf);
  free(param->dxc);
  free(param->yf);
  free(param->yc);
  free(param);
  return SNS_OK;
}

parallel_t *sns_parallel_create(void) {
  parallel_t *p = static_cast<parallel_t *>(calloc(1, sizeof(parallel_t)));
  if (!p) return nullptr;
  p->mpisize = 1;
  p->mpirank = 0;
  p->ymrank = 0;
  p->yprank = 0;
  srand(0);  // src/parallel/init.c:25 on rank 0
  return p;
}

int sns_parallel_destroy(parallel_t *parallel) {
  free(parallel);
  return SNS_OK;
}

fluid_t *fluid_init(const param_t *param, const parallel_t *parallel) {
  if (check_inputs(param, parallel) != SNS_OK) return nullptr;
  Context *c = acquire_context(param);
  if (!c) return nullptr;
  FluidExt *fe = static_cast<FluidExt *>(calloc(1, sizeof(FluidExt)));
  const int nx = param->itot, ny = param->jtot;
  const size_t nu = (size_t)(nx + 1) * (ny + 2), nc = (size_t)(nx + 2) * (ny + 2);
  const size_t sx = (size_t)(nx - 1) * ny, sc = (size_t)nx * ny;
  fe->magic = kFluidMagic;
  fe->ctx = c;
  fluid_t &h = fe->pub;
  h.ux = host_array(nu);
  h.uy = host_array(nc);
  h.p = host_array(nc);
  h.psi = host_array(nc);
  h.srcuxa = host_array(sx);
  h.srcuxb = host_array(sx);
  h.srcuxg = host_array(sx);
  h.srcuya = host_array(sc);
  h.srcuyb = host_array(sc);
  h.srcuyg = host_array(sc);
  Fields &f = fe->f;
  const size_t n = sc;
  int rc = SNS_OK;
  if ((rc = dev_alloc(c, &f.ux, n)) || (rc = dev_alloc(c, &f.uy, n)) || (rc = dev_alloc(c, &f.ux_alt, n)) ||
      (rc = dev_alloc(c, &f.uy_alt, n)) || (rc = dev_alloc(c, &f.p, n)) || (rc = dev_alloc(c, &f.psi, n)) ||
      (rc = dev_alloc(c, &f.aux, n)) || (rc = dev_alloc(c, &f.auy, n)) ||
      (rc = dev_alloc(c, &f.spec, (size_t)nx * c->g.jpitch)) || (rc = dev_alloc(c, &f.colmax, (size_t)nx + 1))) {
    fluid_finalise(&fe->pub);
    return nullptr;
  }
  f.uymax = f.colmax + nx;
  for (double *d : {f.ux, f.uy, f.ux_alt, f.uy_alt, f.p, f.psi, f.aux, f.auy}) cudaMemsetAsync(d, 0, n * sizeof(double), c->stream);
  cudaMemsetAsync(f.spec, 0, (size_t)nx * c->g.jpitch * sizeof(double2), c->stream);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    fail(SNS_ERR_CUDA, "fluid_init: %s", cudaGetErrorString(cudaGetLastError()));
    fluid_finalise(&fe->pub);
    return nullptr;
  }
  // src/fluid/init.c:52-81: zero fields with boundary and halo values
  host_bc_ux(nx, ny, h.ux);
  host_bc_uy(nx, ny, h.uy);
  host_bc_p(nx, ny, h.p);
  return &fe->pub;
}

int fluid_finalise(fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  if (!fe) return fail(SNS_ERR_ARG, "fluid_finalise: not a fluid_t from fluid_init");
  if (int rc = flush_pending(fe->ctx)) return rc;
  fluid_t &h = fe->pub;
  for (double *p : {h.ux, h.uy, h.p, h.psi, h.srcuxa, h.srcuxb, h.srcuxg, h.srcuya, h.srcuyb, h.srcuyg}) host_free(p);
  Context *c = fe->ctx;
  if (c) {
    cudaStreamSynchronize(c->stream);
    std::lock_guard<std::mutex> lk(g_mu);
    // this object's device arrays
    std::vector<void *> mine = {fe->f.ux, fe->f.uy, fe->f.ux_alt, fe->f.uy_alt, fe->f.p, fe->f.psi,
                                fe->f.aux, fe->f.auy, fe->f.spec, fe->f.colmax, fe->f.qx, fe->f.qy};
    for (void *p : mine) {
      if (!p) continue;
      auto it = std::find(c->allocs.begin(), c->allocs.end(), p);
      if (it != c->allocs.end()) {
        cudaFree(p);
        c->allocs.erase(it);
      }
    }
  }
  fe->magic = 0;
  free(fe);
  if (c) release_context(c);
  return SNS_OK;
}

temperature_t *temperature_init(const param_t *param, const parallel_t *parallel) {
  if (check_inputs(param, parallel) != SNS_OK) return nullptr;
  Context *c = acquire_context(param);
  if (!c) return nullptr;
  TempExt *te = static_cast<TempExt *>(calloc(1, sizeof(TempExt)));
  const int nx = param->itot, ny = param->jtot;
  const size_t nc = (size_t)(nx + 2) * (ny + 2), sx = (size_t)(nx - 1) * ny, sc = (size_t)nx * ny;
  te->magic = kTempMagic;
  te->ctx = c;
  te->cur = 0;
  te->snap = -2;
  temperature_t &h = te->pub;
  h.temp = host_array(nc);
  h.tempforcex = host_array(sx);
  h.srctempa = host_array(sc);
  h.srctempb = host_array(sc);
  h.srctempg = host_array(sc);
  // src/temperature/init.c:30-41: linear profile + rand() noise
  {
    const double factor = 0.1;
    const double *xc = param->xc;
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) {
        const double x = xc[i];
        const double r = -0.5 + 1. * rand() / RAND_MAX;
        h.temp[(size_t)j * (nx + 2) + i] = (TEMP_XP - TEMP_XM) * x + TEMP_XM + factor * r;
      }
    host_bc_temp(nx, ny, h.temp);
  }
  int rc = SNS_OK;
  for (int k = 0; k < 3 && rc == SNS_OK; k++) rc = dev_alloc(c, &te->f.t[k], sc);
  if (rc == SNS_OK) rc = dev_alloc(c, &te->f.at, sc);
  if (rc != SNS_OK) {
    temperature_finalise(&te->pub);
    return nullptr;
  }
  for (int k = 0; k < 3; k++) cudaMemsetAsync(te->f.t[k], 0, sc * sizeof(double), c->stream);
  cudaMemsetAsync(te->f.at, 0, sc * sizeof(double), c->stream);
  if (upload_field(c, te->f.t[0], h.temp, nx + 2, 1, 0) != SNS_OK) {
    temperature_finalise(&te->pub);
    return nullptr;
  }
  return &te->pub;
}

int temperature_finalise(temperature_t *temperature) {
  TempExt *te = as_temp(temperature);
  if (!te) return fail(SNS_ERR_ARG, "temperature_finalise: not a temperature_t from temperature_init");
  if (int rc = flush_pending(te->ctx)) return rc;
  temperature_t &h = te->pub;
  for (double *p : {h.temp, h.tempforcex, h.srctempa, h.srctempb, h.srctempg}) host_free(p);
  Context *c = te->ctx;
  if (c) {
    cudaStreamSynchronize(c->stream);
    std::lock_guard<std::mutex> lk(g_mu);
    std::vector<void *> mine = {te->f.t[0], te->f.t[1], te->f.t[2], te->f.at, te->f.qt};
    for (void *p : mine) {
      if (!p) continue;
      auto it = std::find(c->allocs.begin(), c->allocs.end(), p);
      if (it != c->allocs.end()) {
        cudaFree(p);
        c->allocs.erase(it);
      }
    }
  }
  te->magic = 0;
  free(te);
  if (c) release_context(c);
  return SNS_OK;
}

int fluid_update_boundaries_ux(const param_t *param, const parallel_t *parallel, double *ux) {
  if (!param || !ux) return fail(SNS_ERR_ARG, "NULL argument");
  (void)parallel;
  host_bc_ux(param->itot, param->jtot, ux);
  return SNS_OK;
}

int fluid_update_boundaries_uy(const param_t *param, const parallel_t *parallel, double *uy) {
  if (!param || !uy) return fail(SNS_ERR_ARG, "NULL argument");
  (void)parallel;
  host_bc_uy(param->itot, param->jtot, uy);
  return SNS_OK;
}

int fluid_update_boundaries_p(const param_t *param, const parallel_t *parallel, double *p) {
  if (!param || !p) return fail(SNS_ERR_ARG, "NULL argument");
  (void)parallel;
  host_bc_p(param->itot, param->jtot, p);
  return SNS_OK;
}

int temperature_update_boundaries_temp(const param_t *param, const parallel_t *parallel, double *temp) {
  if (!param || !temp) return fail(SNS_ERR_ARG, "NULL argument");
  (void)parallel;
  host_bc_temp(param->itot, param->jtot, temp);
  return SNS_OK;
}

int temperature_compute_force(const param_t *param, const parallel_t *parallel, temperature_t *temperature) {
  TempExt *te = as_temp(temperature);
  if (!param || !parallel || !te) return fail(SNS_ERR_ARG, "temperature_compute_force: bad argument");
  if (int rc = flush_pending(te->ctx)) return rc;
  te->snap = param->with_thermal_forcing ? te->cur : -1;
  return SNS_OK;
}

int temperature_update_temp(const param_t *param, const parallel_t *parallel, const int rkstep, const fluid_t *fluid,
                            temperature_t *temperature) {
  TempExt *te = as_temp(temperature);
  FluidExt *fe = as_fluid(fluid);
  if (!param || !parallel || !te || !fe || rkstep < 0 || rkstep >= RKSTEPMAX)
    return fail(SNS_ERR_ARG, "temperature_update_temp: bad argument");
  Context *c = te->ctx;
  if (int rc = flush_pending(c)) return rc;
  if ((c->form == SNS_FORM_PARALLEL || c->fused) && fe->ctx == c && !param->implicitx && !param->implicity) {
    // explicit: launched by the next fluid_compute_potential, inside the
    // fused launch (exact form) or beside the Poisson kernels (parallel
    // form); it reads the velocity of now, which that call's velocity update
    // leaves in place
    PendingTemp &pt = c->ptemp;
    pt.te = te;
    pt.rk = rkstep;
    pt.out = 0;
    while (pt.out == te->cur || pt.out == te->snap) pt.out++;
    pt.s = stage_scalars(param, rkstep);
    pt.ux_k = fe->f.ux;
    pt.uy_k = fe->f.uy;
    return SNS_OK;
  }
  return do_temp_update(param, rkstep, fe, te);
}

int fluid_update_velocity(const param_t *param, const parallel_t *parallel, const int rkstep, fluid_t *fluid,
                          const temperature_t *temperature) {
  FluidExt *fe = as_fluid(fluid);
  if (!param || !parallel || !fe || rkstep < 0 || rkstep >= RKSTEPMAX)
    return fail(SNS_ERR_ARG, "fluid_update_velocity: bad argument");
  const TempExt *te = temperature ? as_temp(temperature) : nullptr;
  Context *c = fe->ctx;
  // a deferred temperature update may wait across this call (it reads the
  // velocity buffer this call leaves alone) but not across a second one
  if (c->pcorr.fe || (c->ptemp.te && c->ptemp.ux_k == fe->f.ux_alt))
    if (int rc = flush_pending(c)) return rc;
  c->version++;
  return do_velocity_update(param, rkstep, fe, te);
}

int fluid_compute_potential(const param_t *param, const parallel_t *parallel, const int rkstep, fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  if (!param || !parallel || !fe || rkstep < 0 || rkstep >= RKSTEPMAX)
    return fail(SNS_ERR_ARG, "fluid_compute_potential: bad argument");
  Context *c = fe->ctx;
  const StageScalars s = stage_scalars(param, rkstep);
  PendingTemp &pt = c->ptemp;
  if (pt.te && pt.rk == rkstep && same_scalars(pt.s, s)) {
    // the substage's deferred temperature update inside the fused launch
    TempExt *te = pt.te;
    bool fused = false;
    if (int rc = try_fused(c, s, fe->f, te->f.t[te->cur], te->f.t[pt.out], te->f.at, pt.ux_k, pt.uy_k, &fused))
      return rc;
    if (fused) {
      te->cur = pt.out;
      pt = PendingTemp{};
      return SNS_OK;
    }
    if (c->form == SNS_FORM_PARALLEL && !c->pcorr.fe) {
      // the parallel form: the deferred temperature update on the side
      // stream beside the Poisson kernels, as sns_run runs it; the main
      // stream waits for it before anything later in call order
      const PendingTemp p = pt;
      pt = PendingTemp{};
      SNS_CUDA(cudaEventRecord(c->ev_fwd, c->stream));
      SNS_CUDA(cudaStreamWaitEvent(c->side, c->ev_fwd, 0));
      {
        Prof pf(c, K_TEMP, c->side);
        SNS_CUDA(FORM(c, launch_temp_update)(c->g, p.s, 0, 0, te->f.t[te->cur], te->f.t[p.out], te->f.at, nullptr, p.ux_k,
                                             p.uy_k, c->side));
      }
      SNS_CUDA(cudaEventRecord(c->ev_temp, c->side));
      te->cur = p.out;
      if (int rc = poisson(c, s, fe->f)) return rc;
      SNS_CUDA(cudaStreamWaitEvent(c->stream, c->ev_temp, 0));
      return SNS_OK;
    }
  }
  if (int rc = flush_pending(c)) return rc;
  if (int rc = poisson(c, s, fe->f)) return rc;
  return SNS_OK;
}

int fluid_correct_velocity(const param_t *param, const parallel_t *parallel, const int rkstep, fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  if (!param || !parallel || !fe || rkstep < 0 || rkstep >= RKSTEPMAX)
    return fail(SNS_ERR_ARG, "fluid_correct_velocity: bad argument");
  Context *c = fe->ctx;
  if (int rc = flush_pending(c)) return rc;
  c->version++;
  // launched with the next fluid_update_pressure of the substage (one kernel
  // for both, the one sns_run uses), or by the next other call
  PendingCorr &pc = c->pcorr;
  pc.fe = fe;
  pc.rk = rkstep;
  pc.impx = param->implicitx;
  pc.impy = param->implicity;
  pc.s = stage_scalars(param, rkstep);
  return SNS_OK;
}

int fluid_update_pressure(const param_t *param, const parallel_t *parallel, const int rkstep, fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  if (!param || !parallel || !fe || rkstep < 0 || rkstep >= RKSTEPMAX)
    return fail(SNS_ERR_ARG, "fluid_update_pressure: bad argument");
  Context *c = fe->ctx;
  const StageScalars s = stage_scalars(param, rkstep);
  PendingCorr &pc = c->pcorr;
  if (pc.fe == fe && pc.rk == rkstep && pc.impx == param->implicitx && pc.impy == param->implicity &&
      same_scalars(pc.s, s)) {
    pc = PendingCorr{};
    // the last substage also leaves the max-|u| reduction for the next
    // param_decide_dt (the velocity is final for the step)
    const bool red = rkstep == RKSTEPMAX - 1;
    if (red) SNS_CUDA(cudaMemsetAsync(fe->f.colmax, 0, sizeof(unsigned long long) * (c->nx + 1), c->stream));
    {
      Prof pf(c, K_CORR_PRES);
      SNS_CUDA(FORM(c, launch_correct_pressure)(c->g, s, param->implicitx, param->implicity, fe->f.psi, fe->f.ux, fe->f.uy,
                                       fe->f.p, red ? fe->f.colmax : nullptr, red ? fe->f.uymax : nullptr,
                                       c->stream));
    }
    if (red) c->red_version = c->version;
    return SNS_OK;
  }
  if (int rc = flush_pending(c)) return rc;
  Prof pf(c, K_PRES);
  SNS_CUDA(FORM(c, launch_pressure)(c->g, s, param->implicitx, param->implicity, fe->f.psi, fe->f.p, c->stream));
  return SNS_OK;
}

// ------------------------------------------------------------ cost model
int sns_cost_model(int itot, int jtot, int sm_count, double clock_ghz, int with_temperature, double out[4]) {
  if (itot < 2 || jtot < 2 || sm_count < 1 || !(clock_ghz > 0.0) || !out)
    return fail(SNS_ERR_ARG, "sns_cost_model: bad argument");
  double w[2][2];
  cost_model(itot, jtot, sm_count, clock_ghz * 1e9, with_temperature != 0, w);
  for (int k = 0; k < 4; k++) out[k] = w[k / 2][k % 2];
  return SNS_OK;
}

// src/param/estimate_cost.c:44-74 with the deterministic model in place of
// wall-clock emulation: expimp_wtimes[implicity][implicitx] in seconds per
// substage for the current device
int param_estimate_cost(param_t *param, const parallel_t *parallel) {
  if (!param || !parallel) return fail(SNS_ERR_ARG, "param_estimate_cost: bad argument");
  int dev = 0, sms = 0, khz = 0;
  SNS_CUDA(cudaGetDevice(&dev));
  SNS_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  SNS_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
  cost_model(param->itot, param->jtot, sms, khz * 1e3, param->with_temperature, param->expimp_wtimes);
  return SNS_OK;
}

// the reference's emulate() (src/param/estimate_cost.c:11-42) timed with CUDA
// events: per treatment, fresh fields from fluid_init / temperature_init
// (which draw rand() like the reference's), dt = 1e-8, `reps` substages rk = 0
// through the reference-named calls after one warm-up; seconds per substage
int sns_measure_cost(param_t *param, const parallel_t *parallel, int reps, double out[4]) {
  if (!param || !parallel || reps < 1 || !out) return fail(SNS_ERR_ARG, "sns_measure_cost: bad argument");
  const double dt0 = param->dt;
  const int ix0 = param->implicitx, iy0 = param->implicity;
  int rc = SNS_OK;
  for (int k = 0; k < 4 && rc == SNS_OK; k++) {
    param->dt = 1.e-8;
    param->implicitx = k % 2;
    param->implicity = k / 2;
    fluid_t *fl = fluid_init(param, parallel);
    temperature_t *tm = fl ? temperature_init(param, parallel) : nullptr;
    if (!fl || !tm) {
      if (fl) fluid_finalise(fl);
      rc = SNS_ERR_OOM;
      break;
    }
    Context *c = as_fluid(fl)->ctx;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto substage = [&]() -> int {
      int r = SNS_OK;
      if (param->with_temperature) {
        if ((r = temperature_compute_force(param, parallel, tm)) || (r = temperature_update_temp(param, parallel, 0, fl, tm)))
          return r;
      }
      if ((r = fluid_update_velocity(param, parallel, 0, fl, tm)) || (r = fluid_compute_potential(param, parallel, 0, fl)) ||
          (r = fluid_correct_velocity(param, parallel, 0, fl)) || (r = fluid_update_pressure(param, parallel, 0, fl)))
        return r;
      return SNS_OK;
    };
    float ms = 0.f;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) rc = SNS_ERR_CUDA;
    if (rc == SNS_OK) rc = substage();
    if (rc == SNS_OK && cudaEventRecord(e0, c->stream) != cudaSuccess) rc = SNS_ERR_CUDA;
    for (int r = 0; r < reps && rc == SNS_OK; r++) rc = substage();
    if (rc == SNS_OK && (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
                         cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
      rc = SNS_ERR_CUDA;
    out[k] = 1e-3 * ms / reps;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    temperature_finalise(tm);
    fluid_finalise(fl);
  }
  param->dt = dt0;
  param->implicitx = ix0;
  param->implicity = iy0;
  if (rc != SNS_OK) return fail(rc, "sns_measure_cost: %s", sns_last_error());
  return SNS_OK;
}

int param_decide_dt(param_t *param, const parallel_t *parallel, const fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  if (!param || !parallel || !fe) return fail(SNS_ERR_ARG, "param_decide_dt: bad argument");
  Context *c = fe->ctx;
  if (int rc = flush_pending(c)) return rc;
  if (int rc = reduce_to_host(c, fe->f, c->red_version != c->version)) return rc;
  c->red_version = c->version;
  finish_decide_dt(param, fe->ctx);
  return nonfinite_check(c, param);
}

// Device -> host. state_only: ux, uy, p and temp alone, the whole input and
// output of a time step (psi is rewritten before it is read, the explicit
// sources of the last substage are multiplied by zero at the first one, and
// tempforcex is recomputed from temp); the other host arrays keep what they
// held.
static int sync_to_host_impl(const param_t *param, fluid_t *fluid, temperature_t *temperature, bool state_only,
                             const char *fn) {
  if (!param) return fail(SNS_ERR_ARG, "%s: NULL param", fn);
  if (int rc = flush_pending(ctx_of(fluid, temperature))) return rc;
  const int nx = param->itot, ny = param->jtot;
  FluidExt *fe = nullptr;
  TempExt *te = nullptr;
  if (fluid && !(fe = as_fluid(fluid))) return fail(SNS_ERR_ARG, "%s: foreign fluid_t", fn);
  if (temperature && !(te = as_temp(temperature))) return fail(SNS_ERR_ARG, "%s: foreign temperature_t", fn);
  // every copy is enqueued before one wait (a wait between the fluid and the
  // temperature copies left the link idle meanwhile). Pinned host arrays are
  // written in place by copy kernels: the reference-layout fields whole, in
  // one linear pass of aligned 16-byte pairs with their halo and wall values
  // (full cache lines on the link), the sources row by row; arrays that are
  // not pinned go through 2D DMA.
  int rc = SNS_OK;
  const bool same = fe && te && fe->ctx == te->ctx;
  LinList F{};
  F.nx = nx;
  F.ny = ny;
  XferList L{};
  L.rows = ny;
  bool direct = true;
  if (fe) {
    fluid_t &h = fe->pub;
    direct = lin_field(F, fe->f.ux, h.ux, nx + 1, LIN_UX) && lin_field(F, fe->f.uy, h.uy, nx + 2, LIN_UY) &&
             lin_field(F, fe->f.p, h.p, nx + 2, LIN_P);
    if (!state_only)
      direct = direct && lin_field(F, fe->f.psi, h.psi, nx + 2, LIN_P) &&
               xfer_src_down(L, nx, fe->f.aux, h.srcuxa, 1) && xfer_src_down(L, nx, fe->f.auy, h.srcuya, 0);
  }
  if (te) {
    temperature_t &h = te->pub;
    direct = direct && lin_field(F, te->f.t[te->cur], h.temp, nx + 2, LIN_T) &&
             (state_only || xfer_src_down(L, nx, te->f.at, h.srctempa, 0));
  }
  direct = direct && (same || !fe || !te);
  if (direct) {
    cudaStream_t st = (fe ? fe->ctx : te->ctx)->stream;
    if (F.n > 0) SNS_CUDA(launch_lin(F, 1, st));
    if (L.n > 0) SNS_CUDA(launch_xfer(L, st));
  } else if (fe) {
    Context *c = fe->ctx;
    fluid_t &h = fe->pub;
    if ((rc = download(c, fe->f.ux, h.ux, nx + 1, 0, 1)) || (rc = download(c, fe->f.uy, h.uy, nx + 2, 1, 0)) ||
        (rc = download(c, fe->f.p, h.p, nx + 2, 1, 0)))
      return rc;
    if (!state_only &&
        ((rc = download(c, fe->f.psi, h.psi, nx + 2, 1, 0)) || (rc = download_src(c, fe->f.aux, h.srcuxa, 1)) ||
         (rc = download_src(c, fe->f.auy, h.srcuya, 0))))
      return rc;
  }
  int snap = -1;
  double *tf_alias = nullptr;
  if (te) {
    Context *c = te->ctx;
    temperature_t &h = te->pub;
    if (!direct && ((rc = download(c, te->f.t[te->cur], h.temp, nx + 2, 1, 0)) ||
                    (!state_only && (rc = download_src(c, te->f.at, h.srctempa, 0)))))
      return rc;
    snap = state_only ? -1 : te->snap;
    tf_alias = snap >= 0 ? dev_alias(h.tempforcex) : nullptr;
    if (tf_alias) {
      SNS_CUDA(launch_tempforce_to_host(c->g, te->f.t[snap], tf_alias, c->stream));
    } else if (snap >= 0) {
      if (int rc2 = fetch(c, te->f.t[snap])) return rc2;
    }
  }
  if (fe) SNS_CUDA(cudaStreamSynchronize(fe->ctx->stream));
  if (te && (!fe || te->ctx != fe->ctx)) SNS_CUDA(cudaStreamSynchronize(te->ctx->stream));
  // the copy kernels wrote the halo and wall values; DMA copies leave them to the host
  if (fe && !direct) {
    fluid_t &h = fe->pub;
    host_bc_ux(nx, ny, h.ux);
    host_bc_uy(nx, ny, h.uy);
    host_bc_p(nx, ny, h.p);
    if (!state_only) host_bc_p(nx, ny, h.psi);
  }
  if (te) {
    Context *c = te->ctx;
    temperature_t &h = te->pub;
    if (!direct) host_bc_temp(nx, ny, h.temp);
    if (snap >= 0 && !tf_alias) {
      // tempforcex (src/temperature/force.c:17-23) from the snapshot buffer
      for (int j = 1; j <= ny; j++)
        for (int i = 2; i <= nx; i++) {
          const double tm = c->staging[(size_t)(j - 1) * nx + (i - 2)], tp = c->staging[(size_t)(j - 1) * nx + (i - 1)];
          h.tempforcex[(size_t)(j - 1) * (nx - 1) + (i - 2)] = 0.5 * tm + 0.5 * tp;
        }
    }
  }
  return SNS_OK;
}

int sns_sync_to_host(const param_t *param, fluid_t *fluid, temperature_t *temperature) {
  return sync_to_host_impl(param, fluid, temperature, false, "sns_sync_to_host");
}

int sns_sync_state_to_host(const param_t *param, fluid_t *fluid, temperature_t *temperature) {
  return sync_to_host_impl(param, fluid, temperature, true, "sns_sync_state_to_host");
}

// Host -> device: the pinned host arrays are read in place by one copy
// kernel for all fields (strided 2D DMA of ~4 KB rows runs at less than half
// the link rate); arrays that are not pinned go through 2D DMA copies.
// state_only: ux, uy, p and temp alone; the device keeps its psi and sources
// and the buoyancy is recomputed from the uploaded temp.
static int sync_to_device_impl(const param_t *param, fluid_t *fluid, temperature_t *temperature, bool state_only,
                               const char *fn) {
  if (!param) return fail(SNS_ERR_ARG, "%s: NULL param", fn);
  if (int rc = flush_pending(ctx_of(fluid, temperature))) return rc;
  const int nx = param->itot;
  FluidExt *fe = nullptr;
  TempExt *te = nullptr;
  if (fluid && !(fe = as_fluid(fluid))) return fail(SNS_ERR_ARG, "%s: foreign fluid_t", fn);
  if (temperature && !(te = as_temp(temperature))) return fail(SNS_ERR_ARG, "%s: foreign temperature_t", fn);
  if (fe && te && fe->ctx != te->ctx) return fail(SNS_ERR_ARG, "%s: fluid and temperature of different cases", fn);
  Context *c = fe ? fe->ctx : te ? te->ctx : nullptr;
  if (!c) return SNS_OK;
  c->version++;
  // pinned host arrays are read in place by copy kernels: the
  // reference-layout fields whole, in one linear pass of aligned 16-byte
  // pairs (full cache lines on the link; only the interior is kept), the
  // sources row by row
  LinList F{};
  F.nx = nx;
  F.ny = c->ny;
  XferList L{};
  L.rows = c->ny;
  bool direct = true;
  if (fe) {
    const fluid_t &h = fe->pub;
    direct = lin_field(F, fe->f.ux, h.ux, nx + 1, LIN_UX) && lin_field(F, fe->f.uy, h.uy, nx + 2, LIN_UY) &&
             lin_field(F, fe->f.p, h.p, nx + 2, LIN_P);
    if (!state_only)
      direct = direct && lin_field(F, fe->f.psi, h.psi, nx + 2, LIN_P) &&
               xfer_src(L, nx, fe->f.aux, h.srcuxa, 1) && xfer_src(L, nx, fe->f.auy, h.srcuya, 0);
  }
  if (te) {
    te->cur = 0;
    te->snap = -2;
    const temperature_t &h = te->pub;
    direct = direct && lin_field(F, te->f.t[0], h.temp, nx + 2, LIN_T) &&
             (state_only || xfer_src(L, nx, te->f.at, h.srctempa, 0));
  }
  if (direct) {
    if (F.n > 0) SNS_CUDA(launch_lin(F, 0, c->stream));
    if (L.n > 0) SNS_CUDA(launch_xfer(L, c->stream));
  } else {
    int rc = SNS_OK;
    if (fe) {
      const fluid_t &h = fe->pub;
      if ((rc = upload_field(c, fe->f.ux, h.ux, nx + 1, 0, 1)) || (rc = upload_field(c, fe->f.uy, h.uy, nx + 2, 1, 0)) ||
          (rc = upload_field(c, fe->f.p, h.p, nx + 2, 1, 0)))
        return rc;
      if (!state_only &&
          ((rc = upload_field(c, fe->f.psi, h.psi, nx + 2, 1, 0)) || (rc = upload_src(c, fe->f.aux, h.srcuxa, 1)) ||
           (rc = upload_src(c, fe->f.auy, h.srcuya, 0))))
        return rc;
    }
    if (te) {
      const temperature_t &h = te->pub;
      if ((rc = upload_field(c, te->f.t[0], h.temp, nx + 2, 1, 0)) ||
          (!state_only && (rc = upload_src(c, te->f.at, h.srctempa, 0))))
        return rc;
    }
  }
  // the new velocity's max-|u| reduction and its copy to the host inside this
  // call's wait: the next param_decide_dt / sns_run decides dt without a
  // launch and a round trip of its own
  if (fe) {
    SNS_CUDA(cudaMemsetAsync(fe->f.colmax, 0, sizeof(unsigned long long) * (c->nx + 1), c->stream));
    {
      Prof pf(c, K_UMAX);
      SNS_CUDA(launch_umax(c->g, fe->f.ux, fe->f.uy, fe->f.colmax, fe->f.uymax, c->stream));
    }
    SNS_CUDA(cudaMemcpyAsync(c->red_host, fe->f.colmax, sizeof(unsigned long long) * (c->nx + 1),
                             cudaMemcpyDeviceToHost, c->stream));
  }
  SNS_CUDA(cudaStreamSynchronize(c->stream));
  if (fe) {
    c->red_version = c->version;
    c->red_host_version = c->version;
  }
  return SNS_OK;
}

int sns_sync_to_device(const param_t *param, fluid_t *fluid, temperature_t *temperature) {
  return sync_to_device_impl(param, fluid, temperature, false, "sns_sync_to_device");
}

int sns_sync_state_to_device(const param_t *param, fluid_t *fluid, temperature_t *temperature) {
  return sync_to_device_impl(param, fluid, temperature, true, "sns_sync_state_to_device");
}

int sns_diagnostics(const param_t *param, const fluid_t *fluid, const temperature_t *temperature, double out[11]) {
  FluidExt *fe = as_fluid(fluid);
  TempExt *te = as_temp(temperature);
  if (!param || !fe || !te || !out) return fail(SNS_ERR_ARG, "sns_diagnostics: bad argument");
  Context *c = fe->ctx;
  if (int rc = flush_pending(c)) return rc;
  const int nx = c->nx, ny = c->ny;
  const size_t words = diag_partials_words(nx, ny);
  if (!c->diag)
    if (int rc = dev_alloc(c, &c->diag, words)) return rc;
  const double Ra = param->Ra, Pr = param->Pr;
  const DiagArgs<double> a{nx, ny, param->dy, param->ly, sqrt(Pr) * sqrt(Ra), sqrt(Pr) / sqrt(Ra),
                           1. / sqrt(Pr) / sqrt(Ra), c->g.dxf, c->g.dxc, fe->f.ux, fe->f.uy, te->f.t[te->cur]};
  int nb = 0;
  SNS_CUDA(launch_diag(a, c->diag, &nb, c->stream));
  count_launches(1);
  std::vector<double> h(words);
  SNS_CUDA(cudaMemcpyAsync(h.data(), c->diag, sizeof(double) * words, cudaMemcpyDeviceToHost, c->stream));
  SNS_CUDA(cudaStreamSynchronize(c->stream));
  diag_finish(h.data(), nb, param->ly, out);
  return SNS_OK;
}

// ------------------------------------------------------------ checkpoints
// The reference's save layout (src/save.c:13-68, src/fileio.c:226-345): one
// NPY file per quantity; 2D fields hold rows j = 1..jtot of the reference
// arrays, wall and halo columns included.
struct CheckpointJob {
  std::string dir;
  int step, itot, jtot, with_t, device;
  double time, lx, ly, Ra, Pr;
  std::vector<double> xf, xc, yf, yc;
};

static int write_checkpoint(const CheckpointJob &J, const double *snap, std::string *err) {
  const int nx = J.itot, ny = J.jtot;
  const size_t cells = (size_t)nx * ny;
  if (make_dirs(J.dir.c_str(), err)) return 1;
  auto path = [&](const char *name) { return J.dir + "/" + name + ".npy"; };
  int rc = 0;
  auto w0 = [&](const char *name, const char *dtype, const void *v, size_t n) {
    if (!rc) rc = npy_write(path(name).c_str(), dtype, 0, nullptr, v, n, err);
  };
  auto w1 = [&](const char *name, const std::vector<double> &v) {
    const size_t shape[1] = {v.size()};
    if (!rc) rc = npy_write(path(name).c_str(), "'float64'", 1, shape, v.data(), sizeof(double) * v.size(), err);
  };
  w0("step", "'int32'", &J.step, sizeof(int));
  w0("itot", "'int32'", &J.itot, sizeof(int));
  w0("jtot", "'int32'", &J.jtot, sizeof(int));
  w0("time", "'float64'", &J.time, sizeof(double));
  w0("lx", "'float64'", &J.lx, sizeof(double));
  w0("ly", "'float64'", &J.ly, sizeof(double));
  w0("Ra", "'float64'", &J.Ra, sizeof(double));
  w0("Pr", "'float64'", &J.Pr, sizeof(double));
  w1("xf", J.xf);
  w1("xc", J.xc);
  w1("yf", J.yf);
  w1("yc", J.yc);
  // field rows: walls / halo columns by the boundary rules the reference
  // applied after each update (src/fluid/boundary_conditions.c:6-55,
  // src/temperature/boundary_conditions.c:6-21)
  auto field = [&](const char *name, const double *d, int kind) {
    if (rc) return;
    const int w = kind == 0 ? nx + 1 : nx + 2;
    std::vector<double> rows((size_t)ny * w);
    for (int j = 0; j < ny; j++) {
      double *r = rows.data() + (size_t)j * w;
      const double *src = d + (size_t)j * nx;
      if (kind == 0) {  // ux, i = 1..nx+1: dense x = 0..nx-1 is i = 1..nx (x = 0 the wall)
        std::memcpy(r, src, sizeof(double) * nx);
        r[nx] = 0.;
        r[0] = 0.;
      } else {
        std::memcpy(r + 1, src, sizeof(double) * nx);
        if (kind == 1) {  // uy: no-slip walls
          r[0] = 0.;
          r[nx + 1] = 0.;
        } else if (kind == 2) {  // p: Neumann
          r[0] = r[1];
          r[nx + 1] = r[nx];
        } else {  // temperature: fixed wall values
          r[0] = TEMP_XM;
          r[nx + 1] = TEMP_XP;
        }
      }
    }
    const size_t shape[2] = {(size_t)ny, (size_t)w};
    rc = npy_write(path(name).c_str(), "'float64'", 2, shape, rows.data(), sizeof(double) * rows.size(), err);
  };
  field("ux", snap, 0);
  field("uy", snap + cells, 1);
  field("p", snap + 2 * cells, 2);
  if (J.with_t) field("temp", snap + 3 * cells, 3);
  return rc;
}

int sns_checkpoint(const param_t *param, const fluid_t *fluid, const temperature_t *temperature, const char *dirname) {
  FluidExt *fe = as_fluid(fluid);
  TempExt *te = temperature ? as_temp(temperature) : nullptr;
  if (!param || !fe || !dirname || (temperature && !te)) return fail(SNS_ERR_ARG, "sns_checkpoint: bad argument");
  Context *c = fe->ctx;
  if (int rc = flush_pending(c)) return rc;
  if (c->ck_thread.joinable()) c->ck_thread.join();  // one checkpoint in flight per solver
  if (c->ck_status != SNS_OK) {
    // the previous checkpoint failed and nobody collected its error: report
    // it now (once) instead of starting a new snapshot over it
    const int rc = c->ck_status;
    c->ck_status = SNS_OK;
    return fail(rc, "sns_checkpoint: the previous checkpoint failed: %s", c->ck_error.c_str());
  }
  const int nx = c->nx, ny = c->ny;
  const size_t cells = (size_t)nx * ny;
  if (!c->ck_dev) {
    if (int rc = dev_alloc(c, &c->ck_dev, 4 * cells)) return rc;
    SNS_CUDA(counted_malloc_host(&c->ck_host, sizeof(double) * 4 * cells));
    SNS_CUDA(cudaStreamCreateWithFlags(&c->ck_stream, cudaStreamNonBlocking));
    SNS_CUDA(cudaEventCreateWithFlags(&c->ck_snap, cudaEventDisableTiming));
    SNS_CUDA(cudaEventCreateWithFlags(&c->ck_done, cudaEventDisableTiming));
  }
  const bool with_t = param->with_temperature && te;
  // snapshot on the solver's stream: later launches may overwrite the fields
  SNS_CUDA(cudaMemcpyAsync(c->ck_dev, fe->f.ux, sizeof(double) * cells, cudaMemcpyDeviceToDevice, c->stream));
  SNS_CUDA(cudaMemcpyAsync(c->ck_dev + cells, fe->f.uy, sizeof(double) * cells, cudaMemcpyDeviceToDevice, c->stream));
  SNS_CUDA(cudaMemcpyAsync(c->ck_dev + 2 * cells, fe->f.p, sizeof(double) * cells, cudaMemcpyDeviceToDevice, c->stream));
  if (with_t)
    SNS_CUDA(cudaMemcpyAsync(c->ck_dev + 3 * cells, te->f.t[te->cur], sizeof(double) * cells,
                             cudaMemcpyDeviceToDevice, c->stream));
  SNS_CUDA(cudaEventRecord(c->ck_snap, c->stream));
  SNS_CUDA(cudaStreamWaitEvent(c->ck_stream, c->ck_snap, 0));
  SNS_CUDA(cudaMemcpyAsync(c->ck_host, c->ck_dev, sizeof(double) * (with_t ? 4 : 3) * cells, cudaMemcpyDeviceToHost,
                           c->ck_stream));
  SNS_CUDA(cudaEventRecord(c->ck_done, c->ck_stream));
  CheckpointJob J;
  J.dir = dirname;
  J.step = param->step;
  J.itot = param->itot;
  J.jtot = param->jtot;
  J.with_t = with_t ? 1 : 0;
  J.time = param->time;
  J.lx = param->lx;
  J.ly = param->ly;
  J.Ra = param->Ra;
  J.Pr = param->Pr;
  J.xf.assign(param->xf, param->xf + nx + 1);
  J.xc.assign(param->xc, param->xc + nx + 2);
  J.yf.assign(param->yf, param->yf + ny + 1);
  J.yc.assign(param->yc, param->yc + ny);
  SNS_CUDA(cudaGetDevice(&J.device));
  c->ck_status = SNS_OK;
  c->ck_error.clear();
  try {
    c->ck_thread = std::thread([c, J]() {
      std::string err;
      cudaError_t e = cudaSetDevice(J.device);
      if (e == cudaSuccess) e = cudaEventSynchronize(c->ck_done);
      if (e != cudaSuccess) {
        c->ck_status = SNS_ERR_CUDA;
        c->ck_error = std::string("checkpoint copy: ") + cudaGetErrorString(e);
        return;
      }
      if (write_checkpoint(J, c->ck_host, &err)) {
        c->ck_status = SNS_ERR_ARG;
        c->ck_error = err;
      }
    });
  } catch (...) {
    return fail(SNS_ERR_STATE, "sns_checkpoint: cannot start the writer thread");
  }
  return SNS_OK;
}

int sns_npy_write(const char *path, const char *dtype, int ndim, const size_t *shape, const void *data,
                  size_t nbytes) {
  if (!path || !dtype || ndim < 0 || (ndim > 0 && !shape) || (nbytes && !data))
    return fail(SNS_ERR_ARG, "sns_npy_write: bad argument");
  std::string err;
  if (npy_write(path, dtype, ndim, shape, data, nbytes, &err)) return fail(SNS_ERR_ARG, "%s", err.c_str());
  return SNS_OK;
}

int sns_npy_read(const char *path, const char *dtype, int ndim, const size_t *shape, void *data, size_t nbytes) {
  if (!path || !dtype || ndim < 0 || (ndim > 0 && !shape) || (nbytes && !data))
    return fail(SNS_ERR_ARG, "sns_npy_read: bad argument");
  std::string err;
  if (npy_read(path, dtype, ndim, shape, data, nbytes, &err)) return fail(SNS_ERR_ARG, "%s", err.c_str());
  return SNS_OK;
}

int sns_checkpoint_wait(const fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  if (!fe) return fail(SNS_ERR_ARG, "sns_checkpoint_wait: bad argument");
  Context *c = fe->ctx;
  if (c->ck_thread.joinable()) c->ck_thread.join();
  if (c->ck_status != SNS_OK) {
    const int rc = c->ck_status;
    c->ck_status = SNS_OK;  // reported once
    return fail(rc, "sns_checkpoint: %s", c->ck_error.c_str());
  }
  return SNS_OK;
}

int sns_restart(param_t *param, fluid_t *fluid, temperature_t *temperature, const char *dirname) {
  FluidExt *fe = as_fluid(fluid);
  TempExt *te = temperature ? as_temp(temperature) : nullptr;
  if (!param || !fe || !dirname || (temperature && !te)) return fail(SNS_ERR_ARG, "sns_restart: bad argument");
  if (int rc = flush_pending(fe->ctx)) return rc;
  const int nx = param->itot, ny = param->jtot;
  const std::string dir(dirname);
  std::string err;
  int step = 0;
  double time = 0.;
  // src/param/init.c:245-247
  if (npy_read((dir + "/step.npy").c_str(), "'int32'", 0, nullptr, &step, sizeof(int), &err) ||
      npy_read((dir + "/time.npy").c_str(), "'float64'", 0, nullptr, &time, sizeof(double), &err))
    return fail(SNS_ERR_ARG, "sns_restart: %s", err.c_str());
  // src/fluid/init.c:53-81, src/temperature/init.c:51: rows 1..jtot, then the boundary rules
  fluid_t &h = fe->pub;
  const size_t su[2] = {(size_t)ny, (size_t)nx + 1}, sc[2] = {(size_t)ny, (size_t)nx + 2};
  if (npy_read((dir + "/ux.npy").c_str(), "'float64'", 2, su, h.ux + (nx + 1), sizeof(double) * su[0] * su[1], &err) ||
      npy_read((dir + "/uy.npy").c_str(), "'float64'", 2, sc, h.uy + (nx + 2), sizeof(double) * sc[0] * sc[1], &err) ||
      npy_read((dir + "/p.npy").c_str(), "'float64'", 2, sc, h.p + (nx + 2), sizeof(double) * sc[0] * sc[1], &err))
    return fail(SNS_ERR_ARG, "sns_restart: %s", err.c_str());
  host_bc_ux(nx, ny, h.ux);
  host_bc_uy(nx, ny, h.uy);
  host_bc_p(nx, ny, h.p);
  std::memset(h.psi, 0, sizeof(double) * sc[1] * (ny + 2));
  // a restarted reference run starts from zeroed (calloc'd) source arrays
  std::memset(h.srcuxa, 0, sizeof(double) * (size_t)(nx - 1) * ny);
  std::memset(h.srcuya, 0, sizeof(double) * (size_t)nx * ny);
  if (te && param->with_temperature) {
    temperature_t &t = te->pub;
    if (npy_read((dir + "/temp.npy").c_str(), "'float64'", 2, sc, t.temp + (nx + 2), sizeof(double) * sc[0] * sc[1],
                 &err))
      return fail(SNS_ERR_ARG, "sns_restart: %s", err.c_str());
    host_bc_temp(nx, ny, t.temp);
    std::memset(t.srctempa, 0, sizeof(double) * (size_t)nx * ny);
  }
  param->step = step;
  param->time = time;
  return sns_sync_to_device(param, fluid, te ? temperature : nullptr);
}

// ------------------------------------------------------------- statistics
constexpr uint64_t kStatsMagic = 0x534e535354415453ull;  // "SNSSTATS"

struct StatsExt {
  statistics_t pub;  // first member: statistics_t* and StatsExt* coincide
  uint64_t magic;
  int nx, ny, with_t;
  Context *ctx;           // the solver whose stream the sums are taken on (first collect)
  double *dev = nullptr;  // ux1, ux2 [ny][nx+1]; uy1, uy2, temp1, temp2 [ny][nx+2]
};

static StatsExt *as_stats(const statistics_t *s) {
  StatsExt *e = reinterpret_cast<StatsExt *>(const_cast<statistics_t *>(s));
  return (e && e->magic == kStatsMagic) ? e : nullptr;
}

statistics_t *statistics_init(const param_t *param, const parallel_t *parallel) {
  if (!param || !parallel) {
    fail(SNS_ERR_ARG, "statistics_init: bad argument");
    return nullptr;
  }
  const int nx = param->itot, ny = param->jtot;
  StatsExt *e = new (std::nothrow) StatsExt();
  if (!e) {
    fail(SNS_ERR_OOM, "statistics_init: out of host memory");
    return nullptr;
  }
  e->magic = kStatsMagic;
  e->nx = nx;
  e->ny = ny;
  e->with_t = param->with_temperature ? 1 : 0;
  const size_t nu = (size_t)(nx + 1) * (ny + 2), nc = (size_t)(nx + 2) * (ny + 2);
  statistics_t &h = e->pub;
  h.num = 0;
  h.ux1 = static_cast<double *>(calloc(nu, sizeof(double)));
  h.ux2 = static_cast<double *>(calloc(nu, sizeof(double)));
  h.uy1 = static_cast<double *>(calloc(nc, sizeof(double)));
  h.uy2 = static_cast<double *>(calloc(nc, sizeof(double)));
  h.temp1 = static_cast<double *>(calloc(nc, sizeof(double)));
  h.temp2 = static_cast<double *>(calloc(nc, sizeof(double)));
  if (!h.ux1 || !h.ux2 || !h.uy1 || !h.uy2 || !h.temp1 || !h.temp2) {
    statistics_finalise(&h);
    fail(SNS_ERR_OOM, "statistics_init: out of host memory");
    return nullptr;
  }
  return &h;
}

int statistics_finalise(statistics_t *statistics) {
  StatsExt *e = as_stats(statistics);
  if (!e) return fail(SNS_ERR_ARG, "statistics_finalise: not a statistics_t from statistics_init");
  if (e->dev) {
    if (e->ctx && e->ctx->stream) cudaStreamSynchronize(e->ctx->stream);
    cudaFree(e->dev);
  }
  for (double *p : {e->pub.ux1, e->pub.ux2, e->pub.uy1, e->pub.uy2, e->pub.temp1, e->pub.temp2}) free(p);
  e->magic = 0;
  delete e;
  return SNS_OK;
}

int statistics_collect(param_t *param, const parallel_t *parallel, const fluid_t *fluid,
                       const temperature_t *temperature, statistics_t *statistics) {
  StatsExt *e = as_stats(statistics);
  FluidExt *fe = as_fluid(fluid);
  TempExt *te = temperature ? as_temp(temperature) : nullptr;
  if (!param || !parallel || !e || !fe || (temperature && !te))
    return fail(SNS_ERR_ARG, "statistics_collect: bad argument");
  Context *c = fe->ctx;
  if (int rc = flush_pending(c)) return rc;
  if (e->nx != c->nx || e->ny != c->ny) return fail(SNS_ERR_ARG, "statistics_collect: grid size mismatch");
  if (e->ctx && e->ctx != c) return fail(SNS_ERR_ARG, "statistics_collect: statistics of another solver");
  const size_t nx = c->nx, ny = c->ny, words = 2 * (nx + 1) * ny + 4 * (nx + 2) * ny;
  if (!e->dev) {
    e->ctx = c;
    void *p = nullptr;
    cudaError_t err = counted_malloc(&p, sizeof(double) * words);
    if (err != cudaSuccess) return fail(SNS_ERR_OOM, "statistics_collect: cudaMalloc: %s", cudaGetErrorString(err));
    e->dev = static_cast<double *>(p);
    SNS_CUDA(cudaMemsetAsync(e->dev, 0, sizeof(double) * words, c->stream));
  }
  SNS_CUDA(launch_stats(c->g, fe->f.ux, fe->f.uy, te ? te->f.t[te->cur] : nullptr, e->dev, c->stream));
  e->pub.num += 1;
  return SNS_OK;
}

int sns_statistics_output_to(const param_t *param, const statistics_t *statistics, const char *dirname) {
  StatsExt *e = as_stats(statistics);
  if (!param || !e || !dirname) return fail(SNS_ERR_ARG, "sns_statistics_output_to: bad argument");
  const int nx = e->nx, ny = e->ny;
  const size_t wu = (size_t)nx + 1, wc = (size_t)nx + 2;
  statistics_t &h = e->pub;
  if (e->dev) {  // rows j = 1..jtot of the host arrays
    Context *c = e->ctx;
    const size_t nu = wu * ny, nc = wc * ny;
    const double *d = e->dev;
    SNS_CUDA(cudaMemcpyAsync(h.ux1 + wu, d, sizeof(double) * nu, cudaMemcpyDeviceToHost, c->stream));
    SNS_CUDA(cudaMemcpyAsync(h.ux2 + wu, d + nu, sizeof(double) * nu, cudaMemcpyDeviceToHost, c->stream));
    SNS_CUDA(cudaMemcpyAsync(h.uy1 + wc, d + 2 * nu, sizeof(double) * nc, cudaMemcpyDeviceToHost, c->stream));
    SNS_CUDA(cudaMemcpyAsync(h.uy2 + wc, d + 2 * nu + nc, sizeof(double) * nc, cudaMemcpyDeviceToHost, c->stream));
    SNS_CUDA(cudaMemcpyAsync(h.temp1 + wc, d + 2 * nu + 2 * nc, sizeof(double) * nc, cudaMemcpyDeviceToHost,
                             c->stream));
    SNS_CUDA(cudaMemcpyAsync(h.temp2 + wc, d + 2 * nu + 3 * nc, sizeof(double) * nc, cudaMemcpyDeviceToHost,
                             c->stream));
    SNS_CUDA(cudaStreamSynchronize(c->stream));
  }
  // src/statistics/output.c:9-63
  std::string err, dir(dirname);
  if (make_dirs(dirname, &err)) return fail(SNS_ERR_ARG, "sns_statistics_output_to: %s", err.c_str());
  auto path = [&](const char *n) { return dir + "/" + n + ".npy"; };
  int rc = 0;
  auto w0 = [&](const char *n, const char *dt, const void *v, size_t b) {
    if (!rc) rc = npy_write(path(n).c_str(), dt, 0, nullptr, v, b, &err);
  };
  auto w1 = [&](const char *n, const double *v, size_t len) {
    const size_t shape[1] = {len};
    if (!rc) rc = npy_write(path(n).c_str(), "'float64'", 1, shape, v, sizeof(double) * len, &err);
  };
  auto w2 = [&](const char *n, const double *v, size_t w) {
    const size_t shape[2] = {(size_t)ny, w};
    if (!rc) rc = npy_write(path(n).c_str(), "'float64'", 2, shape, v + w, sizeof(double) * w * ny, &err);
  };
  w0("num", "'int32'", &h.num, sizeof(int));
  w0("step", "'int32'", &param->step, sizeof(int));
  w0("itot", "'int32'", &param->itot, sizeof(int));
  w0("jtot", "'int32'", &param->jtot, sizeof(int));
  w0("time", "'float64'", &param->time, sizeof(double));
  w0("lx", "'float64'", &param->lx, sizeof(double));
  w0("ly", "'float64'", &param->ly, sizeof(double));
  w0("Ra", "'float64'", &param->Ra, sizeof(double));
  w0("Pr", "'float64'", &param->Pr, sizeof(double));
  w1("xf", param->xf, (size_t)nx + 1);
  w1("xc", param->xc, (size_t)nx + 2);
  w1("yf", param->yf, (size_t)ny + 1);
  w1("yc", param->yc, (size_t)ny);
  w2("ux1", h.ux1, wu);
  w2("uy1", h.uy1, wc);
  w2("ux2", h.ux2, wu);
  w2("uy2", h.uy2, wc);
  if (param->with_temperature) {
    w2("temp1", h.temp1, wc);
    w2("temp2", h.temp2, wc);
  }
  if (rc) return fail(SNS_ERR_ARG, "sns_statistics_output_to: %s", err.c_str());
  return SNS_OK;
}

int statistics_output(const param_t *param, const parallel_t *parallel, const statistics_t *statistics) {
  if (!param || !parallel) return fail(SNS_ERR_ARG, "statistics_output: bad argument");
  char dir[64];
  snprintf(dir, sizeof dir, "output/stat/step%010d", param->step);  // src/statistics/output.c:41-51
  return sns_statistics_output_to(param, statistics, dir);
}

// sns_diagnostics without allocation, for callers that cannot allocate (a
// monitoring thread sampling a run in flight, where cudaMalloc may
// synchronise the device; a process whose HBM is committed to a batch arena).
// The scratch is one file-scope device array in diagnostics.cu; calls that
// overlap on one device race on it.
int sns_diagnostics_static(const param_t *param, const fluid_t *fluid, const temperature_t *temperature,
                           double out[11]) {
  FluidExt *fe = as_fluid(fluid);
  TempExt *te = as_temp(temperature);
  if (!param || !fe || !te || !out) return fail(SNS_ERR_ARG, "sns_diagnostics_static: bad argument");
  if (int rc = flush_pending(fe->ctx)) return rc;
  Context *c = fe->ctx;
  const int nx = c->nx, ny = c->ny;
  const int nb = diag_blocks(nx, ny);
  if (nb > kDiagStaticBlocks)
    return fail(SNS_ERR_UNSUPPORTED,
                "sns_diagnostics_static: a %d x %d grid needs %d block partials, more than the %d of its static "
                "scratch (at most (ceil((itot+1)/64) * ceil(jtot/16)) <= %d); use sns_diagnostics",
                nx, ny, nb, kDiagStaticBlocks, kDiagStaticBlocks);
  const double Ra = param->Ra, Pr = param->Pr;
  const DiagArgs<double> a{nx, ny, param->dy, param->ly, sqrt(Pr) * sqrt(Ra), sqrt(Pr) / sqrt(Ra),
                           1. / sqrt(Pr) / sqrt(Ra), c->g.dxf, c->g.dxc, fe->f.ux, fe->f.uy, te->f.t[te->cur]};
  SNS_CUDA(diag_static(a, c->stream, out));
  count_launches(2);
  return SNS_OK;
}

static const char *kKindNames[K_NUM_KINDS] = {
    "temperature_update", "velocity_update", "poisson_forward_fft", "poisson_tridiagonal", "poisson_inverse_fft",
    "correct_and_pressure", "correct_velocity", "update_pressure", "max_velocity", "cn_solve_x", "cn_solve_y",
    "add_increment", "poisson_fused", "poisson_pcr"};

int sns_profile(const fluid_t *fluid, int enable) {
  FluidExt *fe = as_fluid(fluid);
  if (!fe) return fail(SNS_ERR_ARG, "sns_profile: bad fluid");
  Context *c = fe->ctx;
  prof_collect(c);
  if (enable) {
    for (int k = 0; k < K_NUM_KINDS; k++) {
      c->prof_ms[k] = 0.0;
      c->prof_n[k] = 0;
    }
  }
  c->prof = enable != 0;
  return SNS_OK;
}

int sns_profile_read(const fluid_t *fluid, double *ms, long long *count, int n) {
  FluidExt *fe = as_fluid(fluid);
  if (!fe || !ms || !count) return fail(SNS_ERR_ARG, "sns_profile_read: bad argument");
  Context *c = fe->ctx;
  prof_collect(c);
  for (int k = 0; k < n && k < K_NUM_KINDS; k++) {
    ms[k] = c->prof_ms[k];
    count[k] = c->prof_n[k];
  }
  return K_NUM_KINDS;
}

const char *sns_profile_kind_name(int kind) {
  return (kind >= 0 && kind < K_NUM_KINDS) ? kKindNames[kind] : "";
}

int sns_synchronize(const fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  if (!fe) return fail(SNS_ERR_ARG, "sns_synchronize: bad fluid");
  if (int rc = flush_pending(fe->ctx)) return rc;
  if (int rc = fused_enqueue_err(fe->ctx)) return rc;
  SNS_CUDA(cudaStreamSynchronize(fe->ctx->stream));
  return fused_check(fe->ctx);
}

int sns_set_form(const fluid_t *fluid, int mode) {
  FluidExt *fe = as_fluid(fluid);
  if (!fe) return fail(SNS_ERR_ARG, "sns_set_form: bad fluid");
  if (mode != SNS_FORM_EXACT && mode != SNS_FORM_PARALLEL)
    return fail(SNS_ERR_ARG, "sns_set_form: unknown mode %d", mode);
  Context *c = fe->ctx;
  if (int rc = flush_pending(c)) return rc;
  if (mode == SNS_FORM_PARALLEL)
    if (int rc = parallel_prepare(c)) return rc;
  c->form = mode;
  return SNS_OK;
}

int sns_get_form(const fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  return fe ? fe->ctx->form : -1;
}

int sns_set_wait_limit(const fluid_t *fluid, unsigned polls, int stale) {
  FluidExt *fe = as_fluid(fluid);
  if (!fe) return fail(SNS_ERR_ARG, "sns_set_wait_limit: bad fluid");
  if (int rc = flush_pending(fe->ctx)) return rc;
  Context *c = fe->ctx;
  c->fz.spin_limit = polls;
  c->par.spin_limit = polls ? polls : (1u << 22);
  // the stale flag arms the next launch of the form in use only
  c->fz.stale = stale != 0 && c->form == SNS_FORM_EXACT;
  c->par.stale = stale != 0 && c->form == SNS_FORM_PARALLEL;
  return SNS_OK;
}

int sns_set_fused(const fluid_t *fluid, int on) {
  FluidExt *fe = as_fluid(fluid);
  if (!fe) return fail(SNS_ERR_ARG, "sns_set_fused: bad fluid");
  if (int rc = flush_pending(fe->ctx)) return rc;
  fe->ctx->fused = on != 0;
  return SNS_OK;
}

void *sns_stream(const fluid_t *fluid) {
  FluidExt *fe = as_fluid(fluid);
  return fe ? (void *)fe->ctx->stream : nullptr;
}

// One time step's substages (src/main.c:80-99) with fused kernels. With the
// explicit scheme the temperature update of a substage, which reads only the
// substage's starting T and u, runs inside the fused Poisson launch on the
// SMs that the latency-bound tridiagonal sweeps leave free (exact form), or
// on a side stream beside the tridiagonal solve and the inverse DFT (Poisson
// solve as separate kernels, either form); the velocity kernel has already
// taken its buoyancy from the starting T, and the next substage reads the
// new T. Same kernels' arithmetic, same inputs, same bits as the sequential
// order.
static int integrate_impl(const param_t *param, FluidExt *fe, TempExt *te, bool reduce_last) {
  Context *c = fe->ctx;
  Fields &f = fe->f;
  for (int rk = 0; rk < RKSTEPMAX; rk++) {
    const bool with_t = param->with_temperature && te;
    const bool overlap = with_t && !param->implicitx && !param->implicity;
    const double *ux_k = f.ux, *uy_k = f.uy;  // the velocity this substage starts from
    const bool implicit = param->implicitx || param->implicity;
    if (with_t) te->snap = param->with_thermal_forcing ? te->cur : -1;
    if (implicit) {
      if (int rc = implicit_updates(param, rk, fe, te)) return rc;
    } else {
      if (int rc = do_velocity_update(param, rk, fe, te)) return rc;
    }
    const StageScalars s = stage_scalars(param, rk);
    int out = 0;
    if (overlap)
      while (out == te->cur || out == te->snap) out++;
    bool fused = false;
    if (overlap && c->fused) {
      if (int rc = try_fused(c, s, f, te->f.t[te->cur], te->f.t[out], te->f.at, ux_k, uy_k, &fused)) return rc;
      if (fused) te->cur = out;
    }
    if (!fused) {
      if (overlap) {
        // the temperature update on the side stream: in the parallel form
        // from the end of the velocity update on, beside the forward DFT,
        // whose 2 columns per block leave SMs unevenly loaded (512 x 1024:
        // 0.502 against 0.511 ms per step with it beside the tridiagonal
        // solve); in the exact form beside the serial tridiagonal sweeps
        const bool early = c->form == SNS_FORM_PARALLEL;
        if (!early)
          if (int rc = poisson_forward(c, s, f)) return rc;
        SNS_CUDA(cudaEventRecord(c->ev_fwd, c->stream));
        SNS_CUDA(cudaStreamWaitEvent(c->side, c->ev_fwd, 0));
        {
          Prof pf(c, K_TEMP, c->side);
          SNS_CUDA(FORM(c, launch_temp_update)(c->g, s, 0, 0, te->f.t[te->cur], te->f.t[out], te->f.at, nullptr, ux_k, uy_k,
                                      c->side));
        }
        SNS_CUDA(cudaEventRecord(c->ev_temp, c->side));
        te->cur = out;
        if (early)
          if (int rc = poisson_forward(c, s, f)) return rc;
        if (int rc = poisson_rest(c, s, f)) return rc;
      } else {
        if (int rc = poisson(c, s, f)) return rc;
      }
    }
    const bool red = reduce_last && rk == RKSTEPMAX - 1;
    if (red) SNS_CUDA(cudaMemsetAsync(f.colmax, 0, sizeof(unsigned long long) * (c->nx + 1), c->stream));
    {
      Prof pf(c, K_CORR_PRES);
      SNS_CUDA(FORM(c, launch_correct_pressure)(c->g, s, param->implicitx, param->implicity, f.psi, f.ux, f.uy, f.p,
                                       red ? f.colmax : nullptr, red ? f.uymax : nullptr, c->stream));
    }
    // the next substage reads the new T and overwrites the buffer of u_k
    if (overlap && !fused) SNS_CUDA(cudaStreamWaitEvent(c->stream, c->ev_temp, 0));
  }
  return SNS_OK;
}

int sns_integrate(const param_t *param, const parallel_t *parallel, fluid_t *fluid, temperature_t *temperature) {
  FluidExt *fe = as_fluid(fluid);
  if (!param || !parallel || !fe) return fail(SNS_ERR_ARG, "sns_integrate: bad argument");
  if (parallel->mpisize != 1) return fail(SNS_ERR_UNSUPPORTED, "single-rank only");
  if (int rc = flush_pending(fe->ctx)) return rc;
  TempExt *te = temperature ? as_temp(temperature) : nullptr;
  Context *c = fe->ctx;
  c->version++;
  // the last substage also leaves the max-|u| reduction for the next
  // param_decide_dt
  if (int rc = integrate_impl(param, fe, te, true)) return rc;
  c->red_version = c->version;
  return SNS_OK;
}

int sns_run(param_t *param, const parallel_t *parallel, fluid_t *fluid, temperature_t *temperature, int nsteps) {
  FluidExt *fe = as_fluid(fluid);
  if (!param || !parallel || !fe || nsteps < 0) return fail(SNS_ERR_ARG, "sns_run: bad argument");
  if (parallel->mpisize != 1) return fail(SNS_ERR_UNSUPPORTED, "single-rank only");
  if (int rc = flush_pending(fe->ctx)) return rc;
  TempExt *te = temperature ? as_temp(temperature) : nullptr;
  Context *c = fe->ctx;
  // the reduction of the current state may be resident from the previous call
  bool have_reduction = c->red_version == c->version;
  for (int s = 0; s < nsteps; s++) {
    if (int rc = reduce_to_host(c, fe->f, !have_reduction)) return rc;
    if (int rc = nonfinite_check(c, param)) return rc;  // stop stepping a diverged state
    finish_decide_dt(param, c);
    c->version++;
    if (int rc = integrate_impl(param, fe, te, true)) return rc;
    c->red_version = c->version;
    have_reduction = true;
    param->step += 1;
    param->time += param->dt;
  }
  if (nsteps > 0) {
    // the last step's reduction to the host with this call's final wait, so
    // that the next call decides dt without a round trip; launch errors of
    // this call are reported by this call
    SNS_CUDA(cudaMemcpyAsync(c->red_host, fe->f.colmax, sizeof(unsigned long long) * (c->nx + 1),
                             cudaMemcpyDeviceToHost, c->stream));
    if (int rc = fused_enqueue_err(c)) return rc;
  }
  SNS_CUDA(cudaStreamSynchronize(c->stream));
  if (nsteps > 0) {
    if (int rc = fused_check(c)) return rc;
    c->red_host_version = c->red_version;
    return nonfinite_check(c, param);
  }
  return SNS_OK;
}

}  // extern "C"
