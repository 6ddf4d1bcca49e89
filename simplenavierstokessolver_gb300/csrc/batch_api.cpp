// Host side of the batched FP32-stencil / FP64-Poisson engine (include/sns_batch.h).
//
// A batch owns one device arena. Each admitted case gets one contiguous
// block of it (first fit, coalescing free list), a slot in the device case
// table and work items in the per-phase work lists. One time step of every
// resident case is a fixed sequence of 16 launches, captured once per case
// set into a CUDA graph and replayed per step; every case carries its own dt,
// time, step count and buffer parity in the device table, so cases of
// different age and size share the launches.
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "batch_internal.h"
#include "diag_internal.h"
#include "host_common.h"
#include "npy.h"
#include "sns_batch.h"
#include "sns_gpu.h"

namespace sns {

static_assert(kSeg == kPartSeg && kPcrLevels == kPartLevels, "one partition layout for both forms");

static int bfail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  record_error(buf);
  return code;
}

#define BCUDA(call)                                                                                     \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess)                                                                              \
      return bfail(SNS_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_));    \
  } while (0)

static size_t align256(size_t v) { return (v + 255) / 256 * 256; }

// byte layout of one case inside its arena block
struct CaseLayout {
  size_t rdxf_f, rdxc_f, ccm_f, ccp_f, cfm_f, cfp_f, rdxf_l;
  size_t rdxf, rdxc, dxi, dxf, dxc, tw, lo, hi, pfac, ccm, ccp, cfm, cfp;
  size_t ux[2], uy[2], t[2], uxl[2], uyl[2], tl[2], aux, auy, at, auxl, auyl, atl, p, psi, spec;
  size_t total;
  size_t pstride;
};

// x2: a compensated case (sns_case_desc::compensated), which also keeps the
// low words of the previous right-hand sides
static CaseLayout layout_for(int nx, int ny, bool x2) {
  CaseLayout L{};
  const int nh = ny / 2 + 1;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += align256(bytes);
    return o;
  };
  const size_t cells = (size_t)nx * ny;
  L.rdxf_f = take(sizeof(float) * nx);
  L.rdxf_l = take(sizeof(float) * nx);
  L.rdxc_f = take(sizeof(float) * (nx + 1));
  L.ccm_f = take(sizeof(float) * nx);
  L.ccp_f = take(sizeof(float) * nx);
  L.cfm_f = take(sizeof(float) * nx);
  L.cfp_f = take(sizeof(float) * nx);
  L.rdxf = take(sizeof(double) * nx);
  L.rdxc = take(sizeof(double) * (nx + 1));
  L.dxi = take(sizeof(double) * (nx + 1));
  L.dxf = take(sizeof(double) * nx);
  L.dxc = take(sizeof(double) * (nx + 1));
  L.tw = take(sizeof(double) * 2 * ny);
  L.lo = take(sizeof(double) * nx);
  L.hi = take(sizeof(double) * nx);
  L.pstride = 4 * (size_t)nx + 2 * kPcrLevels * kSeg + kSeg;
  L.pfac = take(sizeof(double) * L.pstride * nh);
  L.ccm = take(sizeof(double) * nx);
  L.ccp = take(sizeof(double) * nx);
  L.cfm = take(sizeof(double) * nx);
  L.cfp = take(sizeof(double) * nx);
  for (int k = 0; k < 2; k++) {
    L.ux[k] = take(sizeof(float) * cells);
    L.uy[k] = take(sizeof(float) * cells);
    L.t[k] = take(sizeof(float) * cells);
  }
  for (int k = 0; k < 2; k++) {
    L.uxl[k] = take(sizeof(float) * cells);
    L.uyl[k] = take(sizeof(float) * cells);
    L.tl[k] = take(sizeof(float) * cells);
  }
  L.aux = take(sizeof(float) * cells);
  L.auy = take(sizeof(float) * cells);
  L.at = take(sizeof(float) * cells);
  if (x2) {
    L.auxl = take(sizeof(float) * cells);
    L.auyl = take(sizeof(float) * cells);
    L.atl = take(sizeof(float) * cells);
  }
  L.p = take(sizeof(double) * cells);
  L.psi = take(sizeof(double) * cells);
  L.spec = take(sizeof(double2) * (size_t)nh * nx);
  L.total = off;
  return L;
}

static int check_desc(const sns_case_desc *d) {
  if (!d) return bfail(SNS_ERR_ARG, "NULL case description");
  if (d->jtot < 8 || d->jtot > 8192 || (d->jtot & (d->jtot - 1)))
    return bfail(SNS_ERR_UNSUPPORTED, "jtot=%d must be a power of two in [8, 8192]", d->jtot);
  if (d->itot < 64 || d->itot > 4096 || d->itot % kSeg)
    return bfail(SNS_ERR_UNSUPPORTED, "itot=%d must be a multiple of %d in [64, 4096]", d->itot, kSeg);
  if (!(d->Ra > 0) || !(d->Pr > 0) || !(d->ly > 0)) return bfail(SNS_ERR_ARG, "Ra, Pr and ly must be positive");
  return SNS_OK;
}

// SplitMix64 (Steele, Lea, Flood 2014), the seeded noise of sns_case_desc
static inline unsigned long long splitmix64(unsigned long long &state) {
  unsigned long long z = (state += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// initial temperature in the reference's (jtot+2) x (itot+2) layout:
// T = (TEMP_XP - TEMP_XM) x + TEMP_XM + 0.1 r (src/temperature/init.c:30-41)
static void initial_temperature(const sns_case_desc *d, const double *xc, double *temp) {
  const int nx = d->itot, ny = d->jtot;
  std::memset(temp, 0, sizeof(double) * (size_t)(nx + 2) * (ny + 2));
  unsigned long long st = d->seed;
  if (d->seed == 0) srand(0);
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double x = xc[i];
      double r;
      if (d->seed == 0) {
        r = -0.5 + 1. * rand() / RAND_MAX;
      } else {
        r = (double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0) - 0.5;
      }
      temp[(size_t)j * (nx + 2) + i] = (TEMP_XP - TEMP_XM) * x + TEMP_XM + 0.1 * r;
    }
  for (int j = 1; j <= ny; j++) {
    temp[(size_t)j * (nx + 2)] = TEMP_XM;
    temp[(size_t)j * (nx + 2) + nx + 1] = TEMP_XP;
  }
  for (int i = 1; i <= nx; i++) {
    temp[i] = temp[(size_t)ny * (nx + 2) + i];
    temp[(size_t)(ny + 1) * (nx + 2) + i] = temp[(size_t)(nx + 2) + i];
  }
}

struct CaseHost {
  bool used = false;
  sns_case_desc d{};
  size_t off = 0, bytes = 0;
  long long steps_done = 0;  // host mirror: every unfinished case advances one step per batch step
  int fcols = 1;
};

}  // namespace sns

using namespace sns;

struct sns_batch {
  cudaStream_t stream = nullptr;
  char *arena = nullptr;
  size_t arena_bytes = 0;
  std::map<size_t, size_t> free_blocks;  // offset -> size
  int max_cases = 0;
  std::vector<CaseHost> hc;
  std::vector<BCase> table;  // host copies of the static part of each slot
  BCase *d_cases = nullptr;
  BTile *d_tiles = nullptr;
  BCols *d_cols = nullptr;
  BModes *d_modes = nullptr;
  size_t cap_tiles = 0, cap_cols = 0, cap_modes = 0;
  int ntiles = 0, ncols = 0, nmodes = 0;
  int ntiles_x2 = 0;  // the last ntiles_x2 tiles belong to compensated cases
  int graph_launches = 0;  // kernel launches per replay of the step graph
  size_t fft_smem = 0;
  int fft_threads = 64;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool dirty = true;
  double rk_a[3] = {32. / 60., 25. / 60., 45. / 60.};
  double rk_b[3] = {0. / 60., -17. / 60., -25. / 60.};
  double *staging = nullptr;  // pinned
  size_t staging_bytes = 0;
  double *diag = nullptr;  // block partials of sns_batch_diagnostics
  size_t diag_words = 0;
  sns_batch_tuning tune{kBTileX, kBTileY, kBModesPerBlock, 0};
  // this batch's error word: a tridiagonal bulk-copy wait gave up
  unsigned *d_err = nullptr;
  unsigned *h_err = nullptr;  // pinned
  unsigned tri_spin = 1u << 22;  // polls of that wait
  int tri_stale = 0;             // test of the error path: the next step issues no copy
  // one persistent cooperative launch per substage instead of five per-phase
  // launches (sns_batch_set_persistent): barrier words
  bool persistent = false;
  unsigned *d_bar = nullptr;  // [2] arrival count, generation
  std::mutex mu;
};

static bool arena_alloc(sns_batch *b, size_t bytes, size_t *off) {
  for (auto it = b->free_blocks.begin(); it != b->free_blocks.end(); ++it) {
    if (it->second >= bytes) {
      *off = it->first;
      const size_t rest = it->second - bytes;
      const size_t noff = it->first + bytes;
      b->free_blocks.erase(it);
      if (rest) b->free_blocks[noff] = rest;
      return true;
    }
  }
  return false;
}

static void arena_free(sns_batch *b, size_t off, size_t bytes) {
  auto it = b->free_blocks.emplace(off, bytes).first;
  auto next = std::next(it);
  if (next != b->free_blocks.end() && it->first + it->second == next->first) {
    it->second += next->second;
    b->free_blocks.erase(next);
  }
  if (it != b->free_blocks.begin()) {
    auto prev = std::prev(it);
    if (prev->first + prev->second == it->first) {
      prev->second += it->second;
      b->free_blocks.erase(it);
    }
  }
}

template <typename T>
static int ensure_device_list(T **ptr, size_t *cap, size_t need) {
  if (need <= *cap) return SNS_OK;
  if (*ptr) cudaFree(*ptr);
  *ptr = nullptr;
  const size_t n = std::max<size_t>(need, 2 * *cap);
  BCUDA(counted_malloc((void **)ptr, sizeof(T) * n));
  *cap = n;
  return SNS_OK;
}

// work lists for the current case set and the graph of one step
// DFT columns per block for a case under the current tuning: the admission
// default scaled by 2^fcols_shift, within [1, 16], nx and 160 KiB of shared memory
static int tuned_fcols(const sns_batch *b, const CaseHost &h) {
  int fc = h.fcols;
  if (b->tune.fcols_shift > 0) fc <<= b->tune.fcols_shift;
  if (b->tune.fcols_shift < 0) fc >>= -b->tune.fcols_shift;
  fc = std::max(1, std::min(fc, 16));
  while (fc > 1 && (fc > h.d.itot || sizeof(double) * (size_t)fc * h.d.jtot > 160 * 1024)) fc >>= 1;
  return fc;
}

static int rebuild(sns_batch *b) {
  std::vector<BTile> tiles, tiles_x2;
  std::vector<BCols> cols;
  std::vector<BModes> modes;
  size_t smem = 0;
  int threads = 64;
  const int tx = b->tune.tile_x, ty = b->tune.tile_rows;
  // the tridiagonal launch stages each warp's line in shared memory: fewer
  // warps per block when the longest line would not fit
  int nmax = 32;
  for (const CaseHost &h : b->hc)
    if (h.used && !(h.d.steps > 0 && h.steps_done >= h.d.steps)) nmax = std::max(nmax, h.d.itot);
  int mpb = b->tune.modes_per_block;
  while (mpb > 1 && batch_tri_smem(nmax, mpb) > 200 * 1024) mpb /= 2;
  if (b->persistent) mpb = std::min(mpb, 4);  // the persistent launch's four line slots per block
  for (int c = 0; c < b->max_cases; c++) {
    const CaseHost &h = b->hc[c];
    if (!h.used) continue;
    if (h.d.steps > 0 && h.steps_done >= h.d.steps) continue;
    const int nx = h.d.itot, ny = h.d.jtot, nh = ny / 2 + 1;
    const int fc = tuned_fcols(b, h);
    if (b->table[c].fcols != fc) {  // the kernels read a case's column count from its table entry
      b->table[c].fcols = fc;
      BCUDA(cudaMemcpyAsync(reinterpret_cast<char *>(b->d_cases + c) + offsetof(BCase, fcols), &b->table[c].fcols,
                            sizeof(int), cudaMemcpyHostToDevice, b->stream));
    }
    for (int y0 = 0; y0 < ny; y0 += ty)
      for (int x0 = 0; x0 < nx; x0 += tx) (h.d.compensated ? tiles_x2 : tiles).push_back({c, x0, y0});
    for (int x0 = 0; x0 < nx; x0 += fc) cols.push_back({c, x0});
    for (int j0 = 0; j0 < nh; j0 += mpb) modes.push_back({c, j0});
    smem = std::max(smem, sizeof(double) * (size_t)fc * ny);
    threads = std::max(threads, std::min(256, (fc * (ny / 2) / 4 + 31) / 32 * 32));
  }
  const int nx2 = (int)tiles_x2.size();
  tiles.insert(tiles.end(), tiles_x2.begin(), tiles_x2.end());
  if (int rc = ensure_device_list(&b->d_tiles, &b->cap_tiles, std::max<size_t>(tiles.size(), 1))) return rc;
  if (int rc = ensure_device_list(&b->d_cols, &b->cap_cols, std::max<size_t>(cols.size(), 1))) return rc;
  if (int rc = ensure_device_list(&b->d_modes, &b->cap_modes, std::max<size_t>(modes.size(), 1))) return rc;
  if (!tiles.empty())
    BCUDA(cudaMemcpyAsync(b->d_tiles, tiles.data(), sizeof(BTile) * tiles.size(), cudaMemcpyHostToDevice, b->stream));
  if (!cols.empty())
    BCUDA(cudaMemcpyAsync(b->d_cols, cols.data(), sizeof(BCols) * cols.size(), cudaMemcpyHostToDevice, b->stream));
  if (!modes.empty())
    BCUDA(cudaMemcpyAsync(b->d_modes, modes.data(), sizeof(BModes) * modes.size(), cudaMemcpyHostToDevice,
                          b->stream));
  b->ntiles = (int)tiles.size();
  b->ntiles_x2 = nx2;
  // per substage: the stencil launch(es), forward DFT, tridiagonal, inverse
  // DFT, correction; then the dt update
  b->graph_launches = 3 * ((b->ntiles > nx2) + (nx2 > 0) + 4) + 1;
  b->ncols = (int)cols.size();
  b->nmodes = (int)modes.size();
  b->fft_smem = smem;
  b->fft_threads = threads;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  if (b->graph) {
    cudaGraphDestroy(b->graph);
    b->graph = nullptr;
  }
  BCUDA(cudaStreamSynchronize(b->stream));
  // persistent form: its shared memory and grid (every block resident)
  size_t sub_smem = 0;
  int sub_blocks = 0;
  if (b->persistent) {
    if (256 % tx)
      return bfail(SNS_ERR_UNSUPPORTED, "persistent batch step: tile width %d does not divide 256", tx);
    sub_smem = batch_substage_smem(b->fft_smem, nmax, mpb);
    sub_blocks = batch_substage_blocks(sub_smem);
    if (sub_blocks <= 0) return bfail(SNS_ERR_UNSUPPORTED, "persistent batch step: no cooperative grid fits");
    b->graph_launches = 3 + 1;
  }
  // one time step: three substages of five phases, then the per-case dt update
  BCUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  cudaError_t err = cudaSuccess;
  for (int rk = 0; rk < 3 && err == cudaSuccess && b->persistent; rk++)
    err = launch_batch_substage(b->d_cases, b->d_tiles, b->ntiles, b->ntiles_x2, b->d_cols, b->ncols, b->d_modes,
                                b->nmodes, rk, tx, ty, mpb, nmax, sub_smem, b->d_err, b->tri_spin, b->d_bar,
                                sub_blocks, b->stream);
  for (int rk = 0; rk < 3 && err == cudaSuccess && !b->persistent; rk++) {
    if ((err = launch_batch_stencil(b->d_cases, b->d_tiles, b->ntiles, b->ntiles_x2, rk, tx, ty, b->stream)) !=
        cudaSuccess)
      break;
    if ((err = launch_batch_fwd(b->d_cases, b->d_cols, b->ncols, rk, b->fft_smem, b->fft_threads, b->stream)) !=
        cudaSuccess)
      break;
    if ((err = launch_batch_tri(b->d_cases, b->d_modes, b->nmodes, mpb, nmax, b->d_err, b->tri_spin,
                                rk == 0 ? b->tri_stale : 0, b->stream)) != cudaSuccess)
      break;
    if ((err = launch_batch_bwd(b->d_cases, b->d_cols, b->ncols, b->fft_smem, b->fft_threads, b->stream)) !=
        cudaSuccess)
      break;
    if ((err = launch_batch_corr(b->d_cases, b->d_tiles, b->ntiles, rk, tx, ty, b->stream)) != cudaSuccess) break;
  }
  if (err == cudaSuccess) err = launch_batch_dt(b->d_cases, b->max_cases, b->rk_a, b->rk_b, b->stream);
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
  if (err != cudaSuccess) return bfail(SNS_ERR_CUDA, "capturing the batch step: %s", cudaGetErrorString(err));
  if (e2 != cudaSuccess) return bfail(SNS_ERR_CUDA, "capturing the batch step: %s", cudaGetErrorString(e2));
  b->graph = g;
  BCUDA(cudaGraphInstantiate(&b->exec, g, 0));
  b->dirty = false;
  return SNS_OK;
}

extern "C" {

size_t sns_batch_case_bytes(const sns_case_desc *desc) {
  if (check_desc(desc) != SNS_OK) return 0;
  return layout_for(desc->itot, desc->jtot, desc->compensated != 0).total;
}

sns_batch *sns_batch_create(size_t hbm_bytes, int max_cases) {
  if (max_cases <= 0 || hbm_bytes < (1u << 20)) {
    bfail(SNS_ERR_ARG, "sns_batch_create: need max_cases > 0 and at least 1 MiB");
    return nullptr;
  }
  sns_batch *b = new sns_batch();
  b->max_cases = max_cases;
  b->hc.resize(max_cases);
  b->table.resize(max_cases);
  for (BCase &t : b->table) {
    std::memset(&t, 0, sizeof(BCase));
    t.done = 1;  // empty slots are skipped by every kernel
  }
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      batch_kernels_init() != cudaSuccess || counted_malloc((void **)&b->arena, hbm_bytes) != cudaSuccess ||
      counted_malloc((void **)&b->d_cases, sizeof(BCase) * max_cases) != cudaSuccess ||
      counted_malloc((void **)&b->d_err, sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(b->d_err, 0, sizeof(unsigned)) != cudaSuccess ||
      counted_malloc((void **)&b->d_bar, 2 * sizeof(unsigned)) != cudaSuccess ||
      cudaMemset(b->d_bar, 0, 2 * sizeof(unsigned)) != cudaSuccess ||
      counted_malloc_host((void **)&b->h_err, sizeof(unsigned)) != cudaSuccess ||
      cudaMemcpy(b->d_cases, b->table.data(), sizeof(BCase) * max_cases, cudaMemcpyHostToDevice) != cudaSuccess) {
    bfail(SNS_ERR_OOM, "sns_batch_create: %s", cudaGetErrorString(cudaGetLastError()));
    sns_batch_destroy(b);
    return nullptr;
  }
  b->arena_bytes = hbm_bytes;
  b->free_blocks[0] = hbm_bytes;
  return b;
}

int sns_batch_destroy(sns_batch *b) {
  if (!b) return SNS_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  cudaFree(b->arena);
  cudaFree(b->d_cases);
  cudaFree(b->d_tiles);
  cudaFree(b->d_cols);
  cudaFree(b->d_modes);
  cudaFree(b->d_err);
  cudaFree(b->d_bar);
  if (b->h_err) cudaFreeHost(b->h_err);
  if (b->staging) cudaFreeHost(b->staging);
  cudaFree(b->diag);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return SNS_OK;
}

size_t sns_batch_free_bytes(const sns_batch *b) {
  if (!b) return 0;
  size_t best = 0;
  for (const auto &kv : b->free_blocks) best = std::max(best, kv.second);
  return best;
}

void *sns_batch_stream(const sns_batch *b) { return b ? (void *)b->stream : nullptr; }

int sns_batch_initial_temperature(const sns_case_desc *desc, double *temp) {
  if (int rc = check_desc(desc)) return rc;
  if (!temp) return bfail(SNS_ERR_ARG, "NULL output");
  const int nx = desc->itot, ny = desc->jtot;
  std::vector<double> xf(nx + 1), xc(nx + 2), dxf(nx), dxc(nx + 1);
  double dy;
  make_grid(nx, ny, 1.0, desc->ly, desc->stretch, xf.data(), xc.data(), dxf.data(), dxc.data(), nullptr, nullptr, &dy);
  initial_temperature(desc, xc.data(), temp);
  return SNS_OK;
}

}  // extern "C"

// a full starting state in the reference's layouts (restart): ux
// (jtot+2) x (itot+1), uy, p, temp (jtot+2) x (itot+2), rows 1..jtot used
struct StartState {
  const double *ux, *uy, *p, *temp;
  long long step;
  double time;
};

static int admit(sns_batch *b, const sns_case_desc *d, const double *temp_init, const StartState *st,
                 int *slot_out) {
  int slot = -1;
  for (int c = 0; c < b->max_cases; c++)
    if (!b->hc[c].used) {
      slot = c;
      break;
    }
  if (slot < 0) return bfail(SNS_ERR_OOM, "batch full (%d cases)", b->max_cases);
  const int nx = d->itot, ny = d->jtot, nh = ny / 2 + 1;
  const bool x2 = d->compensated != 0;
  const CaseLayout L = layout_for(nx, ny, x2);
  size_t off;
  if (!arena_alloc(b, L.total, &off))
    return bfail(SNS_ERR_OOM, "case needs %zu bytes, largest free block %zu", L.total, sns_batch_free_bytes(b));
  char *base = b->arena + off;
  // ---- grid and metrics (src/param/init.c:124-195)
  std::vector<double> xf(nx + 1), xc(nx + 2), dxf(nx), dxc(nx + 1);
  double dy;
  make_grid(nx, ny, 1.0, d->ly, d->stretch, xf.data(), xc.data(), dxf.data(), dxc.data(), nullptr, nullptr, &dy);
  auto DXF = [&](int i) { return dxf[i - 1]; };
  auto DXC = [&](int i) { return dxc[i - 1]; };
  std::vector<float> rdxf_f(nx), rdxf_l(nx), rdxc_f(nx + 1), ccm(nx), ccp(nx), cfm(nx, 0.f), cfp(nx, 0.f);
  std::vector<double> ccm_d(nx), ccp_d(nx), cfm_d(nx, 0.0), cfp_d(nx, 0.0);
  std::vector<double> rdxf(nx), rdxc(nx + 1), dxi(nx + 1), lo(nx), hi(nx), l_raw(nx), u_raw(nx);
  for (int i = 1; i <= nx; i++) {
    rdxf[i - 1] = 1.0 / DXF(i);
    rdxf_f[i - 1] = (float)rdxf[i - 1];
    rdxf_l[i - 1] = (float)(rdxf[i - 1] - (double)rdxf_f[i - 1]);
    ccm_d[i - 1] = DXC(i) / (2. * DXF(i));
    ccp_d[i - 1] = DXC(i + 1) / (2. * DXF(i));
    ccm[i - 1] = (float)ccm_d[i - 1];
    ccp[i - 1] = (float)ccp_d[i - 1];
    if (i >= 2) {
      cfm_d[i - 1] = DXF(i - 1) / (2. * DXC(i));
      cfp_d[i - 1] = DXF(i) / (2. * DXC(i));
      cfm[i - 1] = (float)cfm_d[i - 1];
      cfp[i - 1] = (float)cfp_d[i - 1];
    }
    l_raw[i - 1] = 1. / DXC(i) / DXF(i);
    u_raw[i - 1] = 1. / DXC(i + 1) / DXF(i);
    lo[i - 1] = i > 1 ? l_raw[i - 1] : 0.0;
    hi[i - 1] = i < nx ? u_raw[i - 1] : 0.0;
  }
  for (int i = 1; i <= nx + 1; i++) {
    rdxc[i - 1] = 1.0 / DXC(i);
    rdxc_f[i - 1] = (float)rdxc[i - 1];
    dxi[i - 1] = 1. / DXC(i);
  }
  std::vector<double> pfac(L.pstride * nh);
  for (int J = 0; J < nh; J++)
    partition_factors(nx, lo.data(), hi.data(), l_raw.data(), u_raw.data(), poisson_eigenvalue(dy, ny, J), J == 0,
                      false, pfac.data() + L.pstride * J);
  const std::vector<double> tw = twiddle_table(ny);
  std::vector<double> temp((size_t)(nx + 2) * (ny + 2));
  if (st) temp_init = st->temp;
  if (temp_init) {
    std::memcpy(temp.data(), temp_init, sizeof(double) * temp.size());
  } else {
    initial_temperature(d, xc.data(), temp.data());
  }
  std::vector<float> t_dense((size_t)nx * ny), t_low((size_t)nx * ny);
  for (int j = 1; j <= ny; j++)
    for (int i = 1; i <= nx; i++) {
      const double v = temp[(size_t)j * (nx + 2) + i];
      const float hi = (float)v;
      t_dense[(size_t)(j - 1) * nx + (i - 1)] = hi;
      t_low[(size_t)(j - 1) * nx + (i - 1)] = (float)(v - (double)hi);
    }
  auto put = [&](size_t o, const void *src, size_t bytes) {
    return cudaMemcpyAsync(base + o, src, bytes, cudaMemcpyHostToDevice, b->stream);
  };
  const size_t cells = (size_t)nx * ny;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  chk(put(L.rdxf_f, rdxf_f.data(), sizeof(float) * nx));
  chk(put(L.rdxf_l, rdxf_l.data(), sizeof(float) * nx));
  chk(put(L.rdxc_f, rdxc_f.data(), sizeof(float) * (nx + 1)));
  chk(put(L.ccm_f, ccm.data(), sizeof(float) * nx));
  chk(put(L.ccp_f, ccp.data(), sizeof(float) * nx));
  chk(put(L.cfm_f, cfm.data(), sizeof(float) * nx));
  chk(put(L.cfp_f, cfp.data(), sizeof(float) * nx));
  chk(put(L.rdxf, rdxf.data(), sizeof(double) * nx));
  chk(put(L.rdxc, rdxc.data(), sizeof(double) * (nx + 1)));
  chk(put(L.dxi, dxi.data(), sizeof(double) * (nx + 1)));
  chk(put(L.dxf, dxf.data(), sizeof(double) * nx));
  chk(put(L.dxc, dxc.data(), sizeof(double) * (nx + 1)));
  chk(put(L.tw, tw.data(), sizeof(double) * tw.size()));
  chk(put(L.lo, lo.data(), sizeof(double) * nx));
  chk(put(L.hi, hi.data(), sizeof(double) * nx));
  chk(put(L.pfac, pfac.data(), sizeof(double) * pfac.size()));
  chk(put(L.ccm, ccm_d.data(), sizeof(double) * nx));
  chk(put(L.ccp, ccp_d.data(), sizeof(double) * nx));
  chk(put(L.cfm, cfm_d.data(), sizeof(double) * nx));
  chk(put(L.cfp, cfp_d.data(), sizeof(double) * nx));
  for (int k = 0; k < 2; k++) {
    chk(cudaMemsetAsync(base + L.ux[k], 0, sizeof(float) * cells, b->stream));
    chk(cudaMemsetAsync(base + L.uy[k], 0, sizeof(float) * cells, b->stream));
  }
  // restart: velocity as compensated pairs, pressure as is; and the first dt
  // from its maximum exactly as the correction kernel and k_b_dt form it
  std::vector<float> ux_h, ux_l, uy_h, uy_l;
  std::vector<double> p_d;
  float ux_max = 0.f, uy_max = 0.f;
  if (st) {
    ux_h.assign(cells, 0.f);
    ux_l.assign(cells, 0.f);
    uy_h.assign(cells, 0.f);
    uy_l.assign(cells, 0.f);
    p_d.assign(cells, 0.0);
    for (int j = 1; j <= ny; j++)
      for (int x = 0; x < nx; x++) {
        const size_t k = (size_t)(j - 1) * nx + x;
        if (x >= 1) {  // ux at i = x+1 (x = 0 is the wall i = 1, kept zero)
          const double v = st->ux[(size_t)j * (nx + 1) + x];
          ux_h[k] = (float)v;
          ux_l[k] = (float)(v - (double)ux_h[k]);
          ux_max = std::fmax(ux_max, std::fabs(ux_h[k]) * rdxc_f[x]);
        }
        const double w = st->uy[(size_t)j * (nx + 2) + x + 1];
        uy_h[k] = (float)w;
        uy_l[k] = (float)(w - (double)uy_h[k]);
        uy_max = std::fmax(uy_max, std::fabs(uy_h[k]) * (float)(1.0 / dy));
        p_d[k] = st->p[(size_t)j * (nx + 2) + x + 1];
      }
    chk(put(L.ux[0], ux_h.data(), sizeof(float) * cells));
    chk(put(L.uxl[0], ux_l.data(), sizeof(float) * cells));
    chk(put(L.uy[0], uy_h.data(), sizeof(float) * cells));
    chk(put(L.uyl[0], uy_l.data(), sizeof(float) * cells));
  }
  chk(put(L.t[0], t_dense.data(), sizeof(float) * cells));
  chk(put(L.tl[0], t_low.data(), sizeof(float) * cells));
  chk(cudaMemsetAsync(base + L.tl[1], 0, sizeof(float) * cells, b->stream));
  for (int k = st ? 1 : 0; k < 2; k++) {
    chk(cudaMemsetAsync(base + L.uxl[k], 0, sizeof(float) * cells, b->stream));
    chk(cudaMemsetAsync(base + L.uyl[k], 0, sizeof(float) * cells, b->stream));
  }
  chk(cudaMemsetAsync(base + L.t[1], 0, sizeof(float) * cells, b->stream));
  for (size_t o : {L.aux, L.auy, L.at}) chk(cudaMemsetAsync(base + o, 0, sizeof(float) * cells, b->stream));
  if (x2)
    for (size_t o : {L.auxl, L.auyl, L.atl}) chk(cudaMemsetAsync(base + o, 0, sizeof(float) * cells, b->stream));
  if (st) {
    chk(put(L.p, p_d.data(), sizeof(double) * cells));
  } else {
    chk(cudaMemsetAsync(base + L.p, 0, sizeof(double) * cells, b->stream));
  }
  chk(cudaMemsetAsync(base + L.psi, 0, sizeof(double) * cells, b->stream));
  chk(cudaMemsetAsync(base + L.spec, 0, sizeof(double2) * (size_t)nh * nx, b->stream));
  // ---- table entry
  BCase t;
  std::memset(&t, 0, sizeof t);
  t.nx = nx;
  t.ny = ny;
  t.nh = nh;
  fft_layout(ny, &t.fft_nst, &t.fft_first2);
  int fc = std::min(8192 / ny, nx / 128);
  fc = std::max(1, std::min(8, fc));
  t.fcols = fc;
  t.with_t = d->with_temperature ? 1 : 0;
  t.with_force = d->with_thermal_forcing ? 1 : 0;
  t.seg = nx / kSeg;
  t.dy = dy;
  t.rdy = 1.0 / dy;
  t.rdy_f = (float)t.rdy;
  t.rdy_l = (float)(t.rdy - (double)t.rdy_f);
  t.kappa_f = (float)(1. / sqrt(d->Pr) / sqrt(d->Ra));
  t.nu_f = (float)(sqrt(d->Pr) / sqrt(d->Ra));
  t.kappa = 1. / sqrt(d->Pr) / sqrt(d->Ra);
  t.nu = sqrt(d->Pr) / sqrt(d->Ra);
  t.x2 = x2 ? 1 : 0;
  {  // explicit diffusive limits (src/param/decide_dt.c:62-74)
    const double diffusivity = fmax(sqrt(d->Pr) / sqrt(d->Ra), 1. / sqrt(d->Pr) / sqrt(d->Ra));
    double dx = 1.0;
    for (int i = 2; i <= nx; i++) dx = fmin(dx, DXC(i));
    const double ddx = 0.25 / diffusivity * pow(dx, 2.) * 0.9, ddy = 0.25 / diffusivity * pow(dy, 2.) * 0.9;
    t.dt_dif = fmin(ddx, ddy);
  }
  t.fixed_dt = d->fixed_dt;
  t.target_steps = d->steps;
  t.rdxf_f = reinterpret_cast<const float *>(base + L.rdxf_f);
  t.rdxf_l = reinterpret_cast<const float *>(base + L.rdxf_l);
  t.rdxc_f = reinterpret_cast<const float *>(base + L.rdxc_f);
  t.ccm_f = reinterpret_cast<const float *>(base + L.ccm_f);
  t.ccp_f = reinterpret_cast<const float *>(base + L.ccp_f);
  t.cfm_f = reinterpret_cast<const float *>(base + L.cfm_f);
  t.cfp_f = reinterpret_cast<const float *>(base + L.cfp_f);
  t.rdxf = reinterpret_cast<const double *>(base + L.rdxf);
  t.rdxc = reinterpret_cast<const double *>(base + L.rdxc);
  t.dxi = reinterpret_cast<const double *>(base + L.dxi);
  t.ccm = reinterpret_cast<const double *>(base + L.ccm);
  t.ccp = reinterpret_cast<const double *>(base + L.ccp);
  t.cfm = reinterpret_cast<const double *>(base + L.cfm);
  t.cfp = reinterpret_cast<const double *>(base + L.cfp);
  t.dxf = reinterpret_cast<const double *>(base + L.dxf);
  t.dxc = reinterpret_cast<const double *>(base + L.dxc);
  t.tw = reinterpret_cast<const double *>(base + L.tw);
  t.lo = reinterpret_cast<const double *>(base + L.lo);
  t.hi = reinterpret_cast<const double *>(base + L.hi);
  t.pfac = reinterpret_cast<const double *>(base + L.pfac);
  t.pstride = L.pstride;
  for (int k = 0; k < 2; k++) {
    t.ux[k] = reinterpret_cast<float *>(base + L.ux[k]);
    t.uy[k] = reinterpret_cast<float *>(base + L.uy[k]);
    t.t[k] = reinterpret_cast<float *>(base + L.t[k]);
  }
  for (int k = 0; k < 2; k++) {
    t.uxl[k] = reinterpret_cast<float *>(base + L.uxl[k]);
    t.uyl[k] = reinterpret_cast<float *>(base + L.uyl[k]);
    t.tl[k] = reinterpret_cast<float *>(base + L.tl[k]);
  }
  t.aux = reinterpret_cast<float *>(base + L.aux);
  t.auy = reinterpret_cast<float *>(base + L.auy);
  t.at = reinterpret_cast<float *>(base + L.at);
  t.auxl = x2 ? reinterpret_cast<float *>(base + L.auxl) : nullptr;
  t.auyl = x2 ? reinterpret_cast<float *>(base + L.auyl) : nullptr;
  t.atl = x2 ? reinterpret_cast<float *>(base + L.atl) : nullptr;
  t.p = reinterpret_cast<double *>(base + L.p);
  t.psi = reinterpret_cast<double *>(base + L.psi);
  t.spec = reinterpret_cast<double2 *>(base + L.spec);
  t.par = 0;
  t.done = 0;
  t.step = st ? st->step : 0;
  t.time = st ? st->time : 0.0;
  if (t.target_steps > 0 && t.step >= t.target_steps) t.done = 1;
  // first dt: from u = 0 the advective limit 0.7 * 0.05 (src/param/decide_dt.c:42);
  // on restart the rule of k_b_dt on the restored velocity
  double dt_adv = 5.e-2;
  if (ux_max > 0.f) dt_adv = fmin(dt_adv, 1.0 / (double)ux_max);
  if (uy_max > 0.f) dt_adv = fmin(dt_adv, 1.0 / (double)uy_max);
  dt_adv *= 0.7;
  t.dt = d->fixed_dt > 0 ? d->fixed_dt : fmin(dt_adv, t.dt_dif);
  for (int k = 0; k < 3; k++) {
    t.adt[k] = b->rk_a[k] * t.dt;
    t.bdt[k] = b->rk_b[k] * t.dt;
    t.gdt[k] = (b->rk_a[k] + b->rk_b[k]) * t.dt;
    t.rgdt[k] = 1. / t.gdt[k];
  }
  chk(cudaMemcpyAsync(b->d_cases + slot, &t, sizeof(BCase), cudaMemcpyHostToDevice, b->stream));
  chk(cudaStreamSynchronize(b->stream));  // host staging vectors die at return
  if (e != cudaSuccess) {
    arena_free(b, off, L.total);
    return bfail(SNS_ERR_CUDA, "sns_batch_add: %s", cudaGetErrorString(e));
  }
  b->table[slot] = t;
  CaseHost &h = b->hc[slot];
  h.used = true;
  h.d = *d;
  h.off = off;
  h.bytes = L.total;
  h.steps_done = t.step;
  h.fcols = fc;
  b->dirty = true;
  if (slot_out) *slot_out = slot;
  return SNS_OK;
}

extern "C" {

int sns_batch_add(sns_batch *b, const sns_case_desc *d, const double *temp_init, int *slot_out) {
  if (!b) return bfail(SNS_ERR_ARG, "NULL batch");
  if (int rc = check_desc(d)) return rc;
  std::lock_guard<std::mutex> lk(b->mu);
  return admit(b, d, temp_init, nullptr, slot_out);
}

// restart of a case from the reference's save layout (src/param/init.c:245-247,
// src/fluid/init.c:53-81, src/temperature/init.c:51)
int sns_batch_add_restart(sns_batch *b, const sns_case_desc *d, const char *dirname, int *slot_out) {
  if (!b || !dirname) return bfail(SNS_ERR_ARG, "sns_batch_add_restart: bad argument");
  if (int rc = check_desc(d)) return rc;
  const int nx = d->itot, ny = d->jtot;
  std::vector<double> ux((size_t)(nx + 1) * (ny + 2), 0.0), uy((size_t)(nx + 2) * (ny + 2), 0.0),
      p(uy.size(), 0.0), temp(uy.size(), 0.0);
  const std::string dir(dirname);
  std::string err;
  int step = 0;
  double time = 0.0;
  const size_t su[2] = {(size_t)ny, (size_t)nx + 1}, sc[2] = {(size_t)ny, (size_t)nx + 2};
  if (npy_read((dir + "/step.npy").c_str(), "'int32'", 0, nullptr, &step, sizeof(int), &err) ||
      npy_read((dir + "/time.npy").c_str(), "'float64'", 0, nullptr, &time, sizeof(double), &err) ||
      npy_read((dir + "/ux.npy").c_str(), "'float64'", 2, su, ux.data() + (nx + 1), sizeof(double) * su[0] * su[1],
               &err) ||
      npy_read((dir + "/uy.npy").c_str(), "'float64'", 2, sc, uy.data() + (nx + 2), sizeof(double) * sc[0] * sc[1],
               &err) ||
      npy_read((dir + "/p.npy").c_str(), "'float64'", 2, sc, p.data() + (nx + 2), sizeof(double) * sc[0] * sc[1],
               &err))
    return bfail(SNS_ERR_ARG, "sns_batch_add_restart: %s", err.c_str());
  if (d->with_temperature &&
      npy_read((dir + "/temp.npy").c_str(), "'float64'", 2, sc, temp.data() + (nx + 2), sizeof(double) * sc[0] * sc[1],
               &err))
    return bfail(SNS_ERR_ARG, "sns_batch_add_restart: %s", err.c_str());
  const StartState st{ux.data(), uy.data(), p.data(), temp.data(), step, time};
  std::lock_guard<std::mutex> lk(b->mu);
  return admit(b, d, nullptr, &st, slot_out);
}

int sns_batch_remove(sns_batch *b, int slot) {
  if (!b || slot < 0 || slot >= b->max_cases || !b->hc[slot].used) return bfail(SNS_ERR_ARG, "bad slot");
  std::lock_guard<std::mutex> lk(b->mu);
  BCUDA(cudaStreamSynchronize(b->stream));
  BCase empty;
  std::memset(&empty, 0, sizeof empty);
  empty.done = 1;
  BCUDA(cudaMemcpy(b->d_cases + slot, &empty, sizeof(BCase), cudaMemcpyHostToDevice));
  b->table[slot] = empty;
  arena_free(b, b->hc[slot].off, b->hc[slot].bytes);
  b->hc[slot] = CaseHost();
  b->dirty = true;
  return SNS_OK;
}

int sns_batch_step(sns_batch *b, int nsteps) {
  if (!b || nsteps < 0) return bfail(SNS_ERR_ARG, "sns_batch_step: bad argument");
  std::lock_guard<std::mutex> lk(b->mu);
  for (int s = 0; s < nsteps; s++) {
    if (b->dirty)
      if (int rc = rebuild(b)) return rc;
    if (b->ntiles == 0) break;
    BCUDA(cudaGraphLaunch(b->exec, b->stream));
    count_launches(b->graph_launches);
    if (b->tri_stale) {  // a test's stale wait applies to one step
      b->tri_stale = 0;
      b->dirty = true;
    }
    bool finished_one = false;
    for (CaseHost &h : b->hc) {
      if (!h.used || (h.d.steps > 0 && h.steps_done >= h.d.steps)) continue;
      h.steps_done++;
      if (h.d.steps > 0 && h.steps_done >= h.d.steps) finished_one = true;
    }
    if (finished_one) b->dirty = true;  // drop finished cases from the work lists
  }
  return SNS_OK;
}

static bool valid_tuning(const sns_batch_tuning &t) {
  return (t.tile_x == 32 || t.tile_x == 64 || t.tile_x == 128) && (t.tile_rows >= 1 && t.tile_rows <= 64) &&
         (t.modes_per_block == 2 || t.modes_per_block == 4 || t.modes_per_block == 8) && t.fcols_shift >= -3 &&
         t.fcols_shift <= 3;
}

int sns_batch_get_tuning(const sns_batch *b, sns_batch_tuning *t) {
  if (!b || !t) return bfail(SNS_ERR_ARG, "sns_batch_get_tuning: bad argument");
  *t = b->tune;
  return SNS_OK;
}

int sns_batch_set_tuning(sns_batch *b, const sns_batch_tuning *t) {
  if (!b || !t || !valid_tuning(*t)) return bfail(SNS_ERR_ARG, "sns_batch_set_tuning: bad tuning");
  std::lock_guard<std::mutex> lk(b->mu);
  b->tune = *t;
  b->dirty = true;
  return SNS_OK;
}

// Coordinate search over the launch shapes on the resident cases. Their
// device state (the arena up to its high-water mark and the case table) is
// copied aside first and put back before every candidate and at the end, so
// tuning leaves every case exactly where it was.
int sns_batch_autotune(sns_batch *b, int steps, sns_batch_tuning *chosen, double *ms_per_step) {
  if (!b || steps < 1) return bfail(SNS_ERR_ARG, "sns_batch_autotune: bad argument");
  std::lock_guard<std::mutex> lk(b->mu);
  size_t high = 0;
  bool any = false;
  for (const CaseHost &h : b->hc)
    if (h.used) {
      high = std::max(high, h.off + h.bytes);
      any = any || !(h.d.steps > 0 && h.steps_done >= h.d.steps);
    }
  if (!any) return bfail(SNS_ERR_STATE, "sns_batch_autotune: no active case to tune on");
  char *save = nullptr;
  BCase *save_table = nullptr;
  if (counted_malloc((void **)&save, std::max<size_t>(high, 1)) != cudaSuccess ||
      counted_malloc((void **)&save_table, sizeof(BCase) * b->max_cases) != cudaSuccess) {
    cudaGetLastError();
    if (save) cudaFree(save);
    return bfail(SNS_ERR_OOM, "sns_batch_autotune: %zu bytes for the state snapshot are not available", high);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = SNS_OK;
  auto cuda = [&](cudaError_t e, const char *what) {
    if (rc == SNS_OK && e != cudaSuccess) rc = bfail(SNS_ERR_CUDA, "sns_batch_autotune: %s: %s", what, cudaGetErrorString(e));
    return rc == SNS_OK;
  };
  std::vector<int> fc0(b->max_cases);
  for (int c = 0; c < b->max_cases; c++) fc0[c] = b->table[c].fcols;
  auto restore = [&]() {
    for (int c = 0; c < b->max_cases; c++) b->table[c].fcols = fc0[c];  // as in the restored device table
    cuda(cudaMemcpyAsync(b->arena, save, high, cudaMemcpyDeviceToDevice, b->stream), "restore");
    cuda(cudaMemcpyAsync(b->d_cases, save_table, sizeof(BCase) * b->max_cases, cudaMemcpyDeviceToDevice, b->stream),
         "restore");
  };
  cuda(cudaEventCreate(&e0), "event");
  cuda(cudaEventCreate(&e1), "event");
  cuda(cudaMemcpyAsync(save, b->arena, high, cudaMemcpyDeviceToDevice, b->stream), "snapshot");
  cuda(cudaMemcpyAsync(save_table, b->d_cases, sizeof(BCase) * b->max_cases, cudaMemcpyDeviceToDevice, b->stream),
       "snapshot");
  const sns_batch_tuning start = b->tune;
  auto measure = [&](const sns_batch_tuning &t) -> double {
    b->tune = t;
    if (rc != SNS_OK || rebuild(b) != SNS_OK) {
      if (rc == SNS_OK) rc = SNS_ERR_CUDA;
      return 1e30;
    }
    float ms = 0.f;
    cuda(cudaGraphLaunch(b->exec, b->stream), "warm-up");  // table's fcols may have changed: one untimed step
    cuda(cudaEventRecord(e0, b->stream), "event");
    for (int s = 0; s < steps; s++) cuda(cudaGraphLaunch(b->exec, b->stream), "step");
    cuda(cudaEventRecord(e1, b->stream), "event");
    cuda(cudaEventSynchronize(e1), "sync");
    cuda(cudaEventElapsedTime(&ms, e0, e1), "timing");
    restore();
    return rc == SNS_OK ? ms / steps : 1e30;
  };
  sns_batch_tuning best = start;
  double best_ms = measure(best);
  const int rows[] = {4, 8, 16}, widths[] = {32, 64, 128}, shifts[] = {-1, 0, 1}, mpbs[] = {2, 4, 8};
  for (int dim = 0; dim < 4 && rc == SNS_OK; dim++) {
    for (int k = 0; k < 3 && rc == SNS_OK; k++) {
      sns_batch_tuning t = best;
      if (dim == 0) t.tile_rows = rows[k];
      if (dim == 1) t.tile_x = widths[k];
      if (dim == 2) t.fcols_shift = shifts[k];
      if (dim == 3) t.modes_per_block = mpbs[k];
      if (std::memcmp(&t, &best, sizeof t) == 0) continue;
      const double ms = measure(t);
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
  }
  b->tune = rc == SNS_OK ? best : start;
  b->dirty = true;
  cudaStreamSynchronize(b->stream);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(save);
  cudaFree(save_table);
  if (rc != SNS_OK) return rc;
  if (int r = rebuild(b)) return r;
  if (chosen) *chosen = best;
  if (ms_per_step) *ms_per_step = best_ms;
  return SNS_OK;
}

int sns_batch_synchronize(sns_batch *b) {
  if (!b) return bfail(SNS_ERR_ARG, "NULL batch");
  // this batch's own error word, read in stream order
  BCUDA(cudaMemcpyAsync(b->h_err, b->d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, b->stream));
  BCUDA(cudaStreamSynchronize(b->stream));
  if (const unsigned e = *b->h_err) {
    *b->h_err = 0;
    BCUDA(cudaMemsetAsync(b->d_err, 0, sizeof(unsigned), b->stream));
    BCUDA(cudaMemsetAsync(b->d_bar, 0, 2 * sizeof(unsigned), b->stream));  // a barrier that gave up
    return bfail(SNS_ERR_STATE,
                 "batched step: a bounded wait gave up (code %u: 1 a tridiagonal bulk copy, 2 a persistent launch's "
                 "grid barrier); results are invalid",
                 e);
  }
  return SNS_OK;
}

int sns_batch_set_persistent(sns_batch *b, int on) {
  if (!b) return bfail(SNS_ERR_ARG, "NULL batch");
  std::lock_guard<std::mutex> lk(b->mu);
  b->persistent = on != 0;
  b->dirty = true;
  return SNS_OK;
}

int sns_batch_set_wait_limit(sns_batch *b, unsigned polls, int stale) {
  if (!b) return bfail(SNS_ERR_ARG, "NULL batch");
  std::lock_guard<std::mutex> lk(b->mu);
  b->tri_spin = polls ? polls : (1u << 22);
  b->tri_stale = stale != 0;
  b->dirty = true;  // the step graph carries both as launch parameters
  return SNS_OK;
}

int sns_batch_cases(const sns_batch *b, int *slots, int max) {
  if (!b) return 0;
  int n = 0;
  for (int c = 0; c < b->max_cases; c++)
    if (b->hc[c].used) {
      if (slots && n < max) slots[n] = c;
      n++;
    }
  return n;
}

long long sns_batch_active_cells(const sns_batch *b) {
  if (!b) return 0;
  long long cells = 0;
  for (const CaseHost &h : b->hc)
    if (h.used && !(h.d.steps > 0 && h.steps_done >= h.d.steps)) cells += (long long)h.d.itot * h.d.jtot;
  return cells;
}

int sns_batch_case_status(sns_batch *b, int slot, double *time, double *dt, long long *step, int *done) {
  if (!b || slot < 0 || slot >= b->max_cases || !b->hc[slot].used) return bfail(SNS_ERR_ARG, "bad slot");
  BCase t;
  BCUDA(cudaStreamSynchronize(b->stream));
  BCUDA(cudaMemcpy(&t, b->d_cases + slot, sizeof(BCase), cudaMemcpyDeviceToHost));
  if (time) *time = t.time;
  if (dt) *dt = t.dt;
  if (step) *step = t.step;
  if (done) *done = t.done;
  if (t.nonfinite)
    return bfail(SNS_ERR_NONFINITE, "case in slot %d holds NaN or infinity (step %lld)", slot, t.step);
  return SNS_OK;
}

int sns_batch_state(sns_batch *b, int slot, double *ux, double *uy, double *p, double *psi, double *temp) {
  if (!b || slot < 0 || slot >= b->max_cases || !b->hc[slot].used) return bfail(SNS_ERR_ARG, "bad slot");
  std::lock_guard<std::mutex> lk(b->mu);
  BCase t;
  BCUDA(cudaStreamSynchronize(b->stream));
  BCUDA(cudaMemcpy(&t, b->d_cases + slot, sizeof(BCase), cudaMemcpyDeviceToHost));
  const int nx = t.nx, ny = t.ny;
  const size_t cells = (size_t)nx * ny;
  if (b->staging_bytes < sizeof(double) * cells) {
    if (b->staging) cudaFreeHost(b->staging);
    b->staging = nullptr;
    BCUDA(counted_malloc_host((void **)&b->staging, sizeof(double) * cells));
    b->staging_bytes = sizeof(double) * cells;
  }
  const int cur = t.par;
  // compensated FP32 storage: value = hi + lo, exact in double
  auto fetch_f = [&](const float *src, const float *low, std::vector<double> &dst) -> int {
    BCUDA(cudaMemcpy(b->staging, src, sizeof(float) * cells, cudaMemcpyDeviceToHost));
    BCUDA(cudaMemcpy(reinterpret_cast<float *>(b->staging) + cells, low, sizeof(float) * cells,
                     cudaMemcpyDeviceToHost));
    const float *f = reinterpret_cast<const float *>(b->staging);
    dst.resize(cells);
    for (size_t k = 0; k < cells; k++) dst[k] = (double)f[k] + (double)f[cells + k];
    return SNS_OK;
  };
  auto fetch_d = [&](const double *src, std::vector<double> &dst) -> int {
    BCUDA(cudaMemcpy(b->staging, src, sizeof(double) * cells, cudaMemcpyDeviceToHost));
    dst.assign(b->staging, b->staging + cells);
    return SNS_OK;
  };
  std::vector<double> v;
  if (ux) {
    if (int rc = fetch_f(t.ux[cur], t.uxl[cur], v)) return rc;
    std::memset(ux, 0, sizeof(double) * (size_t)(nx + 1) * (ny + 2));
    for (int j = 1; j <= ny; j++)
      for (int i = 2; i <= nx; i++) ux[(size_t)j * (nx + 1) + (i - 1)] = v[(size_t)(j - 1) * nx + (i - 1)];
    for (int i = 2; i <= nx; i++) {
      ux[i - 1] = ux[(size_t)ny * (nx + 1) + (i - 1)];
      ux[(size_t)(ny + 1) * (nx + 1) + (i - 1)] = ux[(size_t)(nx + 1) + (i - 1)];
    }
  }
  auto centred = [&](std::vector<double> &src, double *dst, int wall_mode) {
    // wall_mode 0: zero walls (uy), 1: Neumann (p, psi), 2: temperature walls
    std::memset(dst, 0, sizeof(double) * (size_t)(nx + 2) * (ny + 2));
    for (int j = 1; j <= ny; j++)
      for (int i = 1; i <= nx; i++) dst[(size_t)j * (nx + 2) + i] = src[(size_t)(j - 1) * nx + (i - 1)];
    for (int i = 1; i <= nx; i++) {
      dst[i] = dst[(size_t)ny * (nx + 2) + i];
      dst[(size_t)(ny + 1) * (nx + 2) + i] = dst[(size_t)(nx + 2) + i];
    }
    const int j0 = wall_mode == 2 ? 1 : 0, j1 = wall_mode == 2 ? ny : ny + 1;
    for (int j = j0; j <= j1; j++) {
      double *row = dst + (size_t)j * (nx + 2);
      if (wall_mode == 0) {
        row[0] = 0.;
        row[nx + 1] = 0.;
      } else if (wall_mode == 1) {
        row[0] = row[1];
        row[nx + 1] = row[nx];
      } else {
        row[0] = TEMP_XM;
        row[nx + 1] = TEMP_XP;
      }
    }
  };
  if (uy) {
    if (int rc = fetch_f(t.uy[cur], t.uyl[cur], v)) return rc;
    centred(v, uy, 0);
  }
  if (p) {
    if (int rc = fetch_d(t.p, v)) return rc;
    centred(v, p, 1);
  }
  if (psi) {
    if (int rc = fetch_d(t.psi, v)) return rc;
    centred(v, psi, 1);
  }
  if (temp) {
    if (int rc = fetch_f(t.t[cur], t.tl[cur], v)) return rc;
    centred(v, temp, 2);
  }
  return SNS_OK;
}

}  // extern "C"

extern "C" // a case's state in the reference's save layout (src/save.c:13-68): the same
// files sns_checkpoint writes for the plain path; velocity and temperature
// are the compensated FP32 pairs widened exactly (hi + lo)
extern "C" int sns_batch_checkpoint(sns_batch *b, int slot, const char *dirname) {
  if (!b || slot < 0 || slot >= b->max_cases || !b->hc[slot].used || !dirname)
    return bfail(SNS_ERR_ARG, "sns_batch_checkpoint: bad argument");
  const sns_case_desc d = b->hc[slot].d;
  const int nx = d.itot, ny = d.jtot;
  std::vector<double> ux((size_t)(nx + 1) * (ny + 2)), uy((size_t)(nx + 2) * (ny + 2)), p(uy.size()), psi(uy.size()),
      temp(uy.size());
  if (int rc = sns_batch_state(b, slot, ux.data(), uy.data(), p.data(), psi.data(), temp.data())) return rc;
  double time = 0.0, dt = 0.0;
  long long step = 0;
  int done = 0;
  // a diverged case is saved as it is (the reference's save() writes NaN too)
  if (int rc = sns_batch_case_status(b, slot, &time, &dt, &step, &done); rc && rc != SNS_ERR_NONFINITE) return rc;
  std::vector<double> xf(nx + 1), xc(nx + 2), dxf(nx), dxc(nx + 1), yf(ny + 1), yc(ny);
  double dy;
  make_grid(nx, ny, 1.0, d.ly, d.stretch, xf.data(), xc.data(), dxf.data(), dxc.data(), yf.data(), yc.data(), &dy);
  std::string err, dir(dirname);
  if (make_dirs(dirname, &err)) return bfail(SNS_ERR_ARG, "sns_batch_checkpoint: %s", err.c_str());
  auto path = [&](const char *n) { return dir + "/" + n + ".npy"; };
  int rc = 0;
  const int istep = (int)step, itot = nx, jtot = ny;
  const double lx = 1.0;
  auto w0 = [&](const char *n, const char *dtype, const void *v, size_t bytes) {
    if (!rc) rc = npy_write(path(n).c_str(), dtype, 0, nullptr, v, bytes, &err);
  };
  auto w1 = [&](const char *n, const std::vector<double> &v) {
    const size_t shape[1] = {v.size()};
    if (!rc) rc = npy_write(path(n).c_str(), "'float64'", 1, shape, v.data(), sizeof(double) * v.size(), &err);
  };
  auto w2 = [&](const char *n, const std::vector<double> &v, size_t w) {
    const size_t shape[2] = {(size_t)ny, w};
    if (!rc) rc = npy_write(path(n).c_str(), "'float64'", 2, shape, v.data() + w, sizeof(double) * w * ny, &err);
  };
  w0("step", "'int32'", &istep, sizeof(int));
  w0("itot", "'int32'", &itot, sizeof(int));
  w0("jtot", "'int32'", &jtot, sizeof(int));
  w0("time", "'float64'", &time, sizeof(double));
  w0("lx", "'float64'", &lx, sizeof(double));
  w0("ly", "'float64'", &d.ly, sizeof(double));
  w0("Ra", "'float64'", &d.Ra, sizeof(double));
  w0("Pr", "'float64'", &d.Pr, sizeof(double));
  w1("xf", xf);
  w1("xc", xc);
  w1("yf", yf);
  w1("yc", yc);
  w2("ux", ux, (size_t)nx + 1);
  w2("uy", uy, (size_t)nx + 2);
  w2("p", p, (size_t)nx + 2);
  if (d.with_temperature) w2("temp", temp, (size_t)nx + 2);
  if (rc) return bfail(SNS_ERR_ARG, "sns_batch_checkpoint: %s", err.c_str());
  return SNS_OK;
}

int sns_batch_diagnostics(sns_batch *b, int slot, double out[11]) {
  if (!b || slot < 0 || slot >= b->max_cases || !b->hc[slot].used || !out) return bfail(SNS_ERR_ARG, "bad slot");
  std::lock_guard<std::mutex> lk(b->mu);
  BCase t;
  BCUDA(cudaStreamSynchronize(b->stream));
  BCUDA(cudaMemcpy(&t, b->d_cases + slot, sizeof(BCase), cudaMemcpyDeviceToHost));
  const size_t words = diag_partials_words(t.nx, t.ny);
  if (b->diag_words < words) {
    cudaFree(b->diag);
    b->diag = nullptr;
    BCUDA(counted_malloc((void **)&b->diag, sizeof(double) * words));
    b->diag_words = words;
  }
  const sns_case_desc &d = b->hc[slot].d;
  const DiagArgs<float> a{t.nx,
                          t.ny,
                          t.dy,
                          d.ly,
                          sqrt(d.Pr) * sqrt(d.Ra),
                          sqrt(d.Pr) / sqrt(d.Ra),
                          1. / sqrt(d.Pr) / sqrt(d.Ra),
                          t.dxf,
                          t.dxc,
                          t.ux[t.par],
                          t.uy[t.par],
                          t.t[t.par],
                          t.uxl[t.par],
                          t.uyl[t.par],
                          t.tl[t.par]};
  int nb = 0;
  BCUDA(launch_diag(a, b->diag, &nb, b->stream));
  count_launches(1);
  std::vector<double> h(words);
  BCUDA(cudaMemcpyAsync(h.data(), b->diag, sizeof(double) * words, cudaMemcpyDeviceToHost, b->stream));
  BCUDA(cudaStreamSynchronize(b->stream));
  diag_finish(h.data(), nb, d.ly, out);
  return SNS_OK;
}

// ---------------------------------------------------------------- serving
#include <chrono>
#include <deque>
#include <thread>

extern "C" int sns_serve(const sns_case_desc *reqs, const double *arrival_s, int n, size_t hbm_bytes, int max_cases,
                         int chunk_steps, double *admit_s, double *done_s, double *busy_s, sns_done_fn on_done,
                         void *user) {
  if (!reqs || !arrival_s || n <= 0 || chunk_steps <= 0 || !admit_s || !done_s)
    return bfail(SNS_ERR_ARG, "sns_serve: bad argument");
  for (int r = 0; r < n; r++) {
    if (int rc = check_desc(&reqs[r])) return rc;
    if (reqs[r].steps <= 0) return bfail(SNS_ERR_ARG, "sns_serve: request %d has no step count", r);
    if (r > 0 && arrival_s[r] < arrival_s[r - 1]) return bfail(SNS_ERR_ARG, "sns_serve: arrivals must not decrease");
    if (layout_for(reqs[r].itot, reqs[r].jtot, reqs[r].compensated != 0).total > hbm_bytes)
      return bfail(SNS_ERR_OOM, "sns_serve: request %d is larger than the arena", r);
  }
  sns_batch *b = sns_batch_create(hbm_bytes, max_cases);
  if (!b) return SNS_ERR_OOM;
  using clock = std::chrono::steady_clock;
  const auto t0 = clock::now();
  auto now = [&]() { return std::chrono::duration<double>(clock::now() - t0).count(); };
  std::deque<int> waiting;
  std::vector<int> slot_req(max_cases, -1);
  int next = 0, completed = 0, resident = 0;
  double first_admit = -1.0, last_done = 0.0;
  int rc = SNS_OK;
  while (completed < n && rc == SNS_OK) {
    double t = now();
    while (next < n && arrival_s[next] <= t) waiting.push_back(next++);
    while (!waiting.empty()) {  // FIFO admission while the head fits
      const int r = waiting.front();
      int slot = -1;
      const int a = sns_batch_add(b, &reqs[r], nullptr, &slot);
      if (a == SNS_ERR_OOM) break;
      if (a != SNS_OK) {
        rc = a;
        break;
      }
      waiting.pop_front();
      slot_req[slot] = r;
      admit_s[r] = now();
      if (first_admit < 0) first_admit = admit_s[r];
      resident++;
    }
    if (rc != SNS_OK) break;
    if (resident == 0) {
      if (next < n) std::this_thread::sleep_for(std::chrono::duration<double>(std::max(0.0, arrival_s[next] - now())));
      continue;
    }
    if ((rc = sns_batch_step(b, chunk_steps)) != SNS_OK) break;
    if ((rc = sns_batch_synchronize(b)) != SNS_OK) break;
    t = now();
    for (int s = 0; s < max_cases; s++) {
      const int r = slot_req[s];
      if (r < 0) continue;
      const CaseHost &h = b->hc[s];
      if (h.steps_done < h.d.steps) continue;
      done_s[r] = t;
      last_done = t;
      if (on_done) on_done(r, b, s, user);
      if ((rc = sns_batch_remove(b, s)) != SNS_OK) break;
      slot_req[s] = -1;
      resident--;
      completed++;
    }
  }
  if (busy_s) *busy_s = first_admit >= 0 ? last_done - first_admit : 0.0;
  sns_batch_destroy(b);
  return rc;
}
