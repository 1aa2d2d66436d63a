// Host orchestration and C ABI of the GB300 streaming-BASS engine.
//
// One context owns a device workspace sized for the largest frame seen so far.
// A frame is a fixed sequence of kernel launches on the caller's stream with no
// host synchronisation inside the BASS loop: data-dependent loops (split BFS, hole
// filling, connected components) run as bounded cooperative kernels, and the
// values the reference reads back to the host every step (done flags, max_spix,
// counts) stay on the device.  Propagated frames read one small struct back per
// frame (hole count and superpixel count: the iteration ladder and buffer sizing).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace stspix {

__global__ void k_frame_begin(Scalars* sc, int max_spix, int nbuf_logical) {
  sc->max_spix = max_spix;
  sc->nbuf_logical = nbuf_logical;
  sc->status = STSPIX_OK;
  sc->nsplits = sc->nmerges = sc->nrevived = sc->nminted = sc->near_ties = 0;
  sc->fill_iters = 0;
  sc->ninvalid = 0;
  sc->tmp0 = sc->tmp1 = sc->tmp2 = 0;
}
__global__ void k_bass_after_compact(Scalars* sc) {
  sc->max_spix = sc->nspix - 1;
}
__global__ void k_calc_n(Scalars* sc, int lo, int cap) {
  sc->tmp2 = min(sc->max_spix + 1, cap) - lo;  // ids beyond cap were never created
}
__global__ void k_finish_compact(Scalars* sc, int lo, const int* total) {
  sc->nspix = lo + *total;
}

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace stspix

using namespace stspix;

struct stspix_ctx {
  int device = 0;
  int num_sms = 0;
  std::string err;
  long long launches = 0;
  stspix_frame_log log{};
  // sizing
  int npix_cap = 0;
  int sp_cap = 0;
  // pixel buffers
  uint8_t* border = nullptr;
  int *d1 = nullptr, *d2 = nullptr, *smseg = nullptr, *hits = nullptr;
  int *shifted = nullptr, *filled = nullptr, *seg_alt = nullptr;
  unsigned long long* best = nullptr;
  // superpixel buffers
  SpDev sp{}, tmp{};
  SmDev sm{};
  uint8_t *flags = nullptr, *accept = nullptr, *valid0 = nullptr, *living = nullptr,
          *mint = nullptr;
  int *excl = nullptr, *rid = nullptr, *src_of = nullptr, *cnt_pool = nullptr, *cs = nullptr,
      *cf = nullptr;
  long long* fs = nullptr;
  float *fds = nullptr, *ss = nullptr;
  double* centers = nullptr;
  unsigned long long *rbest = nullptr, *ccbest = nullptr;
  // param ping-pong for bist_forward
  stspix_params pp[2]{};
  // control
  int* round_flags = nullptr;
  int* iter_counts = nullptr;
  Scalars* sc = nullptr;
  Scalars* sc_host = nullptr;  // pinned
  std::vector<Buf> pix_bufs, sp_bufs, pp_bufs;
  int pp_cap = 0;
  int coop_relax0 = 0, coop_relax1 = 0, coop_fill = 0;
  // profiling (CUDA events on the launching stream)
  int prof_on = 0;
  int cur_fam = STSPIX_FAM_OTHER;
  std::vector<cudaEvent_t> ev_free;
  struct Pending { int fam; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  long long fam_launches[STSPIX_NFAM] = {0};
  double fam_ms[STSPIX_NFAM] = {0};
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> frame_ev;
  std::vector<double> frame_ms;
};

namespace {

const int kThreads = 256;
inline unsigned blocks_for(long long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

int fail(stspix_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? STSPIX_ERR_NOMEM : STSPIX_ERR_CUDA, \
                  "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

cudaEvent_t ev_get(stspix_ctx* ctx) {
  if (!ctx->ev_free.empty()) {
    cudaEvent_t e = ctx->ev_free.back();
    ctx->ev_free.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}
inline cudaEvent_t prof_begin(stspix_ctx* ctx, cudaStream_t st) {
  if (!ctx->prof_on) return nullptr;
  cudaEvent_t e = ev_get(ctx);
  cudaEventRecord(e, st);
  return e;
}
inline void prof_end(stspix_ctx* ctx, cudaStream_t st, cudaEvent_t a) {
  if (!a) return;
  cudaEvent_t b = ev_get(ctx);
  cudaEventRecord(b, st);
  ctx->pending.push_back({ctx->cur_fam, a, b});
}
// Called after the stream has been synchronised.
void prof_harvest(stspix_ctx* ctx) {
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      ctx->fam_ms[p.fam] += ms;
      ctx->fam_launches[p.fam] += 1;
    }
    ctx->ev_free.push_back(p.a);
    ctx->ev_free.push_back(p.b);
  }
  ctx->pending.clear();
}

#define LAUNCHG(kernel, grid, block, ...)                                      \
  do {                                                                         \
    cudaEvent_t pe_ = prof_begin(ctx, st);                                     \
    kernel<<<grid, block, 0, st>>>(__VA_ARGS__);                               \
    ctx->launches++;                                                           \
    prof_end(ctx, st, pe_);                                                    \
  } while (0)

#define LAUNCH(kernel, n, ...)                                                 \
  do {                                                                         \
    long long n_ = (n);                                                        \
    if (n_ > 0) LAUNCHG(kernel, blocks_for(n_), kThreads, __VA_ARGS__);        \
  } while (0)

#define LAUNCH1(kernel, ...) LAUNCHG(kernel, 1, 1, __VA_ARGS__)

template <typename T>
int alloc(stspix_ctx* ctx, std::vector<Buf>& list, T** p, size_t n) {
  void* q = nullptr;
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&q, bytes);
  if (e != cudaSuccess)
    return fail(ctx, STSPIX_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", bytes, cudaGetErrorString(e));
  list.push_back({q, bytes});
  *p = (T*)q;
  return STSPIX_OK;
}

void free_list(std::vector<Buf>& list) {
  for (auto& b : list) cudaFree(b.p);
  list.clear();
}

#define AL(list, ptr, n)                                      \
  do {                                                        \
    int r_ = alloc(ctx, list, &(ptr), (size_t)(n));           \
    if (r_) return r_;                                        \
  } while (0)

int alloc_spdev(stspix_ctx* ctx, SpDev& s, int cap) {
  s.cap = cap;
  auto& L = ctx->sp_bufs;
  AL(L, s.count, cap); AL(L, s.valid, cap); AL(L, s.prop, cap);
  AL(L, s.prior_count, cap); AL(L, s.icount, cap); AL(L, s.sm_count, cap);
  AL(L, s.mu_app, 3 * (size_t)cap); AL(L, s.mu_shape, 2 * (size_t)cap);
  AL(L, s.sigma_shape, 3 * (size_t)cap); AL(L, s.logdet, cap);
  AL(L, s.prior_mu_app, 3 * (size_t)cap); AL(L, s.prior_mu_shape, 2 * (size_t)cap);
  AL(L, s.prior_sigma_shape, 3 * (size_t)cap); AL(L, s.prior_icov, 3 * (size_t)cap);
  AL(L, s.sample_sigma_shape, 3 * (size_t)cap); AL(L, s.acc, 8 * (size_t)cap);
  AL(L, s.rec, cap);
  return STSPIX_OK;
}

int alloc_params(stspix_ctx* ctx, stspix_params& p, int cap) {
  auto& L = ctx->pp_bufs;
  p.capacity = cap;
  AL(L, p.mu_app, 3 * (size_t)cap); AL(L, p.prior_mu_app, 3 * (size_t)cap);
  AL(L, p.mu_shape, 2 * (size_t)cap); AL(L, p.sigma_shape, 3 * (size_t)cap);
  AL(L, p.logdet_sigma_shape, cap); AL(L, p.prior_mu_shape, 2 * (size_t)cap);
  AL(L, p.prior_sigma_shape, 3 * (size_t)cap); AL(L, p.sample_sigma_shape, 3 * (size_t)cap);
  AL(L, p.counts, cap); AL(L, p.sm_counts, cap); AL(L, p.prior_counts, cap);
  AL(L, p.ids, cap); AL(L, p.invalid_counts, cap);
  return STSPIX_OK;
}

// Make sure pixel buffers hold npix and superpixel buffers hold sp_cap entries.
// Growing synchronises the device and does not preserve contents (callers grow
// only between frames); the bist_forward parameter buffers live in pp_bufs and are
// grown by ensure_pp, which keeps the previous frame's parameters.
int ensure(stspix_ctx* ctx, int npix, int sp_cap) {
  if (npix > ctx->npix_cap) {
    CK(cudaDeviceSynchronize());
    free_list(ctx->pix_bufs);
    auto& L = ctx->pix_bufs;
    int n = npix;
    AL(L, ctx->border, n); AL(L, ctx->d1, n); AL(L, ctx->d2, n); AL(L, ctx->smseg, n);
    AL(L, ctx->hits, n); AL(L, ctx->shifted, n); AL(L, ctx->filled, n); AL(L, ctx->best, n);
    AL(L, ctx->seg_alt, n);
    ctx->npix_cap = npix;
  }
  if (sp_cap > ctx->sp_cap) {
    CK(cudaDeviceSynchronize());
    free_list(ctx->sp_bufs);
    int cap = sp_cap;
    int r;
    if ((r = alloc_spdev(ctx, ctx->sp, cap))) return r;
    if ((r = alloc_spdev(ctx, ctx->tmp, cap))) return r;
    auto& L = ctx->sp_bufs;
    size_t c2 = (size_t)cap + 2;
    AL(L, ctx->sm.count, c2); AL(L, ctx->sm.s, 3 * c2); AL(L, ctx->sm.sq, 3 * c2);
    AL(L, ctx->sm.ninvalid, c2); AL(L, ctx->sm.pair, c2); AL(L, ctx->sm.claim, c2);
    AL(L, ctx->sm.target, c2); AL(L, ctx->sm.newid, c2); AL(L, ctx->sm.flag, c2);
    AL(L, ctx->sm.msingle, c2);
    AL(L, ctx->flags, c2); AL(L, ctx->accept, c2); AL(L, ctx->valid0, c2);
    AL(L, ctx->living, c2); AL(L, ctx->mint, c2);
    AL(L, ctx->excl, c2); AL(L, ctx->rid, c2); AL(L, ctx->src_of, c2);
    AL(L, ctx->cnt_pool, c2); AL(L, ctx->cs, c2); AL(L, ctx->cf, c2);
    AL(L, ctx->fs, 2 * c2); AL(L, ctx->fds, 2 * c2); AL(L, ctx->ss, c2);
    AL(L, ctx->centers, 2 * c2); AL(L, ctx->rbest, c2); AL(L, ctx->ccbest, c2);
    ctx->sp_cap = cap;
  }
  return STSPIX_OK;
}

void hex_geometry(int sp_size, int W, int H, double* hh, double* ww, int* nx, int* ny) {
  double Hh = sqrt(double(pow(sp_size, 2)) / (1.5 * sqrt(3.0)));
  double w = sqrt(3.0) * Hh;
  *hh = Hh; *ww = w;
  *nx = (int)floor(double(W) / w) + 2;
  *ny = (int)floor(double(H) / (1.5 * Hh)) + 2;
}

SmConsts sm_constants(const stspix_config& c) {
  float i_std = (float)(sqrt(c.sigma2_app) * 2);
  float a0 = 1e4f;
  float b0 = i_std * a0;
  float alpha = (float)exp((double)c.alpha_hastings);
  SmConsts K;
  K.b0 = (double)b0;
  K.log_alpha = log((double)alpha);
  K.log_01_b0 = log(0.1) - log((double)b0);
  K.lc = 0.5 * log(M_PI) + log(2.0);
  return K;
}

// Parameter ping-pong buffers of bist_forward: grown to `cap` entries keeping the
// first `keep` entries of buffer `keep_idx`.
int ensure_pp(stspix_ctx* ctx, cudaStream_t st, int cap, int keep_idx, int keep) {
  if (cap <= ctx->pp_cap) return STSPIX_OK;
  std::vector<Buf> old = ctx->pp_bufs;
  stspix_params oldp = ctx->pp[keep_idx];
  ctx->pp_bufs.clear();
  int r;
  for (int i = 0; i < 2; i++)
    if ((r = alloc_params(ctx, ctx->pp[i], cap))) return r;
  if (keep > 0) {
    stspix_params& np = ctx->pp[keep_idx];
    size_t k = (size_t)keep;
    CK(cudaMemcpyAsync(np.mu_app, oldp.mu_app, 12 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.prior_mu_app, oldp.prior_mu_app, 12 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.mu_shape, oldp.mu_shape, 16 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.sigma_shape, oldp.sigma_shape, 24 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.logdet_sigma_shape, oldp.logdet_sigma_shape, 4 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.prior_mu_shape, oldp.prior_mu_shape, 16 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.prior_sigma_shape, oldp.prior_sigma_shape, 24 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.sample_sigma_shape, oldp.sample_sigma_shape, 24 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.counts, oldp.counts, 4 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.sm_counts, oldp.sm_counts, 4 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.prior_counts, oldp.prior_counts, 4 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.ids, oldp.ids, 4 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(np.invalid_counts, oldp.invalid_counts, 4 * k, cudaMemcpyDeviceToDevice, st));
    CK(cudaStreamSynchronize(st));
  }
  free_list(old);
  ctx->pp_cap = cap;
  return STSPIX_OK;
}

int coop_launch(stspix_ctx* ctx, cudaStream_t st, const void* fn, int want_blocks, int max_blocks,
                void** args) {
  int g = std::max(1, std::min(want_blocks, max_blocks));
  cudaEvent_t pe = prof_begin(ctx, st);
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(g), dim3(kThreads), args, 0, st);
  ctx->launches++;
  prof_end(ctx, st, pe);
  if (e != cudaSuccess)
    return fail(ctx, STSPIX_ERR_CUDA, "cooperative launch failed: %s", cudaGetErrorString(e));
  return STSPIX_OK;
}

// ---------------------------------------------------------------------------
// Stages.
struct Frame {
  const float* img;
  int* seg;  // working labels (caller's output buffer)
  int H, W, npix;
  stspix_config cfg;
  SmConsts K;
  const int* shifted;  // prop frames: shifted labels (for invalid counts)
  int prop_mode;
  int n_prev;
  const float* prev_prior_mu_app;
};

int update_params(stspix_ctx* ctx, cudaStream_t st, const Frame& f) {
  SpDev& sp = ctx->sp;
  CK(cudaMemsetAsync(sp.count, 0, sizeof(int) * (size_t)sp.cap, st));
  CK(cudaMemsetAsync(sp.acc, 0, sizeof(long long) * 8 * (size_t)sp.cap, st));
  ctx->cur_fam = STSPIX_FAM_STATS;
  {
    long long nthr = (long long)f.H * ((f.W + 7) / 8);  // one 8-pixel run per thread
    LAUNCHG(k_accumulate, (unsigned)((nthr + 127) / 128), 128, f.img, f.seg, f.H, f.W, sp);
  }
  ctx->cur_fam = STSPIX_FAM_POSTERIOR;
  LAUNCH(k_posterior, sp.cap, sp, f.cfg.sp_size, ctx->sc);
  return STSPIX_OK;
}

// update_seg (update_seg.cu:281-311): niters_seg fused sweeps ping-ponging between
// the frame's labels and a scratch buffer; the trailing border mask is only built
// when the next iteration's merge reads it.
int update_seg(stspix_ctx* ctx, cudaStream_t st, const Frame& f, bool need_border) {
  const int H = f.H, W = f.W;
  ctx->cur_fam = STSPIX_FAM_SWEEP;
  int* a = f.seg;
  int* b = ctx->seg_alt;
  dim3 grid((W + 31) / 32, (H + 31) / 32);
  for (int it = 0; it < f.cfg.niters_seg; it++) {
    LAUNCHG(k_sweep_fused, grid, 256, f.img, a, b, ctx->sp.rec, ctx->sp.cap, H, W,
            f.cfg.sigma2_app, f.cfg.potts);
    std::swap(a, b);
  }
  if (a != f.seg)
    CK(cudaMemcpyAsync(f.seg, a, sizeof(int) * (size_t)f.npix, cudaMemcpyDeviceToDevice, st));
  if (need_border) {
    ctx->cur_fam = STSPIX_FAM_MERGE;
    LAUNCH(k_find_border, f.npix, f.seg, ctx->border, H, W);
  }
  return STSPIX_OK;
}

int run_relax(stspix_ctx* ctx, cudaStream_t st, int mode, const int* seg, int* f1, int* f2,
              int H, int W) {
  CK(cudaMemsetAsync(ctx->round_flags, 0, sizeof(int) * 4096, st));
  int ntiles = ((W + 31) / 32) * ((H + 31) / 32);
  int max_rounds = 4096;
  void* args[] = {(void*)&seg, (void*)&f1, (void*)&f2, (void*)&H, (void*)&W, (void*)&ctx->sc,
                  (void*)&ctx->round_flags, (void*)&max_rounds};
  if (mode == 0)
    return coop_launch(ctx, st, (const void*)k_relax_bfs, ntiles, ctx->coop_relax0, args);
  return coop_launch(ctx, st, (const void*)k_relax_cc, ntiles, ctx->coop_relax1, args);
}

int run_split(stspix_ctx* ctx, cudaStream_t st, const Frame& f, int direction) {
  SpDev& sp = ctx->sp;
  SmDev& sm = ctx->sm;
  const int cap = sp.cap;
  const size_t c2 = (size_t)cap + 2;
  ctx->cur_fam = STSPIX_FAM_SPLIT;
  LAUNCH1(k_split_begin, ctx->sc);
  CK(cudaMemsetAsync(ctx->d1, 0xff, sizeof(int) * (size_t)f.npix, st));
  CK(cudaMemsetAsync(ctx->d2, 0xff, sizeof(int) * (size_t)f.npix, st));
  LAUNCH(k_split_seed, cap, sp, f.seg, f.H, f.W, direction, ctx->sc, ctx->d1, ctx->d2);
  int r = run_relax(ctx, st, 0, f.seg, ctx->d1, ctx->d2, f.H, f.W);
  if (r) return r;
  LAUNCH(k_split_partition, f.npix, f.seg, ctx->d1, ctx->d2, f.npix, ctx->sc, ctx->smseg);
  CK(cudaMemsetAsync(sm.count, 0, sizeof(int) * c2, st));
  CK(cudaMemsetAsync(sm.ninvalid, 0, sizeof(int) * c2, st));
  CK(cudaMemsetAsync(sm.s, 0, sizeof(long long) * 3 * c2, st));
  CK(cudaMemsetAsync(sm.sq, 0, sizeof(long long) * 3 * c2, st));
  LAUNCH(k_sm_accumulate, (long long)f.H * ((f.W + 15) / 16), f.img, ctx->smseg,
         f.prop_mode ? f.shifted : nullptr, f.H, f.W, cap + 2, sm);
  LAUNCH(k_split_decide, cap, sp, sm, ctx->sc, f.K, f.cfg.split_alpha, f.prop_mode,
         ctx->accept);
  LAUNCHG(k_scan_flags, 1, 1024, ctx->accept, nullptr, cap, ctx->excl, &ctx->sc->tmp2);
  LAUNCH(k_split_commit, cap, sp, sm, ctx->sc, ctx->accept, ctx->excl, f.prop_mode);
  LAUNCH(k_split_apply, f.npix, f.seg, ctx->smseg, f.npix, sp, sm, ctx->sc, ctx->accept,
         f.prop_mode);
  LAUNCH1(k_split_end, ctx->sc, &ctx->sc->tmp2);
  return STSPIX_OK;
}

int run_relabel(stspix_ctx* ctx, cudaStream_t st, const Frame& f) {
  SpDev& sp = ctx->sp;
  const int cap = sp.cap;
  ctx->cur_fam = STSPIX_FAM_MERGE;
  CK(cudaMemsetAsync(ctx->living, 0, (size_t)cap + 2, st));
  LAUNCH(k_living, f.npix, f.seg, f.npix, ctx->sc, ctx->living);
  LAUNCH(k_relabel_init, cap, cap, ctx->rbest, ctx->ss);
  const int chunk = 256;
  dim3 g(blocks_for(cap), (unsigned)std::max(1, (f.n_prev + chunk - 1) / chunk));
  LAUNCHG(k_relabel_compare, g, kThreads, sp, f.prev_prior_mu_app, f.n_prev, ctx->sc,
          ctx->living, ctx->rbest, ctx->ss, chunk);
  LAUNCH(k_relabel_mark, cap, cap, ctx->sc, ctx->living, ctx->rbest, ctx->ss,
         f.cfg.thresh_relabel, f.cfg.thresh_new, ctx->rid, ctx->mint);
  LAUNCHG(k_scan_flags, 1, 1024, ctx->mint, nullptr, cap, ctx->excl, &ctx->sc->tmp2);
  CK(cudaMemsetAsync(ctx->src_of, 0xff, sizeof(int) * ((size_t)cap + 2), st));
  LAUNCH(k_relabel_ids, cap, cap, ctx->sc, ctx->mint, ctx->excl, ctx->rid, ctx->src_of);
  LAUNCH(k_relabel_params, cap, sp, ctx->rid, ctx->src_of, f.n_prev);
  LAUNCH(k_relabel_apply, f.npix, f.seg, f.npix, cap, ctx->rid);
  LAUNCH(k_count_revived, cap, ctx->rid, ctx->mint, cap, ctx->sc);
  LAUNCH1(k_relabel_end, ctx->sc, &ctx->sc->tmp2, ctx->rid, cap);
  return STSPIX_OK;
}

int run_merge(stspix_ctx* ctx, cudaStream_t st, const Frame& f, int direction) {
  SpDev& sp = ctx->sp;
  SmDev& sm = ctx->sm;
  const int cap = sp.cap;
  const size_t c2 = (size_t)cap + 2;
  ctx->cur_fam = STSPIX_FAM_MERGE;
  CK(cudaMemsetAsync(sm.pair, 0xff, sizeof(int) * c2, st));
  CK(cudaMemsetAsync(sm.claim, 0x7f, sizeof(int) * c2, st));
  LAUNCH(k_merge_candidates, f.npix, f.seg, ctx->border, f.H, f.W, direction, f.prop_mode,
         sp.prop, cap, sm.pair);
  CK(cudaMemsetAsync(sm.count, 0, sizeof(int) * c2, st));
  CK(cudaMemsetAsync(sm.s, 0, sizeof(long long) * 3 * c2, st));
  CK(cudaMemsetAsync(sm.sq, 0, sizeof(long long) * 3 * c2, st));
  LAUNCH(k_sm_accumulate, (long long)f.H * ((f.W + 15) / 16), f.img, f.seg, nullptr, f.H, f.W,
         cap, sm);
  LAUNCH(k_merge_single, cap, sp, sm, f.K);
  LAUNCH(k_merge_decide, cap, sp, sm, ctx->sc, f.K, f.cfg.merge_alpha);
  LAUNCH(k_merge_flag, cap, sp, sm, ctx->valid0);
  LAUNCH(k_merge_remove, cap, sp, sm, ctx->sc, ctx->valid0, f.prop_mode);
  LAUNCH(k_merge_apply, f.npix, f.seg, f.npix, cap, sm);
  return STSPIX_OK;
}

// bass (bass.cu:46-181) / prop_bass_v3 (prop.cu:326-468) outer loop.
int bass_loop(stspix_ctx* ctx, cudaStream_t st, const Frame& f, int niters, int stop_after,
              int extra_update) {
  int r;
  int count = 1;
  const int P = f.cfg.sm_period > 0 ? f.cfg.sm_period : 4;
  for (int idx = 0; idx < niters; idx++) {
    if (stop_after >= 0 && idx == stop_after) {
      if (extra_update && (r = update_params(ctx, st, f))) return r;
      return STSPIX_OK;
    }
    if ((r = update_params(ctx, st, f))) return r;
    if (idx > f.cfg.sm_start) {
      if (idx % P == 0) {
        count += 1;
        int direction = count % 2 + 1;
        if ((r = run_split(ctx, st, f, direction))) return r;
        if ((r = update_params(ctx, st, f))) return r;
      }
      if (idx % P == P / 2) {
        int direction;
        if (f.prop_mode) {
          count += 1;
          direction = count % 2;
          if ((r = run_relabel(ctx, st, f))) return r;
        } else {
          direction = count % 2;
        }
        if ((r = run_merge(ctx, st, f, direction))) return r;
        if ((r = update_params(ctx, st, f))) return r;
      }
    }
    const int nx = idx + 1;
    const bool merge_next = nx < niters && nx > f.cfg.sm_start && nx % P == P / 2;
    if ((r = update_seg(ctx, st, f, merge_next || stop_after >= 0))) return r;
  }
  if (stop_after >= 0) {
    if (extra_update && (r = update_params(ctx, st, f))) return r;
    return STSPIX_OK;
  }
  if ((r = update_params(ctx, st, f))) return r;
  ctx->cur_fam = STSPIX_FAM_POSTERIOR;
  LAUNCH(k_store_sample, ctx->sp.cap, ctx->sp);
  return STSPIX_OK;
}

// compactify_new_superpixels (compact_spix.cu:41-89) for ids >= lo, moving params.
int compact(stspix_ctx* ctx, cudaStream_t st, const Frame& f, int lo) {
  const int cap = ctx->sp.cap;
  ctx->cur_fam = STSPIX_FAM_OTHER;
  CK(cudaMemsetAsync(ctx->flags, 0, (size_t)cap + 2, st));
  LAUNCH1(k_calc_n, ctx->sc, lo, cap);
  LAUNCH(k_mark_present, f.npix, f.seg, f.npix, lo, &ctx->sc->max_spix, 0, ctx->flags);
  LAUNCHG(k_scan_flags, 1, 1024, ctx->flags, &ctx->sc->tmp2, 0, ctx->excl, &ctx->sc->tmp1);
  LAUNCH(k_compact_gather, cap, ctx->sp, ctx->tmp, lo, &ctx->sc->max_spix, ctx->flags, ctx->excl);
  LAUNCH(k_compact_scatter, cap, ctx->sp, ctx->tmp, lo, &ctx->sc->tmp1);
  LAUNCH(k_remap, f.npix, f.seg, f.npix, lo, ctx->excl);
  LAUNCH1(k_finish_compact, ctx->sc, lo, &ctx->sc->tmp1);
  return STSPIX_OK;
}

// run_bass (bass.cu:221-345) on device buffers; params_out may be null.
int bass_frame(stspix_ctx* ctx, cudaStream_t st, const float* img, int H, int W,
               const stspix_config& cfg, int* seg, const stspix_params* params_out,
               int stop_after, int extra_update) {
  const int npix = H * W;
  double Hh, w;
  int nx, ny;
  hex_geometry(cfg.sp_size, W, H, &Hh, &w, &nx, &ny);
  const int nraw = nx * ny;
  const int nbuf = 30 * nraw;
  int r;
  if ((r = ensure(ctx, npix, std::max(nbuf, 64)))) return r;
  Frame f{img, seg, H, W, npix, cfg, sm_constants(cfg), nullptr, 0, 0, nullptr};
  ctx->cur_fam = STSPIX_FAM_OTHER;
  LAUNCH1(k_frame_begin, ctx->sc, 0, nbuf);
  LAUNCH(k_init_hex, npix, seg, H, W, Hh, w, nx, ny);
  // compact the hex ids (extract_unique_ids + compactify, bass.cu:251-252)
  CK(cudaMemsetAsync(ctx->flags, 0, (size_t)ctx->sp.cap + 2, st));
  LAUNCH(k_mark_present, npix, seg, npix, 0, nullptr, nraw - 1, ctx->flags);
  LAUNCHG(k_scan_flags, 1, 1024, ctx->flags, nullptr, nraw, ctx->excl, &ctx->sc->nspix);
  LAUNCH(k_remap, npix, seg, npix, 0, ctx->excl);
  LAUNCH1(k_bass_after_compact, ctx->sc);
  LAUNCH(k_init_bass_params, ctx->sp.cap, ctx->sp, &ctx->sc->nspix, npix, cfg.sp_size);
  CK(cudaMemsetAsync(ctx->sp.count, 0, sizeof(int) * (size_t)ctx->sp.cap, st));
  CK(cudaMemsetAsync(ctx->sp.acc, 0, sizeof(long long) * 8 * (size_t)ctx->sp.cap, st));
  LAUNCHG(k_accumulate, (unsigned)(((long long)H * ((W + 7) / 8) + 127) / 128), 128, img, seg, H,
          W, ctx->sp);
  LAUNCH(k_init_prior_mu, ctx->sp.cap, ctx->sp, &ctx->sc->nspix);
  LAUNCH(k_find_border, npix, seg, ctx->border, H, W);
  if ((r = bass_loop(ctx, st, f, cfg.niters, stop_after, extra_update))) return r;
  if (stop_after >= 0) return STSPIX_OK;
  if ((r = compact(ctx, st, f, 0))) return r;
  if (params_out) LAUNCH(k_read_params, ctx->sp.cap, ctx->sp, &ctx->sc->nspix, *params_out);
  return STSPIX_OK;
}

// shift_and_fill (shift_and_fill.cu:108-339).
int shift_fill(stspix_ctx* ctx, cudaStream_t st, const int* prev, const stspix_params& pp,
               int n_prev, const float* flow, int H, int W, int* filled, int* shifted) {
  const int npix = H * W;
  int r;
  if ((r = ensure(ctx, npix, std::max(10 * n_prev + 2, 64)))) return r;
  ctx->cur_fam = STSPIX_FAM_PROP;
  CK(cudaMemsetAsync(ctx->cnt_pool, 0, sizeof(int) * (size_t)n_prev, st));
  CK(cudaMemsetAsync(ctx->fs, 0, sizeof(long long) * 2 * (size_t)n_prev, st));
  LAUNCH(k_flow_pool, (long long)H * ((W + 15) / 16), prev, flow, H, W, n_prev, ctx->cnt_pool,
         ctx->fs);
  LAUNCH(k_flow_mean, n_prev, n_prev, ctx->cnt_pool, ctx->fs, pp.mu_shape, ctx->fds,
         ctx->centers);
  CK(cudaMemsetAsync(ctx->hits, 0, sizeof(int) * (size_t)npix, st));
  CK(cudaMemsetAsync(ctx->best, 0xff, sizeof(unsigned long long) * (size_t)npix, st));
  LAUNCH(k_shift, npix, prev, H, W, n_prev, ctx->cnt_pool, ctx->fds, ctx->hits, ctx->best);
  CK(cudaMemsetAsync(&ctx->sc->ninvalid, 0, sizeof(int), st));
  LAUNCH(k_shift_decode, npix, ctx->hits, ctx->best, npix, shifted, filled, ctx->sc);
  CK(cudaMemsetAsync(ctx->cs, 0, sizeof(int) * (size_t)n_prev, st));
  LAUNCH(k_count_labels, npix, filled, npix, n_prev, ctx->cs);
  // fill, invalidate disconnected, fill
  for (int pass = 0; pass < 2; pass++) {
    CK(cudaMemsetAsync(ctx->iter_counts, 0, sizeof(int) * (kFillBreakIter + 2), st));
    int break_iter = kFillBreakIter;
    void* args[] = {(void*)&filled, (void*)&ctx->centers, (void*)&H, (void*)&W,
                    (void*)&ctx->border, (void*)&ctx->sc, (void*)&ctx->iter_counts,
                    (void*)&break_iter};
    if ((r = coop_launch(ctx, st, (const void*)k_fill_coop, (int)blocks_for(npix),
                         ctx->coop_fill, args)))
      return r;
    if (pass == 0) {
      LAUNCH(k_cc_init, npix, filled, npix, ctx->d1);
      if ((r = run_relax(ctx, st, 1, filled, ctx->d1, nullptr, H, W))) return r;
      CK(cudaMemsetAsync(ctx->d2, 0, sizeof(int) * (size_t)npix, st));
      LAUNCH(k_cc_size, npix, ctx->d1, npix, ctx->d2);
      CK(cudaMemsetAsync(ctx->ccbest, 0, sizeof(unsigned long long) * (size_t)n_prev, st));
      LAUNCH(k_cc_best, npix, filled, ctx->d1, ctx->d2, npix, n_prev, ctx->ccbest);
      LAUNCH(k_cc_invalidate, npix, filled, ctx->d1, npix, n_prev, ctx->ccbest);
    }
  }
  CK(cudaMemsetAsync(ctx->cf, 0, sizeof(int) * (size_t)n_prev, st));
  LAUNCH(k_count_labels, npix, filled, npix, n_prev, ctx->cf);
  LAUNCH(k_shift_params, n_prev, n_prev, ctx->cnt_pool, ctx->cs, ctx->cf, pp);
  return STSPIX_OK;
}

// run_prop (prop.cu:677-865); seg already holds the filled labels.
int prop_frame(stspix_ctx* ctx, cudaStream_t st, const float* img, int H, int W,
               const stspix_config& cfg, int niters, int* seg, const int* shifted,
               const stspix_params& prev, int n_prev, const stspix_params* params_out) {
  const int npix = H * W;
  int r;
  if ((r = ensure(ctx, npix, std::max(10 * n_prev + 2, 64)))) return r;
  Frame f{img, seg, H, W, npix, cfg, sm_constants(cfg), shifted, 1, n_prev, prev.prior_mu_app};
  ctx->cur_fam = STSPIX_FAM_OTHER;
  LAUNCH1(k_frame_begin, ctx->sc, n_prev - 1, 10 * n_prev);
  LAUNCH(k_write_params, ctx->sp.cap, ctx->sp, prev, n_prev, cfg.sp_size);
  LAUNCH(k_mark_active, npix, seg, npix, ctx->sp);
  LAUNCH1(k_prop_begin, ctx->sc, n_prev);
  if ((r = bass_loop(ctx, st, f, niters, -1, 0))) return r;
  if ((r = compact(ctx, st, f, n_prev))) return r;
  if (params_out) LAUNCH(k_read_params, ctx->sp.cap, ctx->sp, &ctx->sc->nspix, *params_out);
  return STSPIX_OK;
}

int sync_scalars(stspix_ctx* ctx, cudaStream_t st) {
  CK(cudaMemcpyAsync(ctx->sc_host, ctx->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  prof_harvest(ctx);
  const Scalars& s = *ctx->sc_host;
  ctx->log.nsplits = s.nsplits;
  ctx->log.nmerges = s.nmerges;
  ctx->log.nrevived = s.nrevived;
  ctx->log.nminted = s.nminted;
  ctx->log.near_ties = s.near_ties;
  ctx->log.fill_iters = s.fill_iters;
  ctx->log.nspix = s.nspix;
  return STSPIX_OK;
}

int check_cfg(stspix_ctx* ctx, const stspix_config* cfg) {
  if (!cfg) return fail(ctx, STSPIX_ERR_ARG, "config is NULL");
  if (cfg->sp_size < 1) return fail(ctx, STSPIX_ERR_ARG, "sp_size must be >= 1");
  if (cfg->niters < 0 || cfg->niters_seg < 0)
    return fail(ctx, STSPIX_ERR_ARG, "iteration counts must be >= 0");
  if (!(cfg->sigma2_app > 0)) return fail(ctx, STSPIX_ERR_ARG, "sigma2_app must be > 0");
  return STSPIX_OK;
}

int check_size(stspix_ctx* ctx, int H, int W) {
  if (H < 2 || W < 2) return fail(ctx, STSPIX_ERR_ARG, "frame must be at least 2x2 (got %dx%d)", H, W);
  if ((long long)H * W > (1LL << 26))
    return fail(ctx, STSPIX_ERR_ARG, "frame of %lld pixels exceeds the 2^26 limit of the fixed-point sums",
                (long long)H * W);
  return STSPIX_OK;
}

}  // namespace

// =========================================================================
extern "C" {

void stspix_default_config(stspix_config* c) {
  if (!c) return;
  c->niters = 15; c->niters_seg = 4; c->sp_size = 15; c->sm_start = 0; c->sm_period = 4;
  c->prop_niters = 0;
  c->sigma2_app = 0.009f * 0.009f; c->potts = 0.5f; c->alpha_hastings = (float)log(0.5);
  c->split_alpha = 0.f; c->merge_alpha = 0.f; c->sigma2_size = 0.f;
  c->thresh_relabel = 1e-5f; c->thresh_new = 1e-2f;
}

int stspix_version(void) { return 1; }

int stspix_create(stspix_ctx** out, int device) {
  if (!out) return STSPIX_ERR_ARG;
  *out = nullptr;
  stspix_ctx* ctx = new (std::nothrow) stspix_ctx();
  if (!ctx) return STSPIX_ERR_NOMEM;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete ctx; return STSPIX_ERR_CUDA; }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k_relax_bfs, kThreads, 0);
  // Cooperative grids use at most one block per SM: with up to
  // (resident blocks per SM) streams launching cooperative kernels at once, all of
  // their blocks can still be resident together (other kernels always drain).
  ctx->coop_relax0 = std::min(nb, 1) * ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k_relax_cc, kThreads, 0);
  ctx->coop_relax1 = std::min(nb, 1) * ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (const void*)k_fill_coop, kThreads, 0);
  ctx->coop_fill = std::min(nb, 1) * ctx->num_sms;
  if (!coop || ctx->coop_relax0 <= 0 || ctx->coop_fill <= 0) {
    delete ctx;
    return STSPIX_ERR_CUDA;
  }
  std::vector<Buf> ctl;
  if (cudaMalloc(&ctx->round_flags, sizeof(int) * 4096) != cudaSuccess ||
      cudaMalloc(&ctx->iter_counts, sizeof(int) * (kFillBreakIter + 2)) != cudaSuccess ||
      cudaMalloc(&ctx->sc, sizeof(Scalars)) != cudaSuccess ||
      cudaMallocHost(&ctx->sc_host, sizeof(Scalars)) != cudaSuccess) {
    delete ctx;
    return STSPIX_ERR_NOMEM;
  }
  cudaMemset(ctx->sc, 0, sizeof(Scalars));
  cudaDeviceSynchronize();
  *out = ctx;
  return STSPIX_OK;
}

int stspix_destroy(stspix_ctx* ctx) {
  if (!ctx) return STSPIX_OK;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  free_list(ctx->pix_bufs);
  free_list(ctx->sp_bufs);
  free_list(ctx->pp_bufs);
  prof_harvest(ctx);
  for (auto& e : ctx->frame_ev) { ctx->ev_free.push_back(e.first); ctx->ev_free.push_back(e.second); }
  for (auto e : ctx->ev_free) cudaEventDestroy(e);
  cudaFree(ctx->round_flags);
  cudaFree(ctx->iter_counts);
  cudaFree(ctx->sc);
  cudaFreeHost(ctx->sc_host);
  delete ctx;
  return STSPIX_OK;
}

const char* stspix_last_error(const stspix_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

long long stspix_kernel_launches(const stspix_ctx* ctx) { return ctx ? ctx->launches : 0; }

int stspix_get_frame_log(const stspix_ctx* ctx, stspix_frame_log* out) {
  if (!ctx || !out) return STSPIX_ERR_ARG;
  *out = ctx->log;
  return STSPIX_OK;
}

int stspix_init_seg(stspix_ctx* ctx, void* stream, int32_t* labels, int H, int W, int sp_size,
                    int* nspix_out) {
  if (!ctx || !labels || sp_size < 1) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r = check_size(ctx, H, W);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  double Hh, w;
  int nx, ny;
  hex_geometry(sp_size, W, H, &Hh, &w, &nx, &ny);
  LAUNCH(k_init_hex, (long long)H * W, labels, H, W, Hh, w, nx, ny);
  CK(cudaGetLastError());
  if (nspix_out) *nspix_out = nx * ny;
  return STSPIX_OK;
}

int stspix_find_border(stspix_ctx* ctx, void* stream, const int32_t* labels, uint8_t* border,
                       int H, int W, int mode) {
  if (!ctx || !labels || !border) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r = check_size(ctx, H, W);
  if (r) return r;
  cudaStream_t st = (cudaStream_t)stream;
  if (mode == 0) LAUNCH(k_find_border, (long long)H * W, labels, border, H, W);
  else LAUNCH(k_find_border_end, (long long)H * W, labels, border, H, W, 1);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_run_bass(stspix_ctx* ctx, void* stream, const float* img, int H, int W,
                    const stspix_config* cfg, int32_t* labels_out, stspix_params* params_out,
                    int* nspix_out) {
  if (!ctx || !img || !labels_out) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r;
  if ((r = check_cfg(ctx, cfg)) || (r = check_size(ctx, H, W))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  if ((r = bass_frame(ctx, st, img, H, W, *cfg, labels_out, nullptr, -1, 0))) return r;
  if ((r = sync_scalars(ctx, st))) return r;
  int n = ctx->sc_host->nspix;
  if (params_out) {
    if (params_out->capacity < n)
      return fail(ctx, STSPIX_ERR_CAPACITY, "params capacity %d < %d superpixels",
                  params_out->capacity, n);
    LAUNCH(k_read_params, ctx->sp.cap, ctx->sp, &ctx->sc->nspix, *params_out);
    CK(cudaStreamSynchronize(st));
  }
  ctx->log.niters = cfg->niters;
  if (nspix_out) *nspix_out = n;
  return ctx->sc_host->status ? fail(ctx, ctx->sc_host->status, "device status %d", ctx->sc_host->status) : STSPIX_OK;
}

int stspix_bass_partial(stspix_ctx* ctx, void* stream, const float* img, int H, int W,
                        const stspix_config* cfg, int iters, int extra_update,
                        int32_t* labels_out, stspix_state_dump* dump, int* nbuf_out,
                        int* max_spix_out) {
  if (!ctx || !img || !labels_out) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r;
  if ((r = check_cfg(ctx, cfg)) || (r = check_size(ctx, H, W))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  if ((r = bass_frame(ctx, st, img, H, W, *cfg, labels_out, nullptr, iters < 0 ? 0 : iters,
                      extra_update)))
    return r;
  if (dump) LAUNCH(k_dump_state, ctx->sp.cap, ctx->sp, *dump);
  if ((r = sync_scalars(ctx, st))) return r;
  double Hh, w;
  int nx, ny;
  hex_geometry(cfg->sp_size, W, H, &Hh, &w, &nx, &ny);
  if (nbuf_out) *nbuf_out = 30 * nx * ny;
  if (max_spix_out) *max_spix_out = ctx->sc_host->max_spix;
  return ctx->sc_host->status;
}

int stspix_shift_and_fill(stspix_ctx* ctx, void* stream, const int32_t* labels_prev,
                          stspix_params* params_prev, int n_prev, const float* flow, int H, int W,
                          int32_t* filled_out, int32_t* shifted_out) {
  if (!ctx || !labels_prev || !params_prev || !flow || !filled_out || !shifted_out || n_prev < 1)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r;
  if ((r = check_size(ctx, H, W))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  LAUNCH1(k_frame_begin, ctx->sc, 0, 0);
  if ((r = shift_fill(ctx, st, labels_prev, *params_prev, n_prev, flow, H, W, filled_out,
                      shifted_out)))
    return r;
  if ((r = sync_scalars(ctx, st))) return r;
  return ctx->sc_host->status ? fail(ctx, ctx->sc_host->status, "device status %d", ctx->sc_host->status) : STSPIX_OK;
}

int stspix_run_prop(stspix_ctx* ctx, void* stream, const float* img, int H, int W,
                    const stspix_config* cfg, int niters, const int32_t* filled,
                    const int32_t* shifted, const stspix_params* params_prev, int n_prev,
                    int32_t* labels_out, stspix_params* params_out, int* nspix_out) {
  if (!ctx || !img || !filled || !shifted || !params_prev || !labels_out || n_prev < 1)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r;
  if ((r = check_cfg(ctx, cfg)) || (r = check_size(ctx, H, W))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  CK(cudaMemcpyAsync(labels_out, filled, sizeof(int) * (size_t)H * W, cudaMemcpyDeviceToDevice, st));
  if ((r = prop_frame(ctx, st, img, H, W, *cfg, niters, labels_out, shifted, *params_prev,
                      n_prev, nullptr)))
    return r;
  if ((r = sync_scalars(ctx, st))) return r;
  int n = ctx->sc_host->nspix;
  if (params_out) {
    if (params_out->capacity < n)
      return fail(ctx, STSPIX_ERR_CAPACITY, "params capacity %d < %d superpixels",
                  params_out->capacity, n);
    LAUNCH(k_read_params, ctx->sp.cap, ctx->sp, &ctx->sc->nspix, *params_out);
    CK(cudaStreamSynchronize(st));
  }
  ctx->log.niters = niters;
  if (nspix_out) *nspix_out = n;
  return ctx->sc_host->status ? fail(ctx, ctx->sc_host->status, "device status %d", ctx->sc_host->status) : STSPIX_OK;
}

// main_loop (pyapi.cu:46-195).
int stspix_bist_forward(stspix_ctx* ctx, void* stream, const float* vid, const float* flows,
                        int T, int H, int W, int nftrs, const stspix_config* cfg, int video_mode,
                        int rgb2lab, int32_t* spix_out) {
  (void)rgb2lab;
  if (!ctx || !vid || !spix_out || T < 0) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  if (nftrs != 3) return fail(ctx, STSPIX_ERR_ARG, "nftrs must be 3 (got %d)", nftrs);
  if (video_mode && T > 1 && !flows) return fail(ctx, STSPIX_ERR_ARG, "flows required in video mode");
  int r;
  if ((r = check_cfg(ctx, cfg)) || (r = check_size(ctx, H, W))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t npix = (size_t)H * W;
  int cur = 0;    // ping-pong index of the current frame's params
  int n_prev = 0;
  int status = STSPIX_OK;
  for (auto& e : ctx->frame_ev) { ctx->ev_free.push_back(e.first); ctx->ev_free.push_back(e.second); }
  ctx->frame_ev.clear();
  ctx->frame_ms.clear();
  for (int fi = 0; fi < T; fi++) {
    const float* img = vid + (size_t)fi * npix * 3;
    int* seg = spix_out + (size_t)fi * npix;
    cudaEvent_t fe0 = ev_get(ctx), fe1 = ev_get(ctx);
    cudaEventRecord(fe0, st);
    if (fi == 0 || !video_mode) {
      // params are only needed by the next frame in video mode
      if ((r = bass_frame(ctx, st, img, H, W, *cfg, seg, nullptr, -1, 0))) return r;
      if (video_mode) {
        if ((r = ensure_pp(ctx, st, ctx->sp_cap, cur, 0))) return r;
        LAUNCH(k_read_params, ctx->sp.cap, ctx->sp, &ctx->sc->nspix, ctx->pp[cur]);
        if ((r = sync_scalars(ctx, st))) return r;
        n_prev = ctx->sc_host->nspix;
        if (ctx->sc_host->status) status = ctx->sc_host->status;
      }
      ctx->log.niters = cfg->niters;
    } else {
      const float* flow = flows + (size_t)(fi - 1) * npix * 2;
      const int* prev = spix_out + (size_t)(fi - 1) * npix;
      stspix_params pprev = ctx->pp[cur];
      LAUNCH1(k_frame_begin, ctx->sc, 0, 0);
      if ((r = shift_fill(ctx, st, prev, pprev, n_prev, flow, H, W, seg, ctx->shifted))) return r;
      if ((r = sync_scalars(ctx, st))) return r;
      if (ctx->sc_host->status) status = ctx->sc_host->status;
      int niters;
      if (cfg->prop_niters > 0) {
        niters = cfg->prop_niters;
      } else {
        float iperc = ctx->sc_host->ninvalid / (1.0 * npix);
        niters = iperc > 0.20 ? 12 : (iperc < 0.01 ? 4 : 8);
      }
      int nxt = 1 - cur;
      if ((r = ensure(ctx, (int)npix, 10 * n_prev + 2))) return r;
      if ((r = ensure_pp(ctx, st, ctx->sp_cap, cur, n_prev))) return r;
      pprev = ctx->pp[cur];
      if ((r = prop_frame(ctx, st, img, H, W, *cfg, niters, seg, ctx->shifted, pprev, n_prev,
                          &ctx->pp[nxt])))
        return r;
      if ((r = sync_scalars(ctx, st))) return r;
      if (ctx->sc_host->status) status = ctx->sc_host->status;
      n_prev = ctx->sc_host->nspix;
      cur = nxt;
      ctx->log.niters = niters;
    }
    cudaEventRecord(fe1, st);
    ctx->frame_ev.push_back({fe0, fe1});
  }
  if (!video_mode) {
    if ((r = sync_scalars(ctx, st))) return r;
    if (ctx->sc_host->status) status = ctx->sc_host->status;
  }
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  prof_harvest(ctx);
  for (auto& e : ctx->frame_ev) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.first, e.second);
    ctx->frame_ms.push_back(ms);
  }
  return status ? fail(ctx, status, "device status %d", status) : STSPIX_OK;
}

int stspix_profile_enable(stspix_ctx* ctx, int enable) {
  if (!ctx) return STSPIX_ERR_ARG;
  ctx->prof_on = enable ? 1 : 0;
  for (int i = 0; i < STSPIX_NFAM; i++) { ctx->fam_launches[i] = 0; ctx->fam_ms[i] = 0; }
  return STSPIX_OK;
}

int stspix_profile_get(const stspix_ctx* ctx, int family, long long* launches, double* total_ms) {
  if (!ctx || family < 0 || family >= STSPIX_NFAM) return STSPIX_ERR_ARG;
  if (launches) *launches = ctx->fam_launches[family];
  if (total_ms) *total_ms = ctx->fam_ms[family];
  return STSPIX_OK;
}

int stspix_frame_times(const stspix_ctx* ctx, double* ms_out, int capacity) {
  if (!ctx) return -1;
  int n = (int)ctx->frame_ms.size();
  for (int i = 0; i < n && i < capacity && ms_out; i++) ms_out[i] = ctx->frame_ms[i];
  return n;
}

int stspix_get_marked_video(stspix_ctx* ctx, void* stream, const float* vid, const int32_t* spix,
                            const float* color, int T, int H, int W, int nftrs,
                            float* marked_out) {
  if (!ctx || !vid || !spix || !color || !marked_out) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  if (nftrs != 3) return fail(ctx, STSPIX_ERR_ARG, "nftrs must be 3 (got %d)", nftrs);
  int r;
  if ((r = check_size(ctx, H, W))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  long long n = (long long)T * H * W;
  uint8_t* border = nullptr;
  CK(cudaMallocAsync((void**)&border, (size_t)std::max(n, 1LL), st));
  LAUNCH(k_find_border_end, n, spix, border, H, W, T);
  LAUNCH(k_overlay, n, marked_out, vid, color, border, n);
  CK(cudaFreeAsync(border, st));
  CK(cudaGetLastError());
  return STSPIX_OK;
}

}  // extern "C"
