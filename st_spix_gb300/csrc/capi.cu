// Host orchestration and C ABI of the GB300 streaming-BASS engine.
//
// Every frame, alone or in a batch, goes through one batch runner.  A batch is a
// set of slots (one frame each, uneven sizes allowed) described by device slot
// tables; each phase of the per-frame path is ONE launch over all slots of the
// batch (grid y = slot), so launch count and fixed costs are paid once per batch,
// not once per frame, and a frame's arithmetic is the same alone and in a batch.
// The outer BASS loop runs the slots sorted by iteration count, so at outer
// iteration idx the slots still iterating are a prefix of the table.
//
// No host synchronisation inside the BASS loop and no grid-wide barrier anywhere:
// the reference's host-driven loops (split BFS, hole filling, connected components)
// become a block-per-superpixel BFS, a block-per-frame fill over the hole list and
// a union-find, and the values the reference reads back every step stay on the
// device.  A batch with propagated frames and the 4/8/12 iteration ladder reads the
// hole counts back once (the ladder picks each frame's iteration count from them).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <vector>

#include <map>
#include <mutex>

#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace stspix {

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Working buffers of one batch position.
struct SlotWork {
  std::vector<Buf> pix, sp, lab;
  int npix_cap = 0, sp_cap = 0, lab_cap = 0;
  float* lab_img = nullptr;        // CIELAB frame of stspix_config.lab_ingest (on demand)
  Slot s{};
};

// One frame of a batch as the host sees it.
struct FrameDesc {
  const float* img = nullptr;
  const float* flow = nullptr;
  int H = 0, W = 0, sp_size = 0;
  int* seg = nullptr;              // output labels (propagated: filled labels on entry
                                   // when the shift stage is skipped)
  int mode = 0;                    // 0 BASS, 1 propagated
  const int* prev = nullptr;       // previous labels (shift stage)
  int n_prev = 0;
  stspix_params pprev{}, pout{};
  int* shifted = nullptr;          // shifted labels (null: slot workspace)
  int* resident = nullptr;         // keep the finished labels here
  int niters = -1;                 // -1: decided by the runner
  int slot = 0;                    // batch position (workspace index)
};

enum { kStageShift = 1, kStageSeg = 2 };

// Launch geometry of a slot table.
struct List {
  Slot* d = nullptr;               // device table
  int B = 0;
  int max_npix = 0, max_cap = 0, max_nprev = 0, max_w = 0, max_h = 0;
  bool any_prop = false;
  std::vector<int> tiles_upto[3];  // sweep tiles (32-, 64-, 16-wide) of the first i slots
  std::vector<long long> segs_upto;  // 32-pixel row segments of the first i slots
};

}  // namespace stspix

using namespace stspix;

struct stspix_video {
  stspix_ctx* ctx = nullptr;
  int H = 0, W = 0;
  int n = 0;                 // superpixels of the last frame
  int cur = 0;               // params of the last frame: pp[cur]
  long long frames = 0;
  int* labels = nullptr;     // last frame's labels
  stspix_params pp[2]{};
  int pp_cap = 0;
  std::vector<Buf> lbufs, pbufs;
};

struct stspix_ctx {
  int device = 0;
  int num_sms = 0;
  std::string err;
  long long launches = 0;
  stspix_frame_log log{};
  std::vector<SlotWork> work;
  // per-slot control (bcap slots)
  int bcap = 0;
  Scalars* sc = nullptr;        // device [bcap]
  Scalars* sc_host = nullptr;   // pinned [bcap]
  Slot* d_slots = nullptr;      // device [4 * bcap]: all, BASS, propagated, loop order
  Slot* h_slots = nullptr;      // pinned staging of the same
  std::vector<Buf> ctl_bufs;
  // hole-fill loop graphs (conditional WHILE node), per (slot table, batch size)
  struct FillGraph { cudaGraph_t g; cudaGraphExec_t exec; };
  std::map<std::pair<const Slot*, int>, FillGraph> fill_graphs;
  // sweep tile autotuner
  std::map<std::pair<unsigned long long, int>, int> sweep_choice;  // (tile class, single forced) -> widths
  cudaEvent_t tune_ev[kSweepVariants + 1] = {};
  long long tunes = 0;
  int accumulator = 0;            // cfg.accumulator of the batch being run
  int lab_ingest = 0;             // cfg.lab_ingest of the batch being run
  int* body_iters = nullptr;       // device: [0] fill-loop iterations run (launch count),
                                   // [1] the fill compaction's block counter, [2..3] the
                                   // work-queue sweep's tile and block counters
  int* body_iters_host = nullptr;  // pinned
  long long body_iters_seen = 0;
  // bist_forward's stream state
  stspix_video* fwd = nullptr;
  // profiling (CUDA events on the launching stream)
  int prof_on = 0;
  int cur_fam = STSPIX_FAM_OTHER;
  std::vector<cudaEvent_t> ev_free;
  struct Pending { int fam; const char* name; cudaEvent_t a, b; };
  std::vector<Pending> pending;
  long long fam_launches[STSPIX_NFAM] = {0};
  double fam_ms[STSPIX_NFAM] = {0};
  std::map<std::string, std::pair<long long, double>> kern;  // per kernel: launches, ms
  struct FrameEv { cudaEvent_t a, b; int n; };  // n frames between a and b
  std::vector<FrameEv> frame_ev;
  std::vector<double> frame_ms;
  cudaEvent_t batch_ev[2] = {nullptr, nullptr};
  double batch_ms = 0;
  // batch graphs: a batch step seen before (same signature) is captured once and
  // replayed; launches = kernels one replay runs (for the launch counter)
  bool capturing = false;
  cudaStream_t cap_stream = nullptr;   // records graphs for callers on the legacy stream
  bool graphs_on = true;
  struct BatchGraph { cudaGraph_t g; cudaGraphExec_t exec; long long launches, last; };
  long long graph_tick = 0;
  std::map<std::string, BatchGraph> batch_graphs;
  std::map<std::string, int> batch_seen;
  long long graph_replays = 0;
};

namespace {

// One lock for the rare operations that synchronise the whole device or change its
// allocations (growing workspaces, freeing a video's state, destroying a context)
// and for graph construction: contexts used from several host threads never run a
// device-wide synchronisation or free while another thread captures a graph.
std::mutex g_device_mu;

const int kThreads = 256;
const int kBfsBigSmem = 5 * 512 * 8 * 8;  // kb_split_bfs_big: 5 arrays of 512 rows x 8 words
inline unsigned blocks_for(long long n) { return (unsigned)std::max(1LL, (n + kThreads - 1) / kThreads); }
// Threads of a FOR_PIX kernel over n pixels.
inline long long pix_units(long long n) { return (n + kPixPerThread - 1) / kPixPerThread; }
// 64 x 32 tiles of the largest frame of a slot table (per-slot grids of the warp-block
// kernels; blocks past a smaller frame's tiles return).
inline unsigned tiles64(const List& L) {
  return (unsigned)std::max(1, ((L.max_w + 63) / 64) * ((L.max_h + 31) / 32));
}

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
inline void prof_end(stspix_ctx* ctx, cudaStream_t st, cudaEvent_t a, const char* name) {
  if (!a) return;
  cudaEvent_t b = ev_get(ctx);
  cudaEventRecord(b, st);
  ctx->pending.push_back({ctx->cur_fam, name, a, b});
}
// Called after the stream has been synchronised.
void prof_harvest(stspix_ctx* ctx) {
  for (auto& p : ctx->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      ctx->fam_ms[p.fam] += ms;
      ctx->fam_launches[p.fam] += 1;
      auto& k = ctx->kern[p.name];
      k.first += 1;
      k.second += ms;
    }
    ctx->ev_free.push_back(p.a);
    ctx->ev_free.push_back(p.b);
  }
  ctx->pending.clear();
}

// Every kernel is launched with programmatic stream serialization (see pdl.h).
// (pdl 0: a plain stream dependency, as while a batch graph is captured)
template <typename... KArgs, typename... Args>
void launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, int pdl,
              Args... args) {
  cudaLaunchConfig_t c = {};
  c.gridDim = grid;
  c.blockDim = block;
  c.dynamicSmemBytes = smem;
  c.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = pdl;
  c.attrs = at;
  c.numAttrs = 1;
  cudaLaunchKernelEx(&c, k, args...);
}

#define LAUNCHG(kernel, grid, block, ...)                                      \
  do {                                                                         \
    cudaEvent_t pe_ = prof_begin(ctx, st);                                     \
    launch_k(kernel, dim3(grid), dim3(block), 0, st, ctx->capturing ? 0 : 1, __VA_ARGS__); \
    ctx->launches++;                                                           \
    prof_end(ctx, st, pe_, #kernel);                                           \
  } while (0)

#define LAUNCH(kernel, n, ...)                                                 \
  do {                                                                         \
    long long n_ = (n);                                                        \
    if (n_ > 0) LAUNCHG(kernel, blocks_for(n_), kThreads, __VA_ARGS__);        \
  } while (0)

// One launch over `nb` slots of table L, `n` work items per slot (max over slots).
#define LAUNCHB(kernel, n, L, nb, ...)                                         \
  do {                                                                         \
    long long n_ = (n);                                                        \
    if (n_ > 0 && (nb) > 0)                                                    \
      LAUNCHG(kernel, dim3(blocks_for(n_), (unsigned)(nb)), kThreads, (L).d, ##__VA_ARGS__); \
  } while (0)

// One thread per slot.
#define LAUNCHS(kernel, L, nb, ...)                                            \
  do {                                                                         \
    if ((nb) > 0) LAUNCHG(kernel, blocks_for(nb), kThreads, (L).d, (nb), ##__VA_ARGS__); \
  } while (0)

template <typename T>
int alloc(stspix_ctx* ctx, std::vector<Buf>& list, T** p, size_t n) {
  void* q = nullptr;
  size_t bytes = (std::max<size_t>(n, 1) * sizeof(T) + 15) & ~size_t(15);
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

int alloc_spdev(stspix_ctx* ctx, std::vector<Buf>& L, SpDev& s, int cap) {
  s.cap = cap;
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

int alloc_params(stspix_ctx* ctx, std::vector<Buf>& L, stspix_params& p, int cap) {
  p.capacity = cap;
  AL(L, p.mu_app, 3 * (size_t)cap); AL(L, p.prior_mu_app, 3 * (size_t)cap);
  AL(L, p.mu_shape, 2 * (size_t)cap); AL(L, p.sigma_shape, 3 * (size_t)cap);
  AL(L, p.logdet_sigma_shape, cap); AL(L, p.prior_mu_shape, 2 * (size_t)cap);
  AL(L, p.prior_sigma_shape, 3 * (size_t)cap); AL(L, p.sample_sigma_shape, 3 * (size_t)cap);
  AL(L, p.counts, cap); AL(L, p.sm_counts, cap); AL(L, p.prior_counts, cap);
  AL(L, p.ids, cap); AL(L, p.invalid_counts, cap);
  return STSPIX_OK;
}

// Bytes of the buffers above (for admission under a memory budget).
constexpr long long kPixBytes = 1 + 5 * 4 + 8 + 4 + 2;        // border, d1 d2 smseg hits shifted, best, seg_alt, chg x2
constexpr long long kSpDevBytes = 4 + 1 + 1 + 4 + 4 + 4 + 12 + 16 + 24 + 8 + 12 + 16 + 24 + 24 + 24 +
                                  64 + (long long)sizeof(SweepRec);
constexpr long long kSmBytes = 4 + 24 + 24 + 4 + 4 + 4 + 4 + 4 + 1 + 8;
constexpr long long kAuxBytes = 5 * 1 + 6 * 4 + 16 + 8 + 4 + 16 + 8 + 8 + 72 + 4 + 1 + 24;
constexpr long long kParamBytes = 12 + 12 + 16 + 24 + 4 + 16 + 24 + 24 + 4 + 4 + 4 + 4 + 4;

// Make sure slot position i holds npix pixels and sp_cap superpixels.  Growing
// synchronises the device and does not preserve contents.
int ensure_slot(stspix_ctx* ctx, int i, int npix, int sp_cap) {
  if ((int)ctx->work.size() <= i) ctx->work.resize(i + 1);
  SlotWork& w = ctx->work[i];
  Slot& s = w.s;
  if (npix <= w.npix_cap && sp_cap <= w.sp_cap) return STSPIX_OK;
  std::lock_guard<std::mutex> lk(g_device_mu);
  if (npix > w.npix_cap) {
    CK(cudaDeviceSynchronize());
    free_list(w.pix);
    auto& L = w.pix;
    int n = npix;
    AL(L, s.border, n); AL(L, s.d1, n); AL(L, s.d2, n); AL(L, s.smseg, n);
    AL(L, s.hits, n); AL(L, s.shifted, n); AL(L, s.best, n); AL(L, s.seg_alt, n);
    AL(L, s.chg[0], n); AL(L, s.chg[1], n);
    w.npix_cap = npix;
  }
  if (sp_cap > w.sp_cap) {
    CK(cudaDeviceSynchronize());
    free_list(w.sp);
    auto& L = w.sp;
    int cap = sp_cap;
    int r;
    if ((r = alloc_spdev(ctx, L, s.sp, cap))) return r;
    if ((r = alloc_spdev(ctx, L, s.tmp, cap))) return r;
    size_t c2 = (size_t)cap + 2;
    SmDev& sm = s.sm;
    AL(L, sm.count, c2); AL(L, sm.s, 3 * c2); AL(L, sm.sq, 3 * c2);
    AL(L, sm.ninvalid, c2); AL(L, sm.pair, c2); AL(L, sm.claim, c2);
    AL(L, sm.target, c2); AL(L, sm.newid, c2); AL(L, sm.flag, c2);
    AL(L, sm.msingle, c2);
    AL(L, s.flags, c2); AL(L, s.accept, c2); AL(L, s.valid0, c2);
    AL(L, s.living, c2); AL(L, s.mint, c2);
    AL(L, s.excl, c2); AL(L, s.rid, c2); AL(L, s.src_of, c2);
    AL(L, s.cnt_pool, c2); AL(L, s.cs, c2); AL(L, s.cf, c2);
    AL(L, s.fs, 2 * c2); AL(L, s.fds, 2 * c2); AL(L, s.ss, c2);
    AL(L, s.centers, 2 * c2); AL(L, s.rbest, c2); AL(L, s.ccbest, c2);
    AL(L, s.bbox, 4 * c2);
    AL(L, s.snap, 9 * c2); AL(L, s.post_ids, c2); AL(L, s.recchg, c2);
    AL(L, s.pscache, 3 * c2);
    w.sp_cap = cap;
  }
  return STSPIX_OK;
}

// The CIELAB frame buffer of slot position i (stspix_config.lab_ingest), npix pixels.
int ensure_lab(stspix_ctx* ctx, int i, int npix) {
  SlotWork& w = ctx->work[i];
  if (npix <= w.lab_cap) return STSPIX_OK;
  std::lock_guard<std::mutex> lk(g_device_mu);
  CK(cudaDeviceSynchronize());
  free_list(w.lab);
  AL(w.lab, w.lab_img, 3 * (size_t)npix);
  w.lab_cap = npix;
  return STSPIX_OK;
}

// Graphs hold the slot-table and staging addresses: dropped when those move.
void drop_fill_graphs(stspix_ctx* ctx) {
  for (auto& kv : ctx->fill_graphs) {
    cudaGraphExecDestroy(kv.second.exec);
    cudaGraphDestroy(kv.second.g);
  }
  ctx->fill_graphs.clear();
  for (auto& kv : ctx->batch_graphs) {
    cudaGraphExecDestroy(kv.second.exec);
    cudaGraphDestroy(kv.second.g);
  }
  ctx->batch_graphs.clear();
  ctx->batch_seen.clear();
}

// Load every kernel of the library once per process, before any of them is used.
// With lazy module loading a kernel is otherwise loaded by its first launch, which
// may fall inside another thread's stream capture or run concurrently with other
// threads' launches; querying the attributes of each kernel loads it up front.
std::once_flag g_preload_once;
cudaError_t g_preload_err = cudaSuccess;

void preload_kernels() {
  std::call_once(g_preload_once, [] {
    const void* fns[] = {
      (const void*)k_init_hex,
      (const void*)k_find_border,
      (const void*)k_find_border_end,
      (const void*)k_overlay,
      (const void*)k_dump_state,
      (const void*)kb_scalars,
      (const void*)kb_init_hex,
      (const void*)kb_clear_flags,
      (const void*)kb_mark_present,
      (const void*)kb_scan,
      (const void*)kb_remap,
      (const void*)kb_compact_gather,
      (const void*)kb_compact_scatter,
      (const void*)kb_init_bass_params,
      (const void*)kb_init_prior_mu,
      (const void*)kb_clear_stats,
      (const void*)kb_accumulate,
      (const void*)kb_posterior,
      (const void*)kb_post_list,
      (const void*)kb_store_sample,
      (const void*)kb_find_border,
      (const void*)kb_sweep_t32,
      (const void*)kb_sweep_t64,
      (const void*)kb_sweep_t16,
      (const void*)kb_sweep2_t32,
      (const void*)kb_sweep2_t16,
      (const void*)kb_sweep2_t64,
      (const void*)kb_sweepq_t32,
      (const void*)kb_sweepq_t64,
      (const void*)kb_sweepq_t16,
      (const void*)kb_copy_labels,
      (const void*)kb_read_params,
      (const void*)kb_save_prev,
      (const void*)kb_split_begin,
      (const void*)kb_split_clear,
      (const void*)kb_split_seed,
      (const void*)kb_bbox,
      (const void*)kb_split_bfs,
      (const void*)kb_split_bfs_big,
      (const void*)kb_split_partition,
      (const void*)kb_sm_clear,
      (const void*)kb_sm_accumulate,
      (const void*)kb_split_decide,
      (const void*)kb_split_commit,
      (const void*)kb_split_apply,
      (const void*)kb_split_end,
      (const void*)kb_merge_clear,
      (const void*)kb_merge_candidates,
      (const void*)kb_merge_single,
      (const void*)kb_merge_decide,
      (const void*)kb_merge_flag,
      (const void*)kb_merge_remove,
      (const void*)kb_merge_apply,
      (const void*)kb_prop_clear,
      (const void*)kb_flow_pool,
      (const void*)kb_flow_mean,
      (const void*)kb_shift,
      (const void*)kb_shift_decode,
      (const void*)kb_count_labels,
      (const void*)kb_fill_begin,
      (const void*)kb_fill_split,
      (const void*)kb_fill_phase,
      (const void*)kb_fill_end,
      (const void*)kb_cc_local,
      (const void*)kb_cc_hook,
      (const void*)kb_cc_compress,
      (const void*)kb_list_holes,
      (const void*)kb_cc_best,
      (const void*)kb_cc_invalidate,
      (const void*)kb_shift_params,
      (const void*)kb_write_params,
      (const void*)kb_mark_active,
      (const void*)kb_relabel_init,
      (const void*)kb_living,
      (const void*)kb_relabel_compare,
      (const void*)kb_relabel_mark,
      (const void*)kb_relabel_ids,
      (const void*)kb_relabel_params,
      (const void*)kb_relabel_apply,
      (const void*)kb_relabel_end,
      (const void*)kb_count_revived,
      (const void*)kb_accumulate_fp, (const void*)kb_accumulate_fp_store,
      (const void*)kb_accumulate_fp_clear, (const void*)k_label_stats,
      (const void*)k_label_stats_out,
      (const void*)k_rgb2lab, (const void*)k_lab2rgb, (const void*)k_rescale_u8,
      (const void*)kb_lab_ingest};
    for (const void* f : fns) {
      cudaFuncAttributes a;
      cudaError_t e = cudaFuncGetAttributes(&a, f);
      if (e != cudaSuccess && g_preload_err == cudaSuccess) g_preload_err = e;
    }
  });
}

// Per-slot control arrays for batches of up to B slots.
int ensure_bcap(stspix_ctx* ctx, int B) {
  if (B <= ctx->bcap) return STSPIX_OK;
  std::lock_guard<std::mutex> lk(g_device_mu);
  CK(cudaDeviceSynchronize());
  drop_fill_graphs(ctx);
  free_list(ctx->ctl_bufs);
  if (ctx->sc_host) { cudaFreeHost(ctx->sc_host); ctx->sc_host = nullptr; }
  if (ctx->h_slots) { cudaFreeHost(ctx->h_slots); ctx->h_slots = nullptr; }
  int nb = std::max(B, 2 * ctx->bcap);
  auto& L = ctx->ctl_bufs;
  AL(L, ctx->sc, nb);
  AL(L, ctx->d_slots, 4 * (size_t)nb);
  CK(cudaMallocHost(&ctx->sc_host, sizeof(Scalars) * nb));
  CK(cudaMallocHost(&ctx->h_slots, sizeof(Slot) * 4 * nb));
  CK(cudaMemset(ctx->sc, 0, sizeof(Scalars) * nb));
  ctx->bcap = nb;
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

int slot_cap(const FrameDesc& f) {
  // propagated frames: the reference's 10 x n_prev (+2) rounded up to a power of two,
  // so consecutive frames of a stream keep one capacity (and one launch geometry); the
  // logical buffer size (split rule) stays 10 x n_prev (Scalars::nbuf_logical)
  if (f.mode) {
    int c = 64;
    while (c < 10 * f.n_prev + 2) c <<= 1;
    return c;
  }
  double Hh, w;
  int nx, ny;
  hex_geometry(f.sp_size, f.W, f.H, &Hh, &w, &nx, &ny);
  return std::max(30 * nx * ny, 64);
}

// Fill the slot record of frame f (workspace pointers + frame fields).
Slot make_slot(stspix_ctx* ctx, const FrameDesc& f, int cap) {
  Slot s = ctx->work[f.slot].s;
  s.img = f.img;
  s.img_src = nullptr;
  if (ctx->lab_ingest) {          // converted at ingest into the slot's CIELAB buffer
    s.img_src = f.img;
    s.img = ctx->work[f.slot].lab_img;
  }
  s.seg = f.seg;
  s.H = f.H; s.W = f.W; s.npix = f.H * f.W;
  s.inv_w = 1.0 / (double)f.W;
  s.inv_h = 1.0 / (double)f.H;
  s.cap = cap;
  s.sp.cap = cap;
  s.tmp.cap = cap;
  s.mode = f.mode;
  s.sp_size = f.sp_size;
  s.lo = f.mode ? f.n_prev : 0;
  hex_geometry(f.sp_size, f.W, f.H, &s.hex_h, &s.hex_w, &s.hex_nx, &s.hex_ny);
  s.nraw = s.hex_nx * s.hex_ny;
  s.prev_labels = f.prev;
  s.flow = f.flow;
  s.n_prev = f.n_prev;
  s.pprev = f.pprev;
  s.pout = f.pout;
  if (f.shifted) s.shifted = f.shifted;
  s.resident_labels = f.resident;
  s.sc = ctx->sc + f.slot;
  return s;
}

// Build a slot table at `off` (0 all, 1 BASS, 2 propagated, 3 loop order) of the
// staging area and its launch geometry.  Each table has its own staging area, so no
// host write touches the source of a copy still queued on the stream.
List make_list(stspix_ctx* ctx, int off, const std::vector<Slot>& slots) {
  List L;
  L.d = ctx->d_slots + (size_t)off * ctx->bcap;
  for (int v = 0; v < kSweepVariants; v++) L.tiles_upto[v].assign(1, 0);
  L.segs_upto.assign(1, 0);
  Slot* h = ctx->h_slots + (size_t)off * ctx->bcap;
  L.B = (int)slots.size();
  for (int i = 0; i < L.B; i++) {
    Slot s = slots[i];
    for (int v = 0; v < kSweepVariants; v++) {
      if (L.tiles_upto[v].empty()) L.tiles_upto[v].push_back(0);
      s.tile_base[v] = L.tiles_upto[v].back();
      const int tw = kSweepTileW[v];
      L.tiles_upto[v].push_back(s.tile_base[v] + ((s.W + tw - 1) / tw) * ((s.H + 31) / 32));
    }
    if (L.segs_upto.empty()) L.segs_upto.push_back(0);
    L.segs_upto.push_back(L.segs_upto.back() + (long long)s.H * ((s.W + 31) / 32));
    h[i] = s;
    L.max_npix = std::max(L.max_npix, s.npix);
    L.max_cap = std::max(L.max_cap, s.cap);
    // a bound on n_prev that depends on the capacity only (grids over previous ids)
    if (s.mode) L.max_nprev = std::max(L.max_nprev, (s.cap - 2) / 10);
    L.max_w = std::max(L.max_w, s.W);
    L.max_h = std::max(L.max_h, s.H);
    if (s.mode) L.any_prop = true;
  }
  return L;
}

int upload(stspix_ctx* ctx, cudaStream_t st, const List& L, int off) {
  if (L.B <= 0) return STSPIX_OK;
  CK(cudaMemcpyAsync(L.d, ctx->h_slots + (size_t)off * ctx->bcap, sizeof(Slot) * L.B,
                     cudaMemcpyHostToDevice, st));
  return STSPIX_OK;
}

// ---------------------------------------------------------------------------
// Stages over the first nb slots of a table.

// kb_accumulate: one 8-warp block per 64 x 32 tile of the first nb slots.
unsigned acc_blocks(const stspix_ctx* ctx, const List& L, int nb) {
  (void)ctx;
  return (unsigned)std::max(1LL, (long long)L.tiles_upto[1][nb]);
}

// update_params (update_params.cu:12-52): statistics + posterior.
// The colour sums by FP32 / FP64 atomics instead of int64 fixed point (accumulator
// precision study, cfg.accumulator 1 / 2).
void accumulate_fp(stspix_ctx* ctx, cudaStream_t st, const List& L, int nb, int mode) {
  LAUNCHB(kb_accumulate_fp_clear, L.max_cap, L, nb);
  LAUNCHB(kb_accumulate_fp, L.max_npix, L, nb, mode);
  LAUNCHB(kb_accumulate_fp_store, L.max_cap, L, nb, mode);
}

// stats_ready: the last sweep of the preceding update_seg already cleared and added
// the statistics of the first nb slots (see update_seg).
// incremental: only the ids whose sums changed since their last posterior (kb_post_list);
// only where nothing but sweeps ran since the previous posterior of every slot.
int update_params(stspix_ctx* ctx, cudaStream_t st, const List& L, int nb,
                  bool stats_ready = false, bool incremental = false) {
  ctx->cur_fam = STSPIX_FAM_STATS;
  if (!stats_ready) {
    LAUNCHB(kb_clear_stats, L.max_cap, L, nb);
    LAUNCHG(kb_accumulate, acc_blocks(ctx, L, nb), 256, L.d, nb);
  }
  if (ctx->accumulator) accumulate_fp(ctx, st, L, nb, ctx->accumulator);
  ctx->cur_fam = STSPIX_FAM_POSTERIOR;
  LAUNCHB(kb_post_list, L.max_cap, L, nb, incremental ? 1 : 0);
  // groups of 32 listed ids, about four blocks per SM over the batch (a block loops
  // when a slot lists more groups)
  const unsigned pg = (unsigned)std::min<long long>((L.max_cap + 31) / 32,
                                                    std::max(32, (4 * ctx->num_sms + nb - 1) / nb));
  LAUNCHG(kb_posterior, dim3(pg, (unsigned)nb), 128, L.d, incremental ? 1 : 0);
  return STSPIX_OK;
}

// update_seg (update_seg.cu:281-311): niters_seg fused sweeps ping-ponging between
// the labels and a scratch buffer; the border mask is only built when the next
// iteration's merge reads it.
// fuse_stats: every sweep launch moves the statistics of the pixels it relabels
// (incremental statistics, see kb_sweep_t*), so the statistics stay those of the
// current labels and the next update_params skips its clear and accumulate passes.
// Not while tuning (the trial launches rerun the same sweep).  *fused tells whether
// that happened.
// first_active: the first sweep is an active-set sweep too (mode 2): only the
// previous call's last-sweep changes (change plane 1) and the pixels next to a label
// whose record the posterior between the calls changed can decide differently.  For
// calls that follow one with *chg_ok set, with only an incremental posterior between.
// *chg_ok: this call ran no tuning trials and an even number of launches, so change
// plane 1 holds its last sweep's changes.
int update_seg(stspix_ctx* ctx, cudaStream_t st, const List& L, int nb,
               const stspix_config& cfg, bool need_border, bool fuse_stats, bool* fused,
               bool first_active = false, bool* chg_ok = nullptr) {
  ctx->cur_fam = STSPIX_FAM_SWEEP;
  const int nseg = cfg.niters_seg;
  *fused = false;
  if (chg_ok) *chg_ok = false;
  // the first sweep of the call scores every border pixel; the later ones only the
  // active set next to the previous sweep's changes (same labels, see kb_sweep_t*).
  // Launch j reads the labels of parity j & 1 and writes the other buffer.
  auto sweep1 = [&](int v, int parity, int mode, int stats) {
    const unsigned g = (unsigned)std::max(1, L.tiles_upto[v][nb]);
    if (cfg.sweep_queue) {
      // persistent work queue: the blocks the SMs hold at once (6 per SM), at most one
      // per tile
      unsigned* q = (unsigned*)(ctx->body_iters + 2);
      const unsigned gq = std::min<unsigned>(g, 6u * (unsigned)ctx->num_sms);
      const int nt = (int)g;
      if (v == 1)
        LAUNCHG(kb_sweepq_t64, gq, 256, L.d, nb, nt, q, parity, cfg.sigma2_app, cfg.potts, mode,
                stats);
      else if (v == 2)
        LAUNCHG(kb_sweepq_t16, gq, 256, L.d, nb, nt, q, parity, cfg.sigma2_app, cfg.potts, mode,
                stats);
      else
        LAUNCHG(kb_sweepq_t32, gq, 256, L.d, nb, nt, q, parity, cfg.sigma2_app, cfg.potts, mode,
                stats);
      return;
    }
    if (v == 1)
      LAUNCHG(kb_sweep_t64, g, 256, L.d, nb, parity, cfg.sigma2_app, cfg.potts, mode, stats);
    else if (v == 2)
      LAUNCHG(kb_sweep_t16, g, 256, L.d, nb, parity, cfg.sigma2_app, cfg.potts, mode, stats);
    else
      LAUNCHG(kb_sweep_t32, g, 256, L.d, nb, parity, cfg.sigma2_app, cfg.potts, mode, stats);
  };
  auto sweep2 = [&](int v, int parity, int mode, int stats) {   // v: 0 (32 wide), 1 (64), 2 (16)
    const unsigned g = (unsigned)std::max(1, L.tiles_upto[v][nb]);
    if (v == 2)
      LAUNCHG(kb_sweep2_t16, g, 256, L.d, nb, parity, cfg.sigma2_app, cfg.potts, mode, stats);
    else if (v == 1)
      LAUNCHG(kb_sweep2_t64, g, 256, L.d, nb, parity, cfg.sigma2_app, cfg.potts, mode, stats);
    else
      LAUNCHG(kb_sweep2_t32, g, 256, L.d, nb, parity, cfg.sigma2_app, cfg.potts, mode, stats);
  };
  // Tile autotuner: the first update of a batch size class runs its first sweep with
  // every single-sweep tile width and (with three or more sweeps) its second and
  // third sweeps with every two-sweep width, each on the same input (a launch reads
  // only the labels at its start, so all write the same output); the class keeps the
  // fastest single width and, when the best two-sweep launch beats two single ones,
  // two-sweep launches.  The class is the number of 32x32 tiles of the sweeping slots
  // in quarter octaves: the choice depends on how well the tiles fill the SMs, and
  // mixed serving batches then tune a handful of times.
  const int tl = std::max(1, L.tiles_upto[0][nb]);
  // (a forced single-sweep schedule keeps its own entries: its tuning skips the pairs)
  const auto key = std::make_pair((unsigned long long)std::floor(4.0 * std::log2((double)tl)),
                                  cfg.sweep_schedule == 1 ? 1 : 0);
  auto ch = ctx->sweep_choice.find(key);
  int done = 0, launch = 0;
  int v1 = 1, v2 = -1;      // best single-sweep width, two-sweep width (-1: none)
  int forced = -1;     // the width stspix_config.sweep_tile pins
  for (int c = 0; c < kSweepVariants; c++)
    if (kSweepTileW[c] == cfg.sweep_tile) forced = c;
  if (cfg.sweep_schedule == 2) {
    v1 = forced >= 0 ? forced : 0;
    v2 = v1;
  } else if (forced >= 0) {
    v1 = forced;
    v2 = -1;
  } else if (ch != ctx->sweep_choice.end()) {
    v1 = ch->second & 0xff;
    v2 = cfg.sweep_schedule == 1 ? -1 : (ch->second >> 8) - 1;
  } else if (ctx->capturing) {
    v1 = 1;     // no timing inside a graph capture (a replayed batch was tuned before)
    v2 = -1;
  } else if (nseg > 0) {
    // the whole call's launch count is known only after tuning; the clear rides on the
    // first launch, the accumulation on the last (decided when it is issued)
    // Every trial runs kTuneRounds times and keeps its fastest run: other streams of
    // the device (concurrent lanes) only ever slow a run down.
    float t1[kSweepVariants];
    for (int r = 0; r < kTuneRounds; r++) {
      CK(cudaEventRecord(ctx->tune_ev[0], st));
      for (int c = 0; c < kSweepVariants; c++) {
        sweep1(c, 0, 0, 0);
        CK(cudaEventRecord(ctx->tune_ev[c + 1], st));
      }
      CK(cudaEventSynchronize(ctx->tune_ev[kSweepVariants]));
      for (int c = 0; c < kSweepVariants; c++) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->tune_ev[c], ctx->tune_ev[c + 1]);
        t1[c] = r == 0 ? ms : std::min(t1[c], ms);
      }
    }
    float best1 = t1[0];
    v1 = 0;
    for (int c = 1; c < kSweepVariants; c++)
      if (t1[c] < best1) { best1 = t1[c]; v1 = c; }
    // Large batches keep the widest tile (the least halo work per pixel: 1.41 staged
    // labels per pixel against 1.56 for 32x32) unless another width is 5 % faster:
    // with other lanes' kernels on the SMs the total work decides, and timings of
    // 64x32 and 32x32 alone differ by less than their noise (batches of 8 480x854
    // frames on three lanes: 1545 frames/s when one lane picked 32x32, 1635-1642
    // with 64x32 on all).
    if (tl >= kPairMaxTiles && t1[1] <= kWideMargin * best1) {
      best1 = t1[1];
      v1 = 1;
    }
    done = 1;
    launch = 1;
    // Large batches keep single sweeps: a two-sweep launch holds more registers (4
    // blocks per SM against 6), which costs more than its timing alone shows once other
    // lanes' kernels share the SMs (batches of 8 480x854 frames on three lanes: 1532-1535
    // frames/s when one lane picked 64x32 pairs, 1624-1631 with single sweeps on all).
    if (nseg >= 3 && cfg.sweep_schedule == 0 && tl < kPairMaxTiles) {
      // a two-sweep launch is an active-set sweep plus a full-listing one: with four or
      // more sweeps the second sweep runs alone (timed, active set) and the pair covers
      // the third and fourth, and the pair is compared with that sweep plus a full one
      float ref = 2.f * best1;
      if (nseg >= 4) {
        float ms1 = 0.f;
        for (int r = 0; r < kTuneRounds; r++) {
          CK(cudaEventRecord(ctx->tune_ev[0], st));
          sweep1(v1, launch & 1, 1, 0);
          CK(cudaEventRecord(ctx->tune_ev[1], st));
          CK(cudaEventSynchronize(ctx->tune_ev[1]));
          float ms = 0.f;
          cudaEventElapsedTime(&ms, ctx->tune_ev[0], ctx->tune_ev[1]);
          ms1 = r == 0 ? ms : std::min(ms1, ms);
        }
        ref = best1 + ms1;
        done = 2;
        launch = 2;
      }
      // (both pair runs write the same labels; neither moves statistics, which would
      // count them twice: a tuned call ends with a full statistics pass)
      float t2[kSweepVariants];
      for (int r = 0; r < kTuneRounds; r++) {
        CK(cudaEventRecord(ctx->tune_ev[0], st));
        for (int c = 0; c < kSweepVariants; c++) {
          sweep2(c, launch & 1, 1, 0);
          CK(cudaEventRecord(ctx->tune_ev[c + 1], st));
        }
        CK(cudaEventSynchronize(ctx->tune_ev[kSweepVariants]));
        for (int c = 0; c < kSweepVariants; c++) {
          float ms = 0.f;
          cudaEventElapsedTime(&ms, ctx->tune_ev[c], ctx->tune_ev[c + 1]);
          t2[c] = r == 0 ? ms : std::min(t2[c], ms);
        }
      }
      float best2 = t2[0];
      int b2 = 0;
      for (int c = 1; c < kSweepVariants; c++)
        if (t2[c] < best2) { best2 = t2[c]; b2 = c; }
      v2 = best2 < ref ? b2 : -1;
      done += 2;
      launch += 1;
    }
    ctx->sweep_choice[key] = v1 | ((v2 + 1) << 8);
    ctx->tunes++;
    if (done >= nseg) {
      if (launch & 1) LAUNCHB(kb_copy_labels, pix_units(L.max_npix), L, nb);
      if (need_border) {
        ctx->cur_fam = STSPIX_FAM_MERGE;
        LAUNCHB(kb_find_border, pix_units(L.max_npix), L, nb);
      }
      return STSPIX_OK;
    }
  }
  const bool untuned = done == 0;             // no tuning trials in this call
  const bool fuse = fuse_stats && untuned;
  while (done < nseg) {
    const bool pair = v2 >= 0 && nseg - done >= 2;
    const int deltas = fuse ? 1 : 0;
    const int mode = done > 0 ? 1 : (first_active && untuned ? 2 : 0);
    if (pair) sweep2(v2, launch & 1, mode, deltas);
    else sweep1(v1, launch & 1, mode, deltas);
    done += pair ? 2 : 1;
    launch++;
  }
  *fused = fuse;
  if (chg_ok) *chg_ok = untuned && launch > 0 && (launch & 1) == 0;
  if (launch & 1) LAUNCHB(kb_copy_labels, pix_units(L.max_npix), L, nb);
  if (need_border) {
    ctx->cur_fam = STSPIX_FAM_MERGE;
    LAUNCHB(kb_find_border, pix_units(L.max_npix), L, nb);
  }
  return STSPIX_OK;
}

int run_split(stspix_ctx* ctx, cudaStream_t st, const List& L, int nb, const SmConsts& K,
              const stspix_config& cfg, int dir_b, int dir_p) {
  ctx->cur_fam = STSPIX_FAM_SPLIT;
  LAUNCHS(kb_split_begin, L, nb);
  LAUNCHB(kb_split_clear, pix_units(L.max_npix), L, nb);
  LAUNCHB(kb_split_seed, L.max_cap, L, nb, dir_b, dir_p);
  LAUNCHG(kb_bbox, dim3(tiles64(L), (unsigned)nb), kThreads, L.d);
  LAUNCHG(kb_split_bfs, dim3(256, (unsigned)nb), 128, L.d, dir_b, dir_p);  // 1024 warps per slot
  {
    cudaEvent_t pe_ = prof_begin(ctx, st);
    launch_k(kb_split_bfs_big, dim3(8, (unsigned)nb), dim3(256), kBfsBigSmem, st,
             ctx->capturing ? 0 : 1, L.d);
    ctx->launches++;
    prof_end(ctx, st, pe_, "kb_split_bfs_big");
  }
  LAUNCHB(kb_split_partition, pix_units(L.max_npix), L, nb);
  LAUNCHB(kb_sm_clear, L.max_cap + 2, L, nb);
  LAUNCHG(kb_sm_accumulate, dim3(tiles64(L), (unsigned)nb), kThreads, L.d, 1);
  LAUNCHG(kb_split_decide, dim3((unsigned)((L.max_cap + 31) / 32), (unsigned)nb), 128, L.d, K,
          cfg.split_alpha);
  LAUNCHG(kb_scan, (unsigned)nb, 1024, L.d, 1);
  LAUNCHB(kb_split_commit, L.max_cap, L, nb);
  LAUNCHB(kb_split_apply, pix_units(L.max_npix), L, nb);
  LAUNCHS(kb_split_end, L, nb);
  return STSPIX_OK;
}

// relabel (relabel.cu:126-409) on the propagated slots among the first nb.
int run_relabel(stspix_ctx* ctx, cudaStream_t st, const List& L, int nb,
                const stspix_config& cfg) {
  ctx->cur_fam = STSPIX_FAM_MERGE;
  LAUNCHB(kb_relabel_init, L.max_cap + 2, L, nb);
  LAUNCHG(kb_living, dim3(tiles64(L), (unsigned)nb), kThreads, L.d);
  dim3 g(blocks_for(L.max_cap),
         (unsigned)std::max(1, (L.max_nprev + kRelabelChunk - 1) / kRelabelChunk), (unsigned)nb);
  LAUNCHG(kb_relabel_compare, g, kThreads, L.d);
  LAUNCHB(kb_relabel_mark, L.max_cap, L, nb, cfg.thresh_relabel, cfg.thresh_new);
  LAUNCHG(kb_scan, (unsigned)nb, 1024, L.d, 2);
  LAUNCHB(kb_relabel_ids, L.max_cap, L, nb);
  LAUNCHB(kb_relabel_params, L.max_cap, L, nb);
  LAUNCHB(kb_relabel_apply, pix_units(L.max_npix), L, nb);
  LAUNCHB(kb_count_revived, L.max_cap, L, nb);
  LAUNCHS(kb_relabel_end, L, nb);
  return STSPIX_OK;
}

int run_merge(stspix_ctx* ctx, cudaStream_t st, const List& L, int nb, const SmConsts& K,
              const stspix_config& cfg, int dir_b, int dir_p) {
  ctx->cur_fam = STSPIX_FAM_MERGE;
  LAUNCHB(kb_merge_clear, L.max_cap + 2, L, nb);
  LAUNCHB(kb_merge_candidates, pix_units(L.max_npix), L, nb, dir_b, dir_p);
  LAUNCHB(kb_sm_clear, L.max_cap + 2, L, nb);
  LAUNCHG(kb_sm_accumulate, dim3(tiles64(L), (unsigned)nb), kThreads, L.d, 0);
  LAUNCHG(kb_merge_single, dim3((unsigned)((L.max_cap + 31) / 32), (unsigned)nb), 128, L.d, K);
  LAUNCHG(kb_merge_decide, dim3((unsigned)((L.max_cap + 31) / 32), (unsigned)nb), 128, L.d, K,
          cfg.merge_alpha);
  LAUNCHB(kb_merge_flag, L.max_cap, L, nb);
  LAUNCHB(kb_merge_remove, L.max_cap, L, nb);
  LAUNCHB(kb_merge_apply, pix_units(L.max_npix), L, nb);
  return STSPIX_OK;
}

// bass (bass.cu:46-181) / prop_bass_v3 (prop.cu:326-468) outer loop over a table
// sorted by iteration count (nit[i] descending).  stop_after >= 0 (one slot only):
// stop before that iteration (bass_partial).
int bass_loop(stspix_ctx* ctx, cudaStream_t st, const List& L, const std::vector<int>& nit,
              const stspix_config& cfg, const SmConsts& K, int stop_after, int extra_update) {
  int r;
  int count_b = 1, count_p = 1;
  const int P = cfg.sm_period > 0 ? cfg.sm_period : 4;
  const int maxn = L.B ? nit[0] : 0;
  int nb = L.B;
  // the statistics of the first nb slots were kept current by the previous
  // iteration's sweeps (incremental statistics; integer sums, so identical to a full
  // pass); the int64 accumulator only
  bool stats_ready = false;
  const bool fuse = ctx->accumulator == 0;
  bool chg_ok = false;      // the previous update_seg left its last changes in plane 1
  for (int idx = 0; idx < maxn; idx++) {
    while (nb > 0 && nit[nb - 1] <= idx) nb--;
    if (stop_after >= 0 && idx == stop_after) {
      if (extra_update && (r = update_params(ctx, st, L, nb))) return r;
      return STSPIX_OK;
    }
    // after the first iteration only the sweeps ran since every slot's last posterior
    if ((r = update_params(ctx, st, L, nb, stats_ready, idx > 0))) return r;
    stats_ready = false;
    // the first sweep is an active-set one when only sweeps and that incremental
    // posterior ran since the previous update_seg
    bool first_active = idx > 0 && chg_ok;
    if (idx > cfg.sm_start) {
      if (idx % P == 0 || idx % P == P / 2) first_active = false;
      if (idx % P == 0) {
        count_b += 1;
        count_p += 1;
        if ((r = run_split(ctx, st, L, nb, K, cfg, count_b % 2 + 1, count_p % 2 + 1))) return r;
        if ((r = update_params(ctx, st, L, nb))) return r;
      }
      if (idx % P == P / 2) {
        count_p += 1;  // propagated frames step the direction again before merging
        if (L.any_prop && (r = run_relabel(ctx, st, L, nb, cfg))) return r;
        if ((r = run_merge(ctx, st, L, nb, K, cfg, count_b % 2, count_p % 2))) return r;
        if ((r = update_params(ctx, st, L, nb))) return r;
      }
    }
    const int nx = idx + 1;
    const bool merge_next = nx < maxn && nx > cfg.sm_start && nx % P == P / 2;
    const bool fuse_now = fuse && nx < maxn && !(stop_after >= 0 && nx == stop_after);
    bool fused = false;
    if ((r = update_seg(ctx, st, L, nb, cfg, merge_next || stop_after >= 0, fuse_now, &fused,
                        first_active, &chg_ok)))
      return r;
    stats_ready = fused;
  }
  if (stop_after >= 0) {
    if (extra_update && (r = update_params(ctx, st, L, L.B))) return r;
    return STSPIX_OK;
  }
  // final update_params + store_sample; slots that finished earlier were untouched
  // since, so running theirs here is the same as running it right after their loop
  if ((r = update_params(ctx, st, L, L.B, false, maxn > 0))) return r;
  ctx->cur_fam = STSPIX_FAM_POSTERIOR;
  LAUNCHB(kb_store_sample, L.max_cap, L, L.B);
  return STSPIX_OK;
}

// The legacy prop_cuda split (prop/bass.cu:464-488 run_split_py) on the propagated
// model: update_params, one split step in direction dir, and the outer loop's closing
// update_params + store_sample.
int split_only(stspix_ctx* ctx, cudaStream_t st, const List& L, const stspix_config& cfg,
               const SmConsts& K, int dir) {
  int r;
  if ((r = update_params(ctx, st, L, L.B))) return r;
  if ((r = run_split(ctx, st, L, L.B, K, cfg, dir, dir))) return r;
  if ((r = update_params(ctx, st, L, L.B))) return r;
  ctx->cur_fam = STSPIX_FAM_POSTERIOR;
  LAUNCHB(kb_store_sample, L.max_cap, L, L.B);
  return STSPIX_OK;
}

// compactify_new_superpixels (compact_spix.cu:41-89) for ids >= lo, moving params.
int compact(stspix_ctx* ctx, cudaStream_t st, const List& L) {
  ctx->cur_fam = STSPIX_FAM_OTHER;
  LAUNCHB(kb_clear_flags, L.max_cap + 2, L, L.B);
  LAUNCHS(kb_scalars, L, L.B, (int)kOpCompactN);
  LAUNCHB(kb_mark_present, pix_units(L.max_npix), L, L.B, 1);
  LAUNCHG(kb_scan, (unsigned)L.B, 1024, L.d, 3);
  LAUNCHB(kb_compact_gather, L.max_cap, L, L.B);
  LAUNCHB(kb_compact_scatter, L.max_cap, L, L.B);
  LAUNCHB(kb_remap, pix_units(L.max_npix), L, L.B, 1);
  LAUNCHS(kb_scalars, L, L.B, (int)kOpCompactEnd);
  return STSPIX_OK;
}

// run_bass set-up (bass.cu:221-262) on the BASS slots.
int bass_init(stspix_ctx* ctx, cudaStream_t st, const List& L) {
  if (L.B <= 0) return STSPIX_OK;
  ctx->cur_fam = STSPIX_FAM_OTHER;
  LAUNCHG(kb_init_hex, dim3(tiles64(L), (unsigned)L.B), kThreads, L.d);
  // compact the hex ids (extract_unique_ids + compactify, bass.cu:251-252)
  LAUNCHB(kb_clear_flags, L.max_cap + 2, L, L.B);
  LAUNCHB(kb_mark_present, pix_units(L.max_npix), L, L.B, 0);
  LAUNCHG(kb_scan, (unsigned)L.B, 1024, L.d, 0);
  LAUNCHB(kb_remap, pix_units(L.max_npix), L, L.B, 0);
  LAUNCHS(kb_scalars, L, L.B, (int)kOpAfterHex);
  LAUNCHB(kb_init_bass_params, L.max_cap, L, L.B);
  LAUNCHB(kb_clear_stats, L.max_cap, L, L.B);
  LAUNCHG(kb_accumulate, acc_blocks(ctx, L, L.B), 256, L.d, L.B);
  if (ctx->accumulator) accumulate_fp(ctx, st, L, L.B, ctx->accumulator);
  LAUNCHB(kb_init_prior_mu, L.max_cap, L, L.B);
  LAUNCHB(kb_find_border, pix_units(L.max_npix), L, L.B);
  return STSPIX_OK;
}

constexpr int kFillUnroll = 2;

// The hole-fill loop of the propagated slots of table L as a graph: a WHILE node
// whose body is one iteration (kb_fill_phase x 4, added as kernel nodes); the fourth
// phase's last block sets the condition.  Built once per (table, size).
// The loop body's kernel nodes (four parity phases, the last of which closes the
// iteration and sets `cond`) into graph `body`.
cudaError_t add_fill_body(stspix_ctx* ctx, cudaGraph_t body, const List& L,
                          cudaGraphConditionalHandle cond) {
  const unsigned G = (unsigned)std::max(8, std::min(128, 2048 / std::max(L.B, 1)));
  const dim3 grid(G, (unsigned)L.B);
  Slot* table = L.d;
  int B = L.B, break_iter = kFillBreakIter;
  int ph_arg[4] = {0, 1, 2, 3};
  unsigned* ctr = (unsigned*)(ctx->body_iters + 1);
  cudaGraphNode_t prev = nullptr;
  cudaError_t ce = cudaSuccess;
  auto add = [&](const void* fn, dim3 gd, dim3 bd, void** args) {
    if (ce != cudaSuccess) return;
    cudaKernelNodeParams kp = {};
    kp.func = const_cast<void*>(fn);
    kp.gridDim = gd;
    kp.blockDim = bd;
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    cudaGraphNode_t n;
    ce = cudaGraphAddKernelNode(&n, body, prev ? &prev : nullptr, prev ? 1 : 0, &kp);
    prev = n;
  };
  // kFillUnroll iterations per execution of the body: fewer evaluations of the loop
  // condition; an iteration after the loop's end finds every slot done and returns
  void* a_ph[4][7];
  for (int ph = 0; ph < 4; ph++) {
    a_ph[ph][0] = (void*)&table;
    a_ph[ph][1] = (void*)&ph_arg[ph];
    a_ph[ph][2] = (void*)&B;
    a_ph[ph][3] = (void*)&cond;
    a_ph[ph][4] = (void*)&break_iter;
    a_ph[ph][5] = (void*)&ctx->body_iters;
    a_ph[ph][6] = (void*)&ctr;
  }
  for (int u = 0; u < kFillUnroll; u++)
    for (int ph = 0; ph < 4; ph++) add((const void*)kb_fill_phase, grid, dim3(kThreads), a_ph[ph]);
  return ce;
}

// A conditional WHILE node (cond set to 1 at each launch of the enclosing graph) in
// graph g after deps; its body graph is returned in *body.
cudaError_t add_fill_loop(cudaGraph_t g, const cudaGraphNode_t* deps, const cudaGraphEdgeData* ed,
                          size_t nd, cudaGraphConditionalHandle* cond, cudaGraphNode_t* node,
                          cudaGraph_t* body) {
  cudaError_t ce = cudaGraphConditionalHandleCreate(cond, g, 1, cudaGraphCondAssignDefault);
  if (ce != cudaSuccess) return ce;
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = *cond;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  ce = cudaGraphAddNode(node, g, deps, ed, nd, &np);
  if (ce == cudaSuccess) *body = np.conditional.phGraph_out[0];
  return ce;
}

int fill_graph(stspix_ctx* ctx, const List& L, cudaGraphExec_t* out) {
  auto key = std::make_pair((const Slot*)L.d, L.B);
  auto it = ctx->fill_graphs.find(key);
  if (it != ctx->fill_graphs.end()) { *out = it->second.exec; return STSPIX_OK; }
  std::lock_guard<std::mutex> lk(g_device_mu);
  cudaGraph_t g = nullptr;
  CK(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle cond;
  cudaGraphNode_t node;
  cudaGraph_t body;
  cudaError_t ce = add_fill_loop(g, nullptr, nullptr, 0, &cond, &node, &body);
  if (ce == cudaSuccess) ce = add_fill_body(ctx, body, L, cond);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(ctx, STSPIX_ERR_CUDA, "fill graph construction failed: %s", cudaGetErrorString(ce));
  }
  cudaGraphExec_t exec = nullptr;
  ce = cudaGraphInstantiate(&exec, g, 0);
  if (ce != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(ctx, STSPIX_ERR_CUDA, "fill graph instantiation failed: %s", cudaGetErrorString(ce));
  }
  ctx->fill_graphs[key] = {g, exec};
  *out = exec;
  return STSPIX_OK;
}

int fill_loop(stspix_ctx* ctx, cudaStream_t st, const List& L);

int run_fill(stspix_ctx* ctx, cudaStream_t st, const List& L) {
  LAUNCHS(kb_fill_begin, L, L.B);
  // the hole list split by parity class
  const unsigned G = (unsigned)std::max(8, std::min(128, 2048 / std::max(L.B, 1)));
  LAUNCHG(kb_fill_split, dim3(G, (unsigned)L.B), kThreads, L.d, 0);
  LAUNCHG(kb_fill_split, dim3(G, (unsigned)L.B), kThreads, L.d, 1);
  int r = fill_loop(ctx, st, L);
  if (r) return r;
  LAUNCHG(kb_fill_end, dim3(G, (unsigned)L.B), kThreads, L.d);
  return STSPIX_OK;
}

// The WHILE loop of the fill (recorded into the running capture, or a cached graph).
int fill_loop(stspix_ctx* ctx, cudaStream_t st, const List& L) {
  if (ctx->capturing) {
    // inside a batch capture: the loop node goes into the graph being captured
    cudaStreamCaptureStatus cs;
    cudaGraph_t cg;
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* ed = nullptr;
    size_t nd = 0;
    CK(cudaStreamGetCaptureInfo(st, &cs, nullptr, &cg, &deps, &ed, &nd));
    cudaGraphConditionalHandle cond;
    cudaGraphNode_t node;
    cudaGraph_t body;
    CK(add_fill_loop(cg, deps, ed, nd, &cond, &node, &body));
    CK(add_fill_body(ctx, body, L, cond));
    CK(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                           cudaStreamSetCaptureDependencies));
    return STSPIX_OK;
  }
  cudaGraphExec_t exec;
  int r = fill_graph(ctx, L, &exec);
  if (r) return r;
  cudaEvent_t pe = prof_begin(ctx, st);
  CK(cudaGraphLaunch(exec, st));
  prof_end(ctx, st, pe, "kb_fill_graph");
  return STSPIX_OK;
}

// shift_and_fill (shift_and_fill.cu:108-339) on the propagated slots.
int shift_fill(stspix_ctx* ctx, cudaStream_t st, const List& L) {
  if (L.B <= 0) return STSPIX_OK;
  int r;
  ctx->cur_fam = STSPIX_FAM_PROP;
  LAUNCHB(kb_prop_clear, pix_units(std::max<long long>(L.max_npix, L.max_nprev)), L, L.B);
  LAUNCHG(kb_flow_pool, dim3(tiles64(L), (unsigned)L.B), kThreads, L.d);
  LAUNCHB(kb_flow_mean, L.max_nprev, L, L.B);
  LAUNCHB(kb_shift, pix_units(L.max_npix), L, L.B);
  LAUNCHB(kb_shift_decode, pix_units(L.max_npix), L, L.B);
  LAUNCHG(kb_count_labels, dim3(tiles64(L), (unsigned)L.B), kThreads, L.d, 0);
  // fill, invalidate disconnected, fill
  if ((r = run_fill(ctx, st, L))) return r;
  LAUNCHG(kb_cc_local, dim3((unsigned)(((L.max_w + 31) / 32) * ((L.max_h + 31) / 32)), (unsigned)L.B),
          kThreads, L.d);
  LAUNCHB(kb_cc_hook, (long long)((L.max_w + 31) / 32) * ((L.max_h + 31) / 32) * (32 + 2 * 31), L, L.B);
  LAUNCHB(kb_cc_compress, pix_units(L.max_npix), L, L.B);
  LAUNCHB(kb_cc_best, pix_units(L.max_npix), L, L.B);
  LAUNCHB(kb_cc_invalidate, pix_units(L.max_npix), L, L.B);
  LAUNCHB(kb_list_holes, pix_units(L.max_npix), L, L.B);
  if ((r = run_fill(ctx, st, L))) return r;
  LAUNCHG(kb_count_labels, dim3(tiles64(L), (unsigned)L.B), kThreads, L.d, 1);
  LAUNCHB(kb_shift_params, L.max_nprev, L, L.B);
  return STSPIX_OK;
}

// run_prop set-up (prop.cu:677-720): write_params + mark_active.
int prop_init(stspix_ctx* ctx, cudaStream_t st, const List& L) {
  if (L.B <= 0) return STSPIX_OK;
  ctx->cur_fam = STSPIX_FAM_OTHER;
  LAUNCHB(kb_write_params, L.max_cap, L, L.B);
  LAUNCHG(kb_mark_active, dim3(tiles64(L), (unsigned)L.B), kThreads, L.d);
  return STSPIX_OK;
}

int read_scalars(stspix_ctx* ctx, cudaStream_t st, int B) {
  CK(cudaMemcpyAsync(ctx->sc_host, ctx->sc, sizeof(Scalars) * (size_t)B, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(ctx->body_iters_host, ctx->body_iters, sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  // kernels launched by the fill graphs: 4 per loop iteration
  ctx->launches += 4 * ((long long)*ctx->body_iters_host - ctx->body_iters_seen);
  ctx->body_iters_seen = *ctx->body_iters_host;
  CK(cudaGetLastError());
  prof_harvest(ctx);
  return STSPIX_OK;
}

void fill_log(stspix_frame_log& log, const Scalars& s, int niters) {
  log.nsplits = s.nsplits;
  log.nmerges = s.nmerges;
  log.nrevived = s.nrevived;
  log.nminted = s.nminted;
  log.near_ties = s.near_ties;
  log.fill_iters = s.fill_iters;
  log.nspix = s.nspix;
  log.niters = niters;
}

struct BatchOut {
  std::vector<int> nspix, niters, status;
  std::vector<stspix_frame_log> log;
};

// A batch's work in two parts (eager, or each recorded into a graph): the head, from
// the table uploads to the BASS initialisation (after it the host may read the hole
// fractions for the 4/8/12 ladder), and the tail, from the propagated initialisation
// to the parameter read-out, for known iteration counts and no partial stop.
int batch_head(stspix_ctx* ctx, cudaStream_t st, int stages, const List& La, const List& Lb,
               const List& Lp) {
  int r;
  if ((r = upload(ctx, st, La, 0)) || (r = upload(ctx, st, Lb, 1)) || (r = upload(ctx, st, Lp, 2)))
    return r;
  ctx->cur_fam = STSPIX_FAM_OTHER;
  LAUNCHS(kb_scalars, La, La.B, (int)kOpBegin);
  if (ctx->lab_ingest) LAUNCHB(kb_lab_ingest, La.max_npix, La, La.B);
  if ((stages & kStageShift) && (r = shift_fill(ctx, st, Lp))) return r;
  return bass_init(ctx, st, Lb);
}

int batch_tail(stspix_ctx* ctx, cudaStream_t st, const List& Lp, const List& Ls, bool ls_own,
               const std::vector<int>& nit_sorted, const stspix_config& cfg) {
  int r;
  if (ls_own && (r = upload(ctx, st, Ls, 3))) return r;
  if ((r = prop_init(ctx, st, Lp))) return r;
  const SmConsts K = sm_constants(cfg);
  if ((r = bass_loop(ctx, st, Ls, nit_sorted, cfg, K, -1, 0))) return r;
  if ((r = compact(ctx, st, Ls))) return r;
  LAUNCHB(kb_read_params, Ls.max_cap, Ls, Ls.B);
  LAUNCHB(kb_save_prev, pix_units(Ls.max_npix), Ls, Ls.B);
  return STSPIX_OK;
}

// Runs body(stream) eagerly, or, from the second occurrence of key on, as a replay of
// the CUDA graph recorded on that occurrence.  body only launches work (no host
// synchronisation, no host decision on device results).
int run_graphed(stspix_ctx* ctx, cudaStream_t st, const std::string& key,
                const std::function<int(cudaStream_t)>& body) {
  int r = STSPIX_OK;
  auto g = ctx->batch_graphs.find(key);
  cudaStreamCaptureStatus outer = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(st, &outer));   // a caller's own capture records the eager step
  // a server whose batch compositions rarely repeat keeps the table of seen
  // signatures bounded: it restarts counting when it grows large
  if (g == ctx->batch_graphs.end() && ctx->batch_seen.size() >= 4096 && !ctx->batch_seen.count(key))
    ctx->batch_seen.clear();
  if (outer != cudaStreamCaptureStatusNone) {
    g = ctx->batch_graphs.end();
  } else if (g == ctx->batch_graphs.end() && ++ctx->batch_seen[key] >= 2 &&
             ((int)ctx->batch_graphs.size() < kMaxBatchGraphs || ctx->batch_seen[key] >= 4)) {
    // a full cache takes only signatures seen four times, in place of the least
    // recently replayed graph (a graph still in flight is freed when it completes)
    if ((int)ctx->batch_graphs.size() >= kMaxBatchGraphs) {
      auto lru = ctx->batch_graphs.begin();
      for (auto it = ctx->batch_graphs.begin(); it != ctx->batch_graphs.end(); ++it)
        if (it->second.last < lru->second.last) lru = it;
      cudaGraphExecDestroy(lru->second.exec);
      cudaGraphDestroy(lru->second.g);
      ctx->batch_graphs.erase(lru);
    }
    // record (the legacy default stream cannot be captured: record on the context's
    // own stream then; nothing runs during a capture, and the graph is launched on
    // the caller's stream)
    std::lock_guard<std::mutex> lk(g_device_mu);
    cudaStream_t cst = st;
    if (st == nullptr || st == cudaStreamLegacy) {
      if (!ctx->cap_stream) CK(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
      cst = ctx->cap_stream;
    }
    const long long l0 = ctx->launches;
    cudaError_t ce = cudaStreamBeginCapture(cst, cudaStreamCaptureModeThreadLocal);
    cudaGraph_t graph = nullptr;
    if (ce == cudaSuccess) {
      ctx->capturing = true;
      r = body(cst);
      ctx->capturing = false;
      ce = cudaStreamEndCapture(cst, &graph);
    }
    cudaGraphExec_t exec = nullptr;
    cudaError_t ie = cudaErrorUnknown;
    if (!r && ce == cudaSuccess) ie = cudaGraphInstantiate(&exec, graph, 0);
    const long long nl = ctx->launches - l0;
    ctx->launches = l0;
    if (!r && ce == cudaSuccess && ie == cudaSuccess) {
      g = ctx->batch_graphs.emplace(key, stspix_ctx::BatchGraph{graph, exec, nl, 0}).first;
    } else {
      // nothing recorded ran: clear the capture error and run this step eagerly;
      // the signature is not captured again
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      ctx->batch_seen[key] = -(1 << 30);
    }
  }
  if (g != ctx->batch_graphs.end()) {
    CK(cudaGraphLaunch(g->second.exec, st));
    g->second.last = ++ctx->graph_tick;
    ctx->launches += g->second.launches;
    ctx->graph_replays++;
    return STSPIX_OK;
  }
  return body(st);
}

// The key of a batch step's launch sequence: everything that sets a launch's grid or
// arguments (the slot records themselves are uploaded by the graph's copy nodes).
std::string batch_signature(const std::vector<FrameDesc>& fr, const std::vector<int>& caps,
                            const std::vector<int>& nit, int stages, const stspix_config& cfg) {
  std::string k((const char*)&cfg, sizeof cfg);
  k.append((const char*)&stages, sizeof stages);
  for (size_t i = 0; i < fr.size(); i++) {
    const int v[7] = {fr[i].slot, fr[i].mode, fr[i].H, fr[i].W, fr[i].sp_size, caps[i], nit[i]};
    k.append((const char*)v, sizeof v);
  }
  return k;
}

// The batch runner.  stages: kStageShift and/or kStageSeg.  Frames are processed
// in workspace positions f.slot (distinct).  Returns a call-level error; per-frame
// statuses land in out.  A batch step whose signature was seen before runs as a
// CUDA graph: captured on the second occurrence (the first ran eagerly and tuned
// the sweeps), replayed from then on.
int run_batch(stspix_ctx* ctx, cudaStream_t st, std::vector<FrameDesc>& fr,
              const stspix_config& cfg, int stages, BatchOut& out, int stop_after = -1,
              int extra_update = 0, int split_dir = 0) {
  const int B = (int)fr.size();
  int r;
  ctx->accumulator = cfg.accumulator;
  ctx->lab_ingest = cfg.lab_ingest ? 1 : 0;
  if ((r = ensure_bcap(ctx, B))) return r;
  std::vector<int> caps(B);
  for (int i = 0; i < B; i++) {
    caps[i] = slot_cap(fr[i]);
    if ((r = ensure_slot(ctx, fr[i].slot, fr[i].H * fr[i].W, caps[i]))) return r;
    if (ctx->lab_ingest && (r = ensure_lab(ctx, fr[i].slot, fr[i].H * fr[i].W))) return r;
  }
  std::vector<Slot> all, bass, prop;
  for (int i = 0; i < B; i++) {
    Slot s = make_slot(ctx, fr[i], caps[i]);
    all.push_back(s);
    (fr[i].mode ? prop : bass).push_back(s);
  }
  List La = make_list(ctx, 0, all);
  List Lb = make_list(ctx, 1, bass);
  List Lp = make_list(ctx, 2, prop);
  out.nspix.assign(B, 0);
  out.niters.assign(B, 0);
  out.status.assign(B, 0);
  out.log.assign(B, stspix_frame_log{});
  // iteration counts: BASS frames cfg.niters; propagated frames the explicit count,
  // cfg.prop_niters, or the 4/8/12 ladder on the hole fraction (pyapi.cu:143-146)
  std::vector<int> nit(B, -1);
  bool need_ladder = false;
  for (int i = 0; i < B; i++) {
    if (!fr[i].mode) nit[i] = cfg.niters;
    else if (fr[i].niters >= 0) nit[i] = fr[i].niters;
    else if (cfg.prop_niters > 0) nit[i] = cfg.prop_niters;
    else need_ladder = true;
  }
  auto finish = [&]() -> int {
    int rr;
    if ((rr = read_scalars(ctx, st, B))) return rr;
    for (int i = 0; i < B; i++) {
      const Scalars& sc = ctx->sc_host[i];
      out.nspix[i] = sc.nspix;
      out.niters[i] = nit[i];
      out.status[i] = sc.status;
      fill_log(out.log[i], sc, nit[i]);
    }
    return STSPIX_OK;
  };
  // the loop table: slots sorted by iteration count, descending (stable)
  auto sort_table = [&](std::vector<int>& nit_sorted, bool* own) {
    std::vector<int> order(B);
    for (int i = 0; i < B; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return nit[a] > nit[b]; });
    std::vector<Slot> sorted;
    for (int i : order) { sorted.push_back(all[i]); nit_sorted.push_back(nit[i]); }
    *own = !std::is_sorted(order.begin(), order.end());
    return *own ? make_list(ctx, 3, sorted) : La;
  };
  // full steps (known or laddered iteration counts) run as head + tail, each replayed
  // as a CUDA graph once its launch sequence repeats
  if ((stages & kStageSeg) && stop_after < 0 && !split_dir && !ctx->prof_on && ctx->graphs_on) {
    const std::string key = batch_signature(fr, caps, nit, stages, cfg);
    r = run_graphed(ctx, st, key + "h",
                    [&](cudaStream_t s) { return batch_head(ctx, s, stages, La, Lb, Lp); });
    if (r) return r;
    if (need_ladder) {
      if ((r = read_scalars(ctx, st, B))) return r;
      for (int i = 0; i < B; i++) {
        if (nit[i] >= 0) continue;
        const int npix = fr[i].H * fr[i].W;
        float iperc = ctx->sc_host[i].ninvalid / (1.0 * npix);
        nit[i] = iperc > 0.20 ? 12 : (iperc < 0.01 ? 4 : 8);
      }
    }
    std::vector<int> nit_sorted;
    bool own = false;
    const List Ls = sort_table(nit_sorted, &own);
    const std::string tkey = need_ladder ? batch_signature(fr, caps, nit, stages, cfg) : key;
    r = run_graphed(ctx, st, tkey + "t", [&](cudaStream_t s) {
      return batch_tail(ctx, s, Lp, Ls, own, nit_sorted, cfg);
    });
    if (r) return r;
    return finish();
  }
  if ((r = upload(ctx, st, La, 0)) || (r = upload(ctx, st, Lb, 1)) || (r = upload(ctx, st, Lp, 2)))
    return r;
  ctx->cur_fam = STSPIX_FAM_OTHER;
  LAUNCHS(kb_scalars, La, B, (int)kOpBegin);
  if ((stages & kStageShift) && (r = shift_fill(ctx, st, Lp))) return r;
  if (!(stages & kStageSeg)) {
    if ((r = read_scalars(ctx, st, B))) return r;
    for (int i = 0; i < B; i++) {
      out.status[i] = ctx->sc_host[i].status;
      fill_log(out.log[i], ctx->sc_host[i], 0);
    }
    return STSPIX_OK;
  }
  if ((r = bass_init(ctx, st, Lb))) return r;
  if (need_ladder) {
    if ((r = read_scalars(ctx, st, B))) return r;
    for (int i = 0; i < B; i++) {
      if (nit[i] >= 0) continue;
      const int npix = fr[i].H * fr[i].W;
      float iperc = ctx->sc_host[i].ninvalid / (1.0 * npix);
      nit[i] = iperc > 0.20 ? 12 : (iperc < 0.01 ? 4 : 8);
    }
  }
  if ((r = prop_init(ctx, st, Lp))) return r;
  std::vector<int> nit_sorted;
  bool own = false;
  const List Ls = sort_table(nit_sorted, &own);
  if (own && (r = upload(ctx, st, Ls, 3))) return r;
  const SmConsts K = sm_constants(cfg);
  if (split_dir) {
    if ((r = split_only(ctx, st, Ls, cfg, K, split_dir))) return r;
  } else if ((r = bass_loop(ctx, st, Ls, nit_sorted, cfg, K, stop_after, extra_update))) {
    return r;
  }
  if (stop_after < 0) {
    if ((r = compact(ctx, st, Ls))) return r;
    LAUNCHB(kb_read_params, Ls.max_cap, Ls, Ls.B);
    LAUNCHB(kb_save_prev, pix_units(Ls.max_npix), Ls, Ls.B);
  }
  return finish();
}

int check_cfg(stspix_ctx* ctx, const stspix_config* cfg) {
  if (!cfg) return fail(ctx, STSPIX_ERR_ARG, "config is NULL");
  if (cfg->accumulator < 0 || cfg->accumulator > 2)
    return fail(ctx, STSPIX_ERR_ARG, "accumulator must be 0, 1 or 2");
  if (cfg->sweep_schedule < 0 || cfg->sweep_schedule > 2)
    return fail(ctx, STSPIX_ERR_ARG, "sweep_schedule must be 0, 1 or 2");
  if (cfg->sweep_tile != 0 && cfg->sweep_tile != 16 && cfg->sweep_tile != 32 && cfg->sweep_tile != 64)
    return fail(ctx, STSPIX_ERR_ARG, "sweep_tile must be 0, 16, 32 or 64");
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

int first_status(stspix_ctx* ctx, const BatchOut& o) {
  for (size_t i = 0; i < o.status.size(); i++)
    if (o.status[i]) return fail(ctx, o.status[i], "device status %d (frame %zu)", o.status[i], i);
  return STSPIX_OK;
}

// Video stream state: label buffer and parameter ping-pong grown to `cap`,
// keeping the current parameters.
int video_ensure(stspix_ctx* ctx, cudaStream_t st, stspix_video* v, int cap) {
  if (v->labels && cap <= v->pp_cap) return STSPIX_OK;
  std::lock_guard<std::mutex> lk(g_device_mu);
  if (!v->labels) AL(v->lbufs, v->labels, (size_t)v->H * v->W);
  if (cap <= v->pp_cap) return STSPIX_OK;
  std::vector<Buf> old = v->pbufs;
  stspix_params oldp = v->pp[v->cur];
  v->pbufs.clear();
  int r;
  for (int i = 0; i < 2; i++)
    if ((r = alloc_params(ctx, v->pbufs, v->pp[i], cap))) return r;
  if (v->n > 0) {
    stspix_params& np = v->pp[v->cur];
    size_t k = (size_t)v->n;
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
  v->pp_cap = cap;
  return STSPIX_OK;
}

// A frame of video v: BASS on its first frame, else shift + propagated BASS.
int video_frame(stspix_ctx* ctx, cudaStream_t st, stspix_video* v, const float* img,
                const float* flow, int sp_size, int* labels_out, int slot, FrameDesc& f) {
  f.img = img;
  f.H = v->H; f.W = v->W;
  f.sp_size = sp_size;
  f.seg = labels_out;
  f.slot = slot;
  f.resident = nullptr;
  int r;
  if (v->n <= 0) {
    f.mode = 0;
    int cap = slot_cap(f);
    if ((r = video_ensure(ctx, st, v, cap))) return r;
    f.pout = v->pp[v->cur];
  } else {
    f.mode = 1;
    f.flow = flow;
    f.prev = v->labels;
    f.n_prev = v->n;
    int cap = slot_cap(f);
    if ((r = video_ensure(ctx, st, v, cap))) return r;
    f.pprev = v->pp[v->cur];
    f.pout = v->pp[1 - v->cur];
  }
  f.resident = v->labels;
  return STSPIX_OK;
}

void video_commit(stspix_video* v, int mode, int nspix) {
  if (mode) v->cur = 1 - v->cur;
  v->n = nspix;
  v->frames++;
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
  c->accumulator = 0;
  c->sweep_schedule = 0;
  c->sweep_tile = 0;
  c->sweep_queue = 0;
}

int stspix_version(void) { return 2; }

int stspix_create(stspix_ctx** out, int device) {
  if (!out) return STSPIX_ERR_ARG;
  *out = nullptr;
  stspix_ctx* ctx = new (std::nothrow) stspix_ctx();
  if (!ctx) return STSPIX_ERR_NOMEM;
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete ctx; return STSPIX_ERR_CUDA; }
  {
    std::lock_guard<std::mutex> lk(g_device_mu);
    preload_kernels();
  }
  if (g_preload_err != cudaSuccess) { delete ctx; return STSPIX_ERR_CUDA; }
  cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaFuncSetAttribute((const void*)kb_split_bfs_big,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, kBfsBigSmem) != cudaSuccess) {
    delete ctx;
    return STSPIX_ERR_CUDA;
  }
  // slot tables for 256 frames per batch from the start: they never move for
  // batches up to that size, so the graphs that point at them stay valid
  if (ensure_bcap(ctx, 256) != STSPIX_OK || cudaMalloc(&ctx->body_iters, 4 * sizeof(int)) != cudaSuccess ||
      cudaMallocHost(&ctx->body_iters_host, sizeof(int)) != cudaSuccess) {
    delete ctx;
    return STSPIX_ERR_NOMEM;
  }
  cudaMemset(ctx->body_iters, 0, 4 * sizeof(int));
  cudaEventCreate(&ctx->batch_ev[0]);
  cudaEventCreate(&ctx->batch_ev[1]);
  for (auto& e : ctx->tune_ev) cudaEventCreate(&e);
  cudaDeviceSynchronize();
  *out = ctx;
  return STSPIX_OK;
}

int stspix_destroy(stspix_ctx* ctx) {
  if (!ctx) return STSPIX_OK;
  if (ctx->fwd) stspix_video_destroy(ctx->fwd);
  std::lock_guard<std::mutex> lk(g_device_mu);
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  for (auto& w : ctx->work) { free_list(w.pix); free_list(w.sp); free_list(w.lab); }
  drop_fill_graphs(ctx);
  free_list(ctx->ctl_bufs);
  cudaFree(ctx->body_iters);
  for (auto e : ctx->tune_ev) if (e) cudaEventDestroy(e);
  if (ctx->body_iters_host) cudaFreeHost(ctx->body_iters_host);
  prof_harvest(ctx);
  for (auto& e : ctx->frame_ev) { ctx->ev_free.push_back(e.a); ctx->ev_free.push_back(e.b); }
  for (auto e : ctx->ev_free) cudaEventDestroy(e);
  for (auto e : ctx->batch_ev) if (e) cudaEventDestroy(e);
  if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
  if (ctx->sc_host) cudaFreeHost(ctx->sc_host);
  if (ctx->h_slots) cudaFreeHost(ctx->h_slots);
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
  std::vector<FrameDesc> fr(1);
  FrameDesc& f = fr[0];
  f.img = img; f.H = H; f.W = W; f.sp_size = cfg->sp_size; f.seg = labels_out; f.mode = 0;
  if (params_out) f.pout = *params_out;
  BatchOut o;
  if ((r = run_batch(ctx, st, fr, *cfg, kStageSeg, o))) return r;
  ctx->log = o.log[0];
  if (nspix_out) *nspix_out = o.nspix[0];
  if (params_out && params_out->capacity < o.nspix[0])
    return fail(ctx, STSPIX_ERR_CAPACITY, "params capacity %d < %d superpixels",
                params_out->capacity, o.nspix[0]);
  return first_status(ctx, o);
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
  std::vector<FrameDesc> fr(1);
  FrameDesc& f = fr[0];
  f.img = img; f.H = H; f.W = W; f.sp_size = cfg->sp_size; f.seg = labels_out; f.mode = 0;
  BatchOut o;
  if ((r = run_batch(ctx, st, fr, *cfg, kStageSeg, o, iters < 0 ? 0 : iters, extra_update)))
    return r;
  if (dump) {
    LAUNCH(k_dump_state, ctx->work[0].s.sp.cap, ctx->work[0].s.sp, *dump);
    CK(cudaStreamSynchronize(st));
  }
  if (nbuf_out) {
    double Hh, w;
    int nx, ny;
    hex_geometry(cfg->sp_size, W, H, &Hh, &w, &nx, &ny);
    *nbuf_out = 30 * nx * ny;
  }
  if (max_spix_out) *max_spix_out = ctx->sc_host[0].max_spix;
  return ctx->sc_host[0].status;
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
  std::vector<FrameDesc> fr(1);
  FrameDesc& f = fr[0];
  f.H = H; f.W = W; f.sp_size = 15; f.seg = filled_out; f.mode = 1; f.prev = labels_prev;
  f.n_prev = n_prev; f.flow = flow; f.pprev = *params_prev; f.shifted = shifted_out;
  stspix_config cfg;
  stspix_default_config(&cfg);
  BatchOut o;
  if ((r = run_batch(ctx, st, fr, cfg, kStageShift, o))) return r;
  ctx->log = o.log[0];
  return first_status(ctx, o);
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
  std::vector<FrameDesc> fr(1);
  FrameDesc& f = fr[0];
  f.img = img; f.H = H; f.W = W; f.sp_size = cfg->sp_size; f.seg = labels_out; f.mode = 1;
  f.n_prev = n_prev; f.pprev = *params_prev; f.shifted = const_cast<int*>(shifted);
  f.niters = niters < 0 ? 0 : niters;
  if (params_out) f.pout = *params_out;
  BatchOut o;
  if ((r = run_batch(ctx, st, fr, *cfg, kStageSeg, o))) return r;
  ctx->log = o.log[0];
  if (nspix_out) *nspix_out = o.nspix[0];
  if (params_out && params_out->capacity < o.nspix[0])
    return fail(ctx, STSPIX_ERR_CAPACITY, "params capacity %d < %d superpixels",
                params_out->capacity, o.nspix[0]);
  return first_status(ctx, o);
}

// run_split_py (prop/bass.cu:389-506): legacy direction 0 splits in direction 2, any
// other value in direction 1 (count parity, prop/split_merge.cu:41-43).
int stspix_legacy_split(stspix_ctx* ctx, void* stream, const float* img, int H, int W,
                        const stspix_config* cfg, int direction, const int32_t* spix,
                        const stspix_params* params_prev, int n_prev, int32_t* labels_out,
                        stspix_params* params_out, int* nspix_out) {
  if (!ctx || !img || !spix || !params_prev || !labels_out || n_prev < 1)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r;
  if ((r = check_cfg(ctx, cfg)) || (r = check_size(ctx, H, W))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  CK(cudaMemcpyAsync(labels_out, spix, sizeof(int) * (size_t)H * W, cudaMemcpyDeviceToDevice, st));
  std::vector<FrameDesc> fr(1);
  FrameDesc& f = fr[0];
  f.img = img; f.H = H; f.W = W; f.sp_size = cfg->sp_size; f.seg = labels_out; f.mode = 1;
  f.n_prev = n_prev; f.pprev = *params_prev; f.shifted = const_cast<int*>(spix);
  f.niters = 0;
  if (params_out) f.pout = *params_out;
  BatchOut o;
  if ((r = run_batch(ctx, st, fr, *cfg, kStageSeg, o, -1, 0, direction == 0 ? 2 : 1))) return r;
  ctx->log = o.log[0];
  if (nspix_out) *nspix_out = o.nspix[0];
  if (params_out && params_out->capacity < o.nspix[0])
    return fail(ctx, STSPIX_ERR_CAPACITY, "params capacity %d < %d superpixels",
                params_out->capacity, o.nspix[0]);
  return first_status(ctx, o);
}

// main_loop (pyapi.cu:46-195).  Video mode: frame by frame through one resident
// stream state (each frame needs the previous one).  Image mode: the frames are
// independent and run as batches.
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
  int status = STSPIX_OK;
  for (auto& e : ctx->frame_ev) { ctx->ev_free.push_back(e.a); ctx->ev_free.push_back(e.b); }
  ctx->frame_ev.clear();
  ctx->frame_ms.clear();
  if (video_mode) {
    if (ctx->fwd && (ctx->fwd->H != H || ctx->fwd->W != W)) {
      stspix_video_destroy(ctx->fwd);
      ctx->fwd = nullptr;
    }
    if (!ctx->fwd && (r = stspix_video_create(ctx, &ctx->fwd, H, W))) return r;
    stspix_video_reset(ctx->fwd);
    for (int fi = 0; fi < T; fi++) {
      cudaEvent_t fe0 = ev_get(ctx), fe1 = ev_get(ctx);
      cudaEventRecord(fe0, st);
      std::vector<FrameDesc> fr(1);
      const float* flow = fi > 0 ? flows + (size_t)(fi - 1) * npix * 2 : nullptr;
      if ((r = video_frame(ctx, st, ctx->fwd, vid + (size_t)fi * npix * 3, flow, cfg->sp_size,
                           spix_out + (size_t)fi * npix, 0, fr[0])))
        return r;
      BatchOut o;
      if ((r = run_batch(ctx, st, fr, *cfg, kStageShift | kStageSeg, o))) return r;
      video_commit(ctx->fwd, fr[0].mode, o.nspix[0]);
      if (o.status[0] && !status) status = o.status[0];
      ctx->log = o.log[0];
      cudaEventRecord(fe1, st);
      ctx->frame_ev.push_back({fe0, fe1, 1});
    }
  } else {
    // independent frames: batches sized to keep the workspaces near 4 GiB
    long long vb = 0, sb = 0;
    stspix_footprint(H, W, cfg->sp_size, &vb, &sb);
    int per = (int)std::max(1LL, std::min<long long>(64, (4LL << 30) / std::max(sb, 1LL)));
    for (int f0 = 0; f0 < T; f0 += per) {
      int nb = std::min(per, T - f0);
      cudaEvent_t fe0 = ev_get(ctx), fe1 = ev_get(ctx);
      cudaEventRecord(fe0, st);
      std::vector<FrameDesc> fr(nb);
      for (int i = 0; i < nb; i++) {
        FrameDesc& f = fr[i];
        f.img = vid + (size_t)(f0 + i) * npix * 3;
        f.H = H; f.W = W; f.sp_size = cfg->sp_size;
        f.seg = spix_out + (size_t)(f0 + i) * npix;
        f.mode = 0;
        f.slot = i;
      }
      BatchOut o;
      if ((r = run_batch(ctx, st, fr, *cfg, kStageSeg, o))) return r;
      for (int i = 0; i < nb; i++)
        if (o.status[i] && !status) status = o.status[i];
      ctx->log = o.log[nb - 1];
      cudaEventRecord(fe1, st);
      ctx->frame_ev.push_back({fe0, fe1, nb});
    }
  }
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  prof_harvest(ctx);
  // per-frame times; the frames of one image-mode batch share its time equally
  for (auto& e : ctx->frame_ev) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e.a, e.b);
    for (int i = 0; i < e.n; i++) ctx->frame_ms.push_back(ms / e.n);
  }
  return status ? fail(ctx, status, "device status %d", status) : STSPIX_OK;
}

int stspix_video_create(stspix_ctx* ctx, stspix_video** out, int H, int W) {
  if (!ctx || !out) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r = check_size(ctx, H, W);
  if (r) return r;
  stspix_video* v = new (std::nothrow) stspix_video();
  if (!v) return fail(ctx, STSPIX_ERR_NOMEM, "host allocation failed");
  v->ctx = ctx;
  v->H = H;
  v->W = W;
  std::lock_guard<std::mutex> lk(g_device_mu);
  cudaSetDevice(ctx->device);
  if ((r = alloc(ctx, v->lbufs, &v->labels, (size_t)H * W))) { delete v; return r; }
  *out = v;
  return STSPIX_OK;
}

int stspix_video_destroy(stspix_video* v) {
  if (!v) return STSPIX_OK;
  std::lock_guard<std::mutex> lk(g_device_mu);
  cudaSetDevice(v->ctx->device);
  cudaDeviceSynchronize();
  free_list(v->lbufs);
  free_list(v->pbufs);
  delete v;
  return STSPIX_OK;
}

int stspix_video_reset(stspix_video* v) {
  if (!v) return STSPIX_ERR_ARG;
  v->n = 0;
  v->cur = 0;
  v->frames = 0;
  return STSPIX_OK;
}

namespace {
// Parameter arrays of stspix_params in declaration order: element bytes x count per id.
struct ParamField { size_t elem; int per; };
const ParamField kParamFields[13] = {{4, 3}, {4, 3}, {8, 2}, {8, 3}, {4, 1}, {8, 2}, {8, 3},
                                     {8, 3}, {4, 1}, {4, 1}, {4, 1}, {4, 1}, {4, 1}};
void* param_ptr(const stspix_params& p, int i) {
  void* f[13] = {p.mu_app, p.prior_mu_app, p.mu_shape, p.sigma_shape, p.logdet_sigma_shape,
                 p.prior_mu_shape, p.prior_sigma_shape, p.sample_sigma_shape, p.counts,
                 p.sm_counts, p.prior_counts, p.ids, p.invalid_counts};
  return f[i];
}
struct SnapHeader {
  char magic[8];
  int version, H, W, n;
  long long frames;
  char pad[32];
};
static_assert(sizeof(SnapHeader) == 64, "snapshot header is 64 bytes");
long long snap_bytes(int H, int W, int n) {
  long long b = (long long)sizeof(SnapHeader) + 4LL * H * W;
  for (const auto& f : kParamFields) b += (long long)f.elem * f.per * n;
  return b;
}
}  // namespace

int stspix_video_save(stspix_video* v, void* stream, void* host, long long capacity,
                      long long* bytes) {
  if (!v || !bytes) return STSPIX_ERR_ARG;
  stspix_ctx* ctx = v->ctx;
  const long long need = snap_bytes(v->H, v->W, v->n);
  *bytes = need;
  if (!host || capacity < need) return STSPIX_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  SnapHeader h{};
  memcpy(h.magic, "SPXVIDEO", 8);
  h.version = 1; h.H = v->H; h.W = v->W; h.n = v->n; h.frames = v->frames;
  char* out = (char*)host;
  memcpy(out, &h, sizeof h);
  out += sizeof h;
  const size_t npix = (size_t)v->H * v->W;
  if (v->labels) CK(cudaMemcpyAsync(out, v->labels, 4 * npix, cudaMemcpyDeviceToHost, st));
  else memset(out, 0xff, 4 * npix);
  out += 4 * npix;
  for (int i = 0; i < 13; i++) {
    const size_t b = kParamFields[i].elem * kParamFields[i].per * (size_t)v->n;
    if (b) CK(cudaMemcpyAsync(out, param_ptr(v->pp[v->cur], i), b, cudaMemcpyDeviceToHost, st));
    out += b;
  }
  CK(cudaStreamSynchronize(st));
  return STSPIX_OK;
}

int stspix_video_load(stspix_video* v, void* stream, const void* host, long long bytes) {
  if (!v || !host) return STSPIX_ERR_ARG;
  stspix_ctx* ctx = v->ctx;
  SnapHeader h;
  if (bytes < (long long)sizeof h) return fail(ctx, STSPIX_ERR_ARG, "snapshot too short");
  memcpy(&h, host, sizeof h);
  if (memcmp(h.magic, "SPXVIDEO", 8) != 0 || h.version != 1)
    return fail(ctx, STSPIX_ERR_ARG, "not a version-1 video snapshot");
  if (h.H != v->H || h.W != v->W)
    return fail(ctx, STSPIX_ERR_ARG, "snapshot of a %dx%d video for a %dx%d video", h.H, h.W,
                v->H, v->W);
  if (h.n < 0 || bytes < snap_bytes(h.H, h.W, h.n))
    return fail(ctx, STSPIX_ERR_ARG, "snapshot truncated");
  if (h.frames > 0) {
    // later propagation and statistics kernels index the parameter arrays by these
    // labels, so a corrupt or mismatched snapshot is refused before anything is copied
    const int32_t* lab = (const int32_t*)((const char*)host + sizeof h);
    const size_t np = (size_t)h.H * h.W;
    for (size_t i = 0; i < np; i++) {
      int32_t l;
      memcpy(&l, lab + i, 4);
      if (l < -1 || l >= h.n)
        return fail(ctx, STSPIX_ERR_ARG, "snapshot label %d at pixel %zu outside [-1, %d)", l, i,
                    h.n);
    }
  }
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  v->n = 0;  // nothing to keep while growing
  int r;
  if ((r = video_ensure(ctx, st, v, std::max(10 * h.n + 2, 64)))) return r;
  v->cur = 0;
  const char* in = (const char*)host + sizeof h;
  const size_t npix = (size_t)v->H * v->W;
  CK(cudaMemcpyAsync(v->labels, in, 4 * npix, cudaMemcpyHostToDevice, st));
  in += 4 * npix;
  for (int i = 0; i < 13; i++) {
    const size_t b = kParamFields[i].elem * kParamFields[i].per * (size_t)h.n;
    if (b) CK(cudaMemcpyAsync(param_ptr(v->pp[0], i), in, b, cudaMemcpyHostToDevice, st));
    in += b;
  }
  CK(cudaStreamSynchronize(st));
  v->n = h.n;
  v->frames = h.frames;
  return STSPIX_OK;
}

int stspix_video_nspix(const stspix_video* v) { return v ? v->n : -1; }
long long stspix_video_frames(const stspix_video* v) { return v ? v->frames : -1; }

int stspix_process_batch(stspix_ctx* ctx, void* stream, stspix_frame* frames, int n,
                         const stspix_config* cfg) {
  if (!ctx || (!frames && n > 0) || n < 0) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r;
  if ((r = check_cfg(ctx, cfg))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<FrameDesc> fr(n);
  for (int i = 0; i < n; i++) {
    stspix_frame& F = frames[i];
    if (!F.img || !F.labels_out) return fail(ctx, STSPIX_ERR_ARG, "frame %d: null pointer", i);
    if (F.sp_size < 0) return fail(ctx, STSPIX_ERR_ARG, "frame %d: sp_size < 0", i);
    const int sp = F.sp_size > 0 ? F.sp_size : cfg->sp_size;
    if (F.video) {
      if (F.video->ctx->device != ctx->device)
        return fail(ctx, STSPIX_ERR_ARG, "frame %d: video on another device", i);
      if (F.H != F.video->H || F.W != F.video->W)
        return fail(ctx, STSPIX_ERR_ARG, "frame %d: %dx%d frame for a %dx%d video", i, F.H, F.W,
                    F.video->H, F.video->W);
      for (int j = 0; j < i; j++)
        if (frames[j].video == F.video)
          return fail(ctx, STSPIX_ERR_ARG, "frames %d and %d continue the same video", j, i);
      if (F.video->n > 0 && !F.flow) return fail(ctx, STSPIX_ERR_ARG, "frame %d: flow required", i);
      if ((r = check_size(ctx, F.H, F.W))) return r;
      if ((r = video_frame(ctx, st, F.video, F.img, F.flow, sp, F.labels_out, i, fr[i]))) return r;
    } else {
      if ((r = check_size(ctx, F.H, F.W))) return r;
      FrameDesc& f = fr[i];
      f.img = F.img; f.H = F.H; f.W = F.W; f.sp_size = sp; f.seg = F.labels_out; f.mode = 0;
      f.slot = i;
    }
  }
  cudaEventRecord(ctx->batch_ev[0], st);
  BatchOut o;
  if ((r = run_batch(ctx, st, fr, *cfg, kStageShift | kStageSeg, o))) return r;
  cudaEventRecord(ctx->batch_ev[1], st);
  CK(cudaEventSynchronize(ctx->batch_ev[1]));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->batch_ev[0], ctx->batch_ev[1]);
  ctx->batch_ms = ms;
  for (int i = 0; i < n; i++) {
    if (frames[i].video) video_commit(frames[i].video, fr[i].mode, o.nspix[i]);
    frames[i].nspix = o.nspix[i];
    frames[i].niters = o.niters[i];
    frames[i].status = o.status[i];
    frames[i].log = o.log[i];
  }
  if (n > 0) ctx->log = o.log[n - 1];
  return first_status(ctx, o);
}

int stspix_footprint(int H, int W, int sp_size, long long* video_bytes, long long* slot_bytes) {
  if (H < 1 || W < 1 || sp_size < 1) return STSPIX_ERR_ARG;
  double Hh, w;
  int nx, ny;
  hex_geometry(sp_size, W, H, &Hh, &w, &nx, &ny);
  const long long npix = (long long)H * W;
  const long long cap = std::max(30LL * nx * ny, 64LL);
  if (video_bytes) *video_bytes = 4 * npix + 2 * kParamBytes * cap;
  if (slot_bytes)
    *slot_bytes = kPixBytes * npix + (2 * kSpDevBytes + kSmBytes + kAuxBytes) * (cap + 2);
  return STSPIX_OK;
}

double stspix_last_batch_ms(const stspix_ctx* ctx) { return ctx ? ctx->batch_ms : -1.0; }

long long stspix_graph_replays(const stspix_ctx* ctx) { return ctx ? ctx->graph_replays : -1; }

int stspix_sweep_choice(const stspix_ctx* ctx, int idx, int* tiles_class, int* single_w,
                        int* pair_w) {
  if (!ctx || idx < 0) return 0;
  for (const auto& kv : ctx->sweep_choice) {
    if (kv.first.second != 0 || idx-- > 0) continue;   // autotuned entries only
    const int v1 = kv.second & 0xff, v2 = (kv.second >> 8) - 1;
    if (tiles_class) *tiles_class = (int)kv.first.first;
    if (single_w) *single_w = kSweepTileW[v1];
    if (pair_w) *pair_w = v2 >= 0 ? kSweepTileW[v2] : 0;
    return 1;
  }
  return 0;
}

int stspix_set_batch_graphs(stspix_ctx* ctx, int enable) {
  if (!ctx) return STSPIX_ERR_ARG;
  ctx->graphs_on = enable != 0;
  return STSPIX_OK;
}

int stspix_rgb2lab(stspix_ctx* ctx, void* stream, const float* rgb, float* lab,
                   long long npix) {
  if (!ctx || !rgb || !lab || npix < 0) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  LAUNCH(k_rgb2lab, npix, rgb, lab, npix, 1);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_lab2rgb(stspix_ctx* ctx, void* stream, const float* lab, float* rgb,
                   long long npix) {
  if (!ctx || !rgb || !lab || npix < 0) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  LAUNCH(k_lab2rgb, npix, lab, rgb, npix);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_rescale_u8(stspix_ctx* ctx, void* stream, const uint8_t* in, float* out,
                      long long nvals, float scale) {
  if (!ctx || !in || !out || nvals < 0 || !(scale != 0.f))
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  LAUNCH(k_rescale_u8, nvals, in, out, nvals, scale);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_label_stats(stspix_ctx* ctx, void* stream, const float* img, const int32_t* labels,
                       int H, int W, int nlabels, int accumulator, double* out) {
  if (!ctx || !img || !labels || !out || nlabels < 1 || accumulator < 0 || accumulator > 2)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r;
  if ((r = check_size(ctx, H, W))) return r;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n7 = 7 * (size_t)nlabels;
  long long* iacc = nullptr;
  float* facc = nullptr;
  double* dacc = nullptr;
  CK(cudaMallocAsync((void**)&iacc, sizeof(long long) * n7, st));
  CK(cudaMallocAsync((void**)&facc, sizeof(float) * n7, st));
  CK(cudaMallocAsync((void**)&dacc, sizeof(double) * n7, st));
  CK(cudaMemsetAsync(iacc, 0, sizeof(long long) * n7, st));
  CK(cudaMemsetAsync(facc, 0, sizeof(float) * n7, st));
  CK(cudaMemsetAsync(dacc, 0, sizeof(double) * n7, st));
  const long long npix = (long long)H * W;
  LAUNCH(k_label_stats, npix, img, labels, npix, nlabels, accumulator, iacc, facc, dacc);
  LAUNCH(k_label_stats_out, nlabels, nlabels, accumulator, iacc, facc, dacc, out);
  CK(cudaFreeAsync(iacc, st));
  CK(cudaFreeAsync(facc, st));
  CK(cudaFreeAsync(dacc, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  return STSPIX_OK;
}

// ---- quality metrics (evaluate.py) ------------------------------------------------
namespace {
// Scratch of one evaluation, carved from one allocation (256-byte aligned pieces).
struct QualityScratch {
  int* cnt;                    // [T*S]   per-frame id sizes
  double* fsum;                // [T*S*3] per-frame id colour sums
  double* vsum;                // [S*3]   video-wide id colour sums
  double* msum;                // [T*3]   per-frame colour sums
  double* pix2;                // [T]     sum (v - mean)^2
  double* pix2s;               // [T]     the same at x255 scale
  double* sse;                 // [T]     sum (v - pooled)^2
  double* pool2;               // [T]     sum (pooled - mean)^2, per-frame pooling
  double* pool3;               // [T]     the same, video pooling at x255
  unsigned long long* live;    // [T]     ids alive per frame
  long long* ntot;             // [S]     total size over the video
  double* stdv;                // [S]     size std over the frames alive (-1: < 2)
  int* J;                      // [T*S*G1] id x ground-truth overlaps
  unsigned long long *ue, *sa, *gsize;   // [T*G1]
  unsigned long long *ue3, *sa3;         // [G1]
  size_t bytes;
};

QualityScratch quality_layout(char* base, long long T, long long S, long long G1, bool colour,
                              bool gt) {
  QualityScratch q{};
  size_t off = 0;
  auto take = [&](size_t n) -> char* {
    char* p = base ? base + off : nullptr;
    off += (n + 255) & ~size_t(255);
    return p;
  };
  q.cnt = (int*)take(4 * T * S);
  q.live = (unsigned long long*)take(8 * T);
  q.ntot = (long long*)take(8 * S);
  q.stdv = (double*)take(8 * S);
  if (colour) {
    q.fsum = (double*)take(24 * T * S);
    q.vsum = (double*)take(24 * S);
    q.msum = (double*)take(24 * T);
    q.pix2 = (double*)take(8 * T);
    q.pix2s = (double*)take(8 * T);
    q.sse = (double*)take(8 * T);
    q.pool2 = (double*)take(8 * T);
    q.pool3 = (double*)take(8 * T);
  }
  if (gt) {
    q.J = (int*)take(4 * T * S * G1);
    q.ue = (unsigned long long*)take(8 * T * G1);
    q.sa = (unsigned long long*)take(8 * T * G1);
    q.gsize = (unsigned long long*)take(8 * T * G1);
    q.ue3 = (unsigned long long*)take(8 * G1);
    q.sa3 = (unsigned long long*)take(8 * G1);
  }
  q.bytes = off;
  return q;
}

constexpr size_t kQualityMaxScratch = size_t(64) << 30;

int label_range(stspix_ctx* ctx, cudaStream_t st, const int32_t* a, long long n, int out[2]) {
  int* mm = nullptr;
  CK(cudaMallocAsync((void**)&mm, 2 * sizeof(int), st));
  LAUNCHG(k_q_range_init, 1, 32, mm);
  const long long nb = std::min<long long>((n + kThreads - 1) / kThreads, 4LL * ctx->num_sms);
  LAUNCHG(k_q_range, (unsigned)std::max(1LL, nb), kThreads, a, n, mm);
  CK(cudaMemcpyAsync(out, mm, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
  CK(cudaFreeAsync(mm, st));
  CK(cudaStreamSynchronize(st));
  return STSPIX_OK;
}

// tex / szv from the per-frame live counts and per-id stds (evaluate.py:287-327).
void size_scores(const std::vector<unsigned long long>& live, const std::vector<double>& stdv,
                 int T, long long S, double* tex, double* szv) {
  double a = 0;
  for (int t = 0; t < T; t++) a += (double)live[t] / (double)S;
  *tex = a / T;
  double s = 0;
  long long n = 0;
  for (long long k = 0; k < S; k++)
    if (stdv[k] >= 0) { s += stdv[k]; n++; }
  *szv = n ? s / n : std::nan("");
}

unsigned q_blocks(long long n) { return (unsigned)std::max(1LL, (n + kThreads - 1) / kThreads); }
}  // namespace

int stspix_label_range(stspix_ctx* ctx, void* stream, const int32_t* labels, long long n,
                       int32_t* out) {
  if (!ctx || !labels || !out || n < 1) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  int mm[2];
  int r = label_range(ctx, st, labels, n, mm);
  if (r) return r;
  out[0] = mm[0];
  out[1] = mm[1];
  return STSPIX_OK;
}

int stspix_count_spix(stspix_ctx* ctx, void* stream, const int32_t* spix, int T, long long npix,
                      int32_t id_offset, int nids, int32_t* counts) {
  if (!ctx || !spix || !counts || T < 1 || npix < 1 || npix > INT_MAX || nids < 1 || T > 65535)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  int mm[2];
  int r = label_range(ctx, st, spix, (long long)T * npix, mm);
  if (r) return r;
  if (mm[0] < id_offset || (long long)mm[1] >= (long long)id_offset + nids)
    return fail(ctx, STSPIX_ERR_ARG, "ids %d..%d outside [%d, %lld)", mm[0], mm[1], id_offset,
                (long long)id_offset + nids);
  CK(cudaMemsetAsync(counts, 0, sizeof(int32_t) * (size_t)T * nids, st));
  const long long segs = (long long)T * ((npix + 31) / 32);
  const unsigned nb = (unsigned)std::max(1LL, std::min<long long>((segs + 7) / 8, 8LL * ctx->num_sms));
  LAUNCHG(k_q_accum, nb, kThreads, nullptr, spix, nullptr, T, 1, (int)npix, id_offset, nids, 1,
          counts, nullptr, nullptr, nullptr, nullptr);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_size_variation(stspix_ctx* ctx, void* stream, const int32_t* counts, int T, int S,
                          double* tex, double* szv, double* ave_nsp) {
  if (!ctx || !counts || !tex || !szv || T < 1 || S < 1 || T > 65535)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  QualityScratch q = quality_layout(nullptr, T, S, 1, false, false);
  char* base = nullptr;
  CK(cudaMallocAsync((void**)&base, q.bytes, st));
  q = quality_layout(base, T, S, 1, false, false);
  CK(cudaMemsetAsync(base, 0, q.bytes, st));
  LAUNCHG(k_q_id_time, q_blocks(S), kThreads, counts, T, S, q.ntot, q.stdv);
  LAUNCHG(k_q_frame_ids, dim3(q_blocks(S), T), kThreads, counts, nullptr, nullptr, q.ntot,
          nullptr, S, 1, q.live, nullptr, nullptr);
  std::vector<unsigned long long> live(T);
  std::vector<double> stdv(S);
  CK(cudaMemcpyAsync(live.data(), q.live, 8 * (size_t)T, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(stdv.data(), q.stdv, 8 * (size_t)S, cudaMemcpyDeviceToHost, st));
  CK(cudaFreeAsync(base, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());
  size_scores(live, stdv, T, S, tex, szv);
  if (ave_nsp) {
    double a = 0;
    for (int t = 0; t < T; t++) a += (double)live[t];
    *ave_nsp = a / T;
  }
  return STSPIX_OK;
}

int stspix_sp_pooling(stspix_ctx* ctx, void* stream, const float* vid, const int32_t* spix,
                      int T, int H, int W, int nids, float* pooled, float* down) {
  if (!ctx || !vid || !spix || !down || T < 1 || H < 1 || W < 1 || nids < 1 || T > 65535 ||
      (long long)H * W > INT_MAX)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long npix = (long long)H * W, n = T * npix, TS = (long long)T * nids;
  int mm[2];
  int r = label_range(ctx, st, spix, n, mm);
  if (r) return r;
  if (mm[0] < 0 || mm[1] >= nids)
    return fail(ctx, STSPIX_ERR_ARG, "ids %d..%d outside [0, %d)", mm[0], mm[1], nids);
  // counts, per-frame id sums, and the video-wide id / per-frame sums that the
  // accumulation pass also produces
  const size_t cbytes = (4 * (size_t)TS + 255) & ~size_t(255);
  const size_t bytes = cbytes + 24 * ((size_t)TS + nids + T);
  char* base = nullptr;
  CK(cudaMallocAsync((void**)&base, bytes, st));
  CK(cudaMemsetAsync(base, 0, bytes, st));
  int* cnt = (int*)base;
  double* fsum = (double*)(base + cbytes);
  double* vsum = fsum + 3 * (size_t)TS;
  double* msum = vsum + 3 * (size_t)nids;
  const long long segs = (long long)T * H * ((W + 31) / 32);
  const unsigned nb = (unsigned)std::max(1LL, std::min<long long>((segs + 7) / 8, 8LL * ctx->num_sms));
  LAUNCHG(k_q_accum, nb, kThreads, vid, spix, nullptr, T, H, W, 0, nids, 1, cnt, fsum, vsum, msum,
          nullptr);
  LAUNCHG(k_q_down, q_blocks(TS), kThreads, cnt, fsum, TS, down);
  if (pooled)
    LAUNCHG(k_q_pool_write, q_blocks(n), kThreads, spix, (int)npix, 0, nids, n, down, pooled);
  CK(cudaFreeAsync(base, st));
  CK(cudaGetLastError());
  return STSPIX_OK;
}

// ---- legacy prop_cuda surface (st_spix/csrc/prop) -----------------------------------
int stspix_legacy_shift_labels(stspix_ctx* ctx, void* stream, const int32_t* spix,
                               const int32_t* flow, int nspix, int H, int W, int32_t* shifted,
                               int32_t* counts) {
  if (!ctx || !spix || !flow || !shifted || !counts || nspix < 0 || H < 1 || W < 1 ||
      (long long)H * W > INT_MAX)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = (long long)H * W;
  LAUNCH(k_fill_i32, n, shifted, n, -1);
  CK(cudaMemsetAsync(counts, 0, sizeof(int32_t) * (size_t)n, st));
  LAUNCH(k_lshift, n, spix, flow, nspix, H, W, shifted, counts);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_legacy_fill_missing(stspix_ctx* ctx, void* stream, int32_t* spix, const float* centers,
                               int ncenters, const int32_t* missing, int nmissing, int H, int W,
                               int break_iter, int* iters, int* remaining) {
  if (!ctx || !spix || (nmissing > 0 && (!missing || !centers)) || nmissing < 0 || ncenters < 0 ||
      H < 1 || W < 1 || (long long)H * W > INT_MAX)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  if (iters) *iters = 0;
  if (remaining) *remaining = 0;
  if (nmissing == 0) return STSPIX_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* border = nullptr;
  int* num_neg = nullptr;
  CK(cudaMallocAsync((void**)&border, (size_t)nmissing, st));
  CK(cudaMallocAsync((void**)&num_neg, sizeof(int), st));
  // fill_missing (prop/fill_missing.cu:26-90): count the listed pixels still missing
  // (and mark the border), four parity phases; stop when a count is 0, repeats the
  // previous one (starting from 1), or break_iter iterations ran.
  int neg = 1, prev = 1, it = 0;
  auto count_border = [&]() -> int {
    CK(cudaMemsetAsync(num_neg, 0, sizeof(int), st));
    LAUNCH(k_lfill_border, nmissing, spix, missing, nmissing, H, W, border, num_neg);
    CK(cudaMemcpyAsync(&neg, num_neg, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    return STSPIX_OK;
  };
  int r;
  while (neg > 0) {
    if (break_iter > 0 && it >= break_iter) break;
    if ((r = count_border())) return r;
    for (int xm = 0; xm < 2; xm++)
      for (int ym = 0; ym < 2; ym++)
        LAUNCH(k_lfill_phase, nmissing, spix, centers, ncenters, missing, border, nmissing, H, W,
               xm, ym);
    it++;
    if (neg == prev) break;   // the legacy loop reports that the border won't shrink
    prev = neg;
  }
  if ((r = count_border())) return r;
  CK(cudaFreeAsync(border, st));
  CK(cudaFreeAsync(num_neg, st));
  CK(cudaGetLastError());
  if (iters) *iters = it;
  if (remaining) *remaining = neg;
  return STSPIX_OK;
}

int stspix_legacy_rgb_to_lab(stspix_ctx* ctx, void* stream, const float* rgb, float* lab,
                             long long npix) {
  if (!ctx || !rgb || !lab || npix < 0) return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  LAUNCH(k_rgb2lab, npix, rgb, lab, npix, 0);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_sp_video_pooling(stspix_ctx* ctx, void* stream, const float* img, const int32_t* seg,
                            int B, int T, int H, int W, int F, int nspix, float* pooled,
                            float* down, float* counts) {
  if (!ctx || !img || !seg || !down || B < 1 || T < 1 || H < 1 || W < 1 || F < 1 || nspix < 1 ||
      B > 65535 || T > 65535)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long npix = (long long)H * W, nbs = (long long)B * nspix;
  double* sum = nullptr;
  unsigned long long* cnt = nullptr;
  CK(cudaMallocAsync((void**)&sum, sizeof(double) * (size_t)(nbs * F), st));
  CK(cudaMallocAsync((void**)&cnt, sizeof(unsigned long long) * (size_t)nbs, st));
  CK(cudaMemsetAsync(sum, 0, sizeof(double) * (size_t)(nbs * F), st));
  CK(cudaMemsetAsync(cnt, 0, sizeof(unsigned long long) * (size_t)nbs, st));
  const dim3 grid((unsigned)std::max(1LL, (npix + kThreads - 1) / kThreads), (unsigned)B,
                  (unsigned)T);
  LAUNCHG(k_vpool_accum, grid, kThreads, img, seg, T, npix, F, nspix, sum, cnt);
  LAUNCH(k_vpool_mean, nbs, sum, cnt, nbs, F, down, counts);
  if (pooled) {
    CK(cudaMemsetAsync(pooled, 0, sizeof(float) * (size_t)(B * T * npix * F), st));
    LAUNCHG(k_vpool_write, grid, kThreads, down, seg, T, npix, F, nspix, pooled);
  }
  CK(cudaFreeAsync(sum, st));
  CK(cudaFreeAsync(cnt, st));
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_downsampled_video_to_pooled(stspix_ctx* ctx, void* stream, const float* down,
                                       const int32_t* seg, int B, int T, int H, int W, int F,
                                       int nspix, float* pooled) {
  if (!ctx || !down || !seg || !pooled || B < 1 || T < 1 || H < 1 || W < 1 || F < 1 ||
      nspix < 1 || B > 65535 || T > 65535)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long npix = (long long)H * W;
  CK(cudaMemsetAsync(pooled, 0, sizeof(float) * (size_t)(B * T * npix * F), st));
  const dim3 grid((unsigned)std::max(1LL, (npix + kThreads - 1) / kThreads), (unsigned)B,
                  (unsigned)T);
  LAUNCHG(k_vpool_write, grid, kThreads, down, seg, T, npix, F, nspix, pooled);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_legacy_update_prior(stspix_ctx* ctx, void* stream, const int32_t* spix,
                               long long npix, int nids, const float* mu_app, float* prior_mu_app,
                               const double* mu_shape, double* prior_mu_shape,
                               const double* sigma_shape, double* prior_sigma_shape,
                               int prev_nspix, int invert) {
  if (!ctx || !spix || !mu_app || !prior_mu_app || !mu_shape || !prior_mu_shape || !sigma_shape ||
      !prior_sigma_shape || npix < 0 || nids < 0)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  if (nids == 0 || npix == 0) return STSPIX_OK;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  uint8_t* present = nullptr;
  CK(cudaMallocAsync((void**)&present, (size_t)nids, st));
  CK(cudaMemsetAsync(present, 0, (size_t)nids, st));
  LAUNCH(k_lmark_ids, npix, spix, npix, nids, present);
  LAUNCH(k_lupdate_prior, nids, present, nids, prev_nspix, invert, mu_app, prior_mu_app,
         mu_shape, prior_mu_shape, sigma_shape, prior_sigma_shape);
  CK(cudaFreeAsync(present, st));
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_legacy_shift_tensor(stspix_ctx* ctx, void* stream, const float* in,
                               const int32_t* spix, const int32_t* flow, int B, int H, int W,
                               int F, int nspix, const int32_t* selected, float* out,
                               int32_t* counts, uint8_t* contributors) {
  if (!ctx || !in || !spix || !flow || !out || !counts || B < 1 || H < 1 || W < 1 || F < 1 ||
      nspix < 1 || B > 65535 || (long long)H * W > INT_MAX)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long npix = (long long)H * W, n = B * npix;
  double* acc = nullptr;
  CK(cudaMallocAsync((void**)&acc, sizeof(double) * (size_t)(n * F), st));
  CK(cudaMemsetAsync(acc, 0, sizeof(double) * (size_t)(n * F), st));
  CK(cudaMemsetAsync(counts, 0, sizeof(int32_t) * (size_t)n, st));
  if (contributors) CK(cudaMemsetAsync(contributors, 0, (size_t)(n * nspix), st));
  LAUNCHG(k_lshift_tensor, dim3(blocks_for(npix), (unsigned)B), kThreads, in, spix, flow, H, W, F,
          nspix, selected, acc, counts, contributors);
  LAUNCH(k_round_f32, n * F, acc, n * F, out);
  CK(cudaFreeAsync(acc, st));
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_legacy_shift_order(stspix_ctx* ctx, void* stream, const uint8_t* contributors,
                              int B, int H, int W, int nspix, int32_t* selected) {
  if (!ctx || !contributors || !selected || B < 1 || H < 1 || W < 1 || nspix < 1)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long n = (long long)B * H * W;
  LAUNCH(k_fill_i32, n, selected, n, -1);
  LAUNCH(k_lshift_order, n, contributors, n, nspix, selected);
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_legacy_split_disconnected(stspix_ctx* ctx, void* stream, int32_t* spix, int H, int W,
                                     int nspix, int32_t* split_starts, int32_t* children,
                                     long long children_cap, int* max_nsplits) {
  if (!ctx || !spix || !split_starts || !max_nsplits || H < 1 || W < 1 || nspix < 1 ||
      (long long)H * W > INT_MAX / 2)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  int r, rng[2];
  const int npix = H * W;
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  if ((r = label_range(ctx, st, spix, npix, rng))) return r;
  if (rng[0] < 0 || rng[1] >= nspix)
    return fail(ctx, STSPIX_ERR_ARG, "labels must lie in [0, %d) (got %d..%d)", nspix, rng[0],
                rng[1]);
  // scratch: parent/root, root flags, ranks, region of pixel, per-region label, size and
  // offset (npix each at most), per-label counts, scalars
  int32_t* buf = nullptr;
  const size_t words = 7 * (size_t)npix + (size_t)nspix + 4;
  CK(cudaMallocAsync((void**)&buf, sizeof(int32_t) * words, st));
  int32_t* parent = buf;
  int32_t* is_root = parent + npix;
  int32_t* rank = is_root + npix;
  int32_t* region_of = rank + npix;
  int32_t* region_spix = region_of + npix;
  int32_t* region_size = region_spix + npix;
  int32_t* region_offset = region_size + npix;
  int32_t* spix_counts = region_offset + npix;
  int32_t* sc = spix_counts + nspix;  // [0] status, [1] regions, [2] max_nsplits
  CK(cudaMemsetAsync(sc, 0, 4 * sizeof(int32_t), st));
  CK(cudaMemsetAsync(region_size, 0, sizeof(int32_t) * (size_t)npix, st));
  CK(cudaMemsetAsync(region_offset, 0xff, sizeof(int32_t) * (size_t)npix, st));
  CK(cudaMemsetAsync(spix_counts, 0, sizeof(int32_t) * (size_t)nspix, st));
  LAUNCH(k_lsd_init, npix, parent, npix);
  LAUNCH(k_lsd_hook, npix, spix, H, W, parent, sc);
  LAUNCH(k_lsd_roots, npix, parent, npix, is_root);
  LAUNCHG(k_lscan, 1, 1024, is_root, npix, rank, sc + 1);
  LAUNCH(k_lsd_regions, npix, spix, parent, rank, npix, nspix, region_of, region_spix,
         region_size, spix_counts);
  LAUNCHG(k_lsd_starts, 1, 32, spix_counts, nspix, split_starts, sc + 2);
  int32_t host_sc[4] = {0, 0, 0, 0};
  CK(cudaMemcpyAsync(host_sc, sc, sizeof host_sc, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  if (host_sc[0]) {
    cudaFreeAsync(buf, st);
    return fail(ctx, STSPIX_ERR_ITER_LIMIT, "connected components did not converge");
  }
  const int nregions = host_sc[1], mx = host_sc[2];
  *max_nsplits = mx;
  if ((long long)nspix * mx > children_cap || (mx > 0 && !children)) {
    cudaFreeAsync(buf, st);
    return fail(ctx, STSPIX_ERR_CAPACITY, "children needs %lld entries (%d x %d), capacity %lld",
                (long long)nspix * mx, nspix, mx, children_cap);
  }
  if (mx > 0) {
    LAUNCH(k_fill_i32, (long long)nspix * mx, children, (long long)nspix * mx, -1);
    LAUNCH(k_lsd_offsets, nspix, region_spix, region_size, nregions, nspix, region_offset);
    LAUNCH(k_lsd_update, npix, spix, region_of, region_offset, split_starts, npix, nspix, mx,
           children);
  }
  CK(cudaFreeAsync(buf, st));
  CK(cudaGetLastError());
  return STSPIX_OK;
}

int stspix_evaluate(stspix_ctx* ctx, void* stream, const float* vid, const int32_t* spix,
                    const int32_t* gt, int T, int H, int W, stspix_quality* out) {
  if (!ctx || !vid || !spix || !out || T < 1 || H < 1 || W < 1 || T > 65535 ||
      (long long)H * W > INT_MAX)
    return fail(ctx, STSPIX_ERR_ARG, "bad argument");
  cudaSetDevice(ctx->device);
  cudaStream_t st = (cudaStream_t)stream;
  const long long npix = (long long)H * W, n = T * npix;
  int sr[2], gr[2] = {0, 0};
  int r = label_range(ctx, st, spix, n, sr);
  if (r) return r;
  if (gt && (r = label_range(ctx, st, gt, n, gr))) return r;
  if (gt && gr[0] < 0) return fail(ctx, STSPIX_ERR_ARG, "negative ground-truth id %d", gr[0]);
  const long long S = (long long)sr[1] - sr[0] + 1, G1 = gt ? (long long)gr[1] + 1 : 1;
  if (S > INT_MAX || G1 > INT_MAX) return fail(ctx, STSPIX_ERR_TOO_LARGE, "id range too large");
  QualityScratch q = quality_layout(nullptr, T, S, G1, true, gt != nullptr);
  if (q.bytes > kQualityMaxScratch || (gt && (double)T * S * G1 > 2e9))
    return fail(ctx, STSPIX_ERR_TOO_LARGE, "evaluation tables of %zu bytes (T=%d, ids=%lld, "
                "ground-truth ids=%lld) exceed the limit", q.bytes, T, S, G1);
  char* base = nullptr;
  CK(cudaMallocAsync((void**)&base, q.bytes, st));
  q = quality_layout(base, T, S, G1, true, gt != nullptr);
  CK(cudaMemsetAsync(base, 0, q.bytes, st));
  const long long segs = (long long)T * H * ((W + 31) / 32);
  const unsigned nb = (unsigned)std::max(1LL, std::min<long long>((segs + 7) / 8, 8LL * ctx->num_sms));
  LAUNCHG(k_q_accum, nb, kThreads, vid, spix, gt, T, H, W, sr[0], (int)S, (int)G1, q.cnt, q.fsum,
          q.vsum, q.msum, q.J);
  const unsigned rx = (unsigned)std::max(1LL, std::min<long long>(q_blocks(npix), 8LL * ctx->num_sms / T + 1));
  LAUNCHG(k_q_resid, dim3(rx, T), kThreads, vid, spix, (int)npix, sr[0], (int)S, q.cnt, q.fsum,
          q.msum, q.pix2, q.pix2s, q.sse);
  LAUNCHG(k_q_id_time, q_blocks(S), kThreads, q.cnt, T, (int)S, q.ntot, q.stdv);
  LAUNCHG(k_q_frame_ids, dim3(q_blocks(S), T), kThreads, q.cnt, q.fsum, q.vsum, q.ntot, q.msum,
          (int)S, (int)npix, q.live, q.pool2, q.pool3);
  if (gt) {
    LAUNCHG(k_q_uesa_frame, dim3(q_blocks(S), T), kThreads, q.cnt, q.J, (int)S, (int)G1, q.ue,
            q.sa, q.gsize);
    LAUNCHG(k_q_uesa_id, q_blocks(S), kThreads, q.cnt, q.J, q.ntot, T, (int)S, (int)G1, q.ue3,
            q.sa3);
  }
  // per-frame / per-id results to the host
  std::vector<double> pix2(T), pix2s(T), sse(T), pool2(T), pool3(T), stdv(S);
  std::vector<unsigned long long> live(T), ue, sa, gsize, ue3, sa3;
  auto d2h = [&](void* dst, const void* src, size_t bytes) {
    return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, st);
  };
  CK(d2h(pix2.data(), q.pix2, 8 * (size_t)T));
  CK(d2h(pix2s.data(), q.pix2s, 8 * (size_t)T));
  CK(d2h(sse.data(), q.sse, 8 * (size_t)T));
  CK(d2h(pool2.data(), q.pool2, 8 * (size_t)T));
  CK(d2h(pool3.data(), q.pool3, 8 * (size_t)T));
  CK(d2h(live.data(), q.live, 8 * (size_t)T));
  CK(d2h(stdv.data(), q.stdv, 8 * (size_t)S));
  if (gt) {
    ue.resize(T * G1); sa.resize(T * G1); gsize.resize(T * G1); ue3.resize(G1); sa3.resize(G1);
    CK(d2h(ue.data(), q.ue, 8 * (size_t)(T * G1)));
    CK(d2h(sa.data(), q.sa, 8 * (size_t)(T * G1)));
    CK(d2h(gsize.data(), q.gsize, 8 * (size_t)(T * G1)));
    CK(d2h(ue3.data(), q.ue3, 8 * (size_t)G1));
    CK(d2h(sa3.data(), q.sa3, 8 * (size_t)G1));
  }
  CK(cudaFreeAsync(base, st));
  CK(cudaStreamSynchronize(st));
  CK(cudaGetLastError());

  stspix_quality res{};
  size_scores(live, stdv, T, S, &res.tex, &res.szv);
  double ev = 0, ev3 = 0, ps = 0, nsp = 0;
  for (int t = 0; t < T; t++) {
    ev += pool2[t] / (pix2[t] + 1e-10);
    ev3 += pool3[t] / (pix2s[t] + 1e-10);
    const double mse = sse[t] / (3.0 * npix);
    ps += mse > 0 ? 10.0 * std::log10(1.0 / mse) : INFINITY;
    nsp += (double)live[t];
  }
  res.ev = ev / T;
  res.ev3d = ev3 / T;
  res.psnr = ps / T;
  res.ave_nsp = nsp / T;
  res.spnum = (int)S;
  res.ue2d = res.sa2d = res.ue3d = res.sa3d = -1.0;
  res.has_gt = gt ? 1 : 0;
  if (gt) {
    // evaluate.py:482-510; every ground-truth id 0..max must be present (the
    // reference aligns its columns on that and asserts non-empty objects)
    for (long long g = 0; g < G1; g++) {
      unsigned long long tot = 0;
      for (int t = 0; t < T; t++) tot += gsize[t * G1 + g];
      if (!tot) return fail(ctx, STSPIX_ERR_ARG, "ground-truth id %lld of 0..%lld never occurs", g,
                            G1 - 1);
    }
    double u2 = 0;
    for (long long i = 0; i < T * G1; i++) u2 += (double)ue[i] / (double)npix;
    res.ue2d = u2 / (double)(T * G1);
    double s2 = 0, u3 = 0, s3 = 0;
    for (long long g = 0; g < G1; g++) {
      u3 += (double)ue3[g] / (double)(T * npix);
      if (g == 0) continue;
      double a = 0, tot = 0;
      long long frames = 0;
      for (int t = 0; t < T; t++) {
        const unsigned long long z = gsize[t * G1 + g];
        a += (double)sa[t * G1 + g] / (double)(z ? z : 1);
        frames += z > 0;
        tot += (double)z;
      }
      s2 += a / (double)frames;
      s3 += (double)sa3[g] / tot;
    }
    res.ue3d = u3 / (double)G1;
    res.sa2d = G1 > 1 ? s2 / (double)(G1 - 1) : std::nan("");
    res.sa3d = G1 > 1 ? s3 / (double)(G1 - 1) : std::nan("");
  }
  *out = res;
  return STSPIX_OK;
}

int stspix_profile_enable(stspix_ctx* ctx, int enable) {
  if (!ctx) return STSPIX_ERR_ARG;
  ctx->prof_on = enable ? 1 : 0;
  for (int i = 0; i < STSPIX_NFAM; i++) { ctx->fam_launches[i] = 0; ctx->fam_ms[i] = 0; }
  ctx->kern.clear();
  return STSPIX_OK;
}

int stspix_profile_kernels(const stspix_ctx* ctx, char* buf, int capacity) {
  if (!ctx) return -1;
  std::string out;
  char line[160];
  for (auto& kv : ctx->kern) {
    snprintf(line, sizeof line, "%s %lld %.6f\n", kv.first.c_str(), kv.second.first,
             kv.second.second);
    out += line;
  }
  if (buf && capacity > 0) {
    size_t n = std::min(out.size(), (size_t)capacity - 1);
    memcpy(buf, out.data(), n);
    buf[n] = 0;
  }
  return (int)out.size() + 1;
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
