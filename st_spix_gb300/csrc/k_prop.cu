// GB300 kernels of the optical-flow propagation path (gauenk/st_spix
// st_spix/csrc/bist/shift_and_fill.cu, sp_pooling.cu, shift_labels.cu,
// fill_missing.cu, split_disconnected.cu, relabel.cu, sparams_io.cu, prop.cu).
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace stspix {

// ---------------------------------------------------------------------------
// Clear the per-previous-superpixel sums and the warp targets of every slot.
__global__ void kb_prop_clear(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  FOR_PIX(i, max(S.npix, S.n_prev)) {
    if (i < S.n_prev) {
      S.cnt_pool[i] = 0;
      S.cs[i] = 0;
      S.cf[i] = 0;
      S.fs[2 * (size_t)i] = 0;
      S.fs[2 * (size_t)i + 1] = 0;
      S.ccbest[i] = 0;
    }
    if (i < S.npix) {
      S.hits[i] = 0;
      S.best[i] = ~0ull;
      S.d2[i] = 0;
    }
    if (i == 0) { S.sc->ninvalid = 0; S.sc->nhole = 0; }
  }
}

// Mean flow per superpixel (sp_downsample_kernel / normz_downsample_kernel,
// sp_pooling.cu:27-71), R1 fixed point: pixel counts and flow sums of the previous
// labels by warp-block label rounds.
__global__ void __launch_bounds__(256) kb_flow_pool(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int H = S.H, W = S.W, n = S.n_prev;
  int gx, by;
  if (!warp_block(W, H, gx, by)) return;
  const int lane = threadIdx.x & 31;
  const int* __restrict__ lab_prev = S.prev_labels;
  const float* __restrict__ flow = S.flow;
  int lab[8];
  long long qx[8], qy[8];
  unsigned pend = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int gy = by + i;
    const bool in = gx < W && gy < H;
    const size_t g = (size_t)gy * W + gx;
    lab[i] = in ? lab_prev[g] : -1;
    qx[i] = in ? fx_q(flow[2 * g], kFxFlowShift) : 0;
    qy[i] = in ? fx_q(flow[2 * g + 1], kFxFlowShift) : 0;
    if (lab[i] >= 0 && lab[i] < n) pend |= 1u << i;
  }
  label_rounds(lab, pend, [&](int k, unsigned m, int src) {
    long long sx = 0, sy = 0;
#pragma unroll
    for (int i = 0; i < 8; i++)
      if ((m >> i) & 1u) { sx += qx[i]; sy += qy[i]; }
    const int N = __reduce_add_sync(0xffffffffu, __popc(m));
    const long long SX = warp_sum64(sx), SY = warp_sum64(sy);
    if (lane == src) {
      atomicAdd(&S.cnt_pool[k], N);
      atomicAdd((unsigned long long*)&S.fs[2 * (size_t)k], (unsigned long long)SX);
      atomicAdd((unsigned long long*)&S.fs[2 * (size_t)k + 1], (unsigned long long)SY);
    }
  });
}

// normz + centres = mu_shape + mean flow (shift_and_fill.cu:140-150).
__global__ void kb_flow_mean(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int n = S.n_prev;
  const int* __restrict__ cnt = S.cnt_pool;
  const long long* __restrict__ fs = S.fs;
  const double* __restrict__ mu_shape = S.pprev.mu_shape;
  float* __restrict__ fds = S.fds;
  double* __restrict__ centers = S.centers;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  for (int c = 0; c < 2; c++) {
    float m = cnt[k] > 0 ? (float)(fx_unq(fs[2 * k + c], kFxFlowShift) / (1. * cnt[k])) : 0.f;
    fds[2 * k + c] = m;
    centers[2 * k + c] = mu_shape[2 * k + c] + (double)m;
  }
}

// Forward warp by the rounded mean flow (shift_labels_kernel, shift_labels.cu:33-112),
// collisions resolved by the smallest packed (size, id) (R4).
__global__ void kb_shift(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int* __restrict__ lab = S.prev_labels;
  const int H = S.H, W = S.W, n = S.n_prev;
  const int* __restrict__ cnt = S.cnt_pool;
  const float* __restrict__ fds = S.fds;
  int* __restrict__ hits = S.hits;
  unsigned long long* __restrict__ best = S.best;
  FOR_PIX(t, H * W) {
    const int k = lab[t];
    if (k < 0 || k >= n) continue;
    const int size = cnt[k];
    const int fw = (int)roundf(fds[2 * k]);
    const int fh = (int)roundf(fds[2 * k + 1]);
    const int w = t % W + fw, h = t / W + fh;
    if (w < 0 || w >= W || h < 0 || h >= H) continue;
    const int d = h * W + w;
    atomicAdd(&hits[d], 1);
    const unsigned long long key = ((unsigned long long)(unsigned int)size << 32) | (unsigned int)k;
    atomicMin(&best[d], key);
  }
}

// decode_kernel (shift_labels.cu:128-164) + copy to `filled` + hole count.
// Append pixel t to the slot's hole list (smseg, count sc->nhole) when `hole`;
// block-aggregated: one atomic per block (every thread of the block calls it).  The
// list order depends on scheduling; the fill's result does not (a parity phase updates
// pixels that are never 4-neighbours of each other).  With count_invalid the holes are
// also counted into sc->ninvalid (the hole count after the shift, which the iteration
// ladder reads).
__device__ __forceinline__ void append_hole(const Slot& S, int t, bool hole, bool count_invalid) {
  __shared__ int woff[32];
  __shared__ int base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, hole);
  if (lane == 0) woff[warp] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) { const int c = woff[w]; woff[w] = tot; tot += c; }
    base = tot ? atomicAdd(&S.sc->nhole, tot) : 0;
    if (tot && count_invalid) atomicAdd(&S.sc->ninvalid, tot);
  }
  __syncthreads();
  if (hole) S.smseg[base + woff[warp] + __popc(m & ((1u << lane) - 1))] = t;
  __syncthreads();          // woff and base are free for the block's next call
}

__global__ void kb_shift_decode(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  FOR_PIX_ALL(t, S.npix) {
    const bool in = t < S.npix;
    int v = -1;
    if (in) {
      v = S.hits[t] > 0 ? (int)(unsigned int)S.best[t] : -1;
      S.shifted[t] = v;
      S.seg[t] = v;
    }
    append_hole(S, t, in && v < 0, true);
  }
}

// Per-label pixel counts (get_spix_sizes, seg_utils.cu:56-75), by warp-block label
// rounds.  which 0: counts after the shift (cs), 1: after the fill (cf).
__global__ void __launch_bounds__(256) kb_count_labels(const Slot* __restrict__ slots, int which) {
  pdl_enter();
  SLOT_Y;
  const int H = S.H, W = S.W, n = S.n_prev;
  int gx, by;
  if (!warp_block(W, H, gx, by)) return;
  int* cnt = which ? S.cf : S.cs;
  int lab[8];
  unsigned pend = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int gy = by + i;
    lab[i] = (gx < W && gy < H) ? S.seg[(size_t)gy * W + gx] : -1;
    if (lab[i] >= 0 && lab[i] < n) pend |= 1u << i;
  }
  label_rounds(lab, pend, [&](int k, unsigned m, int src) {
    const int N = __reduce_add_sync(0xffffffffu, __popc(m));
    if ((int)(threadIdx.x & 31) == src) atomicAdd(&cnt[k], N);
  });
}

// ---------------------------------------------------------------------------
// Hole filling (fill_missing.cu:35-130, update_missing_seg_nn :288-441,
// find_border_along_missing :617-647) over lists of hole pixels instead of the frame.
// The reference's iteration: the hole count, the border flag of every hole (a
// 4-neighbour labelled at the start of the iteration), then four parity phases in
// which a bordered hole takes the label of the neighbour whose centre is nearest;
// stop rules: a count equal to the previous one is an error (it exits), no holes
// left ends the loop, both checked after the iteration's phases; break_iter caps it.
//
// Here the fill's hole list is split once into the four parity classes (kb_fill_split,
// into the `hits` buffer), and an iteration is kb_fill_phase x 4, run as the body of a
// CUDA-graph WHILE node whose condition the last block of the fourth phase sets (no
// host round trips, no grid barriers).  A phase scans its class only.  The border
// flags are not stored: a hole filled in this iteration carries a flag bit of the
// iteration's parity in its label until its own class's phase of the next iteration
// (or kb_fill_end) strips it, so "labelled at the start of the iteration" is "labelled
// and not flagged with this iteration's parity" (a 4-neighbour always belongs to
// another class, so a phase never reads a label of its own class written in the same
// phase).  Candidates read the labels without flags.  The order of the holes in a list
// does not matter (a phase's pixels are never 4-neighbours of each other).
constexpr int kFillFlagOdd = 1 << 30, kFillFlagEven = 1 << 29;
constexpr int kFillFlags = kFillFlagOdd | kFillFlagEven;

__global__ void kb_fill_begin(const Slot* __restrict__ slots, int B) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  Scalars* sc = slots[i].sc;
  sc->fl_n = sc->nhole;
  sc->fl_prev = 1410065408;  // (int)10000000000 as the reference truncates it
  sc->fl_iter = 0;
  sc->fl_done = 0;
  sc->fl_fill = 0;
  for (int c = 0; c < 4; c++) { sc->fl_cnt[c] = 0; sc->fl_pos[c] = 0; }
}

__device__ __forceinline__ int fill_class(int idx, int W) {
  const int x = idx % W, y = idx / W;
  return ((x & 1) << 1) | (y & 1);             // phase ph: x parity ph >> 1, y parity ph & 1
}

// pass 0: count the holes of each class; pass 1: write each class's holes into its
// part of `hits` (offset = the counts of the classes before it).  Warp-aggregated.
__global__ void kb_fill_split(const Slot* __restrict__ slots, int pass) {
  pdl_enter();
  SLOT_Y;
  Scalars* sc = S.sc;
  const int n = sc->nhole, W = S.W;
  const int lane = threadIdx.x & 31;
  int off[4] = {0, 0, 0, 0};
  if (pass) {
    off[1] = sc->fl_cnt[0];
    off[2] = off[1] + sc->fl_cnt[1];
    off[3] = off[2] + sc->fl_cnt[2];
  }
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int j = base + threadIdx.x;
    const bool in = j < n;
    const int idx = in ? S.smseg[j] : 0;
    const int c = in ? fill_class(idx, W) : -1;
#pragma unroll
    for (int cc = 0; cc < 4; cc++) {
      const unsigned m = __ballot_sync(0xffffffffu, c == cc);
      if (!m) continue;
      const int leader = __ffs(m) - 1;
      int at = 0;
      if (lane == leader) at = atomicAdd(pass ? &sc->fl_pos[cc] : &sc->fl_cnt[cc], __popc(m));
      at = __shfl_sync(0xffffffffu, at, leader);
      if (pass && c == cc) S.hits[off[cc] + at + __popc(m & ((1u << lane) - 1))] = idx;
    }
  }
}

// (float)(num / d) for the fill's similarity (fill_missing.cu: a float pixel coordinate
// minus a double centre, divided by the float frame size, in double, then stored in a
// float), without the double division where it cannot matter: r = num * (1 / d) is
// within 2 ulps of the double quotient, so unless r lies within 3 ulps of a float
// rounding midpoint (the 29 bits below a float's mantissa equal to 2^28) both round to
// the same float.  The rare rest divides.  GB300's FP64 rate is low, and two divisions
// per candidate made the fill FP64-bound; the result is the same bit for bit.
__device__ __forceinline__ float fill_quot(double num, double inv, double d) {
  const double r = num * inv;
  const unsigned lo29 = (unsigned)(__double_as_longlong(r) & ((1ll << 29) - 1));
  if (fabs(r) >= 0x1p-120 && (lo29 > (1u << 28) + 3u || lo29 < (1u << 28) - 3u)) return (float)r;
  return (float)(num / d);
}

// One parity phase of one iteration.  ph 3 also closes the iteration: its last block
// (a device counter, no waiting) applies the stop rules to every slot, counts the
// iteration (*body_iters) and sets the loop condition.
__global__ void kb_fill_phase(const Slot* __restrict__ slots, int ph, int B,
                              cudaGraphConditionalHandle cond, int break_iter, int* body_iters,
                              unsigned* ctr) {
  pdl_enter();
  SLOT_Y;
  Scalars* sc = S.sc;
  if (!sc->fl_done) {
    const int W = S.W, H = S.H;
    const int cur = (sc->fl_iter & 1) ? kFillFlagOdd : kFillFlagEven;
    const int off = ph == 0 ? 0 : ph == 1 ? sc->fl_cnt[0]
                  : ph == 2 ? sc->fl_cnt[0] + sc->fl_cnt[1]
                            : sc->fl_cnt[0] + sc->fl_cnt[1] + sc->fl_cnt[2];
    const int n = sc->fl_cnt[ph];
    const int* la = S.hits + off;
    int* seg = S.seg;
    const double* centers = S.centers;
    const double inv_w = S.inv_w, inv_h = S.inv_h, dW = 1.0f * W, dH = 1.0f * H;
    const int lane = threadIdx.x & 31;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
      const int j = base + threadIdx.x;
      bool filled_now = false;
      if (j < n) {
        const int idx = la[j];
        const int v = seg[idx];
        if (v != -1) {
          // filled in an earlier iteration: its flag (the previous iteration's) goes
          if (v & kFillFlags) seg[idx] = v & ~kFillFlags;
        } else {
          const int x = idx % W, y = idx / W;
          int N = -1, So = -1, E = -1, Wl = -1;
          if (x > 0) Wl = seg[idx - 1];
          if (y > 0) N = seg[idx - W];
          if (x < W - 1) E = seg[idx + 1];
          if (y < H - 1) So = seg[idx + W];
          // bordered: a neighbour labelled at the start of the iteration
          auto at_start = [&](int u) { return u >= 0 && !(u & cur); };
          if (at_start(N) || at_start(So) || at_start(Wl) || at_start(E)) {
            N = N >= 0 ? (N & ~kFillFlags) : N;
            So = So >= 0 ? (So & ~kFillFlags) : So;
            Wl = Wl >= 0 ? (Wl & ~kFillFlags) : Wl;
            E = E >= 0 ? (E & ~kFillFlags) : E;
            float bx = -999999;
            int bl = -1;
            auto consider = [&](int lab) {
              const double* cp = centers + 2 * (size_t)lab;
              float dx = fill_quot(1.0f * x - cp[0], inv_w, dW);
              float dy = fill_quot(1.0f * y - cp[1], inv_h, dH);
              float sim = -dx * dx - dy * dy;
              if (sim > bx) { bx = sim; bl = lab; }
            };
            if (N >= 0) consider(N);
            if (So >= 0 && So != N) consider(So);
            if (Wl >= 0 && Wl != So && Wl != N) consider(Wl);
            if (E >= 0 && E != Wl && E != So && E != N) consider(E);
            seg[idx] = bl | cur;
            filled_now = true;
          }
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, filled_now);
      if (m && lane == __ffs(m) - 1) atomicAdd(&sc->fl_fill, __popc(m));
    }
  }
  if (ph != 3) return;
  __shared__ int is_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    is_last = atomicAdd(ctr, 1u) == gridDim.x * gridDim.y - 1;
  }
  __syncthreads();
  if (!is_last) return;
  __threadfence();
  int active = 0;
  for (int i = threadIdx.x; i < B; i += blockDim.x) {
    Scalars* si = slots[i].sc;
    if (si->fl_done) continue;
    const int num_neg = si->fl_n;           // holes at the start of this iteration
    si->fill_iters += 1;
    si->fl_iter += 1;
    if (num_neg == si->fl_prev) {
      si->status = STSPIX_ERR_NOPROGRESS;
      si->fl_done = 1;
    } else {
      si->fl_prev = num_neg;
      if (num_neg <= 0 || si->fl_iter >= break_iter) si->fl_done = 1;
    }
    si->fl_n = num_neg - si->fl_fill;
    si->fl_fill = 0;
    if (!si->fl_done) active = 1;
  }
  active = __syncthreads_or(active);
  if (threadIdx.x == 0) {
    *body_iters += 1;
    *ctr = 0u;
    cudaGraphSetConditional(cond, active ? 1u : 0u);
  }
}

// After the loop: the flags of the last iterations' fills go.
__global__ void kb_fill_end(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int n = S.sc->nhole;
  int* seg = S.seg;
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const int idx = S.hits[j];
    const int v = seg[idx];
    if (v >= 0 && (v & kFillFlags)) seg[idx] = v & ~kFillFlags;
  }
}

// ---------------------------------------------------------------------------
// Disconnected regions (split_disconnected.cu:33-96): component roots by
// union-find, sizes, largest region per label (R6), invalidate the rest.
// Connected components (8-connected, same label) by union-find with min-index
// hooking: every tree's root is the smallest pixel index of its component, the
// fixed point of find_spix_min (split_disconnected.cu:458-498).  Parents only
// decrease, so the walks below end; they are capped all the same.
constexpr int kUfLimit = 1 << 26;
// Root of x with path halving (atomicMin keeps parents decreasing under races).
__device__ __forceinline__ int uf_find(int* parent, int x) {
  for (int i = 0; i < kUfLimit; i++) {
    const int p = *(volatile int*)&parent[x];
    if (p == x) return x;
    const int g = *(volatile int*)&parent[p];
    if (g == p) return p;
    atomicMin(&parent[x], g);
    x = g;
  }
  return -1;
}
__device__ __forceinline__ bool uf_unite(int* parent, int a, int b) {
  for (int i = 0; i < kUfLimit; i++) {
    a = uf_find(parent, a);
    b = uf_find(parent, b);
    if (a < 0 || b < 0) return false;
    if (a == b) return true;
    if (a < b) { int t = a; a = b; b = t; }
    const int old = atomicMin(&parent[a], b);
    if (old == a) return true;
    a = old;
  }
  return false;
}

// The unions of pixel t: with the earlier 8-neighbours of the same label; a diagonal one
// is skipped when a 4-path through W or N already joins it (W-NW and N-NW, N-NE are
// united at those pixels).  Each union is made by the pass that owns it: a tile's own
// pass (kb_cc_local, both pixels in one CC tile) or the cross-tile pass (kb_cc_hook);
// union-find with min-index hooking reaches the same roots whatever the order.
constexpr int kCcTile = 32;             // CC tiles of 32 x 32 pixels
__device__ __forceinline__ bool cc_same_tile(int x, int y, int xn, int yn) {
  return (x / kCcTile) == (xn / kCcTile) && (y / kCcTile) == (yn / kCcTile);
}
template <typename Unite>
__device__ __forceinline__ void cc_unions(const int* __restrict__ seg, int t, int W, int L,
                                          bool local, Unite unite) {
  const int x = t % W, y = t / W;
  auto own = [&](int xn, int yn) { return cc_same_tile(x, y, xn, yn) == local; };
  const bool w = x > 0 && seg[t - 1] == L;
  if (w && own(x - 1, y)) unite(t - 1);
  if (y > 0) {
    if (seg[t - W] == L) {
      if (own(x, y - 1)) unite(t - W);
    } else {
      if (!w && x > 0 && seg[t - W - 1] == L && own(x - 1, y - 1)) unite(t - W - 1);
      if (x < W - 1 && seg[t - W + 1] == L && own(x + 1, y - 1)) unite(t - W + 1);
    }
  }
}

// One block per 32 x 32 tile, a warp per tile row (tile rows are 32 pixels): each
// pixel's parent starts as the first pixel of its run of equal labels in the row (one
// ballot, no atomics), then union-find in shared memory (min-index hooking) joins the
// runs.  A pixel p = (x, y) of label L unites, inside the tile, with
//   N  when N has label L, unless the left pixel and NW both have label L (the left
//      pixel is in p's run and NW in N's run, so the left pixel's union joins them);
//   NW when neither the left pixel nor N has label L and NW has;
//   NE when N does not have label L and NE has
// (the 8-connected rule of cc_unions with the W unions given by the runs).  At the
// tile's first column the left pixel is in another tile: no skip there, and the pairs
// across tile edges are kb_cc_hook's.  Then each pixel's global parent = its local root
// (the smallest pixel index of its component in the tile: row-major order within a
// tile is the frame's order).  Replaces the parent initialisation.
__global__ void __launch_bounds__(256) kb_cc_local(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  static_assert(kCcTile == 32, "a tile row is a warp");
  constexpr int kRows = kCcTile / 8;        // rows per warp
  __shared__ int lab[kCcTile][kCcTile];
  __shared__ int par[kCcTile * kCcTile];
  const int W = S.W, H = S.H;
  const int tiles_x = (W + kCcTile - 1) / kCcTile;
  if ((int)blockIdx.x >= tiles_x * ((H + kCcTile - 1) / kCcTile)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) S.sc->nhole = 0;
  const int tx0 = (blockIdx.x % tiles_x) * kCcTile, ty0 = (blockIdx.x / tiles_x) * kCcTile;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int x = tx0 + lane;
  const int* seg = S.seg;
  int v[kRows];
#pragma unroll
  for (int a = 0; a < kRows; a++) {
    const int y = ty0 + warp * kRows + a;
    v[a] = (x < W && y < H) ? seg[(size_t)y * W + x] : -1;
  }
#pragma unroll
  for (int a = 0; a < kRows; a++) {
    const int ly = warp * kRows + a;
    lab[ly][lane] = v[a];
    const int left = __shfl_up_sync(0xffffffffu, v[a], 1);
    const unsigned cont = __ballot_sync(0xffffffffu, lane > 0 && v[a] >= 0 && v[a] == left);
    const unsigned starts = ~cont & (0xffffffffu >> (31 - lane));   // run starts at lanes <= lane
    par[ly * kCcTile + lane] = v[a] >= 0 ? ly * kCcTile + (31 - __clz(starts)) : -1;
  }
  __syncthreads();
  bool ok = true;
#pragma unroll
  for (int a = 0; a < kRows; a++) {
    const int ly = warp * kRows + a;
    const int L = v[a];
    if (L < 0 || ly == 0) continue;
    const int li = ly * kCcTile + lane;
    const int n = lab[ly - 1][lane];
    const bool w = lane > 0 && lab[ly][lane - 1] == L;
    const int nw = lane > 0 ? lab[ly - 1][lane - 1] : -1;
    const int ne = lane < kCcTile - 1 ? lab[ly - 1][lane + 1] : -1;
    if (n == L) {
      if (!(w && nw == L)) ok &= uf_unite(par, li, li - kCcTile);
    } else {
      if (!w && nw == L) ok &= uf_unite(par, li, li - kCcTile - 1);
      if (ne == L) ok &= uf_unite(par, li, li - kCcTile + 1);
    }
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < kRows; a++) {
    const int ly = warp * kRows + a;
    const int y = ty0 + ly;
    if (x >= W || y >= H) continue;
    const int li = ly * kCcTile + lane;
    const int r = par[li] >= 0 ? uf_find(par, li) : -1;
    if (par[li] >= 0 && r < 0) ok = false;
    S.d1[(size_t)y * W + x] = r >= 0 ? (ty0 + r / kCcTile) * W + tx0 + r % kCcTile : -1;
  }
  if (!ok) atomicExch(&S.sc->status, STSPIX_ERR_ITER_LIMIT);
}

// The unions across tile edges, on the global parents.  Only pixels on a tile's first
// row or first / last column have neighbours in another tile: kCcEdge per tile, thread
// u taking edge pixel u % kCcEdge of tile u / kCcEdge.
constexpr int kCcEdge = kCcTile + 2 * (kCcTile - 1);
__global__ void kb_cc_hook(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  const int W = S.W, H = S.H;
  const int tiles_x = (W + kCcTile - 1) / kCcTile;
  const int tile = u / kCcEdge, e = u % kCcEdge;
  if (tile >= tiles_x * ((H + kCcTile - 1) / kCcTile)) return;
  const int lx = e < kCcTile ? e : (e < 2 * kCcTile - 1 ? 0 : kCcTile - 1);
  const int ly = e < kCcTile ? 0 : (e < 2 * kCcTile - 1 ? e - kCcTile + 1 : e - 2 * kCcTile + 2);
  const int x = (tile % tiles_x) * kCcTile + lx, y = (tile / tiles_x) * kCcTile + ly;
  if (x >= W || y >= H) return;
  const int t = y * W + x;
  const int* seg = S.seg;
  const int L = seg[t];
  if (L < 0) return;
  bool ok = true;
  cc_unions(seg, t, W, L, false, [&](int tn) { ok &= uf_unite(S.d1, t, tn); });
  if (!ok) atomicExch(&S.sc->status, STSPIX_ERR_ITER_LIMIT);
}

// Every pixel's parent := its root, and the component sizes: the lanes of a warp with
// the same root (a warp's pixels are consecutive, so few roots) add their count once.
__global__ void kb_cc_compress(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  FOR_PIX_ALL(t, S.npix) {
    int r = -1;
    if (t < S.npix && S.d1[t] >= 0) {
      r = uf_find(S.d1, t);
      S.d1[t] = r;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, r);
    if (r >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&S.d2[r], __popc(peers));
  }
}

__global__ void kb_cc_best(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int* __restrict__ seg = S.seg;
  const int* __restrict__ root = S.d1;
  const int* __restrict__ size = S.d2;
  const int nlab = S.n_prev;
  unsigned long long* __restrict__ best = S.ccbest;
  FOR_PIX(t, S.npix) {
    if (root[t] != t) continue;
    const int L = seg[t];
    if (L < 0 || L >= nlab) continue;
    const unsigned long long key = ((unsigned long long)(unsigned int)size[t] << 32) |
                                   (unsigned long long)(0xffffffffu - (unsigned int)t);
    atomicMax(&best[L], key);
  }
}

__global__ void kb_cc_invalidate(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  int* __restrict__ seg = S.seg;
  const int* __restrict__ root = S.d1;
  const int nlab = S.n_prev;
  const unsigned long long* __restrict__ best = S.ccbest;
  FOR_PIX(t, S.npix) {
    const int L = seg[t];
    if (L < 0 || L >= nlab) continue;
    const unsigned int win = 0xffffffffu - (unsigned int)(best[L] & 0xffffffffull);
    if ((unsigned int)root[t] != win) seg[t] = -1;
  }
}

// Hole list of the second fill: every -1 pixel after the invalidation.
__global__ void kb_list_holes(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  FOR_PIX_ALL(t, S.npix) append_hole(S, t, t < S.npix && S.seg[t] < 0, false);
}

// invalid_counts / prior_counts update (shift_and_fill.cu:300-330).
__global__ void kb_shift_params(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int n = S.n_prev;
  const int* __restrict__ cnt_pool = S.cnt_pool;
  const int* __restrict__ cs = S.cs;
  const int* __restrict__ cf = S.cf;
  const stspix_params& pp = S.pprev;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || k >= pp.capacity) return;
  int f = cf[k], s = cs[k];
  pp.invalid_counts[k] = (float)((f - s) / (static_cast<float>(f) + 1e-8));
  int c = cnt_pool[k];
  if (c > 0) pp.prior_counts[k] = (float)fmin(fmax(1.0 * c, 100.0), 10000.0);
}

// ---------------------------------------------------------------------------
// run_prop set-up: write_params (sparams_io.cu:353-501, prior_icov = invert_cov
// :505-520) then mark_active (init_sparams.cu:195-286).
__global__ void kb_write_params(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const stspix_params& pp = S.pprev;
  const int n = S.n_prev, sp_size = S.sp_size;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= sp.cap) return;
  if (i < n) {
    for (int c = 0; c < 3; c++) {
      sp.mu_app[3 * i + c] = pp.mu_app[3 * i + c];
      sp.prior_mu_app[3 * i + c] = pp.prior_mu_app[3 * i + c];
      sp.sigma_shape[3 * i + c] = pp.sigma_shape[3 * i + c];
      sp.prior_sigma_shape[3 * i + c] = pp.prior_sigma_shape[3 * i + c];
      sp.sample_sigma_shape[3 * i + c] = pp.sample_sigma_shape[3 * i + c];
    }
    for (int c = 0; c < 2; c++) {
      sp.mu_shape[2 * i + c] = pp.mu_shape[2 * i + c];
      sp.prior_mu_shape[2 * i + c] = pp.prior_mu_shape[2 * i + c];
    }
    sp.logdet[i] = pp.logdet_sigma_shape[i];
    double px = pp.prior_sigma_shape[3 * i], py = pp.prior_sigma_shape[3 * i + 1],
           pz = pp.prior_sigma_shape[3 * i + 2];
    double pr_det = px * pz - py * py;
    sp.prior_icov[3 * i] = pz / pr_det;
    sp.prior_icov[3 * i + 1] = py / pr_det;
    sp.prior_icov[3 * i + 2] = px / pr_det;
    sp.count[i] = pp.counts[i];
    sp.icount[i] = pp.invalid_counts[i];
    sp.sm_count[i] = pp.sm_counts[i];
    sp.prior_count[i] = pp.prior_counts[i];
  } else {
    for (int c = 0; c < 3; c++) {
      sp.mu_app[3 * i + c] = 0.f; sp.prior_mu_app[3 * i + c] = 0.f;
      sp.sigma_shape[3 * i + c] = 0.0; sp.sample_sigma_shape[3 * i + c] = 0.0;
      sp.prior_icov[3 * i + c] = 0.0;
    }
    sp.prior_sigma_shape[3 * i] = 1.0 / sp_size;
    sp.prior_sigma_shape[3 * i + 1] = 0;
    sp.prior_sigma_shape[3 * i + 2] = 1.0 / sp_size;
    for (int c = 0; c < 2; c++) { sp.mu_shape[2 * i + c] = 0.0; sp.prior_mu_shape[2 * i + c] = 0.0; }
    sp.logdet[i] = 0.0;
    sp.count[i] = 0; sp.icount[i] = 0.f; sp.sm_count[i] = 0; sp.prior_count[i] = 0.f;
  }
  sp.valid[i] = 0;
  sp.prop[i] = 0;
}

__global__ void kb_mark_active(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  int gx, by;
  if (!warp_block(S.W, S.H, gx, by)) return;
  // one store pair per label of a warp's 32 x 8 block (many blocks share a label)
  int lab[8];
  unsigned pend = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int gy = by + i;
    lab[i] = (gx < S.W && gy < S.H) ? S.seg[(size_t)gy * S.W + gx] : -1;
    if (lab[i] >= 0 && lab[i] < sp.cap) pend |= 1u << i;
  }
  label_rounds(lab, pend, [&](int k, unsigned, int src) {
    if ((int)(threadIdx.x & 31) == src) {
      sp.valid[k] = 1;
      sp.prop[k] = 1;
    }
  });
}



// ---------------------------------------------------------------------------
// Relabel (relabel.cu:126-409), R5.
// Relabel runs on propagated slots only (mode 1); plain BASS slots return at once.
__global__ void kb_relabel_init(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.mode) return;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S.cap + 2) return;
  S.living[s] = 0;
  S.src_of[s] = -1;
  if (s >= S.cap) return;
  S.rbest[s] = ((unsigned long long)__float_as_uint(10000.f) << 32) | 0x7fffffffull;
  S.ss[s] = 0.f;
}

__global__ void kb_living(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.mode) return;
  const int ms = S.sc->max_spix;
  int gx, by;
  if (!warp_block(S.W, S.H, gx, by)) return;
  // one store per label of a warp's 32 x 8 block (many blocks share a label)
  int lab[8];
  unsigned pend = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int gy = by + i;
    lab[i] = (gx < S.W && gy < S.H) ? S.seg[(size_t)gy * S.W + gx] : -1;
    if (lab[i] >= 0 && lab[i] <= ms) pend |= 1u << i;
  }
  label_rounds(lab, pend, [&](int k, unsigned, int src) {
    if ((int)(threadIdx.x & 31) == src) S.living[k] = 1;
  });
}

// find_most_similar_spix (relabel.cu:201-276): grid (s, candidate chunk of
// kRelabelChunk previous superpixels).  A block stages its chunk's prior colours and
// skip flags in shared memory, then every thread scans the chunk for its s.
__global__ void kb_relabel_compare(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Z;
  if (!S.mode) return;
  const SpDev& sp = S.sp;
  const int n_prev = S.n_prev;
  const int c0 = blockIdx.y * kRelabelChunk;
  if (c0 >= n_prev) return;
  const int nspix = S.sc->max_spix + 1;
  if ((int)(blockIdx.x * blockDim.x) >= min(nspix, sp.cap)) return;   // block-uniform
  const uint8_t* __restrict__ living = S.living;
  const float* __restrict__ prev_prior_mu_app = S.pprev.prior_mu_app;
  __shared__ float cmu[3][kRelabelChunk];
  __shared__ uint8_t cskip[kRelabelChunk];
  const int nc = min(n_prev - c0, kRelabelChunk);
  for (int i = threadIdx.x; i < nc; i += blockDim.x) {
    const int c = c0 + i;
    cskip[i] = c < nspix && living[c];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) cmu[ch][i] = prev_prior_mu_app[3 * c + ch];
  }
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nspix || s >= sp.cap || !living[s]) return;
  const float mx = sp.mu_app[3 * s], my = sp.mu_app[3 * s + 1], mz = sp.mu_app[3 * s + 2];
  unsigned long long b = ~0ull;
  for (int i = 0; i < nc; i++) {
    const int c = c0 + i;
    const bool same = (c == s);
    if (cskip[i] && !same) continue;
    const float dx = mx - cmu[0][i];
    const float dy = my - cmu[1][i];
    const float dz = mz - cmu[2][i];
    const float delta = (dx * dx + dy * dy + dz * dz);
    if (same) S.ss[s] = delta;
    if (delta < 10000.f) {
      const unsigned long long key = ((unsigned long long)__float_as_uint(delta) << 32) | (unsigned)c;
      if (key < b) b = key;
    }
  }
  if (b != ~0ull) atomicMin(&S.rbest[s], b);
}

// mark_for_relabel (relabel.cu:126-192): revive flags and mint flags.
__global__ void kb_relabel_mark(const Slot* __restrict__ slots, float thresh_replace,
                                float thresh_new) {
  pdl_enter();
  SLOT_Y;
  if (!S.mode) return;
  const int cap = S.cap;
  const Scalars* __restrict__ sc = S.sc;
  const uint8_t* __restrict__ living = S.living;
  const unsigned long long* __restrict__ best = S.rbest;
  const float* __restrict__ ss = S.ss;
  int* __restrict__ rid = S.rid;
  uint8_t* __restrict__ mint = S.mint;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= cap) return;
  mint[s] = 0;
  rid[s] = -1;
  const int nspix = sc->max_spix + 1;
  if (s >= nspix || !living[s]) return;
  unsigned long long b = best[s];
  float delta = __uint_as_float((unsigned)(b >> 32));
  int c = (int)(unsigned)(b & 0xffffffffull);
  bool revive = (delta < thresh_replace) && (c < nspix) && (c != s);
  if (revive) rid[s] = c;
  else if (ss[s] > thresh_new) mint[s] = 1;
}

__global__ void kb_relabel_ids(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.mode) return;
  const int cap = S.cap;
  Scalars* sc = S.sc;
  const uint8_t* __restrict__ mint = S.mint;
  const int* __restrict__ excl = S.excl;
  int* __restrict__ rid = S.rid;
  int* __restrict__ src_of = S.src_of;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= cap) return;
  if (mint[s]) rid[s] = sc->max_spix + 1 + excl[s];
  int n = rid[s];
  if (n >= 0 && n < cap) atomicMax(&src_of[n], s);
  else if (n >= cap) atomicExch(&sc->status, STSPIX_ERR_CAPACITY);
}

// relabel_spix_kernel parameter copies (relabel.cu:86-120), from the largest
// reviving superpixel.
__global__ void kb_relabel_params(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.mode) return;
  const SpDev& sp = S.sp;
  const int* __restrict__ rid = S.rid;
  const int* __restrict__ src_of = S.src_of;
  const int n_prev = S.n_prev;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= sp.cap) return;
  int n = rid[s];
  if (n < 0 || n >= sp.cap) return;
  sp.valid[s] = 0;
  if (src_of[n] != s) return;
  sp.count[n] = sp.count[s];
  sp.icount[n] = sp.icount[s];
  sp.valid[n] = 1;
  if (n >= n_prev) {
    sp.prop[n] = 0;
    sp.prior_count[n] = sp.prior_count[s];
    for (int c = 0; c < 3; c++) {
      sp.prior_sigma_shape[3 * n + c] = sp.prior_sigma_shape[3 * s + c];
      sp.sample_sigma_shape[3 * n + c] = sp.sample_sigma_shape[3 * s + c];
      sp.prior_mu_app[3 * n + c] = sp.prior_mu_app[3 * s + c];
      sp.prior_icov[3 * n + c] = sp.prior_icov[3 * s + c];
    }
  }
}

__global__ void kb_relabel_apply(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.mode) return;
  int* __restrict__ seg = S.seg;
  const int cap = S.cap;
  const int* __restrict__ rid = S.rid;
  FOR_PIX(t, S.npix) {
    const int v = seg[t];
    if (v < 0 || v >= cap) continue;
    const int n = rid[v];
    if (n >= 0 && n < cap) seg[t] = n;
  }
}

__global__ void kb_relabel_end(const Slot* __restrict__ slots, int B) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B || !slots[i].mode) return;
  Scalars* sc = slots[i].sc;
  // bump max_spix by the minted ids
  int m = sc->tmp2;
  sc->nminted += m;
  sc->max_spix += m;
}

__global__ void kb_count_revived(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.mode) return;
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S.cap) return;
  if (S.rid[s] >= 0 && !S.mint[s]) atomicAdd(&S.sc->nrevived, 1);
}

}  // namespace stspix
