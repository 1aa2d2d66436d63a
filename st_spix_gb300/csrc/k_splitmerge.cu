// GB300 kernels of the split / merge proposals and their Hastings tests
// (gauenk/st_spix st_spix/csrc/bist/split_merge.cu, split_merge_orig.cu,
// split_merge_prop.cu), plus a block-per-superpixel BFS that replaces the
// reference's host-driven BFS (one launch + one device-to-host copy per step).
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace stspix {


// ---------------------------------------------------------------------------
// Split seeds (init_split, split_merge.cu:803-844): seed s (0, 1) of superpixel k is
// the pixel one step from its mean position along +direction (s = 0) or -direction
// (s = 1), x for |direction| = 1 and y otherwise; -1 when that pixel is off the frame or
// not of label k.
__device__ __forceinline__ int split_seed_index(const Slot& S, int k, int s, int direction) {
  const int dir = s == 0 ? direction : -direction;
  int x = int(S.sp.mu_shape[2 * k]), y = int(S.sp.mu_shape[2 * k + 1]);
  if (dir == 1 || dir == -1) x += dir; else y += dir;
  const long long ind = (long long)y * S.W + x;
  if (ind < 0 || ind > (long long)S.W * S.H - 1) return -1;
  return S.seg[ind] == k ? (int)ind : -1;
}

__global__ void kb_split_seed(const Slot* __restrict__ slots, int dir_bass, int dir_prop) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const int direction = S.mode ? dir_prop : dir_bass;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sp.cap) return;
  int* bb = S.bbox + 4 * (size_t)k;
  bb[0] = INT32_MAX; bb[1] = -1; bb[2] = INT32_MAX; bb[3] = -1;
  if (!S.sc->tmp0 /*split_on*/ || !sp.valid[k]) return;
  for (int s = 0; s < 2; s++) {
    const int ind = split_seed_index(S, k, s, direction);
    if (ind >= 0) (s == 0 ? S.d1 : S.d2)[ind] = 1;
  }
}

// d1 = d2 = -1 (unreached) before the split seeds.
__global__ void kb_split_clear(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  FOR_PIX(t, S.npix) {
    S.d1[t] = -1;
    S.d2[t] = -1;
  }
}

__global__ void kb_split_begin(const Slot* __restrict__ slots, int B) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  Scalars* sc = slots[i].sc;
  // split runs unless max_spix > nspix_buffer / 2 (split_merge_orig.cu:215)
  sc->tmp0 = sc->max_spix > sc->nbuf_logical / 2 ? 0 : 1;
  sc->tmp1 = sc->max_spix + 1;  // offset of the second half
  sc->tmp2 = 0;                 // superpixels whose box is too large for one warp
}

// ---------------------------------------------------------------------------
// Bounding box of every superpixel (for the split BFS), by warp-block label rounds:
// a label's columns in the block are the lanes that hold it, its rows the union of
// their row masks; one set of min / max atomics per (block, label).
__global__ void __launch_bounds__(256) kb_bbox(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.sc->tmp0) return;
  const int H = S.H, W = S.W, cap = S.cap;
  int gx, by;
  if (!warp_block(W, H, gx, by)) return;
  const int lane = threadIdx.x & 31;
  const int bx = gx - lane;
  int lab[8];
  unsigned pend = 0;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int gy = by + i;
    lab[i] = (gx < W && gy < H) ? S.seg[(size_t)gy * W + gx] : -1;
    if (lab[i] >= 0 && lab[i] < cap) pend |= 1u << i;
  }
  label_rounds(lab, pend, [&](int k, unsigned m, int src) {
    const unsigned cols = __ballot_sync(0xffffffffu, m != 0);
    const unsigned rows = __reduce_or_sync(0xffffffffu, m);
    if (lane == src) {
      int* bb = S.bbox + 4 * (size_t)k;
      atomicMin(&bb[0], bx + __ffs(cols) - 1);
      atomicMax(&bb[1], bx + 31 - __clz(cols));
      atomicMin(&bb[2], by + __ffs(rows) - 1);
      atomicMax(&bb[3], by + 31 - __clz(rows));
    }
  });
}

// Split BFS (calc_split_candidate, split_merge.cu:758-800): distances from the two
// seeds of every superpixel, 4-connected within its label, seed = 1, unreached =
// -1 -- the reference's layered BFS, run per superpixel over its bounding box as a
// bit-parallel BFS: the box is held as rows of 64-bit words (label mask M, frontier
// F and visited V of each field), and one layer is
//     N = (F << 1 | F >> 1 | F[row-1] | F[row+1]) & M & ~V
// per word, so a layer costs O(rows x words) however the superpixel is shaped;
// each newly reached pixel gets distance L + 1 written once.
// kb_split_bfs runs one warp per superpixel with the box in registers (boxes up to
// 128 x 128 pixels, bfs_reg) and lists larger boxes for kb_split_bfs_big (one block
// each, the box in shared memory up to 512 x 512 pixels, bfs_bits; beyond that the same
// layers run on the global distances).
constexpr int kBigRows = 512, kBigWpr = 8;      // block: 512 rows x 8 words

template <int NT>
__device__ __forceinline__ void group_sync() {
  if (NT == 32) __syncwarp(); else __syncthreads();
}
template <int NT>
__device__ __forceinline__ int group_any(int v) {
  if (NT == 32) { __syncwarp(); return __any_sync(0xffffffffu, v); }
  return __syncthreads_or(v);
}

// t: thread index in the group of NT threads (NT a multiple of 32; whole warps).
// Arrays hold bh * wpr words each.
template <int NT, int ITEMS>
__device__ void bfs_bits(int t, int k, int x0, int y0, int bw, int bh, int W,
                         const int* __restrict__ seg, int* d1, int* d2,
                         unsigned long long* M, unsigned long long* F1, unsigned long long* V1,
                         unsigned long long* F2, unsigned long long* V2) {
  const int wpr = (bw + 63) >> 6;
  const int nwords = bh * wpr;
  const int lane = t & 31;
  // masks and seeds: one warp-wide ballot per 32-pixel chunk of a row
  const int cpr = (bw + 31) >> 5;
  unsigned* M32 = (unsigned*)M;
  unsigned* F132 = (unsigned*)F1;
  unsigned* F232 = (unsigned*)F2;
  for (int c = t >> 5; c < bh * cpr; c += NT >> 5) {
    const int r = c / cpr, cx = c % cpr;
    const int xi = cx * 32 + lane;
    bool m = false, s1 = false, s2 = false;
    if (xi < bw) {
      const int g = (y0 + r) * W + x0 + xi;
      m = seg[g] == k;
      if (m) { s1 = d1[g] == 1; s2 = d2[g] == 1; }
    }
    const unsigned bm = __ballot_sync(0xffffffffu, m);
    const unsigned b1 = __ballot_sync(0xffffffffu, s1);
    const unsigned b2 = __ballot_sync(0xffffffffu, s2);
    if (lane == 0) {
      const int w32 = r * wpr * 2 + cx;   // 32-bit half-word index (little endian)
      M32[w32] = bm; F132[w32] = b1; F232[w32] = b2;
    }
  }
  // zero the upper half of a row's last word when the row has an odd chunk count
  if (cpr & 1)
    for (int r = t; r < bh; r += NT) {
      const int w32 = r * wpr * 2 + cpr;
      M32[w32] = 0; F132[w32] = 0; F232[w32] = 0;
    }
  group_sync<NT>();
  for (int i = t; i < nwords; i += NT) { V1[i] = F1[i]; V2[i] = F2[i]; }
  group_sync<NT>();
  const int area = bw * bh;
  for (int L = 1; L <= area + 1; L++) {
    unsigned long long n1[ITEMS], n2[ITEMS];
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
      const int i = t + j * NT;
      n1[j] = n2[j] = 0;
      if (i < nwords) {
        const int r = i / wpr, w = i - r * wpr;
        const unsigned long long m = M[i];
        if (m) {
          unsigned long long f = F1[i];
          unsigned long long a = (f << 1) | (f >> 1);
          if (w > 0) a |= F1[i - 1] >> 63;
          if (w < wpr - 1) a |= F1[i + 1] << 63;
          if (r > 0) a |= F1[i - wpr];
          if (r < bh - 1) a |= F1[i + wpr];
          n1[j] = a & m & ~V1[i];
          f = F2[i];
          a = (f << 1) | (f >> 1);
          if (w > 0) a |= F2[i - 1] >> 63;
          if (w < wpr - 1) a |= F2[i + 1] << 63;
          if (r > 0) a |= F2[i - wpr];
          if (r < bh - 1) a |= F2[i + wpr];
          n2[j] = a & m & ~V2[i];
        }
      }
    }
    group_sync<NT>();
    int any = 0;
#pragma unroll
    for (int j = 0; j < ITEMS; j++) {
      const int i = t + j * NT;
      if (i < nwords) {
        F1[i] = n1[j];
        F2[i] = n2[j];
        if (n1[j] | n2[j]) {
          any = 1;
          V1[i] |= n1[j];
          V2[i] |= n2[j];
          const int r = i / wpr, w = i - r * wpr;
          const int gb = (y0 + r) * W + x0 + 64 * w;
          for (unsigned long long b = n1[j]; b; b &= b - 1) d1[gb + __ffsll((long long)b) - 1] = L + 1;
          for (unsigned long long b = n2[j]; b; b &= b - 1) d2[gb + __ffsll((long long)b) - 1] = L + 1;
        }
      }
    }
    if (!group_any<NT>(any)) break;
  }
}

// Boxes of at most 128 x 128 pixels (every superpixel of ordinary frames): the box is
// held in registers, lane l holding rows R l .. R l + R - 1 (R = 1..4 by the box height)
// as C 64-bit words each (C = 1, 2 by its width) of each field: label mask m, frontiers
// f1, f2 and visited v1, v2.  A layer is shifts within a row, the rows above and below
// from the lane's own rows or one shuffle, and the masks: no shared memory, no barrier.
// The seeds come as pixel indices (split_seed_index), so the box's distances are not
// read; only the comparison d1 > d2 is written, once, at the end.
template <int R, int C>
__device__ __forceinline__ void bfs_reg(int k, int x0, int y0, int bw, int bh, int W,
                                        const int* __restrict__ seg, int* d1, int* d2,
                                        int seed1, int seed2) {
  using u64 = unsigned long long;
  const int lane = threadIdx.x & 31;
  u64 m[R][C], f1[R][C], f2[R][C], v1[R][C], v2[R][C];
#pragma unroll
  for (int j = 0; j < R; j++)
#pragma unroll
    for (int w = 0; w < C; w++) m[j][w] = 0;
  // label mask: groups of 12 rows (R divides 12, so row rb + i sits in slot i % R of lane
  // (rb + i) / R), each row as 2C coalesced 32-pixel chunks, the group's loads issued
  // together
  constexpr int G = 12;
  for (int rb = 0; rb < bh; rb += G) {
    int v[G][2 * C];
#pragma unroll
    for (int i = 0; i < G; i++)
#pragma unroll
      for (int cx = 0; cx < 2 * C; cx++) {
        const int r = rb + i, xi = cx * 32 + lane;
        v[i][cx] = (r < bh && xi < bw) ? seg[(size_t)(y0 + r) * W + x0 + xi] : -1;
      }
#pragma unroll
    for (int i = 0; i < G; i++)
#pragma unroll
      for (int cx = 0; cx < 2 * C; cx++) {
        const unsigned b = __ballot_sync(0xffffffffu, v[i][cx] == k);
        if (lane == (rb + i) / R) m[i % R][cx >> 1] |= (u64)b << (32 * (cx & 1));
      }
  }
  {
    // seed bits: the owning lane's row slot and word as masks (a conditional write into
    // the arrays would put them in local memory)
    const int r1 = seed1 >= 0 ? seed1 / W - y0 - lane * R : -1, c1 = seed1 >= 0 ? seed1 % W - x0 : 0;
    const int r2 = seed2 >= 0 ? seed2 / W - y0 - lane * R : -1, c2 = seed2 >= 0 ? seed2 % W - x0 : 0;
    const u64 b1 = 1ull << (c1 & 63), b2 = 1ull << (c2 & 63);
#pragma unroll
    for (int j = 0; j < R; j++)
#pragma unroll
      for (int w = 0; w < C; w++) {
        f1[j][w] = b1 & (0ull - (u64)(r1 == j && (c1 >> 6) == w));
        f2[j][w] = b2 & (0ull - (u64)(r2 == j && (c2 >> 6) == w));
      }
  }
#pragma unroll
  for (int j = 0; j < R; j++)
#pragma unroll
    for (int w = 0; w < C; w++) { v1[j][w] = f1[j][w]; v2[j][w] = f2[j][w]; }
  auto layer = [&](u64 (&f)[R][C], u64 (&v)[R][C]) {
    u64 n[R][C];
#pragma unroll
    for (int w = 0; w < C; w++) {
      u64 up = __shfl_up_sync(0xffffffffu, f[R - 1][w], 1);
      u64 dn = __shfl_down_sync(0xffffffffu, f[0][w], 1);
      if (lane == 0) up = 0;
      if (lane == 31) dn = 0;
#pragma unroll
      for (int j = 0; j < R; j++) {
        u64 a = (f[j][w] << 1) | (f[j][w] >> 1);
        if (w > 0) a |= f[j][w - 1] >> 63;
        if (w < C - 1) a |= f[j][w + 1] << 63;
        a |= j > 0 ? f[j - 1][w] : up;
        a |= j < R - 1 ? f[j + 1][w] : dn;
        n[j][w] = a & m[j][w] & ~v[j][w];
      }
    }
    u64 any = 0;
#pragma unroll
    for (int j = 0; j < R; j++)
#pragma unroll
      for (int w = 0; w < C; w++) { f[j][w] = n[j][w]; v[j][w] |= n[j][w]; any |= n[j][w]; }
    return any;
  };
  // The split's only use of the distances is d1 > d2 (kb_split_partition): true where seed
  // 1 reaches a pixel and seed 2 reaches it strictly later or never.  early2: pixels seed 2
  // reached in a layer where seed 1 had not (yet) reached them, seed 2 itself included.
  u64 early2[R][C];
#pragma unroll
  for (int j = 0; j < R; j++)
#pragma unroll
    for (int w = 0; w < C; w++) early2[j][w] = f2[j][w] & ~f1[j][w];
  const int area = bw * bh;
  for (int L = 1; L <= area + 1; L++) {
    const u64 a1 = layer(f1, v1);
    const u64 a2 = layer(f2, v2);
#pragma unroll
    for (int j = 0; j < R; j++)
#pragma unroll
      for (int w = 0; w < C; w++) early2[j][w] |= f2[j][w] & ~v1[j][w];
    if (!__any_sync(0xffffffffu, (a1 | a2) != 0ull)) break;
  }
  // Distances that give the same comparison: d2 keeps -1 but 1 at seed 2 (kb_split_seed),
  // so d1 := 2 on the pixels with d1 > d2 and d1 := -1 at seed 1 when it has not.
#pragma unroll
  for (int j = 0; j < R; j++)
#pragma unroll
    for (int w = 0; w < C; w++) {
      const u64 second = v1[j][w] & (~v2[j][w] | early2[j][w]);
      if (second) {
        int* row = d1 + (size_t)(y0 + lane * R + j) * W + x0 + 64 * w;
        for (u64 b = second; b; b &= b - 1) row[__ffsll((long long)b) - 1] = 2;
      }
    }
  if (seed1 >= 0) {
    // the seed's word selected by masks (an indexed read would put the arrays in local
    // memory)
    const int r1 = seed1 / W - y0 - lane * R, c1 = seed1 % W - x0;
    u64 word = 0;
#pragma unroll
    for (int j = 0; j < R; j++)
#pragma unroll
      for (int w = 0; w < C; w++)
        word |= (v1[j][w] & (~v2[j][w] | early2[j][w])) &
                (0ull - (u64)(r1 == j && (c1 >> 6) == w));
    if (r1 >= 0 && r1 < R && !((word >> (c1 & 63)) & 1ull)) d1[seed1] = -1;
  }
}

__global__ void __launch_bounds__(128, 4) kb_split_bfs(const Slot* __restrict__ slots, int dir_bass,
                                                    int dir_prop) {
  pdl_enter();
  SLOT_Y;
  if (!S.sc->tmp0) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int direction = S.mode ? dir_prop : dir_bass;
  const int n = min(S.cap, S.sc->max_spix + 1);
  for (int k = blockIdx.x * 4 + warp; k < n; k += gridDim.x * 4) {
    if (!S.sp.valid[k]) continue;
    const int* bb = S.bbox + 4 * (size_t)k;
    const int x0 = bb[0], x1 = bb[1], y0 = bb[2], y1 = bb[3];
    if (x1 < x0 || y1 < y0) continue;
    const int bw = x1 - x0 + 1, bh = y1 - y0 + 1;
    if (bw > 128 || bh > 128) {
      if (lane == 0) S.sm.newid[atomicAdd(&S.sc->tmp2, 1)] = k;
      continue;
    }
    const int s1 = split_seed_index(S, k, 0, direction);
    const int s2 = split_seed_index(S, k, 1, direction);
    const int R = (bh + 31) >> 5;
    if (bw <= 64) {
      switch (R) {
        case 1: bfs_reg<1, 1>(k, x0, y0, bw, bh, S.W, S.seg, S.d1, S.d2, s1, s2); break;
        case 2: bfs_reg<2, 1>(k, x0, y0, bw, bh, S.W, S.seg, S.d1, S.d2, s1, s2); break;
        case 3: bfs_reg<3, 1>(k, x0, y0, bw, bh, S.W, S.seg, S.d1, S.d2, s1, s2); break;
        default: bfs_reg<4, 1>(k, x0, y0, bw, bh, S.W, S.seg, S.d1, S.d2, s1, s2); break;
      }
    } else {
      switch (R) {
        case 1: bfs_reg<1, 2>(k, x0, y0, bw, bh, S.W, S.seg, S.d1, S.d2, s1, s2); break;
        case 2: bfs_reg<2, 2>(k, x0, y0, bw, bh, S.W, S.seg, S.d1, S.d2, s1, s2); break;
        case 3: bfs_reg<3, 2>(k, x0, y0, bw, bh, S.W, S.seg, S.d1, S.d2, s1, s2); break;
        default: bfs_reg<4, 2>(k, x0, y0, bw, bh, S.W, S.seg, S.d1, S.d2, s1, s2); break;
      }
    }
  }
}

// Block per large box; dynamic shared memory of 5 * kBigRows * kBigWpr words.
__global__ void __launch_bounds__(256) kb_split_bfs_big(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.sc->tmp0) return;
  extern __shared__ unsigned long long big[];
  const int nbig = S.sc->tmp2;
  const int W = S.W;
  const int* seg = S.seg;
  int* d1 = S.d1;
  int* d2 = S.d2;
  constexpr int kA = kBigRows * kBigWpr;
  for (int j = blockIdx.x; j < nbig; j += gridDim.x) {
    const int k = S.sm.newid[j];
    const int* bb = S.bbox + 4 * (size_t)k;
    const int x0 = bb[0], y0 = bb[2];
    const int bw = bb[1] - x0 + 1, bh = bb[3] - y0 + 1, area = bw * bh;
    if (bw <= 64 * kBigWpr && bh <= kBigRows) {
      bfs_bits<256, kA / 256>(threadIdx.x, k, x0, y0, bw, bh, W, seg, d1, d2, big, big + kA,
                              big + 2 * kA, big + 3 * kA, big + 4 * kA);
    } else {
      for (int L = 1; L <= area + 1; L++) {
        int ch = 0;
        for (int i = threadIdx.x; i < area; i += blockDim.x) {
          const int xi = i % bw, yi = i / bw;
          const int g = (y0 + yi) * W + x0 + xi;
          if (seg[g] != k) continue;
          const int a = __ldcg(d1 + g), b = __ldcg(d2 + g);
          if (a >= 0 && b >= 0) continue;
          bool h1 = false, h2 = false;
          auto look = [&](int q) {
            if (seg[q] != k) return;
            if (__ldcg(d1 + q) == L) h1 = true;
            if (__ldcg(d2 + q) == L) h2 = true;
          };
          if (xi > 0) look(g - 1);
          if (xi < bw - 1) look(g + 1);
          if (yi > 0) look(g - W);
          if (yi < bh - 1) look(g + W);
          if (a < 0 && h1) { __stcg(d1 + g, L + 1); ch = 1; }
          if (b < 0 && h2) { __stcg(d2 + g, L + 1); ch = 1; }
        }
        if (!__syncthreads_or(ch)) break;
      }
    }
    __syncthreads();
  }
}

// calc_seg_split (split_merge.cu:847-859): second half when d1 > d2.
__global__ void kb_split_partition(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int off = S.sc->tmp1;
  FOR_PIX(t, S.npix) {
    int v = S.seg[t];
    if (S.d1[t] > S.d2[t]) v += off;
    S.smseg[t] = v;
  }
}

// Clear the split/merge sums (cap + 2 entries).
__global__ void kb_sm_clear(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SmDev& sm = S.sm;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.cap + 2) return;
  sm.count[k] = 0;
  sm.ninvalid[k] = 0;
#pragma unroll
  for (int c = 0; c < 3; c++) { sm.s[3 * (size_t)k + c] = 0; sm.sq[3 * (size_t)k + c] = 0; }
}

// sum_by_label over split/merge labels (split_merge.cu:862-891,
// split_merge_prop.cu:1942-2018): count, colour sums, square sums, invalid count.
// split: labels = split labels, invalid counts against the shifted labels (prop
// slots); merge: labels = current labels, ids < cap.
// Grid: the 64 x 32 tiles of a slot; warp w of a block owns the tile's 32 x 8 block
// (w & 1, w >> 1), a lane one column of it.  The warp takes the block's labels one at a
// time (the label of the lowest lane that still has pixels): each lane sums its pixels of
// that label, full-warp reductions add the lanes' sums, and one lane adds the totals with
// one set of atomics.  Unit colours (all of the warp's in [0, 1]) are summed in 32 bits;
// other colours wait in shared memory and a lane converts each pixel in its label's round.
// Integer sums (R1): totals do not depend on the grouping.
__global__ void __launch_bounds__(256, 4) kb_sm_accumulate(const Slot* __restrict__ slots, int split) {
  pdl_enter();
  SLOT_Y;
  __shared__ float cs[8][8][3][32];   // [warp][row][channel][lane]
  const int H = S.H, W = S.W;
  int gx, by;
  if (!warp_block(W, H, gx, by)) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int* __restrict__ labp = split ? S.smseg : S.seg;
  const int* __restrict__ shifted = (split && S.mode) ? S.shifted : nullptr;
  const float* __restrict__ img = S.img;
  const int cap = split ? S.cap + 2 : S.cap;
  const SmDev& sm = S.sm;
  float (*cw)[3][32] = cs[warp];
  int lab[8];
  float c[8][3];
  unsigned inv = 0, pend = 0;
  bool unit = true;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int gy = by + i;
    const bool in = gx < W && gy < H;
    const size_t g = (size_t)gy * W + gx;
    lab[i] = in ? labp[g] : -1;
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      c[i][ch] = in ? img[3 * g + ch] : 0.f;
      unit &= unit_colour(c[i][ch]);
    }
    if (shifted && in && shifted[g] < 0) inv |= 1u << i;
    if (lab[i] >= 0 && lab[i] < cap) pend |= 1u << i;
  }
  auto add = [&](int k, unsigned m, int src, const long long (&St)[3], const long long (&Qt)[3]) {
    const int N = __reduce_add_sync(0xffffffffu, __popc(m));
    const int NI = shifted ? __reduce_add_sync(0xffffffffu, __popc(m & inv)) : 0;
    if (lane == src) {
      atomicAdd(&sm.count[k], N);
      if (NI) atomicAdd(&sm.ninvalid[k], NI);
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        atomicAdd((unsigned long long*)&sm.s[3 * (size_t)k + ch], (unsigned long long)St[ch]);
        atomicAdd((unsigned long long*)&sm.sq[3 * (size_t)k + ch], (unsigned long long)Qt[ch]);
      }
    }
  };
  if (__all_sync(0xffffffffu, unit)) {
    unsigned qs[8][3], qq[8][3];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        qs[i][ch] = fx_unit(c[i][ch], kFxAppShift);
        qq[i][ch] = fx_unit(c[i][ch] * c[i][ch], kFxSqShift);
      }
    label_rounds(lab, pend, [&](int k, unsigned m, int src) {
      unsigned s[3] = {0, 0, 0}, q[3] = {0, 0, 0};
#pragma unroll
      for (int i = 0; i < 8; i++)
        if ((m >> i) & 1u) {
#pragma unroll
          for (int ch = 0; ch < 3; ch++) { s[ch] += qs[i][ch]; q[ch] += qq[i][ch]; }
        }
      long long St[3], Qt[3];
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        St[ch] = warp_sum_u32(s[ch]);
        Qt[ch] = (long long)__reduce_add_sync(0xffffffffu, q[ch]);
      }
      add(k, m, src, St, Qt);
    });
    return;
  }
  // other colours: 64-bit sums, the colours wait in shared memory and a lane converts
  // each of its pixels in the round of its label
#pragma unroll
  for (int i = 0; i < 8; i++)
#pragma unroll
    for (int ch = 0; ch < 3; ch++) cw[i][ch][lane] = c[i][ch];
  __syncwarp();
  label_rounds(lab, pend, [&](int k, unsigned m, int src) {
    long long s[3] = {0, 0, 0}, q[3] = {0, 0, 0};
    for (unsigned mm = m; mm; mm &= mm - 1) {
      const int i = __ffs(mm) - 1;
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        const float v = cw[i][ch][lane];
        s[ch] += fx_q(v, kFxAppShift);
        q[ch] += fx_q(v * v, kFxSqShift);
      }
    }
    long long St[3], Qt[3];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) { St[ch] = warp_sum64(s[ch]); Qt[ch] = warp_sum64(q[ch]); }
    add(k, m, src, St, Qt);
  });
}

// Marginal of one superpixel over the three colour channels, FP64: the
// reference's numerator - denominator (split_merge_orig.cu:536-549, 845-877) with
// the identical lgamma(a_n) terms cancelled and log b_0 - log b_n evaluated as
// -log1p((b_n - b_0) / b_0); b_n = b_0 + 0.5 (sum v^2 - (sum v)^2 / n)
// (:480-501).  `clamp` is the merge path's b_n < 0 -> 0.1 rule.
// In two parts, so the decision kernels can spread one id's terms over warps: a channel's
// log ratio, and the sum over the channels in this order.
__device__ __forceinline__ double marginal_lr(double n, const SmConsts& K, long long s, long long sq,
                                              bool clamp) {
  const double S = fx_unq(s, kFxAppShift), Q = fx_unq(sq, kFxSqShift);
  const double d = 0.5 * (Q - S * S / n);
  return (clamp && K.b0 + d < 0) ? K.log_01_b0 : log1p(d / K.b0);
}
__device__ __forceinline__ double marginal_sum(double n, const SmConsts& K, double lr0, double lr1,
                                               double lr2, double logn) {
  const double a_n = 1e4 + n / 2;
  double t = 0;
  t += -a_n * lr0;
  t += -a_n * lr1;
  t += -a_n * lr2;
  return t + 3 * (-0.5 * logn - n * K.lc);
}
__device__ __forceinline__ bool near_tie(double h) { return fabs(h + 2.0) < 1e-6; }

// update_split_flag (split_merge_orig.cu:900-986) / update_split_flag_p
// (split_merge_prop.cu:3026-3149): decision only; ids by scan afterwards (R2).
// One block per 32 consecutive ids, the FP64 terms of an id spread over the 4 warps (this
// part issues FP64 slowly; each warp runs on its own scheduler): warp m < 3 the three
// channel log ratios of marginal m (0: k's half, 1: s's half, 2: the whole superpixel),
// warp 3 the three log counts; warp 0 then adds them in marginal_sum's order and
// decides.  Every value is the same expression as a single-thread evaluation.
__global__ void __launch_bounds__(128) kb_split_decide(const Slot* __restrict__ slots, SmConsts K,
                                                       float split_alpha) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  Scalars* sc = S.sc;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  if ((int)blockIdx.x * 32 >= sp.cap) return;             // block-uniform
  __shared__ double t_lr[3][3][32], t_log[3][32];
  // the preconditions, evaluated alike by every warp
  bool ok = false;
  int s = 0;
  double cnt[3] = {0, 0, 0};                                // k's half, s's half, whole
  if (k < sp.cap) {
    if (w == 0) S.accept[k] = 0;
    if (sc->tmp0 && sp.valid[k]) {
      s = k + sc->tmp1;
      if (s < sc->nbuf_logical && s < sp.cap + 2) {
        cnt[2] = sp.count[k];
        cnt[0] = sm.count[k];
        cnt[1] = sm.count[s];
        ok = cnt[2] >= 1 && cnt[0] >= 1 && cnt[1] >= 1 && cnt[2] == cnt[0] + cnt[1];
      }
    }
  }
  if (!__syncthreads_or(ok)) return;
  if (ok) {
    if (w < 3) {
#pragma unroll
      for (int c = 0; c < 3; c++) {
        long long sv, qv;
        if (w == 0) { sv = sm.s[3 * (size_t)k + c]; qv = sm.sq[3 * (size_t)k + c]; }
        else if (w == 1) { sv = sm.s[3 * (size_t)s + c]; qv = sm.sq[3 * (size_t)s + c]; }
        else { sv = sp.acc[8 * (size_t)k + c]; qv = sm.sq[3 * (size_t)k + c] + sm.sq[3 * (size_t)s + c]; }
        const double nm = w == 0 ? cnt[0] : (w == 1 ? cnt[1] : cnt[2]);
        t_lr[w][c][lane] = marginal_lr(nm, K, sv, qv, false);
      }
    } else {
#pragma unroll
      for (int m = 0; m < 3; m++) t_log[m][lane] = log(cnt[m]);
    }
  }
  __syncthreads();
  if (w != 0 || !ok) return;
  double mm[3];
#pragma unroll
  for (int m = 0; m < 3; m++)
    mm[m] = marginal_sum(cnt[m], K, t_lr[m][0][lane], t_lr[m][1][lane], t_lr[m][2][lane],
                         t_log[m][lane]);
  const double count_k = cnt[0], count_s = cnt[1];
  double h = mm[0] + mm[1] - mm[2] + split_alpha;
  uint8_t fl = 1;
  if (S.mode) {
    bool is_prop = sp.prop[k];
    int ninv_k = sm.ninvalid[k], ninv_s = sm.ninvalid[s];
    bool prop_k = (ninv_k <= ninv_s);
    float iperc_k = (float)(ninv_k / (1.0 * count_k));
    float iperc_s = (float)(ninv_k / (1.0 * count_s));  // reference uses ninvalid_k here
    float iperc = prop_k ? iperc_k : iperc_s;
    iperc = is_prop ? iperc : 1.0f;
    h = h - 2 * (1.0 - iperc);
    if (prop_k || !is_prop) fl |= 8;   // select
    if (prop_k) fl |= 16;              // keep prior count on k
  }
  if (near_tie(h)) atomicAdd(&sc->near_ties, 1);
  if (h > -2) S.accept[k] = fl;
}

// Split commit: new id = max_spix + 1 + rank (R2), prior counts.
__global__ void kb_split_commit(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  Scalars* sc = S.sc;
  const uint8_t* __restrict__ accept = S.accept;
  const int* __restrict__ excl = S.excl;
  const int prop_mode = S.mode;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sp.cap) return;
  uint8_t fl = accept[k];
  if (!fl) return;
  int snew = sc->max_spix + 1 + excl[k];
  sm.newid[k] = snew;
  if (snew >= sp.cap) { atomicExch(&sc->status, STSPIX_ERR_CAPACITY); sm.newid[k] = -1; return; }
  if (!prop_mode) {
    float pcn = (float)fmax(sp.prior_count[k] / 2.0, 8.0);
    sp.prior_count[k] = pcn;
    sp.prior_count[snew] = pcn;
  } else {
    float pc = sp.prior_count[k];
    float half = (float)fmax(pc / 2.0, 36.0);
    if (fl & 16) {
      sp.prior_count[k] = pc;
      sp.prior_count[snew] = (float)(pc / 2.);
    } else {
      sp.prior_count[k] = half;
      sp.prior_count[snew] = half;
      double pcs = half;
      sp.prior_icov[3 * k] = pcs; sp.prior_icov[3 * k + 1] = 0; sp.prior_icov[3 * k + 2] = pcs;
    }
    sp.prop[snew] = 0;
    sp.icount[k] = (float)(sp.icount[k] / 2.0);
    double pcs = sp.prior_count[snew];
    sp.prior_icov[3 * snew] = pcs; sp.prior_icov[3 * snew + 1] = 0; sp.prior_icov[3 * snew + 2] = pcs;
  }
  sp.valid[snew] = 1;
}

// split_sp (split_merge.cu:1002-1031) / split_sp_p (split_merge_prop.cu:2317-2350).
__global__ void kb_split_apply(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  int* __restrict__ seg = S.seg;
  const int* __restrict__ smseg = S.smseg;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  const Scalars* __restrict__ sc = S.sc;
  const uint8_t* __restrict__ accept = S.accept;
  const int prop_mode = S.mode;
  FOR_PIX(t, S.npix) {
    const int k = seg[t];
    if (k < 0 || k >= sp.cap) continue;
    const uint8_t fl = accept[k];
    if (!fl) continue;
    const int s = sm.newid[k];
    if (s < 0) continue;
    const int k2 = k + sc->tmp1;
    if (!prop_mode || (fl & 8)) {
      if (smseg[t] == k2) seg[t] = s;
    } else {
      if (smseg[t] == k) seg[t] = s;
    }
  }
}

__global__ void kb_split_end(const Slot* __restrict__ slots, int B) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  Scalars* sc = slots[i].sc;
  int n = sc->tmp2;
  sc->nsplits += n;
  sc->max_spix += n;
}

// ---------------------------------------------------------------------------
// Merge candidates (calc_merge_candidate, split_merge.cu:719-755;
// calc_merge_candidate_p, split_merge_prop.cu:1808-1845).
__global__ void kb_merge_candidates(const Slot* __restrict__ slots, int dir_bass, int dir_prop) {
  pdl_enter();
  SLOT_Y;
  const int* __restrict__ seg = S.seg;
  const uint8_t* __restrict__ border = S.border;
  const int H = S.H, W = S.W;
  const int prop_mode = S.mode;
  const int direction = prop_mode ? dir_prop : dir_bass;
  const uint8_t* __restrict__ prop = S.sp.prop;
  const int cap = S.cap;
  int* __restrict__ pair = S.sm.pair;
  FOR_PIX(idx, H * W) {
    if (!border[idx]) continue;
    const int x = idx % W, y = idx / W;
    const int C = seg[idx];
    if (C < 0 || C >= cap) continue;
    int Wl = -1;
    if (!prop_mode) {
      if (direction == 1) { if (y >= 0 && y < H - 1) Wl = seg[idx + W]; }
      else { if (x > 0 && x < W) Wl = seg[idx - 1]; }
      if (Wl >= cap) Wl = -1;
      if (Wl >= 0 && C != Wl) atomicMax(&pair[C], Wl);
    } else {
      if (direction == 1) { if (y > 1 && y < H - 2) Wl = seg[idx + W]; }
      else { if (x > 1 && x < W - 2) Wl = seg[idx - 1]; }
      if (Wl >= cap) Wl = -1;
      const bool pC = prop[C];
      const bool pW = (Wl >= 0) ? prop[Wl] : false;
      if (Wl >= 0 && C != Wl && pC != pW) atomicMax(&pair[C], Wl);
    }
  }
}

// Single-superpixel marginal, present only when k has its own candidate
// (calc_merge_stats_step0 computes b_n only then; split_merge_orig.cu:456-520).  One block
// per 32 ids: warps 0-2 one channel's log ratio each, warp 3 the log count, warp 0 adds.
__global__ void __launch_bounds__(128) kb_merge_single(const Slot* __restrict__ slots, SmConsts K) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  if ((int)blockIdx.x * 32 >= sp.cap) return;             // block-uniform
  __shared__ double t_lr[3][32], t_log[32];
  bool ok = false;
  double n = 0;
  if (k < sp.cap) {
    if (w == 0) sm.flag[k] = 0;
    ok = sp.valid[k] && sm.pair[k] >= 0;
    if (ok) n = sp.count[k];
  }
  if (!__syncthreads_or(ok)) return;
  if (ok) {
    if (w < 3) t_lr[w][lane] = marginal_lr(n, K, sp.acc[8 * (size_t)k + w], sm.sq[3 * (size_t)k + w], true);
    else t_log[lane] = log(n);
  }
  __syncthreads();
  if (w != 0 || !ok) return;
  sm.msingle[k] = marginal_sum(n, K, t_lr[0][lane], t_lr[1][lane], t_lr[2][lane], t_log[lane]);
  sm.flag[k] = 16;
}

// calc_merge_stats_step2 + update_merge_flag (split_merge_orig.cu:555-656), R3.  One
// block per 32 ids (only valid ids decide, and none lies above the largest id in use):
// warps 0-2 one channel's log ratio of the merged pair each, warp 3 the log count, warp 0
// adds and decides.
__global__ void __launch_bounds__(128) kb_merge_decide(const Slot* __restrict__ slots, SmConsts K,
                                                       float merge_alpha) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  Scalars* sc = S.sc;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = blockIdx.x * 32 + lane;
  const int n_ids = min(sp.cap, sc->max_spix + 1);
  if ((int)blockIdx.x * 32 >= n_ids) return;              // block-uniform
  __shared__ double t_lr[3][32], t_log[32];
  bool ok = false;
  int f = -1;
  double count_k = 0, count_f = 0;
  if (k < n_ids && sp.valid[k]) {
    f = sm.pair[k];
    if (f >= 0 && sp.valid[f]) {
      count_k = sp.count[k];
      count_f = sp.count[k] + sp.count[f];
      ok = count_k >= 1 && count_f >= 1;
    }
  }
  if (!__syncthreads_or(ok)) return;
  const bool calc = ok && (sm.flag[f] & 16);
  if (calc) {
    if (w < 3) {
      const long long sv = sp.acc[8 * (size_t)k + w] + sp.acc[8 * (size_t)f + w];
      const long long qv = sm.sq[3 * (size_t)k + w] + sm.sq[3 * (size_t)f + w];
      t_lr[w][lane] = marginal_lr(count_f, K, sv, qv, true);
    } else {
      t_log[lane] = log(count_f);
    }
  }
  __syncthreads();
  if (w != 0 || !ok) return;
  double h;
  if (!calc) {
    h = -INFINITY;
  } else {
    const double m_merged =
        marginal_sum(count_f, K, t_lr[0][lane], t_lr[1][lane], t_lr[2][lane], t_log[lane]);
    h = m_merged - (K.log_alpha + sm.msingle[k] + sm.msingle[f]) + merge_alpha;
  }
  if (near_tie(h)) atomicAdd(&sc->near_ties, 1);
  if (h > -2) {
    sm.flag[k] |= 1;  // only thread k writes flag[k] here; readers use bit 16 only
    atomicMin(&sm.claim[f], k);
  }
}

// Merge set-up: candidate pairs unset, claims at +inf (cap + 2 entries).
__global__ void kb_merge_clear(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.cap + 2) return;
  S.sm.pair[k] = -1;
  S.sm.claim[k] = 0x7f7f7f7f;
}

// merge flag := accepted and claimant of its target; snapshot valid; target := pair.
__global__ void kb_merge_flag(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  uint8_t* __restrict__ valid0 = S.valid0;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sp.cap) return;
  valid0[k] = sp.valid[k];
  int f = sm.pair[k];
  sm.target[k] = f;
  uint8_t fl = sm.flag[k];
  if ((fl & 1) && f >= 0 && sm.claim[f] == k) fl |= 2;
  sm.flag[k] = fl;
}

// remove_sp (split_merge.cu:1035-1080) / remove_sp_p (split_merge_prop.cu:2353-2449).
__global__ void kb_merge_remove(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  Scalars* sc = S.sc;
  const uint8_t* __restrict__ valid0 = S.valid0;
  const int prop_mode = S.mode;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sp.cap) return;
  int s = sm.pair[k];
  if (s < 0) return;
  bool is_cycle = sm.pair[s] == k;
  if (!valid0[k] || !valid0[s]) return;
  bool mk = sm.flag[k] & 2, ms = sm.flag[s] & 2;
  if (!prop_mode) {
    if (mk && (!ms || (is_cycle && k < s))) {
      sm.flag[k] |= 4;
      sp.valid[k] = 0;
      sp.prior_count[s] = sp.prior_count[k] + sp.prior_count[s];
      atomicAdd(&sc->nmerges, 1);
    }
  } else {
    bool cond_c = is_cycle && sp.prop[k];
    if (mk && (!ms || cond_c)) {
      int r = k, t = s;
      if (sp.prop[k]) { sm.target[s] = k; r = s; t = k; }
      sm.flag[r] |= 4;  // each superpixel has at most one remover (single writer)
      sp.valid[r] = 0;
      sp.prior_count[t] = sp.prior_count[r] + sp.prior_count[t];
      atomicAdd(&sc->nmerges, 1);
    }
  }
}

// merge_sp (split_merge.cu:984-1000).
__global__ void kb_merge_apply(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  int* __restrict__ seg = S.seg;
  const int cap = S.cap;
  const SmDev& sm = S.sm;
  FOR_PIX(t, S.npix) {
    const int k = seg[t];
    if (k < 0 || k >= cap) continue;
    if (sm.flag[k] & 4) seg[t] = sm.target[k];
  }
}

}  // namespace stspix
