// GB300 kernels of the split / merge proposals and their Hastings tests
// (gauenk/st_spix st_spix/csrc/bist/split_merge.cu, split_merge_orig.cu,
// split_merge_prop.cu), plus the bounded cooperative relaxation loops that replace
// the reference's host-driven BFS (one launch + one device-to-host copy per step).
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace stspix {

constexpr int kTile = 32;
constexpr int kHalo = kTile + 2;
constexpr int kInf = 0x3fffffff;

// ---------------------------------------------------------------------------
// Split seeds (init_split, split_merge.cu:803-844) for both directions.
__global__ void kb_split_seed(const Slot* __restrict__ slots, int dir_bass, int dir_prop) {
  SLOT_Y;
  const SpDev& sp = S.sp;
  const int* __restrict__ seg = S.seg;
  const int H = S.H, W = S.W;
  const int direction = S.mode ? dir_prop : dir_bass;
  int* __restrict__ d1 = S.d1;
  int* __restrict__ d2 = S.d2;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sp.cap || !S.sc->tmp0 /*split_on*/ || !sp.valid[k]) return;
  for (int s = 0; s < 2; s++) {
    int dir = s == 0 ? direction : -direction;
    int x, y;
    if (dir == 1 || dir == -1) {
      x = int(sp.mu_shape[2 * k]) + dir;
      y = int(sp.mu_shape[2 * k + 1]);
    } else {
      x = int(sp.mu_shape[2 * k]);
      y = int(sp.mu_shape[2 * k + 1]) + dir;
    }
    long long ind = (long long)y * W + x;
    if (ind < 0 || ind > (long long)W * H - 1) continue;
    if (seg[ind] != k) continue;
    (s == 0 ? d1 : d2)[ind] = 1;
  }
}

// d1 = d2 = -1 (unreached) before the split seeds.
__global__ void kb_split_clear(const Slot* __restrict__ slots) {
  SLOT_Y;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.npix) return;
  S.d1[t] = -1;
  S.d2[t] = -1;
}

__global__ void kb_split_begin(const Slot* __restrict__ slots, int B) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  Scalars* sc = slots[i].sc;
  // split runs unless max_spix > nspix_buffer / 2 (split_merge_orig.cu:215)
  sc->tmp0 = sc->max_spix > sc->nbuf_logical / 2 ? 0 : 1;
  sc->tmp1 = sc->max_spix + 1;  // offset of the second half
}

// ---------------------------------------------------------------------------
// Relaxation to a fixed point inside 32x32 tiles with a one-pixel halo, repeated
// over the grid until no tile changes (cooperative launch, bounded barrier).
// mode 0: BFS distances of two seed fields (4-connected, same label, +1 per step;
//         -1 = unreached) -- the fixed point equals the reference's layered BFS
//         (calc_split_candidate, split_merge.cu:758-800).
// mode 1: connected-component roots (8-connected, same label, min pixel index) --
//         the fixed point of find_spix_min (split_disconnected.cu:458-498).
// Slot of flattened work item t (slots[i].base ascending, slots[0].base == 0).
__device__ __forceinline__ int slot_of(const Slot* __restrict__ slots, int B, long long t) {
  int lo = 0, hi = B - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (slots[mid].tile_base <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// The tiles of every slot of the launch form one list (slot i owns tiles
// [tile_base_i, tile_base_i + tiles_i)); flags[r * (B + 1) + i] records that slot i
// changed in round r, flags[r * (B + 1) + B] that any slot did.  A slot that did not
// change in round r is at its fixed point (its tiles read final halos) and is
// skipped from round r + 1 on.  Row r + 1 is cleared by block 0 during round r; the
// caller clears row 0.
template <int MODE>
__device__ __forceinline__ void relax_coop(const Slot* __restrict__ slots, int B,
                                           int total_tiles, Scalars* ctl, int* flags,
                                           int max_rounds) {
  __shared__ int sl[kHalo * kHalo];
  __shared__ int s1[kHalo * kHalo];
  __shared__ int s2[MODE == 0 ? kHalo * kHalo : 1];
  __shared__ int any;
  const int row = B + 1;
  for (int round = 0; round < max_rounds; round++) {
    if (blockIdx.x == 0 && round + 1 < max_rounds)
      for (int i = threadIdx.x; i < row; i += blockDim.x) flags[(round + 1) * row + i] = 0;
    int cur_slot = -1, my_changed = 0;
    for (int t = blockIdx.x; t < total_tiles; t += gridDim.x) {
      const int si = slot_of(slots, B, t);
      if (si != cur_slot) {
        if (my_changed) { atomicOr(&flags[round * row + cur_slot], 1); atomicOr(&flags[round * row + B], 1); }
        cur_slot = si;
        my_changed = 0;
      }
      if (round > 0 && *(volatile int*)&flags[(round - 1) * row + si] == 0) continue;
      const Slot& S = slots[si];
      const int H = S.H, W = S.W;
      const int* __restrict__ seg = S.seg;
      int* f1 = S.d1;
      int* f2 = S.d2;
      const int tiles_x = (W + kTile - 1) / kTile;
      const int tl = t - S.tile_base;
      const int tx0 = (tl % tiles_x) * kTile, ty0 = (tl / tiles_x) * kTile;
      for (int i = threadIdx.x; i < kHalo * kHalo; i += blockDim.x) {
        int gx = tx0 + i % kHalo - 1, gy = ty0 + i / kHalo - 1;
        if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
          int g = gy * W + gx;
          sl[i] = seg[g];
          // f1/f2 are written by other blocks of this launch: read past L1.
          if (MODE == 0) {
            int a = __ldcg(f1 + g), b = __ldcg(f2 + g);
            s1[i] = a < 0 ? kInf : a;
            s2[i] = b < 0 ? kInf : b;
          } else {
            int a = __ldcg(f1 + g);
            s1[i] = a < 0 ? kInf : a;
          }
        } else {
          sl[i] = INT32_MIN;
          s1[i] = kInf;
          if (MODE == 0) s2[i] = kInf;
        }
      }
      int local_iter = 0;
      while (true) {
        __syncthreads();
        if (threadIdx.x == 0) any = 0;
        __syncthreads();
        int ch = 0;
        for (int i = threadIdx.x; i < kTile * kTile; i += blockDim.x) {
          int lx = i % kTile + 1, ly = i / kTile + 1;
          if (tx0 + lx - 1 >= W || ty0 + ly - 1 >= H) continue;
          int p = ly * kHalo + lx;
          int L = sl[p];
          if (MODE == 0) {
            int a = s1[p], b = s2[p];
            const int q4[4] = {p - kHalo, p - 1, p + kHalo, p + 1};
#pragma unroll
            for (int j = 0; j < 4; j++) {
              int q = q4[j];
              if (sl[q] != L) continue;
              int qa = s1[q], qb = s2[q];
              if (qa < kInf && qa + 1 < a) a = qa + 1;
              if (qb < kInf && qb + 1 < b) b = qb + 1;
            }
            if (a < s1[p]) { s1[p] = a; ch = 1; }
            if (b < s2[p]) { s2[p] = b; ch = 1; }
          } else {
            if (L < 0) continue;
            int a = s1[p];
#pragma unroll
            for (int dy = -1; dy <= 1; dy++)
#pragma unroll
              for (int dx = -1; dx <= 1; dx++) {
                int q = p + dy * kHalo + dx;
                if (sl[q] == L && s1[q] < a) a = s1[q];
              }
            if (a < s1[p]) { s1[p] = a; ch = 1; }
          }
        }
        if (ch) any = 1;
        __syncthreads();
        if (!any || ++local_iter > 4 * kTile * kTile) break;
      }
      // write back changed interior values
      for (int i = threadIdx.x; i < kTile * kTile; i += blockDim.x) {
        int lx = i % kTile + 1, ly = i / kTile + 1;
        int gx = tx0 + lx - 1, gy = ty0 + ly - 1;
        if (gx >= W || gy >= H) continue;
        int p = ly * kHalo + lx, g = gy * W + gx;
        if (MODE == 0) {
          int a = s1[p] >= kInf ? -1 : s1[p];
          int b = s2[p] >= kInf ? -1 : s2[p];
          if (a != __ldcg(f1 + g)) { __stcg(f1 + g, a); my_changed = 1; }
          if (b != __ldcg(f2 + g)) { __stcg(f2 + g, b); my_changed = 1; }
        } else {
          int a = s1[p] >= kInf ? -1 : s1[p];
          if (a != __ldcg(f1 + g)) { __stcg(f1 + g, a); my_changed = 1; }
        }
      }
      __syncthreads();
    }
    if (my_changed) { atomicOr(&flags[round * row + cur_slot], 1); atomicOr(&flags[round * row + B], 1); }
    if (!grid_barrier(ctl)) return;
    if (*(volatile int*)&flags[round * row + B] == 0) return;
  }
  // round cap reached: flag the slots still changing
  if (blockIdx.x == 0)
    for (int i = threadIdx.x; i < B; i += blockDim.x)
      if (flags[(max_rounds - 1) * row + i]) atomicExch(&slots[i].sc->status, STSPIX_ERR_ITER_LIMIT);
}

__global__ void __launch_bounds__(256) kb_relax_bfs(const Slot* __restrict__ slots, int B,
                                                    int total_tiles, Scalars* ctl, int* flags,
                                                    int max_rounds) {
  relax_coop<0>(slots, B, total_tiles, ctl, flags, max_rounds);
}
__global__ void __launch_bounds__(256) kb_relax_cc(const Slot* __restrict__ slots, int B,
                                                   int total_tiles, Scalars* ctl, int* flags,
                                                   int max_rounds) {
  relax_coop<1>(slots, B, total_tiles, ctl, flags, max_rounds);
}

// calc_seg_split (split_merge.cu:847-859): second half when d1 > d2.
__global__ void kb_split_partition(const Slot* __restrict__ slots) {
  SLOT_Y;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.npix) return;
  int v = S.seg[t];
  if (S.d1[t] > S.d2[t]) v += S.sc->tmp1;
  S.smseg[t] = v;
}

// Clear the split/merge sums (cap + 2 entries).
__global__ void kb_sm_clear(const Slot* __restrict__ slots) {
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
__global__ void kb_sm_accumulate(const Slot* __restrict__ slots, int split) {
  SLOT_Y;
  const float* __restrict__ img = S.img;
  const int* __restrict__ lab = split ? S.smseg : S.seg;
  const int* __restrict__ shifted = (split && S.mode) ? S.shifted : nullptr;
  const int H = S.H, W = S.W;
  const int cap = split ? S.cap + 2 : S.cap;
  const SmDev& sm = S.sm;
  constexpr int R = 16;
  const int cpr = (W + R - 1) / R;
  int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= H * cpr) return;
  int y = tid / cpr, xs = (tid % cpr) * R, xe = min(W, xs + R);
  const int* lrow = lab + (size_t)y * W;
  const float* irow = img + (size_t)y * W * 3;
  const int* shrow = shifted ? shifted + (size_t)y * W : nullptr;
  int cur = -1, n = 0, ninv = 0;
  long long s[3] = {0, 0, 0}, q[3] = {0, 0, 0};
  auto flush = [&]() {
    if (cur < 0 || cur >= cap) return;
    atomicAdd(&sm.count[cur], n);
    if (shrow) atomicAdd(&sm.ninvalid[cur], ninv);
    for (int c = 0; c < 3; c++) {
      atomicAdd((unsigned long long*)&sm.s[3 * (size_t)cur + c], (unsigned long long)s[c]);
      atomicAdd((unsigned long long*)&sm.sq[3 * (size_t)cur + c], (unsigned long long)q[c]);
    }
  };
  for (int x = xs; x < xe; x++) {
    int k = lrow[x];
    if (k != cur) {
      flush();
      cur = k; n = 0; ninv = 0;
      s[0] = s[1] = s[2] = q[0] = q[1] = q[2] = 0;
    }
    if (k >= 0) {
      n++;
      for (int c = 0; c < 3; c++) {
        float v = irow[3 * x + c];
        s[c] += fx_q(v, kFxAppShift);
        q[c] += fx_q(v * v, kFxSqShift);
      }
      if (shrow && shrow[x] < 0) ninv++;
    }
  }
  flush();
}

// Marginal of one superpixel over the three colour channels, FP64: the
// reference's numerator - denominator (split_merge_orig.cu:536-549, 845-877) with
// the identical lgamma(a_n) terms cancelled and log b_0 - log b_n evaluated as
// -log1p((b_n - b_0) / b_0); b_n = b_0 + 0.5 (sum v^2 - (sum v)^2 / n)
// (:480-501).  `clamp` is the merge path's b_n < 0 -> 0.1 rule.
__device__ __forceinline__ double total_marginal(double n, const SmConsts& K, const long long* s,
                                                 const long long* sq, bool clamp) {
  const double a_n = 1e4 + n / 2;
  double t = 0;
  for (int c = 0; c < 3; c++) {
    double S = fx_unq(s[c], kFxAppShift), Q = fx_unq(sq[c], kFxSqShift);
    double d = 0.5 * (Q - S * S / n);
    double lr = (clamp && K.b0 + d < 0) ? K.log_01_b0 : log1p(d / K.b0);
    t += -a_n * lr;
  }
  return t + 3 * (-0.5 * log(n) - n * K.lc);
}
__device__ __forceinline__ bool near_tie(double h) { return fabs(h + 2.0) < 1e-6; }

// update_split_flag (split_merge_orig.cu:900-986) / update_split_flag_p
// (split_merge_prop.cu:3026-3149): decision only; ids by scan afterwards (R2).
__device__ __forceinline__ void split_decide_one(const SpDev& sp, const SmDev& sm, Scalars* sc,
                                                 const SmConsts& K, float split_alpha,
                                                 int prop_mode, uint8_t* __restrict__ accept,
                                                 int k) {
  accept[k] = 0;
  if (!sc->tmp0 || !sp.valid[k]) return;
  const int off = sc->tmp1;
  int s = k + off;
  if (s >= sc->nbuf_logical || s >= sp.cap + 2) return;
  double count_f = sp.count[k], count_k = sm.count[k], count_s = sm.count[s];
  if (count_f < 1 || count_k < 1 || count_s < 1) return;
  if (count_f != count_k + count_s) return;
  long long sq_f[3];
  for (int c = 0; c < 3; c++) sq_f[c] = sm.sq[3 * (size_t)k + c] + sm.sq[3 * (size_t)s + c];
  double mk = total_marginal(count_k, K, &sm.s[3 * (size_t)k], &sm.sq[3 * (size_t)k], false);
  double ms = total_marginal(count_s, K, &sm.s[3 * (size_t)s], &sm.sq[3 * (size_t)s], false);
  double mf = total_marginal(count_f, K, sp.acc + 8 * (size_t)k, sq_f, false);
  double h = mk + ms - mf + split_alpha;
  uint8_t fl = 1;
  if (prop_mode) {
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
  if (h > -2) accept[k] = fl;
}

__global__ void kb_split_decide(const Slot* __restrict__ slots, SmConsts K, float split_alpha) {
  SLOT_Y;
  FOR_SP(k, S.sp.cap) split_decide_one(S.sp, S.sm, S.sc, K, split_alpha, S.mode, S.accept, k);
}

// Split commit: new id = max_spix + 1 + rank (R2), prior counts.
__global__ void kb_split_commit(const Slot* __restrict__ slots) {
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
  SLOT_Y;
  int* __restrict__ seg = S.seg;
  const int* __restrict__ smseg = S.smseg;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  const Scalars* __restrict__ sc = S.sc;
  const uint8_t* __restrict__ accept = S.accept;
  const int prop_mode = S.mode;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.npix) return;
  int k = seg[t];
  if (k < 0 || k >= sp.cap) return;
  uint8_t fl = accept[k];
  if (!fl) return;
  int s = sm.newid[k];
  if (s < 0) return;
  int k2 = k + sc->tmp1;
  if (!prop_mode || (fl & 8)) {
    if (smseg[t] == k2) seg[t] = s;
  } else {
    if (smseg[t] == k) seg[t] = s;
  }
}

__global__ void kb_split_end(const Slot* __restrict__ slots, int B) {
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
  SLOT_Y;
  const int* __restrict__ seg = S.seg;
  const uint8_t* __restrict__ border = S.border;
  const int H = S.H, W = S.W;
  const int prop_mode = S.mode;
  const int direction = prop_mode ? dir_prop : dir_bass;
  const uint8_t* __restrict__ prop = S.sp.prop;
  const int cap = S.cap;
  int* __restrict__ pair = S.sm.pair;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= H * W || !border[idx]) return;
  int x = idx % W, y = idx / W;
  int C = seg[idx];
  if (C < 0 || C >= cap) return;
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
    bool pC = prop[C];
    bool pW = (Wl >= 0) ? prop[Wl] : false;
    if (Wl >= 0 && C != Wl && pC != pW) atomicMax(&pair[C], Wl);
  }
}

// Single-superpixel marginal, present only when k has its own candidate
// (calc_merge_stats_step0 computes b_n only then; split_merge_orig.cu:456-520).
__global__ void kb_merge_single(const Slot* __restrict__ slots, SmConsts K) {
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SmDev& sm = S.sm;
  FOR_SP(k, sp.cap) {
    sm.flag[k] = 0;
    if (!sp.valid[k] || sm.pair[k] < 0) continue;
    sm.msingle[k] = total_marginal(sp.count[k], K, sp.acc + 8 * (size_t)k,
                                   &sm.sq[3 * (size_t)k], true);
    sm.flag[k] = 16;
  }
}

// calc_merge_stats_step2 + update_merge_flag (split_merge_orig.cu:555-656), R3.
__device__ __forceinline__ void merge_decide_one(const SpDev& sp, const SmDev& sm, Scalars* sc,
                                                 const SmConsts& K, float merge_alpha, int k) {
  if (!sp.valid[k]) return;
  int f = sm.pair[k];
  if (f < 0 || !sp.valid[f]) return;
  double count_k = sp.count[k];
  double count_f = sp.count[k] + sp.count[f];
  if (count_k < 1 || count_f < 1) return;
  long long s_f[3], sq_f[3];
  for (int c = 0; c < 3; c++) {
    s_f[c] = sp.acc[8 * (size_t)k + c] + sp.acc[8 * (size_t)f + c];
    sq_f[c] = sm.sq[3 * (size_t)k + c] + sm.sq[3 * (size_t)f + c];
  }
  double h;
  if (!(sm.flag[f] & 16)) {
    h = -INFINITY;
  } else {
    double m_merged = total_marginal(count_f, K, s_f, sq_f, true);
    h = m_merged - (K.log_alpha + sm.msingle[k] + sm.msingle[f]) + merge_alpha;
  }
  if (near_tie(h)) atomicAdd(&sc->near_ties, 1);
  if (h > -2) {
    sm.flag[k] |= 1;  // only thread k writes flag[k] here; readers use bit 16 only
    atomicMin(&sm.claim[f], k);
  }
}

__global__ void kb_merge_decide(const Slot* __restrict__ slots, SmConsts K, float merge_alpha) {
  SLOT_Y;
  FOR_SP(k, S.sp.cap) merge_decide_one(S.sp, S.sm, S.sc, K, merge_alpha, k);
}

// Merge set-up: candidate pairs unset, claims at +inf (cap + 2 entries).
__global__ void kb_merge_clear(const Slot* __restrict__ slots) {
  SLOT_Y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.cap + 2) return;
  S.sm.pair[k] = -1;
  S.sm.claim[k] = 0x7f7f7f7f;
}

// merge flag := accepted and claimant of its target; snapshot valid; target := pair.
__global__ void kb_merge_flag(const Slot* __restrict__ slots) {
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
  SLOT_Y;
  int* __restrict__ seg = S.seg;
  const int cap = S.cap;
  const SmDev& sm = S.sm;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.npix) return;
  int k = seg[t];
  if (k < 0 || k >= cap) return;
  if (sm.flag[k] & 4) seg[t] = sm.target[k];
}

}  // namespace stspix
