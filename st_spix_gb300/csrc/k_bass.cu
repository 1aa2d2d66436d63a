// GB300 kernels of the per-frame BASS path: hex initialisation, compaction,
// sufficient statistics + posterior, boundary sweep, parameter read-out.
// Reference files cited per kernel (gauenk/st_spix, st_spix/csrc/bist/).
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace stspix {

// ---------------------------------------------------------------------------
// Hex initialisation (init_seg.cu:48-75).  The reference tests every centre per
// pixel and keeps the LAST centre at the minimum distance; the nearest centre of
// this pointy-top hex lattice lies within one hexagon radius, so a 5x5 window of
// lattice sites around the pixel, scanned in ascending id order with the same
// `<=` rule and the same double arithmetic, gives the identical label.
// Nearest hexagon centre of pixel (x, y) (InitHexSeg, init_seg.cu:63-75): the
// reference scans every centre in FP64 and keeps the last one at the smallest
// squared distance.  Only the 5x5 lattice neighbourhood of the pixel can hold the
// nearest centre; an FP32 pass finds the smallest distance there, and only the
// centres within an error margin of it are evaluated in FP64 with the reference's
// rule, in the same scan order.  With |dx|, |dy| < 3 hexagon sizes s and centre
// coordinates below x + y + 3s, the FP32 squared distance errs by less than
// ~5e-6 s (x + y + 6s) + 1e-7 d2 px^2; the margin below exceeds twice that, so
// every FP64 minimiser passes the filter and the label is the reference's.
// r0, c0: the search window's centre row floor(y / (1.5 Hh)) and column floor(x / w).
__device__ __forceinline__ int hex_label_rc(int x, int y, double Hh, double w, int nx, int ny,
                                           int r0, int c0) {
  const float wf = (float)w, hf = (float)(1.5 * Hh), half = (float)(0.5 * w);
  const float xf = (float)x, yf = (float)y;
  float mn = 3.0e38f;
  for (int r = r0 - 2; r <= r0 + 2; r++) {
    if (r < 0 || r >= ny) continue;
    for (int c = c0 - 2; c <= c0 + 2; c++) {
      if (c < 0 || c >= nx) continue;
      const float dx = xf - ((float)c * wf + ((r % 2 == 0) ? half : 0.f));
      const float dy = yf - (float)r * hf;
      mn = fminf(mn, dx * dx + dy * dy);
    }
  }
  const float sz = wf + hf;
  const float lim = mn + 8.0f + 1e-5f * mn + 1e-5f * sz * (xf + yf + 8.0f * sz);
  double D2 = 1.7976931348623157e308;
  int best = 0;
  for (int r = r0 - 2; r <= r0 + 2; r++) {
    if (r < 0 || r >= ny) continue;
    for (int c = c0 - 2; c <= c0 + 2; c++) {
      if (c < 0 || c >= nx) continue;
      const float dxf = xf - ((float)c * wf + ((r % 2 == 0) ? half : 0.f));
      const float dyf = yf - (float)r * hf;
      if (dxf * dxf + dyf * dyf > lim) continue;
      double xx = double(c) * w;
      double yy = double(r) * 1.5 * Hh;
      if (r % 2 == 0) xx = xx + 0.5 * w;
      double dx = (x - xx);
      double dy = (y - yy);
      double d2 = dx * dx + dy * dy;
      if (d2 <= D2) { D2 = d2; best = r * nx + c; }
    }
  }
  return best;
}
__device__ __forceinline__ int hex_label(int x, int y, double Hh, double w, int nx, int ny) {
  return hex_label_rc(x, y, Hh, w, nx, ny, (int)floor(y / (1.5 * Hh)), (int)floor(x / w));
}

__global__ void k_init_hex(int* __restrict__ seg, int H, int W, double Hh, double w, int nx,
                           int ny) {
  pdl_enter();
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= H * W) return;
  seg[idx] = hex_label(idx % W, idx / W, Hh, w, nx, ny);
}

// Grid: the 64 x 32 tiles of a slot.  The window row depends on y only and the window
// column on x only, so a block computes those of its 32 rows and 64 columns once (two
// FP64 divisions per row or column instead of per pixel; this part issues FP64 slowly).
__global__ void __launch_bounds__(256) kb_init_hex(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  __shared__ int r0s[32], c0s[64];
  const int W = S.W, H = S.H;
  const int tiles_x = (W + 63) / 64;
  if ((int)blockIdx.x >= tiles_x * ((H + 31) / 32)) return;
  const int tx0 = (blockIdx.x % tiles_x) * 64, ty0 = (blockIdx.x / tiles_x) * 32;
  const double Hh = S.hex_h, w = S.hex_w;
  if (threadIdx.x < 32) r0s[threadIdx.x] = (int)floor((ty0 + (int)threadIdx.x) / (1.5 * Hh));
  else if (threadIdx.x < 96) c0s[threadIdx.x - 32] = (int)floor((tx0 + (int)threadIdx.x - 32) / w);
  __syncthreads();
  for (int i = threadIdx.x; i < 64 * 32; i += blockDim.x) {
    const int lx = i & 63, ly = i >> 6;
    const int x = tx0 + lx, y = ty0 + ly;
    if (x < W && y < H)
      S.seg[(size_t)y * W + x] =
          hex_label_rc(x, y, Hh, w, S.hex_nx, S.hex_ny, r0s[ly], c0s[lx]);
  }
}

// ---------------------------------------------------------------------------
// Compaction (compact_spix.cu:41-122, 196-290): flags of live ids in [lo, hi],
// exclusive scan, remap.
// mode 0: hex ids [0, nraw); mode 1: ids [lo, max_spix] of the finished frame.
__global__ void kb_mark_present(const Slot* __restrict__ slots, int mode) {
  pdl_enter();
  SLOT_Y;
  const int lo = mode == 0 ? 0 : S.lo;
  const int hi = mode == 0 ? S.nraw - 1 : min(S.sc->max_spix, S.cap - 1);
  FOR_PIX(i, S.npix) {
    // one store per run of equal labels (the run's first pixel)
    const int v = S.seg[i];
    if (v >= lo && v <= hi && (i == 0 || S.seg[i - 1] != v)) S.flags[v - lo] = 1;
  }
}

// One block per slot: exclusive scan of n byte flags (n up to a few 10^5), each
// counted as 0 or 1 (the split acceptance flags of propagated frames carry extra bits).
//   mode 0: hex-id presence (n = nraw)        -> total = live hex ids
//   mode 1: split acceptance (n = cap)        -> total = accepted splits
//   mode 2: relabel mint flags (n = cap)      -> total = minted ids
//   mode 3: final presence (n = max_spix+1-lo) -> total = live new ids
__global__ void kb_scan(const Slot* __restrict__ slots, int mode) {
  pdl_enter();
  const Slot& S = slots[blockIdx.x];
  if (mode == 2 && !S.mode) return;  // mint flags exist on propagated slots only
  __shared__ int part[1024];
  const int T = blockDim.x;
  const uint8_t* flags = (mode == 1) ? S.accept : (mode == 2) ? S.mint : S.flags;
  int n = (mode == 0) ? S.nraw : (mode == 3) ? S.sc->tmp2 : S.cap;
  int* excl = S.excl;
  int* total = (mode == 0) ? &S.sc->nspix : (mode == 3) ? &S.sc->tmp1 : &S.sc->tmp2;
  if (n < 0) n = 0;
  int chunk = (n + T - 1) / T;
  int b = threadIdx.x * chunk, e = min(n, b + chunk);
  int s = 0;
  for (int i = b; i < e; i++) s += flags[i] != 0;
  part[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {
    int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int i = b; i < e; i++) { excl[i] = run; run += flags[i] != 0; }
  if (threadIdx.x == T - 1) *total = part[T - 1];
}

__global__ void kb_remap(const Slot* __restrict__ slots, int mode) {
  pdl_enter();
  SLOT_Y;
  const int lo = mode == 0 ? 0 : S.lo;
  FOR_PIX(i, S.npix) {
    const int v = S.seg[i];
    if (v >= lo) S.seg[i] = lo + S.excl[v - lo];
  }
}

// fill_new_params_from_old (compact_spix.cu:220-265): gather moved fields.
__global__ void kb_compact_gather(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SpDev& tmp = S.tmp;
  const uint8_t* flags = S.flags;
  const int* excl = S.excl;
  const int lo = S.lo;
  int v = lo + blockIdx.x * blockDim.x + threadIdx.x;
  if (v > S.sc->max_spix || v >= sp.cap) return;
  if (!flags[v - lo]) return;
  int j = excl[v - lo];
  for (int c = 0; c < 3; c++) {
    tmp.mu_app[3 * j + c] = sp.mu_app[3 * v + c];
    tmp.prior_mu_app[3 * j + c] = sp.prior_mu_app[3 * v + c];
    tmp.sigma_shape[3 * j + c] = sp.sigma_shape[3 * v + c];
    tmp.prior_sigma_shape[3 * j + c] = sp.prior_sigma_shape[3 * v + c];
    tmp.sample_sigma_shape[3 * j + c] = sp.sample_sigma_shape[3 * v + c];
  }
  for (int c = 0; c < 2; c++) {
    tmp.mu_shape[2 * j + c] = sp.mu_shape[2 * v + c];
    tmp.prior_mu_shape[2 * j + c] = sp.prior_mu_shape[2 * v + c];
  }
  tmp.logdet[j] = sp.logdet[v];
  tmp.count[j] = sp.count[v];
  tmp.prior_count[j] = sp.prior_count[v];
  tmp.valid[j] = sp.valid[v];
}

// fill_old_params_from_new (compact_spix.cu:268-290).
__global__ void kb_compact_scatter(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const SpDev& tmp = S.tmp;
  const int lo = S.lo;
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= S.sc->tmp1) return;
  int d = lo + j;
  if (d >= sp.cap) return;
  for (int c = 0; c < 3; c++) {
    sp.mu_app[3 * d + c] = tmp.mu_app[3 * j + c];
    sp.prior_mu_app[3 * d + c] = tmp.prior_mu_app[3 * j + c];
    sp.sigma_shape[3 * d + c] = tmp.sigma_shape[3 * j + c];
    sp.prior_sigma_shape[3 * d + c] = tmp.prior_sigma_shape[3 * j + c];
    sp.sample_sigma_shape[3 * d + c] = tmp.sample_sigma_shape[3 * j + c];
  }
  for (int c = 0; c < 2; c++) {
    sp.mu_shape[2 * d + c] = tmp.mu_shape[2 * j + c];
    sp.prior_mu_shape[2 * d + c] = tmp.prior_mu_shape[2 * j + c];
  }
  sp.logdet[d] = tmp.logdet[j];
  sp.count[d] = tmp.count[j];
  sp.prior_count[d] = tmp.prior_count[j];
  sp.valid[d] = tmp.valid[j];
}

// ---------------------------------------------------------------------------
// init_sp_params_kernel + mark_active_contiguous (init_sparams.cu:45-166,
// 195-286) for a BASS frame; *nspix live ids, count = npix / nspix.
__global__ void kb_init_bass_params(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (S.mode) return;
  const int sp_size = S.sp_size;
  const SpDev& sp = S.sp;
  const int npix = S.npix;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sp.cap) return;
  int nspix = S.sc->nspix;
  int count = (int)(npix / (1. * nspix));
  sp.prior_sigma_shape[3 * k] = 1.0 / sp_size;
  sp.prior_sigma_shape[3 * k + 1] = 0.;
  sp.prior_sigma_shape[3 * k + 2] = 1.0 / sp_size;
  sp.prior_icov[3 * k] = 1; sp.prior_icov[3 * k + 1] = 0; sp.prior_icov[3 * k + 2] = 1;
  sp.prop[k] = 0;
  sp.icount[k] = 0.f;
  sp.sm_count[k] = 0;
  for (int c = 0; c < 3; c++) {
    sp.mu_app[3 * k + c] = 0.f; sp.prior_mu_app[3 * k + c] = 0.f;
    sp.sigma_shape[3 * k + c] = 0.0; sp.sample_sigma_shape[3 * k + c] = 0.0;
  }
  for (int c = 0; c < 2; c++) { sp.mu_shape[2 * k + c] = 0.0; sp.prior_mu_shape[2 * k + c] = 0.0; }
  sp.logdet[k] = 0.0;
  sp.count[k] = 0;
  if (k < nspix) { sp.valid[k] = 1; sp.prior_count[k] = (float)count; }
  else { sp.valid[k] = 0; sp.prior_count[k] = 0.f; }
}

// prior_mu_app := initial mean (calc_summ_stats, update_params.cu:142-203).
__global__ void kb_init_prior_mu(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (S.mode) return;
  const SpDev& sp = S.sp;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.sc->nspix || k >= sp.cap) return;
  int n = sp.count[k];
  double c = n;
  for (int ch = 0; ch < 3; ch++)
    sp.prior_mu_app[3 * k + ch] =
        n > 0 ? (float)(fx_unq(sp.acc[8 * k + ch], kFxAppShift) / c) : 0.f;
}

// ---------------------------------------------------------------------------
// Sufficient statistics (sum_by_label, update_params.cu:89-130), R1.  A warp owns a
// 32 x 8 block of a frame: lane = column, and it holds the block's 8 labels and colours
// of its column in registers (every load issued before any is used).  The warp then
// takes the block's labels one at a time (label_rounds): each lane sums its pixels of
// that label, the warp adds the lanes' sums with full-warp reductions (colour sums in
// 24-bit parts, positions relative to the block so they fit 32 bits) and one lane adds
// the label's totals to its global sums with one set of 64-bit atomics.  A block holds
// a few labels, so a few reductions and atomic sets serve 256 pixels.  Colours in
// [0, 1] are summed in 32 bits (one conversion each); others wait in the warp's shared
// staging rows `cw` and are converted and summed in 64 bits in their label's round.
// Integer sums: the totals do not depend on the grouping or the order of the adds.
__device__ __forceinline__ void block_stats(const Slot& S, int bx, int by, float (*cw)[3][32]) {
  const int lane = threadIdx.x & 31;
  const int H = S.H, W = S.W;
  const SpDev& sp = S.sp;
  const int cap = sp.cap;
  const int gx = bx + lane;
  int lab[8];
  float c[8][3];
  unsigned pend = 0;
  bool unit = true;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const int gy = by + i;
    const bool in = gx < W && gy < H;
    const size_t g = (size_t)gy * W + gx;
    lab[i] = in ? S.seg[g] : -1;
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      c[i][ch] = in ? S.img[3 * g + ch] : 0.f;
      unit &= unit_colour(c[i][ch]);
    }
    if (lab[i] >= 0 && lab[i] < cap) pend |= 1u << i;
  }
  // the warp's totals of label k given its colour sums: count and position moments
  // (relative to the block, so they fit 32 bits), one set of atomics
  auto add = [&](int k, unsigned m, int src, long long S0, long long S1, long long S2) {
    int sy = 0, syy = 0;
#pragma unroll
    for (int i = 0; i < 8; i++)
      if ((m >> i) & 1u) { sy += i; syy += i * i; }
    const int n = __popc(m);
    const int N = __reduce_add_sync(0xffffffffu, n);
    const int SX = __reduce_add_sync(0xffffffffu, n * lane);
    const int SXX = __reduce_add_sync(0xffffffffu, n * lane * lane);
    const int SY = __reduce_add_sync(0xffffffffu, sy);
    const int SYY = __reduce_add_sync(0xffffffffu, syy);
    const int SXY = __reduce_add_sync(0xffffffffu, lane * sy);
    if (lane == src) {
      const long long ln = N, X = bx, Y = by;
      unsigned long long* acc = (unsigned long long*)(sp.acc + 8 * (size_t)k);
      atomicAdd(&sp.count[k], N);
      atomicAdd(acc + 0, (unsigned long long)S0);
      atomicAdd(acc + 1, (unsigned long long)S1);
      atomicAdd(acc + 2, (unsigned long long)S2);
      atomicAdd(acc + 3, (unsigned long long)(ln * X + SX));
      atomicAdd(acc + 4, (unsigned long long)(ln * Y + SY));
      atomicAdd(acc + 5, (unsigned long long)(ln * X * X + 2 * X * SX + SXX));
      atomicAdd(acc + 6, (unsigned long long)(ln * X * Y + X * SY + Y * SX + SXY));
      atomicAdd(acc + 7, (unsigned long long)(ln * Y * Y + 2 * Y * SY + SYY));
    }
  };
  if (__all_sync(0xffffffffu, unit)) {
    unsigned q[8][3];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
      for (int ch = 0; ch < 3; ch++) q[i][ch] = fx_unit(c[i][ch], kFxAppShift);
    label_rounds(lab, pend, [&](int k, unsigned m, int src) {
      unsigned s0 = 0, s1 = 0, s2 = 0;
#pragma unroll
      for (int i = 0; i < 8; i++)
        if ((m >> i) & 1u) { s0 += q[i][0]; s1 += q[i][1]; s2 += q[i][2]; }
      add(k, m, src, warp_sum_u32(s0), warp_sum_u32(s1), warp_sum_u32(s2));
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
    long long s0 = 0, s1 = 0, s2 = 0;
    for (unsigned mm = m; mm; mm &= mm - 1) {
      const int i = __ffs(mm) - 1;
      s0 += fx_q(cw[i][0][lane], kFxAppShift);
      s1 += fx_q(cw[i][1][lane], kFxAppShift);
      s2 += fx_q(cw[i][2][lane], kFxAppShift);
    }
    add(k, m, src, warp_sum64(s0), warp_sum64(s1), warp_sum64(s2));
  });
}

// Grid: the 64 x 32 tiles of the first B slots (a block finds its slot by binary
// search over the slots' first tiles); warp w takes the tile's 32 x 8 block
// (w & 1, w >> 1).
__global__ void __launch_bounds__(256, 4) kb_accumulate(const Slot* __restrict__ slots, int B) {
  pdl_enter();
  if (B <= 0) return;
  const int t = blockIdx.x;
  int lo = 0, hi = B - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (slots[mid].tile_base[1] <= t) lo = mid; else hi = mid - 1;
  }
  const Slot& S = slots[lo];
  const int tl = t - S.tile_base[1];
  const int tiles_x = (S.W + 63) / 64;
  const int warp = threadIdx.x >> 5;
  __shared__ float cs[8][8][3][32];   // [warp][row][channel][lane]
  block_stats(S, (tl % tiles_x) * 64 + (warp & 1) * 32, (tl / tiles_x) * 32 + (warp >> 1) * 8,
              cs[warp]);
}

// Accumulator precision study: colour sums by per-pixel FP32 (mode 1, as the
// reference's sum_by_label, update_params.cu:115-117) or FP64 (mode 2) atomics into
// a scratch array (the compaction buffer's sums), then written over the int64 colour
// sums in 2^-28 units (exact for the magnitudes of colour sums), so the posterior sees
// the precision of that accumulator.  Counts and positions stay exact.
__global__ void kb_accumulate_fp(const Slot* __restrict__ slots, int mode) {
  pdl_enter();
  SLOT_Y;
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S.npix) return;
  const int k = S.seg[t];
  if (k < 0 || k >= S.sp.cap) return;
  const float* p = S.img + 3 * (size_t)t;
  if (mode == 1) {
    float* f = (float*)S.tmp.acc;
    for (int c = 0; c < 3; c++) atomicAdd(&f[3 * (size_t)k + c], p[c]);
  } else {
    double* d = (double*)S.tmp.acc;
    for (int c = 0; c < 3; c++) atomicAdd(&d[3 * (size_t)k + c], (double)p[c]);
  }
}

__global__ void kb_accumulate_fp_store(const Slot* __restrict__ slots, int mode) {
  pdl_enter();
  SLOT_Y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.sp.cap) return;
  for (int c = 0; c < 3; c++) {
    const double v = mode == 1 ? (double)((const float*)S.tmp.acc)[3 * (size_t)k + c]
                               : ((const double*)S.tmp.acc)[3 * (size_t)k + c];
    S.sp.acc[8 * (size_t)k + c] = __double2ll_rn(ldexp(v, kFxAppShift));
  }
}

__global__ void kb_accumulate_fp_clear(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.sp.cap) return;
  double* d = (double*)S.tmp.acc;
  for (int c = 0; c < 3; c++) d[3 * (size_t)k + c] = 0.0;
}

// Statistics of a labelling with a chosen accumulator (study entry point).
__global__ void k_label_stats(const float* __restrict__ img, const int* __restrict__ lab,
                              long long npix, int n, int mode, long long* iacc, float* facc,
                              double* dacc) {
  pdl_enter();
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const int k = lab[t];
  if (k < 0 || k >= n) return;
  const float* p = img + 3 * t;
  atomicAdd((unsigned long long*)&iacc[7 * (size_t)k], 1ull);
  for (int c = 0; c < 3; c++) {
    const float v = p[c];
    if (mode == 0) {
      atomicAdd((unsigned long long*)&iacc[7 * (size_t)k + 1 + c], (unsigned long long)fx_q(v, kFxAppShift));
      atomicAdd((unsigned long long*)&iacc[7 * (size_t)k + 4 + c], (unsigned long long)fx_q(v * v, kFxSqShift));
    } else if (mode == 1) {
      atomicAdd(&facc[7 * (size_t)k + 1 + c], v);
      atomicAdd(&facc[7 * (size_t)k + 4 + c], v * v);
    } else {
      atomicAdd(&dacc[7 * (size_t)k + 1 + c], (double)v);
      atomicAdd(&dacc[7 * (size_t)k + 4 + c], (double)v * (double)v);
    }
  }
}

__global__ void k_label_stats_out(int n, int mode, const long long* iacc, const float* facc,
                                  const double* dacc, double* out) {
  pdl_enter();
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  out[7 * (size_t)k] = (double)iacc[7 * (size_t)k];
  for (int c = 1; c < 7; c++) {
    double v;
    if (mode == 0) v = ldexp((double)iacc[7 * (size_t)k + c], c < 4 ? -kFxAppShift : -kFxSqShift);
    else if (mode == 1) v = facc[7 * (size_t)k + c];
    else v = dacc[7 * (size_t)k + c];
    out[7 * (size_t)k + c] = v;
  }
}

// ---------------------------------------------------------------------------
// Posterior (calc_simple_update, update_params.cu:220-381, with
// _add_sigma_smoothing :206-217) + clear_fields semantics for dead ids.
__device__ __forceinline__ void smooth_prior(double in_x, double in_y, double in_z, int count,
                                             float pc, int sp_size, double* ox, double* oy,
                                             double* oz) {
  int nf = 50;
  double total_count = 1. * (count + pc * nf);
  *ox = (pc * sp_size + count * in_x) / (total_count + 3.0);
  *oy = (count * in_y) / (total_count + 3.0);
  *oz = (pc * sp_size + count * in_z) / (total_count + 3.0);
}

// One block = 32 consecutive ids, four warps splitting each id's FP64 chain (this part
// issues FP64 slowly, so one warp per id set would serialise the whole chain on one
// scheduler): warp 0 the colour means, warp 1 the prior shape term, warp 2 the shape
// mean and scatter; then warps 0-2 one smoothed covariance entry each, then warps 0-2
// one inverse entry each and warp 3 the log determinant.  Every value is the same
// expression as a single-thread evaluation, exchanged through shared memory.
// k: this lane's id (-1: none).  cached: the prior shape term is read from S.pscache,
// which the last full posterior wrote (incremental posteriors: the priors, flags and
// sample covariance it depends on change only in the steps followed by a full one).
__device__ __forceinline__ void posterior_ids(const Slot& S, int k, bool cached) {
  __shared__ double v_ps[3][32], v_raw[3][32], v_m[2][32], v_s[3][32], v_i[4][32];
  __shared__ float v_app[3][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const SpDev& sp = S.sp;
  const bool inr = k >= 0 && k < sp.cap;
  // every load of the id is issued before any is used (one memory round trip): the
  // count and flags, and the fields this warp's part of the posterior reads
  int count_int = 0;
  uint8_t valid = 0, prop = 0;
  float pc = 0.f;
  long long a0 = 0, a1 = 0, a2 = 0, a3 = 0, a4 = 0;
  double q0 = 0, q1 = 0, q2 = 0, i0 = 0, i1 = 0, i2 = 0;
  const long long* a = sp.acc + 8 * (size_t)k;
  if (inr) {
    count_int = sp.count[k];
    valid = sp.valid[k];
    if (w == 0) { a0 = a[0]; a1 = a[1]; a2 = a[2]; }
    else if (w == 1) {
      pc = sp.prior_count[k];
      if (cached) {
        q0 = S.pscache[3 * (size_t)k]; q1 = S.pscache[3 * (size_t)k + 1];
        q2 = S.pscache[3 * (size_t)k + 2];
      } else {
        prop = sp.prop[k];
        q0 = sp.sample_sigma_shape[3 * k]; q1 = sp.sample_sigma_shape[3 * k + 1];
        q2 = sp.sample_sigma_shape[3 * k + 2];
        i0 = sp.prior_icov[3 * k]; i1 = sp.prior_icov[3 * k + 1]; i2 = sp.prior_icov[3 * k + 2];
      }
    } else if (w == 2) { a0 = a[3]; a1 = a[4]; a2 = a[5]; a3 = a[6]; a4 = a[7]; }
    if (w != 1) pc = sp.prior_count[k];
  }
  const bool live = valid && count_int > 0;
  if (w == 0 && inr) {
    if (valid && count_int <= 0) sp.valid[k] = 0;
    if (!live) {
      for (int c = 0; c < 3; c++) { sp.mu_app[3 * k + c] = 0.f; sp.sigma_shape[3 * k + c] = 0.0; }
      sp.mu_shape[2 * k] = 0.0; sp.mu_shape[2 * k + 1] = 0.0;
    }
  }
  if (!__syncthreads_or(live)) return;
  const double count = count_int * 1.0;
  const double total_count = (double)count_int + pc * 50;
  if (live) {
    if (w == 0) {
      // colour means (fixed-point sums, R1)
      const long long ac[3] = {a0, a1, a2};
      for (int c = 0; c < 3; c++) {
        const float m = (float)(fx_unq(ac[c], kFxAppShift) / count);
        sp.mu_app[3 * k + c] = m;
        v_app[c][lane] = m;
      }
    } else if (w == 1) {
      // prior shape term (calc_simple_update with _add_sigma_smoothing)
      if (cached) {
        v_ps[0][lane] = q0; v_ps[1][lane] = q1; v_ps[2][lane] = q2;
      } else {
        double px, py, pz;
        if (prop) {
          smooth_prior(q0, q1, q2, (int)pc, pc, S.sp_size, &px, &py, &pz);
        } else {
          px = i0; py = i1; pz = i2;
        }
        double pr_det = px * pz - py * py;
        if (!(pr_det > 0)) atomicExch(&S.sc->status, STSPIX_ERR_DEGENERATE);
        pr_det = sqrt(pr_det);
        const double t0 = pc / pr_det * px, t1 = pc / pr_det * py, t2 = pc / pr_det * pz;
        v_ps[0][lane] = t0; v_ps[1][lane] = t1; v_ps[2][lane] = t2;
        S.pscache[3 * (size_t)k] = t0; S.pscache[3 * (size_t)k + 1] = t1;
        S.pscache[3 * (size_t)k + 2] = t2;
      }
    } else if (w == 2) {
      // shape mean and scatter
      const double mx = a0 / count, my = a1 / count;
      sp.mu_shape[2 * k] = mx; sp.mu_shape[2 * k + 1] = my;
      v_m[0][lane] = mx; v_m[1][lane] = my;
      v_raw[0][lane] = a2 - count * mx * mx;
      v_raw[1][lane] = a3 - count * mx * my;
      v_raw[2][lane] = a4 - count * my * my;
    }
  }
  __syncthreads();
  if (live && w < 3) v_s[w][lane] = (pc * v_ps[w][lane] + v_raw[w][lane]) / (total_count + 3.0);
  __syncthreads();
  if (live) {
    double sx = v_s[0][lane], sy = v_s[1][lane], sz = v_s[2][lane];
    double det = sx * sz - sy * sy;
    if (det <= 0) {
      sx = sx + 0.00001;
      sz = sz + 0.00001;
      det = sx * sz - sy * sy;
      if (det <= 0) det = 0.00001;
    }
    if (w == 0) v_i[0][lane] = sz / det;
    else if (w == 1) v_i[1][lane] = -sy / det;
    else if (w == 2) v_i[2][lane] = sx / det;
    else v_i[3][lane] = log(det);
  }
  __syncthreads();
  if (live && w == 0) {
    const double ix = v_i[0][lane], iy = v_i[1][lane], iz = v_i[2][lane], ld = v_i[3][lane];
    const double mx = v_m[0][lane], my = v_m[1][lane];
    sp.sigma_shape[3 * k] = ix; sp.sigma_shape[3 * k + 1] = iy; sp.sigma_shape[3 * k + 2] = iz;
    sp.logdet[k] = ld;
    SweepRec r;
    r.mu_r = v_app[0][lane]; r.mu_g = v_app[1][lane]; r.mu_b = v_app[2][lane];
    r.logdet = (float)ld;
    const double fx = floor(mx), fy = floor(my);
    r.mxi = (int)fx; r.myi = (int)fy;
    r.frac = (mx != fx ? 1 : 0) | (my != fy ? 2 : 0);
    r.isx = (float)ix; r.isy = (float)iy; r.isz = (float)iz; r.pad = 0.f;
    r.count = count_int;
    // the sweeps of the next update score again only the pixels next to a changed record
    const uint4* o = (const uint4*)&sp.rec[k];
    const uint4* nw = (const uint4*)&r;
    bool same = true;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const uint4 a = o[q], b = nw[q];
      same &= a.x == b.x && a.y == b.y && a.z == b.z && a.w == b.w;
    }
    if (!same) S.recchg[k] = 1;
    sp.rec[k] = r;
  }
}

// The posterior's work list (ids 0 .. max_spix, below cap): every id, or with
// `incremental` only the ids whose count or sums differ from those its posterior last
// saw.  Between two posteriors of the outer loop only the sweeps run, which change no
// other input of the posterior (priors, flags and the sample covariance change in the
// split, merge and relabel steps and at the frame's set-up, whose posteriors are full),
// so an id with equal sums would get the values it already holds (the same
// expressions of the same inputs).  Listed ids record their sums; the list's order
// varies, each id's result does not.
__global__ void kb_post_list(const Slot* __restrict__ slots, int incremental) {
  pdl_enter();
  SLOT_Y;
  const int last = min(S.sp.cap - 1, S.sc->max_spix);
  if ((int)(blockIdx.x * blockDim.x) > last) return;     // block-uniform
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  bool want = false;
  if (k <= last) {
    S.recchg[k] = 0;                       // set by kb_posterior when the record changes
    const long long* a = S.sp.acc + 8 * (size_t)k;
    long long* snap = S.snap + 9 * (size_t)k;
    long long cur[9];
#pragma unroll
    for (int f = 0; f < 8; f++) cur[f] = a[f];
    cur[8] = S.sp.count[k];
    want = !incremental;
    if (incremental) {
#pragma unroll
      for (int f = 0; f < 9; f++) want |= cur[f] != snap[f];
    }
    if (want) {
#pragma unroll
      for (int f = 0; f < 9; f++) snap[f] = cur[f];
    }
  }
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (!m) return;
  const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(&S.sc->npost, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  const int pos = base + __popc(m & ((1u << lane) - 1));
  if (want && pos < S.sp.cap) S.post_ids[pos] = k;     // at most cap ids are listed
}

// Grid: x blocks per slot, each taking groups of 32 listed ids x, x + gridDim.x, ...
// A group's barriers are block-uniform, and the first barrier of the next group follows
// every read of the previous one's shared values.  The last block of a slot to finish
// clears the list for the next posterior (every block read the list length first).
__global__ void __launch_bounds__(128) kb_posterior(const Slot* __restrict__ slots,
                                                    int incremental) {
  pdl_enter();
  SLOT_Y;
  Scalars* sc = S.sc;
  const int n = min(*(volatile int*)&sc->npost, S.sp.cap);
  for (int g = blockIdx.x; g * 32 < n; g += gridDim.x) {
    const int i = g * 32 + (threadIdx.x & 31);
    posterior_ids(S, i < n ? S.post_ids[i] : -1, incremental != 0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&sc->post_done, 1) == (int)gridDim.x - 1) {
      sc->npost = 0;
      sc->post_done = 0;
      __threadfence();
    }
  }
}

// clear_fields + the helper memset (update_params.cu:54-88, :26): zero the counts
// and the sums of every slot.
__global__ void kb_clear_stats(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= S.sp.cap) return;
  S.sp.count[k] = 0;
  long long* a = S.sp.acc + 8 * (size_t)k;
#pragma unroll
  for (int c = 0; c < 8; c++) a[c] = 0;
}

// store_sample_sigma_shape_k (update_params.cu:397-438).
__global__ void kb_store_sample(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const int n = min(sp.cap, S.sc->max_spix + 1);     // ids above are never valid
  FOR_SP(k, n) {
  if (!sp.valid[k]) continue;
  const long long* a = sp.acc + 8 * (size_t)k;
  double count = sp.count[k] * 1.0;
  double mx = a[3] / count, my = a[4] / count;
  sp.mu_shape[2 * k] = mx; sp.mu_shape[2 * k + 1] = my;
  double sx, sy, sz;
  if (count > 0) {
    sx = a[5] / count - mx * mx;
    sy = a[6] / count - mx * my;
    sz = a[7] / count - my * my;
  } else {
    sx = sp.prior_sigma_shape[3 * k]; sy = sp.prior_sigma_shape[3 * k + 1];
    sz = sp.prior_sigma_shape[3 * k + 2];
  }
  sp.sample_sigma_shape[3 * k] = sx;
  sp.sample_sigma_shape[3 * k + 1] = sy;
  sp.sample_sigma_shape[3 * k + 2] = sz;
  }
}

// ---------------------------------------------------------------------------
// Border masks (seg_utils.cu:164-195 and 218-257).
__global__ void k_find_border(const int* __restrict__ seg, uint8_t* __restrict__ border, int H,
                              int W) {
  pdl_enter();
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= H * W) return;
  int x = idx % W, y = idx / W;
  if (y < 1 || x < 1 || y >= H - 1 || x >= W - 1) { border[idx] = 1; return; }
  int C = seg[idx];
  border[idx] = (C != seg[idx - W] || C != seg[idx + W] || C != seg[idx + 1] ||
                 C != seg[idx - 1]) ? 1 : 0;
}

__global__ void kb_find_border(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const int W = S.W, H = S.H;
  const int* seg = S.seg;
  FOR_PIX(idx, S.npix) {
    const int x = idx % W, y = idx / W;
    if (y < 1 || x < 1 || y >= H - 1 || x >= W - 1) { S.border[idx] = 1; continue; }
    const int C = seg[idx];
    S.border[idx] = (C != seg[idx - W] || C != seg[idx + W] || C != seg[idx + 1] ||
                     C != seg[idx - 1]) ? 1 : 0;
  }
}

__global__ void k_find_border_end(const int* __restrict__ seg, uint8_t* __restrict__ border,
                                  int H, int W, int nframes) {
  pdl_enter();
  long long gi = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  long long npix = (long long)H * W;
  if (gi >= npix * nframes) return;
  int idx = (int)(gi % npix);
  const int* s = seg + (gi - idx);
  int x = idx % W, y = idx / W;
  int C = s[idx];
  int N = -1, S = -1, E = -1, Wl = -1;
  if (y > 0) N = s[idx - W];
  if (x > 0) Wl = s[idx - 1];
  if (y < H - 1) S = s[idx + W];
  if (x < W - 1) E = s[idx + 1];
  uint8_t b = 0;
  if ((N >= 0 && C != N) || (S >= 0 && C != S) || (E >= 0 && C != E) || (Wl >= 0 && C != Wl)) {
    if (N >= 0 && C > N) b = 1;
    if (S >= 0 && C > S) b = 1;
    if (E >= 0 && C > E) b = 1;
    if (Wl >= 0 && C > Wl) b = 1;
  }
  border[gi] = b;
}

// GetImageOverlaid (pyapi.cu:221-246).
__global__ void k_overlay(float* __restrict__ out, const float* __restrict__ img,
                          const float* __restrict__ color, const uint8_t* __restrict__ border,
                          long long n) {
  pdl_enter();
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  if (border[t]) {
    out[3 * t] = color[0]; out[3 * t + 1] = color[1]; out[3 * t + 2] = color[2];
  } else {
    for (int c = 0; c < 3; c++)
      out[3 * t + c] = (float)fmax(fmin((double)img[3 * t + c], 1.), 0.0);
  }
}

// ---------------------------------------------------------------------------
// Boundary sweep (update_seg_subset, update_seg.cu:30-190; calc_joint :194-259;
// simple-point table seg_utils.h:15-79).
// Simple-point table (data, identical to the reference's bass_lut): bit i of the
// index is set when 3x3 neighbour i (NW,N,NE,W,E,SW,S,SE) carries the candidate
// label or lies outside the image.
constexpr unsigned char kSimpleLut[256] = {
    0, 0, 1, 1, 0, 0, 1, 1, 1, 1, 0, 1, 0, 0, 0, 1, 1, 0, 0, 0, 1, 0, 1, 1, 0, 0,
    0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0,
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0,
    1, 1, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 1, 1, 0, 0, 0, 0,
    0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    1, 0, 0, 0, 1, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 1, 1,
    0, 1, 0, 0, 0, 1, 1, 0, 0, 0, 1, 0, 1, 1, 1, 1, 0, 0, 1, 1, 0, 0};

// The table as eight 32-bit words (bit b of word w = entry 32 w + b), computed from it at
// compile time.
struct SimpleBits {
  unsigned w[8];
};
__host__ __device__ constexpr SimpleBits simple_bits() {
  SimpleBits r{};
  for (int i = 0; i < 256; i++)
    if (kSimpleLut[i]) r.w[i >> 5] |= 1u << (i & 31);
  return r;
}
__constant__ SimpleBits c_simple_bits = simple_bits();

__device__ __forceinline__ void joint(float c0, float c1, float c2, int x, int y,
                                      const SweepRec& r, int k, float s2, float neigh_neq,
                                      float beta, float* best, int* best_label) {
  float res = -1000;
  const float x0 = c0 - r.mu_r;
  const float x1 = c1 - r.mu_g;
  const float x2 = c2 - r.mu_b;
  int d0 = x - r.mxi, d1 = y - r.myi;   // == (int)(x - mu_x), see SweepRec
  if ((r.frac & 1) && d0 >= 1) d0 -= 1;
  if ((r.frac & 2) && d1 >= 1) d1 -= 1;
  res = res - (x0 * x0 + x1 * x1 + x2 * x2) / s2;
  res = res - (float)(d0 * d0) * r.isx - (float)(d1 * d1) * r.isz - (float)(2 * d0 * d1) * r.isy;
  res = res - r.logdet;
  res = res - beta * neigh_neq;
  res = res - (float)(100 * (r.count <= 10));
  if (res > *best) { *best = res; *best_label = k; }
}

// ---------------------------------------------------------------------------
// Fused sweep: border pass + the four parity phases of one sweep in one launch.
// A block owns a TX x TY tile and stages labels of the tile plus a 4-pixel halo
// (phase k is evaluated on the tile grown by 3-k pixels, so every label a tile
// pixel depends on is produced inside the block exactly as the four separate
// launches produce it), the image and the border mask of the tile plus 3 pixels.
// Labels are read from seg_in (labels at the sweep start) and the tile is
// written to seg_out, so neighbouring blocks never see each other's updates.
//
// The grid is the list of tiles of every frame of the batch (frame i owns tiles
// [tile_base, tile_base + its tile count)); a block finds its frame by binary
// search, so frames of uneven size cost what their tiles cost.
constexpr int kReach = 4;             // a sweep's labels depend on labels this far away

// NS sweeps per launch (1 or 2): the label halo is 4 NS pixels; sweep s of the launch
// lists and scores the tile grown by G = 4 (NS - s) - 1 pixels (phase k on the tile
// grown by G - k), so after sweep s the labels of the tile grown by 4 (NS - s - 1)
// are exactly those of NS separate launches.
// Incremental statistics.  Between two update_params of the BASS loop the labels
// change only in the sweeps, so the statistics of the new labels are those of the old
// ones plus, for every pixel a sweep relabels from C to bl, its contribution moved
// from C to bl.  A sweep block collects the moves of its tile's own pixels in a small
// table in shared memory (label -> count and sums, 32-bit fields: colours split into
// 16-bit parts, positions relative to the tile) and adds each touched label's net
// change to its 64-bit global sums once per launch.  Integer sums, so the result is
// identical to clearing and summing every pixel again.
constexpr int kDeltaTab = 64;         // labels a tile's moves can touch (a power of two)

struct DeltaTab {
  int key[kDeltaTab];                 // label, -1 free
  int v[kDeltaTab][12];               // count, colour lo/hi x 3, sx, sy, sxx, sxy, syy
};

__device__ __forceinline__ int delta_slot(DeltaTab& tb, int k) {
  const unsigned h = ((unsigned)k * 2654435761u) >> 26;
#pragma unroll 1
  for (int p = 0; p < kDeltaTab; p++) {
    const int s = (int)((h + p) & (kDeltaTab - 1));
    const int cur = ((volatile int*)tb.key)[s];
    if (cur == k) return s;
    if (cur == -1) {
      const int old = atomicCAS(&tb.key[s], -1, k);
      if (old == -1 || old == k) return s;
    }
  }
  return -1;
}

// pixel (gx, gy), tile origin (tx0, ty0), moved from label C to label b.
__device__ __forceinline__ void delta_move(DeltaTab& tb, const SpDev& sp, int C, int b, int gx,
                                           int gy, int tx0, int ty0, float c0, float c1,
                                           float c2) {
  const bool unit = c0 >= 0.f && c0 <= 1.f && c1 >= 0.f && c1 <= 1.f && c2 >= 0.f && c2 <= 1.f;
  const int sc = unit ? delta_slot(tb, C) : -1;
  const int sb = unit ? delta_slot(tb, b) : -1;
  if (sc >= 0 && sb >= 0) {
    // colours in [0, 1]: the fixed-point value is one exact conversion, at most 2^28
    const unsigned q0 = __float2uint_rn(c0 * 0x1p28f), q1 = __float2uint_rn(c1 * 0x1p28f),
                   q2 = __float2uint_rn(c2 * 0x1p28f);
    const int x = gx - tx0, y = gy - ty0;
    const int d[12] = {1, (int)(q0 & 0xFFFF), (int)(q0 >> 16), (int)(q1 & 0xFFFF), (int)(q1 >> 16),
                       (int)(q2 & 0xFFFF), (int)(q2 >> 16), x, y, x * x, x * y, y * y};
#pragma unroll
    for (int f = 0; f < 12; f++) {
      atomicAdd(&tb.v[sb][f], d[f]);
      atomicSub(&tb.v[sc][f], d[f]);
    }
    return;
  }
  // other colours, or a full table: the move goes to the global sums at once
  const long long q[3] = {fx_q(c0, kFxAppShift), fx_q(c1, kFxAppShift), fx_q(c2, kFxAppShift)};
  const long long X = gx, Y = gy;
  const long long d[8] = {q[0], q[1], q[2], X, Y, X * X, X * Y, Y * Y};
  unsigned long long* ab = (unsigned long long*)(sp.acc + 8 * (size_t)b);
  unsigned long long* ac = (unsigned long long*)(sp.acc + 8 * (size_t)C);
  atomicAdd(&sp.count[b], 1);
  atomicSub(&sp.count[C], 1);
#pragma unroll
  for (int f = 0; f < 8; f++) {
    atomicAdd(ab + f, (unsigned long long)d[f]);
    atomicAdd(ac + f, (unsigned long long)(-d[f]));
  }
}

// The table's net changes to the global sums (block-wide; after the last phase).
__device__ __forceinline__ void delta_flush(DeltaTab& tb, const SpDev& sp, int tx0, int ty0) {
  for (int i = threadIdx.x; i < kDeltaTab; i += blockDim.x) {
    const int k = tb.key[i];
    if (k < 0) continue;
    const int* v = tb.v[i];
    const long long n = v[0], X = tx0, Y = ty0;
    const long long sx = v[7], sy = v[8];
    const long long d[8] = {(long long)v[2] * 65536 + v[1], (long long)v[4] * 65536 + v[3],
                            (long long)v[6] * 65536 + v[5], n * X + sx, n * Y + sy,
                            n * X * X + 2 * X * sx + v[9], n * X * Y + X * sy + Y * sx + v[10],
                            n * Y * Y + 2 * Y * sy + v[11]};
    unsigned long long* acc = (unsigned long long*)(sp.acc + 8 * (size_t)k);
    atomicAdd(&sp.count[k], v[0]);
#pragma unroll
    for (int f = 0; f < 8; f++) atomicAdd(acc + f, (unsigned long long)d[f]);
  }
}

template <int TX, int TY, int NS>
struct SweepTile {
  static constexpr int kSH = 4 * NS;                                 // label halo
  static constexpr int kG0 = kSH - 1;                                // first sweep's growth
  static constexpr int kLX = TX + 2 * kSH, kLY = TY + 2 * kSH;      // staged labels
  static constexpr int kMaxList = (TX / 2 + kG0) * (TY / 2 + kG0);
  static_assert(TX + 2 * kG0 < 256 && TY + 2 * kG0 < 256, "list entries pack (ly << 8) | lx");
  static_assert(kLX <= 128, "a label-region row is at most two 64-bit words");
  int L[kLX * kLY];
  unsigned short list[4][kMaxList];   // border pixels of each parity phase, (ly << 8) | lx
  int cnt[4];
  // active-set sweeps: change flags of the label region as row bitmasks (bit x of
  // row y = label-region pixel (x, y)), dilated by 4 pixels
  unsigned long long act[2][kLY];
  // label edges of the label region as row bitmasks: bit x of edE[.][y] is set when
  // pixel (x, y) and its right neighbour differ, of edS[.][y] when (x, y) and the pixel
  // below differ
  unsigned long long edE[2][kLY];
  unsigned long long edS[2][kLY];
  // pixels of the tile whose label the launch's last sweep changed, as row bitmasks
  // over label-region columns (the change flags the launch writes)
  unsigned long long chg[TY][2];
  DeltaTab delta;                     // statistics moves of the tile's pixels (deltas on)
};

// Bit masks over a label-region row (two 64-bit words, bit x of word x >> 6).
__host__ __device__ constexpr unsigned long long bits_below(int n) {
  return n <= 0 ? 0ull : n >= 64 ? ~0ull : ((1ull << n) - 1ull);
}
// bits [a, b) of word w
__host__ __device__ constexpr unsigned long long range_word(int a, int b, int w) {
  return bits_below(b - 64 * w) & ~bits_below(a - 64 * w);
}
constexpr unsigned long long kEvenBits = 0x5555555555555555ull;
constexpr unsigned long long kOddBits = 0xAAAAAAAAAAAAAAAAull;

// Active-set sweeps.  The parameters are fixed across the sweeps of one update_seg
// call and a pixel's decision depends only on its 3x3 labels (after the earlier
// phases of the sweep), its colour and the parameters, so a pixel of phase k can
// only change if a label within Chebyshev distance k + 1 <= 4 changed during the
// previous sweep or earlier in this one.  Sweeps after the first of a call (mode 1)
// therefore list only the border pixels within 4 pixels of a change flagged by the
// previous sweep (chg_in), and a tile whose whole label region saw no change keeps
// its labels.  Every sweep writes its own change flags (chg_out).
// One sweep inside a launch: list the border pixels of each parity class on the tile
// grown by G (phase k on the tile grown by G - k), then score them phase by phase in
// shared memory.  OFF = label-region offset of the grown-by-G region; use_act: only
// pixels flagged in sm.act (active-set sweeps).
// The 32-bit chunk ballots of a label-region row as its two 64-bit words.
template <int kCK>
__device__ __forceinline__ void pack_row(const unsigned (&b)[kCK], unsigned long long* w0,
                                         unsigned long long* w1) {
  unsigned long long lo = b[0], hi = 0;
  if (kCK > 1) lo |= (unsigned long long)b[1 % kCK] << 32;
  if (kCK > 2) hi = b[2 % kCK];
  if (kCK > 3) hi |= (unsigned long long)b[3 % kCK] << 32;
  *w0 = lo; *w1 = hi;
}

// STAGED: the label edges of the staged rows are already in sm.edE / sm.edS (computed
// from the staging registers, rows in contiguous spans of kLY / 8 per warp) except the
// lower edges of each span's last row, which need the next warp's first row.
template <int TX, int TY, int NS, int G, bool STAGED>
__device__ __forceinline__ void sweep_pass(const Slot& S, SweepTile<TX, TY, NS>& sm,
                                           const unsigned* lut_bits, int tx0, int ty0,
                                           float s2, float potts, bool use_act, bool last,
                                           bool deltas) {
  constexpr int kLX = SweepTile<TX, TY, NS>::kLX;
  constexpr int kLY = SweepTile<TX, TY, NS>::kLY;
  constexpr int kSH = SweepTile<TX, TY, NS>::kSH;
  constexpr int OFF = kSH - G;
  constexpr int kIY = TY + 2 * G;
  constexpr int kCK = (kLX + 31) / 32;
  static_assert(OFF >= 1, "every listed pixel has its 4 neighbours in the label region");
  int* L = sm.L;
  auto& list = sm.list;
  int* cnt = sm.cnt;
  const int H = S.H, W = S.W;
  const float* __restrict__ img = S.img;
  const SweepRec* __restrict__ rec = S.sp.rec;
  const SpDev& spd = S.sp;
  const int cap = S.sp.cap;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int ix0 = tx0 - G, iy0 = ty0 - G;
  const int rx0 = tx0 - kSH, ry0 = ty0 - kSH;
  // Border mask at the sweep start (find_border_pixels, seg_utils.cu:164-195) as row
  // bitmasks: a pixel is a border pixel when one of its 4 neighbours carries another
  // label (labels outside the image are staged as -1, so in-image pixels of the image's
  // edge rows and columns count as border pixels as in the reference).  First the
  // edges of the label region, one warp per row in 32-pixel chunks (rows with no
  // change in reach are skipped in active-set sweeps).
  if (STAGED) {
    constexpr int kSpan = kLY / 8;
    const int ay = warp * kSpan + kSpan - 1;   // this warp's span's last row
    if (ay + 1 < kLY) {
      unsigned d[kCK];
#pragma unroll
      for (int c = 0; c < kCK; c++) {
        const int x = lane + 32 * c;
        const bool in = x < kLX;
        const int v = in ? L[ay * kLX + x] : -1;
        const int dn = in ? L[(ay + 1) * kLX + x] : v;
        d[c] = __ballot_sync(0xffffffffu, v != dn);
      }
      if (lane == 0) pack_row<kCK>(d, &sm.edS[0][ay], &sm.edS[1][ay]);
    }
  } else {
    for (int ay = OFF - 1 + warp; ay < OFF + kIY; ay += nwarps) {
      if (use_act) {
        const int an = min(ay + 1, kLY - 1);
        if (!(sm.act[0][ay] | sm.act[1][ay] | sm.act[0][an] | sm.act[1][an])) continue;
      }
      unsigned e[kCK], d[kCK];
#pragma unroll
      for (int c = 0; c < kCK; c++) {
        const int x = lane + 32 * c;
        const bool in = x < kLX;
        const int v = in ? L[ay * kLX + x] : -1;
        const int r = (x + 1 < kLX) ? L[ay * kLX + x + 1] : v;
        const int dn = (in && ay + 1 < kLY) ? L[(ay + 1) * kLX + x] : v;
        e[c] = __ballot_sync(0xffffffffu, v != r);
        d[c] = __ballot_sync(0xffffffffu, v != dn);
      }
      if (lane == 0) {
        pack_row<kCK>(e, &sm.edE[0][ay], &sm.edE[1][ay]);
        pack_row<kCK>(d, &sm.edS[0][ay], &sm.edS[1][ay]);
      }
    }
  }
  __syncthreads();
  // Then the border pixels of each parity class inside the tile grown by G minus the
  // class (the class's phase), one warp per row: the row's border mask, restricted to
  // the image, the active set and the two classes of the row's y parity, is counted
  // per class (one shared atomic per class and row) and its set bits appended in
  // ascending x order.
  {
    const unsigned lt = (1u << lane) - 1u;
    const unsigned long long img0 = range_word(-rx0, W - rx0, 0);
    const unsigned long long img1 = range_word(-rx0, W - rx0, 1);
    for (int ly = warp; ly < kIY; ly += nwarps) {
      const int gy = iy0 + ly;
      if (gy < 0 || gy >= H) continue;
      const int ay = ly + OFF;                   // label-region row
      unsigned long long m0 = img0, m1 = img1;
      if (use_act) {
        m0 &= sm.act[0][ay];
        m1 &= sm.act[1][ay];
        if (!(m0 | m1)) continue;
      }
      const int cy = gy & 1;
      // the two classes of this row: (xo << 1) | cy, listed on the tile grown by
      // G - class; x parity of a label-region column equals that of the image column.
      // The column masks of the four classes are constants of the template.
      constexpr unsigned long long A00 = range_word(kSH - G, kSH + TX + G, 0) & kEvenBits;
      constexpr unsigned long long A01 = range_word(kSH - G, kSH + TX + G, 1) & kEvenBits;
      constexpr unsigned long long B00 = range_word(kSH - G + 2, kSH + TX + G - 2, 0) & kOddBits;
      constexpr unsigned long long B01 = range_word(kSH - G + 2, kSH + TX + G - 2, 1) & kOddBits;
      constexpr unsigned long long A10 = range_word(kSH - G + 1, kSH + TX + G - 1, 0) & kEvenBits;
      constexpr unsigned long long A11 = range_word(kSH - G + 1, kSH + TX + G - 1, 1) & kEvenBits;
      constexpr unsigned long long B10 = range_word(kSH - G + 3, kSH + TX + G - 3, 0) & kOddBits;
      constexpr unsigned long long B11 = range_word(kSH - G + 3, kSH + TX + G - 3, 1) & kOddBits;
      const int ga = G - cy, gb = G - (2 | cy);
      const int ry = ay - kSH;                   // row relative to the tile
      const bool ya = ry >= -ga && ry < TY + ga, yb = ry >= -gb && ry < TY + gb;
      const unsigned long long k0 = (ya ? (cy ? A10 : A00) : 0ull) | (yb ? (cy ? B10 : B00) : 0ull);
      const unsigned long long k1 = (ya ? (cy ? A11 : A01) : 0ull) | (yb ? (cy ? B11 : B01) : 0ull);
      const unsigned long long e0 = sm.edE[0][ay], e1 = sm.edE[1][ay];
      const unsigned long long b0 = e0 | (e0 << 1) | sm.edS[0][ay] | sm.edS[0][ay - 1];
      const unsigned long long b1 =
          e1 | (e1 << 1) | (e0 >> 63) | sm.edS[1][ay] | sm.edS[1][ay - 1];
      m0 &= b0 & k0;
      m1 &= b1 & k1;
      if (!(m0 | m1)) continue;
      const int na = __popcll(m0 & kEvenBits) + __popcll(m1 & kEvenBits);
      const int nb = __popcll(m0 & kOddBits) + __popcll(m1 & kOddBits);
      int base = 0;
      if (lane < 2) {
        const int n = lane ? nb : na;
        if (n) base = atomicAdd(&cnt[(lane << 1) | cy], n);
      }
      int base_a = __shfl_sync(0xffffffffu, base, 0);
      int base_b = __shfl_sync(0xffffffffu, base, 1);
      const bool odd = lane & 1;
      const unsigned mine = odd ? 0xAAAAAAAAu : 0x55555555u;
      unsigned short* out = list[((int)odd << 1) | cy];
#pragma unroll
      for (int c = 0; c < kCK; c++) {
        const unsigned w = (unsigned)((c < 2 ? m0 : m1) >> (32 * (c & 1)));
        if (!w) continue;
        const int ax = 32 * c + lane;
        if ((w >> lane) & 1u) {
          const int pos = (odd ? base_b : base_a) + __popc(w & mine & lt);
          out[pos] = (unsigned short)((ly << 8) | (ax - OFF));
        }
        base_a += __popc(w & 0x55555555u);
        base_b += __popc(w & 0xAAAAAAAAu);
      }
    }
  }
  __syncthreads();
  for (int ph = 0; ph < 4; ph++) {
    const int n = cnt[ph];
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      const int bi = list[ph][j];
      const int lxi = bi & 255, lyi = bi >> 8;
      int gx = ix0 + lxi, gy = iy0 + lyi;
      int p = (lyi + OFF) * kLX + (lxi + OFF);
      // the pixel's colour is loaded first: its latency overlaps the simple-point tests
      const float* pix = img + 3 * ((size_t)gy * W + gx);
      const float c0 = __ldg(pix), c1 = __ldg(pix + 1), c2 = __ldg(pix + 2);
      int C = L[p];
      if (C < 0 || C >= cap) continue;
      const int N = L[p - kLX], S = L[p + kLX], Wl = L[p - 1], E = L[p + 1];
      const int NW = L[p - kLX - 1], NE = L[p - kLX + 1], SW = L[p + kLX - 1],
                SE = L[p + kLX + 1];
      // simple-point codes of the four candidates: bit i set when neighbour i
      // (NW,N,NE,W,E,SW,S,SE) carries the candidate or lies outside the image;
      // equal candidates share one code; differing neighbours = 8 - popcount
      const int nb[8] = {NW, N, NE, Wl, E, SW, S, SE};
      unsigned m1 = 0;
#pragma unroll
      for (int q = 0; q < 8; q++) m1 |= (unsigned)(nb[q] == -1) << q;
      auto code = [&](int v) {
        unsigned c = m1;
#pragma unroll
        for (int q = 0; q < 8; q++) c |= (unsigned)(nb[q] == v) << q;
        return c;
      };
      const unsigned cN = code(N);
      const unsigned cW = (Wl == N) ? cN : code(Wl);
      const unsigned cS = (S == N) ? cN : (S == Wl) ? cW : code(S);
      const unsigned cE = (E == N) ? cN : (E == Wl) ? cW : (E == S) ? cS : code(E);
      auto simple = [&](unsigned c) { return (lut_bits[c >> 5] >> (c & 31)) & 1u; };
      if (!simple(cN) || !simple(cW) || !simple(cS) || !simple(cE)) continue;
      const int dN = 8 - __popc(cN), dW = 8 - __popc(cW), dS = 8 - __popc(cS),
                dE = 8 - __popc(cE);
      if (N >= cap || S >= cap || Wl >= cap || E >= cap) continue;
      float best = -9999.f;
      int bl = C;
      if (N >= 0) joint(c0, c1, c2, gx, gy, rec[N], N, s2, (float)dN, potts, &best, &bl);
      if (S != N && S >= 0) joint(c0, c1, c2, gx, gy, rec[S], S, s2, (float)dS, potts, &best, &bl);
      if (Wl != S && Wl != N && Wl >= 0)
        joint(c0, c1, c2, gx, gy, rec[Wl], Wl, s2, (float)dW, potts, &best, &bl);
      if (E != Wl && E != S && E != N && E >= 0)
        joint(c0, c1, c2, gx, gy, rec[E], E, s2, (float)dE, potts, &best, &bl);
      if (rec[C].count <= 2 && bl == C) {
        if (N >= 0) bl = N;
        else if (E >= 0) bl = E;
        else if (S >= 0) bl = S;
        else if (Wl >= 0) bl = Wl;
      }
      if (bl != C) {
        L[p] = bl;
        // a tile pixel changed by the launch's last sweep: its change flag (each pixel
        // is scored once per sweep, so a changed pixel keeps its new label); with
        // deltas, the move of its statistics from C to bl
        const int ty = lyi + OFF - kSH, ax = lxi + OFF;
        if (ty >= 0 && ty < TY && ax >= kSH && ax < kSH + TX) {
          if (last) atomicOr(&sm.chg[ty][ax >> 6], 1ull << (ax & 63));
          if (deltas) delta_move(sm.delta, spd, C, bl, gx, gy, tx0, ty0, c0, c1, c2);
        }
      }
    }
    __syncthreads();
  }
  (void)rx0; (void)ry0;
}

// Active-set sweeps.  The parameters are fixed across the sweeps of one update_seg
// call and a pixel's decision depends only on its 3x3 labels (after the earlier
// phases of the sweep), its colour and the parameters, so a pixel of phase k can
// only change if a label within Chebyshev distance k + 1 <= 4 changed during the
// previous sweep or earlier in this one.  Sweeps after the first of a call (mode 1)
// therefore list only the border pixels within 4 pixels of a change flagged by the
// previous sweep (chg_in), and a tile whose whole label region saw no change keeps
// its labels.  Every launch writes the change flags of its last sweep (chg_out); in
// a two-sweep launch the second sweep lists every border pixel.
template <int TX, int TY, int NS>
__device__ __forceinline__ void sweep_tile(const Slot& S, int bx, int by, int parity, float s2,
                                           float potts, SweepTile<TX, TY, NS>& sm,
                                           const unsigned* lut_bits, int mode, int deltas) {
  constexpr int kTX = TX, kTY = TY;
  constexpr int kSH = SweepTile<TX, TY, NS>::kSH;
  constexpr int kLX = SweepTile<TX, TY, NS>::kLX, kLY = SweepTile<TX, TY, NS>::kLY;
  int* L = sm.L;
  int* cnt = sm.cnt;

  const int H = S.H, W = S.W;
  const int* __restrict__ seg_in = parity ? S.seg_alt : S.seg;
  int* __restrict__ seg_out = parity ? S.seg : S.seg_alt;
  if (threadIdx.x < 4) cnt[threadIdx.x] = 0;
  const int tx0 = bx * kTX, ty0 = by * kTY;
  const int rx0 = tx0 - kSH, ry0 = ty0 - kSH;        // label region origin
  // change flags: one bit per pixel, rows of P16 16-bit words (bit x & 15 of word
  // x >> 4); a tile's x origin is a multiple of 16, so every word has one writer
  const uint16_t* __restrict__ chg_in = (const uint16_t*)S.chg[parity ^ 1];
  uint16_t* __restrict__ chg_out = (uint16_t*)S.chg[parity];
  const int P16 = (W + 15) >> 4;
  // The label region is loaded first, into registers: warp w takes rows w, w + 8, ...
  // in 32-label chunks, every load issued before any is used, so the block waits for
  // one memory round trip (overlapping the change-flag loads of active-set sweeps).
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kRW = kLY / 8, kCK = (kLX + 31) / 32;   // warp w: rows kRW w .. kRW w + kRW - 1
  static_assert(kLY % 8 == 0, "label-region rows in whole warp spans");
  int lv[kRW][kCK];
  if (rx0 >= 0 && ry0 >= 0 && rx0 + kLX <= W && ry0 + kLY <= H) {
    // the label region lies inside the frame (most tiles): one row pointer per row,
    // no per-label bounds but the region's width
    const int* base = seg_in + (size_t)(ry0 + warp * kRW) * W + rx0 + lane;
#pragma unroll
    for (int a = 0; a < kRW; a++) {
#pragma unroll
      for (int c = 0; c < kCK; c++)
        lv[a][c] = (lane + 32 * c < kLX) ? base[(size_t)a * W + 32 * c] : -1;
    }
  } else {
#pragma unroll
    for (int a = 0; a < kRW; a++) {
      const int r = warp * kRW + a, gy = ry0 + r;
      const bool row_ok = r < kLY && gy >= 0 && gy < H;
#pragma unroll
      for (int c = 0; c < kCK; c++) {
        const int x = lane + 32 * c, gx = rx0 + x;
        lv[a][c] = (row_ok && x < kLX && gx >= 0 && gx < W) ? seg_in[gy * W + gx] : -1;
      }
    }
  }
  // tile pixels of the staging layout: (a, c) -> label-region (r, x)
  auto in_tile = [&](int r, int x) {
    return r >= kSH && r < kSH + kTY && x >= kSH && x < kSH + kTX && ry0 + r < H && rx0 + x < W;
  };
  if (mode) {
    unsigned long long* a0 = sm.act[0];
    unsigned long long* a1 = sm.act[1];
    if (mode == 2) {
      // first sweep after an incremental posterior: besides the previous sweep's changes,
      // every pixel whose label or 4-neighbour's label got a new record may decide
      // differently.  The label-region pixels whose label's record changed, as row
      // bitmasks (from the staging registers; sm.edE is free until the edges below).
      const int cap = S.sp.cap;
#pragma unroll
      for (int a = 0; a < kRW; a++) {
        const int rr = warp * kRW + a;
        unsigned q[kCK];
#pragma unroll
        for (int c = 0; c < kCK; c++) {
          const int v = lv[a][c];
          q[c] = __ballot_sync(0xffffffffu, v >= 0 && v < cap && S.recchg[v] != 0);
        }
        if (lane == 0) pack_row<kCK>(q, &sm.edE[0][rr], &sm.edE[1][rr]);
      }
      __syncthreads();
    }
    // each row of the label region: its change bits from the previous sweep's plane
    // (kNW 16-bit words starting at word rx0 >> 4, shifted by the region's offset in
    // the first word), then dilated by the reach horizontally
    constexpr int kNW = (kLX + 15) / 16 + 1;
    static_assert(kNW <= 8 && kLX <= 128, "a label-region row spans at most 8 words");
    const int w0 = rx0 >> 4;                     // rx0 >= -8: arithmetic shift floors
    const int off = rx0 - (w0 << 4);             // 16 - halo, in 1..15
    unsigned long long h0 = 0, h1 = 0;
    bool nz = false;
    const int r = threadIdx.x;
    if (r < kLY) {
      const int gy = ry0 + r;
      unsigned long long lo = 0, hi = 0;
      if (gy >= 0 && gy < H) {
        const uint16_t* row = chg_in + (size_t)gy * P16;
#pragma unroll
        for (int k = 0; k < kNW; k++) {
          const int wi = w0 + k;
          const unsigned long long v = (wi >= 0 && wi < P16) ? (unsigned long long)row[wi] : 0ull;
          if (k < 4) lo |= v << (16 * k);
          else hi |= v << (16 * (k - 4));
        }
      }
      unsigned long long f0 = (lo >> off) | (hi << (64 - off));
      unsigned long long f1 = hi >> off;
      if (mode == 2) {
        // changed records seed the active set one pixel further out (a pixel reads the
        // records of its 4-neighbours' labels)
        unsigned long long q0 = sm.edE[0][r], q1 = sm.edE[1][r];
        if (r > 0) { q0 |= sm.edE[0][r - 1]; q1 |= sm.edE[1][r - 1]; }
        if (r + 1 < kLY) { q0 |= sm.edE[0][r + 1]; q1 |= sm.edE[1][r + 1]; }
        f0 |= q0 | (q0 << 1) | (q0 >> 1) | (q1 << 63);
        f1 |= q1 | (q1 << 1) | (q1 >> 1) | (q0 >> 63);
      }
      if (kLX < 64) { f0 &= (1ull << (kLX & 63)) - 1ull; f1 = 0; }
      else if (kLX < 128) { f1 &= (1ull << ((kLX - 64) & 63)) - 1ull; }
      nz = (f0 | f1) != 0;
      h0 = f0; h1 = f1;
#pragma unroll
      for (int sft = 1; sft <= kReach; sft++) {
        h0 |= (f0 << sft) | (f0 >> sft) | (f1 << (64 - sft));
        h1 |= (f1 << sft) | (f1 >> sft) | (f0 >> (64 - sft));
      }
      a0[r] = h0;
      a1[r] = h1;
    }
    if (!__syncthreads_or(nz)) {
      // nothing within reach changed: the tile keeps its labels (for every sweep of
      // the launch: a later sweep can only move pixels within reach of an earlier
      // change, and there is none in the label region)
#pragma unroll
      for (int a = 0; a < kRW; a++) {
        const int rr = warp * kRW + a;
#pragma unroll
        for (int c = 0; c < kCK; c++) {
          const int x = lane + 32 * c;
          if (rr < kLY && x < kLX && in_tile(rr, x))
            seg_out[(size_t)(ry0 + rr) * W + (rx0 + x)] = lv[a][c];
        }
      }
      // zero change words of the tile's rows
      constexpr int kTW = kTX / 16;
      for (int i = threadIdx.x; i < kTY * kTW; i += blockDim.x) {
        const int gy = ty0 + i / kTW, wi = (tx0 >> 4) + i % kTW;
        if (gy < H && wi < P16) chg_out[(size_t)gy * P16 + wi] = 0;
      }
      return;
    }
    // vertical dilation
    unsigned long long v0 = 0, v1 = 0;
    if (r < kLY) {
      for (int k = max(0, r - kReach); k <= min(kLY - 1, r + kReach); k++) {
        v0 |= a0[k]; v1 |= a1[k];
      }
    }
    __syncthreads();
    if (r < kLY) { a0[r] = v0; a1[r] = v1; }
    // (the barrier after the label stores below orders these before the border pass)
  }
  // labels to shared memory (colours are not staged: the scored border pixels read
  // theirs from global memory), and the label edges of the warp's rows from the
  // registers: right neighbours by shuffles, lower neighbours from the next row of
  // the span (the span's last row waits for the shared copy, see sweep_pass)
#pragma unroll
  for (int a = 0; a < kRW; a++) {
    const int r = warp * kRW + a;
    unsigned e[kCK], d[kCK];
#pragma unroll
    for (int c = 0; c < kCK; c++) {
      const int x = lane + 32 * c;
      const int v = lv[a][c];
      if (x < kLX) L[r * kLX + x] = v;
      int right = __shfl_down_sync(0xffffffffu, v, 1);
      const int nxt = __shfl_sync(0xffffffffu, lv[a][c + 1 < kCK ? c + 1 : c], 0);
      if (lane == 31) right = c + 1 < kCK ? nxt : v;
      e[c] = __ballot_sync(0xffffffffu, x + 1 < kLX && v != right);
      d[c] = __ballot_sync(0xffffffffu, x < kLX && a + 1 < kRW && v != lv[a + 1 < kRW ? a + 1 : a][c]);
    }
    if (lane == 0) {
      pack_row<kCK>(e, &sm.edE[0][r], &sm.edE[1][r]);
      if (a + 1 < kRW) pack_row<kCK>(d, &sm.edS[0][r], &sm.edS[1][r]);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < 2 * kTY; i += blockDim.x) (&sm.chg[0][0])[i] = 0ull;
  if (deltas) {
    for (int i = threadIdx.x; i < kDeltaTab; i += blockDim.x) {
      sm.delta.key[i] = -1;
#pragma unroll
      for (int f = 0; f < 12; f++) sm.delta.v[i][f] = 0;
    }
  }
  // (the listing barrier of the first pass orders these clears before any use)
  if (NS == 1) {
    sweep_pass<TX, TY, NS, 4 * NS - 1, true>(S, sm, lut_bits, tx0, ty0, s2, potts, mode != 0,
                                             true, deltas != 0);
  } else {
    sweep_pass<TX, TY, NS, 4 * NS - 1, true>(S, sm, lut_bits, tx0, ty0, s2, potts, mode != 0,
                                             false, deltas != 0);
    if (threadIdx.x < 4) cnt[threadIdx.x] = 0;   // fresh lists (the phases' last barrier
                                                 // ordered every read of the counts)
    sweep_pass<TX, TY, NS, 3, false>(S, sm, lut_bits, tx0, ty0, s2, potts, false, true,
                                     deltas != 0);
  }
  if (deltas) delta_flush(sm.delta, S.sp, tx0, ty0);   // after the last phase's barrier
  // write back the tile (a warp covers 32 consecutive pixels of a row; 16-wide tiles:
  // two rows), then the change words of the last sweep: word i of a tile row holds
  // tile columns 16 i .. 16 i + 15 = label-region columns kSH + 16 i ..
  for (int i = threadIdx.x; i < kTX * kTY; i += blockDim.x) {
    const int x = i % kTX, y = i / kTX;
    const int gx = tx0 + x, gy = ty0 + y;
    if (gx < W && gy < H) seg_out[(size_t)gy * W + gx] = L[(y + kSH) * kLX + (x + kSH)];
  }
  constexpr int kTW = kTX / 16;
  for (int i = threadIdx.x; i < kTY * kTW; i += blockDim.x) {
    const int y = i / kTW, q = i % kTW;
    const int gy = ty0 + y, wi = (tx0 >> 4) + q;
    if (gy < H && wi < P16) {
      const int b0 = kSH + 16 * q;
      const unsigned long long lo = sm.chg[y][0], hi = sm.chg[y][1];
      const unsigned long long v = b0 < 64 ? ((lo >> b0) | (b0 > 48 ? hi << (64 - b0) : 0ull))
                                           : (hi >> (b0 - 64));
      chg_out[(size_t)gy * P16 + wi] = (uint16_t)v;
    }
  }
}

template <int TX, int TY, int NS>
__device__ __forceinline__ void sweep_flat(const Slot* __restrict__ slots, int B, int parity,
                                           float s2, float potts, int mode, int deltas) {
  __shared__ SweepTile<TX, TY, NS> sm;
  __shared__ unsigned lut_bits[8];
  if (threadIdx.x < 8) lut_bits[threadIdx.x] = c_simple_bits.w[threadIdx.x];
  const int v = TX == 32 ? 0 : TX == 64 ? 1 : 2;   // which tile_base of the slots
  const int t = blockIdx.x;
  int lo = 0, hi = B - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (slots[mid].tile_base[v] <= t) lo = mid; else hi = mid - 1;
  }
  const Slot& S = slots[lo];
  const int tl = t - S.tile_base[v];
  const int tiles_x = (S.W + TX - 1) / TX;
  sweep_tile<TX, TY, NS>(S, tl % tiles_x, tl / tiles_x, parity, s2, potts, sm, lut_bits, mode,
                         deltas);
}

// Persistent work-queue form of the single-sweep launch: a resident set of blocks
// (the SM count times the blocks an SM holds, at most the tile count) takes the
// batch's tiles in index order from an atomic counter, queue[0], and sweeps each as
// the one-block-per-tile kernel does (the same labels: a launch reads only the labels
// at its start).  The last block to finish, counted in queue[1], sets both counters
// back to zero for the next launch (stream order and the dependent-launch wait make
// that store visible to it).  No block waits on another.
template <int TX, int TY>
__device__ __forceinline__ void sweep_queue(const Slot* __restrict__ slots, int B, int ntiles,
                                            unsigned* queue, int parity, float s2, float potts,
                                            int mode, int deltas) {
  __shared__ SweepTile<TX, TY, 1> sm;
  __shared__ unsigned lut_bits[8];
  __shared__ int next;
  if (threadIdx.x < 8) lut_bits[threadIdx.x] = c_simple_bits.w[threadIdx.x];
  const int v = TX == 32 ? 0 : TX == 64 ? 1 : 2;   // which tile_base of the slots
  for (;;) {
    if (threadIdx.x == 0) next = (int)atomicAdd(&queue[0], 1u);
    __syncthreads();
    const int t = next;
    if (t >= ntiles) break;
    int lo = 0, hi = B - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (slots[mid].tile_base[v] <= t) lo = mid; else hi = mid - 1;
    }
    const Slot& S = slots[lo];
    const int tl = t - S.tile_base[v];
    const int tiles_x = (S.W + TX - 1) / TX;
    sweep_tile<TX, TY, 1>(S, tl % tiles_x, tl / tiles_x, parity, s2, potts, sm, lut_bits, mode,
                          deltas);
    __syncthreads();          // the tile's shared memory and `next` are free again
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&queue[1], 1u) == gridDim.x - 1) {
      queue[0] = 0u;
      queue[1] = 0u;
      __threadfence();
    }
  }
}

#define STSPIX_SWEEPQ_KERNEL(name, TX, MINB)                                                \
  __global__ void __launch_bounds__(256, MINB) name(const Slot* __restrict__ slots, int B,    \
                                                    int ntiles, unsigned* queue, int parity,  \
                                                    float s2, float potts, int mode,          \
                                                    int deltas) {                             \
    pdl_enter();                                                                             \
    sweep_queue<TX, 32>(slots, B, ntiles, queue, parity, s2, potts, mode, deltas);           \
  }
STSPIX_SWEEPQ_KERNEL(kb_sweepq_t32, 32, 6)
STSPIX_SWEEPQ_KERNEL(kb_sweepq_t64, 64, 6)
STSPIX_SWEEPQ_KERNEL(kb_sweepq_t16, 16, 6)
#undef STSPIX_SWEEPQ_KERNEL

// One block per tile of the batch (grid = the batch's total tile count), one sweep
// (kb_sweep_t*) or two consecutive sweeps (kb_sweep2_t*) per launch.
// mode 0: every border pixel (first sweep of an update_seg call); 1: active set.
// deltas 1: move the statistics of every relabelled tile pixel (incremental
// statistics: the sums of the labels at the call's start stay current); 0: not.
#define STSPIX_SWEEP_KERNEL(name, TX, NS, MINB)                                          \
  __global__ void __launch_bounds__(256, MINB) name(const Slot* __restrict__ slots, int B, \
                                                    int parity, float s2, float potts,     \
                                                    int mode, int deltas) {                \
    pdl_enter();                                                                          \
    sweep_flat<TX, 32, NS>(slots, B, parity, s2, potts, mode, deltas);                    \
  }
STSPIX_SWEEP_KERNEL(kb_sweep_t32, 32, 1, 6)
STSPIX_SWEEP_KERNEL(kb_sweep_t64, 64, 1, 6)
STSPIX_SWEEP_KERNEL(kb_sweep_t16, 16, 1, 6)
STSPIX_SWEEP_KERNEL(kb_sweep2_t32, 32, 2, 4)
STSPIX_SWEEP_KERNEL(kb_sweep2_t16, 16, 2, 4)
STSPIX_SWEEP_KERNEL(kb_sweep2_t64, 64, 2, 4)
#undef STSPIX_SWEEP_KERNEL

// ---------------------------------------------------------------------------
// Parameter read-out (read_params, sparams_io.cu:190-286) and prior update
// (update_prior_kernel, sparams_io.cu:584-640) into the caller's SoA params.
__global__ void kb_read_params(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  const SpDev& sp = S.sp;
  const stspix_params& out = S.pout;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n = S.sc->nspix;
  if (i >= n || i >= out.capacity || i >= sp.cap) return;
  bool upd = sp.count[i] > 0;
  for (int c = 0; c < 3; c++) {
    float m = sp.mu_app[3 * i + c];
    out.mu_app[3 * i + c] = m;
    out.prior_mu_app[3 * i + c] = upd ? m : sp.prior_mu_app[3 * i + c];
    double s = sp.sigma_shape[3 * i + c];
    out.sigma_shape[3 * i + c] = s;
    out.prior_sigma_shape[3 * i + c] = upd ? s : sp.prior_sigma_shape[3 * i + c];
    out.sample_sigma_shape[3 * i + c] = sp.sample_sigma_shape[3 * i + c];
  }
  for (int c = 0; c < 2; c++) {
    double m = sp.mu_shape[2 * i + c];
    out.mu_shape[2 * i + c] = m;
    out.prior_mu_shape[2 * i + c] = upd ? m : sp.prior_mu_shape[2 * i + c];
  }
  out.logdet_sigma_shape[i] = (float)sp.logdet[i];
  out.counts[i] = sp.count[i];
  out.invalid_counts[i] = sp.icount[i];
  out.sm_counts[i] = sp.sm_count[i];
  out.prior_counts[i] = sp.prior_count[i];
  out.ids[i] = i;
}

// Per-slot scalar steps, one thread per slot.
__global__ void kb_scalars(const Slot* __restrict__ slots, int B, int op) {
  pdl_enter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= B) return;
  const Slot& S = slots[i];
  Scalars* sc = S.sc;
  switch (op) {
    case kOpBegin:  // frame start: counters, buffer sizes of the reference
      sc->status = STSPIX_OK;
      sc->nsplits = sc->nmerges = sc->nrevived = sc->nminted = sc->near_ties = 0;
      sc->fill_iters = 0;
      sc->ninvalid = 0;
      sc->tmp0 = sc->tmp1 = sc->tmp2 = 0;
      sc->npost = sc->post_done = 0;
      sc->nspix = 0;
      if (S.mode) { sc->max_spix = S.n_prev - 1; sc->nbuf_logical = 10 * S.n_prev; }
      else { sc->max_spix = 0; sc->nbuf_logical = 30 * S.nraw; }
      break;
    case kOpAfterHex:  // max_spix after compacting the hex ids
      if (!S.mode) sc->max_spix = sc->nspix - 1;
      break;
    case kOpCompactN:  // ids beyond cap were never created
      sc->tmp2 = min(sc->max_spix + 1, S.cap) - S.lo;
      break;
    case kOpCompactEnd:
      sc->nspix = S.lo + sc->tmp1;
      break;
  }
}

// flags := 0 (cap + 2 entries) before a presence scan.
__global__ void kb_clear_flags(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < S.cap + 2) S.flags[k] = 0;
}

// Keep a copy of the finished labels where the slot's video stream resides.
__global__ void kb_save_prev(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  if (!S.resident_labels) return;
  FOR_PIX(i, S.npix) S.resident_labels[i] = S.seg[i];
}

__global__ void kb_copy_labels(const Slot* __restrict__ slots) {
  pdl_enter();
  SLOT_Y;
  FOR_PIX(i, S.npix) S.seg[i] = S.seg_alt[i];
}

__global__ void k_dump_state(SpDev sp, stspix_state_dump d) {
  pdl_enter();
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= sp.cap || k >= d.capacity) return;
  if (d.count) d.count[k] = sp.count[k];
  if (d.valid) d.valid[k] = sp.valid[k];
  if (d.prior_count) d.prior_count[k] = sp.prior_count[k];
  for (int c = 0; c < 3; c++) {
    if (d.mu_app) d.mu_app[3 * k + c] = sp.mu_app[3 * k + c];
    if (d.sigma_shape) d.sigma_shape[3 * k + c] = sp.sigma_shape[3 * k + c];
  }
  for (int c = 0; c < 2; c++)
    if (d.mu_shape) d.mu_shape[2 * k + c] = sp.mu_shape[2 * k + c];
  if (d.logdet) d.logdet[k] = sp.logdet[k];
  if (d.sums)
    for (int c = 0; c < 8; c++) d.sums[8 * (size_t)k + c] = sp.acc[8 * (size_t)k + c];
}

}  // namespace stspix
