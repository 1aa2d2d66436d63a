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
__global__ void k_init_hex(int* __restrict__ seg, int H, int W, double Hh, double w, int nx,
                           int ny) {
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= H * W) return;
  int x = idx % W, y = idx / W;
  int r0 = (int)floor(y / (1.5 * Hh));
  int c0 = (int)floor(x / w);
  double D2 = 1.7976931348623157e308;
  int best = 0;
  for (int r = r0 - 2; r <= r0 + 2; r++) {
    if (r < 0 || r >= ny) continue;
    for (int c = c0 - 2; c <= c0 + 2; c++) {
      if (c < 0 || c >= nx) continue;
      double xx = double(c) * w;
      double yy = double(r) * 1.5 * Hh;
      if (r % 2 == 0) xx = xx + 0.5 * w;
      double dx = (x - xx);
      double dy = (y - yy);
      double d2 = dx * dx + dy * dy;
      if (d2 <= D2) { D2 = d2; best = r * nx + c; }
    }
  }
  seg[idx] = best;
}

__global__ void kb_init_hex(const Slot* __restrict__ slots) {
  SLOT_Y;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= S.npix) return;
  const int W = S.W, nx = S.hex_nx, ny = S.hex_ny;
  const double Hh = S.hex_h, w = S.hex_w;
  int x = idx % W, y = idx / W;
  int r0 = (int)floor(y / (1.5 * Hh));
  int c0 = (int)floor(x / w);
  double D2 = 1.7976931348623157e308;
  int best = 0;
  for (int r = r0 - 2; r <= r0 + 2; r++) {
    if (r < 0 || r >= ny) continue;
    for (int c = c0 - 2; c <= c0 + 2; c++) {
      if (c < 0 || c >= nx) continue;
      double xx = double(c) * w;
      double yy = double(r) * 1.5 * Hh;
      if (r % 2 == 0) xx = xx + 0.5 * w;
      double dx = (x - xx);
      double dy = (y - yy);
      double d2 = dx * dx + dy * dy;
      if (d2 <= D2) { D2 = d2; best = r * nx + c; }
    }
  }
  S.seg[idx] = best;
}

// ---------------------------------------------------------------------------
// Compaction (compact_spix.cu:41-122, 196-290): flags of live ids in [lo, hi],
// exclusive scan, remap.
// mode 0: hex ids [0, nraw); mode 1: ids [lo, max_spix] of the finished frame.
__global__ void kb_mark_present(const Slot* __restrict__ slots, int mode) {
  SLOT_Y;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.npix) return;
  int lo = mode == 0 ? 0 : S.lo;
  int hi = mode == 0 ? S.nraw - 1 : min(S.sc->max_spix, S.cap - 1);
  int v = S.seg[i];
  if (v >= lo && v <= hi) S.flags[v - lo] = 1;
}

// One block per slot: exclusive scan of n byte flags (n up to a few 10^5).
//   mode 0: hex-id presence (n = nraw)        -> total = live hex ids
//   mode 1: split acceptance (n = cap)        -> total = accepted splits
//   mode 2: relabel mint flags (n = cap)      -> total = minted ids
//   mode 3: final presence (n = max_spix+1-lo) -> total = live new ids
__global__ void kb_scan(const Slot* __restrict__ slots, int mode) {
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
  for (int i = b; i < e; i++) s += flags[i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int off = 1; off < T; off <<= 1) {
    int v = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int i = b; i < e; i++) { excl[i] = run; run += flags[i]; }
  if (threadIdx.x == T - 1) *total = part[T - 1];
}

__global__ void kb_remap(const Slot* __restrict__ slots, int mode) {
  SLOT_Y;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.npix) return;
  int lo = mode == 0 ? 0 : S.lo;
  int v = S.seg[i];
  if (v >= lo) S.seg[i] = lo + S.excl[v - lo];
}

// fill_new_params_from_old (compact_spix.cu:220-265): gather moved fields.
__global__ void kb_compact_gather(const Slot* __restrict__ slots) {
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
// Sufficient statistics (sum_by_label, update_params.cu:89-130), R1.
// Each thread owns a run of kRun pixels of one row, accumulates in registers while
// the label stays the same and flushes one set of 64-bit atomics per label run;
// position sums of a run are closed-form.
constexpr int kRun = 8;

__device__ __forceinline__ void flush_run(const SpDev& sp, int k, int y, int x0, int x1,
                                          long long sr, long long sg, long long sb) {
  long long n = x1 - x0 + 1;
  long long sx = (long long)(x0 + x1) * n / 2;
  long long a = x0 - 1, b = x1;
  long long sxx = b * (b + 1) * (2 * b + 1) / 6 - (a >= 0 ? a * (a + 1) * (2 * a + 1) / 6 : 0);
  unsigned long long* acc = (unsigned long long*)(sp.acc + 8 * (size_t)k);
  atomicAdd(&sp.count[k], (int)n);
  atomicAdd(acc + 0, (unsigned long long)sr);
  atomicAdd(acc + 1, (unsigned long long)sg);
  atomicAdd(acc + 2, (unsigned long long)sb);
  atomicAdd(acc + 3, (unsigned long long)sx);
  atomicAdd(acc + 4, (unsigned long long)(n * y));
  atomicAdd(acc + 5, (unsigned long long)sxx);
  atomicAdd(acc + 6, (unsigned long long)(sx * y));
  atomicAdd(acc + 7, (unsigned long long)(n * y * (long long)y));
}

__global__ void kb_accumulate(const Slot* __restrict__ slots) {
  SLOT_Y;
  const float* __restrict__ img = S.img;
  const int* __restrict__ seg = S.seg;
  const int H = S.H, W = S.W;
  const SpDev& sp = S.sp;
  const int cpr = (W + kRun - 1) / kRun;
  int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= H * cpr) return;
  int y = tid / cpr, xs = (tid % cpr) * kRun, xe = min(W, xs + kRun);
  const int* srow = seg + (size_t)y * W;
  const float* irow = img + (size_t)y * W * 3;
  int cur = -1, x0 = xs;
  long long sr = 0, sg = 0, sb = 0;
  for (int x = xs; x < xe; x++) {
    int k = srow[x];
    if (k != cur) {
      if (cur >= 0 && cur < sp.cap) flush_run(sp, cur, y, x0, x - 1, sr, sg, sb);
      cur = k; x0 = x; sr = sg = sb = 0;
    }
    if (k >= 0) {
      sr += fx_q(irow[3 * x], kFxAppShift);
      sg += fx_q(irow[3 * x + 1], kFxAppShift);
      sb += fx_q(irow[3 * x + 2], kFxAppShift);
    }
  }
  if (cur >= 0 && cur < sp.cap) flush_run(sp, cur, y, x0, xe - 1, sr, sg, sb);
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

__device__ __forceinline__ void posterior_one(const SpDev& sp, int sp_size, Scalars* sc, int k) {
  int count_int = sp.count[k];
  bool live = sp.valid[k] && count_int > 0;
  if (sp.valid[k] && count_int <= 0) sp.valid[k] = 0;
  if (!live) {
    for (int c = 0; c < 3; c++) { sp.mu_app[3 * k + c] = 0.f; sp.sigma_shape[3 * k + c] = 0.0; }
    sp.mu_shape[2 * k] = 0.0; sp.mu_shape[2 * k + 1] = 0.0;
    return;
  }
  float pc = sp.prior_count[k];
  double count = count_int * 1.0;
  double total_count = (double)count_int + pc * 50;
  double px, py, pz;
  if (sp.prop[k]) {
    smooth_prior(sp.sample_sigma_shape[3 * k], sp.sample_sigma_shape[3 * k + 1],
                 sp.sample_sigma_shape[3 * k + 2], (int)pc, pc, sp_size, &px, &py, &pz);
  } else {
    px = sp.prior_icov[3 * k]; py = sp.prior_icov[3 * k + 1]; pz = sp.prior_icov[3 * k + 2];
  }
  double pr_det = px * pz - py * py;
  if (!(pr_det > 0)) atomicExch(&sc->status, STSPIX_ERR_DEGENERATE);
  pr_det = sqrt(pr_det);
  double psx = pc / pr_det * px, psy = pc / pr_det * py, psz = pc / pr_det * pz;
  const long long* a = sp.acc + 8 * (size_t)k;
  float mr = (float)(fx_unq(a[0], kFxAppShift) / count);
  float mg = (float)(fx_unq(a[1], kFxAppShift) / count);
  float mb = (float)(fx_unq(a[2], kFxAppShift) / count);
  sp.mu_app[3 * k] = mr; sp.mu_app[3 * k + 1] = mg; sp.mu_app[3 * k + 2] = mb;
  double mx = a[3] / count, my = a[4] / count;
  sp.mu_shape[2 * k] = mx; sp.mu_shape[2 * k + 1] = my;
  double sx = a[5] - count * mx * mx;
  double sy = a[6] - count * mx * my;
  double sz = a[7] - count * my * my;
  sx = (pc * psx + sx) / (total_count + 3.0);
  sy = (pc * psy + sy) / (total_count + 3.0);
  sz = (pc * psz + sz) / (total_count + 3.0);
  double det = sx * sz - sy * sy;
  if (det <= 0) {
    sx = sx + 0.00001;
    sz = sz + 0.00001;
    det = sx * sz - sy * sy;
    if (det <= 0) det = 0.00001;
  }
  double ix = sz / det, iy = -sy / det, iz = sx / det;
  double ld = log(det);
  sp.sigma_shape[3 * k] = ix; sp.sigma_shape[3 * k + 1] = iy; sp.sigma_shape[3 * k + 2] = iz;
  sp.logdet[k] = ld;
  SweepRec r;
  r.mu_r = mr; r.mu_g = mg; r.mu_b = mb; r.logdet = (float)ld;
  double fx = floor(mx), fy = floor(my);
  r.mxi = (int)fx; r.myi = (int)fy;
  r.frac = (mx != fx ? 1 : 0) | (my != fy ? 2 : 0);
  r.isx = (float)ix; r.isy = (float)iy; r.isz = (float)iz; r.pad = 0.f;
  r.count = count_int;
  sp.rec[k] = r;
}

__global__ void kb_posterior(const Slot* __restrict__ slots) {
  SLOT_Y;
  FOR_SP(k, S.sp.cap) posterior_one(S.sp, S.sp_size, S.sc, k);
}

// clear_fields + the helper memset (update_params.cu:54-88, :26): zero the counts
// and the sums of every slot.
__global__ void kb_clear_stats(const Slot* __restrict__ slots) {
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
  SLOT_Y;
  const SpDev& sp = S.sp;
  FOR_SP(k, sp.cap) {
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
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= H * W) return;
  int x = idx % W, y = idx / W;
  if (y < 1 || x < 1 || y >= H - 1 || x >= W - 1) { border[idx] = 1; return; }
  int C = seg[idx];
  border[idx] = (C != seg[idx - W] || C != seg[idx + W] || C != seg[idx + 1] ||
                 C != seg[idx - 1]) ? 1 : 0;
}

__global__ void kb_find_border(const Slot* __restrict__ slots) {
  SLOT_Y;
  int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= S.npix) return;
  const int W = S.W, H = S.H;
  const int* seg = S.seg;
  int x = idx % W, y = idx / W;
  if (y < 1 || x < 1 || y >= H - 1 || x >= W - 1) { S.border[idx] = 1; return; }
  int C = seg[idx];
  S.border[idx] = (C != seg[idx - W] || C != seg[idx + W] || C != seg[idx + 1] ||
                   C != seg[idx - 1]) ? 1 : 0;
}

__global__ void k_find_border_end(const int* __restrict__ seg, uint8_t* __restrict__ border,
                                  int H, int W, int nframes) {
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
__constant__ unsigned char c_simple_lut[256] = {
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

__device__ __forceinline__ int nbr_code(const int nb[8], int label, int* diff) {
  int num = 0, d = 0;
#pragma unroll
  for (int i = 7; i >= 0; i--) {
    num <<= 1;
    bool b = (label == nb[i]) || (nb[i] == -1);
    if (b) num++; else d++;
  }
  *diff = d;
  return num;
}
__device__ __forceinline__ bool simple_point(const int nb[8], int label, int* diff) {
  return c_simple_lut[nbr_code(nb, label, diff)] != 0;
}
// Same test against the table packed as 8 words in shared memory (divergent
// constant-memory reads serialise across a warp).
__device__ __forceinline__ bool simple_point_s(const unsigned* lut_bits, const int nb[8],
                                               int label, int* diff) {
  int num = nbr_code(nb, label, diff);
  return (lut_bits[num >> 5] >> (num & 31)) & 1u;
}

__device__ __forceinline__ void joint(const float* __restrict__ pix, int x, int y,
                                      const SweepRec& r, int k, float s2, float neigh_neq,
                                      float beta, float* best, int* best_label) {
  float res = -1000;
  const float x0 = pix[0] - r.mu_r;
  const float x1 = pix[1] - r.mu_g;
  const float x2 = pix[2] - r.mu_b;
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
// A block owns a 32x32 tile and stages labels of the tile plus a 4-pixel halo
// (phase k is evaluated on the tile grown by 3-k pixels, so every label a tile
// pixel depends on is produced inside the block exactly as the four separate
// launches produce it), the image and the border mask of the tile plus 3 pixels.
// Labels are read from seg_in (labels at the sweep start) and the tile is
// written to seg_out, so neighbouring blocks never see each other's updates.
constexpr int kST = 32;               // tile side
constexpr int kSH = 4;                // label halo
constexpr int kSL = kST + 2 * kSH;    // 40: staged label side
constexpr int kSI = kST + 2 * (kSH - 1);  // 38: staged image / border side

__global__ void __launch_bounds__(256) kb_sweep(const Slot* __restrict__ slots, int parity,
                                                float s2, float potts) {
  SLOT_Z;
  const int H = S.H, W = S.W;
  if ((int)blockIdx.x * kST >= W || (int)blockIdx.y * kST >= H) return;
  const float* __restrict__ img = S.img;
  const int* __restrict__ seg_in = parity ? S.seg_alt : S.seg;
  int* __restrict__ seg_out = parity ? S.seg : S.seg_alt;
  const SweepRec* __restrict__ rec = S.sp.rec;
  const int cap = S.sp.cap;
  constexpr int kMaxList = (kST / 2 + kSH - 1) * (kST / 2 + kSH - 1);  // 19 x 19
  __shared__ int L[kSL * kSL];
  __shared__ float I[kSI * kSI * 3];
  __shared__ short list[4][kMaxList];   // border pixels of each parity phase
  __shared__ int cnt[4];
  __shared__ unsigned lut_bits[8];
  if (threadIdx.x < 8) {
    unsigned w = 0;
    for (int b = 0; b < 32; b++) w |= (unsigned)(c_simple_lut[threadIdx.x * 32 + b] != 0) << b;
    lut_bits[threadIdx.x] = w;
  }
  if (threadIdx.x < 4) cnt[threadIdx.x] = 0;
  const int tx0 = blockIdx.x * kST, ty0 = blockIdx.y * kST;
  const int rx0 = tx0 - kSH, ry0 = ty0 - kSH;        // label region origin
  const int ix0 = tx0 - (kSH - 1), iy0 = ty0 - (kSH - 1);  // image region origin
  for (int i = threadIdx.x; i < kSL * kSL; i += blockDim.x) {
    int gx = rx0 + i % kSL, gy = ry0 + i / kSL;
    L[i] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? seg_in[gy * W + gx] : -1;
  }
  for (int i = threadIdx.x; i < kSI * kSI; i += blockDim.x) {
    int gx = ix0 + i % kSI, gy = iy0 + i / kSI;
    if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
      const float* p = img + 3 * ((size_t)gy * W + gx);
      I[3 * i] = p[0]; I[3 * i + 1] = p[1]; I[3 * i + 2] = p[2];
    }
  }
  __syncthreads();
  // Border mask at the sweep start (find_border_pixels, seg_utils.cu:164-195); the
  // border pixels of parity class k inside the tile grown by 3-k pixels are listed
  // for phase k, so each phase scores only its border pixels, densely.
  for (int i = threadIdx.x; i < kSI * kSI; i += blockDim.x) {
    int lx = i % kSI, ly = i / kSI;
    int gx = ix0 + lx, gy = iy0 + ly;
    if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
    bool b;
    if (gy < 1 || gx < 1 || gy >= H - 1 || gx >= W - 1) {
      b = true;
    } else {
      int p = (ly + 1) * kSL + (lx + 1);
      int C = L[p];
      b = (C != L[p - kSL] || C != L[p + kSL] || C != L[p + 1] || C != L[p - 1]);
    }
    if (!b) continue;
    int ph = ((gx & 1) << 1) | (gy & 1);
    int grow = 3 - ph;
    if (gx < tx0 - grow || gx >= tx0 + kST + grow || gy < ty0 - grow || gy >= ty0 + kST + grow)
      continue;
    int slot = atomicAdd(&cnt[ph], 1);
    list[ph][slot] = (short)i;
  }
  __syncthreads();
  for (int ph = 0; ph < 4; ph++) {
    const int n = cnt[ph];
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
      int bi = list[ph][j];
      int lxi = bi % kSI, lyi = bi / kSI;
      int gx = ix0 + lxi, gy = iy0 + lyi;
      int p = (lyi + 1) * kSL + (lxi + 1);
      int C = L[p];
      if (C < 0 || C >= cap) continue;
      const int N = L[p - kSL], S = L[p + kSL], Wl = L[p - 1], E = L[p + 1];
      const int NW = L[p - kSL - 1], NE = L[p - kSL + 1], SW = L[p + kSL - 1],
                SE = L[p + kSL + 1];
      const int nb[8] = {NW, N, NE, Wl, E, SW, S, SE};
      int dN, dW, dS, dE;
      bool vN = simple_point_s(lut_bits, nb, N, &dN);
      bool vW = simple_point_s(lut_bits, nb, Wl, &dW);
      bool vS = simple_point_s(lut_bits, nb, S, &dS);
      bool vE = simple_point_s(lut_bits, nb, E, &dE);
      if (!vN || !vW || !vS || !vE) continue;
      if (N >= cap || S >= cap || Wl >= cap || E >= cap) continue;
      const float* pix = &I[3 * bi];
      float best = -9999.f;
      int bl = C;
      if (N >= 0) joint(pix, gx, gy, rec[N], N, s2, (float)dN, potts, &best, &bl);
      if (S != N && S >= 0) joint(pix, gx, gy, rec[S], S, s2, (float)dS, potts, &best, &bl);
      if (Wl != S && Wl != N && Wl >= 0)
        joint(pix, gx, gy, rec[Wl], Wl, s2, (float)dW, potts, &best, &bl);
      if (E != Wl && E != S && E != N && E >= 0)
        joint(pix, gx, gy, rec[E], E, s2, (float)dE, potts, &best, &bl);
      if (rec[C].count <= 2 && bl == C) {
        if (N >= 0) bl = N;
        else if (E >= 0) bl = E;
        else if (S >= 0) bl = S;
        else if (Wl >= 0) bl = Wl;
      }
      L[p] = bl;
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < kST * kST; i += blockDim.x) {
    int gx = tx0 + i % kST, gy = ty0 + i / kST;
    if (gx < W && gy < H) seg_out[gy * W + gx] = L[(gy - ry0) * kSL + (gx - rx0)];
  }
}

// ---------------------------------------------------------------------------
// Parameter read-out (read_params, sparams_io.cu:190-286) and prior update
// (update_prior_kernel, sparams_io.cu:584-640) into the caller's SoA params.
__global__ void kb_read_params(const Slot* __restrict__ slots) {
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
  SLOT_Y;
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < S.cap + 2) S.flags[k] = 0;
}

// Keep a copy of the finished labels where the slot's video stream resides.
__global__ void kb_save_prev(const Slot* __restrict__ slots) {
  SLOT_Y;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (S.resident_labels && i < S.npix) S.resident_labels[i] = S.seg[i];
}

__global__ void kb_copy_labels(const Slot* __restrict__ slots) {
  SLOT_Y;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < S.npix) S.seg[i] = S.seg_alt[i];
}

__global__ void k_dump_state(SpDev sp, stspix_state_dump d) {
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
