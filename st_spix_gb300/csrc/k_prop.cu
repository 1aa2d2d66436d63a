// GB300 kernels of the optical-flow propagation path (gauenk/st_spix
// st_spix/csrc/bist/shift_and_fill.cu, sp_pooling.cu, shift_labels.cu,
// fill_missing.cu, split_disconnected.cu, relabel.cu, sparams_io.cu, prop.cu).
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace stspix {

// ---------------------------------------------------------------------------
// Mean flow per superpixel (sp_downsample_kernel / normz_downsample_kernel,
// sp_pooling.cu:27-71), R1 fixed point.  Runs of equal labels in a row are
// aggregated before the atomics.
__global__ void k_flow_pool(const int* __restrict__ lab, const float* __restrict__ flow, int H,
                            int W, int n, int* __restrict__ cnt,
                            long long* __restrict__ fs) {
  constexpr int R = 16;
  const int cpr = (W + R - 1) / R;
  int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= H * cpr) return;
  int y = tid / cpr, xs = (tid % cpr) * R, xe = min(W, xs + R);
  const int* lrow = lab + (size_t)y * W;
  const float* frow = flow + (size_t)y * W * 2;
  int cur = -1, c = 0;
  long long sx = 0, sy = 0;
  for (int x = xs; x <= xe; x++) {
    int k = x < xe ? lrow[x] : -2;
    if (k != cur) {
      if (cur >= 0 && cur < n) {
        atomicAdd(&cnt[cur], c);
        atomicAdd((unsigned long long*)&fs[2 * (size_t)cur], (unsigned long long)sx);
        atomicAdd((unsigned long long*)&fs[2 * (size_t)cur + 1], (unsigned long long)sy);
      }
      cur = k; c = 0; sx = sy = 0;
    }
    if (x < xe && k >= 0) {
      c++;
      sx += fx_q(frow[2 * x], kFxFlowShift);
      sy += fx_q(frow[2 * x + 1], kFxFlowShift);
    }
  }
}

// normz + centres = mu_shape + mean flow (shift_and_fill.cu:140-150).
__global__ void k_flow_mean(int n, const int* __restrict__ cnt,
                            const long long* __restrict__ fs, const double* __restrict__ mu_shape,
                            float* __restrict__ fds, double* __restrict__ centers) {
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
__global__ void k_shift(const int* __restrict__ lab, int H, int W, int n,
                        const int* __restrict__ cnt, const float* __restrict__ fds,
                        int* __restrict__ hits, unsigned long long* __restrict__ best) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= H * W) return;
  int k = lab[t];
  if (k < 0 || k >= n) return;
  int size = cnt[k];
  int fw = (int)roundf(fds[2 * k]);
  int fh = (int)roundf(fds[2 * k + 1]);
  int w = t % W + fw, h = t / W + fh;
  if (w < 0 || w >= W || h < 0 || h >= H) return;
  int d = h * W + w;
  atomicAdd(&hits[d], 1);
  unsigned long long key = ((unsigned long long)(unsigned int)size << 32) | (unsigned int)k;
  atomicMin(&best[d], key);
}

// decode_kernel (shift_labels.cu:128-164) + copy to `filled` + hole count.
__global__ void k_shift_decode(const int* __restrict__ hits,
                               const unsigned long long* __restrict__ best, int npix,
                               int* __restrict__ shifted, int* __restrict__ filled,
                               Scalars* sc) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  int v = hits[t] > 0 ? (int)(unsigned int)best[t] : -1;
  shifted[t] = v;
  filled[t] = v;
  unsigned mask = __ballot_sync(__activemask(), v < 0);
  if ((threadIdx.x & 31) == (__ffs(__activemask()) - 1) && mask)
    atomicAdd(&sc->ninvalid, __popc(mask));
}

// Per-label pixel counts (get_spix_sizes, seg_utils.cu:56-75).
__global__ void k_count_labels(const int* __restrict__ lab, int npix, int n,
                               int* __restrict__ cnt) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  int k = lab[t];
  if (k >= 0 && k < n) atomicAdd(&cnt[k], 1);
}

// ---------------------------------------------------------------------------
// Hole filling (fill_missing.cu:35-130, update_missing_seg_nn :288-441,
// find_border_along_missing :617-647) as one cooperative kernel: per iteration a
// border/count pass and four parity phases, separated by bounded grid barriers.
__global__ void __launch_bounds__(256) k_fill_coop(int* seg, const double* __restrict__ centers,
                                                   int H, int W, uint8_t* border, Scalars* sc,
                                                   int* iter_counts, int break_iter) {
  const int npix = H * W;
  const int nthr = gridDim.x * blockDim.x;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  __shared__ int red[8];
  int prev_neg = 1410065408;  // (int)10000000000 as the reference truncates it
  for (int iter = 0;; iter++) {
    if (break_iter > 0 && iter >= break_iter) break;
    int local = 0;
    for (int idx = gt; idx < npix; idx += nthr) {
      int x = idx % W, y = idx / W;
      int N = -1, S = -1, E = -1, Wl = -1;
      if (y > 0) N = __ldcg(seg + idx - W);
      if (x > 0) Wl = __ldcg(seg + idx - 1);
      if (y < H - 1) S = __ldcg(seg + idx + W);
      if (x < W - 1) E = __ldcg(seg + idx + 1);
      border[idx] = (N >= 0 || Wl >= 0 || S >= 0 || E >= 0) ? 1 : 0;
      if (__ldcg(seg + idx) < 0) local++;
    }
    // block reduction of the hole count
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
      int s = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
      if (s) atomicAdd(&iter_counts[iter], s);
    }
    if (!grid_barrier(sc)) return;
    const int num_neg = *(volatile int*)&iter_counts[iter];
    for (int ph = 0; ph < 4; ph++) {
      const int xm = ph >> 1, ym = ph & 1;
      const int hw = (W - xm + 1) / 2, hh = (H - ym + 1) / 2;
      for (int i = gt; i < hw * hh; i += nthr) {
        int x = 2 * (i % hw) + xm, y = 2 * (i / hw) + ym;
        int idx = y * W + x;
        if (!__ldcg(border + idx) || __ldcg(seg + idx) != -1) continue;
        int N = -1, S = -1, E = -1, Wl = -1;
        if (x > 0) Wl = __ldcg(seg + idx - 1);
        if (y > 0) N = __ldcg(seg + idx - W);
        if (x < W - 1) E = __ldcg(seg + idx + 1);
        if (y < H - 1) S = __ldcg(seg + idx + W);
        float bx = -999999;
        int bl = -1;
        auto consider = [&](int lab) {
          const double* cp = centers + 2 * (size_t)lab;
          float dx = (1.0f * x - cp[0]) / (1.0f * W);
          float dy = (1.0f * y - cp[1]) / (1.0f * H);
          float sim = -dx * dx - dy * dy;
          if (sim > bx) { bx = sim; bl = lab; }
        };
        if (N >= 0) consider(N);
        if (S >= 0 && S != N) consider(S);
        if (Wl >= 0 && Wl != S && Wl != N) consider(Wl);
        if (E >= 0 && E != Wl && E != S && E != N) consider(E);
        __stcg(seg + idx, bl);
      }
      if (!grid_barrier(sc)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&sc->fill_iters, 1);
    if (num_neg == prev_neg) {
      if (blockIdx.x == 0 && threadIdx.x == 0) atomicExch(&sc->status, STSPIX_ERR_NOPROGRESS);
      return;
    }
    prev_neg = num_neg;
    if (num_neg <= 0) return;
  }
}

// ---------------------------------------------------------------------------
// Disconnected regions (split_disconnected.cu:33-96): roots from the cooperative
// relaxation (mode 1), sizes, largest region per label (R6), invalidate the rest.
__global__ void k_cc_init(const int* __restrict__ seg, int npix, int* __restrict__ root) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  root[t] = seg[t] >= 0 ? t : -1;
}

__global__ void k_cc_size(const int* __restrict__ root, int npix, int* __restrict__ size) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  int r = root[t];
  if (r >= 0) atomicAdd(&size[r], 1);
}

__global__ void k_cc_best(const int* __restrict__ seg, const int* __restrict__ root,
                          const int* __restrict__ size, int npix, int nlab,
                          unsigned long long* __restrict__ best) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix || root[t] != t) return;
  int L = seg[t];
  if (L < 0 || L >= nlab) return;
  unsigned long long key = ((unsigned long long)(unsigned int)size[t] << 32) |
                           (unsigned long long)(0xffffffffu - (unsigned int)t);
  atomicMax(&best[L], key);
}

__global__ void k_cc_invalidate(int* __restrict__ seg, const int* __restrict__ root, int npix,
                                int nlab, const unsigned long long* __restrict__ best) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  int L = seg[t];
  if (L < 0 || L >= nlab) return;
  unsigned int win = 0xffffffffu - (unsigned int)(best[L] & 0xffffffffull);
  if ((unsigned int)root[t] != win) seg[t] = -1;
}

// invalid_counts / prior_counts update (shift_and_fill.cu:300-330).
__global__ void k_shift_params(int n, const int* __restrict__ cnt_pool,
                               const int* __restrict__ cs, const int* __restrict__ cf,
                               stspix_params pp) {
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
__global__ void k_write_params(SpDev sp, const stspix_params pp, int n, int sp_size) {
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

__global__ void k_mark_active(const int* __restrict__ lab, int npix, SpDev sp) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  int v = lab[t];
  if (v >= 0 && v < sp.cap) { sp.valid[v] = 1; sp.prop[v] = 1; }
}

__global__ void k_prop_begin(Scalars* sc, int n) {
  sc->max_spix = n - 1;
  sc->nbuf_logical = 10 * n;
}

// ---------------------------------------------------------------------------
// Relabel (relabel.cu:126-409), R5.
__global__ void k_living(const int* __restrict__ seg, int npix, const Scalars* __restrict__ sc,
                         uint8_t* __restrict__ living) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  int v = seg[t];
  if (v >= 0 && v <= sc->max_spix) living[v] = 1;
}

__global__ void k_relabel_init(int cap, unsigned long long* __restrict__ best,
                               float* __restrict__ ss) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= cap) return;
  best[s] = ((unsigned long long)__float_as_uint(10000.f) << 32) | 0x7fffffffull;
  ss[s] = 0.f;
}

// find_most_similar_spix (relabel.cu:201-276): grid (s, candidate chunk).
__global__ void k_relabel_compare(const SpDev sp, const float* __restrict__ prev_prior_mu_app,
                                  int n_prev, const Scalars* __restrict__ sc,
                                  const uint8_t* __restrict__ living,
                                  unsigned long long* __restrict__ best, float* __restrict__ ss,
                                  int chunk) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int nspix = sc->max_spix + 1;
  if (s >= nspix || s >= sp.cap || !living[s]) return;
  int c0 = blockIdx.y * chunk, c1 = min(n_prev, c0 + chunk);
  const float mx = sp.mu_app[3 * s], my = sp.mu_app[3 * s + 1], mz = sp.mu_app[3 * s + 2];
  unsigned long long b = ~0ull;
  for (int c = c0; c < c1; c++) {
    bool same = (c == s);
    if (c < nspix && living[c] && !same) continue;
    float dx = mx - prev_prior_mu_app[3 * c];
    float dy = my - prev_prior_mu_app[3 * c + 1];
    float dz = mz - prev_prior_mu_app[3 * c + 2];
    float delta = (dx * dx + dy * dy + dz * dz);
    if (same) ss[s] = delta;
    if (delta < 10000.f) {
      unsigned long long key = ((unsigned long long)__float_as_uint(delta) << 32) | (unsigned)c;
      if (key < b) b = key;
    }
  }
  if (b != ~0ull) atomicMin(&best[s], b);
}

// mark_for_relabel (relabel.cu:126-192): revive flags and mint flags.
__global__ void k_relabel_mark(int cap, const Scalars* __restrict__ sc,
                               const uint8_t* __restrict__ living,
                               const unsigned long long* __restrict__ best,
                               const float* __restrict__ ss, float thresh_replace,
                               float thresh_new, int* __restrict__ rid,
                               uint8_t* __restrict__ mint) {
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

__global__ void k_relabel_ids(int cap, Scalars* sc, const uint8_t* __restrict__ mint,
                              const int* __restrict__ excl, int* __restrict__ rid,
                              int* __restrict__ src_of) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= cap) return;
  if (mint[s]) rid[s] = sc->max_spix + 1 + excl[s];
  int n = rid[s];
  if (n >= 0 && n < cap) atomicMax(&src_of[n], s);
  else if (n >= cap) atomicExch(&sc->status, STSPIX_ERR_CAPACITY);
}

// relabel_spix_kernel parameter copies (relabel.cu:86-120), from the largest
// reviving superpixel.
__global__ void k_relabel_params(SpDev sp, const int* __restrict__ rid,
                                 const int* __restrict__ src_of,
                                 int n_prev) {
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

__global__ void k_relabel_apply(int* __restrict__ seg, int npix, int cap,
                                const int* __restrict__ rid) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  int v = seg[t];
  if (v < 0 || v >= cap) return;
  int n = rid[v];
  if (n >= 0 && n < cap) seg[t] = n;
}

__global__ void k_relabel_end(Scalars* sc, const int* __restrict__ nminted,
                              const int* __restrict__ rid, int cap) {
  // single thread: bump max_spix, count revived ids for the log
  int m = *nminted;
  sc->nminted += m;
  sc->max_spix += m;
}

__global__ void k_count_revived(const int* __restrict__ rid, const uint8_t* __restrict__ mint,
                                int cap, Scalars* sc) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= cap) return;
  if (rid[s] >= 0 && !mint[s]) atomicAdd(&sc->nrevived, 1);
}

}  // namespace stspix
