// Kernels of the legacy prop_cuda surface (gauenk/st_spix st_spix/csrc/prop/,
// bound by st_spix/csrc/pybind_prop.cpp): the per-superpixel integer-flow label
// shift, the hole fill on a given list of missing pixels with FP32 centres, and
// video superpixel pooling for any number of features.  Each kernel restates the
// legacy kernel's arithmetic; the pooling sums in FP64 where the legacy kernel adds
// FP32 atomics in arbitrary order.
#include <cstdint>
#include <cuda_runtime.h>

#include "kernels.h"

namespace stspix {

__global__ void k_fill_i32(int32_t* p, long long n, int32_t v) {
  pdl_enter();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// shift_labels_kernel (prop/shift_labels.cu:31-80): every pixel moves by its
// superpixel's integer flow (dx, dy); a destination counts its arrivals and keeps
// the largest arriving label.  Labels outside [0, nspix) are skipped (the legacy
// kernel reads the flow table out of bounds for them).
__global__ void k_lshift(const int32_t* __restrict__ spix, const int32_t* __restrict__ flow,
                         int nspix, int H, int W, int32_t* shifted, int32_t* counts) {
  pdl_enter();
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= H * W) return;
  const int s = spix[idx];
  if (s < 0 || s >= nspix) return;
  const int y = idx / W, x = idx % W;
  const int yd = y + flow[2 * s + 1], xd = x + flow[2 * s];
  if (yd < 0 || yd >= H || xd < 0 || xd >= W) return;
  const int d = yd * W + xd;
  atomicAdd(&counts[d], 1);
  atomicMax(&shifted[d], s);
}

// find_border_along_missing (prop/fill_missing.cu:258-292): a listed pixel still
// missing and with a labelled 4-neighbour is on the border; *num_neg counts the
// listed pixels still missing.
__global__ void k_lfill_border(const int32_t* __restrict__ seg, const int32_t* __restrict__ missing,
                               int nmissing, int H, int W, uint8_t* border, int* num_neg) {
  pdl_enter();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nmissing) return;
  const int idx = missing[j];
  const int x = idx % W, y = idx / W;
  const int C = seg[idx];
  int N = -1, S = -1, E = -1, Wl = -1;
  if (y > 0) N = seg[idx - W];
  if (x > 0) Wl = seg[idx - 1];
  if (y < H - 1) S = seg[idx + W];
  if (x < W - 1) E = seg[idx + 1];
  const bool valid = N >= 0 || Wl >= 0 || S >= 0 || E >= 0;
  border[j] = (valid && C < 0) ? 1 : 0;
  if (C < 0) atomicAdd(num_neg, 1);
}

// update_missing_seg_nn (prop/fill_missing.cu:142-256) for parity (xm, ym): a border
// pixel takes the 4-neighbour label whose FP32 centre is nearest in normalised
// coordinates (first maximum in N, S, W, E order).
__global__ void k_lfill_phase(int32_t* seg, const float* __restrict__ centers, int ncenters,
                              const int32_t* __restrict__ missing, const uint8_t* __restrict__ border,
                              int nmissing, int H, int W, int xm, int ym) {
  pdl_enter();
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nmissing || !border[j]) return;
  const int idx = missing[j];
  const int x = idx % W, y = idx / W;
  if (x % 2 != xm || y % 2 != ym) return;
  int N = -1, S = -1, E = -1, Wl = -1;
  if (x > 0) Wl = seg[idx - 1];
  if (y > 0) N = seg[idx - W];
  if (x < W - 1) E = seg[idx + 1];
  if (y < H - 1) S = seg[idx + W];
  float best = -999999.f, lab = -1.f;
  auto consider = [&](int l) {
    if (l >= ncenters) return;   // no centre row (the legacy kernel reads out of bounds)
    const float dx = (1.0f * x - centers[2 * l]) / (1.0f * W);
    const float dy = (1.0f * y - centers[2 * l + 1]) / (1.0f * H);
    const float sim = -dx * dx - dy * dy;
    if (sim > best) { best = sim; lab = (float)l; }
  };
  if (N >= 0) consider(N);
  if (S >= 0 && S != N) consider(S);
  if (Wl >= 0 && Wl != S && Wl != N) consider(Wl);
  if (E >= 0 && E != Wl && E != S && E != N) consider(E);
  seg[idx] = (int)lab;
}

// sp_video_pooling (prop/sp_video_pooling.cu:20-58, 61-120): per batch item, the
// feature sums and pixel counts of every id over all frames, the mean
// (sum / (count + 1e-10) in FP32, as the legacy in-place division), and the pooled
// video.  Grid: (pixel blocks, batch, frames).
__global__ void k_vpool_accum(const float* __restrict__ img, const int32_t* __restrict__ seg,
                              int T, long long npix, int F, int nspix, double* sum,
                              unsigned long long* cnt) {
  pdl_enter();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int b = blockIdx.y, t = blockIdx.z;
  const long long g = ((long long)b * T + t) * npix + p;
  const int s = seg[g];
  if (s < 0 || s >= nspix) return;
  const size_t bs = (size_t)b * nspix + s;
  for (int f = 0; f < F; f++) atomicAdd(&sum[bs * F + f], (double)img[g * F + f]);
  atomicAdd(&cnt[bs], 1ull);
}

__global__ void k_vpool_mean(const double* __restrict__ sum, const unsigned long long* __restrict__ cnt,
                             long long nbs, int F, float* down, float* counts) {
  pdl_enter();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbs) return;
  const float c = (float)cnt[i];
  if (counts) counts[i] = c;
  for (int f = 0; f < F; f++) down[i * F + f] = (float)sum[i * F + f] / (c + 1e-10f);
}

// run_sp_video_pooling (prop/sp_video_pooling.cu:33-58): pooled pixel = its id's
// row of down (pixels with a negative id stay 0).
__global__ void k_vpool_write(const float* __restrict__ down, const int32_t* __restrict__ seg,
                              int T, long long npix, int F, int nspix, float* pooled) {
  pdl_enter();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const int b = blockIdx.y, t = blockIdx.z;
  const long long g = ((long long)b * T + t) * npix + p;
  const int s = seg[g];
  if (s < 0 || s >= nspix) return;
  const float* d = down + ((size_t)b * nspix + s) * F;
  for (int f = 0; f < F; f++) pooled[g * F + f] = d[f];
}

// run_update_prior (prop/sparams_io.cu:795-834): the ids present in spix (unique ids
// there, presence flags here) at or above prev_nspix take their estimates as priors
// (update_prior_kernel, :743-792; the shape prior is the covariance, inverted when
// `invert`, with a negative determinant replaced by 1e-6).
__global__ void k_lmark_ids(const int32_t* __restrict__ spix, long long n, int nids,
                            uint8_t* present) {
  pdl_enter();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int s = spix[i];
  if (s >= 0 && s < nids) present[s] = 1;
}

__global__ void k_lupdate_prior(const uint8_t* __restrict__ present, int nids, int prev_nspix,
                                int invert, const float* __restrict__ mu_app, float* prior_mu_app,
                                const double* __restrict__ mu_shape, double* prior_mu_shape,
                                const double* __restrict__ sigma_shape, double* prior_sigma_shape) {
  pdl_enter();
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nids || !present[k] || k < prev_nspix) return;
  for (int c = 0; c < 3; c++) prior_mu_app[3 * k + c] = mu_app[3 * k + c];
  for (int c = 0; c < 2; c++) prior_mu_shape[2 * k + c] = mu_shape[2 * k + c];
  const double xx = sigma_shape[3 * k], xy = sigma_shape[3 * k + 1], yy = sigma_shape[3 * k + 2];
  double det = xx * yy - xy * xy;
  if (det < 0) det = 0.000001;
  if (invert) {
    prior_sigma_shape[3 * k] = yy / det;
    prior_sigma_shape[3 * k + 1] = -xy / det;
    prior_sigma_shape[3 * k + 2] = xx / det;
  } else {
    prior_sigma_shape[3 * k] = xx;
    prior_sigma_shape[3 * k + 1] = xy;
    prior_sigma_shape[3 * k + 2] = yy;
  }
}

// shift_tensor_kernel (prop/shift_tensor.cu:15-57) and shift_tensor_ordered_kernel
// (prop/shift_tensor_ordered.cu:14-50): every pixel moves by its superpixel's integer
// flow; a destination adds the moved features and counts the arrivals (ordered: only
// pixels of the destination's selected id); contributors[dest, id] marks the ids that
// arrive.  Features are added in FP64 (the legacy kernels add FP32 atomics in arbitrary
// order) and rounded once.  Labels outside [0, nspix) are skipped (the legacy kernels
// read the flow table out of bounds for them).  Grid: (pixel blocks, batch).
__global__ void k_lshift_tensor(const float* __restrict__ in, const int32_t* __restrict__ spix,
                                const int32_t* __restrict__ flow, int H, int W, int F, int nspix,
                                const int32_t* __restrict__ selected, double* acc,
                                int32_t* counts, uint8_t* contributors) {
  pdl_enter();
  const int npix = H * W;
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix) return;
  const long long b = blockIdx.y;
  const long long src = b * npix + p;
  const int s = spix[src];
  if (s < 0 || s >= nspix) return;
  const int y = p / W, x = p % W;
  const int* f = flow + 2 * (b * nspix + s);
  const int yd = y + f[1], xd = x + f[0];
  if (yd < 0 || yd > H - 1 || xd < 0 || xd > W - 1) return;
  const long long dst = b * npix + (long long)yd * W + xd;
  if (selected && selected[dst] != s) return;
  atomicAdd(&counts[dst], 1);
  for (int c = 0; c < F; c++) atomicAdd(&acc[dst * F + c], (double)in[src * F + c]);
  if (contributors) contributors[dst * nspix + s] = 1;
}

__global__ void k_round_f32(const double* __restrict__ acc, long long n, float* out) {
  pdl_enter();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (float)acc[i];
}

// shift_order_kernel (prop/shift_order.cu:14-40): the legacy loop updates its running
// minimum only while the current value is below it, which after the first
// contributing id never holds again, so the selected id is the first (smallest)
// contributing one, or -1.
__global__ void k_lshift_order(const uint8_t* __restrict__ contributors, long long npix_all,
                               int nspix, int32_t* selected) {
  pdl_enter();
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npix_all) return;
  const uint8_t* c = contributors + p * nspix;
  int sel = -1;
  for (int s = 0; s < nspix; s++)
    if (c[s]) { sel = s; break; }
  if (sel >= 0) selected[p] = sel;
}

// split_disconnected (prop/split_disconnected.cu:31-255): regions are the connected
// components of equal labels in which two pixels within Chebyshev distance 2 are
// neighbours (find_spix_min's 5x5 window, :303-330), numbered by their smallest pixel
// index; every region but the largest of a label (the first largest in region order)
// gets a new id nspix + split_start[label] + its rank among the label's regions.
// Union-find with min-index hooking gives every pixel its region's smallest index,
// the fixed point of find_spix_min.
__global__ void k_lsd_init(int32_t* parent, int npix) {
  pdl_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < npix) parent[t] = t;
}

__device__ __forceinline__ int lsd_find(int32_t* parent, int x) {
  for (int i = 0; i < (1 << 26); i++) {
    const int p = *(volatile int32_t*)&parent[x];
    if (p == x) return x;
    const int g = *(volatile int32_t*)&parent[p];
    if (g == p) return p;
    atomicMin(&parent[x], g);
    x = g;
  }
  return -1;
}

__global__ void k_lsd_hook(const int32_t* __restrict__ spix, int H, int W, int32_t* parent,
                           int* status) {
  pdl_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= H * W) return;
  const int x = t % W, y = t / W, L = spix[t];
  // the 12 earlier pixels of the 5x5 window (the later ones hook to this one)
  for (int dy = -2; dy <= 0; dy++) {
    for (int dx = -2; dx <= 2; dx++) {
      if (dy == 0 && dx >= 0) break;
      const int yy = y + dy, xx = x + dx;
      if (yy < 0 || xx < 0 || xx >= W) continue;
      const int q = yy * W + xx;
      if (spix[q] != L) continue;
      int a = t, b = q;
      bool done = false;
      for (int i = 0; i < (1 << 26) && !done; i++) {
        a = lsd_find(parent, a);
        b = lsd_find(parent, b);
        if (a < 0 || b < 0) break;
        if (a == b) { done = true; break; }
        if (a < b) { const int tmp = a; a = b; b = tmp; }
        const int old = atomicMin(&parent[a], b);
        if (old == a) done = true;
        else a = old;
      }
      if (!done) atomicExch(status, 1);
    }
  }
}

__global__ void k_lsd_roots(int32_t* parent, int npix, int32_t* is_root) {
  pdl_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const int r = lsd_find(parent, t);
  parent[t] = r;
  is_root[t] = r == t ? 1 : 0;
}

// Exclusive scan of n ints in one block (n up to a few million: each thread scans a
// contiguous chunk, the chunk totals are scanned in shared memory); total -> *total.
__global__ void k_lscan(const int32_t* __restrict__ in, int n, int32_t* out, int32_t* total) {
  pdl_enter();
  __shared__ int32_t part[1024];
  const int nt = blockDim.x, t = threadIdx.x;
  const int chunk = (n + nt - 1) / nt;
  const int i0 = min(n, t * chunk), i1 = min(n, i0 + chunk);
  int s = 0;
  for (int i = i0; i < i1; i++) s += in[i];
  part[t] = s;
  __syncthreads();
  for (int off = 1; off < nt; off <<= 1) {
    const int v = t >= off ? part[t - off] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  int run = part[t] - s;
  for (int i = i0; i < i1; i++) { const int v = in[i]; out[i] = run; run += v; }
  if (t == nt - 1 && total) *total = part[t];
}

// Per region (index = rank of its root): its label and size; per label: its number
// of regions.
__global__ void k_lsd_regions(const int32_t* __restrict__ spix, const int32_t* __restrict__ root,
                              const int32_t* __restrict__ rank, int npix, int nspix,
                              int32_t* region_of, int32_t* region_spix, int32_t* region_size,
                              int32_t* spix_counts) {
  pdl_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const int r = rank[root[t]];
  region_of[t] = r;
  atomicAdd(&region_size[r], 1);
  if (root[t] == t) {
    region_spix[r] = spix[t];
    atomicAdd(&spix_counts[spix[t]], 1);
  }
}

// get_split_starts (prop/split_disconnected.cu:126-152): c = max(count - 1, 0); over the
// labels with c > 0, split_start = inclusive prefix sum of c minus the first such c
// (which gives ids that collide when a label has three or more regions, as the
// legacy code does); max_nsplits = the last prefix sum.  One block.
__global__ void k_lsd_starts(const int32_t* __restrict__ spix_counts, int nspix,
                             int32_t* split_starts, int32_t* max_nsplits) {
  pdl_enter();
  if (threadIdx.x != 0) return;
  int cum = 0, first = -1;
  for (int s = 0; s < nspix; s++) {
    const int c = max(spix_counts[s] - 1, 0);
    split_starts[s] = 0;
    if (c <= 0) continue;
    cum += c;
    if (first < 0) first = cum;
    split_starts[s] = cum - first;
  }
  *max_nsplits = cum;
}

// compute_offsets (prop/split_disconnected.cu:194-226): a label's regions are ranked in
// region order; the first largest one swaps ranks with the first one (rank 0 keeps
// the label).
__global__ void k_lsd_offsets(const int32_t* __restrict__ region_spix,
                              const int32_t* __restrict__ region_size, int nregions, int nspix,
                              int32_t* region_offset) {
  pdl_enter();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nspix) return;
  int child = 0, cur_max = -1, idx_max = -1, idx_zero = -1;
  for (int r = 0; r < nregions; r++) {
    if (region_spix[r] != s) continue;
    if (child == 0) idx_zero = r;
    region_offset[r] = child;
    if (region_size[r] > cur_max) { idx_max = r; cur_max = region_size[r]; }
    child++;
  }
  if (child > 0 && idx_max != idx_zero) {
    region_offset[idx_zero] = region_offset[idx_max];
    region_offset[idx_max] = 0;
  }
}

// update_spix (prop/split_disconnected.cu:156-181).
__global__ void k_lsd_update(int32_t* spix, const int32_t* __restrict__ region_of,
                             const int32_t* __restrict__ region_offset,
                             const int32_t* __restrict__ split_starts, int npix, int nspix,
                             int max_nchild, int32_t* children) {
  pdl_enter();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const int s = spix[t];
  const int off = region_offset[region_of[t]];
  if (off > 0) {
    const int id = nspix + split_starts[s] + off;
    spix[t] = id;
    children[(size_t)s * max_nchild + off - 1] = id;
  }
}

}  // namespace stspix
