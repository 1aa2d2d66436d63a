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

}  // namespace stspix
