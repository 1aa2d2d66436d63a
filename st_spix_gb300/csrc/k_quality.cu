// Superpixel quality metrics on the device (gauenk/st_spix
// st_spix/spix_utils/evaluate.py:94-512): per-frame id sizes, temporal extent and
// size variation, explained variance (per frame and over the video), PSNR of the
// pooled video, and under-segmentation error / segmentation accuracy against a
// ground-truth segmentation.
//
// Two passes over the pixels, then small per-id kernels:
//   k_q_accum  one warp per 32-pixel row segment; runs of equal (id, ground-truth id)
//              along the row are summed with warp scans and added with one set of
//              atomics per run: per-frame id counts (int32) and colour sums (FP64),
//              video-wide id colour sums, id x ground-truth overlap counts (int32),
//              per-frame colour sums;
//   k_q_resid  per pixel: squared distance to the frame mean (x1 and x255 scale) and
//              to the pixel's pooled colour, block-reduced per frame;
//   k_q_id_time / k_q_frame_ids / k_q_uesa_*  per id: size statistics over time,
//              pooled-vs-mean sums, overlap-based UE / SA sums (integers, exact).
// Pooled colours follow sp_pooling.py:36 (sum / (count + 1e-8)) and
// sp_video_pooling.cu (sum / (count + 1e-10)).
#include <cstdint>
#include <climits>
#include <cuda_runtime.h>

#include "kernels.h"

namespace stspix {

__global__ void k_q_range_init(int* mm) {
  pdl_enter();
  if (threadIdx.x == 0) { mm[0] = INT_MAX; mm[1] = INT_MIN; }
}

// min / max of n labels into mm[0], mm[1] (grid-stride, block reduction).
__global__ void k_q_range(const int32_t* __restrict__ a, long long n, int* mm) {
  pdl_enter();
  int lo = INT_MAX, hi = INT_MIN;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int v = a[i];
    lo = min(lo, v);
    hi = max(hi, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ int slo[32], shi[32];
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) { slo[w] = lo; shi[w] = hi; }
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
    lo = l < nw ? slo[l] : INT_MAX;
    hi = l < nw ? shi[l] : INT_MIN;
    for (int o = 16; o > 0; o >>= 1) {
      lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if (l == 0) { atomicMin(&mm[0], lo); atomicMax(&mm[1], hi); }
  }
}

__device__ __forceinline__ double q_scan(double v, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += t;
  }
  return v;
}

// Pass 1.  Ids are spix - off in [0, S); ground-truth ids in [0, G1) (gt may be null,
// then G1 = 1 and J null).  vid null: counts (and J) only.
__global__ void __launch_bounds__(256) k_q_accum(
    const float* __restrict__ vid, const int32_t* __restrict__ spix,
    const int32_t* __restrict__ gt, int T, int H, int W, int off, int S, int G1,
    int* __restrict__ cnt, double* __restrict__ fsum, double* __restrict__ vsum,
    double* __restrict__ msum, int* __restrict__ J) {
  pdl_enter();
  const int lane = threadIdx.x & 31;
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  const int spr = (W + 31) >> 5;
  const long long per_frame = (long long)H * spr;
  const long long nseg = (long long)T * per_frame;
  for (long long sgi = wid; sgi < nseg; sgi += nw) {
    const int t = (int)(sgi / per_frame);
    const long long r = sgi - t * per_frame;
    const int y = (int)(r / spr), xb = (int)(r - (long long)y * spr) << 5;
    const int x = xb + lane;
    long long key = -1;
    int k = 0, g = 0;
    double q0 = 0, q1 = 0, q2 = 0;
    if (x < W) {
      const size_t idx = ((size_t)t * H + y) * W + x;
      k = spix[idx] - off;
      g = gt ? gt[idx] : 0;
      key = (long long)k * G1 + g;
      if (vid) {
        const float* p = vid + 3 * idx;
        q0 = p[0]; q1 = p[1]; q2 = p[2];
      }
    }
    const long long kprev = __shfl_up_sync(0xffffffffu, key, 1);
    const long long knext = __shfl_down_sync(0xffffffffu, key, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || kprev != key);
    const bool tail = lane == 31 || knext != key;
    const int start = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
    const size_t ts = (size_t)t * S + k;
    if (vid) {
      const double p0 = q_scan(q0, lane), p1 = q_scan(q1, lane), p2 = q_scan(q2, lane);
      const int src = start > 0 ? start - 1 : 0;
      double b0 = __shfl_sync(0xffffffffu, p0, src);
      double b1 = __shfl_sync(0xffffffffu, p1, src);
      double b2 = __shfl_sync(0xffffffffu, p2, src);
      if (start == 0) b0 = b1 = b2 = 0;
      if (lane == 31) {
        atomicAdd(&msum[3 * t], p0);
        atomicAdd(&msum[3 * t + 1], p1);
        atomicAdd(&msum[3 * t + 2], p2);
      }
      if (tail && key >= 0) {
        atomicAdd(&fsum[3 * ts], p0 - b0);
        atomicAdd(&fsum[3 * ts + 1], p1 - b1);
        atomicAdd(&fsum[3 * ts + 2], p2 - b2);
        atomicAdd(&vsum[3 * (size_t)k], p0 - b0);
        atomicAdd(&vsum[3 * (size_t)k + 1], p1 - b1);
        atomicAdd(&vsum[3 * (size_t)k + 2], p2 - b2);
      }
    }
    if (tail && key >= 0) {
      const int n = lane - start + 1;
      atomicAdd(&cnt[ts], n);
      if (J) atomicAdd(&J[ts * G1 + g], n);
    }
  }
}

__device__ __forceinline__ double q_block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0;
  if (w == 0) {
    s = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  return s;   // valid in thread 0
}

// Pass 2, grid (x blocks, T): pix2[t] += sum_c (v - m)^2, pix2s[t] the same at x255
// scale, sse[t] += sum_c (v - pooled)^2.
__global__ void __launch_bounds__(256) k_q_resid(
    const float* __restrict__ vid, const int32_t* __restrict__ spix, int npix, int off, int S,
    const int* __restrict__ cnt, const double* __restrict__ fsum,
    const double* __restrict__ msum, double* pix2, double* pix2s, double* sse) {
  pdl_enter();
  __shared__ double sh[32];
  const int t = blockIdx.y;
  const double m0 = msum[3 * t] / npix, m1 = msum[3 * t + 1] / npix, m2 = msum[3 * t + 2] / npix;
  const double M0 = 255.0 * m0, M1 = 255.0 * m1, M2 = 255.0 * m2;
  double a = 0, as = 0, b = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x) {
    const size_t idx = (size_t)t * npix + i;
    const float* p = vid + 3 * idx;
    const double v0 = p[0], v1 = p[1], v2 = p[2];
    const size_t ts = (size_t)t * S + (spix[idx] - off);
    const double n = (double)cnt[ts] + 1e-8;
    const double u0 = fsum[3 * ts] / n, u1 = fsum[3 * ts + 1] / n, u2 = fsum[3 * ts + 2] / n;
    a += (v0 - m0) * (v0 - m0) + (v1 - m1) * (v1 - m1) + (v2 - m2) * (v2 - m2);
    const double s0 = 255.0 * v0 - M0, s1 = 255.0 * v1 - M1, s2 = 255.0 * v2 - M2;
    as += s0 * s0 + s1 * s1 + s2 * s2;
    b += (v0 - u0) * (v0 - u0) + (v1 - u1) * (v1 - u1) + (v2 - u2) * (v2 - u2);
  }
  a = q_block_sum(a, sh);
  if (threadIdx.x == 0) atomicAdd(&pix2[t], a);
  as = q_block_sum(as, sh);
  if (threadIdx.x == 0) atomicAdd(&pix2s[t], as);
  b = q_block_sum(b, sh);
  if (threadIdx.x == 0) atomicAdd(&sse[t], b);
}

// Per id over time: frames alive, total size, and the unbiased standard deviation
// of its size over the frames it is alive in (-1 if alive in fewer than two).
__global__ void k_q_id_time(const int* __restrict__ cnt, int T, int S, long long* ntot,
                            double* std_out) {
  pdl_enter();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  long long n = 0, s1 = 0;
  __int128 s2 = 0;
  for (int t = 0; t < T; t++) {
    const long long c = cnt[(size_t)t * S + s];
    if (c > 0) { n++; s1 += c; s2 += (__int128)(c * c); }
  }
  ntot[s] = s1;
  if (n > 1) {
    const __int128 num = (__int128)n * s2 - (__int128)s1 * s1;
    std_out[s] = sqrt((double)num / ((double)n * (double)(n - 1)));
  } else {
    std_out[s] = -1.0;
  }
}

// Grid (x blocks over ids, T): live ids per frame, and the pooled-vs-frame-mean sums
// of the per-frame pooling (x1) and of the video pooling (x255); live ids only when
// fsum is null.
__global__ void __launch_bounds__(256) k_q_frame_ids(
    const int* __restrict__ cnt, const double* __restrict__ fsum,
    const double* __restrict__ vsum, const long long* __restrict__ ntot,
    const double* __restrict__ msum, int S, int npix, unsigned long long* live, double* pool2,
    double* pool3) {
  pdl_enter();
  __shared__ double sh[32];
  const int t = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  double a = 0, b = 0;
  int alive = 0;
  if (s < S) {
    const size_t ts = (size_t)t * S + s;
    const int c = cnt[ts];
    if (c > 0 && !fsum) {
      alive = 1;
    } else if (c > 0) {
      alive = 1;
      const double m0 = msum[3 * t] / npix, m1 = msum[3 * t + 1] / npix,
                   m2 = msum[3 * t + 2] / npix;
      const double n = (double)c + 1e-8;
      const double d0 = fsum[3 * ts] / n - m0, d1 = fsum[3 * ts + 1] / n - m1,
                   d2 = fsum[3 * ts + 2] / n - m2;
      a = c * (d0 * d0 + d1 * d1 + d2 * d2);
      const double N = (double)ntot[s] + 1e-10;
      const double e0 = 255.0 * vsum[3 * (size_t)s] / N - 255.0 * m0;
      const double e1 = 255.0 * vsum[3 * (size_t)s + 1] / N - 255.0 * m1;
      const double e2 = 255.0 * vsum[3 * (size_t)s + 2] / N - 255.0 * m2;
      b = c * (e0 * e0 + e1 * e1 + e2 * e2);
    }
  }
  const unsigned nl = __popc(__ballot_sync(0xffffffffu, alive));
  if ((threadIdx.x & 31) == 0 && nl) atomicAdd(&live[t], (unsigned long long)nl);
  if (!fsum) return;
  a = q_block_sum(a, sh);
  if (threadIdx.x == 0) atomicAdd(&pool2[t], a);
  b = q_block_sum(b, sh);
  if (threadIdx.x == 0) atomicAdd(&pool3[t], b);
}

// Grid (x blocks over ids, T): per ground-truth id g of frame t, the corrected
// under-segmentation sum (min(out, in) over ids overlapping g), the accuracy sum (in
// over ids at least half inside g) and g's size (evaluate.py:436-461).  Block sums in
// shared memory when G1 <= kQGtShared.
__global__ void __launch_bounds__(256) k_q_uesa_frame(
    const int* __restrict__ cnt, const int* __restrict__ J, int S, int G1,
    unsigned long long* ue, unsigned long long* sa, unsigned long long* size) {
  pdl_enter();
  __shared__ unsigned long long sue[kQGtShared], ssa[kQGtShared], ssz[kQGtShared];
  const bool shared = G1 <= kQGtShared;
  if (shared)
    for (int g = threadIdx.x; g < G1; g += blockDim.x) sue[g] = ssa[g] = ssz[g] = 0;
  __syncthreads();
  const int t = blockIdx.y;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < S) {
    const size_t ts = (size_t)t * S + s;
    const long long n = cnt[ts];
    if (n > 0) {
      const int* j = J + ts * G1;
      for (int g = 0; g < G1; g++) {
        const long long in = j[g];
        if (in <= 0) continue;
        const unsigned long long u = (unsigned long long)min(n - in, in);
        const unsigned long long a = 2 * in >= n ? (unsigned long long)in : 0ull;
        if (shared) {
          if (u) atomicAdd(&sue[g], u);
          if (a) atomicAdd(&ssa[g], a);
          atomicAdd(&ssz[g], (unsigned long long)in);
        } else {
          const size_t tg = (size_t)t * G1 + g;
          if (u) atomicAdd(&ue[tg], u);
          if (a) atomicAdd(&sa[tg], a);
          atomicAdd(&size[tg], (unsigned long long)in);
        }
      }
    }
  }
  if (!shared) return;
  __syncthreads();
  for (int g = threadIdx.x; g < G1; g += blockDim.x) {
    const size_t tg = (size_t)t * G1 + g;
    if (sue[g]) atomicAdd(&ue[tg], sue[g]);
    if (ssa[g]) atomicAdd(&sa[tg], ssa[g]);
    if (ssz[g]) atomicAdd(&size[tg], ssz[g]);
  }
}

// One thread per id: the video-level (3D) sums (evaluate.py:449-468): in and out
// summed over frames (out only where the id overlaps g in that frame).
__global__ void __launch_bounds__(256) k_q_uesa_id(
    const int* __restrict__ cnt, const int* __restrict__ J, const long long* __restrict__ ntot,
    int T, int S, int G1, unsigned long long* ue3, unsigned long long* sa3) {
  pdl_enter();
  __shared__ unsigned long long sue[kQGtShared], ssa[kQGtShared];
  const bool shared = G1 <= kQGtShared;
  if (shared)
    for (int g = threadIdx.x; g < G1; g += blockDim.x) sue[g] = ssa[g] = 0;
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < S && ntot[s] > 0) {
    for (int g = 0; g < G1; g++) {
      long long in = 0, out = 0;
      for (int t = 0; t < T; t++) {
        const size_t ts = (size_t)t * S + s;
        const long long j = J[ts * G1 + g];
        if (j > 0) { in += j; out += cnt[ts] - j; }
      }
      if (in <= 0) continue;
      const unsigned long long u = (unsigned long long)min(out, in);
      const unsigned long long a = 2 * in >= ntot[s] ? (unsigned long long)in : 0ull;
      if (shared) {
        if (u) atomicAdd(&sue[g], u);
        if (a) atomicAdd(&ssa[g], a);
      } else {
        if (u) atomicAdd(&ue3[g], u);
        if (a) atomicAdd(&sa3[g], a);
      }
    }
  }
  if (!shared) return;
  __syncthreads();
  for (int g = threadIdx.x; g < G1; g += blockDim.x) {
    if (sue[g]) atomicAdd(&ue3[g], sue[g]);
    if (ssa[g]) atomicAdd(&sa3[g], ssa[g]);
  }
}

// sp_pooling (st_spix/sp_pooling.py:10-47) outputs: down[t][s] = colour sum / (count
// + 1e-8) for every id 0..S-1 of every frame, pooled[p] = down of the pixel's id.
__global__ void k_q_down(const int* __restrict__ cnt, const double* __restrict__ fsum,
                         long long TS, float* __restrict__ down) {
  pdl_enter();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= TS) return;
  const double n = (double)cnt[i] + 1e-8;
  for (int c = 0; c < 3; c++) down[3 * i + c] = (float)(fsum[3 * i + c] / n);
}

__global__ void k_q_pool_write(const int32_t* __restrict__ spix, int npix, int off, int S,
                               long long n, const float* __restrict__ down,
                               float* __restrict__ pooled) {
  pdl_enter();
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const long long t = i / npix;
  const size_t ts = (size_t)t * S + (spix[i] - off);
  for (int c = 0; c < 3; c++) pooled[3 * i + c] = down[3 * ts + c];
}

}  // namespace stspix
