// Internal header of the GB300 streaming-BASS engine (device layout, kernels,
// host workspace).  Public C ABI: include/st_spix_gb300.h.
//
// Deterministic rules shared with the CPU oracle (oracle/bass_oracle.cpp):
//   R1 int64 fixed-point colour sums (2^-28; squares 2^-20; flow 2^-24), exact
//      integer position sums.
//   R2 split ids in ascending order of the split superpixel (exclusive scan).
//   R3 merge claims: smallest claimant id wins (atomicMin).
//   R4 forward-warp collisions: smallest packed (size, id) wins (64-bit atomicMin).
//   R5 relabel: smallest packed (distance bits, candidate) wins; minted ids by scan;
//      a revived id copies its count from the largest reviving superpixel.
//   R6 connected components: per label keep the largest region, ties to the
//      smallest root pixel index.
//   R7 reference reads of uninitialised memory are zero.
//   R8 IEEE FP32/FP64 with no FMA contraction (-fmad=false); Hastings in FP64.
#pragma once
#include "pdl.h"
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/st_spix_gb300.h"

namespace stspix {

constexpr int kFxAppShift = 28;
constexpr int kFxSqShift = 20;
constexpr int kFxFlowShift = 24;
constexpr int kFillBreakIter = 1000;      // fill_missing.cu: break_iter
constexpr int kSweepVariants = 3;         // sweep tile shapes: 32x32, 64x32, 16x32
constexpr int kTuneRounds = 3;            // timed runs per autotuner trial (fastest kept)
constexpr int kMaxBatchGraphs = 64;       // captured batch steps kept per context
constexpr float kWideMargin = 1.05f;      // large batches: 64x32 unless 5 % slower
constexpr int kPairMaxTiles = 2048;       // two-sweep launches only below this many 32x32 tiles
constexpr int kSweepTileW[kSweepVariants] = {32, 64, 16};
constexpr int kRelabelChunk = 64;         // previous superpixels per relabel-compare block

// Packed record read by the boundary sweep: the fields calc_joint reads
// (update_seg.cu:194-259), already converted to the types it uses.  The reference
// truncates d0 = (int)(x - mu_x) in double; since x - mu_x is exact in double for
// |x - mu_x| < 2^13, trunc(x - mu_x) = k - (k >= 1 && frac) with k = x - floor(mu_x),
// so the record carries floor(mu) and a has-fraction flag and the sweep needs no FP64.
struct __align__(16) SweepRec {
  float mu_r, mu_g, mu_b, logdet;  // mean colour, (float) log det Sigma
  int mxi, myi;                    // floor(mu_x), floor(mu_y)
  int frac;                        // bit0: mu_x not integral, bit1: mu_y not integral
  int count;                       // pixel count
  float isx, isy, isz, pad;        // (float) inverse shape covariance
};
static_assert(sizeof(SweepRec) == 48, "three 16-byte words");

// Per-superpixel kernels with FP64 work: live ids are the low ones, and this part issues
// FP64 slowly, at a cost per warp instruction whatever its active lanes.  So a warp takes
// 32 consecutive ids (full lanes) and consecutive groups of 32 go to different blocks
// (different SMs): thread j of block b takes id 32 (b + grid (j / 32)) + j % 32.  The id
// grows with j, so the loop ends at the first id >= n.
__device__ __forceinline__ int spread_id(int j) {
  return (blockIdx.x + gridDim.x * (j >> 5)) * 32 + (j & 31);
}
#define FOR_SP(k, n)                                                              \
  for (int j_ = threadIdx.x, k = spread_id(j_); k < (n); j_ += blockDim.x, k = spread_id(j_))

// Per-superpixel working state, structure of arrays, `cap` entries each.
struct SpDev {
  int cap;
  int* count;
  uint8_t* valid;
  uint8_t* prop;
  float* prior_count;
  float* icount;
  int* sm_count;
  float* mu_app;           // [3*cap]
  double* mu_shape;        // [2*cap]
  double* sigma_shape;     // [3*cap]
  double* logdet;          // [cap]
  float* prior_mu_app;     // [3*cap]
  double* prior_mu_shape;  // [2*cap]
  double* prior_sigma_shape;   // [3*cap]
  double* prior_icov;          // [3*cap]
  double* sample_sigma_shape;  // [3*cap]
  long long* acc;          // [8*cap]: r,g,b (2^-28), x, y, xx, xy, yy
  SweepRec* rec;           // [cap]
};

// Split / merge scratch, cap+2 entries.
struct SmDev {
  int* count;
  long long* s;      // [3*(cap+2)]
  long long* sq;     // [3*(cap+2)]
  int* ninvalid;
  int* pair;         // merge candidate (sm_pairs[2k+1])
  int* claim;        // merge claim (sm_pairs[2f])
  int* target;
  int* newid;
  uint8_t* flag;     // bit0 accept/want, bit1 merge, bit2 remove, bit3 select, bit4 has_single
  double* msingle;
};

// Split/merge constants computed once on the host (split_merge_orig.cu:97-106):
// b_0 = 2 sqrt(sigma2_app) a_0 (a_0 = 1e4), log alpha, log(0.1) - log b_0 and
// lc = 0.5 log(pi) + log 2.
struct SmConsts {
  double b0, log_alpha, log_01_b0, lc;
};

// Frame-level device scalars.
struct Scalars {
  int max_spix;
  int nspix;          // live superpixels after compaction / init
  int nbuf_logical;   // reference's nspix_buffer (30 x hex count, or 10 x n_prev)
  int status;
  int nsplits, nmerges, nrevived, nminted, near_ties;
  int fill_iters;
  int ninvalid;       // -1 pixels after the shift
  int tmp0, tmp1, tmp2;
  int nhole;          // length of the hole list of the fill
  // hole-fill loop state: holes left, previous count, iterations run, finished flag,
  // holes filled in the running iteration; the hole list split by parity class
  // (class counts, write cursors)
  int fl_n, fl_prev, fl_iter, fl_done, fl_fill;
  int fl_cnt[4], fl_pos[4];
  // posterior work list: ids listed, blocks of the posterior launch done
  int npost, post_done;
};

// One frame of a batch: its inputs, outputs, workspace and scalars.  Kernels take
// the device array of slots and pick theirs from the launch's slot dimension, so one
// launch processes every frame of the batch (frames of uneven size: blocks past a
// frame's extent return).
struct Slot {
  // frame
  const float* img;        // [npix*3] the colours the path reads
  const float* img_src;    // [npix*3] the caller's frame when it is converted to CIELAB
                           // into img at ingest (stspix_config.lab_ingest), else null
  double inv_w, inv_h;     // 1 / W, 1 / H (the hole fill's quotients, see fill_quot)
  int* seg;                // working labels (the caller's output)
  int* seg_alt;            // ping-pong labels for the sweeps
  int H, W, npix;
  int cap;                 // superpixel capacity of this slot's buffers
  int mode;                // 0 plain BASS, 1 propagated frame
  int sp_size;             // superpixel size (hex grid, shape prior)
  int lo;                  // compaction keeps ids < lo (0, or n_prev on propagated frames)
  // hex geometry (BASS frames)
  double hex_h, hex_w;
  int hex_nx, hex_ny, nraw;
  // propagation inputs
  const int* prev_labels;  // previous frame's labels
  const float* flow;       // [npix*2]
  int n_prev;              // superpixels of the previous frame
  stspix_params pprev;     // previous frame's params (updated in place by the shift)
  stspix_params pout;      // this frame's params (capacity 0: not wanted)
  int* resident_labels;    // where the finished labels are kept for the next frame
  // pixel workspace
  uint8_t* border;
  uint8_t* chg[2];         // change flags of the last two sweeps (active-set sweeps)
  int *d1, *d2, *smseg, *hits, *shifted;
  unsigned long long* best;
  // superpixel workspace
  SpDev sp, tmp;
  SmDev sm;
  uint8_t *flags, *accept, *valid0, *living, *mint;
  int *excl, *rid, *src_of, *cnt_pool, *cs, *cf;
  long long* fs;
  float *fds, *ss;
  double* centers;
  unsigned long long *rbest, *ccbest;
  int* bbox;               // [4*(cap+2)]: x0, x1, y0, y1 per superpixel (split BFS)
  long long* snap;         // [9*(cap+2)]: count and the 8 sums each id's posterior last saw
  uint8_t* recchg;         // [cap+2]: the last posterior changed the id's SweepRec
  double* pscache;         // [3*(cap+2)]: the prior shape term of the last full posterior
  int* post_ids;           // [cap+2]: ids of the running posterior (kb_post_list)
  Scalars* sc;
  int tile_base[3];        // first sweep tile of this slot in the batch (32-, 64-, 16-wide)
};

// kb_scalars operations.
enum { kOpBegin = 0, kOpAfterHex = 1, kOpCompactN = 2, kOpCompactEnd = 3 };

#define SLOT_Y const Slot& S = slots[blockIdx.y]
// Light per-pixel kernels: thread i of block b takes the pixels
// kPixPerThread * blockDim.x * b + i + blockDim.x * j (j < kPixPerThread), coalesced, so
// a launch has a quarter of the blocks of one pixel per thread (block scheduling and the
// per-block set-up dominate passes this light).  Grids: pix_units(n) threads.
constexpr int kPixPerThread = 4;
#define FOR_PIX(t, n)                                                                    \
  for (int j_ = 0, t = (int)blockIdx.x * (kPixPerThread * (int)blockDim.x) + (int)threadIdx.x; \
       j_ < kPixPerThread && t < (n); j_++, t += (int)blockDim.x)
// Block-uniform form, for bodies with warp or block collectives: every thread of a block
// runs the same iterations (t - threadIdx.x is the block's first pixel of the iteration),
// so t may be >= n in the last one.
#define FOR_PIX_ALL(t, n)                                                                \
  for (int j_ = 0, t = (int)blockIdx.x * (kPixPerThread * (int)blockDim.x) + (int)threadIdx.x; \
       j_ < kPixPerThread && t - (int)threadIdx.x < (n); j_++, t += (int)blockDim.x)
#define SLOT_Z const Slot& S = slots[blockIdx.z]

// ---------------------------------------------------------------------------
// Device helpers shared by the kernels.
// round(v * 2^shift) (round half to even, as llrintf(ldexpf(v, shift))) for
// |v * 2^shift| < 2^41, without a float -> 64-bit integer conversion (those run on the
// FP64 pipe, which GB300 has little of).  t = v * 2^shift is exact (a power of two);
// h = trunc(t / 2^18) is an exact integer-valued float; l = t - h * 2^18 holds the bits
// of t below 2^18 (same sign, |l| < 2^18) and is exact; h * 2^18 is an even integer, so
// round(t) = h * 2^18 + round(l), ties included.
// Values in [0, 1] (colours, their squares) take one conversion: t <= 2^shift < 2^32.
__device__ __forceinline__ long long fx_q(float v, int shift) {
  const float t = v * (float)(1u << shift);
  if (v >= 0.f && v <= 1.f) return (long long)__float2uint_rn(t);
  const float h = truncf(t * 0x1p-18f);
  const float l = t - h * 0x1p18f;
  return (long long)__float2int_rz(h) * 262144LL + (long long)__float2int_rn(l);
}
__device__ __forceinline__ double fx_unq(long long q, int shift) {
  return ldexp((double)q, -shift);
}
// Full-warp sum of a 64-bit integer by 32-bit reductions: v = hi * 2^24 + lo with lo in
// [0, 2^24), so the lo parts of 32 lanes stay below 2^29; |v| < 2^54 per lane.
__device__ __forceinline__ long long warp_sum64(long long v) {
  const unsigned lo = (unsigned)(v & 0xFFFFFF);
  const int hi = (int)(v >> 24);
  return (long long)__reduce_add_sync(0xffffffffu, hi) * (1LL << 24) +
         (long long)__reduce_add_sync(0xffffffffu, lo);
}

// Full-warp sum of 32-bit unsigned values (any value per lane): hi = v >> 24 < 2^8 and
// lo < 2^24 summed separately.
__device__ __forceinline__ long long warp_sum_u32(unsigned v) {
  return (long long)__reduce_add_sync(0xffffffffu, v >> 24) * (1LL << 24) +
         (long long)__reduce_add_sync(0xffffffffu, v & 0xFFFFFFu);
}
// Colours in [0, 1] (the usual RGB input): their 2^28 fixed point is one conversion and
// fits 32 bits, and so does a lane's sum of 8 (< 2^31); squares at 2^20 likewise, and a
// warp's sum of 256 of those (< 2^29) fits one 32-bit reduction.
__device__ __forceinline__ bool unit_colour(float v) { return v >= 0.f && v <= 1.f; }
__device__ __forceinline__ unsigned fx_unit(float v, int shift) {
  return __float2uint_rn(v * (float)(1u << shift));     // fx_q(v, shift) for v in [0, 1]
}

// Warp-block label sums.  A warp owns a 32 x 8 block of a frame, lane l its column l,
// lab[i] the label of row i.  The warp takes the block's labels one at a time (the label
// of the lowest lane with rows pending) and calls body(k, m, src) on every lane: m = the
// lane's rows of label k, src = the lane that adds the warp's totals to the global sums.
// pend = the rows to take (labels in range).  A block holds a few labels, so a few warp
// reductions and one set of atomics per label serve its 256 pixels.
template <typename Body>
__device__ __forceinline__ void label_rounds(const int (&lab)[8], unsigned pend, Body body) {
  for (;;) {
    const unsigned any = __ballot_sync(0xffffffffu, pend != 0);
    if (!any) break;
    const int src = __ffs(any) - 1;
    int first = -1;
#pragma unroll
    for (int i = 7; i >= 0; i--)
      if ((pend >> i) & 1u) first = lab[i];
    const int k = __shfl_sync(0xffffffffu, first, src);
    unsigned m = 0;
#pragma unroll
    for (int i = 0; i < 8; i++) m |= (unsigned)(lab[i] == k) << i;
    pend &= ~m;
    body(k, m, src);
  }
}

// The 32 x 8 block of warp w of a block of the 64 x 32 tile grid of a W-wide frame:
// its lane's column gx and first row by.  False for blocks past the frame's tiles.
__device__ __forceinline__ bool warp_block(int W, int H, int& gx, int& by) {
  const int tiles_x = (W + 63) / 64;
  if ((int)blockIdx.x >= tiles_x * ((H + 31) / 32)) return false;
  const int warp = threadIdx.x >> 5;
  gx = (blockIdx.x % tiles_x) * 64 + (warp & 1) * 32 + (threadIdx.x & 31);
  by = (blockIdx.x / tiles_x) * 32 + (warp >> 1) * 8;
  return true;
}

}  // namespace stspix
