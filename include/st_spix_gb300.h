/*
 * st_spix_gb300 — C ABI of the GB300 streaming-BASS ("BIST") superpixel engine.
 *
 * Every entry point takes caller-owned DEVICE pointers (unless a parameter says
 * "host"), plain sizes and an explicit cudaStream_t (passed as void*), returns an
 * int status (STSPIX_OK == 0) and never exits the process.  Work is enqueued on
 * the given stream; entry points that must return a host-side value (a count)
 * synchronise that stream and say so.  A context is NOT safe for concurrent use
 * from several host threads; use one context per thread / per stream.
 *
 * Reference interfaces replaced (paths inside gauenk/st_spix):
 *   stspix_bist_forward        st_spix/csrc/bist/pyapi.cu:200 bist_forward_cuda (+ :46 main_loop)
 *   stspix_get_marked_video    st_spix/csrc/bist/pyapi.cu:260 get_marked_video
 *   stspix_run_bass            st_spix/csrc/bist/bass.cu:221  run_bass
 *   stspix_shift_and_fill      st_spix/csrc/bist/shift_and_fill.cu:108 shift_and_fill
 *   stspix_run_prop            st_spix/csrc/bist/prop.cu:677  run_prop
 *   stspix_find_border         st_spix/csrc/bist/seg_utils.cu:156,211 CudaFindBorderPixels(_end)
 *   stspix_init_seg            st_spix/csrc/bist/init_seg.cu:20 init_seg
 *   stspix_rgb2lab/_lab2rgb    st_spix/csrc/bist/rgb2lab.cu:39,46 rgb2lab / lab2rgb
 *   stspix_rescale_u8          st_spix/csrc/bist/rgb2lab.cu:21 rescale_image
 *   stspix_bass_partial        st_spix/csrc/bist/bass.cu:46 bass() stopped after k iterations
 *                              (exposes update_params.cu:12 and update_seg.cu:281 state)
 *   stspix_evaluate            st_spix/spix_utils/evaluate.py:94 computeSummary
 *   stspix_count_spix          st_spix/spix_utils/evaluate.py:71 count_spix
 *   stspix_size_variation      st_spix/spix_utils/evaluate.py:284 scoreMeanDurationAndSizeVariation
 *   stspix_sp_pooling          st_spix/sp_pooling.py:10 pooling
 *   stspix_legacy_shift_labels st_spix/csrc/prop/shift_labels.cu:82 run_shift_labels
 *   stspix_legacy_fill_missing st_spix/csrc/prop/fill_missing.cu:317 run_fill_missing
 *   stspix_legacy_split        st_spix/csrc/prop/bass.cu:389 run_split_py
 *   stspix_legacy_rgb_to_lab   st_spix/csrc/prop/rgb2lab.cu:167 run_rgb_to_lab
 *   stspix_sp_video_pooling    st_spix/csrc/prop/sp_video_pooling.cu:62 sp_video_pooling
 *   stspix_downsampled_video_to_pooled  st_spix/csrc/prop/sp_video_pooling.cu:211
 *   stspix_legacy_update_prior st_spix/csrc/prop/sparams_io.cu:795 run_update_prior
 *   stspix_legacy_shift_tensor st_spix/csrc/prop/shift_tensor.cu:60 run_shift_tensor
 *                              (+ shift_tensor_ordered.cu:53 run_shift_tensor_ordered)
 *   stspix_legacy_shift_order  st_spix/csrc/prop/shift_order.cu:43 run_shift_order
 *   stspix_legacy_split_disconnected  st_spix/csrc/prop/split_disconnected.cu:390
 */
#ifndef ST_SPIX_GB300_H
#define ST_SPIX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define STSPIX_OK                 0
#define STSPIX_ERR_ARG            1   /* bad argument (null pointer, size out of range)        */
#define STSPIX_ERR_CUDA           2   /* a CUDA runtime call failed (see stspix_last_error)    */
#define STSPIX_ERR_NOMEM          3   /* device allocation failed                               */
#define STSPIX_ERR_NOPROGRESS     4   /* hole filling stopped shrinking (reference exits here)  */
#define STSPIX_ERR_ITER_LIMIT     5   /* a bounded device loop hit its iteration cap            */
#define STSPIX_ERR_CAPACITY       6   /* superpixel ids exceeded the parameter buffer           */
#define STSPIX_ERR_BARRIER        7   /* a grid barrier timed out (kernel returned early)       */
#define STSPIX_ERR_DEGENERATE     8   /* non-positive prior covariance determinant              */
#define STSPIX_ERR_TOO_LARGE      9   /* input larger than a fixed-size scratch array           */

/* ---- configuration ------------------------------------------------------
 * Defaults (stspix_default_config) are the reference's values:
 *   niters_seg=4, sm_start=0, sigma2_size=0, merge_alpha=0 (pyapi.cu:63-73),
 *   thresh_relabel=1e-5, thresh_new=1e-2 (pyapi.cu:72-73), split/merge period 4
 *   (bass.cu:117-135), sp_size=15, sigma2_app=0.009^2, potts=0.5,
 *   alpha_hastings=log(0.5), split_alpha=0 (demo.cu:45-57,141).            */
typedef struct stspix_config {
  int   niters;          /* outer BASS iterations (image mode / first frame)          */
  int   niters_seg;      /* boundary sweeps per outer iteration                       */
  int   sp_size;         /* hexagon side: sqrt of the initial superpixel area         */
  int   sm_start;        /* split/merge only when iteration index > sm_start          */
  int   sm_period;       /* split when idx%P==0, merge when idx%P==P/2                */
  int   prop_niters;     /* >0: fixed iterations on propagated frames; 0: the
                            reference's 4/8/12 ladder on the hole fraction            */
  float sigma2_app;      /* appearance variance                                       */
  float potts;           /* Potts weight per differing 8-neighbour                    */
  float alpha_hastings;  /* log alpha of the merge Hastings ratio                     */
  float split_alpha;     /* additive split bias                                       */
  float merge_alpha;     /* additive merge bias                                       */
  float sigma2_size;     /* kept for API parity (unused by the reference path)        */
  float thresh_relabel;  /* revive a dead id when appearance distance < this          */
  float thresh_new;      /* mint a new id when self distance > this                   */
  int   accumulator;     /* colour sums of the statistics: 0 int64 fixed point
                            (default, exact and order-independent), 1 FP32 atomics (as
                            the reference; order-dependent), 2 FP64 atomics -- 1 and 2
                            exist for the accumulator precision study               */
  int   sweep_schedule;  /* boundary sweeps per launch: 0 autotuned (default), 1 one,
                            2 two whenever two remain; the labels are the same       */
  int   sweep_tile;      /* tile width: 0 autotuned (default), or 16, 32, 64 (no
                            timing; schedules 0 and 1 then run single sweeps of that
                            width, schedule 2 two-sweep launches of that width)      */
  int   sweep_queue;     /* single-sweep launches: 0 one block per tile (default), 1 a
                            persistent work-queue kernel (one resident block set that
                            takes tiles from an atomic counter); same labels         */
  int   lab_ingest;      /* 0 frames used as given (default; the reference's
                            bist_forward ignores its rgb2lab flag), 1 every frame is
                            converted sRGB -> CIELAB (the reference's rgb2lab steps,
                            first channel blue) once at ingest into an engine buffer,
                            which the statistics and sweeps then read              */
} stspix_config;

void stspix_default_config(stspix_config* cfg);

/* ---- superpixel parameters ----------------------------------------------
 * Structure-of-arrays mirror of the reference's SuperpixelParams
 * (st_spix/csrc/bist/structs.h:13-48).  `capacity` entries are allocated by the
 * caller; entry i describes superpixel id i.  sigma_shape holds the INVERSE shape
 * covariance (xx, xy, yy) as the reference stores it.                          */
typedef struct stspix_params {
  float*  mu_app;             /* [cap*3] */
  float*  prior_mu_app;       /* [cap*3] */
  double* mu_shape;           /* [cap*2] */
  double* sigma_shape;        /* [cap*3] */
  float*  logdet_sigma_shape; /* [cap]   */
  double* prior_mu_shape;     /* [cap*2] */
  double* prior_sigma_shape;  /* [cap*3] */
  double* sample_sigma_shape; /* [cap*3] */
  int*    counts;             /* [cap]   */
  int*    sm_counts;          /* [cap]   */
  float*  prior_counts;       /* [cap]   */
  int*    ids;                /* [cap]   */
  float*  invalid_counts;     /* [cap]   */
  int     capacity;
} stspix_params;

/* Per-frame decision log (near-threshold ties are what label disagreements
 * with the reference's racy FP32 path trace back to).                          */
typedef struct stspix_frame_log {
  int nsplits;        /* accepted splits                                   */
  int nmerges;        /* accepted merges (superpixels removed)              */
  int nrevived;       /* relabel: dead ids revived                          */
  int nminted;        /* relabel: new ids minted                            */
  int near_ties;      /* Hastings decisions with |ratio + 2| < 1e-6        */
  int fill_iters;     /* hole-fill iterations (both fills)                  */
  int niters;         /* outer iterations run                               */
  int nspix;          /* superpixels after compaction                       */
} stspix_frame_log;

/* ---- context ------------------------------------------------------------ */
typedef struct stspix_ctx stspix_ctx;

int         stspix_create(stspix_ctx** ctx, int device);
int         stspix_destroy(stspix_ctx* ctx);
const char* stspix_last_error(const stspix_ctx* ctx);
int         stspix_version(void);
/* Number of kernels this context has launched since creation. */
long long   stspix_kernel_launches(const stspix_ctx* ctx);
/* Number of batch steps this context ran as replays of a captured CUDA graph (a batch
 * step whose frame sizes, capacities, iteration counts and configuration repeat is
 * captured on its second occurrence and replayed from then on).                    */
long long   stspix_graph_replays(const stspix_ctx* ctx);
/* The sweep autotuner's choices, entry idx (0..): *tiles_class = the batch's 32x32 tile
 * count class (4 log2 tiles), *single_w = the single-sweep tile width, *pair_w = the
 * two-sweep width (0: single sweeps only).  Returns 1 while idx is an entry, else 0.  */
int         stspix_sweep_choice(const stspix_ctx* ctx, int idx, int* tiles_class, int* single_w,
                                int* pair_w);
/* Enable (default) or disable the capture and replay of repeated batch steps; with
 * them off every step launches its kernels one by one (same results).              */
int         stspix_set_batch_graphs(stspix_ctx* ctx, int enable);
/* Copy of the log of the last frame processed by this context (host). */
int         stspix_get_frame_log(const stspix_ctx* ctx, stspix_frame_log* out);

/* ---- measurement --------------------------------------------------------------
 * Kernel-family profiling with CUDA events recorded on the launching stream
 * around every launch of the family (off by default; enabling resets totals).
 * Per-frame GPU durations of the last stspix_bist_forward call are always kept. */
#define STSPIX_FAM_SWEEP     0   /* boundary sweep (border + 4 parity phases)      */
#define STSPIX_FAM_STATS     1   /* sufficient statistics (sum_by_label)           */
#define STSPIX_FAM_POSTERIOR 2   /* posterior / parameter kernels                  */
#define STSPIX_FAM_SPLIT     3   /* split proposal + BFS + Hastings                */
#define STSPIX_FAM_MERGE     4   /* merge proposal + Hastings (+ relabel)          */
#define STSPIX_FAM_PROP      5   /* flow pooling, shift, fill, components          */
#define STSPIX_FAM_OTHER     6   /* init, compaction, read-out                     */
#define STSPIX_NFAM          7
int stspix_profile_enable(stspix_ctx* ctx, int enable);
int stspix_profile_get(const stspix_ctx* ctx, int family, long long* launches,
                       double* total_ms);
/* Per-kernel totals of the profiled launches as text, one "name launches ms" line
 * per kernel; returns the bytes needed (including the terminating zero).       */
int stspix_profile_kernels(const stspix_ctx* ctx, char* buf, int capacity);
/* Per-frame durations (ms) of the last bist_forward call; returns the count. */
int stspix_frame_times(const stspix_ctx* ctx, double* ms_out, int capacity);

/* ---- drop-in surface ------------------------------------------------------ */

/* bist_forward: vid f32 [T,H,W,3] contiguous; flows f32 [>=T-1,H,W,2]
 * interleaved (dx,dy), read at index fidx-1 for frame fidx (may be NULL when
 * video_mode==0); spix_out i32 [T,H,W].  rgb2lab is accepted and ignored, as in
 * the reference (pyapi.cu:95-102).  Stream state stays on the device.          */
int stspix_bist_forward(stspix_ctx* ctx, void* stream,
                        const float* vid, const float* flows,
                        int T, int H, int W, int nftrs,
                        const stspix_config* cfg, int video_mode, int rgb2lab,
                        int32_t* spix_out);

/* get_marked_video: border (find_border_pixels_end) painted with `color`
 * (3 floats, device), elsewhere the frame clipped to [0,1].  Frames have 3
 * channels (nftrs != 3 returns STSPIX_ERR_ARG).                                  */
int stspix_get_marked_video(stspix_ctx* ctx, void* stream,
                            const float* vid, const int32_t* spix,
                            const float* color, int T, int H, int W, int nftrs,
                            float* marked_out);

/* get_marked_video without any allocation.  No counterpart in the reference: it is
 * for callers that must not allocate device memory while they run (a process that
 * reserves its GPU memory up front, a plugin whose host owns every allocation, a
 * real-time loop).  The border-mask scratch lives in a 16 MiB array compiled into
 * the library (held on every GPU that loads it until exit); T*H*W above 2^24 pixels
 * returns STSPIX_ERR_TOO_LARGE.  Frames have 3 channels (else STSPIX_ERR_ARG).  No
 * context is needed; it runs on `stream`, which must belong to the current device
 * (else STSPIX_ERR_ARG).  All calls share that one array, so calls that overlap on
 * the GPU race and must be serialised by the caller.  The first call on a device
 * looks up the array's address and caches it for the process; make it before any
 * stream capture, and do not use the entry point across a cudaDeviceReset.       */
int stspix_get_marked_video_noalloc(void* stream, const float* vid, const int32_t* spix,
                                    const float* color, int T, int H, int W, int nftrs,
                                    float* marked_out);

/* ---- reference C++ entry points --------------------------------------------- */

/* run_bass on one frame.  labels_out i32 [H*W]; params_out capacity must be >=
 * the number of superpixels produced (<= 30 x initial hex count); *nspix_out
 * (host) receives that number.  Synchronises the stream.                        */
int stspix_run_bass(stspix_ctx* ctx, void* stream, const float* img, int H, int W,
                    const stspix_config* cfg, int32_t* labels_out,
                    stspix_params* params_out, int* nspix_out);

/* shift_and_fill: prev labels + prev params (n_prev entries) + flow [H,W,2]
 * -> filled and shifted labels; updates prev params' prior_counts and
 * invalid_counts in place.                                                    */
int stspix_shift_and_fill(stspix_ctx* ctx, void* stream, const int32_t* labels_prev,
                          stspix_params* params_prev, int n_prev, const float* flow,
                          int H, int W, int32_t* filled_out, int32_t* shifted_out);

/* run_prop: propagated BASS on one frame given filled/shifted labels and the
 * previous frame's params (n_prev entries).  niters as given (the ladder is
 * applied by bist_forward).  Synchronises the stream.                          */
int stspix_run_prop(stspix_ctx* ctx, void* stream, const float* img, int H, int W,
                    const stspix_config* cfg, int niters,
                    const int32_t* filled, const int32_t* shifted,
                    const stspix_params* params_prev, int n_prev,
                    int32_t* labels_out, stspix_params* params_out, int* nspix_out);

/* ---- stage-level entry points (used by the parity tests) ------------------ */

/* Hex-grid initialisation; returns the raw hex centre count in *nspix_out (host).
 * Labels are NOT compacted (as the reference's init_seg).                     */
int stspix_init_seg(stspix_ctx* ctx, void* stream, int32_t* labels, int H, int W,
                    int sp_size, int* nspix_out);

/* Border mask: mode 0 = find_border_pixels (image edge counts), mode 1 =
 * find_border_pixels_end (only the larger label marks).                       */
int stspix_find_border(stspix_ctx* ctx, void* stream, const int32_t* labels,
                       uint8_t* border_out, int H, int W, int mode);

/* Run a BASS frame (run_bass) but stop after `iters` outer iterations and dump
 * the working state; with extra_update != 0 the next iteration's update_params
 * (statistics + posterior, no split/merge, no sweep) also runs before the dump.  State arrays (device) have `nbuf` entries
 * (nbuf = 30 x compacted hex count, returned in *nbuf_out):
 *   count i32[nbuf], valid u8[nbuf], prior_count f32[nbuf],
 *   mu_app f32[nbuf*3], mu_shape f64[nbuf*2], sigma_shape f64[nbuf*3],
 *   logdet f64[nbuf], sums i64[nbuf*8] (sum r,g,b in 2^-28 units, sum x, y,
 *   xx, xy, yy).  Any state pointer may be NULL.  Synchronises.               */
typedef struct stspix_state_dump {
  int32_t* count; uint8_t* valid; float* prior_count; float* mu_app;
  double* mu_shape; double* sigma_shape; double* logdet; int64_t* sums;
  int capacity;
} stspix_state_dump;

int stspix_bass_partial(stspix_ctx* ctx, void* stream, const float* img, int H, int W,
                        const stspix_config* cfg, int iters, int extra_update,
                        int32_t* labels_out, stspix_state_dump* dump,
                        int* nbuf_out, int* max_spix_out);

/* ---- colour front end (rgb2lab.cu; not called by bist_forward) ----------------
 * rgb2lab: f32 [npix,3] (first channel read as blue, as the reference) -> CIELAB
 * stored as (L/-100, a/100, b/100) (rgb2lab.cu:51-122); lab2rgb: the inverse
 * (rgb2lab.cu:124-181); rescale_u8: u8 values -> f32 value/scale
 * (rgb2lab.cu:184 rescale_image_kernel).  Pixels with a NaN channel are left
 * unwritten, as in the reference.                                              */
int stspix_rgb2lab(stspix_ctx* ctx, void* stream, const float* rgb, float* lab, long long npix);
int stspix_lab2rgb(stspix_ctx* ctx, void* stream, const float* lab, float* rgb, long long npix);
int stspix_rescale_u8(stspix_ctx* ctx, void* stream, const uint8_t* in, float* out,
                      long long nvals, float scale);

/* Sufficient statistics of a labelling (precision study): per label id < nlabels,
 * out[7*k .. 7*k+6] = count, sum r, sum g, sum b, sum r^2, sum g^2, sum b^2 of the
 * pixels carrying k, accumulated as `accumulator` says (0 int64 fixed point: colours
 * 2^-28, squares 2^-20; 1 FP32 atomics; 2 FP64 atomics), returned as doubles.
 * Synchronises the stream.                                                     */
int stspix_label_stats(stspix_ctx* ctx, void* stream, const float* img, const int32_t* labels,
                       int H, int W, int nlabels, int accumulator, double* out);

/* ---- quality metrics -------------------------------------------------------------
 * The superpixel quality scores of st_spix/spix_utils/evaluate.py, on the device.
 * Labels are offset by their minimum first, as computeSummary does (evaluate.py:97).
 *   tex, szv   scoreMeanDurationAndSizeVariation (evaluate.py:284): fraction of ids
 *              alive per frame (mean over frames); mean over ids alive in more than
 *              one frame of the unbiased std of their size (NaN if none)
 *   ev         scoreExplainedVariance (evaluate.py:230): per-frame pooled colours
 *   ev3d       scoreExplainedVariance3D (evaluate.py:254): ids pooled over the video
 *   psnr       scoreSpixPoolingQuality (evaluate.py:214): 10 log10(1/mse) of the
 *              per-frame pooled video, data range 1, mean over frames
 *   ave_nsp    averge_unique_spix_v1 (evaluate.py:184); spnum = max - min + 1
 *   ue2d, sa2d, ue3d, sa3d   scoreUEandSA (evaluate.py:372), given a ground truth
 *              whose ids are 0..max, each present (else STSPIX_ERR_ARG); -1 without.
 * Integer tables are exact; colour sums are FP64.                                   */
typedef struct {
  double tex, szv, ev, ev3d, psnr, ave_nsp;
  double ue2d, sa2d, ue3d, sa3d;
  int spnum;
  int has_gt;
} stspix_quality;

/* vid f32 [T,H,W,3], spix i32 [T,H,W], gt i32 [T,H,W] or NULL (device pointers).
 * Synchronises the stream.                                                          */
int stspix_evaluate(stspix_ctx* ctx, void* stream, const float* vid, const int32_t* spix,
                    const int32_t* gt, int T, int H, int W, stspix_quality* out);

/* Minimum and maximum of n labels into out[0], out[1] (host). Synchronises.          */
int stspix_label_range(stspix_ctx* ctx, void* stream, const int32_t* labels, long long n,
                       int32_t* out);

/* count_spix (evaluate.py:71): counts[t*nids + k] = pixels of frame t carrying id
 * id_offset + k; every id must lie in [id_offset, id_offset + nids) (else
 * STSPIX_ERR_ARG).  counts is a device array of T*nids int32.                        */
int stspix_count_spix(stspix_ctx* ctx, void* stream, const int32_t* spix, int T, long long npix,
                      int32_t id_offset, int nids, int32_t* counts);

/* scoreMeanDurationAndSizeVariation (evaluate.py:284) on a device table of per-frame
 * id sizes, int32 [T, S]: *tex, *szv as in stspix_quality, and (when ave_nsp is not
 * NULL) averge_unique_spix_v1 (evaluate.py:184), the mean number of ids alive per
 * frame. Synchronises.                                                               */
int stspix_size_variation(stspix_ctx* ctx, void* stream, const int32_t* counts, int T, int S,
                          double* tex, double* szv, double* ave_nsp);

/* sp_pooling (st_spix/sp_pooling.py:10) for 3-channel frames: with ids 0..nids-1
 * (every id of spix must be in range, else STSPIX_ERR_ARG), down f32 [T, nids, 3] =
 * per-frame id mean colour (sum / (count + 1e-8); 0 for absent ids) and, when pooled
 * is not NULL, pooled f32 [T,H,W,3] = the mean colour of each pixel's id.            */
int stspix_sp_pooling(stspix_ctx* ctx, void* stream, const float* vid, const int32_t* spix,
                      int T, int H, int W, int nids, float* pooled, float* down);

/* ---- legacy prop_cuda surface ------------------------------------------------------
 * The ops of the older extension st_spix/csrc/prop (bound by pybind_prop.cpp, called by
 * st_spix/prop and st_spix/models/bass.py) whose arithmetic is self-contained; its
 * BASS drivers (bass, prop_bass, refine, refine_missing) map onto stspix_run_bass /
 * stspix_run_prop in the Python layer (st_spix_gb300.prop_cuda).
 *
 * shift_labels (prop/shift_labels.cu:82): every pixel of superpixel s moves by
 * flow[2s], flow[2s+1] (integer dx, dy; nspix rows); shifted = the largest label
 * arriving at a pixel (-1 if none), counts = arrivals.  Ids outside [0, nspix) stay. */
int stspix_legacy_shift_labels(stspix_ctx* ctx, void* stream, const int32_t* spix,
                               const int32_t* flow, int nspix, int H, int W, int32_t* shifted,
                               int32_t* counts);

/* fill_missing (prop/fill_missing.cu:317): fills the listed missing pixels (indices
 * into the frame) in place by the nearest FP32 centre (centers [ncenters, 2] = x, y)
 * among labelled 4-neighbours, parity phase by phase, until none is left, the count
 * repeats or break_iter iterations (0: no cap) ran.  *iters and *remaining (host,
 * may be NULL): iterations run and pixels still missing.  Synchronises per iteration.
 * Labels >= ncenters are not candidates.                                               */
int stspix_legacy_fill_missing(stspix_ctx* ctx, void* stream, int32_t* spix, const float* centers,
                               int ncenters, const int32_t* missing, int nmissing, int H, int W,
                               int break_iter, int* iters, int* remaining);

/* split (prop/bass.cu:389 run_split_py): one split step of the propagated model on
 * the labels spix [H,W] with the previous params (n_prev entries): update_params, a
 * split in direction 2 (direction == 0) or 1 (any other value, the count-parity rule of
 * prop/split_merge.cu:41-43), update_params, compaction of the new ids.  Output as
 * stspix_run_prop.  Synchronises the stream.                                          */
int stspix_legacy_split(stspix_ctx* ctx, void* stream, const float* img, int H, int W,
                        const stspix_config* cfg, int direction, const int32_t* spix,
                        const stspix_params* params_prev, int n_prev, int32_t* labels_out,
                        stspix_params* params_out, int* nspix_out);

/* rgb_to_lab (prop/rgb2lab.cu:167): as stspix_rgb2lab but the first channel is red.   */
int stspix_legacy_rgb_to_lab(stspix_ctx* ctx, void* stream, const float* rgb, float* lab,
                             long long npix);

/* sp_video_pooling (prop/sp_video_pooling.cu:62): img f32 [B,T,H,W,F], seg i32
 * [B,T,H,W] with ids < nspix -> down f32 [B,nspix,F] = per batch item mean feature of
 * each id over all frames (sum / (count + 1e-10)), counts f32 [B,nspix] (may be NULL),
 * pooled f32 [B,T,H,W,F] (may be NULL; 0 where the id is negative).                  */
int stspix_sp_video_pooling(stspix_ctx* ctx, void* stream, const float* img, const int32_t* seg,
                            int B, int T, int H, int W, int F, int nspix, float* pooled,
                            float* down, float* counts);

/* downsampled_video_to_pooled (prop/sp_video_pooling.cu:211): pooled[b,t,p] =
 * down[b, seg[b,t,p]] (0 where the id is negative).                                  */
int stspix_downsampled_video_to_pooled(stspix_ctx* ctx, void* stream, const float* down,
                                       const int32_t* seg, int B, int T, int H, int W, int F,
                                       int nspix, float* pooled);

/* run_update_prior (prop/sparams_io.cu:795-834): every id present in spix [npix] that
 * is >= prev_nspix (and < nids, the rows of the arrays) takes its estimates as priors:
 * prior_mu_app = mu_app [nids,3] (f32), prior_mu_shape = mu_shape [nids,2] (f64),
 * prior_sigma_shape = sigma_shape [nids,3] (f64; its 2x2 inverse when invert, with a
 * negative determinant replaced by 1e-6).                                            */
int stspix_legacy_update_prior(stspix_ctx* ctx, void* stream, const int32_t* spix,
                               long long npix, int nids, const float* mu_app, float* prior_mu_app,
                               const double* mu_shape, double* prior_mu_shape,
                               const double* sigma_shape, double* prior_sigma_shape,
                               int prev_nspix, int invert);

/* shift_tensor (prop/shift_tensor.cu:60-139; selected == NULL) and shift_tensor_ordered
 * (prop/shift_tensor_ordered.cu:53-137; selected i32 [B,H,W]): every pixel of in f32
 * [B,H,W,F] moves by its superpixel's integer flow (flow i32 [B,nspix,2] = dx, dy; labels
 * outside [0, nspix) stay); out [B,H,W,F] = sum of the features arriving at a pixel
 * (ordered: only those of its selected id), counts i32 [B,H,W] = their number,
 * contributors u8 [B,H,W,nspix] (may be NULL) = which ids arrive.  Sums are FP64, rounded
 * once (the legacy kernels add FP32 atomics in arbitrary order).                    */
int stspix_legacy_shift_tensor(stspix_ctx* ctx, void* stream, const float* in,
                               const int32_t* spix, const int32_t* flow, int B, int H, int W,
                               int F, int nspix, const int32_t* selected, float* out,
                               int32_t* counts, uint8_t* contributors);

/* shift_order (prop/shift_order.cu:43-119): selected i32 [B,H,W] = the first (smallest)
 * id whose contributors flag is set at the pixel, -1 if none (the legacy loop's running
 * minimum never updates after its first contributor).                               */
int stspix_legacy_shift_order(stspix_ctx* ctx, void* stream, const uint8_t* contributors,
                              int B, int H, int W, int nspix, int32_t* selected);

/* split_disconnected (prop/split_disconnected.cu:31-255, :390): spix i32 [H,W] with
 * labels in [0, nspix) is relabelled in place so that every connected region (equal
 * labels, neighbours within Chebyshev distance 2) but the largest of its label gets
 * the id nspix + split_starts[label] + its rank among the label's regions;
 * split_starts i32 [nspix]; children i32 [nspix, *max_nsplits] lists the new ids of
 * each label (-1 elsewhere).  *max_nsplits (host) = the total number of extra regions.
 * When nspix * *max_nsplits exceeds children_cap, nothing is relabelled and
 * STSPIX_ERR_CAPACITY is returned with *max_nsplits set.  Synchronises the stream.   */
int stspix_legacy_split_disconnected(stspix_ctx* ctx, void* stream, int32_t* spix, int H, int W,
                                     int nspix, int32_t* split_starts, int32_t* children,
                                     long long children_cap, int* max_nsplits);

/* ---- batched and serving forms -----------------------------------------------
 * No single reference counterpart: the reference processes one frame per call
 * (pyapi.cu:46 main_loop).  stspix_process_batch runs many frames, of uneven
 * sizes, in one pass: every kernel of the per-frame path is launched once for all
 * frames of the batch, so a frame's result is the same alone and in any batch.
 * A frame is either independent (run_bass on it, video == NULL) or the next frame
 * of a video stream whose labels, superpixel parameters and superpixel count stay
 * resident on the device between calls (shift_and_fill + run_prop, as
 * bist_forward does for frames after the first).                                 */
typedef struct stspix_video stspix_video;

/* Resident state of one video stream of frames of H x W pixels.  Any context on the
 * same device may process its next frame; the caller keeps a video out of two
 * batches that run at the same time (stspix_process_batch returns only when its
 * batch has finished, so sequential calls from different contexts are safe).  */
int stspix_video_create(stspix_ctx* ctx, stspix_video** out, int H, int W);
int stspix_video_destroy(stspix_video* video);
/* Forget the stream's history: its next frame starts a new video. */
int stspix_video_reset(stspix_video* video);
/* Superpixels of the stream's last frame (0 before its first frame). */
int stspix_video_nspix(const stspix_video* video);
/* Frames processed since creation or the last reset. */
long long stspix_video_frames(const stspix_video* video);

/* Snapshot / restore of a stream's resident state (labels, superpixel count and
 * parameters of its last frame) to and from host memory, e.g. to move a stream to
 * another context or process or to resume it later.  Layout: a 64-byte header
 * (magic "SPXVIDEO", version 1, H, W, nspix, frames) then the labels (i32, H*W) and
 * the 13 parameter arrays of stspix_params for nspix entries, in declaration order.
 * stspix_video_save: returns the bytes needed in *bytes; writes when capacity is
 * large enough.  stspix_video_load: the video must have the snapshot's H and W.
 * Both synchronise the stream.                                                */
int stspix_video_save(stspix_video* video, void* stream, void* host, long long capacity,
                      long long* bytes);
int stspix_video_load(stspix_video* video, void* stream, const void* host, long long bytes);

typedef struct stspix_frame {
  const float* img;       /* f32 [H,W,3] device                                         */
  const float* flow;      /* f32 [H,W,2] device, (dx,dy) from the video's previous
                             frame to this one; ignored on a video's first frame        */
  int H, W;
  int sp_size;            /* superpixel size of this frame; 0: cfg->sp_size             */
  int32_t* labels_out;    /* i32 [H,W] device                                           */
  stspix_video* video;    /* NULL: independent frame; else the video it continues       */
  /* set by stspix_process_batch (host): */
  int nspix;              /* superpixels of the frame                                   */
  int niters;             /* outer iterations run                                       */
  int status;             /* per-frame status (STSPIX_OK, NOPROGRESS, ...)              */
  stspix_frame_log log;
} stspix_frame;

/* Process `nframes` frames (at most one per video) as one batch on `stream`;
 * synchronises the stream.  Returns the first non-zero per-frame status, or an
 * error of the call itself.                                                      */
int stspix_process_batch(stspix_ctx* ctx, void* stream, stspix_frame* frames, int nframes,
                         const stspix_config* cfg);

/* Device bytes held per video stream (resident state) and per batch slot (the
 * working buffers of one frame in flight), for admission under a memory budget. */
int stspix_footprint(int H, int W, int sp_size, long long* video_bytes,
                     long long* slot_bytes);
/* GPU time (ms) of the last stspix_process_batch call, from CUDA events. */
double stspix_last_batch_ms(const stspix_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* ST_SPIX_GB300_H */
