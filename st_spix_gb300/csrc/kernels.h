// Kernel declarations of the GB300 streaming-BASS engine.
//
// kb_* kernels are batched: they take the device array of slots (one frame each)
// and pick their slot from the launch's y dimension (z for 3-D grids; x for the
// one-block-per-slot kb_scan).  k_* kernels serve the stand-alone
// utility entry points.
#pragma once
#include "engine.h"

namespace stspix {

// k_bass.cu
__global__ void k_init_hex(int* seg, int H, int W, double Hh, double w, int nx, int ny);
__global__ void k_find_border(const int* seg, uint8_t* border, int H, int W);
__global__ void k_find_border_end(const int* seg, uint8_t* border, int H, int W, int nframes);
__global__ void k_overlay(float* out, const float* img, const float* color,
                          const uint8_t* border, long long n);
__global__ void k_dump_state(SpDev sp, stspix_state_dump d);

__global__ void kb_scalars(const Slot* slots, int B, int op);
__global__ void kb_init_hex(const Slot* slots);
__global__ void kb_clear_flags(const Slot* slots);
__global__ void kb_mark_present(const Slot* slots, int mode);
__global__ void kb_scan(const Slot* slots, int mode);
__global__ void kb_remap(const Slot* slots, int mode);
__global__ void kb_compact_gather(const Slot* slots);
__global__ void kb_compact_scatter(const Slot* slots);
__global__ void kb_init_bass_params(const Slot* slots);
__global__ void kb_init_prior_mu(const Slot* slots);
__global__ void kb_clear_stats(const Slot* slots);
__global__ void kb_accumulate(const Slot* slots, int B);
__global__ void kb_posterior(const Slot* slots, int incremental);
__global__ void kb_post_list(const Slot* slots, int incremental);
__global__ void kb_accumulate_fp(const Slot* slots, int mode);
__global__ void kb_accumulate_fp_store(const Slot* slots, int mode);
__global__ void kb_accumulate_fp_clear(const Slot* slots);
__global__ void k_label_stats(const float* img, const int* lab, long long npix, int n, int mode,
                              long long* iacc, float* facc, double* dacc);
__global__ void k_label_stats_out(int n, int mode, const long long* iacc, const float* facc,
                                  const double* dacc, double* out);
__global__ void kb_store_sample(const Slot* slots);
__global__ void kb_find_border(const Slot* slots);
// boundary sweep, one block per 32x32 / 64x32 / 16x32 tile of the batch
__global__ void kb_sweep_t32(const Slot* slots, int B, int parity, float s2, float potts,
                             int mode, int deltas);
__global__ void kb_sweep_t64(const Slot* slots, int B, int parity, float s2, float potts,
                             int mode, int deltas);
__global__ void kb_sweep_t16(const Slot* slots, int B, int parity, float s2, float potts,
                             int mode, int deltas);
// the same single sweep as a persistent work-queue kernel (queue: 2 counters, zero
// between launches)
__global__ void kb_sweepq_t32(const Slot* slots, int B, int ntiles, unsigned* queue, int parity,
                              float s2, float potts, int mode, int deltas);
__global__ void kb_sweepq_t64(const Slot* slots, int B, int ntiles, unsigned* queue, int parity,
                              float s2, float potts, int mode, int deltas);
__global__ void kb_sweepq_t16(const Slot* slots, int B, int ntiles, unsigned* queue, int parity,
                              float s2, float potts, int mode, int deltas);
// two consecutive sweeps per launch (8-pixel halo)
__global__ void kb_sweep2_t32(const Slot* slots, int B, int parity, float s2, float potts,
                              int mode, int deltas);
__global__ void kb_sweep2_t16(const Slot* slots, int B, int parity, float s2, float potts,
                              int mode, int deltas);
__global__ void kb_sweep2_t64(const Slot* slots, int B, int parity, float s2, float potts,
                              int mode, int deltas);
__global__ void kb_copy_labels(const Slot* slots);
__global__ void kb_read_params(const Slot* slots);
__global__ void kb_save_prev(const Slot* slots);

// k_splitmerge.cu
__global__ void kb_split_begin(const Slot* slots, int B);
__global__ void kb_split_clear(const Slot* slots);
__global__ void kb_split_seed(const Slot* slots, int dir_bass, int dir_prop);
__global__ void kb_bbox(const Slot* slots);
__global__ void kb_split_bfs(const Slot* slots, int dir_bass, int dir_prop);
__global__ void kb_split_bfs_big(const Slot* slots);
__global__ void kb_split_partition(const Slot* slots);
__global__ void kb_sm_clear(const Slot* slots);
__global__ void kb_sm_accumulate(const Slot* slots, int split);
__global__ void kb_split_decide(const Slot* slots, SmConsts K, float split_alpha);
__global__ void kb_split_commit(const Slot* slots);
__global__ void kb_split_apply(const Slot* slots);
__global__ void kb_split_end(const Slot* slots, int B);
__global__ void kb_merge_clear(const Slot* slots);
__global__ void kb_merge_candidates(const Slot* slots, int dir_bass, int dir_prop);
__global__ void kb_merge_single(const Slot* slots, SmConsts K);
__global__ void kb_merge_decide(const Slot* slots, SmConsts K, float merge_alpha);
__global__ void kb_merge_flag(const Slot* slots);
__global__ void kb_merge_remove(const Slot* slots);
__global__ void kb_merge_apply(const Slot* slots);

// k_prop.cu
__global__ void kb_prop_clear(const Slot* slots);
__global__ void kb_flow_pool(const Slot* slots);
__global__ void kb_flow_mean(const Slot* slots);
__global__ void kb_shift(const Slot* slots);
__global__ void kb_shift_decode(const Slot* slots);
__global__ void kb_count_labels(const Slot* slots, int which);
__global__ void kb_fill_begin(const Slot* slots, int B);
__global__ void kb_fill_split(const Slot* slots, int pass);
__global__ void kb_fill_phase(const Slot* slots, int ph, int B, cudaGraphConditionalHandle cond,
                              int break_iter, int* body_iters, unsigned* ctr);
__global__ void kb_fill_end(const Slot* slots);
__global__ void kb_cc_local(const Slot* slots);
__global__ void kb_cc_hook(const Slot* slots);
__global__ void kb_cc_compress(const Slot* slots);
__global__ void kb_list_holes(const Slot* slots);
__global__ void kb_cc_best(const Slot* slots);
__global__ void kb_cc_invalidate(const Slot* slots);
__global__ void kb_shift_params(const Slot* slots);
__global__ void kb_write_params(const Slot* slots);
__global__ void kb_mark_active(const Slot* slots);
__global__ void kb_relabel_init(const Slot* slots);
__global__ void kb_living(const Slot* slots);
__global__ void kb_relabel_compare(const Slot* slots);
__global__ void kb_relabel_mark(const Slot* slots, float thresh_replace, float thresh_new);
__global__ void kb_relabel_ids(const Slot* slots);
__global__ void kb_relabel_params(const Slot* slots);
__global__ void kb_relabel_apply(const Slot* slots);
__global__ void kb_relabel_end(const Slot* slots, int B);
__global__ void kb_count_revived(const Slot* slots);

// k_color.cu
__global__ void k_rgb2lab(const float* rgb, float* lab, long long npix, int first_blue);
__global__ void kb_lab_ingest(const Slot* slots);
__global__ void k_lab2rgb(const float* lab, float* rgb, long long npix);
__global__ void k_rescale_u8(const uint8_t* in, float* out, long long nvals, float mval);

// k_quality.cu
constexpr int kQGtShared = 256;
__global__ void k_q_range_init(int* mm);
__global__ void k_q_range(const int32_t* a, long long n, int* mm);
__global__ void k_q_accum(const float* vid, const int32_t* spix, const int32_t* gt, int T, int H,
                          int W, int off, int S, int G1, int* cnt, double* fsum, double* vsum,
                          double* msum, int* J);
__global__ void k_q_resid(const float* vid, const int32_t* spix, int npix, int off, int S,
                          const int* cnt, const double* fsum, const double* msum, double* pix2,
                          double* pix2s, double* sse);
__global__ void k_q_id_time(const int* cnt, int T, int S, long long* ntot, double* std_out);
__global__ void k_q_frame_ids(const int* cnt, const double* fsum, const double* vsum,
                              const long long* ntot, const double* msum, int S, int npix,
                              unsigned long long* live, double* pool2, double* pool3);
__global__ void k_q_uesa_frame(const int* cnt, const int* J, int S, int G1, unsigned long long* ue,
                               unsigned long long* sa, unsigned long long* size);
__global__ void k_q_uesa_id(const int* cnt, const int* J, const long long* ntot, int T, int S,
                            int G1, unsigned long long* ue3, unsigned long long* sa3);
__global__ void k_q_down(const int* cnt, const double* fsum, long long TS, float* down);

// k_legacy.cu
__global__ void k_fill_i32(int32_t* p, long long n, int32_t v);
__global__ void k_lshift(const int32_t* spix, const int32_t* flow, int nspix, int H, int W,
                         int32_t* shifted, int32_t* counts);
__global__ void k_lfill_border(const int32_t* seg, const int32_t* missing, int nmissing, int H,
                               int W, uint8_t* border, int* num_neg);
__global__ void k_lfill_phase(int32_t* seg, const float* centers, int ncenters,
                              const int32_t* missing, const uint8_t* border, int nmissing, int H,
                              int W, int xm, int ym);
__global__ void k_vpool_accum(const float* img, const int32_t* seg, int T, long long npix, int F,
                              int nspix, double* sum, unsigned long long* cnt);
__global__ void k_vpool_mean(const double* sum, const unsigned long long* cnt, long long nbs,
                             int F, float* down, float* counts);
__global__ void k_vpool_write(const float* down, const int32_t* seg, int T, long long npix, int F,
                              int nspix, float* pooled);
__global__ void k_q_pool_write(const int32_t* spix, int npix, int off, int S, long long n,
                               const float* down, float* pooled);
__global__ void k_lmark_ids(const int32_t* spix, long long n, int nids, uint8_t* present);
__global__ void k_lupdate_prior(const uint8_t* present, int nids, int prev_nspix, int invert,
                                const float* mu_app, float* prior_mu_app, const double* mu_shape,
                                double* prior_mu_shape, const double* sigma_shape,
                                double* prior_sigma_shape);
__global__ void k_lshift_tensor(const float* in, const int32_t* spix, const int32_t* flow, int H,
                                int W, int F, int nspix, const int32_t* selected, double* acc,
                                int32_t* counts, uint8_t* contributors);
__global__ void k_round_f32(const double* acc, long long n, float* out);
__global__ void k_lshift_order(const uint8_t* contributors, long long npix_all, int nspix,
                               int32_t* selected);
__global__ void k_lsd_init(int32_t* parent, int npix);
__global__ void k_lsd_hook(const int32_t* spix, int H, int W, int32_t* parent, int* status);
__global__ void k_lsd_roots(int32_t* parent, int npix, int32_t* is_root);
__global__ void k_lscan(const int32_t* in, int n, int32_t* out, int32_t* total);
__global__ void k_lsd_regions(const int32_t* spix, const int32_t* root, const int32_t* rank,
                              int npix, int nspix, int32_t* region_of, int32_t* region_spix,
                              int32_t* region_size, int32_t* spix_counts);
__global__ void k_lsd_starts(const int32_t* spix_counts, int nspix, int32_t* split_starts,
                             int32_t* max_nsplits);
__global__ void k_lsd_offsets(const int32_t* region_spix, const int32_t* region_size,
                              int nregions, int nspix, int32_t* region_offset);
__global__ void k_lsd_update(int32_t* spix, const int32_t* region_of,
                             const int32_t* region_offset, const int32_t* split_starts, int npix,
                             int nspix, int max_nchild, int32_t* children);

}  // namespace stspix
