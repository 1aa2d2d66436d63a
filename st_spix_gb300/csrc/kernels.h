// Kernel declarations of the GB300 streaming-BASS engine.
#pragma once
#include "engine.h"

namespace stspix {

// k_bass.cu
__global__ void k_init_hex(int* seg, int H, int W, double Hh, double w, int nx, int ny);
__global__ void k_mark_present(const int* seg, int npix, int lo, const int* hi_ptr,
                               int hi_static, uint8_t* flags);
__global__ void k_scan_flags(const uint8_t* flags, const int* n_ptr, int n_static, int* excl,
                             int* total);
__global__ void k_remap(int* seg, int npix, int lo, const int* excl);
__global__ void k_compact_gather(SpDev sp, SpDev tmp, int lo, const int* hi_ptr,
                                 const uint8_t* flags, const int* excl);
__global__ void k_compact_scatter(SpDev sp, SpDev tmp, int lo, const int* nnew);
__global__ void k_init_bass_params(SpDev sp, const int* nspix_ptr, int npix, int sp_size);
__global__ void k_init_prior_mu(SpDev sp, const int* nspix_ptr);
__global__ void k_accumulate(const float* img, const int* seg, int H, int W, SpDev sp);
__global__ void k_posterior(SpDev sp, int sp_size, Scalars* sc);
__global__ void k_store_sample(SpDev sp);
__global__ void k_find_border(const int* seg, uint8_t* border, int H, int W);
__global__ void k_find_border_end(const int* seg, uint8_t* border, int H, int W, int nframes);
__global__ void k_overlay(float* out, const float* img, const float* color,
                          const uint8_t* border, long long n);
__global__ void k_update_phase(const float* img, int* seg, const uint8_t* border,
                               const SweepRec* rec, int cap, int H, int W, int xmod, int ymod,
                               float s2, float potts);
__global__ void k_sweep_fused(const float* img, const int* seg_in, int* seg_out,
                              const SweepRec* rec, int cap, int H, int W, float s2, float potts);
__global__ void k_read_params(SpDev sp, const int* n_ptr, stspix_params out);
__global__ void k_dump_state(SpDev sp, stspix_state_dump d);

// k_splitmerge.cu
__global__ void k_split_begin(Scalars* sc);
__global__ void k_split_seed(SpDev sp, const int* seg, int H, int W, int direction,
                             const Scalars* sc, int* d1, int* d2);
__global__ void k_relax_bfs(const int* seg, int* f1, int* f2, int H, int W, Scalars* sc,
                            int* round_flags, int max_rounds);
__global__ void k_relax_cc(const int* seg, int* f1, int* f2, int H, int W, Scalars* sc,
                           int* round_flags, int max_rounds);
__global__ void k_split_partition(const int* seg, const int* d1, const int* d2, int npix,
                                  const Scalars* sc, int* sm);
__global__ void k_sm_accumulate(const float* img, const int* lab, const int* shifted, int H,
                                int W, int cap, SmDev sm);
__global__ void k_split_decide(SpDev sp, SmDev sm, Scalars* sc, SmConsts K, float split_alpha,
                               int prop_mode, uint8_t* accept);
__global__ void k_split_commit(SpDev sp, SmDev sm, Scalars* sc, const uint8_t* accept,
                               const int* excl, int prop_mode);
__global__ void k_split_apply(int* seg, const int* smseg, int npix, SpDev sp, SmDev sm,
                              const Scalars* sc, const uint8_t* accept, int prop_mode);
__global__ void k_split_end(Scalars* sc, const int* nsplits);
__global__ void k_merge_candidates(const int* seg, const uint8_t* border, int H, int W,
                                   int direction, int prop_mode, const uint8_t* prop, int cap,
                                   int* pair);
__global__ void k_merge_single(SpDev sp, SmDev sm, SmConsts K);
__global__ void k_merge_decide(SpDev sp, SmDev sm, Scalars* sc, SmConsts K, float merge_alpha);
__global__ void k_merge_flag(SpDev sp, SmDev sm, uint8_t* valid0);
__global__ void k_merge_remove(SpDev sp, SmDev sm, Scalars* sc, const uint8_t* valid0,
                               int prop_mode);
__global__ void k_merge_apply(int* seg, int npix, int cap, SmDev sm);

// k_prop.cu
__global__ void k_flow_pool(const int* lab, const float* flow, int H, int W, int n, int* cnt,
                            long long* fs);
__global__ void k_flow_mean(int n, const int* cnt, const long long* fs, const double* mu_shape,
                            float* fds, double* centers);
__global__ void k_shift(const int* lab, int H, int W, int n, const int* cnt, const float* fds,
                        int* hits, unsigned long long* best);
__global__ void k_shift_decode(const int* hits, const unsigned long long* best, int npix,
                               int* shifted, int* filled, Scalars* sc);
__global__ void k_count_labels(const int* lab, int npix, int n, int* cnt);
__global__ void k_fill_coop(int* seg, const double* centers, int H, int W, uint8_t* border,
                            Scalars* sc, int* iter_counts, int break_iter);
__global__ void k_cc_init(const int* seg, int npix, int* root);
__global__ void k_cc_size(const int* root, int npix, int* size);
__global__ void k_cc_best(const int* seg, const int* root, const int* size, int npix, int nlab,
                          unsigned long long* best);
__global__ void k_cc_invalidate(int* seg, const int* root, int npix, int nlab,
                                const unsigned long long* best);
__global__ void k_shift_params(int n, const int* cnt_pool, const int* cs, const int* cf,
                               stspix_params pp);
__global__ void k_write_params(SpDev sp, const stspix_params pp, int n, int sp_size);
__global__ void k_mark_active(const int* lab, int npix, SpDev sp);
__global__ void k_prop_begin(Scalars* sc, int n);
__global__ void k_living(const int* seg, int npix, const Scalars* sc, uint8_t* living);
__global__ void k_relabel_init(int cap, unsigned long long* best, float* ss);
__global__ void k_relabel_compare(const SpDev sp, const float* prev_prior_mu_app, int n_prev,
                                  const Scalars* sc, const uint8_t* living,
                                  unsigned long long* best, float* ss, int chunk);
__global__ void k_relabel_mark(int cap, const Scalars* sc, const uint8_t* living,
                               const unsigned long long* best, const float* ss,
                               float thresh_replace, float thresh_new, int* rid, uint8_t* mint);
__global__ void k_relabel_ids(int cap, Scalars* sc, const uint8_t* mint, const int* excl,
                              int* rid, int* src_of);
__global__ void k_relabel_params(SpDev sp, const int* rid, const int* src_of, int n_prev);
__global__ void k_relabel_apply(int* seg, int npix, int cap, const int* rid);
__global__ void k_relabel_end(Scalars* sc, const int* nminted, const int* rid, int cap);
__global__ void k_count_revived(const int* rid, const uint8_t* mint, int cap, Scalars* sc);

}  // namespace stspix
