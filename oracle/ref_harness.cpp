// ORACLE -- test infrastructure only.  Runs the reference's OWN CUDA kernels (the
// cubins oracle/ref_build.py compiles from gauenk/st_spix st_spix/csrc/bist/*.cu,
// unmodified, into oracle/_ref/) through the CUDA driver API, sequenced the way the
// reference's host functions sequence them, on inputs supplied by the tests.  It is
// how the CPU oracle and the engine are pinned against the reference itself on the
// GPU host.
//
// Two layers:
//   * stage functions (refh_find_border ... refh_rescale) that run one reference
//     stage on host arrays, used by the stage pins;
//   * a generic layer (refh_variant_load, refh_fn, refh_malloc, refh_launch, ...)
//     over which oracle/ref_runner.py restates the reference's whole host drivers
//     (run_bass, shift_and_fill, run_prop, main_loop) in Python.
//
// Host code here is this project's; it mirrors the reference's host loops:
//   update_seg            update_seg.cu:281-311
//   update_params         update_params.cu:12-31
//   init_seg              init_seg.cu:20-46
//   split BFS             split_merge_orig.cu:262-356 (init_split + calc_split_candidate)
//   fill_missing          fill_missing.cu:35-130
//   find_spix_min loop    split_disconnected.cu:107-150
// The reference's spix_params layout comes from oracle/_ref/spix_layout.h (generated
// from its structs.h).
#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "_ref/spix_layout.h"

namespace {

CUcontext g_ctx = nullptr;
CUmodule g_mod[8] = {};
std::string g_err;

struct Fn { const char* module; const char* name; CUfunction f; };
// Mangled names of the reference kernels (C++ signatures in the reference sources).
Fn g_fn[] = {
    {"seg_utils", "_Z18find_border_pixelsPKiPbiii", nullptr},
    {"seg_utils", "_Z22find_border_pixels_endPKiPbiii", nullptr},
    {"update_seg", "_Z17update_seg_subsetPfPiPbP11spix_paramsffiiiiiii", nullptr},
    {"update_params", "_Z12clear_fieldsP11spix_paramsP11spix_helperii", nullptr},
    {"update_params", "_Z12sum_by_labelPKfPKiP11spix_paramsP11spix_helperiiii", nullptr},
    {"update_params", "_Z18calc_simple_updateP11spix_paramsP11spix_helperfii", nullptr},
    {"init_seg", "_Z13InitHexCenterPdddiiii", nullptr},
    {"init_seg", "_Z10InitHexSegPiPdiii", nullptr},
    {"split_merge", "_Z20calc_split_candidatePiS_PbiS_iiii", nullptr},
    {"split_merge", "_Z10init_splitPKbPiP11spix_paramsiiiiiPKiS1_i", nullptr},
    {"fill_missing", "_Z21update_missing_seg_nnPiPdPbiiiiiib", nullptr},
    {"fill_missing", "_Z25find_border_along_missingPKiPbiiiPi", nullptr},
    {"split_disconnected", "_Z13find_spix_minPiS_S_S_iii", nullptr},
    {"rgb2lab", "_Z10rgb_to_labPfS_i", nullptr},
    {"rgb2lab", "_Z10lab_to_rgbPfS_i", nullptr},
    {"rgb2lab", "_Z20rescale_image_kernelPhPfif", nullptr},
};
enum { F_BORDER, F_BORDER_END, F_UPDATE_SUBSET, F_CLEAR, F_SUM, F_SIMPLE_UPDATE, F_HEX_CENTER,
       F_HEX_SEG, F_SPLIT_CAND, F_INIT_SPLIT, F_FILL_NN, F_FILL_BORDER, F_SPIX_MIN, F_RGB2LAB,
       F_LAB2RGB, F_RESCALE };
const char* kModules[] = {"seg_utils", "update_seg", "update_params", "init_seg", "split_merge",
                          "fill_missing", "split_disconnected", "rgb2lab"};
constexpr int kHelperSize = 96;  // sizeof(spix_helper): float3, double3, longlong2, longlong3

#define CU(call)                                                      \
  do {                                                                \
    CUresult r_ = (call);                                             \
    if (r_ != CUDA_SUCCESS) {                                         \
      const char* s_ = nullptr;                                       \
      cuGetErrorString(r_, &s_);                                      \
      g_err = std::string(#call) + ": " + (s_ ? s_ : "?");            \
      return -1;                                                      \
    }                                                                 \
  } while (0)

int launch(int fn, unsigned grid, unsigned block, void** args) {
  CU(cuLaunchKernel(g_fn[fn].f, grid, 1, 1, block, 1, 1, 0, nullptr, args, nullptr));
  return 0;
}
unsigned nblk(long long n) { return (unsigned)((n + 511) / 512); }  // THREADS_PER_BLOCK 512

struct Dev {
  CUdeviceptr p = 0;
  ~Dev() { if (p) cuMemFree(p); }
};
int alloc(Dev& d, size_t bytes) {
  CU(cuMemAlloc(&d.p, bytes ? bytes : 1));
  return 0;
}

// Build the reference's AoS spix_params array from SoA fields (nullptr = zero).
std::vector<unsigned char> pack_params(int n, const int* count, const float* mu_app,
                                       const double* mu_shape, const double* sigma_shape,
                                       const double* logdet, const float* prior_count,
                                       const int* valid, const int* prop,
                                       const double* prior_icov, const double* sample_sigma) {
  std::vector<unsigned char> b((size_t)n * REF_SP_SIZE, 0);
  for (int k = 0; k < n; k++) {
    unsigned char* e = b.data() + (size_t)k * REF_SP_SIZE;
    if (mu_app) memcpy(e + REF_OFF_mu_app, mu_app + 3 * k, 12);
    if (mu_shape) memcpy(e + REF_OFF_mu_shape, mu_shape + 2 * k, 16);
    if (sigma_shape) memcpy(e + REF_OFF_sigma_shape, sigma_shape + 3 * k, 24);
    if (logdet) memcpy(e + REF_OFF_logdet_sigma_shape, logdet + k, 8);
    if (count) memcpy(e + REF_OFF_count, count + k, 4);
    if (prior_count) memcpy(e + REF_OFF_prior_count, prior_count + k, 4);
    if (valid) memcpy(e + REF_OFF_valid, valid + k, 4);
    if (prop) { bool v = prop[k] != 0; memcpy(e + REF_OFF_prop, &v, 1); }
    if (prior_icov) memcpy(e + REF_OFF_prior_icov, prior_icov + 3 * k, 24);
    if (sample_sigma) memcpy(e + REF_OFF_sample_sigma_shape, sample_sigma + 3 * k, 24);
  }
  return b;
}

}  // namespace

extern "C" {

const char* refh_error() { return g_err.c_str(); }

int refh_init(const char* dir) {
  if (g_ctx) return 0;
  CU(cuInit(0));
  CUdevice dev;
  CU(cuDeviceGet(&dev, 0));
  CU(cuDevicePrimaryCtxRetain(&g_ctx, dev));
  CU(cuCtxSetCurrent(g_ctx));
  constexpr int kNumModules = (int)(sizeof(kModules) / sizeof(kModules[0]));
  static_assert(kNumModules <= (int)(sizeof(g_mod) / sizeof(g_mod[0])), "module table too small");
  for (int m = 0; m < kNumModules; m++) {
    std::string path = std::string(dir) + "/" + kModules[m] + ".cubin";
    CU(cuModuleLoad(&g_mod[m], path.c_str()));
  }
  for (auto& fn : g_fn) {
    int m = 0;
    while (strcmp(kModules[m], fn.module) != 0) m++;
    CU(cuModuleGetFunction(&fn.f, g_mod[m], fn.name));
  }
  return 0;
}

// find_border_pixels (mode 0) / find_border_pixels_end (mode 1).
int refh_find_border(const int32_t* labels, uint8_t* border, int H, int W, int mode) {
  CU(cuCtxSetCurrent(g_ctx));
  int npix = H * W;
  Dev s, b;
  if (alloc(s, 4 * (size_t)npix) || alloc(b, npix)) return -1;
  CU(cuMemcpyHtoD(s.p, labels, 4 * (size_t)npix));
  CU(cuMemsetD8(b.p, 0, npix));
  void* args[] = {&s.p, &b.p, &npix, &W, &H};
  if (launch(mode ? F_BORDER_END : F_BORDER, nblk(npix), 512, args)) return -1;
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(border, b.p, npix));
  return 0;
}

// init_seg (init_seg.cu:20-46): host geometry as there, reference kernels.
int refh_init_seg(int H, int W, int sp_size, int32_t* labels) {
  CU(cuCtxSetCurrent(g_ctx));
  double Hh = sqrt(double(pow(sp_size, 2)) / (1.5 * sqrt(3.0)));
  double w = sqrt(3.0) * Hh;
  int nx = (int)floor(double(W) / w) + 2;
  int ny = (int)floor(double(H) / (1.5 * Hh)) + 2;
  int nspix = nx * ny, npix = H * W;
  Dev c, s;
  if (alloc(c, 16 * (size_t)nspix) || alloc(s, 4 * (size_t)npix)) return -1;
  void* a1[] = {&c.p, &Hh, &w, &nspix, &nx, &W, &H};
  if (launch(F_HEX_CENTER, nblk(nspix), 512, a1)) return -1;
  void* a2[] = {&s.p, &c.p, &nspix, &npix, &W};
  if (launch(F_HEX_SEG, nblk(npix), 512, a2)) return -1;
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(labels, s.p, 4 * (size_t)npix));
  return nspix;
}

// update_params (update_params.cu:12-31) on given labels and priors.
int refh_update_params(const float* img, const int32_t* labels, int H, int W, int nbuf,
                       int sp_size, float sigma2_app, const int* valid, const int* prop,
                       const float* prior_count, const double* prior_icov,
                       const double* sample_sigma, int* count_out, float* mu_app_out,
                       double* mu_shape_out, double* sigma_shape_out, double* logdet_out,
                       int* valid_out) {
  CU(cuCtxSetCurrent(g_ctx));
  int npix = H * W, nbatch = 1, nftrs = 3;
  auto host = pack_params(nbuf, nullptr, nullptr, nullptr, nullptr, nullptr, prior_count, valid,
                          prop, prior_icov, sample_sigma);
  Dev im, sg, sp, hp;
  if (alloc(im, 12 * (size_t)npix) || alloc(sg, 4 * (size_t)npix) ||
      alloc(sp, host.size()) || alloc(hp, (size_t)kHelperSize * nbuf))
    return -1;
  CU(cuMemcpyHtoD(im.p, img, 12 * (size_t)npix));
  CU(cuMemcpyHtoD(sg.p, labels, 4 * (size_t)npix));
  CU(cuMemcpyHtoD(sp.p, host.data(), host.size()));
  void* a1[] = {&sp.p, &hp.p, &nbuf, &nftrs};
  if (launch(F_CLEAR, nblk(nbuf), 512, a1)) return -1;
  CU(cuMemsetD8(hp.p, 0, (size_t)kHelperSize * nbuf));
  void* a2[] = {&im.p, &sg.p, &sp.p, &hp.p, &npix, &nbatch, &W, &nftrs};
  if (launch(F_SUM, nblk(npix), 512, a2)) return -1;
  void* a3[] = {&sp.p, &hp.p, &sigma2_app, &sp_size, &nbuf};
  if (launch(F_SIMPLE_UPDATE, nblk(nbuf), 512, a3)) return -1;
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(host.data(), sp.p, host.size()));
  for (int k = 0; k < nbuf; k++) {
    const unsigned char* e = host.data() + (size_t)k * REF_SP_SIZE;
    memcpy(count_out + k, e + REF_OFF_count, 4);
    memcpy(mu_app_out + 3 * k, e + REF_OFF_mu_app, 12);
    memcpy(mu_shape_out + 2 * k, e + REF_OFF_mu_shape, 16);
    memcpy(sigma_shape_out + 3 * k, e + REF_OFF_sigma_shape, 24);
    memcpy(logdet_out + k, e + REF_OFF_logdet_sigma_shape, 8);
    memcpy(valid_out + k, e + REF_OFF_valid, 4);
  }
  return 0;
}

// update_seg (update_seg.cu:281-311) on given parameters; labels updated in place.
int refh_update_seg(const float* img, int32_t* labels, int H, int W, int nbuf, int niters_seg,
                    float sigma2_app, float potts, const int* count, const float* mu_app,
                    const double* mu_shape, const double* sigma_shape, const double* logdet) {
  CU(cuCtxSetCurrent(g_ctx));
  int npix = H * W, nbatch = 1, nftrs = 3;
  auto host = pack_params(nbuf, count, mu_app, mu_shape, sigma_shape, logdet, nullptr, nullptr,
                          nullptr, nullptr, nullptr);
  Dev im, sg, sp, bd;
  if (alloc(im, 12 * (size_t)npix) || alloc(sg, 4 * (size_t)npix) ||
      alloc(sp, host.size()) || alloc(bd, npix))
    return -1;
  CU(cuMemcpyHtoD(im.p, img, 12 * (size_t)npix));
  CU(cuMemcpyHtoD(sg.p, labels, 4 * (size_t)npix));
  CU(cuMemcpyHtoD(sp.p, host.data(), host.size()));
  for (int it = 0; it < niters_seg; it++) {
    CU(cuMemsetD8(bd.p, 0, npix));
    void* ab[] = {&sg.p, &bd.p, &npix, &W, &H};
    if (launch(F_BORDER, nblk(npix), 512, ab)) return -1;
    for (int xm = 0; xm < 2; xm++)
      for (int ym = 0; ym < 2; ym++) {
        void* au[] = {&im.p, &sg.p, &bd.p, &sp.p, &sigma2_app, &potts, &npix, &nbatch, &W, &H,
                      &nftrs, &xm, &ym};
        if (launch(F_UPDATE_SUBSET, nblk(npix), 512, au)) return -1;
      }
  }
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(labels, sg.p, 4 * (size_t)npix));
  return 0;
}

// init_split + calc_split_candidate loop (split_merge_orig.cu:262-356): distance
// field of the seeds for `direction`.
int refh_split_bfs(const int32_t* labels, int H, int W, int nbuf, const int* valid,
                   const double* mu_shape, int direction, int max_spix, int32_t* dist_out) {
  CU(cuCtxSetCurrent(g_ctx));
  int npix = H * W, nbatch = 1;
  auto host = pack_params(nbuf, nullptr, nullptr, mu_shape, nullptr, nullptr, nullptr, valid,
                          nullptr, nullptr, nullptr);
  Dev sg, sp, ds, bd, mx, done;
  if (alloc(sg, 4 * (size_t)npix) || alloc(sp, host.size()) || alloc(ds, 4 * (size_t)npix) ||
      alloc(bd, npix) || alloc(mx, 4) || alloc(done, 4))
    return -1;
  CU(cuMemcpyHtoD(sg.p, labels, 4 * (size_t)npix));
  CU(cuMemcpyHtoD(sp.p, host.data(), host.size()));
  CU(cuMemsetD8(ds.p, 0xff, 4 * (size_t)npix));
  CU(cuMemsetD8(bd.p, 0, npix));
  void* ai[] = {&bd.p, &ds.p, &sp.p, &nbuf, &nbatch, &W, &H, &direction, &sg.p, &mx.p, &max_spix};
  if (launch(F_INIT_SPLIT, nblk(nbuf), 512, ai)) return -1;
  int distance = 1, flag = 1, steps = 0;
  while (flag) {
    CU(cuMemsetD32(done.p, 0, 1));
    void* ac[] = {&ds.p, &sg.p, &bd.p, &distance, &done.p, &npix, &nbatch, &W, &H};
    if (launch(F_SPLIT_CAND, nblk(npix), 512, ac)) return -1;
    distance++;
    CU(cuMemcpyDtoH(&flag, done.p, 4));
    if (++steps > 5005) { g_err = "BFS did not finish"; return -1; }
  }
  CU(cuMemcpyDtoH(dist_out, ds.p, 4 * (size_t)npix));
  return steps;
}

// fill_missing (fill_missing.cu:35-130); returns iterations, or -2 on no progress.
int refh_fill(int32_t* seg, const double* centers, int ncenters, int H, int W, int break_iter) {
  CU(cuCtxSetCurrent(g_ctx));
  int npix = H * W, nbatch = 1;
  Dev sg, ct, bd, nn;
  if (alloc(sg, 4 * (size_t)npix) || alloc(ct, 16 * (size_t)ncenters) || alloc(bd, npix) ||
      alloc(nn, 4))
    return -1;
  CU(cuMemcpyHtoD(sg.p, seg, 4 * (size_t)npix));
  CU(cuMemcpyHtoD(ct.p, centers, 16 * (size_t)ncenters));
  int iter = 0, prev_neg = (int)1410065408, num_neg = 1, status = 0;
  bool print_values = false;
  while (num_neg > 0) {
    if (break_iter > 0 && iter >= break_iter) break;
    CU(cuMemsetD32(nn.p, 0, 1));
    CU(cuMemsetD8(bd.p, 0, npix));
    void* ab[] = {&sg.p, &bd.p, &nbatch, &H, &W, &nn.p};
    if (launch(F_FILL_BORDER, nblk(npix), 512, ab)) return -1;
    CU(cuMemcpyDtoH(&num_neg, nn.p, 4));
    for (int xm = 0; xm < 2; xm++)
      for (int ym = 0; ym < 2; ym++) {
        void* af[] = {&sg.p, &ct.p, &bd.p, &nbatch, &H, &W, &npix, &xm, &ym, &print_values};
        if (launch(F_FILL_NN, nblk(npix), 512, af)) return -1;
      }
    iter++;
    if (num_neg == prev_neg) { status = -2; break; }
    prev_neg = num_neg;
  }
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(seg, sg.p, 4 * (size_t)npix));
  return status ? status : iter;
}

// find_spix_min iterated to a fixed point (split_disconnected.cu:107-150): region
// roots (minimum pixel index of each 8-connected equal-label region).
int refh_cc_roots(const int32_t* seg, int H, int W, int32_t* roots) {
  CU(cuCtxSetCurrent(g_ctx));
  int npix = H * W;
  std::vector<int32_t> init(npix);
  for (int i = 0; i < npix; i++) init[i] = i;
  Dev sg, cur, prev, ch;
  if (alloc(sg, 4 * (size_t)npix) || alloc(cur, 4 * (size_t)npix) ||
      alloc(prev, 4 * (size_t)npix) || alloc(ch, 4))
    return -1;
  CU(cuMemcpyHtoD(sg.p, seg, 4 * (size_t)npix));
  CU(cuMemcpyHtoD(cur.p, init.data(), 4 * (size_t)npix));
  int changes = 1, steps = 0;
  while (changes) {
    CU(cuMemcpyDtoD(prev.p, cur.p, 4 * (size_t)npix));
    CU(cuMemsetD32(ch.p, 0, 1));
    void* a[] = {&sg.p, &cur.p, &prev.p, &ch.p, &H, &W, &npix};
    if (launch(F_SPIX_MIN, nblk(npix), 512, a)) return -1;
    CU(cuMemcpyDtoH(&changes, ch.p, 4));
    if (++steps > 100000) { g_err = "components did not converge"; return -1; }
  }
  CU(cuMemcpyDtoH(roots, cur.p, 4 * (size_t)npix));
  return steps;
}

// rgb_to_lab / lab_to_rgb (one batch); the input is copied, the output starts as a
// copy of the input (the kernels leave NaN pixels unwritten).
int refh_color(int which, const float* in, float* out, int npix) {
  CU(cuCtxSetCurrent(g_ctx));
  Dev a, b;
  if (alloc(a, 12 * (size_t)npix) || alloc(b, 12 * (size_t)npix)) return -1;
  CU(cuMemcpyHtoD(a.p, in, 12 * (size_t)npix));
  CU(cuMemcpyHtoD(b.p, in, 12 * (size_t)npix));
  // rgb_to_lab(img_rgb, img_lab, npix); lab_to_rgb(img_rgb, img_lab, npix)
  void* args_fwd[] = {&a.p, &b.p, &npix};
  void* args_inv[] = {&b.p, &a.p, &npix};
  if (launch(which == 0 ? F_RGB2LAB : F_LAB2RGB, nblk(npix), 512,
             which == 0 ? args_fwd : args_inv))
    return -1;
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(out, b.p, 12 * (size_t)npix));
  return 0;
}

int refh_rescale(const uint8_t* in, float* out, int npix, float mval) {
  CU(cuCtxSetCurrent(g_ctx));
  Dev a, b;
  if (alloc(a, 3 * (size_t)npix) || alloc(b, 12 * (size_t)npix)) return -1;
  CU(cuMemcpyHtoD(a.p, in, 3 * (size_t)npix));
  void* args[] = {&a.p, &b.p, &npix, &mval};
  if (launch(F_RESCALE, nblk(npix), 512, args)) return -1;
  CU(cuCtxSynchronize());
  CU(cuMemcpyDtoH(out, b.p, 12 * (size_t)npix));
  return 0;
}


// ---------------------------------------------------------------------------------
// Generic layer.  A "variant" is one directory of cubins (oracle/_ref for the
// -fmad=false build, oracle/_ref/stock for nvcc's default contraction).  Kernels are
// looked up by module and unmangled name from the functions the driver enumerates in
// that module.  Every launch goes to the legacy default stream, as the reference's.
// ---------------------------------------------------------------------------------
namespace {
struct Variant {
  std::vector<std::string> names;
  std::vector<CUmodule> mods;
};
std::vector<Variant> g_var;
std::vector<CUfunction> g_gfn;
std::vector<std::string> g_gfn_name;
std::vector<CUevent> g_ev;
}  // namespace

// Load the cubins `units` (comma separated) from `dir`; returns the variant index.
int refh_variant_load(const char* dir, const char* units) {
  if (!g_ctx) { g_err = "refh_init first"; return -1; }
  CU(cuCtxSetCurrent(g_ctx));
  Variant v;
  std::string all(units), cur;
  for (size_t i = 0; i <= all.size(); i++) {
    if (i == all.size() || all[i] == ',') {
      if (!cur.empty()) {
        CUmodule m;
        std::string path = std::string(dir) + "/" + cur + ".cubin";
        CU(cuModuleLoad(&m, path.c_str()));
        v.names.push_back(cur);
        v.mods.push_back(m);
      }
      cur.clear();
    } else {
      cur += all[i];
    }
  }
  g_var.push_back(v);
  return (int)g_var.size() - 1;
}

// Kernel `name` (unmangled) of `module` in variant `var`.  When the module holds
// several kernels of that name, `mangled` (non-empty) picks one.  Returns a handle.
int refh_fn(int var, const char* module, const char* name, const char* mangled) {
  CU(cuCtxSetCurrent(g_ctx));
  if (var < 0 || var >= (int)g_var.size()) { g_err = "bad variant"; return -1; }
  Variant& v = g_var[var];
  int mi = -1;
  for (int i = 0; i < (int)v.names.size(); i++)
    if (v.names[i] == module) mi = i;
  if (mi < 0) { g_err = std::string("module not loaded: ") + module; return -1; }
  unsigned n = 0;
  CU(cuModuleGetFunctionCount(&n, v.mods[mi]));
  std::vector<CUfunction> fs(n);
  if (n) CU(cuModuleEnumerateFunctions(fs.data(), n, v.mods[mi]));
  std::string prefix = "_Z" + std::to_string(strlen(name)) + name;
  CUfunction hit = nullptr;
  std::string hit_name, seen;
  int hits = 0;
  for (CUfunction f : fs) {
    const char* nm = nullptr;
    CU(cuFuncGetName(&nm, f));
    if (!nm) continue;
    std::string s(nm);
    bool match = mangled && *mangled ? s == mangled : s.rfind(prefix, 0) == 0;
    if (match) { hit = f; hit_name = s; hits++; seen += s + " "; }
  }
  if (hits != 1) {
    g_err = std::string(module) + "." + name + ": " + std::to_string(hits) + " matches " + seen;
    return -1;
  }
  g_gfn.push_back(hit);
  g_gfn_name.push_back(hit_name);
  return (int)g_gfn.size() - 1;
}

const char* refh_fn_name(int h) {
  return (h >= 0 && h < (int)g_gfn_name.size()) ? g_gfn_name[h].c_str() : "";
}

unsigned long long refh_malloc(unsigned long long bytes) {
  if (cuCtxSetCurrent(g_ctx) != CUDA_SUCCESS) return 0;
  CUdeviceptr p = 0;
  CUresult r = cuMemAlloc(&p, bytes ? bytes : 16);
  if (r != CUDA_SUCCESS) { g_err = "cuMemAlloc failed"; return 0; }
  return (unsigned long long)p;
}
int refh_free(unsigned long long p) { CU(cuMemFree((CUdeviceptr)p)); return 0; }
int refh_memset8(unsigned long long p, unsigned v, unsigned long long n) {
  CU(cuMemsetD8((CUdeviceptr)p, (unsigned char)v, n)); return 0;
}
int refh_memset32(unsigned long long p, unsigned v, unsigned long long n) {
  CU(cuMemsetD32((CUdeviceptr)p, v, n)); return 0;
}
int refh_h2d(unsigned long long p, const void* h, unsigned long long n) {
  CU(cuMemcpyHtoD((CUdeviceptr)p, h, n)); return 0;
}
int refh_d2h(void* h, unsigned long long p, unsigned long long n) {
  CU(cuMemcpyDtoH(h, (CUdeviceptr)p, n)); return 0;
}
int refh_d2d(unsigned long long d, unsigned long long s, unsigned long long n) {
  CU(cuMemcpyDtoD((CUdeviceptr)d, (CUdeviceptr)s, n)); return 0;
}
// Launch handle `h` on grid (gx, gy) x block (bx) with `nargs` arguments, each held in
// one 8-byte slot (its value in the slot's low bytes, as the kernel's parameter type).
int refh_launch(int h, unsigned gx, unsigned gy, unsigned bx, unsigned long long* slots,
                int nargs) {
  if (h < 0 || h >= (int)g_gfn.size()) { g_err = "bad kernel handle"; return -1; }
  if (gx == 0 || gy == 0) return 0;  // an empty grid launches nothing
  void* params[32];
  if (nargs > 32) { g_err = "too many kernel arguments"; return -1; }
  for (int i = 0; i < nargs; i++) params[i] = &slots[i];
  CU(cuLaunchKernel(g_gfn[h], gx, gy, 1, bx, 1, 1, 0, nullptr, params, nullptr));
  return 0;
}
int refh_sync() { CU(cuCtxSynchronize()); return 0; }
// Events for timing reference kernels on the default stream.
int refh_event_record(int i) {
  while ((int)g_ev.size() <= i) {
    CUevent e;
    CU(cuEventCreate(&e, CU_EVENT_DEFAULT));
    g_ev.push_back(e);
  }
  CU(cuEventRecord(g_ev[i], nullptr));
  return 0;
}
int refh_event_ms(int a, int b, float* ms) {
  if (a < 0 || b < 0 || a >= (int)g_ev.size() || b >= (int)g_ev.size()) {
    g_err = "bad event index"; return -1;
  }
  CU(cuEventSynchronize(g_ev[b]));
  CU(cuEventElapsedTime(ms, g_ev[a], g_ev[b]));
  return 0;
}

}  // extern "C"
