// Colour front end of the reference's frame pipeline (gauenk/st_spix
// st_spix/csrc/bist/rgb2lab.cu): sRGB -> CIELAB and back, and 8-bit frame ingest.
// Not called by bist_forward in the reference (pyapi.cu:95-102), so the drop-in path
// leaves frames as given; these serve callers that feed LAB, as the reference's
// command-line pipeline does, and the opt-in ingest conversion of the batched path
// (stspix_config.lab_ingest).
//
// The steps follow the reference exactly (they define the values callers compare
// against): the first channel is read as blue (rgb2lab.cu:64-66), the arithmetic is
// FP64 except that every power goes through the FP32 powf, L is stored divided by
// -100 and a, b by 100 in FP32, and pixels with a NaN channel are left unwritten.
// The colour constants are the CIE standard ones (D65 white, epsilon 0.008856,
// kappa 903.3, the sRGB transfer curve).
#include <cstdint>
#include <cuda_runtime.h>

#include "engine.h"
#include "pdl.h"

namespace stspix {

// One pixel: first_blue: the first channel is blue (bist/rgb2lab.cu:64-66); 0: red
// (the legacy prop/rgb2lab.cu:42-44 reads the channels in RGB order, otherwise
// identical).  Returns false (nothing written) for a pixel with a NaN channel.
__device__ __forceinline__ bool rgb2lab_px(const float* __restrict__ in, float* __restrict__ out,
                                           int first_blue) {
  const double c0 = (double)in[0];
  const double sG = (double)in[1];
  const double c2 = (double)in[2];
  const double sB = first_blue ? c0 : c2;
  const double sR = first_blue ? c2 : c0;
  if (sR != sR || sG != sG || sB != sB) return false;
  auto lin = [](double c) {
    return c <= 0.04045 ? c / 12.92 : (double)powf((float)((c + 0.055) / 1.055), (float)2.4);
  };
  const double r = lin(sR), g = lin(sG), b = lin(sB);
  const double X = r * 0.4124564 + g * 0.3575761 + b * 0.1804375;
  const double Y = r * 0.2126729 + g * 0.7151522 + b * 0.0721750;
  const double Z = r * 0.0193339 + g * 0.1191920 + b * 0.9503041;
  const double eps = 0.008856, kappa = 903.3;
  auto f = [&](double v) {
    return v > eps ? (double)powf((float)v, (float)(1.0 / 3.0)) : (kappa * v + 16.0) / 116.0;
  };
  const double fx = f(X / 0.950456), fy = f(Y / 1.0), fz = f(Z / 1.088754);
  const float lval = (float)(116.0 * fy - 16.0);
  const float aval = (float)(500.0 * (fx - fy));
  const float bval = (float)(200.0 * (fy - fz));
  out[0] = lval / (-100);
  out[1] = aval / 100;
  out[2] = bval / 100;
  return true;
}

__global__ void k_rgb2lab(const float* __restrict__ rgb, float* __restrict__ lab, long long npix,
                          int first_blue) {
  pdl_enter();
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  rgb2lab_px(rgb + 3 * t, lab + 3 * t, first_blue);
}

// Ingest of a batch with stspix_config.lab_ingest: every frame's colours converted
// once into the slot's engine buffer (img), which every later kernel reads.  A pixel
// with a NaN channel keeps its input values (the reference leaves it unwritten).
__global__ void kb_lab_ingest(const Slot* __restrict__ slots) {
  pdl_enter();
  const Slot& S = slots[blockIdx.y];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!S.img_src || t >= S.npix) return;
  float* out = const_cast<float*>(S.img) + 3 * t;
  const float* in = S.img_src + 3 * t;
  if (!rgb2lab_px(in, out, 1)) {
    out[0] = in[0];
    out[1] = in[1];
    out[2] = in[2];
  }
}

__global__ void k_lab2rgb(const float* __restrict__ lab, float* __restrict__ rgb, long long npix) {
  pdl_enter();
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= npix) return;
  const double L = lab[3 * t] * (-100);
  const double La = lab[3 * t + 1] * 100;
  const double Lb = lab[3 * t + 2] * 100;
  if (L != L || La != La || Lb != Lb) return;
  const double fy = (L + 16) / 116;
  const double fx = La / 500 + fy;
  const double fz = fy - Lb / 200;
  auto inv = [](double v) {
    const double c = (double)powf((float)v, (float)3);
    return c > 0.008856 ? c : (v - 16.0 / 116.0) / 7.787;
  };
  const double x = inv(fx), y = inv(fy), z = inv(fz);
  const double X = 0.950456 * x, Y = 1.000 * y, Z = 1.088754 * z;
  const double R = X * 3.2406 + Y * (-1.5372) + Z * (-0.4986);
  const double G = X * -0.9689 + Y * 1.8758 + Z * 0.0415;
  const double B = X * 0.0557 + Y * (-0.2040) + Z * 1.0570;
  auto gam = [](double c) {
    return c > 0.0031308 ? 1.055 * ((double)powf((float)c, (float)(1.0 / 2.4))) - 0.055 : 12.92 * c;
  };
  const double r = gam(R), g = gam(G), b = gam(B);
  // clamp to [0, 1] through float, written in RGB order
  float px = (float)fmin(1.0, b * 1.0), py = (float)fmin(1.0, g * 1.0), pz = (float)fmin(1.0, r * 1.0);
  px = (float)fmax(0.0, (double)px);
  py = (float)fmax(0.0, (double)py);
  pz = (float)fmax(0.0, (double)pz);
  rgb[3 * t] = pz;
  rgb[3 * t + 1] = py;
  rgb[3 * t + 2] = px;
}

// rescale_image_kernel (rgb2lab.cu:184-198): 8-bit frames to float, divided by mval.
__global__ void k_rescale_u8(const uint8_t* __restrict__ in, float* __restrict__ out,
                             long long nvals, float mval) {
  pdl_enter();
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nvals) return;
  out[t] = float(in[t] / mval);
}

}  // namespace stspix
