// Allocation-free variant of get_marked_video (stspix_get_marked_video_noalloc).
//
// Some callers cannot allocate device memory at call time: a process that reserves
// all of its GPU memory up front and forbids later cudaMalloc, a plugin whose host
// application owns every device allocation, or a real-time loop where an allocation
// (and the device synchronisation cudaFree implies) is not allowed.
// stspix_get_marked_video needs a one-byte-per-pixel border mask as scratch; this
// variant keeps that scratch in a fixed array compiled into the library instead.
//
// Limits and sharing rules:
//  * the scratch holds kMarkedMaxPixels = 2^24 pixels (16 MiB, T*H*W across all
//    frames); larger inputs are rejected with STSPIX_ERR_TOO_LARGE before any work;
//  * every GPU that loads the library holds the 16 MiB until the process exits;
//  * all calls share the one array: calls that overlap on the GPU (different
//    streams, or different host threads) race on it and must be serialised by the
//    caller; each call rewrites every byte it reads, so nothing needs clearing;
//  * the first call on a device looks up the array's device address (set-up, once
//    per device, with that device current); make that first call before starting any
//    stream capture.  The address is cached per device for the life of the process,
//    so the entry point must not be used across a cudaDeviceReset of that device;
//  * frames have 3 channels (nftrs == 3), as for stspix_get_marked_video;
//  * `stream` must belong to the current device (checked: STSPIX_ERR_ARG otherwise);
//  * launch failures are read from the launch calls themselves, so an error left
//    pending by unrelated earlier work is neither reported here nor cleared.
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "engine.h"
#include "kernels.h"

namespace {

constexpr long long kMarkedMaxPixels = 1LL << 24;
constexpr int kMaxDevices = 64;

// Border-mask scratch.  In host code this name is only a stand-in for the symbol;
// the device address comes from cudaGetSymbolAddress below.
__device__ __align__(256) uint8_t g_marked_border[kMarkedMaxPixels];

std::mutex g_setup_mu;
void* g_border_addr[kMaxDevices] = {};

}  // namespace

extern "C" int stspix_get_marked_video_noalloc(void* stream, const float* vid,
                                                const int32_t* spix, const float* color, int T,
                                                int H, int W, int nftrs, float* marked_out) {
  if (!vid || !spix || !color || !marked_out) return STSPIX_ERR_ARG;
  if (nftrs != 3 || T < 0 || H < 1 || W < 1) return STSPIX_ERR_ARG;
  const long long n = (long long)T * H * W;
  if (n > kMarkedMaxPixels) return STSPIX_ERR_TOO_LARGE;
  if (n == 0) return STSPIX_OK;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return STSPIX_ERR_CUDA;
  void* border = nullptr;
  {
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_border_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_marked_border) != cudaSuccess || !p) return STSPIX_ERR_CUDA;
      g_border_addr[dev] = p;
    }
    border = g_border_addr[dev];
  }
  cudaStream_t st = (cudaStream_t)stream;
  int sdev = -1;
  if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) return STSPIX_ERR_ARG;
  if (sdev != dev) return STSPIX_ERR_ARG;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  uint8_t* bmask = (uint8_t*)border;
  const uint8_t* cmask = bmask;
  int h = H, w = W, t = T;
  long long nn = n;
  void* a1[] = {(void*)&spix, (void*)&bmask, (void*)&h, (void*)&w, (void*)&t};
  if (cudaLaunchKernel((const void*)stspix::k_find_border_end, dim3(blocks), dim3(256), a1, 0,
                       st) != cudaSuccess)
    return STSPIX_ERR_CUDA;
  void* a2[] = {(void*)&marked_out, (void*)&vid, (void*)&color, (void*)&cmask, (void*)&nn};
  if (cudaLaunchKernel((const void*)stspix::k_overlay, dim3(blocks), dim3(256), a2, 0, st) !=
      cudaSuccess)
    return STSPIX_ERR_CUDA;
  return STSPIX_OK;
}
