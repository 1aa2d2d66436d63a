// Allocation-free variant of get_marked_video (stspix_get_marked_video_noalloc).
//
// Some callers cannot allocate device memory at call time: a process that reserves
// all of its GPU memory up front and forbids later cudaMalloc, code running inside
// a stream capture owned by another library, or a real-time loop where an
// allocation (and the device synchronisation cudaFree implies) is not allowed.
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
//    stream capture.
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
  const unsigned blocks = (unsigned)((n + 255) / 256);
  stspix::k_find_border_end<<<blocks, 256, 0, st>>>(spix, (uint8_t*)border, H, W, T);
  stspix::k_overlay<<<blocks, 256, 0, st>>>(marked_out, vid, color, (const uint8_t*)border, n);
  return cudaGetLastError() == cudaSuccess ? STSPIX_OK : STSPIX_ERR_CUDA;
}
