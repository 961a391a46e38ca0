// lj_noalloc.cu -- mixed-precision force call that allocates nothing.
//
// Who needs it: callers that may not allocate device memory at all -- code
// running inside a host that owns every allocation (a pooled allocator the
// engine cannot see, a real-time loop where cudaMalloc's implicit device
// synchronisation is not allowed, or a plugin host that forbids its plugins
// to allocate).  The regular mixed path keeps its scratch (the fixed-point
// position image and, for open boxes, the frame words) in buffers the
// context allocates; this entry point keeps that scratch in a fixed,
// file-scope device array instead.
//
// Limits and sharing:
//   * at most kNoAllocMaxParticles particles (16 MiB of scratch, held by
//     every GPU that loads the library until the process exits);
//   * every call shares the one array and leaves its contents behind, so two
//     calls that overlap on the GPU (different streams, or different host
//     threads on one device) race and must be ordered by the caller;
//   * the first call on each device resolves the array's device address
//     with cudaGetSymbolAddress and arms the open-box frame words with one
//     small kernel on the caller's stream; make that first call before any
//     stream capture on that device;
//   * the list is not validated (the reference's kernels do not validate
//     theirs either): every index must be in [0, n).
#include <mutex>

#include "lj_gb300.h"
#include "lj_internal.h"

namespace ljg {
namespace {

constexpr int kNoAllocMaxParticles = 1 << 20;
constexpr size_t kImageBytes = sizeof(int4) * (size_t)kNoAllocMaxParticles;
constexpr size_t kScratchBytes = kImageBytes + 256;  // + the open-box frame words

// The scratch: fixed-point image of q, then the open-box frame words
// (kOpenFrameWords long longs, open boundaries only).  Host code must not use
// this symbol's name as an address: it is a host-side stand-in.  The device
// address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];
static_assert(sizeof(long long) * kOpenFrameWords <= kScratchBytes - kImageBytes,
              "frame words fit behind the image");

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device.  Set-up on the
// first call per device: the address lookup and the arming of the frame
// words (a kernel on stream s, ahead of that call's own work).
cudaError_t scratch_address(void** out, cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    e = launch_open_frame_init(
        reinterpret_cast<long long*>(static_cast<unsigned char*>(p) + kImageBytes), s);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

}  // namespace
}  // namespace ljg

using namespace ljg;

extern "C" int lj_force_mixed_noalloc_aos(const double* q, double* p, int32_t n, double dt,
                                          double cl2, const int32_t* sorted_list,
                                          const int32_t* number_of_partners,
                                          const int32_t* pointer, const double* box,
                                          void* stream) {
  if (n < 0 || n > kNoAllocMaxParticles) return LJ_ERR_INVALID_ARGUMENT;
  if (n > 0 && (!q || !p || !sorted_list || !number_of_partners || !pointer))
    return LJ_ERR_INVALID_ARGUMENT;
  if ((reinterpret_cast<uintptr_t>(q) & 15u) || (reinterpret_cast<uintptr_t>(p) & 15u))
    return LJ_ERR_INVALID_ARGUMENT;
  if (!(cl2 >= 0.0) || !(dt - dt == 0.0)) return LJ_ERR_INVALID_ARGUMENT;  // dt finite
  if (n == 0) return LJ_OK;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  void* base = nullptr;
  if (scratch_address(&base, s) != cudaSuccess) return LJ_ERR_CUDA;
  ForceLaunch L{};
  L.part.soa = 0;
  L.part.q = q;
  L.part.p = p;
  L.csr = Csr{n, 0, number_of_partners, pointer, sorted_list, 0, 0};
  if (box) {
    L.box.on = 1;
    for (int d = 0; d < 3; d++) {
      if (!(box[d] > 0.0)) return LJ_ERR_INVALID_ARGUMENT;
      L.box.len[d] = box[d];
      L.box.half[d] = 0.5 * box[d];
    }
    const double mn = box[0] < box[1] ? (box[0] < box[2] ? box[0] : box[2])
                                      : (box[1] < box[2] ? box[1] : box[2]);
    if (cl2 > 0.25 * mn * mn) return LJ_ERR_INVALID_ARGUMENT;
  }
  L.dt = dt;
  L.cl2 = cl2;
  L.precision = LJ_PREC_MIXED;
  L.method = LJ_METHOD_GATHER_FULL;
  L.kernel = 2;
  L.unroll = 4;
  L.lanes = 4;
  L.block = 128;
  L.qfix = static_cast<int4*>(base);
  if (!L.box.on) {
    // the open frame from the coordinates' bounds, chosen on the device into
    // the frame words behind the image (no host round trip)
    long long* words =
        reinterpret_cast<long long*>(static_cast<unsigned char*>(base) + kImageBytes);
    if (launch_open_bounds(L.part, n, words, s) != cudaSuccess) return LJ_ERR_CUDA;
    make_device_frame(L, words);
  } else {
    make_fixed_frame(L);
  }
  if (launch_fixed_image(L, s) != cudaSuccess) return LJ_ERR_CUDA;
  return launch_force(L, s) == cudaSuccess ? LJ_OK : LJ_ERR_CUDA;
}
