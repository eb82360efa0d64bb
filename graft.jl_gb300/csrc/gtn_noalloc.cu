// Allocation-free entry point: the batched Gram-Schmidt projections of the Krylov solvers
// (out[j] = <V_j, w>) for callers that cannot allocate device memory.
//
// Who needs it: a host that gives all of the GPU's memory to its own pool (a Julia
// CUDA.jl memory pool, a serving arena) cannot let a library call cudaMalloc behind its
// back, and a latency-critical loop cannot afford the device-wide synchronisation that
// cudaMalloc / cudaFree imply.  The regular path (gtn_dot, gtn_lanczos_min) keeps its
// partial sums in context- or map-owned device buffers; this variant keeps them in one
// file-scope __device__ array instead, so it needs neither a context nor an allocation.
//
// Limits and sharing:
//  * J <= 64 vectors; at most 512 partial-sum blocks: the scratch array holds
//    64 * 512 complex FP64 values (512 KiB) and every GPU that loads the library keeps it
//    until the process exits.
//  * Every call on a device uses the same array.  Calls whose kernels overlap on the GPU
//    (different streams, or different host threads without ordering) race on it; order
//    them on one stream.  Each call overwrites every partial it later reads, so nothing has
//    to be cleared between calls; the array keeps the last call's partials.
//  * The first call on a device resolves the array's device address with
//    cudaGetSymbolAddress (and reads the SM count) with that device current; make that
//    first call before any stream capture.  The resolved address is cached per device for
//    the life of the process: it does not survive cudaDeviceReset.
//  * An error left pending on the calling thread by earlier, unrelated CUDA work is not
//    consumed: the call then returns GTN_ERR_CUDA without launching, and the caller's own
//    cudaGetLastError still reports that error.
#include "gtn_internal.h"

#include <algorithm>
#include <mutex>

namespace {

constexpr int kNoAllocMaxJ = 64;
constexpr int kNoAllocMaxBlocks = 512;
constexpr int kMaxDevices = 64;

// Partial sums [block][j] of the two-pass reduction.
static __device__ __align__(256) double2 g_multidot_scratch[kNoAllocMaxJ * kNoAllocMaxBlocks];

std::mutex g_mu;
double2* g_scratch_addr[kMaxDevices] = {};
int g_blocks[kMaxDevices] = {};

}  // namespace

extern "C" int gtn_multidot_noalloc(void* stream, int64_t n, int J, const void* V, int64_t ldv,
                                    const void* w, void* out) {
  if (J < 1 || J > kNoAllocMaxJ) return GTN_ERR_INVALID;
  if (n < 0 || !V || !w || !out || (J > 1 && ldv < n)) return GTN_ERR_INVALID;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return GTN_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return GTN_ERR_UNSUPPORTED;
  // Do not launch over (and then swallow) an error that the caller's own work left pending.
  if (cudaPeekAtLastError() != cudaSuccess) return GTN_ERR_CUDA;
  double2* scratch = nullptr;
  int nblk = 0;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
      // Host code must not use g_multidot_scratch directly: its name here is a host-side
      // stand-in.  The device address comes from the runtime, once per device.
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_multidot_scratch) != cudaSuccess || !p) return GTN_ERR_CUDA;
      int sms = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return GTN_ERR_CUDA;
      g_blocks[dev] = std::max(1, std::min(2 * sms, kNoAllocMaxBlocks));
      g_scratch_addr[dev] = static_cast<double2*>(p);
    }
    scratch = g_scratch_addr[dev];
    nblk = g_blocks[dev];
  }
  const cudaError_t e = launch_multidot(static_cast<const double2*>(V), ldv, J, static_cast<const double2*>(w), n,
                                        static_cast<double2*>(out), scratch, nblk, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? GTN_OK : GTN_ERR_CUDA;
}
