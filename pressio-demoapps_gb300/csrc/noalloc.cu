// Face-flux scratch held in the library's own static device memory, for the
// allocation-free velocity entry point (pda_velocity_noalloc).
//
// Who needs it: callers that may not allocate device memory while they
// evaluate the right-hand side -- real-time or embedded loops whose memory
// budget is fixed at start-up, and hosts with their own pool allocators that
// forbid a library allocating behind their back.  The regular entry point allocates its face buffers on
// the first call of each problem (and grows them on demand), which none of
// those callers can accept.
//
// The buffer is one file-scope __device__ array of PDA_NOALLOC_SCRATCH_DOUBLES
// doubles.  Nothing in it needs to start at zero: every face flux the
// balance kernel reads is written earlier in the same call by the face
// kernels.  The array is shared by every problem of the process on a device,
// so two calls that overlap in time (different streams or threads without
// ordering between them) race on it.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/pda_gb300.h"

namespace pda {

static __device__ __align__(256) double g_noalloc_face_scratch[PDA_NOALLOC_SCRATCH_DOUBLES];

namespace {
constexpr int kMaxCachedDevices = 64;
std::mutex g_mu;
double *g_addr[kMaxCachedDevices] = {};
}  // namespace

// Device address of the scratch array on the current device.  The symbol is
// looked up once per device (this first lookup may load the module that
// holds the array) and cached for the process: like every problem handle,
// the cached address does not survive cudaDeviceReset.  Devices beyond the
// cache's 64 entries look the symbol up on every call (it allocates nothing).
cudaError_t noalloc_face_scratch(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_mu);
  if (dev >= 0 && dev < kMaxCachedDevices && g_addr[dev]) {
    *out = g_addr[dev];
    return cudaSuccess;
  }
  void *p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_face_scratch);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kMaxCachedDevices) g_addr[dev] = static_cast<double *>(p);
  *out = static_cast<double *>(p);
  return cudaSuccess;
}

}  // namespace pda
