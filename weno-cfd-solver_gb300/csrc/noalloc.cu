// weno_l_local_noalloc: the residual of weno_l_local with its scratch in a
// fixed array that the library owns, for callers that cannot allocate device
// memory.
//
// Who needs it: hosts that must not call into the CUDA allocator while they
// run this code -- a plugin whose host owns all device memory through its own
// pool, a loop that must not pay cudaMalloc's implicit device-wide
// synchronisation, or code being recorded into a CUDA graph.  They still pass
// their own input and output buffers; only the workspace comes from here.
//
// The scratch is one file-scope __device__ array of kScratchBytes (64 MiB).
// Every GPU that loads the library holds it until the process exits, and all
// calls on a device share it: two calls whose kernels overlap on the GPU (for
// instance on different streams) race on it, so callers must order them.  The
// array keeps the previous call's contents; nothing needs to start at zero,
// because every workspace element the kernels read is written earlier in the
// same call.
//
// Host code cannot use the array's name as a device address, so the first call
// on each device (with that device current) looks the address up with
// cudaGetSymbolAddress and caches it together with the identity of the
// device's current context.  A later call that finds another context (after
// cudaDeviceReset, or a context torn down and created again in the same
// process) looks the address up again instead of using the stale one.  That
// first call may load the module, so it should happen before any stream
// capture.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/weno_gb300.h"
#include "ctx_id.h"
#include "errors.h"

namespace {

constexpr size_t kScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};
unsigned long long g_scratch_ctx[kMaxDevices] = {};

}  // namespace

extern "C" int weno_l_local_noalloc(const double* u, int64_t m, int64_t n, int64_t c, int64_t s0, int64_t s1,
                                    int64_t s2, double dx, double gamma, int force_hlle, double jp_lo, double jp_hi,
                                    int cons, int mode, double* out, void* stream) {
  const size_t need = weno_l_local_workspace(m, n, force_hlle);
  if (need > kScratchBytes) {
    char msg[256];
    snprintf(msg, sizeof(msg),
             "l_local_noalloc: a %lld x %lld array needs %zu bytes of scratch, more than the fixed %zu-byte "
             "array; use weno_l_local with a caller workspace", (long long)m, (long long)n, need, kScratchBytes);
    return weno::set_last_error(WENO_ERR_WORKSPACE, msg);
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return weno::set_last_error(WENO_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return weno::set_last_error(WENO_ERR_ARG, "l_local_noalloc: device index too large");
  // 0 when no context is current yet: the lookup below creates the device's
  // primary context, and the id is read again after it.
  const unsigned long long ctx = weno::current_context_id();
  void* ptr = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_addr[dev] || ctx == 0 || g_scratch_ctx[dev] != ctx) {
      e = cudaGetSymbolAddress(&ptr, g_scratch);
      if (e != cudaSuccess) {
        char msg[256];
        snprintf(msg, sizeof(msg), "l_local_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return weno::set_last_error(WENO_ERR_CUDA, msg);
      }
      g_scratch_addr[dev] = ptr;
      g_scratch_ctx[dev] = weno::current_context_id();
    }
    ptr = g_scratch_addr[dev];
  }
  return weno_l_local(u, m, n, c, s0, s1, s2, dx, gamma, force_hlle, jp_lo, jp_hi, cons, mode, out, ptr,
                      kScratchBytes, stream);
}
