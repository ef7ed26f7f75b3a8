// ss_iterated_noalloc: the iterated smoother for callers that cannot allocate
// device memory.
//
// Some hosts hand a library nothing but data pointers and a stream: plug-ins
// running inside another runtime's memory pool (where a stray cudaMalloc would
// bypass the host's accounting or fail outright), code that must not
// synchronise the device (cudaMalloc/cudaFree may), and deployments whose
// device memory is fully reserved up front.  For them this entry point takes
// its scratch space from a fixed array that lives in this library's own
// device image instead of a caller-provided workspace.
//
// The array costs SS_NOALLOC_SCRATCH_BYTES on every GPU that loads the
// library, for as long as the process runs.  Problems that need more scratch
// than that are rejected with SS_ERR_WORKSPACE.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sqrtsmooth.h"

namespace {

constexpr int kMaxDevices = 64;

// The scratch space.  Device code could name it directly; host code must ask
// the runtime for its device address (below), once per device.
__device__ __align__(256) unsigned char ss_noalloc_scratch[SS_NOALLOC_SCRATCH_BYTES];

std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  The first call
// on a device resolves it with cudaGetSymbolAddress (with that device
// current) and remembers it; later calls reuse the cached address.
int scratch_on_current_device(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SS_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_scratch_addr[dev] == nullptr) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, ss_noalloc_scratch) != cudaSuccess || p == nullptr) return SS_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return SS_OK;
}

}  // namespace

extern "C" int ss_iterated_noalloc(const ss_problem* p, const void* ys, const void* m0, const void* L0,
                                   int32_t prior_per_sequence, const void* init_m, const void* init_L,
                                   int32_t n_iter, double tol, void* out_m, void* out_L, double* out_ell,
                                   int32_t* out_iters, uint32_t* out_flags, ss_stream_t stream) {
  size_t need = 0;
  int rc = ss_workspace_bytes(p, &need);
  if (rc != SS_OK) return rc;
  if (need > (size_t)SS_NOALLOC_SCRATCH_BYTES) return SS_ERR_WORKSPACE;
  void* scratch = nullptr;
  rc = scratch_on_current_device(&scratch);
  if (rc != SS_OK) return rc;
  // Every region of the scratch that the smoother reads is written earlier in
  // the same call, so leftovers of a previous call need no clearing.
  return ss_iterated(p, ys, m0, L0, prior_per_sequence, init_m, init_L, n_iter, tol, out_m, out_L, out_ell,
                     out_iters, out_flags, scratch, (size_t)SS_NOALLOC_SCRATCH_BYTES, stream);
}
