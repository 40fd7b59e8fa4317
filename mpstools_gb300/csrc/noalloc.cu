// Two-site matvec that allocates no device memory.
//
// Some callers cannot allocate device memory at the point where they need a matvec: host
// applications that hand the whole GPU memory budget to their own allocator and forbid libraries
// from allocating, and latency-bound loops that may not block on an allocation.
// For them the FP64 matvec can run with its stage-A intermediate X in a fixed device array that
// lives inside this library instead of the plan's own arena.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "host_ops.h"

namespace mpsg {

// Largest stage-A intermediate accepted: 1 Mi FP64 elements (8 MiB).
constexpr int64_t kNoAllocScratchElems = int64_t(1) << 20;

// The scratch.  Every GPU that loads this library holds these 8 MiB until the process exits, and
// every call shares them.  Host code must not use this name as a device address: the address is
// resolved with cudaGetSymbolAddress below.
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchElems];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_addr[256] = {};  // device address of g_noalloc_scratch per device ordinal
}  // namespace

// Resolves (once per device, with that device current) the device address of the scratch array.
// mpsg_ctx_create calls it for the context's device, so this module is loaded and the array placed
// when the library is set up; an execute call then only reads the cached address.  The cache is
// never invalidated: a device reset (cudaDeviceReset) while the library is loaded is not supported.
double* noalloc_scratch_address(int device) {
  MPSG_CHECK(device >= 0 && device < 256, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[device]) {
    double* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      throw Err(2, std::string("cudaGetSymbolAddress of the no-allocation scratch failed: ") + cudaGetErrorString(e));
    g_noalloc_addr[device] = p;
  }
  return g_noalloc_addr[device];
}

// Stage A writes every intermediate block in full (no accumulation into old contents) before
// stage C reads it, so nothing in the scratch has to be cleared between calls.
void matvec_noalloc(MatvecPlan& P, const double* theta_in, double* theta_out) {
  MPSG_CHECK(P.prec == MPSG_PREC_FP64, "the no-allocation matvec runs FP64 plans only");
  if (P.xa.nelem > kNoAllocScratchElems)
    throw Err(1, "the no-allocation matvec needs " + std::to_string(P.xa.nelem) +
                     " FP64 elements of intermediate storage; its limit is " +
                     std::to_string(kNoAllocScratchElems) + " (8 MiB)");
  int dev = -1;
  MPSG_CUDA(cudaGetDevice(&dev));
  MPSG_CHECK(dev == P.ctx->device, "the current CUDA device is not the device of the plan");
  double* X = noalloc_scratch_address(dev);
  const double* bases[8] = {P.dLt, theta_in, X, P.dRt, theta_out, nullptr, nullptr, nullptr};
  P.stageA.run(bases);
  P.stageC.run(bases);
  MPSG_CUDA(cudaGetLastError());
}

}  // namespace mpsg
