/*
 * cf_noalloc.cu -- cf_step_noalloc: the step with its edge-flux scratch in a static device
 * array, for callers that may not allocate device memory while they step (a host model whose
 * GPU memory is budgeted among coupled components at start-up, a process under a fixed
 * device-memory limit).  The entry point has no counterpart in the reference.
 *
 * The scratch is the array of 48-byte slots through which the edge kernel passes each edge
 * side's flux and bed source to the element kernel.  Here it is one file-scope array of
 * CF_NOALLOC_SCRATCH_SLOTS slots (16 MiB), present on every GPU that loads the library until
 * the process exits.  Its name is a host-side stand-in, not a device address: the address is
 * taken with cudaGetSymbolAddress once per device, on the first call with that device
 * current, and handed to the kernels as their slot pointer.  Calls share the array and race
 * if their work overlaps on the GPU.
 */
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "cf_internal.h"

static __device__ __align__(256) cf::Slot g_noalloc_slots[CF_NOALLOC_SCRATCH_SLOTS];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
cf::Slot* g_addr[kMaxDevices] = {};

/* The device address of the array on the current device (looked up on first use). */
int scratch_address(cf_ctx* c, cf::Slot** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cf::ctx_error(c, CF_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return cf::ctx_error(c, CF_ENOTSUP, "device index beyond 63");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_slots);
    if (e != cudaSuccess || !p)
      return cf::ctx_error(c, CF_ECUDA, std::string("cudaGetSymbolAddress of the static scratch: ") +
                                            cudaGetErrorString(e));
    g_addr[dev] = static_cast<cf::Slot*>(p);
  }
  *out = g_addr[dev];
  return CF_OK;
}

}  // namespace

extern "C" int cf_step_noalloc(cf_ctx* ctx, int32_t nsteps, cf_step_info* info) {
  if (!ctx) return CF_EINVAL;
  int rc = cf::ctx_set_device(ctx);
  if (rc != CF_OK) return rc;
  cf::Slot* scratch = nullptr;
  if ((rc = scratch_address(ctx, &scratch)) != CF_OK) return rc;
  return cf::step_with_slots(ctx, nsteps, info, scratch, CF_NOALLOC_SCRATCH_SLOTS);
}
