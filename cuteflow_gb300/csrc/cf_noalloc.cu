/*
 * cf_noalloc.cu -- cf_step_noalloc: the step with its edge-flux scratch in a static device
 * array, for callers that may not allocate device memory while they step (a host model whose
 * GPU memory is budgeted among coupled components at start-up, a process under a fixed
 * device-memory limit).  The entry point has no counterpart in the reference.
 *
 * The scratch is the array of 48-byte slots through which the edge kernel passes each edge
 * side's flux and bed source to the element kernel.  Here it is one file-scope array of
 * CF_NOALLOC_SCRATCH_SLOTS slots (16 MiB), present on every GPU that loads the library until
 * the process exits.  Its name is a host-side stand-in, not a device address: every call takes
 * the address in the current device's context with cudaGetSymbolAddress (which allocates nothing;
 * on a device's first call it can load the library's device code there) and hands it to the
 * kernels as their slot pointer.  Looking it up on every call, rather than caching it per
 * device, keeps it valid after cudaDeviceReset or under a context other than the primary one,
 * where the module and its array are loaded again at another address.  Calls share the array
 * and race if their work overlaps on the GPU.
 */
#include <cuda_runtime.h>

#include <string>

#include "cf_internal.h"

static __device__ __align__(256) cf::Slot g_noalloc_slots[CF_NOALLOC_SCRATCH_SLOTS];

namespace {

/* The device address of the array in the current context. */
int scratch_address(cf_ctx* c, cf::Slot** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_slots);
  if (e != cudaSuccess || !p)
    return cf::ctx_error(c, CF_ECUDA, std::string("cudaGetSymbolAddress of the static scratch: ") +
                                          cudaGetErrorString(e));
  *out = static_cast<cf::Slot*>(p);
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
