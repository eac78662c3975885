/*
 * cf_ctx.h -- the context object behind the C ABI and the helpers its implementation files
 * share (cf_api.cpp: the step; cf_adjoint_api.cpp: the adjoint).  Host code only.
 */
#ifndef CF_CTX_H
#define CF_CTX_H

#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include <exception>
#include <new>

#include "cf_internal.h"

namespace cf {

/* One simulation of a context: its inputs, host tables and place in the flat space. */
struct Member {
  cf_params params{};
  Prep prep;
  int32_t n = 0, ne = 0;
  int32_t cell_off = 0, edge_off = 0;
  int32_t ctile_begin = 0, ctile_end = 0;
  int32_t inl_off = 0;      /* first phys_inflow entry of the member */
  MemberDev dev{};
};

}  // namespace cf

struct cf_ctx {
  int device = 0;
  int32_t iflux = 1, ilimiteur = 1, flux_mode = 0;
  std::vector<cf::Member> mem;
  int32_t n_pad = 0, ne_pad = 0, n_etiles = 0, n_ctiles = 0, max_n = 0;
  cudaStream_t stream = nullptr;
  /* device memory (flat over members) */
  double4* U[2] = {nullptr, nullptr};
  int4* cslot = nullptr;
  int4* cnbr = nullptr;
  double4* cstat = nullptr;
  double* zcell = nullptr;
  int32_t* perm = nullptr;   /* new -> old, member-local */
  int32_t* iperm = nullptr;  /* old -> new, member-local */
  int2* ecell = nullptr;
  double4* egeo = nullptr;
  double4* ez = nullptr;   /* per edge: the beds it reads */
  int32_t* ebid = nullptr;
  int4* eupw = nullptr;
  double4* ewts = nullptr;
  double4* edk = nullptr;
  double4* einv = nullptr;
  cf::Slot* slots = nullptr;
  int32_t* etile_mem = nullptr;
  int32_t* ctile_mem = nullptr;
  cf::MemberDev* mdev = nullptr;
  cf::MemberState* mst = nullptr;
  double* staging = nullptr;           /* 3 * max_n doubles, reference order */
  int32_t* inl_cell = nullptr;         /* phys_inflow entries of all members */
  double* inl_len = nullptr;
  int64_t n_inl = 0;
  bool any_phys_inflow = false;        /* some member has inlet 3 */
  bool any_steady = false;             /* some member tests for steady state */
  int32_t* ids = nullptr;              /* max_n element ids (cf_get_elements / cf_set_elements) */
  int32_t xd_cmp = 0;                  /* edge kernel: integer comparisons (cf_set_tuning) */
  int32_t xd_mul_mask = 0;             /* edge kernel: warps multiplying on the integer pipes */
  /* launch shape (cf_set_launch_shape): the autotuner's usual choice on the 1M WAF step, 2-3 %
   * faster there than (128, 1, 256) */
  int32_t eblock = 256, ept = 1;       /* edge kernel: threads per block, edges per thread */
  int32_t cblock = 128;                /* threads per block of the element kernel */
  cf::MemberState* host_state = nullptr;   /* pinned, one record per member */
  bool direct_io = true;               /* kernels read / write callers' pinned host states directly */
  int32_t* bq = nullptr;               /* boundary edges of every member in reference order */
  /* a part of a decomposed mesh (cf_create_part): elements ordered send, interior, halo */
  bool is_part = false;
  int32_t n_send = 0, n_own = 0;
  int32_t* elist1 = nullptr;           /* edges of the send elements */
  int32_t* elist2 = nullptr;           /* the other edges of the interior elements */
  int32_t nel1 = 0, nel2 = 0;
  int32_t* xsend = nullptr;            /* exchange plan: element ids (device order) packed, unpacked */
  int32_t* xrecv = nullptr;
  int32_t nxsend = 0, nxrecv = 0;
  bool external_sums = false;          /* phys_inflow sums set by the caller (cf_part_set_inlet_sums) */
  double* terms = nullptr;             /* a part's inlet or discharge terms, for the caller's sums */
  cudaEvent_t ev_pack = nullptr;       /* the send buffer of the last cf_part_step_begin is complete */
  /* stepping */
  int64_t launched = 0;                /* steps launched since creation (buffer parity) */
  cudaGraphExec_t graph2 = nullptr;    /* two steps: parity 0 then 1 */
  bool use_graph = true;
  /* timing */
  bool timing = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};   /* 0-2 timing, 3: inputs of cf_set_state consumed */
  double flux_ms = 0.0, update_ms = 0.0;
  int64_t launches = 0;
  std::string err;
};

namespace cf {

/* record msg as the context's last error (the create error when c is NULL), return code */
int fail(cf_ctx* c, int code, const std::string& msg);

/* Runs the body of a C ABI entry point: a C++ exception of the host preprocessing (an allocation
 * beyond host memory for an enormous input) becomes an error code with a message, recorded on c (or
 * as the creation error when c is NULL), instead of crossing the C ABI. */
template <class F>
int abi_guard(cf_ctx* c, F&& body) {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    return fail(c, CF_ENOMEM, "host allocation failed (input too large for host memory?)");
  } catch (const std::exception& e) {
    return fail(c, CF_EINVAL, std::string("host error: ") + e.what());
  }
}
int cuda_fail(cf_ctx* c, cudaError_t e, const char* what);

#define CF_CUDA(c, call)                                     \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cf::cuda_fail((c), e_, #call); \
  } while (0)

template <class T>
int dalloc(cf_ctx* c, T** dst, size_t count) {
  size_t bytes = std::max<size_t>(1, count) * sizeof(T);
  CF_CUDA(c, cudaMalloc((void**)dst, bytes));
  CF_CUDA(c, cudaMemset(*dst, 0, bytes));
  return CF_OK;
}

template <class T>
int put(cf_ctx* c, T* dst, const T* src, size_t count) {
  if (count) CF_CUDA(c, cudaMemcpy(dst, src, count * sizeof(T), cudaMemcpyHostToDevice));
  return CF_OK;
}

StepArgs step_args(const cf_ctx* c, int parity);  /* the context's buffers for a step of this parity */
int read_states(cf_ctx* c);                        /* mst -> host_state, synchronising the stream */
int status_code(uint32_t status);                  /* CF_* code of a status word */

}  // namespace cf

#endif
