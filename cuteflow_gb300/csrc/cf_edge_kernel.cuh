/*
 * cf_edge_kernel.cuh -- the edge kernel of the step (included by one small translation unit per
 * scheme, cf_edges_<IFLUX>.cu, so that the launch shapes of the four schemes compile in parallel).
 *
 * k_edges<IFLUX, BE, EPT>: blocks of BE threads, each thread evaluating EPT edges (e, e + BE, ...
 * of its block's BE * EPT consecutive edges).  Edges keep their layout of tiles of TILE_E = 128
 * edges, each owned by one member, whatever the shape: a thread looks up its edge's member, and
 * the integer-pipe warp mask bit w applies to the edges (e mod 128) / 32 = w of a tile.  Every
 * shape evaluates the same edges with the same arithmetic, so results do not depend on it (the
 * autotuner chooses one).
 *
 * Register budget: every IFLUX 1-3 shape keeps 1024 threads per SM (at most 64 registers; with
 * spills to L1): the tuned edge is chains of dependent integer-pipe products and quotients between
 * its FP64 sums and the warps hide their latency (1M WAF, tuned, 128-thread blocks: 0.462 ms at
 * four blocks per SM, 0.434 at five, 0.421 at six, 0.408 at eight; HLLC 0.266 -> 0.215 ms).
 * MUSCL-Hancock keeps 512 threads per SM (128 registers): at 1024 its spills cost more than the
 * warps gain (1.39 ms), at 384 (138 registers) it takes 1.32 ms, at 512 1.21 ms.
 */
#ifndef CF_EDGE_KERNEL_CUH
#define CF_EDGE_KERNEL_CUH

#include <cuda_runtime.h>

#include "cf_flux.h"
#include "cf_xd.h"

namespace cf {
namespace {

/* Start of member M's step (by the thread of its first edge, or by k_begin_step): the dt sanity
 * test of cfl_condition.cuf:129-132 (a failing dt ends the run with the current state), the next
 * time, and the start value of the next dt minimum (cflcond sets dt_d = 1e6 and the block
 * reduction pads a partial last block with 1e5, cfl_condition.cuf:21,86). */
__device__ __forceinline__ void step_start(const MemberDev& M, MemberState* S, int p) {
  const double dt = S->dt[p];
  const double t = S->t[p];
  if (S->nstep > 0 && (dt > 9999.0 || dt < DT_LOW)) {   /* the initial dt is not tested (:113-116) */
    atomicOr(&S->status, CF_STATUS_DT_RANGE);
  } else if (S->nstep > 0 && !((S->tc + dt) - S->ts + 2.0 * TOL_LOOP < TOL_LOOP)) {
    /* the time loop's test (finite_volumes_method.cuf:123) on tc = tc + dt (:232); tc keeps
     * its value, so that a later cf_run adds this dt once and tests again */
    atomicOr(&S->status, CF_STATUS_END);
  } else if (S->nstep == 0 && !(S->tc - S->ts + 2.0 * TOL_LOOP < TOL_LOOP)) {
    atomicOr(&S->status, CF_STATUS_END);
  } else {
    if (S->nstep > 0) S->tc = S->tc + dt;
    S->t[1 - p] = t + dt;
    S->dt[1 - p] = M.dt_reset;
    S->nstep += 1;
  }
}

/* The edge of index e of a step (member M, state S, parity p), in the context's arithmetic type. */
template <int IFLUX>
__device__ __forceinline__ void edge_in_step(const StepArgs& a, const MemberDev& M, MemberState* S, int e, double dt,
                                             double t) {
  if (a.xd_cmp) {
    /* the same arithmetic with exact integer comparisons and, in the warps of xd_mul_mask,
     * exact integer products: the FP64 pipe and the integer pipes share the work.  The WAF edge
     * keys its comparisons on the plain bit patterns (faster there: 0.261 against 0.269 ms on the
     * 1M step), the other schemes on the opaque ones (MUSCL edge 0.585 -> 0.534 ms, first-order
     * HLLC forward ~4 % faster) */
    constexpr bool OC = IFLUX != 3;
    if ((a.xd_mul_mask >> ((e % TILE_E) >> 5)) & 1) edge_body<IFLUX, XD<true, OC>>(a, M, e, dt, t, S->surf);
    else edge_body<IFLUX, XD<false, OC>>(a, M, e, dt, t, S->surf);
  } else {
    edge_body<IFLUX>(a, M, e, dt, t, S->surf);
  }
}

template <int IFLUX, int BE, int EPT>
__global__ void __launch_bounds__(BE, ((IFLUX == 4) ? 512 : 1024) / BE) k_edges(StepArgs a) {
  const int p = a.parity;
  const int nedge = a.n_etiles * TILE_E;
#pragma unroll 1
  for (int j = 0; j < EPT; ++j) {
    const int e = (blockIdx.x * EPT + j) * BE + threadIdx.x;
    if (e >= nedge) return;
    const int m = __ldg(a.etile_mem + e / TILE_E);
    const MemberDev& M = a.mdev[m];
    MemberState* S = a.mst + m;
    if (S->status) continue;
    const double dt = S->dt[p];
    const double t = S->t[p];
    if (e == M.edge_begin) step_start(M, S, p);
    if (e >= M.edge_end) continue;
    edge_in_step<IFLUX>(a, M, S, e, dt, t);
  }
}

/* The edges of a list (a part's phase of its step): 128-thread blocks, one edge per thread; the
 * step's start is made by k_begin_step before the first phase. */
template <int IFLUX>
__global__ void __launch_bounds__(TILE_E, (IFLUX == 4) ? 4 : 8) k_edges_list(StepArgs a, const int32_t* list, int n) {
  const int i = blockIdx.x * TILE_E + threadIdx.x;
  if (i >= n) return;
  const int e = list[i];
  const int m = __ldg(a.etile_mem + e / TILE_E);
  const MemberDev& M = a.mdev[m];
  MemberState* S = a.mst + m;
  if (S->status || e >= M.edge_end) return;
  edge_in_step<IFLUX>(a, M, S, e, S->dt[a.parity], S->t[a.parity]);
}

template <int IFLUX, int BE, int EPT>
void launch_edges_shape(const StepArgs& a, cudaStream_t st) {
  const int nedge = a.n_etiles * TILE_E;
  const int per = BE * EPT;
  k_edges<IFLUX, BE, EPT><<<(nedge + per - 1) / per, BE, 0, st>>>(a);
}

}  // namespace

template <int IFLUX>
int launch_edges_list_iflux(const StepArgs& a, const int32_t* list, int32_t n, cudaStream_t st) {
  if (n <= 0) return CF_OK;
  k_edges_list<IFLUX><<<(n + TILE_E - 1) / TILE_E, TILE_E, 0, st>>>(a, list, n);
  return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ECUDA;
}

/* The shapes a context can choose (cf_set_launch_shape): BE in {64, 128, 256}, EPT in {1, 2}. */
template <int IFLUX>
int launch_edges_iflux(const StepArgs& a, cudaStream_t st) {
  const int key = a.eblock * 10 + a.ept;
  switch (key) {
    case 641: launch_edges_shape<IFLUX, 64, 1>(a, st); break;
    case 642: launch_edges_shape<IFLUX, 64, 2>(a, st); break;
    case 1281: launch_edges_shape<IFLUX, 128, 1>(a, st); break;
    case 1282: launch_edges_shape<IFLUX, 128, 2>(a, st); break;
    case 2561: launch_edges_shape<IFLUX, 256, 1>(a, st); break;
    case 2562: launch_edges_shape<IFLUX, 256, 2>(a, st); break;
    default: return CF_EINVAL;
  }
  return cudaGetLastError() == cudaSuccess ? CF_OK : CF_ECUDA;
}

}  // namespace cf

#endif
