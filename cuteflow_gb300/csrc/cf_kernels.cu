/*
 * cf_kernels.cu -- sm_103a kernels of the explicit St-Venant step.
 *
 * One step is two kernels on the context's stream:
 *
 *   k_edges : one thread per edge (cf_edge_kernel.cuh, in every launch shape).  Loads both elements' {h, hu, hv, z}, solves the Riemann
 *             problem once (wave speeds, physical and HLL fluxes), and writes into the edge's
 *             two slots the flux each side computes for itself in the reference
 *             (flux_riemann.cuf:33-426 evaluates every interior edge from both elements).
 *             The two evaluations share everything but a few branch decisions and, for WAF,
 *             the limiter ratios; those are re-evaluated for the second side from exact
 *             mirror identities, so the result is the reference's two-sided flux at about
 *             the cost of one evaluation.  flux_mode 1 writes the negated A-side flux to side
 *             B instead (exactly conservative).  The bed-slope source of each side
 *             (source_terms.cuf:54-100) is computed here as well.
 *   k_cells : one thread per element.  Gathers its three slots in the reference's edge order,
 *             applies Manning friction with the semi-implicit (I - dt/2 J)^-1 matrix
 *             (source_terms.cuf:102-210), updates with the wet/dry clamp
 *             (finite_volumes_method.cuf:283-303), and evaluates the CFL time step of the new
 *             state (cfl_condition.cuf:20-37); a warp-shuffle + block minimum per tile folds
 *             it into the member's next dt with one ordered-integer atomicMin.
 *
 * Everything is FP64.  The step is bound by the FP64 pipe (GB300: 2 DFMA/clk/SM), not by
 * HBM, so the code spends FP64 instructions carefully: geometry is precomputed, divisions
 * that share a denominator become one reciprocal, and sign tests are integer tests.
 */
#include <cuda_runtime.h>

#include <cstdio>

#include "cf_edge_kernel.cuh"
#include "cf_flux.h"
#include "cf_xd.h"

namespace cf {
namespace {

/* phys_inflow: per member (one warp) and inlet, calcul_surf_entree (maillage.cuf:1368-1421)
 * on the state at the step's start: the entries' length * depth in blocks of 32 in list
 * order, each block summed by the reference's tree (s(t) += s(t + i), i = 16 .. 1), the
 * block sums added in block order (the reference adds them with atomicAdd, in whatever order
 * the blocks finish; entries past the end of the list count 0, where the reference reads
 * beyond its list). */
__global__ void __launch_bounds__(32) k_surf(StepArgs a) {
  const int m = blockIdx.x;
  const MemberDev& M = a.mdev[m];
  MemberState* S = a.mst + m;
  if (M.inlet != 3 || S->status) return;
  const int lane = threadIdx.x;
  for (int id = 0; id < M.nin; ++id) {
    double total = 0.0;
    for (int b = 0; b < M.inl_count; b += 32) {
      const int j = b + lane;
      double v = 0.0;
      if (j < M.inl_count)
        v = a.inl_len[M.inl_len_off + (size_t)j * M.nin + id] * a.Uin[a.inl_cell[M.inl_begin + j]].x;
      #pragma unroll
      for (int i = 16; i > 0; i >>= 1) v = v + __shfl_down_sync(0xffffffffu, v, i);
      total = total + v;   /* lane 0 holds the block's tree sum */
    }
    if (lane == 0) S->surf[id] = total;
  }
}

/* ---- the element kernel ----------------------------------------------------------------- */

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }

__device__ __forceinline__ Slot load_slot(const Slot* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
  Slot s;
  s.f1 = a.x; s.f2 = a.y; s.f3 = b.x; s.bx = b.y; s.by = c.x; s.q = c.y;
  return s;
}

/* Minimum over the block, folded into *target with one atomic.  The values are positive (or
 * NaN, which the minimum ignores as fmin would), so they order like their bit patterns: the
 * reduction is integer work. */
template <int BC>
__device__ __forceinline__ void block_min_atomic(double v, double* target) {
  __shared__ unsigned long long red[BC / 32];
  unsigned long long b = dbits(v);
  #pragma unroll
  for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = b;
  __syncthreads();
  if (wid == 0) {
    b = (lane < BC / 32) ? red[lane] : dbits(1.0e300);
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_xor_sync(0xffffffffu, b, o));
    if (lane == 0) atomicMin(reinterpret_cast<unsigned long long*>(target), b);
  }
}

/* Minimum over the block of a float, returned to every thread. */
template <int BC>
__device__ __forceinline__ float block_min_f32(float v) {
  __shared__ float red[BC / 32];
  #pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  v = red[0];
  #pragma unroll
  for (int w = 1; w < BC / 32; ++w) v = fminf(v, red[w]);
  return v;
}

/* x truncated to float by integer operations (relative error below 2^-23); false when x is
 * outside float's normal range, infinite or NaN.  Zero converts exactly. */
__device__ __forceinline__ bool f32_trunc(double x, float& f) {
  const unsigned long long b = dbits(x);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  if (zero_u(b)) {
    f = __uint_as_float(sign);
    return true;
  }
  const int e = (int)((b >> 52) & 0x7ff) - 1023;
  if (e < -126 || e > 127) return false;
  f = __uint_as_float(sign | ((unsigned)(e + 127) << 23) | (unsigned)((b >> 29) & 0x7fffffu));
  return true;
}

/* cfl_dt_elem of a wet element (h > tolisec) in single precision: the inputs truncated to float,
 * every operation correctly rounded.  Relative to the FP64 value it is within
 *   2^-23 (truncation of hu or hv, and of h) x 2 + 2^-24 for u = hu/h; twice that + 2^-24 for u^2;
 *   + 2^-24 for the sum of squares (positive terms); half of it + 2^-24 for the root;
 *   below that for sqrt(g h); + 2^-24 for the sum; 2^-23 (cfl L) + 2^-24 for the last quotient
 * = 7e-7 (the max with 0.01 and the min with 1e6 are monotone and add nothing; the FP64 value's
 * own rounding is ~1e-15).  Returns false (the caller takes the FP64 value) where an input is out
 * of float's range or the result is not in (1e-30, 1e6]. */
__device__ __forceinline__ bool cfl_dt_f32(const MemberDev& M, double cflL, double h, double hu, double hv,
                                           float& d) {
  float hf, huf, hvf, lf, gf;
  if (!(f32_trunc(h, hf) & f32_trunc(hu, huf) & f32_trunc(hv, hvf) & f32_trunc(cflL, lf) & f32_trunc(M.gp, gf)))
    return false;
  const float vu = __fdiv_rn(huf, hf), vv = __fdiv_rn(hvf, hf);
  const float nv = __fsqrt_rn(__fadd_rn(__fmul_rn(vu, vu), __fmul_rn(vv, vv)));
  const float c = __fsqrt_rn(__fmul_rn(gf, hf));
  const float vmax = fmaxf(0.01f, __fadd_rn(nv, c));
  d = fminf(__fdiv_rn(lf, vmax), 1.0e6f);
  return d > 1.0e-30f && d <= 1.0e6f;
}

/* The minimum of cfl_dt_elem over the block's elements with the FP64 evaluation only where it
 * can be the minimum.  RN is monotone, so the block minimum of the FP64 values is the FP64 value
 * of an element whose single-precision value lies within the error bound of the block's
 * single-precision minimum: m_f >= (1 - 7e-7) d_min and d_f(argmin) <= (1 + 7e-7) d_min, so the
 * element of the minimum passes d_f <= 1.000004 m_f.  Elements without a single-precision value
 * (dry ones, constant dt, out-of-range inputs) take their FP64 value directly. */
template <int BC>
__device__ __forceinline__ void block_cfl_min(const MemberDev& M, bool active, double cflL, const double4& V,
                                              double* target) {
  double dti = 1.0e300;
  float df = __int_as_float(0x7f800000);
  bool pending = false;
  if (active) {
    if (M.is_dt_constant == 1 || !(V.x > M.tolisec)) dti = cfl_dt_elem(M, cflL, V.x, V.y, V.z, V.w);
    else if (cfl_dt_f32(M, cflL, V.x, V.y, V.z, df)) pending = true;
    else dti = cfl_dt_elem(M, cflL, V.x, V.y, V.z, V.w);
  }
  const float mf = block_min_f32<BC>(df);
  if (pending && df <= mf * 1.000004f) dti = cfl_dt_elem(M, cflL, V.x, V.y, V.z, V.w);
  block_min_atomic<BC>(dti, target);
}

/* 1024 threads per SM (at most 64 registers; 116 bytes spilled): the element update is a chain of
 * dependent integer-pipe quotients and products, and since the dry-region shortcuts most of the
 * kernel's time is memory latency, which more warps hide (1M WAF step, tuned, 256-thread blocks:
 * 0.152 -> 0.130 ms from two to three blocks per SM before the shortcuts; 0.088 -> 0.082 ms from
 * three to four after them).  A block of BC threads (128 or 256, the launch shape) lies within one
 * tile of TILE_C elements, so within one member; each block folds its dt minimum into the member's
 * with one atomic.  SUMS (the recording forward) also stores the element's slot sums; it is a
 * separate instantiation because the compiler shares those sums with the general update's and then
 * forms them ahead of the dry-element test, for every element (1M WAF step: 9 -> 19 FP64 sums per
 * element, 0.088 -> 0.098 ms). */
template <int BC, bool SUMS>
__global__ void __launch_bounds__(BC, 1024 / BC) k_cells(StepArgs a) {
  const int c0 = a.c_lo + blockIdx.x * BC;   /* the block's first element (c_lo: a part's phase) */
  const int tile = c0 / TILE_C;
  const int m = __ldg(a.ctile_mem + tile);
  const MemberDev& M = a.mdev[m];
  MemberState* S = a.mst + m;
  const int p = a.parity;
  /* the stop test must be uniform over the block (the dt reduction below synchronises it) */
  __shared__ uint32_t s_stop;
  if (threadIdx.x == 0) s_stop = *((volatile uint32_t*)&S->status);
  __syncthreads();
  if (s_stop) return;
  const double dt = S->dt[p];
  const int c = c0 + threadIdx.x;
  const int cend = min(M.cell_end, a.c_hi);
  double4 V = make_double4(0.0, 0.0, 0.0, 0.0);
  double cflL = 0.0;
  if (c < cend) {
    const double4 U = ld4(a.Uin + c);
    /* a dry element amid dry ones (most of an unflooded plain): its slots are signed zeros and
     * its update is +0, known from four depths and its neighbour entry, without its slots or its
     * statics (a dry element's CFL value does not use its length) */
    bool dry = false;
    if (!SUMS) {
      const int4 nb = __ldg(a.cnbr + c);
      dry = dry_state_ok(M, U, dt) &&
            dry_neighbourhood(M, nb, U, [&](int k) { return ldro(reinterpret_cast<const double*>(a.Uin + k)); });
    }
    if (!dry) {
      const double4 st = ld4(a.cstat + c);   /* area, manning n, cfl L, - */
      const int4 sl = __ldg(a.cslot + c);
      const Slot s0 = load_slot(a.slots + sl.x);
      const Slot s1 = load_slot(a.slots + sl.y);
      const Slot s2 = load_slot(a.slots + sl.z);
      if (SUMS) {
        /* the sums element_update forms (same expressions, same values) */
        double2* q = reinterpret_cast<double2*>(a.sums_out + c);
        q[0] = make_double2(s0.f1 + s1.f1 + s2.f1, s0.f2 + s1.f2 + s2.f2);
        q[1] = make_double2(s0.f3 + s1.f3 + s2.f3, s0.bx + s1.bx + s2.bx);
        q[2] = make_double2(s0.by + s1.by + s2.by, 0.0);
      }
      bool nonfinite = false;
      /* bit 4 of xd_mul_mask: the element's arithmetic on the integer pipes (cf_xd.h) */
      if (a.xd_cmp && (a.xd_mul_mask & XD_CELLS)) V = element_update<XD<true>>(M, U, st, s0, s1, s2, dt, nonfinite);
      else V = element_update(M, U, st, s0, s1, s2, dt, nonfinite);
      if (nonfinite) atomicOr(&S->status, CF_STATUS_NONFINITE);
      cflL = st.z;
    }
    double4* o = a.Uout + c;
    reinterpret_cast<double2*>(o)[0] = make_double2(V.x, V.y);
    reinterpret_cast<double2*>(o)[1] = make_double2(V.z, V.w);
  }
  block_cfl_min<BC>(M, c < cend, cflL, V, &S->dt[1 - p]);
}

/* CFL of a state into mst[m].dt[slot] (the initial dt, finite_volumes_method.cuf:113-116). */
__global__ void __launch_bounds__(TILE_C) k_cfl(const double4* U, const double4* cstat, const int32_t* ctile_mem,
                                                int tile_begin, const MemberDev* mdev, MemberState* mst, int slot) {
  const int tile = tile_begin + blockIdx.x;
  const int m = __ldg(ctile_mem + tile);
  const MemberDev& M = mdev[m];
  const int c = tile * TILE_C + threadIdx.x;
  double4 u = make_double4(0.0, 0.0, 0.0, 0.0);
  double cflL = 0.0;
  if (c < M.cell_end) {
    u = ld4(U + c);
    cflL = ld4(cstat + c).z;
  }
  block_cfl_min<TILE_C>(M, c < M.cell_end, cflL, u, &mst[m].dt[slot]);
}

/* Discharge diagnostics of the last step (debit_entree_sum, debit_sortie,
 * finite_volumes_method.cuf:197-214): per member, fixed-order sums over its boundary edges
 * (deterministic: each thread sums a fixed stride of the reference-order list, then a fixed tree).  With steady set (the
 * launch at the end of every step of a context that tests for steady state) it also applies
 * check_steady_state (finite_volumes_method.cuf:370-393) to the members that stepped:
 * Q_in > 1e-8 (single precision) and |Q_in - Q_out| / Q_in < tol_reg_perm counts a step, any
 * other step resets the count, and more than steady_count stops the member. */
__global__ void __launch_bounds__(256) k_discharge(const Slot* slots, const int2* ecell, const int32_t* bq,
                                                    const MemberDev* mdev, MemberState* mst, int steady) {
  __shared__ double si[256], so[256];
  const int m = blockIdx.x;
  const MemberDev& M = mdev[m];
  double qi = 0.0, qo = 0.0;
  /* the boundary edges in reference order (element, local edge): thread t sums entries t, t + 256,
   * ..., then a fixed tree, an order a decomposed mesh reproduces from its parts' entries */
  for (int j = threadIdx.x; j < M.bq_count; j += 256) {
    const int e = bq[M.bq_begin + j];
    const int kind = ecell[e].y;
    const double q = slots[2 * (size_t)e].q;
    if (kind == -1) qi += q;
    else if (kind == -2) qo += q;
  }
  si[threadIdx.x] = qi;
  so[threadIdx.x] = qo;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      si[threadIdx.x] += si[threadIdx.x + w];
      so[threadIdx.x] += so[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    MemberState* S = mst + m;
    S->q_in = si[0];
    S->q_out = so[0];
    if (steady && M.tol_reg_perm > 0.0 && S->status == 0) {
      const double qi = si[0], qo = so[0];
      if (qi > (double)1e-8f && fabs(qi - qo) / qi < M.tol_reg_perm) {
        S->steady_iter += 1;
        if (S->steady_iter > M.steady_count) S->status |= CF_STATUS_STEADY;
      } else {
        S->steady_iter = 0;
      }
    }
  }
}

__global__ void k_scatter(const double* hu3, const int32_t* perm, const double* zcell, double4* U, int n) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int o = perm[c];
  const double h = hu3[3 * (size_t)o];
  U[c] = make_double4(h, hu3[3 * (size_t)o + 1], hu3[3 * (size_t)o + 2], h > 0.0 ? 1.0 / h : 0.0);
}

__global__ void k_gather(const double4* U, const int32_t* iperm, double* hu3, int n) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n) return;
  const double4 u = U[iperm[o]];
  hu3[3 * (size_t)o] = u.x;
  hu3[3 * (size_t)o + 1] = u.y;
  hu3[3 * (size_t)o + 2] = u.z;
}

/* The same, out of the buffer that holds member m's current state, chosen on the device from its
 * record (U[(base + nstep) & 1]): correct after steps whose count the host has not read back. */
__global__ void k_gather_current(const double4* U0, const double4* U1, const MemberState* mst, int m,
                                 const int32_t* iperm, double* hu3, int n) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n) return;
  const MemberState& s = mst[m];
  const double4* U = ((s.base + s.nstep) & 1) ? U1 : U0;
  const double4 u = U[iperm[o]];
  hu3[3 * (size_t)o] = u.x;
  hu3[3 * (size_t)o + 1] = u.y;
  hu3[3 * (size_t)o + 2] = u.z;
}

/* The state of one member between a caller's buffer in reference order, hu3[3 n], and U (new
 * order), where hu3 is any address the GPU can reach: device memory or pinned host memory, which
 * GB300 reads and writes over its coherent CPU link, so that no separate copy pass is needed.  A
 * block moves 256 elements = 768 consecutive doubles of hu3 with fully coalesced loads or stores
 * (one double per thread and instruction, three instructions) through shared memory; the element
 * side is U[iperm[o]].  The store form takes its buffer from member m's record when mst is given
 * (U[(base + nstep) & 1], as k_gather_current). */
constexpr int REF_BLOCK = 256;

__global__ void __launch_bounds__(REF_BLOCK) k_load_ref(const double* __restrict__ hu3, const int32_t* iperm,
                                                        double4* U, int n, const double4* cstat,
                                                        const MemberDev* mdev, MemberState* mst, int m, int slot) {
  __shared__ double s[3 * REF_BLOCK];
  const long long base = (long long)blockIdx.x * REF_BLOCK;
  const long long nd = 3 * (long long)min(REF_BLOCK, (int)(n - base));
  const double* src = hu3 + 3 * base;
  #pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int j = threadIdx.x + k * REF_BLOCK;
    if (j < nd) s[j] = src[j];
  }
  __syncthreads();
  const long long o = base + threadIdx.x;
  const bool active = o < n;
  double4 V = make_double4(0.0, 0.0, 0.0, 0.0);
  double cflL = 0.0;
  if (active) {
    const double h = s[3 * threadIdx.x], hu = s[3 * threadIdx.x + 1], hv = s[3 * threadIdx.x + 2];
    const int c = iperm[o];
    V = make_double4(h, hu, hv, h > 0.0 ? 1.0 / h : 0.0);
    double4* u = U + c;
    reinterpret_cast<double2*>(u)[0] = make_double2(V.x, V.y);
    reinterpret_cast<double2*>(u)[1] = make_double2(V.z, V.w);
    if (mst) cflL = ld4(cstat + c).z;
  }
  /* with mst: the initial dt of the state (k_cfl's minimum), folded into mst[m].dt[slot] */
  if (mst) block_cfl_min<REF_BLOCK>(mdev[m], active, cflL, V, &mst[m].dt[slot]);
}

__global__ void __launch_bounds__(REF_BLOCK) k_store_ref(const double4* U0, const double4* U1, const MemberState* mst,
                                                         int m, const int32_t* iperm, double* __restrict__ hu3, int n) {
  __shared__ double s[3 * REF_BLOCK];
  const double4* U = U0;
  if (mst) {
    const MemberState& st = mst[m];
    U = ((st.base + st.nstep) & 1) ? U1 : U0;
  }
  const long long base = (long long)blockIdx.x * REF_BLOCK;
  const long long o = base + threadIdx.x;
  if (o < n) {
    const double2 a = __ldg(reinterpret_cast<const double2*>(U + iperm[o]));
    const double b = __ldg(reinterpret_cast<const double*>(U + iperm[o]) + 2);
    s[3 * threadIdx.x] = a.x;
    s[3 * threadIdx.x + 1] = a.y;
    s[3 * threadIdx.x + 2] = b;
  }
  __syncthreads();
  const long long nd = 3 * (long long)min(REF_BLOCK, (int)(n - base));
  double* dst = hu3 + 3 * base;
  #pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int j = threadIdx.x + k * REF_BLOCK;
    if (j < nd) dst[j] = s[j];
  }
}

/* (h, hu, hv) of the listed elements (member-local reference ids) out of / into U */
__global__ void k_gather_ids(const double4* U, const int32_t* iperm, const int32_t* ids, double* out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4 u = U[iperm[ids[i]]];
  out[3 * (size_t)i] = u.x;
  out[3 * (size_t)i + 1] = u.y;
  out[3 * (size_t)i + 2] = u.z;
}

__global__ void k_scatter_ids(double4* U, const int32_t* iperm, const int32_t* ids, const double* in, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4* u = U + iperm[ids[i]];
  const double h = in[3 * (size_t)i];
  reinterpret_cast<double2*>(u)[0] = make_double2(h, in[3 * (size_t)i + 1]);
  reinterpret_cast<double2*>(u)[1] = make_double2(in[3 * (size_t)i + 2], h > 0.0 ? 1.0 / h : 0.0);
}

/* Throughput probe of the FP64 pipe: eight independent FMA chains per thread, x <- x a + b with
 * a = 1 - 2^-20 and b = 2^-20, so every value stays a normal number near 1. */
__global__ void __launch_bounds__(256) k_probe_fp64(double* out, long long iters) {
  const double a = 1.0 - 0x1p-20, b = 0x1p-20;
  double x[8];
  #pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = 0.5 + 0.01 * k + 1e-6 * threadIdx.x;
  for (long long i = 0; i < iters; ++i) {
    #pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double sum = 0.0;
  #pragma unroll
  for (int k = 0; k < 8; ++k) sum += x[k];
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = sum;
}

/* ---- a part of a decomposed mesh ------------------------------------------------------- */

/* The start of every member's step (step_start), made once before a part's phased step. */
__global__ void k_begin_step(StepArgs a) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= a.nmembers) return;
  MemberState* S = a.mst + m;
  if (S->status) return;
  step_start(a.mdev[m], S, a.parity);
}

/* (h, hu, hv) of the listed elements (device order) into buf[3 i ..], and back (with RN(1/h));
 * buf may be pinned host memory (read and written over the CPU link). */
__global__ void k_pack(const double4* U, const int32_t* ids, int n, double* buf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double4 u = U[ids[i]];
  buf[3 * (size_t)i] = u.x;
  buf[3 * (size_t)i + 1] = u.y;
  buf[3 * (size_t)i + 2] = u.z;
}

__global__ void k_unpack(double4* U, const int32_t* ids, int n, const double* buf) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double h = buf[3 * (size_t)i];
  double4* u = U + ids[i];
  reinterpret_cast<double2*>(u)[0] = make_double2(h, buf[3 * (size_t)i + 1]);
  reinterpret_cast<double2*>(u)[1] = make_double2(buf[3 * (size_t)i + 2], h > 0.0 ? 1.0 / h : 0.0);
}

/* Member 0's phys_inflow terms of the state U: for every entry j of its inlet list (reference
 * order) and inlet id, the length * depth that calcul_surf_entree sums, out[j * nin + id]. */
__global__ void k_inlet_terms(StepArgs a, const double4* U, double* out) {
  const MemberDev& M = a.mdev[0];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M.inl_count) return;
  const double h = U[a.inl_cell[M.inl_begin + j]].x;
  for (int id = 0; id < M.nin; ++id)
    out[(size_t)j * M.nin + id] = a.inl_len[M.inl_len_off + (size_t)j * M.nin + id] * h;
}

/* Member 0's boundary discharges of the last step, in the reference order of its boundary edges. */
__global__ void k_bq_terms(const Slot* slots, const int32_t* bq, const MemberDev* mdev, double* out) {
  const MemberDev& M = mdev[0];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= M.bq_count) return;
  out[j] = slots[2 * (size_t)bq[M.bq_begin + j]].q;
}

/* The discharge diagnostics and the steady-state test (check_steady_state,
 * finite_volumes_method.cuf:370-393) of member 0 with the whole mesh's discharges. */
__global__ void k_steady_apply(const MemberDev* mdev, MemberState* mst, double qi, double qo) {
  const MemberDev& M = mdev[0];
  MemberState* S = mst;
  S->q_in = qi;
  S->q_out = qo;
  if (M.tol_reg_perm > 0.0 && S->status == 0) {
    if (qi > (double)1e-8f && fabs(qi - qo) / qi < M.tol_reg_perm) {
      S->steady_iter += 1;
      if (S->steady_iter > M.steady_count) S->status |= CF_STATUS_STEADY;
    } else {
      S->steady_iter = 0;
    }
  }
}

/* Self-test of the integer-pipe arithmetic of cf_xd.h against the FP64 unit.  Pair i comes from
 * a splitmix64 sequence: exponents over the whole range or near the step's values, all-ones and
 * near-all-ones significands, signed zeros, subnormals, infinities, NaN, and quotients and roots
 * within a few units of a rounding midpoint.  Counts the results of em_mul, em_div,
 * em_sqrt, the exponent-change scalings, negation and the integer comparisons whose bits differ
 * from the hardware's (two NaNs count as equal). */
__device__ unsigned long long st_next(unsigned long long& s) {
  s += 0x9e3779b97f4a7c15ull;
  unsigned long long z = s;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ double st_operand(unsigned long long& s, int emin, int emax) {
  unsigned long long m = st_next(s) & ((1ull << 52) - 1);
  const unsigned long long r = st_next(s);
  const int mode = (int)(r & 7u);
  if (mode == 0) m = (1ull << 52) - 1;
  if (mode == 1) m = 0;
  if (mode == 2) m = (r >> 8) & 15u;
  if (mode == 3) m = ((1ull << 52) - 1) ^ ((r >> 8) & 15u);
  const unsigned long long e = (unsigned long long)emin + (r >> 16) % (unsigned long long)(emax - emin + 1);
  return xdbl(((r >> 63) << 63) | (e << 52) | m);
}
__device__ bool st_same(double x, double y) { return xbits(x) == xbits(y) || (x != x && y != y); }

__global__ void __launch_bounds__(256) k_selftest_xd(long long n, unsigned long long seed,
                                                     unsigned long long* bad) {
  unsigned long long nbad = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    unsigned long long s = seed ^ ((unsigned long long)i * 0xd1342543de82ef95ull);
    const int mode = (int)(st_next(s) % 8u);
    double a, b;
    if (mode == 0) { a = st_operand(s, 1, 2046); b = st_operand(s, 1, 2046); }
    else if (mode == 1) { a = st_operand(s, 0, 2047); b = st_operand(s, 0, 2047); }
    else if (mode == 2) { a = st_operand(s, 1000, 1050); b = st_operand(s, 1000, 1050); }
    else if (mode == 3) { a = st_operand(s, 1, 30); b = st_operand(s, 990, 1030); }
    else if (mode == 4) { a = st_operand(s, 2000, 2046); b = st_operand(s, 1000, 1100); }
    else if (mode == 5) { a = (st_next(s) & 1) ? -0.0 : 0.0; b = st_operand(s, 0, 2047); }
    else if (mode == 6) { a = st_operand(s, 0, 2047); b = (st_next(s) & 1) ? -0.0 : 0.0; }
    else {
      /* a / b close to a rounding midpoint: A = RN((2N+1) B / 2^sh), moved by up to two units */
      const unsigned long long N = (1ull << 52) | (st_next(s) & ((1ull << 52) - 1));
      const unsigned long long B = (1ull << 52) | (st_next(s) & ((1ull << 52) - 1));
      const unsigned long long u = 2 * N + 1;
      const unsigned long long lo = u * B, hi = __umul64hi(u, B);  /* (2N+1) B = hi 2^64 + lo */
      const int sh = ((hi >> 42) != 0 || (st_next(s) & 1)) ? 54 : 53;
      const unsigned long long half = 1ull << (sh - 1);
      const unsigned long long lo2 = lo + half, hi2 = hi + (lo2 < lo ? 1u : 0u);
      unsigned long long A = (hi2 << (64 - sh)) | (lo2 >> sh);
      A += st_next(s) % 5u;
      A -= 2;
      if (A >= (1ull << 53)) A = (1ull << 53) - 1;
      if (A < (1ull << 52)) A = 1ull << 52;
      const unsigned long long r = st_next(s);
      a = xdbl(((r >> 63) << 63) | ((1000ull + (r >> 8) % 40u) << 52) | (A & ((1ull << 52) - 1)));
      b = xdbl((((r >> 62) & 1) << 63) | ((1000ull + (r >> 20) % 40u) << 52) | (B & ((1ull << 52) - 1)));
    }
    if (mode == 4 && (st_next(s) & 1)) {
      /* sqrt(a) close to a rounding midpoint: the significand of RN((N + 1/2)^2 / 2^(52 + p)),
       * moved by up to two units, with an exponent of parity p */
      const unsigned long long N = (1ull << 52) | (st_next(s) & ((1ull << 52) - 1));
      const unsigned long long u = 2 * N + 1;
      const unsigned long long lo = u * u, hi = __umul64hi(u, u);  /* (2N+1)^2 = hi 2^64 + lo */
      const int sh = (hi >> 43) ? 55 : 54;
      const unsigned long long half = 1ull << (sh - 1);
      const unsigned long long lo2 = lo + half, hi2 = hi + (lo2 < lo ? 1u : 0u);
      unsigned long long A = (hi2 << (64 - sh)) | (lo2 >> sh);
      A += st_next(s) % 5u;
      A -= 2;
      if (A >= (1ull << 53)) A = (1ull << 53) - 1;
      if (A < (1ull << 52)) A = 1ull << 52;
      const unsigned long long ex = 1001ull + 2 * (st_next(s) % 20u) - (sh == 55 ? 1u : 0u);
      a = xdbl((ex << 52) | (A & ((1ull << 52) - 1)));
    }
    nbad += !st_same(em_sqrt(a), sqrt(a));
    if (st_next(s) & 1) { const double t = a; a = b; b = t; }
    nbad += !st_same(em_mul(a, b), a * b);
    nbad += !st_same(em_div(a, b), a / b);
    nbad += !st_same(xscale<-2>(a), a * 0.25) + !st_same(xscale<-1>(a), a * 0.5) + !st_same(xscale<1>(a), a * 2.0);
    nbad += !st_same(val(-XD<true>(a)), -a);
    /* the key comparisons on opaque and on plain bit patterns */
    nbad += (xlt(a, b) != (a < b)) + (xle(a, b) != (a <= b)) + (xeq(a, b) != (a == b));
    nbad += (xlt<false>(a, b) != (a < b)) + (xle<false>(a, b) != (a <= b)) + (xeq<false>(a, b) != (a == b));
  }
  if (nbad) atomicAdd(bad, nbad);
}

int check(cudaError_t e) { return e == cudaSuccess ? CF_OK : CF_ECUDA; }

}  // namespace

int launch_selftest_xd(int64_t n, uint64_t seed, unsigned long long* bad, int32_t nblocks, stream_t s) {
  k_selftest_xd<<<nblocks, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>((long long)n, (unsigned long long)seed, bad);
  return check(cudaGetLastError());
}

int launch_probe_fp64(double* out, int32_t nblocks, int64_t iters, stream_t s) {
  k_probe_fp64<<<nblocks, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(out, (long long)iters);
  return check(cudaGetLastError());
}

int launch_step(const StepArgs& a, stream_t s, void* ev_mid, void* ev_end) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
  if (a.phys_inflow) k_surf<<<a.nmembers, 32, 0, st>>>(a);
  int rc;
  switch (a.iflux) {
    case 1: rc = launch_edges_1(a, s); break;
    case 2: rc = launch_edges_2(a, s); break;
    case 3: rc = launch_edges_3(a, s); break;
    case 4: rc = launch_edges_4(a, s); break;
    default: return CF_ENOTSUP;
  }
  if (rc != CF_OK) return rc;
  if (ev_mid) cudaEventRecord(reinterpret_cast<cudaEvent_t>(ev_mid), st);
  if (a.sums_out) k_cells<TILE_C, true><<<a.n_ctiles, TILE_C, 0, st>>>(a);
  else if (a.cblock == 128) k_cells<128, false><<<a.n_ctiles * (TILE_C / 128), 128, 0, st>>>(a);
  else k_cells<TILE_C, false><<<a.n_ctiles, TILE_C, 0, st>>>(a);
  if (a.steady) k_discharge<<<a.nmembers, 256, 0, st>>>(a.slots, a.ecell, a.bq, a.mdev, a.mst, 1);
  if (ev_end) cudaEventRecord(reinterpret_cast<cudaEvent_t>(ev_end), st);
  return check(cudaGetLastError());
}

int launch_cfl(const double4* U, const double4* cstat, const int32_t* ctile_mem, int32_t tile_begin,
               int32_t n_tiles, const MemberDev* mdev, MemberState* mst, int32_t slot, stream_t s) {
  if (n_tiles <= 0) return CF_OK;
  k_cfl<<<n_tiles, TILE_C, 0, reinterpret_cast<cudaStream_t>(s)>>>(U, cstat, ctile_mem, tile_begin, mdev, mst, slot);
  return check(cudaGetLastError());
}

int launch_discharge(const Slot* slots, const int2* ecell, const int32_t* bq, const MemberDev* mdev, MemberState* mst,
                     int32_t nmembers, stream_t s) {
  k_discharge<<<nmembers, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(slots, ecell, bq, mdev, mst, 0);
  return check(cudaGetLastError());
}

int launch_scatter_state(const double* hu3, const int32_t* perm, const double* zcell, double4* U, int32_t n, stream_t s) {
  k_scatter<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(hu3, perm, zcell, U, n);
  return check(cudaGetLastError());
}

int launch_gather_ids(const double4* U, const int32_t* iperm, const int32_t* ids, double* out, int32_t n, stream_t s) {
  if (n <= 0) return CF_OK;
  k_gather_ids<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(U, iperm, ids, out, n);
  return check(cudaGetLastError());
}

int launch_scatter_ids(double4* U, const int32_t* iperm, const int32_t* ids, const double* in, int32_t n, stream_t s) {
  if (n <= 0) return CF_OK;
  k_scatter_ids<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(U, iperm, ids, in, n);
  return check(cudaGetLastError());
}

int launch_gather_current(const double4* U0, const double4* U1, const MemberState* mst, int32_t m,
                          const int32_t* iperm, double* hu3, int32_t n, stream_t s) {
  k_gather_current<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(U0, U1, mst, m, iperm, hu3, n);
  return check(cudaGetLastError());
}

int launch_part_phase(const StepArgs& a, int phase, const int32_t* elist, int32_t nel, int32_t c_lo, int32_t c_hi,
                      stream_t s) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
  if (phase == 1) k_begin_step<<<(a.nmembers + 31) / 32, 32, 0, st>>>(a);
  int rc = CF_OK;
  switch (a.iflux) {
    case 1: rc = launch_edges_list_1(a, elist, nel, s); break;
    case 2: rc = launch_edges_list_2(a, elist, nel, s); break;
    case 3: rc = launch_edges_list_3(a, elist, nel, s); break;
    case 4: rc = launch_edges_list_4(a, elist, nel, s); break;
    default: return CF_ENOTSUP;
  }
  if (rc != CF_OK) return rc;
  if (c_hi > c_lo) {
    StepArgs b = a;
    b.c_lo = c_lo;
    b.c_hi = c_hi;
    const int nb = (c_hi - c_lo + TILE_C - 1) / TILE_C;
    if (b.sums_out) k_cells<TILE_C, true><<<nb, TILE_C, 0, st>>>(b);
    else k_cells<TILE_C, false><<<nb, TILE_C, 0, st>>>(b);
  }
  return check(cudaGetLastError());
}

int launch_pack(const double4* U, const int32_t* ids, int32_t n, double* buf, stream_t s) {
  if (n <= 0) return CF_OK;
  k_pack<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(U, ids, n, buf);
  return check(cudaGetLastError());
}

int launch_unpack(double4* U, const int32_t* ids, int32_t n, const double* buf, stream_t s) {
  if (n <= 0) return CF_OK;
  k_unpack<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(U, ids, n, buf);
  return check(cudaGetLastError());
}

int launch_inlet_terms(const StepArgs& a, const double4* U, int32_t count, double* out, stream_t s) {
  if (count <= 0) return CF_OK;
  k_inlet_terms<<<(count + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(a, U, out);
  return check(cudaGetLastError());
}

int launch_bq_terms(const Slot* slots, const int32_t* bq, const MemberDev* mdev, int32_t count, double* out, stream_t s) {
  if (count <= 0) return CF_OK;
  k_bq_terms<<<(count + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(slots, bq, mdev, out);
  return check(cudaGetLastError());
}

int launch_steady_apply(const MemberDev* mdev, MemberState* mst, double qi, double qo, stream_t s) {
  k_steady_apply<<<1, 1, 0, reinterpret_cast<cudaStream_t>(s)>>>(mdev, mst, qi, qo);
  return check(cudaGetLastError());
}

int launch_load_ref(const double* hu3, const int32_t* iperm, double4* U, int32_t n, stream_t s, const double4* cstat,
                    const MemberDev* mdev, MemberState* mst, int32_t m, int32_t slot) {
  if (n <= 0) return CF_OK;
  k_load_ref<<<(n + REF_BLOCK - 1) / REF_BLOCK, REF_BLOCK, 0, reinterpret_cast<cudaStream_t>(s)>>>(
      hu3, iperm, U, n, cstat, mdev, mst, m, slot);
  return check(cudaGetLastError());
}

int launch_store_ref(const double4* U0, const double4* U1, const MemberState* mst, int32_t m, const int32_t* iperm,
                     double* hu3, int32_t n, stream_t s) {
  if (n <= 0) return CF_OK;
  k_store_ref<<<(n + REF_BLOCK - 1) / REF_BLOCK, REF_BLOCK, 0, reinterpret_cast<cudaStream_t>(s)>>>(
      U0, U1, mst, m, iperm, hu3, n);
  return check(cudaGetLastError());
}

int launch_gather_state(const double4* U, const int32_t* iperm, double* hu3, int32_t n, stream_t s) {
  k_gather<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(U, iperm, hu3, n);
  return check(cudaGetLastError());
}

}  // namespace cf
