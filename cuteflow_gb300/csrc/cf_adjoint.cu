/*
 * cf_adjoint.cu -- sm_103a kernels of the discrete adjoint of the step (dt of every step frozen).
 *
 * The step maps U^n to U^{n+1} in two stages: every edge computes the slot values of its two
 * sides (flux * len and bed source) from the states of its elements (and, second order, of
 * their upwind elements); every element then combines its state, the sums of its three slots
 * and its Manning n.  The adjoint runs the stages backwards:
 *
 *   k_adj_cells  : per element, lambda^{n+1} gathered (its own part of the previous reverse
 *                  step, the contributions of its three edge slots and of the edges it is
 *                  an upwind element of, the objective's weights on its gauges; fixed order,
 *                  no atomics), then the transposed local Jacobian of the element stage
 *                  applied to it: its own part of lambda^n, the adjoint of its flux and bed
 *                  sums (cadj) and dJ/dn += .. ,
 *   k_adj_edges  : per edge, the transposed Jacobian of the edge stage applied to the cadj of
 *                  its two elements: one contribution per side (and per upwind element).
 * The flux and bed sums at U^n come from the replay of the checkpoint segment (k_rep_cells
 * stores them), so a reverse step recomputes no edge fluxes.
 *
 * The local Jacobians come from the step's own arithmetic (cf_flux.h) instantiated on
 * Dual<D> numbers, whose value lane repeats the forward's IEEE operations, so every branch
 * (wet/dry masks, hydrostatic reconstruction, wave regions, limiter cases, friction
 * floors, the wet/dry clamp of the update) is the one the forward took.  For an edge the D
 * derivative lanes run in chunks over its 6 (first order) or 10 (WAF: + the upwind
 * reconstructions) inputs; D trades registers for repeated value lanes.  The element stage
 * is linear in the sums and is transposed by hand around a Dual<4> friction block.
 *
 * Replay kernels (k_rep_edges, k_rep_cells) advance a state with a recorded dt / time
 * sequence; they run the step's own edge_body / element_update, so a replayed trajectory is
 * bit-identical to the recorded one.
 */
#include <cuda_runtime.h>

#include <algorithm>

#include "cf_dual.h"
#include "cf_xd.h"

namespace cf {
namespace {

__device__ __forceinline__ Slot load_slot_adj(const Slot* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  const double2 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2);
  Slot s;
  s.f1 = a.x; s.f2 = a.y; s.f3 = b.x; s.bx = b.y; s.by = c.x; s.q = c.y;
  return s;
}

/* Dual<D> for input k of the lane chunk starting at base */
template <int D>
__device__ __forceinline__ Dual<D> seed(double v, int k, int base) {
  Dual<D> r(v);
#pragma unroll
  for (int i = 0; i < D; ++i) r.d[i] = (k - base == i) ? 1.0 : 0.0;
  return r;
}

/* ---- replay of the forward -------------------------------------------------------------- */

/* The recorded dt and start time of step n of member m: histories are [N][members]. */
__device__ __forceinline__ size_t hidx(int n, int m, int nm) { return (size_t)n * nm + m; }

/* The replays keep the forward kernels' occupancy: eight edge blocks and four element blocks per SM
 * (64 registers), where the latency of the integer-pipe chains is hidden by more warps. */
template <int IFLUX>
__global__ void __launch_bounds__(TILE_E, 8) k_rep_edges(StepArgs a, const double* dt_hist, const double* t_hist, int n) {
  const int tile = blockIdx.x;
  const int m = __ldg(a.etile_mem + tile);
  const MemberDev& M = a.mdev[m];
  const int e = tile * TILE_E + threadIdx.x;
  if (e >= M.edge_end) return;
  const size_t h = hidx(n, m, a.nmembers);
  const double dt = __ldg(dt_hist + h), t = __ldg(t_hist + h);
  if (a.xd_cmp) {   /* the context's integer-pipe setting, as the step's edge kernel (same results) */
    constexpr bool OC = IFLUX != 3;   /* as the forward edge kernel */
    if ((a.xd_mul_mask >> (threadIdx.x >> 5)) & 1) edge_body<IFLUX, XD<true, OC>>(a, M, e, dt, t);
    else edge_body<IFLUX, XD<false, OC>>(a, M, e, dt, t);
  } else {
    edge_body<IFLUX>(a, M, e, dt, t);
  }
}

__global__ void __launch_bounds__(TILE_C, 4) k_rep_cells(StepArgs a, const double* dt_hist, int n, uint32_t* flag,
                                                         Slot* sums) {
  const int tile = blockIdx.x;
  const int m = __ldg(a.ctile_mem + tile);
  const MemberDev& M = a.mdev[m];
  const int c = tile * TILE_C + threadIdx.x;
  if (c >= M.cell_end) return;
  const double dt = __ldg(dt_hist + hidx(n, m, a.nmembers));
  const double4 U = ld4(a.Uin + c);
  const double4 st = ld4(a.cstat + c);
  const int4 sl = __ldg(a.cslot + c);
  const Slot s0 = load_slot_adj(a.slots + sl.x), s1 = load_slot_adj(a.slots + sl.y), s2 = load_slot_adj(a.slots + sl.z);
  bool nonfinite = false;
  const double4 V = (a.xd_cmp && (a.xd_mul_mask & XD_CELLS))
                        ? element_update<XD<true>>(M, U, st, s0, s1, s2, dt, nonfinite)
                        : element_update(M, U, st, s0, s1, s2, dt, nonfinite);
  if (nonfinite) atomicOr(flag, CF_STATUS_NONFINITE);
  if (a.Uout) {
    double4* o = a.Uout + c;
    reinterpret_cast<double2*>(o)[0] = make_double2(V.x, V.y);
    reinterpret_cast<double2*>(o)[1] = make_double2(V.z, V.w);
  }
  if (sums) {
    /* the sums element_update forms (same expressions, same values) */
    double2* q = reinterpret_cast<double2*>(sums + c);
    q[0] = make_double2(s0.f1 + s1.f1 + s2.f1, s0.f2 + s1.f2 + s2.f2);
    q[1] = make_double2(s0.f3 + s1.f3 + s2.f3, s0.bx + s1.bx + s2.bx);
    q[2] = make_double2(s0.by + s1.by + s2.by, 0.0);
  }
}

/* After step n: the gauge elevations h + z of the new state and, when recording, every
 * member's dt and start time of the step (read from its record of parity p). */
__global__ void k_record(const double4* Unew, const double* zcell, const MemberState* S, int nm, int p, int n,
                         double* dt_hist, double* t_hist, const int32_t* gcell, int G, double* eta) {
  for (int g = threadIdx.x; g < G; g += blockDim.x) {
    const int c = gcell[g];
    eta[(size_t)n * G + g] = Unew[c].x + zcell[c];
  }
  if (S)
    for (int m = threadIdx.x; m < nm; m += blockDim.x) {
      dt_hist[hidx(n, m, nm)] = S[m].dt[p];
      t_hist[hidx(n, m, nm)] = S[m].t[p];
    }
}

/* ---- adjoint of the element stage --------------------------------------------------------- */

/* lambda^{n+1} of element c: its own part plus the contributions the edge adjoint of step n+1
 * left in its three slots and in the upwind entries it belongs to, plus the objective's
 * weights of the gauges it carries; fixed order. */
__device__ __forceinline__ double4 gather_lambda(const AdjArgs& A, int c, const double* gw) {
  double4 L = ld4(A.lam_own + c);
  const int4 sl = __ldg(A.s.cslot + c);
  const double4 e0 = ld4(A.eadj + sl.x), e1 = ld4(A.eadj + sl.y), e2 = ld4(A.eadj + sl.z);
  L.x = L.x + e0.x + e1.x + e2.x;
  L.y = L.y + e0.y + e1.y + e2.y;
  L.z = L.z + e0.z + e1.z + e2.z;
  if (A.uoff) {
    for (int j = __ldg(A.uoff + c), j1 = __ldg(A.uoff + c + 1); j < j1; ++j) {
      const double4 u = ld4(A.uadj + __ldg(A.uidx + j));
      L.x += u.x;
      L.y += u.y;
      L.z += u.z;
    }
  }
  if (gw)
    for (int j = __ldg(A.goff + c), j1 = __ldg(A.goff + c + 1); j < j1; ++j) L.x += __ldg(gw + __ldg(A.gidx + j));
  return L;
}

/* The element update is linear in its flux and bed sums: U^{n+1} = q + dt R (S + sf(q, n) - rc)
 * / area (R = I, or the semi-implicit matrix of rows (1, 0, 0), (m4, m5, m6), (m7, m8, m9)),
 * then the wet/dry clamp.  Its transpose is applied by hand; only the friction block
 * (q1, q2, q3, n) -> (sf2, sf3, m4..m9) is differentiated with Dual<4> numbers of the step's own
 * friction_terms.  128-thread blocks capped at 168 registers: three blocks per SM (a 256-thread
 * block at its 170 registers left room for one). */
constexpr int ADJ_CELLS_BLOCK = 128;
__global__ void __launch_bounds__(ADJ_CELLS_BLOCK, 3) k_adj_cells(AdjArgs A) {
  const StepArgs& a = A.s;
  const int c = blockIdx.x * ADJ_CELLS_BLOCK + threadIdx.x;
  const int mem = __ldg(a.ctile_mem + c / TILE_C);
  const MemberDev& M = a.mdev[mem];
  if (c >= M.cell_end) return;
  const double4 L = A.gather ? gather_lambda(A, c, A.gw) : ld4(A.lam_init + c);
  const double dt = __ldg(A.dt_hist + hidx(A.n, mem, a.nmembers));
  const double4 U = ld4(a.Uin + c);
  const double4 st = ld4(a.cstat + c);
  const double2* sp = reinterpret_cast<const double2*>(A.sums + c);
  const double2 sa = __ldg(sp), sb = __ldg(sp + 1), sc = __ldg(sp + 2);
  const double rc1 = sa.x, rc2 = sa.y, rc3 = sb.x, sb2 = sb.y, sb3 = sc.x;
  const double area = st.x, y = st.w;
  const bool fric = M.friction == 1;
  const bool impl = fric && (M.fricimplic == 1 || M.fricimplic == 2);
  Dual<4> sf2(0.0), sf3(0.0), m[6];
  double r1, ri1, ri2, ri3;
  if (fric) {
    friction_terms(M, area, dt, Dual<4>::var(st.y, 3), Dual<4>::var(U.x, 0), Dual<4>::var(U.y, 1),
                   Dual<4>::var(U.z, 2), sf2, sf3, m, U.w);
    ri1 = div_rn(0. + 0. - rc1, area, y);
    ri2 = div_rn(sb2 + sf2.v - rc2, area, y);
    ri3 = div_rn(sb3 + sf3.v - rc3, area, y);
    r1 = impl ? 1. * ri1 + 0. * ri2 + 0. * ri3 : ri1;
  } else {
    ri1 = div_rn(0. - rc1, area, y);
    ri2 = div_rn(sb2 - rc2, area, y);
    ri3 = div_rn(sb3 - rc3, area, y);
    r1 = ri1;
  }
  const double h = U.x + dt * r1;
  double4 own = make_double4(0.0, 0.0, 0.0, 0.0);
  Slot w;
  w.f1 = w.f2 = w.f3 = w.bx = w.by = w.q = 0.0;
  double nb = 0.0;
  if (!(h <= M.tolisec)) {   /* a clamped element is a constant of its inputs */
    own = make_double4(L.x, L.y, L.z, 0.0);
    const double r1b = dt * L.x, r2b = dt * L.y, r3b = dt * L.z;
    double ri1b = r1b, ri2b = r2b, ri3b = r3b;
    if (impl) {
      ri1b = r1b + r2b * m[0].v + r3b * m[3].v;
      ri2b = r2b * m[1].v + r3b * m[4].v;
      ri3b = r2b * m[2].v + r3b * m[5].v;
    }
    w.f1 = -ri1b * y;
    w.f2 = -ri2b * y;
    w.f3 = -ri3b * y;
    w.bx = ri2b * y;
    w.by = ri3b * y;
    if (fric) {
      const double sf2b = ri2b * y, sf3b = ri3b * y;
      const double mb[6] = {r2b * ri1, r2b * ri2, r2b * ri3, r3b * ri1, r3b * ri2, r3b * ri3};
      double g[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        double v = sf2b * sf2.d[k] + sf3b * sf3.d[k];
        if (impl) {
#pragma unroll
          for (int j = 0; j < 6; ++j) v = fma(mb[j], m[j].d[k], v);
        }
        g[k] = v;
      }
      own.x += g[0];
      own.y += g[1];
      own.z += g[2];
      nb = g[3];
    }
  }
  A.lam_own[c] = own;
  A.cadj[c] = w;
  A.gman[c] += nb;
}

/* ---- adjoint of the edge stage ---------------------------------------------------------- */

/* lambda contributions of one upwind pair (U_i1, U_i2 -> the side's (h, v) reconstruction)
 * given the adjoints wh, wv of that reconstruction. */
__device__ __forceinline__ void upwind_chain(const double4* U, int i1, int i2, double d1, double d2, double ysum,
                                             double nx, double ny, double tolisec, double wh, double wv, double4* o1,
                                             double4* o2) {
  const double4 A1 = ld4(U + i1);
  const double4 A2 = (d1 < 0.0) ? make_double4(0.0, 0.0, 0.0, 0.0) : ld4(U + i2);
  Dual<6> hu_, vu_;
  upwind_mix(Dual<6>::var(A1.x, 0), Dual<6>::var(A1.y, 1), Dual<6>::var(A1.z, 2), A1.w, Dual<6>::var(A2.x, 3),
             Dual<6>::var(A2.y, 4), Dual<6>::var(A2.z, 5), A2.w, d1, d2, ysum, nx, ny, tolisec, hu_, vu_);
  *o1 = make_double4(wh * hu_.d[0] + wv * vu_.d[0], wh * hu_.d[1] + wv * vu_.d[1], wh * hu_.d[2] + wv * vu_.d[2], 0.0);
  *o2 = make_double4(wh * hu_.d[3] + wv * vu_.d[3], wh * hu_.d[4] + wv * vu_.d[4], wh * hu_.d[5] + wv * vu_.d[5], 0.0);
}

/* The transposed edge stage of boundary edge e (side A only): its flux differentiated in three
 * Dual lanes, contracted with the side's slot adjoint. */
template <int IFLUX>
__device__ __forceinline__ void adj_boundary_edge(const AdjArgs& A, const MemberDev& M, int e, int2 ab, double t) {
  const StepArgs& a = A.s;
  const double4 UA = ld4(a.Uin + ab.x);
  const double4 ez = ld4(a.ez + e);
  const Slot wa = A.cadj[ab.x];
  const double4 geo = ld4(a.egeo + e);
  const int id = ldro(a.ebid + e);
  Dual<3> f1, f2, f3, q;
  boundary_flux(IFLUX, M, ab.y, id, t, geo.x, geo.y, Dual<3>::var(UA.x, 0), Dual<3>::var(UA.y, 1),
                Dual<3>::var(UA.z, 2), UA.w, ez.x, f1, f2, f3, q);
  const double len = geo.z;
  double o[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) o[i] = (wa.f1 * f1.d[i] + wa.f2 * f2.d[i] + wa.f3 * f3.d[i]) * len;
  A.eadj[2 * (size_t)e] = make_double4(o[0], o[1], o[2], 0.0);
}

/* The transposed edge stage of interior edge e: the edge's slot values differentiated in Dual<D>
 * chunks over its 6 (first order) or 10 (WAF: + the upwind reconstructions) inputs, contracted
 * with the slot adjoints of its two elements. */
template <int IFLUX, int D>
__device__ __forceinline__ void adj_interior_edge(const AdjArgs& A, const MemberDev& M, int e, int2 ab, double dt) {
  const StepArgs& a = A.s;
  const double4 UA = ld4(a.Uin + ab.x);
  const double4 ez = ld4(a.ez + e);
  const Slot wa = A.cadj[ab.x];
  const double4 UB = ld4(a.Uin + ab.y);
  const Slot wb = A.cadj[ab.y];
  const EdgeGeo G = edge_geo(a, e, IFLUX >= 3);
  double hl_upw = 0.0, vl_upw = 0.0, hr_upw = 0.0, vr_upw = 0.0;
  int4 up = make_int4(0, 0, 0, 0);
  double4 dw = make_double4(0.0, 0.0, 0.0, 0.0);
  if (IFLUX >= 3) {
    up = ldro(a.eupw + e);
    dw = ld4(a.ewts + e);
    upwind_state(a.Uin, up.x, up.y, dw.x, dw.y, G.ysum_a, G.nx, G.ny, M.tolisec, hl_upw, vl_upw);
    upwind_state(a.Uin, up.z, up.w, dw.z, dw.w, G.ysum_b, G.nx, G.ny, M.tolisec, hr_upw, vr_upw);
  }
  constexpr int NDIR = (IFLUX >= 3) ? 10 : 6;
  const double w[10] = {wa.f1, wa.f2, wa.f3, wa.bx, wa.by, wb.f1, wb.f2, wb.f3, wb.bx, wb.by};
  double acc[NDIR];
#pragma unroll
  for (int base = 0; base < NDIR; base += D) {
    Dual<D> o[10];
    interior_edge<IFLUX>(M, a.ilimiteur, a.flux_mode, G, dt, seed<D>(UA.x, 0, base), seed<D>(UA.y, 1, base),
                         seed<D>(UA.z, 2, base), ez.x, UA.w, seed<D>(UB.x, 3, base), seed<D>(UB.y, 4, base),
                         seed<D>(UB.z, 5, base), ez.y, UB.w, seed<D>(hl_upw, 6, base), seed<D>(vl_upw, 7, base), ez.z,
                         seed<D>(hr_upw, 8, base), seed<D>(vr_upw, 9, base), ez.w, o, A.freeze_r != 0);
#pragma unroll
    for (int i = 0; i < D; ++i) {
      if (base + i < NDIR) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 10; ++k) s = fma(w[k], o[k].d[i], s);
        acc[base + i] = s;
      }
    }
  }
  A.eadj[2 * (size_t)e] = make_double4(acc[0], acc[1], acc[2], 0.0);
  A.eadj[2 * (size_t)e + 1] = make_double4(acc[3], acc[4], acc[5], 0.0);
  if constexpr (IFLUX >= 3) {
    double4 c0, c1, c2, c3;
    upwind_chain(a.Uin, up.x, up.y, dw.x, dw.y, G.ysum_a, G.nx, G.ny, M.tolisec, acc[6], acc[7], &c0, &c1);
    upwind_chain(a.Uin, up.z, up.w, dw.z, dw.w, G.ysum_b, G.nx, G.ny, M.tolisec, acc[8], acc[9], &c2, &c3);
    double4* u = A.uadj + 4 * (size_t)e;
    u[0] = c0;
    u[1] = c1;
    u[2] = c2;
    u[3] = c3;
  }
}

template <int IFLUX, int D>
__global__ void __launch_bounds__(TILE_E) k_adj_edges(AdjArgs A) {
  const StepArgs& a = A.s;
  const int tile = blockIdx.x;
  const int m = __ldg(a.etile_mem + tile);
  const MemberDev& M = a.mdev[m];
  const int e = tile * TILE_E + threadIdx.x;
  if (e >= M.edge_end) return;
  const size_t h = hidx(A.n, m, a.nmembers);
  const double dt = __ldg(A.dt_hist + h), t = __ldg(A.t_hist + h);
  const int2 ab = ldro(a.ecell + e);
  if (ab.y < 0) adj_boundary_edge<IFLUX>(A, M, e, ab, t);
  else adj_interior_edge<IFLUX, D>(A, M, e, ab, dt);
}

/* First-order HLLC (flux_mode 0): the closed-form reverse edge (adj_edge_hllc: frame change,
 * reconstruction, tangential velocities and bed sources by hand around a Dual<4> flux core) for
 * every interior edge it covers, at three blocks per SM; the edges it leaves (a nearly dry side
 * whose raw and masked depths differ) are queued for k_adj_edges_rest. */
__global__ void __launch_bounds__(TILE_E, 3) k_adj_edges_hllc(AdjArgs A) {
  const StepArgs& a = A.s;
  const int tile = blockIdx.x;
  const int m = __ldg(a.etile_mem + tile);
  const MemberDev& M = a.mdev[m];
  const int e = tile * TILE_E + threadIdx.x;
  if (e >= M.edge_end) return;
  const int2 ab = ldro(a.ecell + e);
  if (ab.y < 0) {
    adj_boundary_edge<1>(A, M, e, ab, __ldg(A.t_hist + hidx(A.n, m, a.nmembers)));
    return;
  }
  const double4 UA = ld4(a.Uin + ab.x), UB = ld4(a.Uin + ab.y);
  const double4 ez = ld4(a.ez + e);
  const Slot wa = A.cadj[ab.x], wb = A.cadj[ab.y];
  const EdgeGeo G = edge_geo(a, e, false);
  const double w[10] = {wa.f1, wa.f2, wa.f3, wa.bx, wa.by, wb.f1, wb.f2, wb.f3, wb.bx, wb.by};
  double la[3], lb[3];
  if (adj_edge_hllc(M, G, UA, UB, ez.x, ez.y, w, la, lb)) {
    A.eadj[2 * (size_t)e] = make_double4(la[0], la[1], la[2], 0.0);
    A.eadj[2 * (size_t)e + 1] = make_double4(lb[0], lb[1], lb[2], 0.0);
  } else {
    A.pend[atomicAdd(A.npend, 1)] = e;
  }
}

/* The queued interior edges of k_adj_edges_hllc, differentiated in six Dual lanes (grid-stride
 * over the queue; the queue's order does not matter, every edge writes only its own entries). */
__global__ void __launch_bounds__(TILE_E) k_adj_edges_rest(AdjArgs A) {
  const StepArgs& a = A.s;
  const int n = *A.npend;
  for (int i = blockIdx.x * TILE_E + threadIdx.x; i < n; i += gridDim.x * TILE_E) {
    const int e = A.pend[i];
    const int m = __ldg(a.etile_mem + e / TILE_E);
    const MemberDev& M = a.mdev[m];
    const double dt = __ldg(A.dt_hist + hidx(A.n, m, a.nmembers));
    adj_interior_edge<1, 6>(A, M, e, ldro(a.ecell + e), dt);
  }
}

/* ---- lambda^0 -------------------------------------------------------------------------- */

__global__ void __launch_bounds__(TILE_C) k_adj_final(AdjArgs A) {
  const int tile = blockIdx.x;
  const MemberDev& M = A.s.mdev[__ldg(A.s.ctile_mem + tile)];
  const int c = tile * TILE_C + threadIdx.x;
  if (c >= M.cell_end) return;
  A.lam_own[c] = gather_lambda(A, c, nullptr);
}

/* lambda.h += the objective's weights of the gauges an element carries (the final state's
 * gauge terms) */
__global__ void k_add_gauges(double4* lam, const int32_t* goff, const int32_t* gidx, const double* gw, int n) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  for (int j = goff[c]; j < goff[c + 1]; ++j) lam[c].x += gw[gidx[j]];
}

__global__ void k_gather_scalar(const double* x, const int32_t* iperm, double* out, int n) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o < n) out[o] = x[iperm[o]];
}

__global__ void k_set_manning(double4* cstat, const int32_t* perm, const double* nref, int n) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) cstat[c].y = nref[perm[c]];
}

/* ---- Manning zones (calibration parameters) ------------------------------------------------ */

/* dJ/d(zone value) = the sum of dJ/dn over the zone's elements, in the fixed order of the
 * zone's element list (one block per zone: strided partial sums, then a tree). */
__global__ void __launch_bounds__(256) k_zone_sum(const double* gman, const int32_t* zoff, const int32_t* zidx,
                                                  double* gz) {
  __shared__ double s[256];
  const int z = blockIdx.x;
  double v = 0.0;
  for (int j = zoff[z] + threadIdx.x; j < zoff[z + 1]; j += 256) v += gman[zidx[j]];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) gz[z] = s[0];
}

/* projected gradient step on the zone values: v = min(hi, max(lo, v - lr g)) */
__global__ void k_zone_step(double* v, const double* g, int nz, double lr, double lo, double hi) {
  const int z = blockIdx.x * blockDim.x + threadIdx.x;
  if (z < nz) v[z] = fmin(hi, fmax(lo, v[z] - lr * g[z]));
}

/* the Manning n of every element of a zone (elements without a zone keep theirs) */
__global__ void k_zone_apply(double4* cstat, const int32_t* zone_of, const double* v, int n) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n && zone_of[c] >= 0) cstat[c].y = v[zone_of[c]];
}

int chk(cudaError_t e) { return e == cudaSuccess ? CF_OK : CF_ECUDA; }

}  // namespace

int launch_replay_step(const StepArgs& a, const double* dt_hist, const double* t_hist, int n, uint32_t* flag,
                       Slot* sums, stream_t s) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
  switch (a.iflux) {
    case 1: k_rep_edges<1><<<a.n_etiles, TILE_E, 0, st>>>(a, dt_hist, t_hist, n); break;
    case 2: k_rep_edges<2><<<a.n_etiles, TILE_E, 0, st>>>(a, dt_hist, t_hist, n); break;
    case 3: k_rep_edges<3><<<a.n_etiles, TILE_E, 0, st>>>(a, dt_hist, t_hist, n); break;
    default: return CF_ENOTSUP;
  }
  k_rep_cells<<<a.n_ctiles, TILE_C, 0, st>>>(a, dt_hist, n, flag, sums);
  return chk(cudaGetLastError());
}

int launch_record(const double4* Unew, const double* zcell, const MemberState* S, int nm, int p, int n, double* dt_hist,
                  double* t_hist, const int32_t* gcell, int G, double* eta, stream_t s) {
  k_record<<<1, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(Unew, zcell, S, nm, p, n, dt_hist, t_hist, gcell, G, eta);
  return chk(cudaGetLastError());
}

int launch_adjoint_step(const AdjArgs& A, stream_t s) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
  const StepArgs& a = A.s;
  k_adj_cells<<<a.n_ctiles * (TILE_C / ADJ_CELLS_BLOCK), ADJ_CELLS_BLOCK, 0, st>>>(A);
  switch (a.iflux) {
    case 1:
      if (a.flux_mode == 0 && A.pend && A.npend) {
        cudaMemsetAsync(A.npend, 0, sizeof(int32_t), st);
        k_adj_edges_hllc<<<a.n_etiles, TILE_E, 0, st>>>(A);
        k_adj_edges_rest<<<std::min(a.n_etiles, 304), TILE_E, 0, st>>>(A);
      } else {
        k_adj_edges<1, 6><<<a.n_etiles, TILE_E, 0, st>>>(A);
      }
      break;
    case 2: k_adj_edges<2, 3><<<a.n_etiles, TILE_E, 0, st>>>(A); break;
    case 3: k_adj_edges<3, 2><<<a.n_etiles, TILE_E, 0, st>>>(A); break;
    default: return CF_ENOTSUP;
  }
  return chk(cudaGetLastError());
}

int launch_adjoint_final(const AdjArgs& A, stream_t s) {
  k_adj_final<<<A.s.n_ctiles, TILE_C, 0, reinterpret_cast<cudaStream_t>(s)>>>(A);
  return chk(cudaGetLastError());
}

int launch_add_gauges(double4* lam, const int32_t* goff, const int32_t* gidx, const double* gw, int32_t n, stream_t s) {
  if (n <= 0) return CF_OK;
  k_add_gauges<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(lam, goff, gidx, gw, n);
  return chk(cudaGetLastError());
}

int launch_gather_scalar(const double* x, const int32_t* iperm, double* out, int32_t n, stream_t s) {
  if (n <= 0) return CF_OK;
  k_gather_scalar<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(x, iperm, out, n);
  return chk(cudaGetLastError());
}

int launch_set_manning(double4* cstat, const int32_t* perm, const double* nref, int32_t n, stream_t s) {
  if (n <= 0) return CF_OK;
  k_set_manning<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(cstat, perm, nref, n);
  return chk(cudaGetLastError());
}

int launch_zone_sum(const double* gman, const int32_t* zoff, const int32_t* zidx, double* gz, int32_t nz, stream_t s) {
  if (nz <= 0) return CF_OK;
  k_zone_sum<<<nz, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(gman, zoff, zidx, gz);
  return chk(cudaGetLastError());
}

int launch_zone_step(double* v, const double* g, int32_t nz, double lr, double lo, double hi, stream_t s) {
  if (nz <= 0) return CF_OK;
  k_zone_step<<<(nz + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(v, g, nz, lr, lo, hi);
  return chk(cudaGetLastError());
}

int launch_zone_apply(double4* cstat, const int32_t* zone_of, const double* v, int32_t n, stream_t s) {
  if (n <= 0) return CF_OK;
  k_zone_apply<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(cstat, zone_of, v, n);
  return chk(cudaGetLastError());
}

}  // namespace cf
