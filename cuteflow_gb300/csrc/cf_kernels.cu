/*
 * cf_kernels.cu -- sm_103a kernels of the explicit St-Venant step.
 *
 * One step is two kernels on the context's stream:
 *
 *   k_edges : one thread per edge.  Loads both elements' {h, hu, hv, z}, solves the Riemann
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

#include "cf_internal.h"

namespace cf {
namespace {

/* ---- small helpers --------------------------------------------------------------------- */

__device__ __forceinline__ double4 ld4(const double4* p) {
  const double2* q = reinterpret_cast<const double2*>(p);
  double2 a = __ldg(q), b = __ldg(q + 1);
  return make_double4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ bool finite_bits(double x) {
  return (__double_as_longlong(x) & 0x7ff0000000000000ll) != 0x7ff0000000000000ll;
}

/* Masked primitive state in the edge frame (flux_riemann.cuf:105-112). */
__device__ __forceinline__ void to_frame(double h, double hu, double hv, double nx, double ny,
                                         double tolisec, double& hm, double& un, double& ut) {
  if (h > tolisec) {
    const double r = 1.0 / h;
    un = (hu * nx + hv * ny) * r;
    ut = (hv * nx - hu * ny) * r;
    hm = h;
  } else {
    hm = 0.0; un = 0.0; ut = 0.0;
  }
}

/* Wave speeds shared by all solvers (flux_riemann.cuf:930-983 and copies).  Returns false
 * when both depths are below eps; the reference then reads uninitialised speeds, and the
 * flux defined for that case is zero. */
__device__ __forceinline__ bool wave_speeds(double g, double eps, double hl, double ul, double hr,
                                            double ur, double& sl, double& sr, double& set) {
  if (hl < eps && hr < eps) return false;
  const double al = sqrt(g * hl), ar = sqrt(g * hr);
  const double hs = hl + hr;
  const double het = hs * 0.5 - (ur - ul) * hs / (al + ar) * 0.25;
  double pql = 1.0, pqr = 1.0;
  if (!(het < hl)) pql = (hl > eps) ? sqrt(0.5 * (het + hl) * het / (hl * hl)) : 0.0;
  if (!(het < hr)) pqr = (hr > eps) ? sqrt(0.5 * (het + hr) * het / (hr * hr)) : 0.0;
  if (hl > eps) {
    if (hr > eps) { sl = ul - al * pql; sr = ur + ar * pqr; }
    else { sl = ul - al; sr = ul + 2.0 * al; }
  } else {
    sl = ur - 2.0 * ar; sr = ur + ar;
  }
  const double denom = hr * (ur - sr) - hl * (ul - sl);
  if (fabs(denom) < eps) set = (ul + ur) * 0.5 - (hr - hl) * (al + ar) / hs;
  else set = (sl * hr * (ur - sr) - sr * hl * (ul - sl)) / denom;
  return true;
}

/* Edge-frame flux vector (mass, normal momentum, tangential momentum) -> global frame. */
__device__ __forceinline__ void reproject(double nx, double ny, double x1, double x2, double x3,
                                          double& g1, double& g2, double& g3) {
  g1 = x1;
  g2 = nx * x2 - ny * x3;
  g3 = ny * x2 + nx * x3;
}

struct TwoFlux {
  /* global-frame flux of side A (normal out of A) and of side B (normal out of B) */
  double a1, a2, a3, b1, b2, b3;
};

/* First-order HLLC (IFLUX 1, flux_riemann.cuf:902-1026) or the Ata et al. star-state HLLC
 * (IFLUX 2, :1029-1182) for both sides of an edge.  Side B's evaluation in the reference is
 * the mirror image (h -> h, u_n -> -u_n, u_t -> -u_t, s_L -> -s_R, s_* -> -s_*); its flux is
 * minus the A-frame reprojection of the region vector it selects. */
template <int IFLUX>
__device__ __forceinline__ void first_order_flux(double g, double nx, double ny, double hl, double ul,
                                                 double vl, double hr, double ur, double vr, TwoFlux& F) {
  const double eps = (IFLUX == 1) ? EPS_HLLC : EPS_RIADH;
  double sl, sr, set;
  if (!wave_speeds(g, eps, hl, ul, hr, ur, sl, sr, set)) {
    F.a1 = F.a2 = F.a3 = F.b1 = F.b2 = F.b3 = 0.0;
    return;
  }
  const double fl1 = hl * ul, fl2 = hl * ul * ul + g * hl * hl * 0.5, fl3 = hl * ul * vl;
  const double fr1 = hr * ur, fr2 = hr * ur * ur + g * hr * hr * 0.5, fr3 = hr * ur * vr;
  double xa1, xa2, xa3, xb1, xb2, xb3;
  if (IFLUX == 1) {
    /* A: sl>0 -> FL, sr<0 -> FR, else HLL with the HLLC tangential correction.
     * B: (-sr)>0 -> mirror(FR), (-sl)<0 -> mirror(FL), else HLL, tangential by -set. */
    const int ra = (sl > 0.0) ? 0 : ((sr < 0.0) ? 1 : 2);
    const int rb = (sr < 0.0) ? 1 : ((sl > 0.0) ? 0 : 2);
    double h1 = 0.0, h2 = 0.0;
    if (ra == 2 || rb == 2) {
      const double rden = 1.0 / (sr - sl + eps);
      h1 = (sr * fl1 - sl * fr1 + sl * sr * (hr - hl)) * rden;
      h2 = (sr * fl2 - sl * fr2 + sl * sr * (hr * ur - hl * ul)) * rden;
    }
    if (ra == 0) { xa1 = fl1; xa2 = fl2; xa3 = fl3; }
    else if (ra == 1) { xa1 = fr1; xa2 = fr2; xa3 = fr3; }
    else { xa1 = h1; xa2 = h2; xa3 = (set > 0.0) ? h1 * vl : h1 * vr; }
    if (rb == 0) { xb1 = fl1; xb2 = fl2; xb3 = fl3; }
    else if (rb == 1) { xb1 = fr1; xb2 = fr2; xb3 = fr3; }
    else { xb1 = h1; xb2 = h2; xb3 = (set < 0.0) ? h1 * vr : h1 * vl; }
  } else {
    const double pl = (fabs(sl - set) > eps) ? hl * (sl - ul) / (sl - set) : 0.0;
    const double pr = (fabs(sr - set) > eps) ? hr * (sr - ur) / (sr - set) : 0.0;
    const double el1 = fl1 + sl * (pl - hl), el2 = fl2 + sl * (pl * set - hl * ul), el3 = fl3 + sl * (pl * vl - hl * vl);
    const double er1 = fr1 + sr * (pr - hr), er2 = fr2 + sr * (pr * set - hr * ur), er3 = fr3 + sr * (pr * vr - hr * vr);
    /* A: 0<sl FL | 0<set & 0>sl EL | 0>set & 0<sr ER | FR.
     * B (sl'=-sr, set'=-set, sr'=-sl): 0<-sr FR | 0<-set & 0>-sr ER | 0>-set & 0<-sl EL | FL. */
    int ra, rb;
    if (0.0 < sl) ra = 0; else if (0.0 < set && 0.0 > sl) ra = 2; else if (0.0 > set && 0.0 < sr) ra = 3; else ra = 1;
    if (0.0 > sr) rb = 1; else if (0.0 > set && 0.0 < sr) rb = 3; else if (0.0 < set && 0.0 > sl) rb = 2; else rb = 0;
    #define CF_PICK(r, x1, x2, x3)                                   \
      if (r == 0) { x1 = fl1; x2 = fl2; x3 = fl3; }                  \
      else if (r == 1) { x1 = fr1; x2 = fr2; x3 = fr3; }             \
      else if (r == 2) { x1 = el1; x2 = el2; x3 = el3; }             \
      else { x1 = er1; x2 = er2; x3 = er3; }
    CF_PICK(ra, xa1, xa2, xa3)
    CF_PICK(rb, xb1, xb2, xb3)
    #undef CF_PICK
  }
  reproject(nx, ny, xa1, xa2, xa3, F.a1, F.a2, F.a3);
  double q1, q2, q3;
  reproject(nx, ny, xb1, xb2, xb3, q1, q2, q3);
  F.b1 = -q1; F.b2 = -q2; F.b3 = -q3;
}

/* WAF limiter (flux_riemann.cuf:465-524); c enters through |c| only. */
__device__ __forceinline__ double waf_limiter(int ilim, double r, double ac) {
  if (ilim == 1) {
    if (r <= 0.0) return 1.0;
    if (r > 0.0 && r < 0.5) return 1.0 - 2.0 * (1.0 - ac) * r;
    if (r > 0.5 && r < 1.0) return ac;
    if (r > 1.0 && r < 2.0) return 1.0 - (1.0 - ac) * r;
    return 2.0 * ac - 1.0;
  } else if (ilim == 2) {
    if (r <= 0.0) return 1.0;
    return 1.0 - 2.0 * (1.0 - ac) * r / (1.0 + r);
  } else if (ilim == 3) {
    if (r <= 0.0) return 1.0;
    return 1.0 - (1.0 - ac) * r * (1.0 + r) / (1.0 + r * r);
  } else if (ilim == 4) {
    if (r <= 0.0) return 1.0;
    if (r <= 1.0) return 1.0 - (1.0 - ac) * r;
    return ac;
  }
  return 1.0;
}

__device__ __forceinline__ double sgn1(double x) { return copysign(1.0, x); }

/* Second-order WAF (IFLUX 3, flux_riemann.cuf:720-900) for both sides.  Inputs are the
 * reconstructed and masked edge-frame states of A (left) and B (right) and the upwind
 * reconstructions of each side. */
__device__ __forceinline__ void waf_flux(double g, int ilim, double nx, double ny, double dt,
                                         double inv_dmrl, double inv_dka, double inv_dkb, double hl,
                                         double ul, double vl, double hr, double ur, double vr,
                                         double hlu, double vlu, double hru, double vru, TwoFlux& F) {
  const double eps = EPS_SECOND;
  double sl, sr, set;
  if (!wave_speeds(g, eps, hl, ul, hr, ur, sl, sr, set)) {
    F.a1 = F.a2 = F.a3 = F.b1 = F.b2 = F.b3 = 0.0;
    return;
  }
  const double fl1 = hl * ul, fl2 = hl * ul * ul + g * hl * hl * 0.5;
  const double fr1 = hr * ur, fr2 = hr * ur * ur + g * hr * hr * 0.5;
  const int ra = (sl > 0.0) ? 0 : ((sr < 0.0) ? 1 : 2);
  const int rb = (sr < 0.0) ? 1 : ((sl > 0.0) ? 0 : 2);
  double h1 = 0.0, h2 = 0.0;
  if (ra == 2 || rb == 2) {
    const double rden = 1.0 / (sr - sl + eps);
    h1 = (sr * fl1 - sl * fr1 + sl * sr * (hr - hl)) * rden;
    h2 = (sr * fl2 - sl * fr2 + sl * sr * (hr * ur - hl * ul)) * rden;
  }
  const double ha1 = (ra == 0) ? fl1 : ((ra == 1) ? fr1 : h1);
  const double ha2 = (ra == 0) ? fl2 : ((ra == 1) ? fr2 : h2);
  const double hb1 = (rb == 0) ? fl1 : ((rb == 1) ? fr1 : h1);
  const double hb2 = (rb == 0) ? fl2 : ((rb == 1) ? fr2 : h2);

  const double dtdx = dt * inv_dmrl;
  const double acl = fabs(sl * dtdx), acr = fabs(sr * dtdx), acet = fabs(set * dtdx);
  const double dloc = (hr - hl) * inv_dmrl;
  const double dloc_et = (vr - vl) * inv_dmrl;
  const double up_l = (hl - hlu) * inv_dka;   /* upwind difference on side A */
  const double up_r = (hru - hr) * inv_dkb;   /* upwind difference on side B */
  const double upv_l = (vl - vlu) * inv_dka;
  const double upv_r = (vru - vr) * inv_dkb;
  const double inv_et = 1.0 / (dloc_et + eps);

  /* ---- side A (:854-899) */
  {
    const double rinv = 1.0 / (dloc + eps);
    const double rr = ((sr > 0.0) ? up_l : up_r) * rinv;
    const double rl = ((sl > 0.0) ? up_l : up_r) * rinv;
    const double ret = ((set > 0.0) ? upv_l : upv_r) * inv_et;
    const double Ll = waf_limiter(ilim, rl, acl), Lr = waf_limiter(ilim, rr, acr), Le = waf_limiter(ilim, ret, acet);
    const double s_l = sgn1(sl), s_r = sgn1(sr), s_e = sgn1(set);
    const double wl = (1.0 + s_l * Ll) * 0.5, wlr = (s_r * Lr - s_l * Ll) * 0.5, wr = (1.0 - s_r * Lr) * 0.5;
    const double wlet = (1.0 + s_e * Le) * 0.5, wret = (1.0 - s_e * Le) * 0.5;
    const double w1 = wl * fl1 + wlr * ha1 + wr * fr1;
    const double w2 = wl * fl2 + wlr * ha2 + wr * fr2;
    const double w3 = (wlet * vl + wret * vr) * w1;
    reproject(nx, ny, w1, w2, w3, F.a1, F.a2, F.a3);
  }
  /* ---- side B: the same formulas on the mirrored states.  sl'=-sr, sr'=-sl, set'=-set,
   * Δloc' = -Δloc, Δloc_et' = Δloc_et; B's upwind differences are minus A's for the same
   * wave, and the tangential one coincides unless set == 0. */
  {
    const double rinv = 1.0 / (eps - dloc);
    const double rr = ((-sl > 0.0) ? -up_r : -up_l) * rinv;
    const double rl = ((-sr > 0.0) ? -up_r : -up_l) * rinv;
    const double ret = ((-set > 0.0) ? upv_r : upv_l) * inv_et;
    const double Ll = waf_limiter(ilim, rl, acr), Lr = waf_limiter(ilim, rr, acl), Le = waf_limiter(ilim, ret, acet);
    const double s_l = sgn1(-sr), s_r = sgn1(-sl), s_e = sgn1(-set);
    const double wl = (1.0 + s_l * Ll) * 0.5, wlr = (s_r * Lr - s_l * Ll) * 0.5, wr = (1.0 - s_r * Lr) * 0.5;
    const double wlet = (1.0 + s_e * Le) * 0.5, wret = (1.0 - s_e * Le) * 0.5;
    /* mirrored physical fluxes: FL' = (-fr1, fr2), FR' = (-fl1, fl2), HLL' = (-hb1, hb2) */
    const double w1 = -(wl * fr1 + wlr * hb1 + wr * fl1);
    const double w2 = wl * fr2 + wlr * hb2 + wr * fl2;
    const double w3 = -(wlet * vr + wret * vl) * w1;
    /* B's normal is -n: flux' = (w1, -nx*w2 + ny*w3, -ny*w2 - nx*w3) */
    F.b1 = w1;
    F.b2 = -nx * w2 + ny * w3;
    F.b3 = -ny * w2 - nx * w3;
  }
}

/* Discharge of an inlet at time t: debitglob, or a linear ramp from debitglob_start. */
__device__ __forceinline__ double inlet_discharge(const MemberDev& M, int id, double t) {
  const double q1 = M.debit_end[id - 1];
  if (M.ramp_time > 0.0 && t < M.ramp_time) {
    const double q0 = M.debit_start[id - 1];
    return q0 + (q1 - q0) * (t / M.ramp_time);
  }
  return q1;
}

/* Boundary-edge flux of side A (flux_riemann.cuf:114-171). */
template <int IFLUX>
__device__ __forceinline__ void boundary_flux(const MemberDev& M, int kind, int id, double t,
                                              double nx, double ny, double h, double hu, double hv,
                                              double z, double& f1, double& f2, double& f3, double& q) {
  const double g = M.gp, tolisec = M.tolisec;
  double hm, un, ut;
  to_frame(h, hu, hv, nx, ny, tolisec, hm, un, ut);
  f1 = f2 = f3 = 0.0;
  q = 0.0;
  if (kind == -1) {
    if (M.inlet == 1) {
      const double p = hm * un * un + g * hm * hm * 0.5, s = hm * un * ut;
      f1 = hm * un; f2 = nx * p - ny * s; f3 = ny * p + nx * s;
    } else if (M.inlet == 2) {
      const double dn = -inlet_discharge(M, id, t) / M.long_entree[id - 1];
      const double p = dn * dn / (hm + tolisec) + g * hm * hm * 0.5;
      f1 = dn; f2 = nx * p; f3 = ny * p;
      q = -dn;
    }
  } else if (kind == -3) {
    const double p = g * hm * hm * 0.5;
    f2 = nx * p; f3 = ny * p;
  } else if (kind == -2) {
    if (M.outlet == 1) {
      if (un >= 0.0 && un / sqrt(g * hm) < 1.0) {
        double ho = M.h_sortie[id - 1] - z;
        ho = fmax(0.0, ho);
        const double p = ho * un * un + g * ho * ho * 0.5, s = ho * un * ut;
        f1 = ho * un; f2 = nx * p - ny * s; f3 = ny * p + nx * s;
      } else {
        const double p = g * hm * hm * 0.5;
        f2 = nx * p; f3 = ny * p;
      }
      q = f1;
    } else {
      /* transmissive outlet: the element is its own neighbour (:169-171); second-order
       * schemes fall back to the first-order HLLC flux there (zero centroid distance). */
      TwoFlux F;
      double hmm = (hm < tolisec) ? 0.0 : hm;
      double uu = (hm < tolisec) ? 0.0 : un, vv = (hm < tolisec) ? 0.0 : ut;
      if (IFLUX == 2) first_order_flux<2>(g, nx, ny, hmm, uu, vv, hmm, uu, vv, F);
      else first_order_flux<1>(g, nx, ny, hmm, uu, vv, hmm, uu, vv, F);
      f1 = F.a1; f2 = F.a2; f3 = F.a3;
    }
  }
}

/* ---- the edge kernel ------------------------------------------------------------------ */

template <int IFLUX>
__global__ void __launch_bounds__(TILE_E) k_edges(StepArgs a) {
  const int tile = blockIdx.x;
  const int m = __ldg(a.etile_mem + tile);
  const MemberDev& M = a.mdev[m];
  MemberState* S = a.mst + m;
  const int p = a.parity;
  if (S->status) return;
  const double dt = S->dt[p];
  const double t = S->t[p];
  const int e = tile * TILE_E + threadIdx.x;
  if (e == M.edge_begin) {
    /* Start of the member's step: the dt sanity test of cfl_condition.cuf:129-132 (a failing
     * dt ends the run with the current state), the next time, and the start value of the
     * next dt minimum (cflcond sets dt_d = 1e6 and the block reduction pads a partial last
     * block with 1e5, cfl_condition.cuf:21,86). */
    if (dt > 9999.0 || dt < DT_LOW) {
      atomicOr(&S->status, CF_STATUS_DT_RANGE);
    } else {
      S->t[1 - p] = t + dt;
      S->dt[1 - p] = M.dt_reset;
      S->nstep += 1;
    }
  }
  if (e >= M.edge_end) return;
  const int2 ab = __ldg(a.ecell + e);
  const double4 geo = ld4(a.egeo + e);
  const double nx = geo.x, ny = geo.y, len = geo.z;
  const double4 UA = ld4(a.Uin + ab.x);
  const double g = M.gp, tolisec = M.tolisec;
  Slot* sa = a.slots + 2 * (size_t)e;

  if (ab.y < 0) {
    double f1, f2, f3, q;
    boundary_flux<(IFLUX == 2) ? 2 : 1>(M, ab.y, __ldg(a.ebid + e), t, nx, ny, UA.x, UA.y, UA.z, UA.w, f1, f2, f3, q);
    sa->f1 = f1 * len; sa->f2 = f2 * len; sa->f3 = f3 * len;
    sa->bx = 0.0; sa->by = 0.0; sa->q = q * len;
    return;
  }

  const double4 UB = ld4(a.Uin + ab.y);
  const double zij = fmax(UA.w, UB.w);
  TwoFlux F;
  if (IFLUX <= 2) {
    double hl, ul, vl, hr, ur, vr;
    to_frame(UA.x, UA.y, UA.z, nx, ny, tolisec, hl, ul, vl);
    to_frame(UB.x, UB.y, UB.z, nx, ny, tolisec, hr, ur, vr);
    /* hydrostatic reconstruction (:176-181, :200-210); the reference reconstructs the
     * neighbour from its raw depth, which differs from the masked one only for
     * 0 < h <= tolisec (possible in a user-supplied initial state): that rare case evaluates
     * the two sides separately. */
    double hsl = fmax(0.0, hl + UA.w - zij), hsr = fmax(0.0, UB.x + UB.w - zij);
    const bool raw_diff = (hl != UA.x) || (hr != UB.x);
    double a_ul = ul, a_vl = vl, a_ur = ur, a_vr = vr;
    if (hsl < tolisec) { hsl = 0.0; a_ul = 0.0; a_vl = 0.0; }
    if (hsr < tolisec) { hsr = 0.0; a_ur = 0.0; a_vr = 0.0; }
    first_order_flux<IFLUX>(g, nx, ny, hsl, a_ul, a_vl, hsr, a_ur, a_vr, F);
    if (raw_diff) {
      /* side B as the reference evaluates it: B masked, A raw, normal -n */
      double bhl = fmax(0.0, hr + UB.w - zij), bhr = fmax(0.0, UA.x + UA.w - zij);
      double bul = -ur, bvl = -vr, bur = -ul, bvr = -vl;
      if (bhl < tolisec) { bhl = 0.0; bul = 0.0; bvl = 0.0; }
      if (bhr < tolisec) { bhr = 0.0; bur = 0.0; bvr = 0.0; }
      TwoFlux G;
      first_order_flux<IFLUX>(g, -nx, -ny, bhl, bul, bvl, bhr, bur, bvr, G);
      F.b1 = G.a1; F.b2 = G.a2; F.b3 = G.a3;
    }
  } else {
    const int4 up = __ldg(a.eupw + e);
    const double4 w = ld4(a.ewts + e);
    const double2 dk = __ldg(a.edk + e);
    const double4 A1 = ld4(a.Uin + up.x), A2 = ld4(a.Uin + up.y);
    const double4 B1 = ld4(a.Uin + up.z), B2 = ld4(a.Uin + up.w);
    double hl, ul, vl, hr, ur, vr;
    to_frame(UA.x, UA.y, UA.z, nx, ny, tolisec, hl, ul, vl);
    to_frame(UB.x, UB.y, UB.z, nx, ny, tolisec, hr, ur, vr);
    /* upwind states: masked, in this edge's frame, distance-weighted (:240-366) */
    double h1, u1, v1, h2, u2, v2;
    to_frame(A1.x, A1.y, A1.z, nx, ny, tolisec, h1, u1, v1);
    to_frame(A2.x, A2.y, A2.z, nx, ny, tolisec, h2, u2, v2);
    double hlu = w.x * h1 + w.y * h2, vlu = w.x * v1 + w.y * v2, zlu = w.x * A1.w + w.y * A2.w;
    to_frame(B1.x, B1.y, B1.z, nx, ny, tolisec, h1, u1, v1);
    to_frame(B2.x, B2.y, B2.z, nx, ny, tolisec, h2, u2, v2);
    double hru = w.z * h1 + w.w * h2, vru = w.z * v1 + w.w * v2, zru = w.z * B1.w + w.w * B2.w;
    /* hydrostatic reconstruction of all four states (:370-400) */
    double hsl = fmax(0.0, hl + UA.w - zij);
    hlu = fmax(0.0, hlu + zlu - zij);
    double hsr = fmax(0.0, hr + UB.w - zij);
    hru = fmax(0.0, hru + zru - zij);
    if (hsl < tolisec) { hsl = 0.0; ul = 0.0; vl = 0.0; }
    if (hlu < tolisec) { hlu = 0.0; vlu = 0.0; }
    if (hsr < tolisec) { hsr = 0.0; ur = 0.0; vr = 0.0; }
    if (hru < tolisec) { hru = 0.0; vru = 0.0; }
    waf_flux(g, a.ilimiteur, nx, ny, dt, geo.w, dk.x, dk.y, hsl, ul, vl, hsr, ur, vr, hlu, vlu, hru, vru, F);
  }
  if (a.flux_mode == 1) { F.b1 = -F.a1; F.b2 = -F.a2; F.b3 = -F.a3; }

  /* bed-slope source of both sides from the raw depths (source_terms.cuf:90-97) */
  const double hga = fmax(0.0, UA.x + UA.w - zij), hgb = fmax(0.0, UB.x + UB.w - zij);
  const double ba = 0.5 * g * (hga * hga - UA.x * UA.x) * len;
  const double bb = 0.5 * g * (hgb * hgb - UB.x * UB.x) * len;
  Slot* sb = sa + 1;
  sa->f1 = F.a1 * len; sa->f2 = F.a2 * len; sa->f3 = F.a3 * len;
  sa->bx = ba * nx; sa->by = ba * ny; sa->q = 0.0;
  sb->f1 = F.b1 * len; sb->f2 = F.b2 * len; sb->f3 = F.b3 * len;
  sb->bx = -(bb * nx); sb->by = -(bb * ny); sb->q = 0.0;
}

/* ---- the element kernel ----------------------------------------------------------------- */

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }

/* CFL time step of one element (cfl_condition.cuf:20-37). */
__device__ __forceinline__ double cfl_dt_elem(const MemberDev& M, double cflL, double h, double hu, double hv) {
  double d = 1000000.0;
  if (h > M.tolisec) {
    const double r = 1.0 / h;
    const double vu = hu * r, vv = hv * r;
    const double vmax = fmax(0.01, sqrt(vu * vu + vv * vv) + sqrt(M.gp * fabs(h)));
    d = fmin(cflL / vmax, 1000000.0);
  }
  if (M.is_dt_constant == 1) d = M.constant_dt;
  return d;
}

/* Minimum over the block, folded into *target with one atomic (positive doubles order
 * like their bit patterns). */
__device__ __forceinline__ void block_min_atomic(double v, double* target) {
  __shared__ double red[TILE_C / 32];
  #pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    v = (lane < TILE_C / 32) ? red[lane] : 1.0e300;
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (lane == 0) atomicMin(reinterpret_cast<unsigned long long*>(target), dbits(v));
  }
}

__global__ void __launch_bounds__(TILE_C) k_cells(StepArgs a) {
  const int tile = blockIdx.x;
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
  const int c = tile * TILE_C + threadIdx.x;
  double dti = 1.0e300;
  if (c < M.cell_end) {
    const double4 U = ld4(a.Uin + c);
    const double4 st = ld4(a.cstat + c);   /* area, g n^2, cfl L, 1/area */
    const int4 sl = __ldg(a.cslot + c);
    const Slot* s0 = a.slots + sl.x;
    const Slot* s1 = a.slots + sl.y;
    const Slot* s2 = a.slots + sl.z;
    /* reference order: flux sum e1+e2+e3 (flux_riemann.cuf:411-426), bed sum e1,e2,e3 */
    const double rc1 = s0->f1 + s1->f1 + s2->f1;
    const double rc2 = s0->f2 + s1->f2 + s2->f2;
    const double rc3 = s0->f3 + s1->f3 + s2->f3;
    const double sb2 = s0->bx + s1->bx + s2->bx;
    const double sb3 = s0->by + s1->by + s2->by;
    const double q1 = U.x, q2 = U.y, q3 = U.z;
    double r1, r2, r3;
    if (M.friction == 1) {
      double sf2 = 0.0, sf3 = 0.0;
      double m4 = 0.0, m5 = 1.0, m6 = 0.0, m7 = 0.0, m8 = 0.0, m9 = 1.0;
      if (q1 > M.tolisec) {
        const double rq = 1.0 / q1;
        const double vu = q2 * rq, vv = q3 * rq;
        double nv = sqrt(vu * vu + vv * vv);
        if (nv < M.tol) nv = M.tol;
        const double r13 = rcbrt(q1);
        const double k = st.y * st.x * nv * r13;     /* g n^2 area |u| h^(-1/3) */
        sf2 = -(k * vu);
        sf3 = -(k * vv);
        if (nv > M.tol) {
          if (M.fricimplic == 1) {
            const double d = 0.5 * dt * st.y * r13 * rq; /* dt/2 g n^2 h^(-4/3) */
            const double rnv = 1.0 / nv;
            const double a21 = -(7.0 / 3.0) * d * vu * nv, a31 = -(7.0 / 3.0) * d * vv * nv;
            const double a22 = 1.0 + d * (2.0 * vu * vu + vv * vv) * rnv;
            const double a23 = d * vu * vv * rnv;
            const double a33 = 1.0 + d * (vu * vu + 2.0 * vv * vv) * rnv;
            const double rdet = 1.0 / (a22 * a33 - a23 * a23);
            m4 = -(a21 * a33 - a23 * a31) * rdet; m5 = a33 * rdet; m6 = -a23 * rdet;
            m7 = (a21 * a23 - a22 * a31) * rdet; m8 = -a23 * rdet; m9 = a22 * rdet;
          } else if (M.fricimplic == 2) {
            const double beta = -(dt * st.y * nv * r13 * rq);
            const double omb = 1.0 - beta;
            m5 = omb / (omb * omb); m9 = m5;
          }
        }
      }
      const double ri1 = -rc1 * st.w;
      const double ri2 = (sb2 + sf2 - rc2) * st.w;
      const double ri3 = (sb3 + sf3 - rc3) * st.w;
      if (M.fricimplic == 1 || M.fricimplic == 2) {
        r1 = ri1;
        r2 = m4 * ri1 + m5 * ri2 + m6 * ri3;
        r3 = m7 * ri1 + m8 * ri2 + m9 * ri3;
      } else {
        r1 = ri1; r2 = ri2; r3 = ri3;
      }
    } else {
      r1 = -rc1 * st.w;
      r2 = (sb2 - rc2) * st.w;
      r3 = (sb3 - rc3) * st.w;
    }
    double h = q1 + dt * r1, hu = q2 + dt * r2, hv = q3 + dt * r3;
    if (!(finite_bits(h) && finite_bits(hu) && finite_bits(hv))) atomicOr(&S->status, CF_STATUS_NONFINITE);
    if (h <= M.tolisec) { h = 0.0; hu = 0.0; hv = 0.0; }
    double4* o = a.Uout + c;
    reinterpret_cast<double2*>(o)[0] = make_double2(h, hu);
    reinterpret_cast<double2*>(o)[1] = make_double2(hv, U.w);
    dti = cfl_dt_elem(M, st.z, h, hu, hv);
  }
  block_min_atomic(dti, &S->dt[1 - p]);
}

/* CFL of a state into mst[m].dt[slot] (the initial dt, finite_volumes_method.cuf:113-116). */
__global__ void __launch_bounds__(TILE_C) k_cfl(const double4* U, const double4* cstat, const int32_t* ctile_mem,
                                                const MemberDev* mdev, MemberState* mst, int slot) {
  const int tile = blockIdx.x;
  const int m = __ldg(ctile_mem + tile);
  const MemberDev& M = mdev[m];
  const int c = tile * TILE_C + threadIdx.x;
  double dti = 1.0e300;
  if (c < M.cell_end) {
    const double4 u = ld4(U + c);
    dti = cfl_dt_elem(M, ld4(cstat + c).z, u.x, u.y, u.z);
  }
  block_min_atomic(dti, &mst[m].dt[slot]);
}

/* Discharge diagnostics of the last step (debit_entree_sum, debit_sortie,
 * finite_volumes_method.cuf:197-214): per member, fixed-order sums over its boundary edges
 * (deterministic: each thread sums a fixed stride, then a fixed tree). */
__global__ void __launch_bounds__(256) k_discharge(const Slot* slots, const int2* ecell, const MemberDev* mdev,
                                                    MemberState* mst) {
  __shared__ double si[256], so[256];
  const int m = blockIdx.x;
  const MemberDev& M = mdev[m];
  double qi = 0.0, qo = 0.0;
  for (int e = M.bedge_begin + threadIdx.x; e < M.bedge_end; e += 256) {
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
    mst[m].q_in = si[0];
    mst[m].q_out = so[0];
  }
}

__global__ void k_scatter(const double* hu3, const int32_t* perm, const double* zcell, double4* U, int n) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int o = perm[c];
  U[c] = make_double4(hu3[3 * (size_t)o], hu3[3 * (size_t)o + 1], hu3[3 * (size_t)o + 2], zcell[c]);
}

__global__ void k_gather(const double4* U, const int32_t* iperm, double* hu3, int n) {
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n) return;
  const double4 u = U[iperm[o]];
  hu3[3 * (size_t)o] = u.x;
  hu3[3 * (size_t)o + 1] = u.y;
  hu3[3 * (size_t)o + 2] = u.z;
}

int check(cudaError_t e) { return e == cudaSuccess ? CF_OK : CF_ECUDA; }

}  // namespace

int launch_step(const StepArgs& a, stream_t s, void* ev_mid, void* ev_end) {
  cudaStream_t st = reinterpret_cast<cudaStream_t>(s);
  switch (a.iflux) {
    case 1: k_edges<1><<<a.n_etiles, TILE_E, 0, st>>>(a); break;
    case 2: k_edges<2><<<a.n_etiles, TILE_E, 0, st>>>(a); break;
    case 3: k_edges<3><<<a.n_etiles, TILE_E, 0, st>>>(a); break;
    default: return CF_ENOTSUP;
  }
  if (ev_mid) cudaEventRecord(reinterpret_cast<cudaEvent_t>(ev_mid), st);
  k_cells<<<a.n_ctiles, TILE_C, 0, st>>>(a);
  if (ev_end) cudaEventRecord(reinterpret_cast<cudaEvent_t>(ev_end), st);
  return check(cudaGetLastError());
}

int launch_cfl(const double4* U, const double4* cstat, const int32_t* ctile_mem, int32_t n_ctiles,
               const MemberDev* mdev, MemberState* mst, int32_t slot, stream_t s) {
  k_cfl<<<n_ctiles, TILE_C, 0, reinterpret_cast<cudaStream_t>(s)>>>(U, cstat, ctile_mem, mdev, mst, slot);
  return check(cudaGetLastError());
}

int launch_discharge(const Slot* slots, const int2* ecell, const MemberDev* mdev, MemberState* mst, int32_t nmembers,
                     stream_t s) {
  k_discharge<<<nmembers, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(slots, ecell, mdev, mst);
  return check(cudaGetLastError());
}

int launch_scatter_state(const double* hu3, const int32_t* perm, const double* zcell, double4* U, int32_t n, stream_t s) {
  k_scatter<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(hu3, perm, zcell, U, n);
  return check(cudaGetLastError());
}

int launch_gather_state(const double4* U, const int32_t* iperm, double* hu3, int32_t n, stream_t s) {
  k_gather<<<(n + 255) / 256, 256, 0, reinterpret_cast<cudaStream_t>(s)>>>(U, iperm, hu3, n);
  return check(cudaGetLastError());
}

}  // namespace cf
