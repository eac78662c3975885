/*
 * flux_harness.cpp -- TEST INFRASTRUCTURE.  Compiles the GPU step's per-edge flux mathematics
 * (cuteflow_gb300/csrc/cf_flux.h) and host preprocessing (cf_mesh.cpp) for the CPU so that the
 * tests can compare, edge by edge, the fluxes the edge kernel writes with the oracle's
 * per-(element, edge) evaluation of the reference.  Not part of the product library.
 */
#include "../cuteflow_gb300/csrc/cf_flux.h"
#include "../cuteflow_gb300/csrc/cf_xd.h"

#include <cmath>
#include <vector>

using namespace cf;

/* The member constants of a one-member context, as cf_api.cpp builds them. */
static void fill_member(MemberDev& M, const cf_params* p, const Prep& P) {
  std::memset(&M, 0, sizeof(M));
  M.gp = p->gp; M.tolisec = p->tolisec; M.tol = p->tol; M.constant_dt = p->constant_dt;
  M.ramp_time = p->ramp_time;
  M.dt_reset = ((p->dt_reset_nelt > 0 ? p->dt_reset_nelt : P.nelt) % 1024 != 0) ? 100000.0 : 1000000.0;
  for (int i = 0; i < CF_MAX_IO; ++i) {
    M.debit_end[i] = p->debitglob[i]; M.debit_start[i] = p->debitglob_start[i];
    M.long_entree[i] = P.long_entree[i]; M.h_sortie[i] = p->h_sortie[i];
  }
  M.inlet = p->inlet; M.outlet = p->outlet; M.friction = p->friction; M.fricimplic = p->fricimplic;
  M.is_dt_constant = p->is_dt_constant;
  M.inl_begin = 0;
  M.inl_count = (int32_t)P.inl_cell.size();
  M.inl_len_off = 0;
  M.nin = P.nin;
  M.tol_reg_perm = p->tol_reg_perm;
  M.steady_count = p->steady_count > 0 ? p->steady_count : 1000;
}

/* The edge kernel's arithmetic type: 0 double, 1 integer comparisons (XD<false>), 2 integer
 * comparisons and products (XD<true>); results must not depend on it. */
static int g_xd = 0;
extern "C" void harness_set_xd(int mode) { g_xd = mode; }

template <int IFLUX>
static void edge_xd(const StepArgs& a, const MemberDev& M, int e, double dt, double t, const double* surf) {
  if (g_xd == 1) edge_body<IFLUX, XD<false>>(a, M, e, dt, t, surf);
  else if (g_xd == 2) edge_body<IFLUX, XD<true>>(a, M, e, dt, t, surf);
  else edge_body<IFLUX>(a, M, e, dt, t, surf);
}

/* k_surf on the CPU: per inlet, blocks of 32 entries summed by the tree s[t] += s[t + i]
 * (i = 16 .. 1), block sums added in order. */
static void surf_sums(const Prep& P, const MemberDev& M, const double4* U, double* surf) {
  for (int id = 0; id < M.nin; ++id) {
    double total = 0.0;
    for (int b = 0; b < M.inl_count; b += 32) {
      double s[32];
      for (int l = 0; l < 32; ++l) {
        const int j = b + l;
        s[l] = j < M.inl_count ? P.inl_len[(size_t)j * M.nin + id] * U[P.inl_cell[j]].x : 0.0;
      }
      for (int i = 16; i > 0; i >>= 1)
        for (int l = 0; l < i; ++l) s[l] = s[l] + s[l + i];
      total = total + s[0];
    }
    surf[id] = total;
  }
}

/* k_discharge on the CPU: 256 strided partial sums over the boundary edges, then a tree. */
static void discharge(const Prep& P, const std::vector<Slot>& slots, double& qin, double& qout) {
  double si[256] = {0}, so[256] = {0};
  const int ne = (int)P.edges.size();
  for (int t = 0; t < 256; ++t)
    for (int e = P.n_interior + t; e < ne; e += 256) {
      const int kind = P.ecell[e].y;
      if (kind == -1) si[t] += slots[2 * (size_t)e].q;
      else if (kind == -2) so[t] += slots[2 * (size_t)e].q;
    }
  for (int w = 128; w > 0; w >>= 1)
    for (int t = 0; t < w; ++t) { si[t] += si[t + w]; so[t] += so[t + w]; }
  qin = si[0];
  qout = so[0];
}

extern "C" int harness_edge_fluxes(const cf_mesh* m, const cf_params* p, const double* U, double dt, double t,
                                   double* out /* [nelt][3][3] flux*len, reference order */,
                                   double* bed /* [nelt][3][2] bed source per (element, edge), or NULL */) {
  Prep P;
  std::string err;
  int rc = prepare_mesh(m, p, P, err);
  if (rc != CF_OK) return rc;
  const int n = P.nelt;
  std::vector<double4> Un(n);
  for (int c = 0; c < n; ++c) {
    int o = P.perm[c];
    Un[c] = make_double4(U[3 * o], U[3 * o + 1], U[3 * o + 2], U[3 * o] > 0.0 ? 1.0 / U[3 * o] : 0.0);
  }
  MemberDev M;
  fill_member(M, p, P);
  const int ne = (int)P.edges.size();
  std::vector<Slot> slots(2 * (size_t)ne);
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Uin = Un.data();
  a.ecell = P.ecell.data(); a.egeo = P.egeo.data(); a.ebid = P.ebid.data(); a.ez = P.ez.data();
  a.eupw = P.eupw.empty() ? nullptr : P.eupw.data();
  a.ewts = P.ewts.empty() ? nullptr : P.ewts.data();
  a.edk = P.edk.empty() ? nullptr : P.edk.data();
  a.einv = P.einv.empty() ? nullptr : P.einv.data();
  a.slots = slots.data();
  a.iflux = p->iflux; a.ilimiteur = p->ilimiteur; a.flux_mode = p->flux_mode;
  double surf[CF_MAX_IO] = {0};
  surf_sums(P, M, Un.data(), surf);
  for (int e = 0; e < ne; ++e) {
    if (p->iflux == 1) edge_xd<1>(a, M, e, dt, t, surf);
    else if (p->iflux == 2) edge_xd<2>(a, M, e, dt, t, surf);
    else if (p->iflux == 3) edge_xd<3>(a, M, e, dt, t, surf);
    else edge_xd<4>(a, M, e, dt, t, surf);
  }
  for (int c = 0; c < n; ++c) {
    int o = P.perm[c];
    const int* s = &P.cslot[c].x;
    for (int k = 0; k < 3; ++k) {
      const Slot& S = slots[s[k]];
      out[(o * 3 + k) * 3 + 0] = S.f1;
      out[(o * 3 + k) * 3 + 1] = S.f2;
      out[(o * 3 + k) * 3 + 2] = S.f3;
      if (bed) { bed[(o * 3 + k) * 2 + 0] = S.bx; bed[(o * 3 + k) * 2 + 1] = S.by; }
    }
  }
  return 0;
}

/* Elements of the last harness_run that took the element kernel's dry-neighbourhood shortcut,
 * and those among them whose slots were not all signed zeros (the shortcut would be wrong). */
static long long g_nbhd_took = 0, g_nbhd_bad = 0;
extern "C" void harness_nbhd_stats(long long* took, long long* bad) {
  *took = g_nbhd_took;
  *bad = g_nbhd_bad;
}

/* The whole GPU step algorithm on the CPU: edge pass, element pass (with the element kernel's
 * dry-neighbourhood shortcut, checked against the slots it skips), device dt rule, for nsteps
 * steps from U (reference order); U_out and dt_hist (nsteps+1) like the oracle. */
extern "C" int harness_run(const cf_mesh* m, const cf_params* p, const double* U, int nsteps, double* U_out,
                           double* dt_hist, double* t_out, int* steps_out) {
  int done = 0, steady_iter = 0;
  Prep P;
  std::string err;
  int rc = prepare_mesh(m, p, P, err);
  if (rc != CF_OK) return rc;
  g_nbhd_took = g_nbhd_bad = 0;
  const int n = P.nelt;
  std::vector<double4> Ua(n), Ub(n);
  for (int c = 0; c < n; ++c) {
    int o = P.perm[c];
    Ua[c] = make_double4(U[3 * o], U[3 * o + 1], U[3 * o + 2], U[3 * o] > 0.0 ? 1.0 / U[3 * o] : 0.0);
  }
  MemberDev M;
  fill_member(M, p, P);
  const int ne = (int)P.edges.size();
  std::vector<Slot> slots(2 * (size_t)ne);
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.ecell = P.ecell.data(); a.egeo = P.egeo.data(); a.ebid = P.ebid.data(); a.ez = P.ez.data();
  a.eupw = P.eupw.empty() ? nullptr : P.eupw.data();
  a.ewts = P.ewts.empty() ? nullptr : P.ewts.data();
  a.edk = P.edk.empty() ? nullptr : P.edk.data();
  a.einv = P.einv.empty() ? nullptr : P.einv.data();
  a.slots = slots.data();
  a.iflux = p->iflux; a.ilimiteur = p->ilimiteur; a.flux_mode = p->flux_mode;
  double4* cur = Ua.data();
  double4* nxt = Ub.data();
  double dt = M.dt_reset;
  for (int c = 0; c < n; ++c) dt = dmin(dt, cfl_dt_elem(M, P.cstat[c].z, cur[c].x, cur[c].y, cur[c].z, cur[c].w));
  if (dt_hist) dt_hist[0] = dt;
  double t = 0.0;
  for (int s = 0; s < nsteps; ++s) {
    if (s > 0 && (dt > 9999.0 || dt < DT_LOW)) { rc = -2; break; }
    a.Uin = cur;
    double surf[CF_MAX_IO] = {0};
    surf_sums(P, M, cur, surf);
    for (int e = 0; e < ne; ++e) {
      if (p->iflux == 1) edge_xd<1>(a, M, e, dt, t, surf);
      else if (p->iflux == 2) edge_xd<2>(a, M, e, dt, t, surf);
      else if (p->iflux == 3) edge_xd<3>(a, M, e, dt, t, surf);
      else edge_xd<4>(a, M, e, dt, t, surf);
    }
    double next = M.dt_reset;
    for (int c = 0; c < n; ++c) {
      const int* sl = &P.cslot[c].x;
      bool nf = false;
      if (dry_state_ok(M, cur[c], dt) && dry_neighbourhood(M, P.cnbr[c], cur[c], [&](int k) { return cur[k].x; })) {
        ++g_nbhd_took;
        if (!dry_element(M, cur[c], P.cstat[c], slots[sl[0]], slots[sl[1]], slots[sl[2]], dt)) ++g_nbhd_bad;
        nxt[c] = make_double4(0.0, 0.0, 0.0, 0.0);
      } else
      nxt[c] = g_xd == 0 ? element_update(M, cur[c], P.cstat[c], slots[sl[0]], slots[sl[1]], slots[sl[2]], dt, nf)
               : g_xd == 1 ? element_update<XD<false>>(M, cur[c], P.cstat[c], slots[sl[0]], slots[sl[1]], slots[sl[2]], dt, nf)
                           : element_update<XD<true>>(M, cur[c], P.cstat[c], slots[sl[0]], slots[sl[1]], slots[sl[2]], dt, nf);
      next = dmin(next, cfl_dt_elem(M, P.cstat[c].z, nxt[c].x, nxt[c].y, nxt[c].z, nxt[c].w));
    }
    t = t + dt;
    dt = next;
    if (dt_hist) dt_hist[s + 1] = dt;
    std::swap(cur, nxt);
    ++done;
    if (M.tol_reg_perm > 0.0) {   /* check_steady_state, as k_discharge applies it */
      double qi, qo;
      discharge(P, slots, qi, qo);
      if (qi > (double)1e-8f && std::fabs(qi - qo) / qi < M.tol_reg_perm) {
        if (++steady_iter > M.steady_count) { rc = 1; break; }
      } else {
        steady_iter = 0;
      }
    }
  }
  if (steps_out) *steps_out = done;
  for (int c = 0; c < n; ++c) {
    int o = P.perm[c];
    U_out[3 * o] = cur[c].x; U_out[3 * o + 1] = cur[c].y; U_out[3 * o + 2] = cur[c].z;
  }
  if (t_out) *t_out = t;
  return rc;
}

/* div_rn (Markstein's correction with y = RN(1/d)) against the IEEE quotient on n samples of
 * adversarial operands: random exponents over 2^[-70, 50) / 2^[-30, 30), all-ones and
 * near-all-ones significands, powers of two, a close to d, exact multiples, signed zeros.
 * Returns the number of bitwise mismatches. */
extern "C" long long harness_div_check(long long n, unsigned long long seed) {
  unsigned long long s = seed | 1;
  auto rnd = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  auto mk = [](unsigned long long sign, int exp, unsigned long long mant) {
    unsigned long long b = (sign << 63) | ((unsigned long long)(exp + 1023) << 52) | (mant & ((1ull << 52) - 1));
    double x;
    memcpy(&x, &b, 8);
    return x;
  };
  long long bad = 0;
  for (long long i = 0; i < n; ++i) {
    unsigned long long r1 = rnd(), r2 = rnd(), md = rnd(), ma = rnd();
    int ed = (int)(r1 % 60) - 30, ea = (int)((r1 >> 8) % 120) - 70, mode = (int)((r2 >> 3) % 9);
    if (mode == 0) md = (1ull << 52) - 1;
    if (mode == 1) md = (1ull << 52) - 1 - (rnd() % 16);
    if (mode == 2) ma = md;
    if (mode == 3) md = 0;
    if (mode == 4) ma = (1ull << 52) - 1;
    double d = mk(r2 >> 63, ed, md), a = mk(r2 & 1, ea, ma);
    if (mode == 5) a = d * (double)(rnd() % 1000);
    if (mode == 6) a = (r2 & 2) ? -0.0 : 0.0;
    const double got = div_rn(a, d, 1.0 / d), ref = a / d;
    if (memcmp(&got, &ref, 8) != 0) ++bad;
  }
  return bad;
}

/* cf::rcbrt (the kernels' x^(-1/3)) elementwise, on the host. */
extern "C" void harness_rcbrt(const double* x, double* y, long long n) {
  for (long long i = 0; i < n; ++i) y[i] = cf::rcbrt(x[i]);
}

/* em_mul, em_div, em_sqrt, the exponent-change scalings and the integer comparisons of cf_xd.h against the hardware on n adversarial operand
 * pairs: exponents over the whole range (subnormals, near overflow and underflow), all-ones and
 * near-all-ones significands, signed zeros, infinities and NaN.  Returns the mismatches. */
extern "C" long long harness_xd_check(long long n, unsigned long long seed) {
  unsigned long long s = seed | 1;
  auto rnd = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  auto mk = [&](int emin, int emax) {
    unsigned long long m = rnd() & ((1ull << 52) - 1);
    const int mode = (int)(rnd() % 8);
    if (mode == 0) m = (1ull << 52) - 1;
    if (mode == 1) m = 0;
    if (mode == 2) m = rnd() % 16;
    if (mode == 3) m = ((1ull << 52) - 1) ^ (rnd() % 16);
    const int e = emin + (int)(rnd() % (unsigned long long)(emax - emin + 1));
    const unsigned long long b = ((rnd() & 1) << 63) | ((unsigned long long)e << 52) | m;
    double x;
    memcpy(&x, &b, 8);
    return x;
  };
  long long bad = 0;
  for (long long i = 0; i < n; ++i) {
    const int mode = (int)(rnd() % 7);
    double a, b;
    if (mode == 0) { a = mk(1, 2046); b = mk(1, 2046); }              /* any normal */
    else if (mode == 1) { a = mk(0, 2047); b = mk(0, 2047); }         /* incl. subnormal, inf, NaN */
    else if (mode == 2) { a = mk(1000, 1050); b = mk(1000, 1050); }   /* the step's range */
    else if (mode == 3) { a = mk(1, 30); b = mk(990, 1030); }         /* underflow edge */
    else if (mode == 4) { a = mk(2000, 2046); b = mk(1000, 1100); }   /* overflow edge */
    else { a = (rnd() & 1) ? -0.0 : 0.0; b = mk(0, 2047); }           /* signed zero times anything */
    if (mode == 6) std::swap(a, b);
    if (mode == 5 && (rnd() & 1)) {
      /* a / b close to a rounding midpoint: A = RN((2N+1) B / 2^sh) moved by up to two units */
      const unsigned long long N = (1ull << 52) | (rnd() & ((1ull << 52) - 1));
      const unsigned long long B = (1ull << 52) | (rnd() & ((1ull << 52) - 1));
      const unsigned __int128 num = (unsigned __int128)(2 * N + 1) * B;
      const int sh = ((num >> 106) != 0 || (rnd() & 1)) ? 54 : 53;  /* A / B below or above 1 */
      unsigned long long A = (unsigned long long)((num + ((unsigned __int128)1 << (sh - 1))) >> sh);
      A += (rnd() % 5) - 2;
      if (A >= (1ull << 53)) A = (1ull << 53) - 1;
      if (A < (1ull << 52)) A = 1ull << 52;
      const unsigned long long ba = ((rnd() & 1) << 63) | ((unsigned long long)(1000 + rnd() % 40) << 52) | (A & ((1ull << 52) - 1));
      const unsigned long long bb = ((rnd() & 1) << 63) | ((unsigned long long)(1000 + rnd() % 40) << 52) | (B & ((1ull << 52) - 1));
      memcpy(&a, &ba, 8);
      memcpy(&b, &bb, 8);
    }
    if (mode == 4 && (rnd() & 1)) {
      /* sqrt(a) close to a rounding midpoint: significand of RN((N + 1/2)^2 / 2^(52 + p)), moved
       * by up to two units */
      const unsigned long long N = (1ull << 52) | (rnd() & ((1ull << 52) - 1));
      const unsigned __int128 sq = (unsigned __int128)(2 * N + 1) * (2 * N + 1);  /* 4 (N + 1/2)^2 */
      const int sh = (sq >> 107) ? 55 : 54;
      unsigned long long A = (unsigned long long)((sq + ((unsigned __int128)1 << (sh - 1))) >> sh);
      A += (rnd() % 5) - 2;
      if (A >= (1ull << 53)) A = (1ull << 53) - 1;
      if (A < (1ull << 52)) A = 1ull << 52;
      const unsigned long long ex = (unsigned long long)(1001 + 2 * (rnd() % 20) - (sh == 55 ? 1 : 0));  /* parity p = sh - 54 */
      const unsigned long long ba = (ex << 52) | (A & ((1ull << 52) - 1));
      memcpy(&a, &ba, 8);
    }
    const double r1 = em_sqrt(a), r2 = std::sqrt(a);
    if (memcmp(&r1, &r2, 8) != 0 && !(r1 != r1 && r2 != r2)) ++bad;
    const double q1 = em_div(a, b), q2 = a / b;
    if (memcmp(&q1, &q2, 8) != 0 && !(q1 != q1 && q2 != q2)) ++bad;
    const double p1 = em_mul(a, b), p2 = a * b;
    const double n1 = val(-XD<true>(a)), n2 = -a;
    if (memcmp(&n1, &n2, 8) != 0) ++bad;
    if (memcmp(&p1, &p2, 8) != 0 && !(p1 != p1 && p2 != p2)) ++bad;
    const double s1[3] = {xscale<-2>(a), xscale<-1>(a), xscale<1>(a)}, s2[3] = {a * 0.25, a * 0.5, a * 2.0};
    for (int k = 0; k < 3; ++k)
      if (memcmp(&s1[k], &s2[k], 8) != 0 && !(s1[k] != s1[k] && s2[k] != s2[k])) ++bad;
    if (xlt(a, b) != (a < b) || xle(a, b) != (a <= b) || xeq(a, b) != (a == b)) ++bad;
    const double z = (rnd() & 1) ? -0.0 : 0.0;
    if (xlt(a, z) != (a < z) || xlt(z, a) != (z < a) || xle(a, z) != (a <= z) || xeq(a, z) != (a == z)) ++bad;
  }
  return bad;
}

/* ---- tangent-linear run: the discrete step differentiated in forward mode -------------------- */

#include "../cuteflow_gb300/csrc/cf_dual.h"

typedef Dual<1> D1;

/* nsteps steps from U0 with Manning n, replaying the dt / start-time sequence, carrying the
 * tangent of the direction (dU0, dn) along (every branch is the one the values take: the same
 * templated arithmetic as the GPU step).  Outputs (reference order): the gauge elevations
 * eta [nsteps][G] and their tangents, the final state and its tangent. */
extern "C" int harness_tangent(const cf_mesh* m, const cf_params* p, const double* U0, const double* dU0,
                               const double* nman, const double* dn, int nsteps, const double* dt_seq,
                               const double* t_seq, const int32_t* gauges, int G, double* eta, double* deta,
                               double* U_out, double* dU_out, int freeze_r) {
  Prep P;
  std::string err;
  int rc = prepare_mesh(m, p, P, err);
  if (rc != CF_OK) return rc;
  const int n = P.nelt;
  MemberDev M;
  fill_member(M, p, P);
  std::vector<D1> h(n), hu(n), hv(n), nm(n), nh(n), nhu(n), nhv(n);
  std::vector<double> z(n);
  for (int c = 0; c < n; ++c) {
    const int o = P.perm[c];
    h[c] = D1(U0[3 * o]); h[c].d[0] = dU0[3 * o];
    hu[c] = D1(U0[3 * o + 1]); hu[c].d[0] = dU0[3 * o + 1];
    hv[c] = D1(U0[3 * o + 2]); hv[c].d[0] = dU0[3 * o + 2];
    nm[c] = D1(nman[o]); nm[c].d[0] = dn[o];
    z[c] = P.zcell[c];
  }
  const int ne = (int)P.edges.size();
  std::vector<D1> slot(10 * (size_t)ne);   /* per slot s: 5 values at 5 s */
  const bool second = p->iflux >= 3;
  for (int s = 0; s < nsteps; ++s) {
    const double dt = dt_seq[s], t = t_seq[s];
    for (int e = 0; e < ne; ++e) {
      const int2 ab = P.ecell[e];
      const double4 geo = P.egeo[e];
      D1* sa = &slot[10 * (size_t)e];
      if (ab.y < 0) {
        D1 f1, f2, f3, q;
        boundary_flux(p->iflux, M, ab.y, P.ebid[e], t, geo.x, geo.y, h[ab.x], hu[ab.x], hv[ab.x], 0.0, z[ab.x], f1, f2,
                      f3, q);
        sa[0] = f1 * geo.z; sa[1] = f2 * geo.z; sa[2] = f3 * geo.z; sa[3] = D1(0.0); sa[4] = D1(0.0);
        continue;
      }
      EdgeGeo Gm;
      Gm.nx = geo.x; Gm.ny = geo.y; Gm.len = geo.z; Gm.d_mrl = geo.w;
      Gm.y_mrl = Gm.d_mkvol = Gm.y_mkvol = Gm.d_mkvoisin = Gm.y_mkvoisin = Gm.ysum_a = Gm.ysum_b = 0.0;
      D1 hlu(0.0), vlu(0.0), hru(0.0), vru(0.0);
      double zlu = 0.0, zru = 0.0;
      if (second) {
        const double4 dk = P.edk[e], yi = P.einv[e], dw = P.ewts[e];
        const int4 up = P.eupw[e];
        Gm.y_mrl = yi.x; Gm.d_mkvol = dk.x; Gm.y_mkvol = dk.z; Gm.d_mkvoisin = dk.y; Gm.y_mkvoisin = dk.w;
        Gm.ysum_a = yi.y; Gm.ysum_b = yi.z;
        const int a2 = dw.x < 0.0 ? up.x : up.y, b2 = dw.z < 0.0 ? up.z : up.w;
        upwind_mix(h[up.x], hu[up.x], hv[up.x], 0.0, h[a2], hu[a2], hv[a2], 0.0, dw.x, dw.y, yi.y, geo.x, geo.y,
                   M.tolisec, hlu, vlu);
        upwind_mix(h[up.z], hu[up.z], hv[up.z], 0.0, h[b2], hu[b2], hv[b2], 0.0, dw.z, dw.w, yi.z, geo.x, geo.y,
                   M.tolisec, hru, vru);
        zlu = dw.x < 0.0 ? z[up.x] : div_rn(dw.x * z[up.x] + dw.y * z[up.y], dw.x + dw.y, yi.y);
        zru = dw.z < 0.0 ? z[up.z] : div_rn(dw.z * z[up.z] + dw.w * z[up.w], dw.z + dw.w, yi.z);
      }
      if (p->iflux == 1)
        interior_edge<1>(M, p->ilimiteur, p->flux_mode, Gm, dt, h[ab.x], hu[ab.x], hv[ab.x], z[ab.x], 0.0, h[ab.y],
                         hu[ab.y], hv[ab.y], z[ab.y], 0.0, hlu, vlu, zlu, hru, vru, zru, sa);
      else if (p->iflux == 2)
        interior_edge<2>(M, p->ilimiteur, p->flux_mode, Gm, dt, h[ab.x], hu[ab.x], hv[ab.x], z[ab.x], 0.0, h[ab.y],
                         hu[ab.y], hv[ab.y], z[ab.y], 0.0, hlu, vlu, zlu, hru, vru, zru, sa);
      else
        interior_edge<3>(M, p->ilimiteur, p->flux_mode, Gm, dt, h[ab.x], hu[ab.x], hv[ab.x], z[ab.x], 0.0, h[ab.y],
                         hu[ab.y], hv[ab.y], z[ab.y], 0.0, hlu, vlu, zlu, hru, vru, zru, sa, freeze_r != 0);
    }
    for (int c = 0; c < n; ++c) {
      const int* sl = &P.cslot[c].x;
      const D1* s0 = &slot[5 * (size_t)sl[0]];
      const D1* s1 = &slot[5 * (size_t)sl[1]];
      const D1* s2 = &slot[5 * (size_t)sl[2]];
      const D1 rc1 = s0[0] + s1[0] + s2[0], rc2 = s0[1] + s1[1] + s2[1], rc3 = s0[2] + s1[2] + s2[2];
      const D1 sb2 = s0[3] + s1[3] + s2[3], sb3 = s0[4] + s1[4] + s2[4];
      bool nf = false;
      element_core(M, P.cstat[c].x, P.cstat[c].w, nm[c], h[c], hu[c], hv[c], rc1, rc2, rc3, sb2, sb3, dt, nh[c],
                   nhu[c], nhv[c], nf, 0.0);
    }
    h.swap(nh);
    hu.swap(nhu);
    hv.swap(nhv);
    for (int g = 0; g < G; ++g) {
      const int c = P.iperm[gauges[g]];
      eta[(size_t)s * G + g] = h[c].v + z[c];
      deta[(size_t)s * G + g] = h[c].d[0];
    }
  }
  for (int c = 0; c < n; ++c) {
    const int o = P.perm[c];
    U_out[3 * o] = h[c].v; U_out[3 * o + 1] = hu[c].v; U_out[3 * o + 2] = hv[c].v;
    dU_out[3 * o] = h[c].d[0]; dU_out[3 * o + 1] = hu[c].d[0]; dU_out[3 * o + 2] = hv[c].d[0];
  }
  return 0;
}

/* The dry-region shortcuts of the step against the general evaluation they skip, on n random
 * adversarial cases each: dry_edge_slots against interior_edge (IFLUX 1-3) and
 * interior_edge_muscl (IFLUX 4), every limiter, both
 * flux modes, the three arithmetic types) for two elements of depth +0 with random beds (signed
 * zeros, ties, infinities, NaN), random upwind states (wet ones too), random signs of g, nx, ny
 * and len (zeros included); dry_element against element_update_full with random friction
 * options, thresholds, areas, time steps and signed-zero slots.  Counts the cases a shortcut
 * takes whose bits differ from the general result; *taken returns how many it took. */
extern "C" long long harness_dry_check(long long n, unsigned long long seed, long long* taken) {
  unsigned long long s = seed | 1;
  auto rnd = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  auto unif = [&]() { return (double)(rnd() >> 11) * (1.0 / 9007199254740992.0); };
  auto sgn = [&](double x) { return (rnd() & 1) ? -x : x; };
  auto special = [&](double x) {
    const unsigned k = (unsigned)(rnd() % 16);
    if (k == 0) return 0.0;
    if (k == 1) return -0.0;
    if (k == 2) return (double)INFINITY;
    if (k == 3) return -(double)INFINITY;
    if (k == 4) return (double)NAN;
    return x;
  };
  auto same = [](double a, double b) { return memcmp(&a, &b, 8) == 0; };
  long long bad = 0, took = 0;
  for (long long i = 0; i < n; ++i) {
    /* ---- one edge ---- */
    MemberDev M;
    std::memset(&M, 0, sizeof(M));
    M.gp = (rnd() % 8 == 0) ? special(sgn(9.81)) : sgn(0.5 + 20.0 * unif());
    M.tolisec = (rnd() % 4 == 0) ? 0.0 : 1e-4 * unif();
    EdgeGeo G;
    G.nx = (rnd() % 6 == 0) ? sgn(0.0) : (rnd() % 20 == 0 ? special(1.0) : sgn(unif()));
    G.ny = (rnd() % 6 == 0) ? sgn(0.0) : (rnd() % 20 == 0 ? special(1.0) : sgn(unif()));
    G.len = (rnd() % 8 == 0) ? special(0.3) : 0.01 + 5.0 * unif();
    G.d_mrl = 0.1 + unif(); G.y_mrl = 1.0 / G.d_mrl;
    G.d_mkvol = 0.1 + unif(); G.y_mkvol = 1.0 / G.d_mkvol;
    G.d_mkvoisin = 0.1 + unif(); G.y_mkvoisin = 1.0 / G.d_mkvoisin;
    G.ysum_a = G.ysum_b = 0.5;
    const double zl = (rnd() % 3 == 0) ? special(3.0 * unif()) : 3.0 * unif();
    const double zr = (rnd() % 3 == 0) ? zl : ((rnd() % 3 == 0) ? special(3.0 * unif()) : 3.0 * unif());
    const double up[4] = {(rnd() & 1) ? 2.0 * unif() : 0.0, sgn(unif()), (rnd() & 1) ? 2.0 * unif() : 0.0, sgn(unif())};
    const double zu[2] = {3.0 * unif(), 3.0 * unif()};
    const double dt = 1e-3 + unif();
    const int iflux = 1 + (int)(rnd() % 4), ilim = (int)(rnd() % 5), fm = (int)(rnd() % 2), xd = (int)(rnd() % 3);
    const double huA = sgn(unif()), hvA = sgn(unif()), huB = sgn(unif()), hvB = sgn(unif());
    double o[10];
    auto general = [&](auto tag) {
      using T = decltype(tag);
      T ot[10];
      if (iflux == 1)
        interior_edge<1, T>(M, ilim, fm, G, dt, T(0.0), T(huA), T(hvA), zl, 0.0, T(0.0), T(huB), T(hvB), zr, 0.0,
                            T(up[0]), T(up[1]), zu[0], T(up[2]), T(up[3]), zu[1], ot);
      else if (iflux == 2)
        interior_edge<2, T>(M, ilim, fm, G, dt, T(0.0), T(huA), T(hvA), zl, 0.0, T(0.0), T(huB), T(hvB), zr, 0.0,
                            T(up[0]), T(up[1]), zu[0], T(up[2]), T(up[3]), zu[1], ot);
      else if (iflux == 3)
        interior_edge<3, T>(M, ilim, fm, G, dt, T(0.0), T(huA), T(hvA), zl, 0.0, T(0.0), T(huB), T(hvB), zr, 0.0,
                            T(up[0]), T(up[1]), zu[0], T(up[2]), T(up[3]), zu[1], ot);
      else {
        const T ua[3] = {T(up[0]), T(up[1]), T(-up[3])}, ub[3] = {T(up[2]), T(up[3]), T(up[1])};
        interior_edge_muscl<T>(M, ilim, fm, G, dt, T(0.0), T(huA), T(hvA), zl, 0.0, T(0.0), T(huB), T(hvB), zr, 0.0, ua,
                               zu[0], ub, zu[1], ot);
      }
      for (int k = 0; k < 10; ++k) o[k] = val(ot[k]);
    };
    if (xd == 0) general(0.0);
    else if (xd == 1) general(XD<false>(0.0));
    else general(XD<true>(0.0));
    Slot sl[2];
    const double4 geo = make_double4(G.nx, G.ny, G.len, G.d_mrl);
    const bool took_edge = iflux == 1   ? dry_edge_slots<1>(M.gp, fm, geo, sl, dt)
                           : iflux == 2 ? dry_edge_slots<2>(M.gp, fm, geo, sl, dt)
                           : iflux == 3 ? dry_edge_slots<3>(M.gp, fm, geo, sl, dt)
                                        : dry_edge_slots<4>(M.gp, fm, geo, sl, dt);
    if (took_edge) {
      ++took;
      const double w[10] = {sl[0].f1, sl[0].f2, sl[0].f3, sl[0].bx, sl[0].by, sl[1].f1, sl[1].f2, sl[1].f3, sl[1].bx, sl[1].by};
      bool ok = same(sl[0].q, 0.0) && same(sl[1].q, 0.0);
      for (int k = 0; k < 10; ++k) ok = ok && same(w[k], o[k]);
      if (!ok) ++bad;
    }
    /* ---- one element ---- */
    M.friction = (int)(rnd() % 2);
    M.fricimplic = (int)(rnd() % 3);
    M.tol = 1e-6;
    M.tolisec = (rnd() % 8 == 0) ? special(1e-4) : ((rnd() % 4 == 0) ? 0.0 : 1e-3 * unif());
    const double area = (rnd() % 8 == 0) ? special(sgn(2.0)) : 0.1 + 4.0 * unif();
    const double4 st = make_double4(area, 0.01 + 0.05 * unif(), 0.5 * unif(), 1.0 / area);
    const double4 U = make_double4((rnd() % 8 == 0) ? 1e-5 * unif() : sgn(0.0), (rnd() % 10 == 0) ? special(0.5) : sgn(unif()),
                                   (rnd() % 10 == 0) ? special(0.5) : sgn(unif()), 0.0);
    Slot c[3];
    for (int k = 0; k < 3; ++k) {
      double* f = &c[k].f1;
      for (int j = 0; j < 6; ++j) f[j] = sgn(0.0);
      if (rnd() % 10 == 0) f[rnd() % 5] = sgn(1e-3 * unif());
    }
    const double dte = (rnd() % 10 == 0) ? special(0.05) : sgn(0.05 * unif());
    if (dry_element(M, U, st, c[0], c[1], c[2], dte)) {
      ++took;
      bool nf = true;
      const double4 V = xd == 0 ? element_update_full(M, U, st, c[0], c[1], c[2], dte, nf)
                      : xd == 1 ? element_update_full<XD<false>>(M, U, st, c[0], c[1], c[2], dte, nf)
                                : element_update_full<XD<true>>(M, U, st, c[0], c[1], c[2], dte, nf);
      if (nf || !same(V.x, 0.0) || !same(V.y, 0.0) || !same(V.z, 0.0) || !same(V.w, 0.0)) ++bad;
    }
  }
  if (taken) *taken = took;
  return bad;
}

/* adj_edge_hllc (the reverse edge kernel's closed-form first-order HLLC path) against the generic
 * path it replaces (the edge differentiated in six Dual lanes and contracted with the weights) on n
 * random interior edges: wet, dry and nearly dry sides (clamped reconstructions, masked frames),
 * equal and unequal beds, random normals, velocities and weights.  Returns the largest difference
 * relative to the largest contribution of the edge; *taken counts the edges the path handled. */
#include "../cuteflow_gb300/csrc/cf_dual.h"
extern "C" double harness_adj_hllc_check(long long n, unsigned long long seed, long long* taken) {
  unsigned long long s = seed | 1;
  auto rnd = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  auto unif = [&]() { return (double)(rnd() >> 11) * (1.0 / 9007199254740992.0); };
  double worst = 0.0;
  long long took = 0;
  for (long long i = 0; i < n; ++i) {
    MemberDev M;
    std::memset(&M, 0, sizeof(M));
    M.gp = 9.81;
    M.tolisec = (rnd() & 1) ? 1e-4 : 1e-5;
    auto depth = [&]() {
      const unsigned k = (unsigned)(rnd() % 8);
      if (k == 0) return 0.0;
      if (k == 1) return 0.5 * M.tolisec * unif();
      if (k == 2) return 1e-3 * unif();
      return 0.01 + 5.0 * unif();
    };
    const double hA = depth(), hB = depth();
    auto state = [&](double h) {
      const double u = 3.0 * (unif() - 0.5), v = 3.0 * (unif() - 0.5);
      return make_double4(h, h * u, h * v, h > 0.0 ? 1.0 / h : 0.0);
    };
    const double4 UA = state(hA), UB = state(hB);
    const double ang = 6.283185307179586 * unif();
    EdgeGeo G;
    std::memset(&G, 0, sizeof(G));
    G.nx = std::cos(ang);
    G.ny = std::sin(ang);
    G.len = 0.2 + 2.0 * unif();
    G.d_mrl = 1.0;
    const double zml = (rnd() % 4 == 0) ? 0.0 : 2.0 * unif();
    const double zmr = (rnd() % 4 == 0) ? zml : 2.0 * unif();
    double w[10];
    for (int k = 0; k < 10; ++k) w[k] = unif() - 0.5;
    double la[3], lb[3];
    if (!adj_edge_hllc(M, G, UA, UB, zml, zmr, w, la, lb)) continue;
    ++took;
    Dual<6> o[10];
    auto sd = [](double v, int k) { Dual<6> r(v); r.d[k] = 1.0; return r; };
    interior_edge<1>(M, 1, 0, G, 0.01, sd(UA.x, 0), sd(UA.y, 1), sd(UA.z, 2), zml, UA.w, sd(UB.x, 3), sd(UB.y, 4),
                     sd(UB.z, 5), zmr, UB.w, Dual<6>(0.0), Dual<6>(0.0), 0.0, Dual<6>(0.0), Dual<6>(0.0), 0.0, o);
    double acc[6], scale = 1e-300;
    for (int j = 0; j < 6; ++j) {
      double v = 0.0;
      for (int k = 0; k < 10; ++k) {
        v = std::fma(w[k], o[k].d[j], v);
        scale = std::max(scale, std::fabs(w[k] * o[k].d[j]));
      }
      acc[j] = v;
    }
    const double got[6] = {la[0], la[1], la[2], lb[0], lb[1], lb[2]};
    for (int j = 0; j < 6; ++j) {
      const double d = std::fabs(got[j] - acc[j]);
      if (!(d <= 1e300)) return 1e300;   /* a NaN or an infinity on either side */
      worst = std::max(worst, d / scale);
    }
  }
  if (taken) *taken = took;
  return worst;
}
