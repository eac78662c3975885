/*
 * flux_harness.cpp -- TEST INFRASTRUCTURE.  Compiles the GPU step's per-edge flux mathematics
 * (cuteflow_gb300/csrc/cf_flux.h) and host preprocessing (cf_mesh.cpp) for the CPU so that the
 * tests can compare, edge by edge, the fluxes the edge kernel writes with the oracle's
 * per-(element, edge) evaluation of the reference.  Not part of the product library.
 */
#include "../cuteflow_gb300/csrc/cf_flux.h"

#include <vector>

using namespace cf;

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
    Un[c] = make_double4(U[3 * o], U[3 * o + 1], U[3 * o + 2], P.zcell[c]);
  }
  MemberDev M;
  std::memset(&M, 0, sizeof(M));
  M.gp = p->gp; M.tolisec = p->tolisec; M.tol = p->tol; M.constant_dt = p->constant_dt;
  M.ramp_time = p->ramp_time;
  for (int i = 0; i < CF_MAX_IO; ++i) {
    M.debit_end[i] = p->debitglob[i]; M.debit_start[i] = p->debitglob_start[i];
    M.long_entree[i] = P.long_entree[i]; M.h_sortie[i] = p->h_sortie[i];
  }
  M.inlet = p->inlet; M.outlet = p->outlet; M.friction = p->friction; M.fricimplic = p->fricimplic;
  const int ne = (int)P.edges.size();
  std::vector<Slot> slots(2 * (size_t)ne);
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.Uin = Un.data();
  a.ecell = P.ecell.data(); a.egeo = P.egeo.data(); a.ebid = P.ebid.data();
  a.eupw = P.eupw.empty() ? nullptr : P.eupw.data();
  a.ewts = P.ewts.empty() ? nullptr : P.ewts.data();
  a.edk = P.edk.empty() ? nullptr : P.edk.data();
  a.einv = P.einv.empty() ? nullptr : P.einv.data();
  a.slots = slots.data();
  a.iflux = p->iflux; a.ilimiteur = p->ilimiteur; a.flux_mode = p->flux_mode;
  for (int e = 0; e < ne; ++e) {
    if (p->iflux == 1) edge_body<1>(a, M, e, dt, t);
    else if (p->iflux == 2) edge_body<2>(a, M, e, dt, t);
    else edge_body<3>(a, M, e, dt, t);
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

/* The whole GPU step algorithm on the CPU: edge pass, element pass, device dt rule, for
 * nsteps steps from U (reference order); U_out and dt_hist (nsteps+1) like the oracle. */
extern "C" int harness_run(const cf_mesh* m, const cf_params* p, const double* U, int nsteps, double* U_out,
                           double* dt_hist, double* t_out) {
  Prep P;
  std::string err;
  int rc = prepare_mesh(m, p, P, err);
  if (rc != CF_OK) return rc;
  const int n = P.nelt;
  std::vector<double4> Ua(n), Ub(n);
  for (int c = 0; c < n; ++c) {
    int o = P.perm[c];
    Ua[c] = make_double4(U[3 * o], U[3 * o + 1], U[3 * o + 2], P.zcell[c]);
  }
  MemberDev M;
  std::memset(&M, 0, sizeof(M));
  M.gp = p->gp; M.tolisec = p->tolisec; M.tol = p->tol; M.constant_dt = p->constant_dt;
  M.ramp_time = p->ramp_time; M.dt_reset = (n % 1024 != 0) ? 100000.0 : 1000000.0;
  for (int i = 0; i < CF_MAX_IO; ++i) {
    M.debit_end[i] = p->debitglob[i]; M.debit_start[i] = p->debitglob_start[i];
    M.long_entree[i] = P.long_entree[i]; M.h_sortie[i] = p->h_sortie[i];
  }
  M.inlet = p->inlet; M.outlet = p->outlet; M.friction = p->friction; M.fricimplic = p->fricimplic;
  M.is_dt_constant = p->is_dt_constant;
  const int ne = (int)P.edges.size();
  std::vector<Slot> slots(2 * (size_t)ne);
  StepArgs a;
  std::memset(&a, 0, sizeof(a));
  a.ecell = P.ecell.data(); a.egeo = P.egeo.data(); a.ebid = P.ebid.data();
  a.eupw = P.eupw.empty() ? nullptr : P.eupw.data();
  a.ewts = P.ewts.empty() ? nullptr : P.ewts.data();
  a.edk = P.edk.empty() ? nullptr : P.edk.data();
  a.einv = P.einv.empty() ? nullptr : P.einv.data();
  a.slots = slots.data();
  a.iflux = p->iflux; a.ilimiteur = p->ilimiteur; a.flux_mode = p->flux_mode;
  double4* cur = Ua.data();
  double4* nxt = Ub.data();
  double dt = M.dt_reset;
  for (int c = 0; c < n; ++c) dt = dmin(dt, cfl_dt_elem(M, P.cstat[c].z, cur[c].x, cur[c].y, cur[c].z));
  if (dt_hist) dt_hist[0] = dt;
  double t = 0.0;
  for (int s = 0; s < nsteps; ++s) {
    if (s > 0 && (dt > 9999.0 || dt < DT_LOW)) { rc = -2; break; }
    a.Uin = cur;
    for (int e = 0; e < ne; ++e) {
      if (p->iflux == 1) edge_body<1>(a, M, e, dt, t);
      else if (p->iflux == 2) edge_body<2>(a, M, e, dt, t);
      else edge_body<3>(a, M, e, dt, t);
    }
    double next = M.dt_reset;
    for (int c = 0; c < n; ++c) {
      const int* sl = &P.cslot[c].x;
      bool nf = false;
      nxt[c] = element_update(M, cur[c], P.cstat[c], slots[sl[0]], slots[sl[1]], slots[sl[2]], dt, nf);
      next = dmin(next, cfl_dt_elem(M, P.cstat[c].z, nxt[c].x, nxt[c].y, nxt[c].z));
    }
    t = t + dt;
    dt = next;
    if (dt_hist) dt_hist[s + 1] = dt;
    std::swap(cur, nxt);
  }
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
