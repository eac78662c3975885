/*
 * cf_oracle.cpp -- CPU restatement of the CuteFlow explicit finite-volume St-Venant step.
 *
 * TEST INFRASTRUCTURE ONLY: the correctness checker and the timed CPU baseline of the GPU
 * step in cuteflow_gb300/.  Nothing in the product links, calls or falls back to it.
 *
 * Parity status: pinned against outputs of the reference itself.  Its meshes for the test
 * cases are Git LFS stubs and it cannot be built here (CUDA Fortran + MPI + libcgns), but its
 * calibration folders ship two real CGNS meshes, the boundary tables CuteFlow wrote for them,
 * and the logs of three runs on a Tesla P100 (tests/golden/make_golden.py).  This restatement
 * reproduces both boundary tables exactly and the logged outflow discharge of all three runs
 * to the printed 16 digits at every 1000-step checkpoint (up to 30,000 steps checked).  It is
 * further checked by known-answer properties: lake at rest, mass conservation with walls,
 * mirror symmetry, and the 1-D dam break.
 *
 * Every routine below follows the reference file:line it cites, in the reference's own
 * order of floating-point operations (compile with -ffp-contract=off).  Fortran default-real
 * literals (single precision) are kept as float-rounded doubles.  Where the reference reads
 * an uninitialised variable (quirks Q8/Q9) the defined behaviour chosen here is stated at
 * the place it applies.
 */
#include "cf_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

uint64_t double_bits(double x) {
  uint64_t b;
  std::memcpy(&b, &x, sizeof(b));
  return b;
}
double bits_double(uint64_t b) {
  double x;
  std::memcpy(&x, &b, sizeof(x));
  return x;
}
float bits_float(uint32_t b) {
  float x;
  std::memcpy(&x, &b, sizeof(x));
  return x;
}

/* Fortran default-real literals of the reference, rounded to single precision. */
const double EPS_HLLC = (double)1e-8f;    /* flux_riemann.cuf:926 */
const double EPS_RIADH = (double)1e-6f;   /* flux_riemann.cuf:1051 */
const double EPS_SECOND = (double)1e-16f; /* flux_riemann.cuf:555, :749 */
const double EPS_VLEER = (double)1e-12f;  /* flux_riemann.cuf:454 */
const double F_1_8 = (double)1.8f;        /* maillage.cuf:157 */
const double DT_LOW = (double)1e-12f;     /* cfl_condition.cuf:129 */

struct Setup {
  int nnt = 0, nelt = 0;
  const double *x = nullptr, *y = nullptr, *z = nullptr;
  const int32_t* tri = nullptr;
  std::vector<int32_t> bnd;     /* nelt*3*2, boundary(gi,k,1:2) */
  std::vector<int32_t> nbr_k;   /* local edge index of the shared edge in the neighbour, -1 */
  std::vector<int32_t> upw;     /* nelt*3*2 upwind_cells(1:2,c,gi), 1-based */
  std::vector<double> area, zm, cotemin, xc, yc;
  std::vector<double> long_entree;
};

inline int node(const Setup& S, int gi, int k) { return S.tri[3 * gi + k] - 1; }
inline int32_t& B(Setup& S, int gi, int k, int w) { return S.bnd[(gi * 3 + k) * 2 + w]; }
inline int32_t Bc(const Setup& S, int gi, int k, int w) { return S.bnd[(gi * 3 + k) * 2 + w]; }

/* ---- Mesh preprocessing -------------------------------------------------------------- */

/* Adjacency, maillage.cuf:881-914 (find_neighbour): the neighbour across edge k of cell gi,
 * edge k = (node k, node k+1 mod 3), is a cell gj != gi holding the REVERSED node pair.
 * Cells of inconsistent orientation are therefore not neighbours.  Where several cells
 * qualify (a non-manifold mesh) the reference's result is a race; the smallest gj is taken. */
void build_adjacency(Setup& S) {
  const int n = S.nelt;
  struct DE { uint64_t key; int32_t cell; int32_t k; };
  std::vector<DE> de(3 * (size_t)n);
  for (int gi = 0; gi < n; ++gi)
    for (int k = 0; k < 3; ++k) {
      uint64_t a = (uint32_t)S.tri[3 * gi + k], b = (uint32_t)S.tri[3 * gi + (k + 1) % 3];
      de[3 * gi + k] = {(a << 32) | b, gi, k};
    }
  std::sort(de.begin(), de.end(), [](const DE& p, const DE& q) {
    return p.key < q.key || (p.key == q.key && p.cell < q.cell);
  });
  S.bnd.assign((size_t)n * 6, 0);
  S.nbr_k.assign((size_t)n * 3, -1);
  for (int gi = 0; gi < n; ++gi)
    for (int k = 0; k < 3; ++k) {
      B(S, gi, k, 0) = gi + 1; /* set_boundary, maillage.cuf:850-879 */
      B(S, gi, k, 1) = gi + 1;
    }
  for (int gi = 0; gi < n; ++gi)
    for (int k = 0; k < 3; ++k) {
      uint64_t a = (uint32_t)S.tri[3 * gi + k], b = (uint32_t)S.tri[3 * gi + (k + 1) % 3];
      uint64_t rev = (b << 32) | a;
      auto it = std::lower_bound(de.begin(), de.end(), rev,
                                 [](const DE& p, uint64_t key) { return p.key < key; });
      for (; it != de.end() && it->key == rev; ++it)
        if (it->cell != gi) {
          B(S, gi, k, 0) = it->cell + 1;
          S.nbr_k[gi * 3 + k] = it->k;
          break;
        }
    }
}

/* Node-list membership with the first list position of each node (1-based positions). */
std::vector<int32_t> first_pos(int nnt, int nd, const int32_t* list) {
  std::vector<int32_t> pos(nnt + 1, 0);
  for (int i = nd - 1; i >= 0; --i) {
    int v = list[i];
    if (v >= 1 && v <= nnt) pos[v] = i + 1;
  }
  return pos;
}

/* Boundary tagging, maillage.cuf:981-1110 with assign_type_1(_numero) :1123-1173,
 * assign_type_2 :1201-1225 and set_undefined_boudaries_as_walls :1454-1471.
 * An unmatched edge is inflow (-1) when both endpoints are inflow nodes, else outflow (-2)
 * when both are outflow nodes, else a wall (-3).  The inlet/outlet number is the one of the
 * endpoint listed first (assign_type_1_numero writes numero(gi) with gi < gj). */
void tag_boundaries(Setup& S, const orc_mesh* m) {
  std::vector<int32_t> pin = first_pos(S.nnt, m->ndi, m->ndinput);
  std::vector<int32_t> pout = first_pos(S.nnt, m->ndo, m->ndoutput);
  for (int gi = 0; gi < S.nelt; ++gi)
    for (int k = 0; k < 3; ++k) {
      if (Bc(S, gi, k, 0) != gi + 1) continue;
      int n1 = S.tri[3 * gi + k], n2 = S.tri[3 * gi + (k + 1) % 3];
      if (m->ndi > 0 && n1 != n2 && pin[n1] > 0 && pin[n2] > 0) {
        B(S, gi, k, 0) = -1;
        B(S, gi, k, 1) = m->numero_ndinput[std::min(pin[n1], pin[n2]) - 1];
        continue;
      }
      if (m->ndo > 0 && n1 != n2 && pout[n1] > 0 && pout[n2] > 0) {
        B(S, gi, k, 0) = -2;
        B(S, gi, k, 1) = m->numero_ndoutput[std::min(pout[n1], pout[n2]) - 1];
        continue;
      }
      B(S, gi, k, 0) = -3;
    }
}

/* Upwind cells, maillage.cuf:954-978: for edge c the two cells across edges c+1 and c+2
 * (the cell itself where that edge is not interior). */
void build_upwind(Setup& S) {
  S.upw.assign((size_t)S.nelt * 6, 0);
  for (int gi = 0; gi < S.nelt; ++gi)
    for (int c = 0; c < 3; ++c) {
      int v1 = Bc(S, gi, (c + 1) % 3, 0), v2 = Bc(S, gi, (c + 2) % 3, 0);
      S.upw[(gi * 3 + c) * 2 + 0] = v1 > 0 ? v1 : gi + 1;
      S.upw[(gi * 3 + c) * 2 + 1] = v2 > 0 ? v2 : gi + 1;
    }
}

/* Geometry: area by Heron and distance-weighted cell bed (maillage.cuf:1284-1331),
 * centroids (:1264-1274), CFL length 1.8*0.5*area/semiperimeter (:132-159),
 * inlet lengths (:1423-1452). */
void build_geometry(Setup& S, const orc_mesh* m) {
  const int n = S.nelt;
  S.area.resize(n); S.zm.resize(n); S.cotemin.resize(n); S.xc.resize(n); S.yc.resize(n);
  for (int gi = 0; gi < n; ++gi) {
    int i1 = node(S, gi, 0), i2 = node(S, gi, 1), i3 = node(S, gi, 2);
    double x1 = S.x[i1], y1 = S.y[i1], z1 = S.z[i1];
    double x2 = S.x[i2], y2 = S.y[i2], z2 = S.z[i2];
    double x3 = S.x[i3], y3 = S.y[i3], z3 = S.z[i3];
    double a = std::sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
    double b = std::sqrt((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2));
    double c = std::sqrt((x1 - x3) * (x1 - x3) + (y1 - y3) * (y1 - y3));
    double s = (a + b + c) / 2.;
    S.area[gi] = std::sqrt(s * (s - a) * (s - b) * (s - c));
    double xg = (x1 + x2 + x3) / 3.00, yg = (y1 + y2 + y3) / 3.00;
    double d1 = std::sqrt((x1 - xg) * (x1 - xg) + (y1 - yg) * (y1 - yg));
    double d2 = std::sqrt((x2 - xg) * (x2 - xg) + (y2 - yg) * (y2 - yg));
    double d3 = std::sqrt((x3 - xg) * (x3 - xg) + (y3 - yg) * (y3 - yg));
    S.zm[gi] = (d1 * z1 + d2 * z2 + d3 * z3) / (d1 + d2 + d3);
    S.xc[gi] = (x1 + x2 + x3) / 3;
    S.yc[gi] = (y1 + y2 + y3) / 3;
    double ca = std::sqrt((x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2));
    double cb = std::sqrt((x2 - x3) * (x2 - x3) + (y2 - y3) * (y2 - y3));
    double cc = std::sqrt((x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1));
    double p = (ca + cb + cc) / 2.;
    double aire = std::sqrt(p * (p - ca) * (p - cb) * (p - cc));
    double cm = 0.5 * aire / p;
    S.cotemin[gi] = F_1_8 * cm;
  }
  int ne = std::max(1, std::max(m->nombre_entrees, 1));
  S.long_entree.assign(std::max(ne, ORC_MAX_IO), 0.0);
  for (int gi = 0; gi < n; ++gi)
    for (int k = 0; k < 3; ++k)
      if (Bc(S, gi, k, 0) == -1) {
        int id = Bc(S, gi, k, 1);
        int n1 = node(S, gi, k), n2 = node(S, gi, (k + 1) % 3);
        if (id >= 1 && id <= ORC_MAX_IO)
          S.long_entree[id - 1] += std::sqrt((S.x[n1] - S.x[n2]) * (S.x[n1] - S.x[n2]) +
                                             (S.y[n1] - S.y[n2]) * (S.y[n1] - S.y[n2]));
      }
}

/* the inlet lengths a caller passes (a part of a decomposed mesh takes the whole mesh's) */
void apply_overrides(Setup& S, const orc_params* prm) {
  if (!prm) return;
  for (int i = 0; i < ORC_MAX_IO && i < (int)S.long_entree.size(); ++i)
    if (prm->long_entree[i] > 0.0) S.long_entree[i] = prm->long_entree[i];
}

bool do_setup(Setup& S, const orc_mesh* m) {
  if (!m || m->nelt <= 0 || m->nnt <= 0 || !m->x || !m->y || !m->z || !m->tri) return false;
  S.nnt = m->nnt; S.nelt = m->nelt; S.x = m->x; S.y = m->y; S.z = m->z; S.tri = m->tri;
  for (int i = 0; i < 3 * m->nelt; ++i)
    if (m->tri[i] < 1 || m->tri[i] > m->nnt) return false;
  build_adjacency(S);
  tag_boundaries(S, m);
  build_upwind(S);
  build_geometry(S, m);
  return true;
}

/* ---- x**(-1/3) ------------------------------------------------------------------------- */

/* The reference raises the depth to -1/3 and -4/3 with the compiler's pow
 * (source_terms.cuf:112,119-120,127).  pow is not correctly rounded and differs between math
 * libraries, so the restatement fixes one evaluation of q^(-1/3), with no division:
 *   q = m 2^(3k), m in [1, 8), by integer arithmetic on the exponent field;
 *   a float seed for m^(-1/3): the cubic c0 + u (c1 + u (c2 + u c3)) in u = 1 + f (the leading 23
 *   mantissa bits; c = least-squares fit of u^(-1/3) on [1, 2)), times the float 2^(-r/3), then
 *   y <- y + y (1 - mf y^3) (1/3) in float with mf = u 2^r;
 *   in double: e = 1 - m y^3, y <- y + y e (1/3 + 2e/9), then y 2^(-k).
 * Every step is a named IEEE operation (fma / fmaf where written), within 1.2 ulp of the exact
 * power.  q^(-4/3) = q^(-1/3) / q. */
double rcbrt_normal(uint64_t b) {
  const uint32_t ex = (uint32_t)(b >> 52);
  const uint32_t k3 = (ex + 177u) / 3u;        /* exponent - 1023 + 1200 = 3 k3 + r */
  const uint32_t r = ex + 177u - 3u * k3;
  const uint64_t frac = b & 0x000fffffffffffffull;
  const double m = bits_double(frac | ((uint64_t)(1023u + r) << 52));
  const float u = bits_float((127u << 23) | (uint32_t)(frac >> 29));
  const float mf = bits_float(((127u + r) << 23) | (uint32_t)(frac >> 29));
  const float c0 = 0x1.8ab91ap+0f, c1 = -0x1.9eb31ap-1f, c2 = 0x1.45621ap-2f, c3 = -0x1.99153cp-5f;
  const float s_r[3] = {1.0f, 0x1.965feap-1f, 0x1.428a30p-1f};   /* 2^(-1/3), 2^(-2/3) as floats */
  float y = std::fma(std::fma(std::fma(c3, u, c2), u, c1), u, c0) * s_r[r];
  const float y3 = y * y * y;
  y = std::fma(y, std::fma(-mf, y3, 1.0f) * 0x1.555556p-2f, y);
  const double yd = y;
  const double e = std::fma(-m, yd * yd * yd, 1.0);
  const double v = std::fma(yd, e * std::fma(e, 2.0 / 9.0, 1.0 / 3.0), yd);
  return bits_double(double_bits(v) - (uint64_t)((int64_t)k3 - 400) * (1ull << 52));
}

double rcbrt(double q) {
  const uint64_t b = double_bits(q);
  const uint32_t ex = (uint32_t)(b >> 52);
  if (ex >= 1u && ex <= 2046u) return rcbrt_normal(b);
  if (std::isnan(q)) return q;
  if (q < 0.0) return std::numeric_limits<double>::quiet_NaN();
  if (q == 0.0) return 1.0 / q;
  if (std::isinf(q)) return 0.0;
  return rcbrt_normal(double_bits(q * 0x1p54)) * 0x1p18;      /* subnormal */
}

/* ---- Riemann solvers ---------------------------------------------------------------- */

struct P {
  double gp, tolisec, cfl, tol, dt;
  int iflux, ilimiteur;
};

/* Wave speeds shared by the HLLC / Riadh / WAF / MUSCL solvers (e.g. flux_riemann.cuf:930-983).
 * Returns false when both sides are below eps: the reference then jumps past the speed
 * estimates and reads uninitialised al/ar/pql/pqr (Q9).  Defined here: the flux is zero,
 * which is the reference's value whenever those uninitialised reads are finite. */
bool wave_speeds(double gp, double eps, double hl, double ul, double hr, double ur,
                 double& sl, double& sr, double& set) {
  if (hl < eps && hr < eps) return false;
  double al = std::sqrt(gp * hl);
  double ar = std::sqrt(gp * hr);
  double het = (hl + hr) / 2. - (ur - ul) * (hl + hr) / (al + ar) / 4.;
  double uet = (ul + ur) / 2. - (hr - hl) * (al + ar) / (hl + hr);
  double pql, pqr;
  if (het < hl) pql = 1.;
  else pql = (hl > eps) ? std::sqrt(0.5 * (het + hl) * het / (hl * hl)) : 0.;
  if (het < hr) pqr = 1.;
  else pqr = (hr > eps) ? std::sqrt(0.5 * (het + hr) * het / (hr * hr)) : 0.;
  if (hl > eps) {
    sl = ul - al * pql;
    if (hr > eps) {
      sr = ur + ar * pqr;
    } else {
      sl = ul - al;
      sr = ul + 2 * al;
    }
  } else {
    sl = ur - 2 * ar;
    sr = ur + ar;
  }
  double denom = hr * (ur - sr) - hl * (ul - sl);
  if (std::fabs(denom) < eps) set = uet;
  else set = (sl * hr * (ur - sr) - sr * hl * (ul - sl)) / denom;
  return true;
}

/* solver_Riemann_hllc, flux_riemann.cuf:902-1026 (eps single-precision 1e-8). */
void hllc(double gp, double n1, double n2, double hl, double ul, double vl, double hr, double ur,
          double vr, double flux[3]) {
  const double eps = EPS_HLLC;
  double sl, sr, set;
  if (!wave_speeds(gp, eps, hl, ul, hr, ur, sl, sr, set)) { flux[0] = flux[1] = flux[2] = 0.; return; }
  double q1[3] = {hl, hl * ul, hl * vl}, q2[3] = {hr, hr * ur, hr * vr};
  double f1[3] = {hl * ul, hl * (ul * ul) + gp * hl * hl / 2.0, hl * ul * vl};
  double f2[3] = {hr * ur, hr * (ur * ur) + gp * hr * hr / 2.0, hr * ur * vr};
  double fh[3];
  if (sl > 0) {
    for (int c = 0; c < 3; ++c) fh[c] = f1[c];
  } else if (sr < 0) {
    for (int c = 0; c < 3; ++c) fh[c] = f2[c];
  } else {
    for (int c = 0; c < 3; ++c) fh[c] = (sr * f1[c] - sl * f2[c] + sl * sr * (q2[c] - q1[c])) / (sr - sl + eps);
    fh[2] = (set > 0) ? fh[0] * vl : fh[0] * vr;
  }
  flux[0] = fh[0];
  flux[1] = n1 * fh[1] - n2 * fh[2];
  flux[2] = n2 * fh[1] + n1 * fh[2];
}

/* solver_Riemann_riadh, flux_riemann.cuf:1029-1182 (eps single-precision 1e-6). */
void riadh(double gp, double n1, double n2, double hl, double ul, double vl, double hr, double ur,
           double vr, double flux[3]) {
  const double eps = EPS_RIADH;
  double sl, sr, set;
  if (!wave_speeds(gp, eps, hl, ul, hr, ur, sl, sr, set)) { flux[0] = flux[1] = flux[2] = 0.; return; }
  double q1[3] = {hl, hl * ul, hl * vl}, q2[3] = {hr, hr * ur, hr * vr};
  double pond = (std::fabs(sl - set) > eps) ? hl * (sl - ul) / (sl - set) : 0.0;
  double qe1[3] = {pond, pond * set, pond * vl};
  pond = (std::fabs(sr - set) > eps) ? hr * (sr - ur) / (sr - set) : 0.0;
  double qe2[3] = {pond, pond * set, pond * vr};
  double f1[3] = {hl * ul, hl * (ul * ul) + gp * hl * hl / 2.0, hl * ul * vl};
  double f2[3] = {hr * ur, hr * (ur * ur) + gp * hr * hr / 2.0, hr * ur * vr};
  double fe1[3], fe2[3];
  for (int c = 0; c < 3; ++c) {
    fe1[c] = f1[c] + sl * (qe1[c] - q1[c]);
    fe2[c] = f2[c] + sr * (qe2[c] - q2[c]);
  }
  const double* f;
  if (0. < sl) f = f1;
  else if (0. < set && 0. > sl) f = fe1;
  else if (0. > set && 0. < sr) f = fe2;
  else f = f2;
  flux[0] = f[0];
  flux[1] = n1 * f[1] - n2 * f[2];
  flux[2] = n2 * f[1] + n1 * f[2];
}

/* limiter, flux_riemann.cuf:465-524.  The superbee branch leaves r = 0.5, 1 and 2 to the last
 * branch (Q10); that is kept. */
double waf_limiter(int ilim, double r, double c) {
  double A = 1.;
  if (ilim == 0) {
    A = 1.;
  } else if (ilim == 1) {
    if (r <= 0) A = 1.;
    else if (r > 0. && r < 0.5) A = 1. - 2. * (1. - std::fabs(c)) * r;
    else if (r > 0.5 && r < 1.) A = std::fabs(c);
    else if (r > 1. && r < 2.) A = 1. - (1. - std::fabs(c)) * r;
    else A = 2. * std::fabs(c) - 1.;
  } else if (ilim == 2) {
    if (r <= 0) A = 1.;
    else A = 1 - 2 * (1 - std::fabs(c)) * r / (1 + r);
  } else if (ilim == 3) {
    if (r <= 0) A = 1.;
    else A = 1. - (1. - std::fabs(c)) * r * (1. + r) / (1. + r * r);
  } else if (ilim == 4) {
    if (r <= 0) A = 1.;
    else if (r <= 1) A = 1 - (1 - std::fabs(c)) * r;
    else A = std::fabs(c);
  }
  return A;
}

/* simple_limiter, flux_riemann.cuf:431-463.  ilimiteur values other than 0..3 leave A
 * unset in the reference (intent(inout) garbage); defined here as 0. */
double simple_limiter(int ilim, double r1, double r2) {
  double A = 0.;
  if (ilim == 0) A = 0.;
  else if (ilim == 1) {
    if (r2 > 0) A = std::max(0.0, std::max(std::min(2 * r1, r2), std::min(r1, 2 * r2)));
    else A = std::min(0.0, std::min(std::max(2 * r1, r2), std::max(r1, 2 * r2)));
  } else if (ilim == 2) {
    A = (r1 * r2 + std::fabs(r1 * r2)) / (r1 + r2 + EPS_VLEER);
  } else if (ilim == 3) {
    if (r2 > 0) A = std::max(0.0, std::min(r1, r2));
    else A = std::min(0.0, std::max(r1, r2));
  }
  return A;
}

inline double dsign1(double x) { return std::copysign(1.0, x); }

/* solver_Riemann_waf, flux_riemann.cuf:720-900 (eps single-precision 1e-16). */
void waf(const P& p, double n1, double n2, double hl, double ul, double vl, double hr, double ur,
         double vr, double hl_upw, double vl_upw, double hr_upw, double vr_upw, double d_mrl,
         double d_mkvol, double d_mkvoisin, double flux[3]) {
  const double eps = EPS_SECOND;
  const double gp = p.gp;
  double sl, sr, set;
  if (!wave_speeds(gp, eps, hl, ul, hr, ur, sl, sr, set)) { flux[0] = flux[1] = flux[2] = 0.; return; }
  double q1[3] = {hl, hl * ul, hl * vl}, q2[3] = {hr, hr * ur, hr * vr};
  double f1[3] = {hl * ul, hl * (ul * ul) + gp * hl * hl / 2.0, hl * ul * vl};
  double f2[3] = {hr * ur, hr * (ur * ur) + gp * hr * hr / 2.0, hr * ur * vr};
  double fh[3];
  if (sl > 0) {
    for (int c = 0; c < 3; ++c) fh[c] = f1[c];
  } else if (sr < 0) {
    for (int c = 0; c < 3; ++c) fh[c] = f2[c];
  } else {
    for (int c = 0; c < 3; ++c) fh[c] = (sr * f1[c] - sl * f2[c] + sl * sr * (q2[c] - q1[c])) / (sr - sl + eps);
    fh[2] = (set > 0) ? fh[0] * vl : fh[0] * vr;
  }
  double dtoverdx = p.dt / d_mrl;
  double cr = sr * dtoverdx, cl = sl * dtoverdx, cet = set * dtoverdx;
  double delta_loc_r = (hr - hl) / d_mrl;
  double delta_loc_l = (hr - hl) / d_mrl;
  double delta_loc_et = (vr - vl) / d_mrl;
  double delta_upw_r = (sr > 0) ? (hl - hl_upw) / d_mkvol : (hr_upw - hr) / d_mkvoisin;
  double delta_upw_l = (sl > 0) ? (hl - hl_upw) / d_mkvol : (hr_upw - hr) / d_mkvoisin;
  double delta_upw_et = (set > 0) ? (vl - vl_upw) / d_mkvol : (vr_upw - vr) / d_mkvoisin;
  double rl = delta_upw_l / (delta_loc_l + eps);
  double rr = delta_upw_r / (delta_loc_r + eps);
  double ret = delta_upw_et / (delta_loc_et + eps);
  double limit_l = waf_limiter(p.ilimiteur, rl, cl);
  double limit_r = waf_limiter(p.ilimiteur, rr, cr);
  double limit_et = waf_limiter(p.ilimiteur, ret, cet);
  double wl = (1 + dsign1(sl) * limit_l) / 2.;
  double wlet = (1 + dsign1(set) * limit_et) / 2.;
  double wlr = (dsign1(sr) * limit_r - dsign1(sl) * limit_l) / 2.;
  double wr = (1 - dsign1(sr) * limit_r) / 2.;
  double wret = (1 - dsign1(set) * limit_et) / 2.;
  double fw1 = wl * f1[0] + wlr * fh[0] + wr * f2[0];
  double fw2 = wl * f1[1] + wlr * fh[1] + wr * f2[1];
  double fw3 = (wlet * vl + wret * vr) * fw1;
  flux[0] = fw1;
  flux[1] = n1 * fw2 - n2 * fw3;
  flux[2] = n2 * fw2 + n1 * fw3;
}

/* solver_Riemann_muscl, flux_riemann.cuf:526-718 (eps single-precision 1e-16). */
void muscl(const P& p, double n1, double n2, double hl, double ul, double vl, double hr, double ur,
           double vr, double hl_upw, double ul_upw, double vl_upw, double hr_upw, double ur_upw,
           double vr_upw, double d_mrl, double d_mkvol, double d_mkvoisin, double flux[3]) {
  const double eps = EPS_SECOND;
  const double gp = p.gp, tolisec = p.tolisec;
  const int L = p.ilimiteur;
  double dtoverdx = p.dt / d_mrl;
  double dN1 = (hl - hl_upw) / d_mkvol, dN2 = (ul - ul_upw) / d_mkvol, dN3 = (vl - vl_upw) / d_mkvol;
  double dM1 = (hr - hl) / d_mrl, dM2 = (ur - ul) / d_mrl, dM3 = (vr - vl) / d_mrl;
  double delta_hl = simple_limiter(L, dN1, dM1);
  double hll = std::max(0.0, hl - 0.5 * delta_hl * d_mrl);
  double hlr = std::max(0.0, hl + 0.5 * delta_hl * d_mrl);
  double ull, vll, ulr, vlr;
  if (hlr < tolisec || hll < tolisec) {
    ulr = vlr = ull = vll = 0.;
  } else {
    double delta_ul = simple_limiter(L, dN2, dM2);
    double delta_vl = simple_limiter(L, dN3, dM3);
    ull = ul - 0.5 * delta_ul * d_mrl;
    vll = vl - 0.5 * delta_vl * d_mrl;
    ulr = ul + 0.5 * delta_ul * d_mrl;
    vlr = vl + 0.5 * delta_vl * d_mrl;
  }
  dM1 = (hr_upw - hr) / d_mkvoisin; dM2 = (ur_upw - ur) / d_mkvoisin; dM3 = (vr_upw - vr) / d_mkvoisin;
  dN1 = (hr - hl) / d_mrl; dN2 = (ur - ul) / d_mrl; dN3 = (vr - vl) / d_mrl;
  double delta_hr = simple_limiter(L, dN1, dM1);
  double hrr = std::max(0.0, hr + 0.5 * delta_hr * d_mrl);
  double hrl = std::max(0.0, hr - 0.5 * delta_hr * d_mrl);
  double url, vrl, urr, vrr;
  if (hrl < tolisec || hrr < tolisec) {
    url = vrl = urr = vrr = 0.;
  } else {
    double delta_ur = simple_limiter(L, dN2, dM2);
    double delta_vr = simple_limiter(L, dN3, dM3);
    urr = ur + 0.5 * delta_ur * d_mrl;
    vrr = vr + 0.5 * delta_vr * d_mrl;
    url = ur - 0.5 * delta_ur * d_mrl;
    vrl = vr - 0.5 * delta_vr * d_mrl;
  }
  /* data reconstruction II (:615-621) */
  hl = hlr + 0.5 * dtoverdx * (hll * ull - hlr * ulr);
  ul = ulr + 0.5 * dtoverdx * (hll * (ull * ull) + 0.5 * gp * (hll * hll) - (hlr * (ulr * ulr) + 0.5 * gp * (hlr * hlr)));
  vl = vlr + 0.5 * dtoverdx * (hll * ull * vll - hlr * ulr * vlr);
  hr = hrl + 0.5 * dtoverdx * (hrl * url - hrr * urr);
  ur = url + 0.5 * dtoverdx * (hrl * (url * url) + 0.5 * gp * (hrl * hrl) - (hrr * (urr * urr) + 0.5 * gp * (hrr * hrr)));
  vr = vrl + 0.5 * dtoverdx * (hrl * url * vrl - hrr * urr * vrr);
  double sl, sr, set;
  if (!wave_speeds(gp, eps, hl, ul, hr, ur, sl, sr, set)) { flux[0] = flux[1] = flux[2] = 0.; return; }
  double q1[3] = {hl, hl * ul, hl * vl}, q2[3] = {hr, hr * ur, hr * vr};
  double f1[3] = {hl * ul, hl * (ul * ul) + gp * hl * hl / 2.0, hl * ul * vl};
  double f2[3] = {hr * ur, hr * (ur * ur) + gp * hr * hr / 2.0, hr * ur * vr};
  double fh[3];
  if (sl > 0) {
    for (int c = 0; c < 3; ++c) fh[c] = f1[c];
  } else if (sr < 0) {
    for (int c = 0; c < 3; ++c) fh[c] = f2[c];
  } else {
    for (int c = 0; c < 3; ++c) fh[c] = (sr * f1[c] - sl * f2[c] + sl * sr * (q2[c] - q1[c])) / (sr - sl + eps);
    fh[2] = (set > 0) ? fh[0] * vl : fh[0] * vr;
  }
  flux[0] = fh[0];
  flux[1] = n1 * fh[1] - n2 * fh[2];
  flux[2] = n2 * fh[1] + n1 * fh[2];
}

/* ---- compute_flux for one (cell, edge), flux_riemann.cuf:33-409 ------------------------ */

struct Ctx {
  const Setup* S;
  const orc_mesh* m;
  const orc_params* prm;
  P p;
  double t;  /* time at the start of the step (inflow ramp) */
  double surf[ORC_MAX_IO];  /* phys_inflow: calcul_surf_entree of the step's start state */
};

inline double inlet_discharge(const orc_params* prm, int id, double t) {
  /* debitglob(id); with ramp_time > 0 the discharge ramps linearly from debitglob_start
   * to debitglob over [0, ramp_time] of the time t_n = sum of the dt already used. */
  double q1 = prm->debitglob[id - 1];
  if (prm->ramp_time > 0.0 && t < prm->ramp_time) {
    double q0 = prm->debitglob_start[id - 1];
    return q0 + (q1 - q0) * (t / prm->ramp_time);
  }
  return q1;
}

inline void masked_state(const double* U, double tolisec, double n1, double n2, int k, double& h,
                         double& u, double& v) {
  h = U[3 * k];
  if (h > tolisec) {
    u = (U[3 * k + 1] * n1 + U[3 * k + 2] * n2) / h;
    v = (U[3 * k + 2] * n1 - U[3 * k + 1] * n2) / h;
  } else {
    h = 0.; u = 0.; v = 0.;
  }
}

inline double cdist(const Setup& S, int a, int b) {
  return std::sqrt((S.xc[a] - S.xc[b]) * (S.xc[a] - S.xc[b]) + (S.yc[a] - S.yc[b]) * (S.yc[a] - S.yc[b]));
}

/* Returns the flux of edge tj of cell gi (0-based) and its length; qin/qout receive the
 * discharge diagnostics of boundary edges. */
void cell_edge_flux(const Ctx& C, const double* U0, int gi, int tj, double flux[3], double& ln,
                    double& qin, double& qout) {
  const Setup& S = *C.S;
  const orc_params* prm = C.prm;
  const double gp = C.p.gp, tolisec = C.p.tolisec;
  int nc1 = tj, nc2 = (tj + 1) % 3, nc3 = (tj + 2) % 3;
  int a = node(S, gi, nc1), b = node(S, gi, nc2), c = node(S, gi, nc3);
  double x1 = S.x[a], y1 = S.y[a], x2 = S.x[b], y2 = S.y[b], x3 = S.x[c], y3 = S.y[c];
  ln = std::sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
  double n1 = (y2 - y1) / ln, n2 = (x1 - x2) / ln;
  double orient = n1 * ((x1 + x2) / 2. - (x1 + x2 + x3) / 3.) + n2 * ((y1 + y2) / 2. - (y1 + y2 + y3) / 3.);
  if (orient < 0.) { n1 = (y1 - y2) / ln; n2 = (x2 - x1) / ln; }
  flux[0] = flux[1] = flux[2] = 0.;
  int kvoisin = Bc(S, gi, tj, 0);
  int id = Bc(S, gi, tj, 1);
  double zml = S.zm[gi];
  double hautl, vitul, vitvl;
  masked_state(U0, tolisec, n1, n2, gi, hautl, vitul, vitvl);

  if (kvoisin == -1) {
    if (prm->inlet == 1) {
      flux[0] = hautl * vitul;
      flux[1] = n1 * (hautl * (vitul * vitul) + gp * (hautl * hautl) / 2.) - n2 * hautl * vitul * vitvl;
      flux[2] = n2 * (hautl * (vitul * vitul) + gp * (hautl * hautl) / 2.) + n1 * hautl * vitul * vitvl;
    } else if (prm->inlet == 2) {
      double debitnorm = -inlet_discharge(prm, id, C.t) / S.long_entree[id - 1];
      flux[0] = debitnorm;
      flux[1] = n1 * ((debitnorm * debitnorm) / (hautl + tolisec) + gp * (hautl * hautl) / 2.);
      flux[2] = n2 * ((debitnorm * debitnorm) / (hautl + tolisec) + gp * (hautl * hautl) / 2.);
      qin += (-debitnorm) * ln;
    } else if (prm->inlet == 3) {
      /* phys_inflow, flux_riemann.cuf:127-138: the discharge shared in proportion to depth;
       * 1e-8 is a single-precision literal */
      double surf = (id >= 1 && id <= ORC_MAX_IO) ? C.surf[id - 1] : 0.0;
      double debitnorm = (surf > (double)1e-8f) ? -(inlet_discharge(prm, id, C.t) * hautl / surf) : 0.;
      flux[0] = debitnorm;
      flux[1] = n1 * ((debitnorm * debitnorm) / (hautl + tolisec) + gp * (hautl * hautl) / 2.);
      flux[2] = n2 * ((debitnorm * debitnorm) / (hautl + tolisec) + gp * (hautl * hautl) / 2.);
      qin += (-debitnorm) * ln;
    }
  }
  if (kvoisin == -3) {
    flux[0] = 0.;
    flux[1] = n1 * gp * (hautl * hautl) / 2.;
    flux[2] = n2 * gp * (hautl * hautl) / 2.;
  }
  if (kvoisin == -2 && prm->outlet == 1) {
    if (vitul >= 0. && vitul / std::sqrt(gp * hautl) < 1.0) {
      double h = prm->h_sortie[id - 1] - zml;
      h = std::max(0.0, h);
      flux[0] = h * vitul;
      flux[1] = n1 * (h * (vitul * vitul) + gp * (h * h) / 2.) - n2 * h * vitul * vitvl;
      flux[2] = n2 * (h * (vitul * vitul) + gp * (h * h) / 2.) + n1 * h * vitul * vitvl;
    } else {
      flux[0] = 0.;
      flux[1] = n1 * gp * (hautl * hautl) / 2.;
      flux[2] = n2 * gp * (hautl * hautl) / 2.;
    }
    qout += flux[0] * ln;
  }
  if (kvoisin > 0 || (kvoisin == -2 && prm->outlet == 2)) {
    int kv = (kvoisin > 0) ? kvoisin - 1 : gi;
    double hautr = U0[3 * kv];
    double zmr = S.zm[kv];
    double zij = std::max(zml, zmr);
    double hijet = std::max(0.0, hautl + zml - zij);
    double hjiet = std::max(0.0, hautr + zmr - zij); /* unmasked hautr, as at :180 */
    double vitur, vitvr;
    masked_state(U0, tolisec, n1, n2, kv, hautr, vitur, vitvr);
    double d_mrl = cdist(S, gi, kv);
    if (C.p.iflux == 1 || C.p.iflux == 2) {
      if (hijet < tolisec) { hijet = 0.; vitul = 0.; vitvl = 0.; }
      if (hjiet < tolisec) { hjiet = 0.; vitur = 0.; vitvr = 0.; }
      if (C.p.iflux == 1) hllc(gp, n1, n2, hijet, vitul, vitvl, hjiet, vitur, vitvr, flux);
      else riadh(gp, n1, n2, hijet, vitul, vitvl, hjiet, vitur, vitvr, flux);
    } else {
      /* second-neighbour reconstruction, :229-400 */
      int v1 = S.upw[(gi * 3 + tj) * 2] - 1, v2 = S.upw[(gi * 3 + tj) * 2 + 1] - 1;
      double v1h, v1u, v1v, v2h, v2u, v2v;
      masked_state(U0, tolisec, n1, n2, v1, v1h, v1u, v1v);
      masked_state(U0, tolisec, n1, n2, v2, v2h, v2u, v2v);
      int tjv;
      if (kvoisin > 0) tjv = S.nbr_k[gi * 3 + tj]; /* :262-277 */
      else tjv = tj;                                /* transmissive outlet: the cell itself */
      int w1 = S.upw[(kv * 3 + tjv) * 2] - 1, w2 = S.upw[(kv * 3 + tjv) * 2 + 1] - 1;
      double w1h, w1u, w1v, w2h, w2u, w2v;
      masked_state(U0, tolisec, n1, n2, w1, w1h, w1u, w1v);
      masked_state(U0, tolisec, n1, n2, w2, w2h, w2u, w2v);
      double hl_upw, ul_upw, vl_upw, hr_upw, ur_upw, vr_upw, d_mkvol, d_mkvoisin, zml_upw, zmr_upw;
      if ((v1 == gi && v2 == gi) || (w1 == kv && w2 == kv)) {
        hl_upw = hautl; ul_upw = vitul; vl_upw = vitvl;
        hr_upw = hautr; ur_upw = vitur; vr_upw = vitvr;
        d_mkvol = d_mrl; d_mkvoisin = d_mrl;
        zml_upw = zml; zmr_upw = zmr;
      } else {
        /* Q8: with exactly one upwind cell equal to the cell itself the reference reads the
         * distance to the other one uninitialised (:320-331); it is computed here as the
         * right-hand side does (:342-357). */
        if (v1 == gi) {
          hl_upw = v2h; ul_upw = v2u; vl_upw = v2v;
          d_mkvol = cdist(S, v2, gi);
          zml_upw = S.zm[v2];
        } else if (v2 == gi) {
          hl_upw = v1h; ul_upw = v1u; vl_upw = v1v;
          d_mkvol = cdist(S, v1, gi);
          zml_upw = S.zm[v1];
        } else {
          double d1 = cdist(S, v1, gi), d2 = cdist(S, v2, gi);
          hl_upw = (d1 * v1h + d2 * v2h) / (d1 + d2);
          ul_upw = (d1 * v1u + d2 * v2u) / (d1 + d2);
          vl_upw = (d1 * v1v + d2 * v2v) / (d1 + d2);
          zml_upw = (d1 * S.zm[v1] + d2 * S.zm[v2]) / (d1 + d2);
          d_mkvol = (d1 + d2) / 2.;
        }
        if (w1 == kv) {
          hr_upw = w2h; ur_upw = w2u; vr_upw = w2v;
          d_mkvoisin = cdist(S, w2, kv);
          zmr_upw = S.zm[w2];
        } else if (w2 == kv) {
          hr_upw = w1h; ur_upw = w1u; vr_upw = w1v;
          d_mkvoisin = cdist(S, w1, kv);
          zmr_upw = S.zm[w1];
        } else {
          double d1 = cdist(S, w1, kv), d2 = cdist(S, w2, kv);
          hr_upw = (d1 * w1h + d2 * w2h) / (d1 + d2);
          ur_upw = (d1 * w1u + d2 * w2u) / (d1 + d2);
          vr_upw = (d1 * w1v + d2 * w2v) / (d1 + d2);
          zmr_upw = (d1 * S.zm[w1] + d2 * S.zm[w2]) / (d1 + d2);
          d_mkvoisin = (d1 + d2) / 2.;
        }
      }
      /* hydrostatic reconstruction, :370-400 (both sides masked at this point) */
      zij = std::max(zml, zmr);
      hijet = std::max(0.0, hautl + zml - zij);
      hl_upw = std::max(0.0, hl_upw + zml_upw - zij);
      hjiet = std::max(0.0, hautr + zmr - zij);
      hr_upw = std::max(0.0, hr_upw + zmr_upw - zij);
      if (hijet < tolisec) { hijet = 0.; vitul = 0.; vitvl = 0.; }
      if (hl_upw < tolisec) { hl_upw = 0.; ul_upw = 0.; vl_upw = 0.; }
      if (hjiet < tolisec) { hjiet = 0.; vitur = 0.; vitvr = 0.; }
      if (hr_upw < tolisec) { hr_upw = 0.; ur_upw = 0.; vr_upw = 0.; }
      if (d_mrl == 0.0) {
        /* Transmissive outlet: the reference divides by a zero centroid distance here and
         * produces NaN; defined as the first-order HLLC flux of the edge. */
        hllc(gp, n1, n2, hijet, vitul, vitvl, hjiet, vitur, vitvr, flux);
      } else if (C.p.iflux == 3) {
        waf(C.p, n1, n2, hijet, vitul, vitvl, hjiet, vitur, vitvr, hl_upw, vl_upw, hr_upw, vr_upw,
            d_mrl, d_mkvol, d_mkvoisin, flux);
      } else {
        muscl(C.p, n1, n2, hijet, vitul, vitvl, hjiet, vitur, vitvr, hl_upw, ul_upw, vl_upw, hr_upw,
              ur_upw, vr_upw, d_mrl, d_mkvol, d_mkvoisin, flux);
      }
    }
  }
}

/* calcul_surf_entree, maillage.cuf:1368-1421, on state U: the list of compute_input_elems
 * (:1333-1363) holds an element once per inflow edge, in element order; for inlet id each
 * list entry contributes the element's depth times the length of its last inflow edge of
 * that id (the loop over its edges overwrites s(ti)), 0 when it has none.  Entries are
 * summed in blocks of 32 threads by the tree s(t) = s(t) + s(t+i), i = 16, 8, .., 1, and the
 * block sums added with atomicAdd.  Defined here: blocks are added in block order (the
 * reference's order is whatever order its blocks finish in), and the threads of the last
 * block beyond the list, which read past its end in the reference (the bound tested is
 * nelt, not the list length), contribute 0. */
void surf_entree(const Setup& S, const orc_mesh* m, const double* U, double* surf) {
  std::vector<int> list;
  for (int gi = 0; gi < S.nelt; ++gi)
    for (int j = 0; j < 3; ++j)
      if (Bc(S, gi, j, 0) == -1) list.push_back(gi);
  const int nin = std::max(0, std::min(m->nombre_entrees, ORC_MAX_IO));
  for (int id = 1; id <= ORC_MAX_IO; ++id) surf[id - 1] = 0.0;
  for (int id = 1; id <= nin; ++id) {
    double acc = 0.0;
    for (size_t b0 = 0; b0 < list.size(); b0 += 32) {
      double s[32];
      for (int ti = 0; ti < 32; ++ti) {
        s[ti] = 0.0;
        if (b0 + ti >= list.size()) continue;
        const int kvol = list[b0 + ti];
        for (int kfac = 0; kfac < 3; ++kfac) {
          if (Bc(S, kvol, kfac, 0) == -1 && Bc(S, kvol, kfac, 1) == id) {
            const int n1 = node(S, kvol, kfac), n2 = node(S, kvol, (kfac + 1) % 3);
            s[ti] = std::sqrt((S.x[n1] - S.x[n2]) * (S.x[n1] - S.x[n2]) + (S.y[n1] - S.y[n2]) * (S.y[n1] - S.y[n2])) *
                    U[3 * kvol];
          }
        }
      }
      for (int i = 16; i >= 1; i /= 2)
        for (int ti = 0; ti < i; ++ti) s[ti] = s[ti] + s[ti + i];
      acc = acc + s[0];
    }
    surf[id - 1] = acc;
  }
}

/* compute_source_terms, source_terms.cuf:33-211, and update_sol_with_flux_and_source,
 * finite_volumes_method.cuf:283-304, for one cell. */
void cell_update(const Ctx& C, const double* U0, const double* resc, int gi, double* U) {
  const Setup& S = *C.S;
  const orc_params* prm = C.prm;
  const double gp = C.p.gp, tolisec = C.p.tolisec, tol = C.p.tol, dt = C.p.dt;
  double q1 = U0[3 * gi], q2 = U0[3 * gi + 1], q3 = U0[3 * gi + 2];
  double area = S.area[gi];
  double manning = prm->is_override_manning ? prm->override_manning : C.m->manning_elt[gi];
  double sb[3] = {0., 0., 0.};
  for (int k = 0; k < 3; ++k) {
    int kv = Bc(S, gi, k, 0);
    if (kv > 0) {
      int a = node(S, gi, k), b = node(S, gi, (k + 1) % 3), c = node(S, gi, (k + 2) % 3);
      double x1 = S.x[a], y1 = S.y[a], x2 = S.x[b], y2 = S.y[b], x3 = S.x[c], y3 = S.y[c];
      double ln = std::sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
      double n1 = (y2 - y1) / ln, n2 = (x1 - x2) / ln;
      double orient = n1 * ((x1 + x2) / 2. - (x1 + x2 + x3) / 3.) + n2 * ((y1 + y2) / 2. - (y1 + y2 + y3) / 3.);
      if (orient < 0.) { n1 = (y1 - y2) / ln; n2 = (x2 - x1) / ln; }
      double zij = std::max(S.zm[gi], S.zm[kv - 1]);
      double hijet = q1 + S.zm[gi] - zij;
      hijet = std::max(0.0, hijet);
      sb[1] = sb[1] + gp / 2.0 * (hijet * hijet - q1 * q1) * ln * n1;
      sb[2] = sb[2] + gp / 2.0 * (hijet * hijet - q1 * q1) * ln * n2;
    }
  }
  double sf[3] = {0., 0., 0.};
  double afm1[9] = {1., 0., 0., 0., 1., 0., 0., 0., 1.};
  if (prm->friction == 1) {
    double normvit = 0.;
    double vitu = 0., vitv = 0.;
    if (q1 > tolisec) {
      vitu = q2 / q1;
      vitv = q3 / q1;
      normvit = std::sqrt(vitu * vitu + vitv * vitv);
      if (normvit < tol) normvit = tol;
      const double p13 = rcbrt(q1); /* q1**(-1/3) */
      sf[1] = -(gp * manning * manning * vitu * normvit * area * p13);
      sf[2] = -(gp * manning * manning * vitv * normvit * area * p13);
    }
    if (prm->fricimplic == 1) {
      if (normvit > tol && q1 > tolisec) {
        double dtgn2h = dt / 2.0 * gp * manning * manning * (rcbrt(q1) / q1);
        double af21 = -(7.0 / 3.0 * dtgn2h * vitu * normvit);
        double af22 = 1.0 + dtgn2h * (2 * (vitu * vitu) + vitv * vitv) / normvit;
        double af23 = dtgn2h * vitu * vitv / normvit;
        double af31 = -(7.0 / 3.0 * dtgn2h * vitv * normvit);
        double af32 = af23;
        double af33 = 1.0 + dtgn2h * (vitu * vitu + 2 * (vitv * vitv)) / normvit;
        double detaf = af22 * af33 - af23 * af32;
        afm1[0] = 1; afm1[1] = 0.; afm1[2] = 0.;
        afm1[3] = -(af21 * af33 - af23 * af31) / detaf;
        afm1[4] = af33 / detaf;
        afm1[5] = -af23 / detaf;
        afm1[6] = (af21 * af32 - af22 * af31) / detaf;
        afm1[7] = -af32 / detaf;
        afm1[8] = af22 / detaf;
      }
    } else if (prm->fricimplic == 2) {
      if (normvit > tol && q1 > tolisec) {
        double beta = -(dt * gp * manning * manning * normvit * (rcbrt(q1) / q1));
        double detaf = (1 - beta) * (1 - beta);
        afm1[4] = (1 - beta) / detaf;
        afm1[8] = (1 - beta) / detaf;
      }
    }
  }
  double res[3];
  const double* rc = resc + 3 * gi;
  if (prm->friction == 1) {
    if (prm->fricimplic == 1 || prm->fricimplic == 2) {
      double ri[3];
      for (int c = 0; c < 3; ++c) ri[c] = (sb[c] + sf[c] - rc[c]) / area;
      for (int c = 0; c < 3; ++c) res[c] = afm1[3 * c] * ri[0] + afm1[3 * c + 1] * ri[1] + afm1[3 * c + 2] * ri[2];
    } else {
      for (int c = 0; c < 3; ++c) res[c] = (sb[c] + sf[c] - rc[c]) / area;
    }
  } else {
    for (int c = 0; c < 3; ++c) res[c] = (sb[c] - rc[c]) / area;
  }
  for (int c = 0; c < 3; ++c) U[3 * gi + c] = U0[3 * gi + c] + dt * res[c];
  if (U[3 * gi] <= tolisec) { U[3 * gi] = 0.; U[3 * gi + 1] = 0.; U[3 * gi + 2] = 0.; }
}

/* cflcond + reduction, cfl_condition.cuf:4-39, :68-104.  The tree reduction pads a partial
 * last block of 1024 threads with 1e5, and dt_d starts from 1e6. */
double cfl_dt(const Setup& S, const orc_params* prm, const double* U) {
  const int n = S.nelt;
  double dtmin = 1000000.0;
#pragma omp parallel for reduction(min : dtmin) schedule(static)
  for (int gi = 0; gi < n; ++gi) {
    double d = 1000000.0;
    double h = U[3 * gi];
    if (h > prm->tolisec) {
      double vu = U[3 * gi + 1] / h, vv = U[3 * gi + 2] / h;
      double nv = std::sqrt(vu * vu + vv * vv);
      double vmax = std::max(0.01, nv + std::sqrt(prm->gp * std::fabs(h)));
      d = std::min(prm->cfl * S.cotemin[gi] / vmax, 1000000.0);
    }
    if (prm->is_dt_constant == 1) d = prm->constant_dt;
    dtmin = std::min(dtmin, d);
  }
  if (((prm->dt_reset_nelt > 0) ? prm->dt_reset_nelt : n) % 1024 != 0) dtmin = std::min(dtmin, 100000.0);
  return dtmin;
}

}  // namespace

extern "C" {

/* flux*len of edge tj of element gi (0-based) for state U at time t with time step dt;
 * fl_out: 3 doubles, flux_riemann.cuf:411-426 before the per-element sum. */
int orc_edge_flux(const orc_mesh* m, const orc_params* prm, const double* U, double dt, double t,
                  int32_t gi, int32_t tj, double* fl_out) {
  Setup S;
  if (!prm || !U || !fl_out || !do_setup(S, m) || gi < 0 || gi >= m->nelt || tj < 0 || tj > 2) return -1;
  apply_overrides(S, prm);
  Ctx C;
  C.S = &S; C.m = m; C.prm = prm;
  C.p.gp = prm->gp; C.p.tolisec = prm->tolisec; C.p.cfl = prm->cfl; C.p.tol = prm->tol;
  C.p.iflux = prm->iflux; C.p.ilimiteur = prm->ilimiteur; C.p.dt = dt;
  C.t = t;
  surf_entree(S, m, U, C.surf);
  double f[3], ln, qi = 0., qo = 0.;
  cell_edge_flux(C, U, gi, tj, f, ln, qi, qo);
  for (int c = 0; c < 3; ++c) fl_out[c] = f[c] * ln;
  return 0;
}

/* All 3*nelt edge fluxes (flux*len, [gi][tj][c]) of state U, evaluated per (element, edge). */
int orc_all_edge_fluxes(const orc_mesh* m, const orc_params* prm, const double* U, double dt,
                        double t, double* fl_out) {
  Setup S;
  if (!prm || !U || !fl_out || !do_setup(S, m)) return -1;
  apply_overrides(S, prm);
  Ctx C;
  C.S = &S; C.m = m; C.prm = prm;
  C.p.gp = prm->gp; C.p.tolisec = prm->tolisec; C.p.cfl = prm->cfl; C.p.tol = prm->tol;
  C.p.iflux = prm->iflux; C.p.ilimiteur = prm->ilimiteur; C.p.dt = dt;
  C.t = t;
  surf_entree(S, m, U, C.surf);
  for (int gi = 0; gi < m->nelt; ++gi)
    for (int tj = 0; tj < 3; ++tj) {
      double f[3], ln, qi = 0., qo = 0.;
      cell_edge_flux(C, U, gi, tj, f, ln, qi, qo);
      for (int c = 0; c < 3; ++c) fl_out[(gi * 3 + tj) * 3 + c] = f[c] * ln;
    }
  return 0;
}

/* x^(-1/3) of the friction term, elementwise (the restatement's fixed evaluation). */
void orc_rcbrt(const double* x, double* y, int64_t n) {
  for (int64_t i = 0; i < n; ++i) y[i] = rcbrt(x[i]);
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int orc_setup(const orc_mesh* m, int32_t* boundary, double* area, double* zm, double* cotemin,
              double* xc, double* yc) {
  Setup S;
  if (!do_setup(S, m)) return -1;
  const size_t n = (size_t)m->nelt;
  if (boundary) std::memcpy(boundary, S.bnd.data(), n * 6 * sizeof(int32_t));
  if (area) std::memcpy(area, S.area.data(), n * sizeof(double));
  if (zm) std::memcpy(zm, S.zm.data(), n * sizeof(double));
  if (cotemin) std::memcpy(cotemin, S.cotemin.data(), n * sizeof(double));
  if (xc) std::memcpy(xc, S.xc.data(), n * sizeof(double));
  if (yc) std::memcpy(yc, S.yc.data(), n * sizeof(double));
  return 0;
}

/* set_initial_condition, initial_condition.cuf:18-79. */
int orc_initial_condition(const orc_mesh* m, const orc_params* p, const orc_ic* ic, double* U0) {
  Setup S;
  if (!do_setup(S, m) || !ic || !U0) return -1;
  const double tolisec = p->tolisec;
  for (int gi = 0; gi < S.nelt; ++gi) {
    double zmd = S.zm[gi];
    int i1 = node(S, gi, 0), i2 = node(S, gi, 1), i3 = node(S, gi, 2);
    double v1 = (S.x[i1] + S.x[i2] + S.x[i3]) / 3;
    double v2 = (S.y[i1] + S.y[i2] + S.y[i3]) / 3;
    double* u = U0 + 3 * gi;
    if (ic->eqlin_barrage == 1) {
      double alpha = (ic->y1eqbar - ic->y2eqbar) / (ic->x1eqbar - ic->x2eqbar);
      double beta = ic->y1eqbar - alpha * ic->x1eqbar;
      double h, uu, vv;
      if (alpha * v1 - v2 + beta >= 0.00) { h = ic->h_amont - zmd; uu = ic->u_amont; vv = ic->v_amont; }
      else { h = ic->h_aval - zmd; uu = ic->u_aval; vv = ic->v_aval; }
      u[0] = h;
      if (h > tolisec) { u[1] = h * uu; u[2] = h * vv; }
      else { u[0] = 0.; u[1] = 0.; u[2] = 0.; }
    }
    if (ic->plan == 1) {
      double h = (-(ic->xplan * (ic->xpoint - v1)) - ic->yplan * (ic->ypoint - v2)) / ic->zplan + ic->zpoint - zmd;
      u[0] = h;
      if (h > tolisec) { u[1] = h * ic->u_aval; u[2] = h * ic->v_aval; }
      else { u[0] = 0.; u[1] = 0.; u[2] = 0.; }
    }
  }
  return 0;
}

/* The time loop of solve_finite_volumes, finite_volumes_method.cuf:113-242, for nsteps. */
int orc_run(const orc_mesh* m, const orc_params* prm, const double* U0in, double t0, int32_t nsteps,
            double* U_out, double* dt_hist, const double* dt_replay, double* t_out, double* q_out,
            int32_t nthreads, double* loop_seconds, int32_t* steps_out) {
#ifdef _OPENMP
  int saved = omp_get_max_threads();
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  Setup S;
  if (!prm || !U0in || !U_out || nsteps < 0 || !do_setup(S, m) ||
      (!prm->is_override_manning && !m->manning_elt) || prm->iflux < 1 || prm->iflux > 4) {
#ifdef _OPENMP
    omp_set_num_threads(saved);
#endif
    return -1;
  }
  apply_overrides(S, prm);
  const int n = S.nelt;
  const bool two_sided = prm->flux_mode == 0;
  std::vector<double> Ua(U0in, U0in + 3 * (size_t)n), Ub(3 * (size_t)n, 0.0);
  std::vector<double> fl(9 * (size_t)n, 0.0); /* flux*len per (cell, edge, component) */
  std::vector<double> resc(3 * (size_t)n, 0.0);
  double* U0 = Ua.data();
  double* U = Ub.data();
  Ctx C;
  C.S = &S; C.m = m; C.prm = prm;
  C.p.gp = prm->gp; C.p.tolisec = prm->tolisec; C.p.cfl = prm->cfl; C.p.tol = prm->tol;
  C.p.iflux = prm->iflux; C.p.ilimiteur = prm->ilimiteur;
  double dt = cfl_dt(S, prm, U0);
  if (dt_hist) dt_hist[0] = dt;
  double t = t0, qin = 0., qout = 0.;
  int rc = 0, done = 0, steady_iter = 0;
  /* boundary (cell, edge) pairs in reference order: their discharges are summed in this
   * order after every step (finite_volumes_method.cuf:197-214), so that the sums do not
   * depend on the thread count */
  std::vector<int> bpos(3 * (size_t)n, -1);
  int nb = 0;
  for (int gi = 0; gi < n; ++gi)
    for (int tj = 0; tj < 3; ++tj)
      if (Bc(S, gi, tj, 0) < 0) bpos[gi * 3 + tj] = nb++;
  std::vector<double> bq_in((size_t)nb, 0.0), bq_out((size_t)nb, 0.0);
  for (int i = 0; i < ORC_MAX_IO; ++i) C.surf[i] = 0.0;
  const auto wall0 = std::chrono::steady_clock::now();
  for (int step = 0; step < nsteps; ++step) {
    C.p.dt = dt_replay ? dt_replay[step] : dt;
    C.t = t;
    if (prm->inlet == 3) surf_entree(S, m, U0, C.surf);
    /* compute_flux: per (cell, edge); in the once-per-edge mode the cell with the larger
     * index takes the negated flux of its neighbour instead of evaluating it. */
#pragma omp parallel for schedule(static)
    for (int gi = 0; gi < n; ++gi)
      for (int tj = 0; tj < 3; ++tj) {
        int kv = Bc(S, gi, tj, 0);
        if (!two_sided && kv > 0 && kv - 1 < gi) continue;
        double f[3], ln, qi = 0., qo = 0.;
        cell_edge_flux(C, U0, gi, tj, f, ln, qi, qo);
        for (int c = 0; c < 3; ++c) fl[(gi * 3 + tj) * 3 + c] = f[c] * ln;
        if (kv < 0) {
          bq_in[bpos[gi * 3 + tj]] = qi;
          bq_out[bpos[gi * 3 + tj]] = qo;
        }
      }
    qin = 0.;
    qout = 0.;
    for (int i = 0; i < nb; ++i) {
      qin += bq_in[i];
      qout += bq_out[i];
    }
    if (!two_sided) {
#pragma omp parallel for schedule(static)
      for (int gi = 0; gi < n; ++gi)
        for (int tj = 0; tj < 3; ++tj) {
          int kv = Bc(S, gi, tj, 0);
          if (kv > 0 && kv - 1 < gi) {
            int k2 = S.nbr_k[gi * 3 + tj];
            for (int c = 0; c < 3; ++c) fl[(gi * 3 + tj) * 3 + c] = -fl[((kv - 1) * 3 + k2) * 3 + c];
          }
        }
    }
#pragma omp parallel for schedule(static)
    for (int gi = 0; gi < n; ++gi)
      for (int c = 0; c < 3; ++c)
        resc[3 * gi + c] = fl[(gi * 3 + 0) * 3 + c] + fl[(gi * 3 + 1) * 3 + c] + fl[(gi * 3 + 2) * 3 + c];
    /* compute_source_terms + update_sol_with_flux_and_source */
#pragma omp parallel for schedule(static)
    for (int gi = 0; gi < n; ++gi) cell_update(C, U0, resc.data(), gi, U);
    /* compute_time_step */
    dt = cfl_dt(S, prm, U);
    if (dt_hist) dt_hist[step + 1] = dt;
    t = t + C.p.dt;
    std::swap(U0, U);
    ++done;
    /* check_steady_state, finite_volumes_method.cuf:370-393 (1e-8 single precision) */
    if (prm->tol_reg_perm > 0.0) {
      const int count = prm->steady_count > 0 ? prm->steady_count : 1000;
      if (qin > (double)1e-8f && std::fabs(qin - qout) / qin < prm->tol_reg_perm) {
        if (++steady_iter > count) { rc = 1; break; }
      } else {
        steady_iter = 0;
      }
    }
    if (!dt_replay && (dt > 9999 || dt < DT_LOW)) { rc = -2; break; }
  }
  if (steps_out) *steps_out = done;
  if (loop_seconds)
    *loop_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - wall0).count();
  std::memcpy(U_out, U0, 3 * (size_t)n * sizeof(double));
  if (t_out) *t_out = t;
  if (q_out) { q_out[0] = qin; q_out[1] = qout; }
#ifdef _OPENMP
  omp_set_num_threads(saved);
#endif
  return rc;
}

}  // extern "C"
