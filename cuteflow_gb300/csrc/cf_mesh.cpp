/*
 * cf_mesh.cpp -- host preprocessing of the reference mesh inputs into the device layout.
 *
 * Replaces the reference's setup kernels and host loops (maillage.cuf): the O(N^2)
 * all-pairs neighbour search (find_neighbour, :881-914) becomes a sort of directed edges,
 * the per-boundary-edge kernel launches of boundary_kind (:981-1110) become one pass over
 * node-list membership, and the geometry (:132-165, :1254-1331, :1423-1452) is computed
 * once in the same floating-point order as the reference (this file is compiled with
 * -ffp-contract=off, so area, cell bed and CFL length are bit-identical to a plain FP64
 * evaluation of the reference formulas).
 *
 * Elements are then renumbered along a Hilbert curve of their centroids and every edge is
 * stored once, next to the elements that use it, with its normal and length precomputed.
 */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "cf_flux.h"
#include "cf_internal.h"

namespace cf {
namespace {

/* Hilbert index of (x, y) on a 2^order grid (the iterative xy -> d conversion with
 * quadrant rotation). */
uint64_t hilbert_index(uint32_t x, uint32_t y, int order) {
  const uint32_t n = 1u << order;
  uint64_t d = 0;
  for (uint32_t s = n >> 1; s > 0; s >>= 1) {
    uint32_t rx = (x & s) ? 1u : 0u;
    uint32_t ry = (y & s) ? 1u : 0u;
    d += (uint64_t)s * (uint64_t)s * (uint64_t)((3u * rx) ^ ry);
    if (ry == 0) {
      if (rx == 1) {
        x = n - 1 - x;
        y = n - 1 - y;
      }
      std::swap(x, y);
    }
  }
  return d;
}

/* Morton (Z-order) index of (x, y): the bits of x and y interleaved, x in the even bits. */
uint64_t morton_index(uint32_t x, uint32_t y) {
  auto spread = [](uint64_t v) {
    v &= 0xffffffffull;
    v = (v | (v << 16)) & 0x0000ffff0000ffffull;
    v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
    v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
    v = (v | (v << 2)) & 0x3333333333333333ull;
    v = (v | (v << 1)) & 0x5555555555555555ull;
    return v;
  };
  return spread(x) | (spread(y) << 1);
}

inline int nd(const cf_mesh* m, int e, int k) { return m->tri[3 * e + k] - 1; }

/* Unit normal and length of local edge k of element e, oriented out of the element by the
 * centroid test of flux_riemann.cuf:56-74 (and source_terms.cuf:70-88). */
void edge_normal(const cf_mesh* m, int e, int k, double& n1, double& n2, double& ln) {
  int a = nd(m, e, k), b = nd(m, e, (k + 1) % 3), c = nd(m, e, (k + 2) % 3);
  double x1 = m->x[a], y1 = m->y[a], x2 = m->x[b], y2 = m->y[b], x3 = m->x[c], y3 = m->y[c];
  ln = std::sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
  n1 = (y2 - y1) / ln;
  n2 = (x1 - x2) / ln;
  double orient = n1 * ((x1 + x2) / 2. - (x1 + x2 + x3) / 3.) + n2 * ((y1 + y2) / 2. - (y1 + y2 + y3) / 3.);
  if (orient < 0.) {
    n1 = (y1 - y2) / ln;
    n2 = (x2 - x1) / ln;
  }
}

}  // namespace

int prepare_mesh(const cf_mesh* m, const cf_params* p, Prep& P, std::string& err, const int32_t* elem_class) {
  if (!m || !p) { err = "null mesh or params"; return CF_EINVAL; }
  const int n = m->nelt, nnt = m->nnt;
  if (n <= 0 || nnt <= 0 || !m->x || !m->y || !m->z || !m->tri) { err = "empty mesh"; return CF_EINVAL; }
  if (!p->is_override_manning && !m->manning_elt) { err = "manning_elt is NULL without is_override_manning"; return CF_EINVAL; }
  if ((m->ndi > 0 && (!m->ndinput || !m->numero_ndinput)) || (m->ndo > 0 && (!m->ndoutput || !m->numero_ndoutput)) ||
      (m->ndw > 0 && !m->ndwall) || m->ndi < 0 || m->ndo < 0 || m->ndw < 0) {
    err = "inconsistent boundary node lists";
    return CF_EINVAL;
  }
  for (int64_t i = 0; i < 3 * (int64_t)n; ++i)
    if (m->tri[i] < 1 || m->tri[i] > nnt) { err = "connectivity refers to a node outside 1..nnt"; return CF_EINVAL; }
  P.nelt = n;
  P.nnt = nnt;

  /* -- adjacency: neighbour across edge (a,b) holds the directed edge (b,a) -------------- */
  std::vector<uint64_t> key(3 * (size_t)n);
  std::vector<int32_t> order(3 * (size_t)n);
  for (int e = 0; e < n; ++e)
    for (int k = 0; k < 3; ++k) {
      uint64_t a = (uint32_t)m->tri[3 * e + k], b = (uint32_t)m->tri[3 * e + (k + 1) % 3];
      key[3 * e + k] = (a << 32) | b;
    }
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int32_t i, int32_t j) {
    return key[i] < key[j] || (key[i] == key[j] && i < j);
  });
  std::vector<uint64_t> skey(order.size());
  for (size_t i = 0; i < order.size(); ++i) skey[i] = key[order[i]];
  P.bnd.assign((size_t)n * 6, 0);
  P.nbr_k.assign((size_t)n * 3, -1);
  for (int e = 0; e < n; ++e)
    for (int k = 0; k < 3; ++k) {
      P.bnd[(e * 3 + k) * 2 + 0] = e + 1;
      P.bnd[(e * 3 + k) * 2 + 1] = e + 1;
      uint64_t a = (uint32_t)m->tri[3 * e + k], b = (uint32_t)m->tri[3 * e + (k + 1) % 3];
      uint64_t rev = (b << 32) | a;
      size_t lo = std::lower_bound(skey.begin(), skey.end(), rev) - skey.begin();
      for (size_t i = lo; i < skey.size() && skey[i] == rev; ++i) {
        int other = order[i] / 3;
        if (other != e) { /* smallest qualifying element (sorted by position) */
          P.bnd[(e * 3 + k) * 2 + 0] = other + 1;
          P.nbr_k[e * 3 + k] = order[i] % 3;
          break;
        }
      }
    }

  /* -- boundary kinds: inflow if both ends are inflow nodes, else outflow, else wall ------- */
  std::vector<int32_t> pin(nnt + 1, 0), pout(nnt + 1, 0);
  for (int i = m->ndi - 1; i >= 0; --i) {
    int v = m->ndinput[i];
    if (v >= 1 && v <= nnt) pin[v] = i + 1;
  }
  for (int i = m->ndo - 1; i >= 0; --i) {
    int v = m->ndoutput[i];
    if (v >= 1 && v <= nnt) pout[v] = i + 1;
  }
  for (int e = 0; e < n; ++e)
    for (int k = 0; k < 3; ++k) {
      int32_t* b = &P.bnd[(e * 3 + k) * 2];
      if (b[0] != e + 1) continue;
      int n1 = m->tri[3 * e + k], n2 = m->tri[3 * e + (k + 1) % 3];
      if (m->ndi > 0 && n1 != n2 && pin[n1] && pin[n2]) {
        b[0] = -1;
        b[1] = m->numero_ndinput[std::min(pin[n1], pin[n2]) - 1];
      } else if (m->ndo > 0 && n1 != n2 && pout[n1] && pout[n2]) {
        b[0] = -2;
        b[1] = m->numero_ndoutput[std::min(pout[n1], pout[n2]) - 1];
      } else {
        b[0] = -3;
      }
      if ((b[0] == -1 || b[0] == -2) && (b[1] < 1 || b[1] > CF_MAX_IO)) {
        err = "inlet/outlet number outside 1..20";
        return CF_EINVAL;
      }
    }

  /* -- geometry in reference order ------------------------------------------------------ */
  P.area.resize(n); P.zm.resize(n); P.cotemin.resize(n); P.xc.resize(n); P.yc.resize(n);
  const double f18 = (double)1.8f;
  for (int e = 0; e < n; ++e) {
    int i1 = nd(m, e, 0), i2 = nd(m, e, 1), i3 = nd(m, e, 2);
    double x1 = m->x[i1], y1 = m->y[i1], z1 = m->z[i1];
    double x2 = m->x[i2], y2 = m->y[i2], z2 = m->z[i2];
    double x3 = m->x[i3], y3 = m->y[i3], z3 = m->z[i3];
    double a = std::sqrt((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1));
    double b = std::sqrt((x3 - x2) * (x3 - x2) + (y3 - y2) * (y3 - y2));
    double c = std::sqrt((x1 - x3) * (x1 - x3) + (y1 - y3) * (y1 - y3));
    double s = (a + b + c) / 2.;
    double ar = std::sqrt(s * (s - a) * (s - b) * (s - c));
    if (!(ar > 0.0)) { err = "degenerate element (zero area)"; return CF_EINVAL; }
    P.area[e] = ar;
    double xg = (x1 + x2 + x3) / 3.00, yg = (y1 + y2 + y3) / 3.00;
    double d1 = std::sqrt((x1 - xg) * (x1 - xg) + (y1 - yg) * (y1 - yg));
    double d2 = std::sqrt((x2 - xg) * (x2 - xg) + (y2 - yg) * (y2 - yg));
    double d3 = std::sqrt((x3 - xg) * (x3 - xg) + (y3 - yg) * (y3 - yg));
    P.zm[e] = (d1 * z1 + d2 * z2 + d3 * z3) / (d1 + d2 + d3);
    P.xc[e] = (x1 + x2 + x3) / 3;
    P.yc[e] = (y1 + y2 + y3) / 3;
    /* maillage.cuf:148-157 measures the sides in the other direction; the squares agree. */
    double half_area_over_p = 0.5 * ar / s;
    P.cotemin[e] = f18 * half_area_over_p;
  }
  for (int i = 0; i < CF_MAX_IO; ++i) P.long_entree[i] = 0.0;
  for (int e = 0; e < n; ++e)
    for (int k = 0; k < 3; ++k)
      if (P.bnd[(e * 3 + k) * 2] == -1) {
        int id = P.bnd[(e * 3 + k) * 2 + 1];
        int a = nd(m, e, k), b = nd(m, e, (k + 1) % 3);
        P.long_entree[id - 1] += std::sqrt((m->x[a] - m->x[b]) * (m->x[a] - m->x[b]) +
                                           (m->y[a] - m->y[b]) * (m->y[a] - m->y[b]));
      }
  for (int i = 0; i < CF_MAX_IO; ++i)
    if (p->long_entree[i] > 0.0) P.long_entree[i] = p->long_entree[i];   /* a part of a decomposed mesh */
  if (p->inlet == 2)
    for (int e = 0; e < n; ++e)
      for (int k = 0; k < 3; ++k)
        if (P.bnd[(e * 3 + k) * 2] == -1 && !(P.long_entree[P.bnd[(e * 3 + k) * 2 + 1] - 1] > 0.0)) {
          err = "inflow edges with zero total inlet length";
          return CF_EINVAL;
        }

  /* -- renumbering along a space-filling curve of the centroids: reorder 1 Hilbert, 2 Morton,
   * 0 the caller's order ------------------------------------------------------------------ */
  P.perm.resize(n);
  P.iperm.resize(n);
  std::iota(P.perm.begin(), P.perm.end(), 0);
  if (elem_class)
    for (int e = 0; e < n; ++e)
      if (elem_class[e] < 0 || elem_class[e] > 2) {
        err = "element class outside 0..2";
        return CF_EINVAL;
      }
  if (p->reorder == 1 || p->reorder == 2) {
    double xmin = P.xc[0], xmax = P.xc[0], ymin = P.yc[0], ymax = P.yc[0];
    for (int e = 1; e < n; ++e) {
      xmin = std::min(xmin, P.xc[e]); xmax = std::max(xmax, P.xc[e]);
      ymin = std::min(ymin, P.yc[e]); ymax = std::max(ymax, P.yc[e]);
    }
    const int order_bits = 16;
    const double span = std::max(xmax - xmin, ymax - ymin);
    const double scale = span > 0 ? ((double)((1u << order_bits) - 1)) / span : 0.0;
    std::vector<uint64_t> h(n);
    for (int e = 0; e < n; ++e) {
      uint32_t ix = (uint32_t)((P.xc[e] - xmin) * scale), iy = (uint32_t)((P.yc[e] - ymin) * scale);
      h[e] = p->reorder == 1 ? hilbert_index(ix, iy, order_bits) : morton_index(ix, iy);
    }
    std::stable_sort(P.perm.begin(), P.perm.end(), [&](int32_t i, int32_t j) { return h[i] < h[j]; });
  }
  P.n_send = P.n_own = 0;
  if (elem_class) {
    /* a part: send elements first, then the other owned ones, then the halo (each group in the
     * curve's order) */
    auto rank = [&](int32_t e) { return elem_class[e] == 1 ? 0 : (elem_class[e] == 0 ? 1 : 2); };
    std::stable_sort(P.perm.begin(), P.perm.end(), [&](int32_t i, int32_t j) { return rank(i) < rank(j); });
    for (int e = 0; e < n; ++e) {
      P.n_send += elem_class[e] == 1;
      P.n_own += elem_class[e] != 2;
    }
  }
  for (int i = 0; i < n; ++i) P.iperm[P.perm[i]] = i;

  /* -- phys_inflow entry list (compute_input_elems, maillage.cuf:1333-1363): one entry per
   * (element, inflow edge) in reference order; calcul_surf_entree (:1368-1421) gives each
   * entry, for inlet number id, length * depth of the element's last inflow edge of that
   * number (the same value for every entry of an element) ------------------------------- */
  P.inl_cell.clear();
  P.inl_len.clear();
  P.nin = 0;
  if (p->inlet == 3) {
    P.nin = std::max(0, std::min<int32_t>(m->nombre_entrees, CF_MAX_IO));
    for (int e = 0; e < n; ++e)
      for (int k = 0; k < 3; ++k) {
        if (P.bnd[(e * 3 + k) * 2] != -1) continue;
        P.inl_cell.push_back(P.iperm[e]);
        for (int id = 1; id <= P.nin; ++id) {
          double len = 0.0;
          for (int kf = 0; kf < 3; ++kf)
            if (P.bnd[(e * 3 + kf) * 2] == -1 && P.bnd[(e * 3 + kf) * 2 + 1] == id) {
              int a = nd(m, e, kf), b = nd(m, e, (kf + 1) % 3);
              len = std::sqrt((m->x[a] - m->x[b]) * (m->x[a] - m->x[b]) + (m->y[a] - m->y[b]) * (m->y[a] - m->y[b]));
            }
          P.inl_len.push_back(len);
        }
      }
  }

  /* -- edges: interior edges at their first element in the new order, then boundary ------- */
  P.edges.clear();
  P.edges.reserve((size_t)n * 3 / 2 + 16);
  for (int c = 0; c < n; ++c) {
    int o = P.perm[c];
    for (int k = 0; k < 3; ++k) {
      int nb = P.bnd[(o * 3 + k) * 2];
      if (nb <= 0) continue;
      int onb = nb - 1;
      if (P.iperm[onb] < c) continue; /* emitted from the neighbour already */
      if (P.iperm[onb] == c) continue;
      int kb = P.nbr_k[o * 3 + k];
      if (kb < 0 || P.bnd[(onb * 3 + kb) * 2] != o + 1) {
        err = "non-manifold neighbour relation (an edge shared by more than two elements)";
        return CF_EINVAL;
      }
      HostEdge E;
      if (o < onb) { E.a = c; E.ka = k; E.b = P.iperm[onb]; E.kb = kb; }
      else { E.a = P.iperm[onb]; E.ka = kb; E.b = c; E.kb = k; }
      E.id = 0;
      P.edges.push_back(E);
    }
  }
  P.n_interior = (int32_t)P.edges.size();
  for (int c = 0; c < n; ++c) {
    int o = P.perm[c];
    for (int k = 0; k < 3; ++k) {
      int nb = P.bnd[(o * 3 + k) * 2];
      if (nb > 0) continue;
      HostEdge E;
      E.a = c; E.ka = k; E.b = nb; E.kb = -1; E.id = P.bnd[(o * 3 + k) * 2 + 1];
      P.edges.push_back(E);
    }
  }
  const size_t ne = P.edges.size();
  /* boundary edges in reference order (element, local edge) */
  {
    std::vector<int32_t> bslot(3 * (size_t)n, -1);
    for (size_t e = (size_t)P.n_interior; e < ne; ++e) bslot[3 * (size_t)P.perm[P.edges[e].a] + P.edges[e].ka] = (int32_t)e;
    P.bq_ref.clear();
    for (size_t i = 0; i < bslot.size(); ++i)
      if (bslot[i] >= 0) P.bq_ref.push_back(bslot[i]);
  }
  /* a part: the edges of the send elements (first phase of its step), then those of the interior */
  P.elist1.clear();
  P.elist2.clear();
  if (elem_class) {
    const int32_t ns = P.n_send, no = P.n_own;
    for (size_t e = 0; e < ne; ++e) {
      const HostEdge& E = P.edges[e];
      const bool s1 = E.a < ns || (E.b >= 0 && E.b < ns);
      const bool s2 = (E.a >= ns && E.a < no) || (E.b >= ns && E.b < no);
      if (s1) P.elist1.push_back((int32_t)e);
      else if (s2) P.elist2.push_back((int32_t)e);
    }
  }

  /* -- per-element tables (new order) --------------------------------------------------- */
  P.cslot.assign(n, make_int4(-1, -1, -1, 0));
  P.cstat.resize(n);
  P.zcell.resize(n);
  for (int c = 0; c < n; ++c) {
    int o = P.perm[c];
    double man = p->is_override_manning ? p->override_manning : m->manning_elt[o];
    P.cstat[c] = make_double4(P.area[o], man, p->cfl * P.cotemin[o], 1.0 / P.area[o]);
    P.zcell[c] = P.zm[o];
  }
  auto set_slot = [&](int c, int k, int s) {
    int* v = &P.cslot[c].x;
    v[k] = s;
  };
  for (size_t e = 0; e < ne; ++e) {
    const HostEdge& E = P.edges[e];
    set_slot(E.a, E.ka, (int)(2 * e));
    if (E.b >= 0) set_slot(E.b, E.kb, (int)(2 * e + 1));
  }
  for (int c = 0; c < n; ++c)
    if (P.cslot[c].x < 0 || P.cslot[c].y < 0 || P.cslot[c].z < 0) {
      err = "internal error: element without an edge slot";
      return CF_EINVAL;
    }

  /* -- per-edge tables -------------------------------------------------------------------- */
  const bool second = p->iflux >= 3;
  P.ecell.resize(ne);
  P.egeo.resize(ne);
  P.ebid.resize(ne);
  if (second) { P.eupw.resize(ne); P.ewts.resize(ne); P.edk.resize(ne); P.einv.resize(ne); }
  auto cdist = [&](int oa, int ob) {
    return std::sqrt((P.xc[oa] - P.xc[ob]) * (P.xc[oa] - P.xc[ob]) + (P.yc[oa] - P.yc[ob]) * (P.yc[oa] - P.yc[ob]));
  };
  /* upwind element of (old element o, local edge c, which): the element across edge c+1 or
   * c+2, or o itself where that edge is not interior (find_upwind_cells). */
  auto upw = [&](int o, int c, int which) {
    int nb = P.bnd[(o * 3 + (c + 1 + which) % 3) * 2];
    return nb > 0 ? nb - 1 : o;
  };
  for (size_t e = 0; e < ne; ++e) {
    const HostEdge& E = P.edges[e];
    int oa = P.perm[E.a];
    double n1, n2, ln;
    edge_normal(m, oa, E.ka, n1, n2, ln);
    double inv_d = 0.0; /* d_mrl of an interior edge */
    if (E.b >= 0) {
      int ob = P.perm[E.b];
      inv_d = cdist(oa, ob); /* d_mrl (:195) */
      P.ecell[e] = make_int2(E.a, E.b);
      P.ebid[e] = 0;
      if (second) {
        /* upwind reconstruction of each side (flux_riemann.cuf:302-366): d1 < 0 marks a copy
         * of one element's state (one upwind element, or the first-order fallback of
         * :303-316 where the element itself is copied and d_mkvol = d_mrl). */
        double dmrl = cdist(oa, ob);
        int v1 = upw(oa, E.ka, 0), v2 = upw(oa, E.ka, 1);
        int w1 = upw(ob, E.kb, 0), w2 = upw(ob, E.kb, 1);
        int ua1, ua2, ub1, ub2;
        double da1, da2, db1, db2, dka, dkb;
        if ((v1 == oa && v2 == oa) || (w1 == ob && w2 == ob)) {
          ua1 = ua2 = oa; da1 = -1.0; da2 = 0.0; dka = dmrl;
          ub1 = ub2 = ob; db1 = -1.0; db2 = 0.0; dkb = dmrl;
        } else {
          /* one upwind element: the reference reads the distance to it uninitialised on
           * the kvol side (Q8); it is the centroid distance, as on the kvoisin side. */
          if (v1 == oa) { ua1 = ua2 = v2; da1 = -1.0; da2 = 0.0; dka = cdist(v2, oa); }
          else if (v2 == oa) { ua1 = ua2 = v1; da1 = -1.0; da2 = 0.0; dka = cdist(v1, oa); }
          else {
            ua1 = v1; ua2 = v2; da1 = cdist(v1, oa); da2 = cdist(v2, oa); dka = (da1 + da2) / 2.;
          }
          if (w1 == ob) { ub1 = ub2 = w2; db1 = -1.0; db2 = 0.0; dkb = cdist(w2, ob); }
          else if (w2 == ob) { ub1 = ub2 = w1; db1 = -1.0; db2 = 0.0; dkb = cdist(w1, ob); }
          else {
            ub1 = w1; ub2 = w2; db1 = cdist(w1, ob); db2 = cdist(w2, ob); dkb = (db1 + db2) / 2.;
          }
        }
        P.eupw[e] = make_int4(P.iperm[ua1], P.iperm[ua2], P.iperm[ub1], P.iperm[ub2]);
        P.ewts[e] = make_double4(da1, da2, db1, db2);
        P.edk[e] = make_double4(dka, dkb, 1.0 / dka, 1.0 / dkb);
        /* reciprocals of the sums the weighted averages divide by (copies divide by nothing) */
        P.einv[e] = make_double4(1.0 / dmrl, da1 < 0.0 ? 0.0 : 1.0 / (da1 + da2), db1 < 0.0 ? 0.0 : 1.0 / (db1 + db2), 0.0);
      }
    } else {
      P.ecell[e] = make_int2(E.a, E.b);
      P.ebid[e] = E.id;
      if (second) {
        P.eupw[e] = make_int4(E.a, E.a, E.a, E.a);
        P.ewts[e] = make_double4(-1.0, 0.0, -1.0, 0.0);
        P.edk[e] = make_double4(0.0, 0.0, 0.0, 0.0);
        P.einv[e] = make_double4(0.0, 0.0, 0.0, 0.0);
      }
    }
    P.egeo[e] = make_double4(n1, n2, ln, inv_d);
  }
  /* the elements across each element's edges, and whether all three are interior edges with
   * finite geometry and the element's area is one for which a dry update is exact zeros (then the
   * edges between two elements of depth +0 take the edge kernel's dry shortcut, and the element
   * kernel knows their slots without reading them) */
  P.cnbr.assign(n, make_int4(-1, -1, -1, 1));
  for (size_t e = 0; e < ne; ++e) {
    const HostEdge& E = P.edges[e];
    const double4 g = P.egeo[e];
    const bool fin = std::isfinite(g.x) && std::isfinite(g.y) && std::isfinite(g.z);
    if (E.b < 0) {
      P.cnbr[E.a].w = 0;
      continue;
    }
    (&P.cnbr[E.a].x)[E.ka] = E.b;
    (&P.cnbr[E.b].x)[E.kb] = E.a;
    if (!fin) P.cnbr[E.a].w = P.cnbr[E.b].w = 0;
  }
  for (int c = 0; c < n; ++c)
    if (P.cnbr[c].x < 0 || P.cnbr[c].y < 0 || P.cnbr[c].z < 0 || !area_ok(P.cstat[c].x)) P.cnbr[c].w = 0;
  /* the beds an edge reads: its elements' and, second order, its upwind reconstructions' (the
   * distance-weighted bed of two upwind elements, flux_riemann.cuf:320-366; static) */
  P.ez.resize(ne);
  for (size_t e = 0; e < ne; ++e) {
    const HostEdge& E = P.edges[e];
    double4 z = make_double4(P.zcell[E.a], E.b >= 0 ? P.zcell[E.b] : 0.0, 0.0, 0.0);
    if (second && E.b >= 0) {
      const int4 u = P.eupw[e];
      const double4 w = P.ewts[e], yi = P.einv[e];
      z.z = upwind_bed(P.zcell[u.x], P.zcell[u.y], w.x, w.y, yi.y);
      z.w = upwind_bed(P.zcell[u.z], P.zcell[u.w], w.z, w.w, yi.z);
    }
    P.ez[e] = z;
  }
  return CF_OK;
}

}  // namespace cf
