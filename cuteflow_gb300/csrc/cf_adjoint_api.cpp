/*
 * cf_adjoint_api.cpp -- the discrete adjoint behind the C ABI (cf_adjoint_*, cf_set_manning).
 *
 * Objective.  For a run of N steps from the context's current state U^0 with the Manning field
 * n, the caller weighs the free-surface elevation eta^k_g = h + z of G gauge elements after
 * every step k = 1..N and the final state:
 *     J = sum_k sum_g w_eta[k-1][g] eta^k_g + sum_e w_state[e] . U^N_e .
 * cf_adjoint_backward returns dJ/dU^0 and dJ/dn (every element), with the dt of every step held
 * at its recorded value (the time step is not differentiated).  A caller with a non-linear
 * misfit passes its derivative with respect to eta and U^N as the weights (chain rule).
 *
 * Schedule.  A reverse step k needs the state U^k and every element's flux and bed sums at U^k
 * (a step record: 32 + 48 bytes per element).  The recording forward keeps the records of the
 * last T steps itself and a checkpoint state every K steps of the first M = N - T; the backward
 * sweep runs the reverse steps of the stored tail directly, then walks the checkpointed
 * segments from the last: it recomputes a segment's records from its checkpoint with the
 * recorded dt sequence (bit-identical to the recorded run) into the same record pool and runs
 * their reverse steps.  Cost: the reverse steps plus M replayed forward steps; memory: R = max(T,
 * K, 2) records, ceil(M / K) checkpoints and two run states.  With no budget T = 0 and
 * K = ceil(sqrt(N)) (or the caller's interval).  With a device-memory budget the schedule keeps
 * the largest record pool that fits it: T = min(N, R) and K = R (or the caller's interval),
 * every replay is saved when the whole run fits.  The gradient does not depend on the schedule:
 * a record written by the recording forward and the same record written by a replay are the
 * same bits.
 *
 * Batches.  On a context of several members the run, the checkpoints, the replay and the reverse
 * steps cover every member in the same launches, each with its own recorded dt (histories are
 * [N][members]); gauges are (member, element) pairs; states and gradients are concatenated in
 * member order.  cf_zones_* sums dJ/dn over Manning zones in a fixed order and steps the zone
 * values on the device, for gradient-descent calibration without host round trips.
 */
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "cf_ctx.h"

using namespace cf;

struct cf_adjoint {
  cf_ctx* ctx = nullptr;
  int32_t N = 0, K = 1, G = 0, nseg = 0, nseg_states = 2;   /* nseg_states: R, the record pool */
  int32_t T = 0;             /* stored tail steps N - T .. N - 1 (records of the recording forward) */
  int32_t Mc = 0;            /* checkpointed steps 0 .. Mc - 1 (Mc = N - T) */
  int64_t bytes = 0;         /* device bytes of the adjoint */
  double4* pp = nullptr;     /* two run states of the forward */
  bool tail_valid = false;   /* the pool holds the stored tail's records (a backward that replays
                                checkpointed segments reuses the pool and clears this) */
  int32_t nm = 1;            /* members */
  int64_t n_all = 0;         /* elements of all members */
  int32_t n_pad = 0;
  double4* ckpt = nullptr;   /* nseg states */
  double4* seg = nullptr;    /* nseg_states states */
  MemberState* mst = nullptr;
  double* dt_hist = nullptr;
  double* t_hist = nullptr;
  double* eta = nullptr;     /* N x G */
  double* wbuf = nullptr;    /* N x G objective weights */
  int32_t* gcell = nullptr;
  int32_t* goff = nullptr;
  int32_t* gidx = nullptr;
  double4* lam[2] = {nullptr, nullptr};   /* lambda^N (terminal weights); own part of lambda^n */
  Slot* sums = nullptr;      /* nseg_states x n_pad: flux and bed sums of every step of a segment */
  Slot* cadj = nullptr;
  double4* eadj = nullptr;
  double4* uadj = nullptr;
  int32_t* uoff = nullptr;
  int32_t* uidx = nullptr;
  double* gman = nullptr;
  uint32_t* flag = nullptr;
  int32_t* pend = nullptr;   /* the reverse edge kernel's queue of edges for its six-lane path */
  int32_t* npend = nullptr;
  int32_t freeze_r = 0;      /* linearization of the WAF limiter ratios: 0 exact, 1 held */
  bool recorded = false;     /* a recording forward has filled dt_hist / t_hist */
  bool have_traj = false;    /* the checkpoints hold the last forward's trajectory */
};

/* Manning zones of a context: every element's zone (flat new order, -1: none), the CSR zone ->
 * elements, the zone values and the last zone gradient (device memory). */
struct cf_zones {
  cf_ctx* ctx = nullptr;
  int32_t nz = 0;
  int32_t* zoff = nullptr;
  int32_t* zidx = nullptr;
  int32_t* zone_of = nullptr;
  double* gz = nullptr;
  double* vals = nullptr;
};

namespace {

void adj_free(cf_adjoint* a) {
  void* ptrs[] = {a->pend, a->npend, a->pp, a->ckpt, a->seg, a->mst, a->dt_hist, a->t_hist, a->eta, a->wbuf, a->gcell, a->goff, a->gidx,
                  a->lam[0], a->lam[1], a->sums, a->cadj, a->eadj, a->uadj, a->uoff, a->uidx, a->gman, a->flag};
  for (void* p : ptrs)
    if (p) cudaFree(p);
}

template <class T>
int get(cf_ctx* c, T* dst, const T* src, size_t count) {
  if (count) CF_CUDA(c, cudaMemcpy(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost));
  return CF_OK;
}

/* CSR (ascending element, then ascending entry) of the pairs (element, entry) */
void build_csr(int32_t n, const std::vector<int32_t>& elem, const std::vector<int32_t>& entry,
               std::vector<int32_t>& off, std::vector<int32_t>& idx) {
  off.assign((size_t)n + 1, 0);
  for (int32_t e : elem) off[(size_t)e + 1]++;
  for (int32_t i = 0; i < n; ++i) off[(size_t)i + 1] += off[i];
  idx.assign(elem.size(), 0);
  std::vector<int32_t> pos(off.begin(), off.end() - 1);
  for (size_t k = 0; k < elem.size(); ++k) idx[(size_t)pos[elem[k]]++] = entry[k];
}

int create_impl(cf_ctx* c, int32_t nsteps, int32_t interval, const int32_t* gauge_member, const int32_t* gauges,
                int32_t ngauges, int64_t budget, cf_adjoint** out) {
  if (!out) return fail(c, CF_EINVAL, "out is NULL");
  *out = nullptr;
  if (c->iflux > 3) return fail(c, CF_ENOTSUP, "the adjoint covers iflux 1..3");
  if (c->any_phys_inflow) return fail(c, CF_ENOTSUP, "the adjoint does not cover inlet 3 (phys_inflow)");
  if (nsteps < 1) return fail(c, CF_EINVAL, "nsteps < 1");
  if (ngauges < 0 || (ngauges > 0 && !gauges)) return fail(c, CF_EINVAL, "gauges NULL or ngauges < 0");
  const int32_t nm = (int32_t)c->mem.size();
  for (int32_t g = 0; g < ngauges; ++g) {
    const int32_t m = gauge_member ? gauge_member[g] : 0;
    if (m < 0 || m >= nm) return fail(c, CF_EINVAL, "gauge member out of range");
    if (gauges[g] < 0 || gauges[g] >= c->mem[m].n) return fail(c, CF_EINVAL, "gauge element out of range");
  }
  CF_CUDA(c, cudaSetDevice(c->device));
  cf_adjoint* a = new (std::nothrow) cf_adjoint();
  if (!a) return fail(c, CF_ENOMEM, "host allocation failed");
  auto done = [&](int rc) {
    if (rc != CF_OK) {
      adj_free(a);
      delete a;
    } else {
      *out = a;
    }
    return rc;
  };
  a->ctx = c;
  a->N = nsteps;
  a->G = ngauges;
  a->nm = nm;
  for (const Member& M : c->mem) a->n_all += M.n;
  a->n_pad = c->n_pad;
  const size_t np = (size_t)c->n_pad, nep = (size_t)c->ne_pad;
  const bool second = c->iflux >= 3;
  /* device bytes besides the record pool and the checkpoints (upper bound for the upwind lists) */
  const int64_t st4 = (int64_t)np * (int64_t)sizeof(double4), rec = st4 + (int64_t)np * (int64_t)sizeof(Slot);
  const int64_t fixed = 4 * st4 + (int64_t)np * (int64_t)sizeof(Slot) + 2 * (int64_t)nep * (int64_t)sizeof(double4) +
                        4 * (int64_t)nep + 4 +
                        (int64_t)np * 8 + (int64_t)nsteps * (16 * (int64_t)nm + 16 * (int64_t)ngauges) +
                        (int64_t)(np + 1) * 4 + 8 * (int64_t)ngauges + (int64_t)nm * (int64_t)sizeof(MemberState) +
                        (second ? 4 * (int64_t)nep * (int64_t)sizeof(double4) + (int64_t)(np + 1) * 4 +
                                      4 * (int64_t)nep * 4
                                : 0);
  if (budget <= 0) {
    a->T = 0;
    a->K = interval > 0 ? std::min(interval, nsteps) : std::max(1, (int32_t)std::ceil(std::sqrt((double)nsteps)));
    a->nseg_states = std::max(a->K, 2);
  } else {
    /* the largest record pool R whose schedule fits the budget: T = min(N, R) stored steps, the
     * other M = N - T in checkpointed segments of K = R steps (or the caller's interval) */
    int32_t best = 0;
    for (int32_t R = nsteps; R >= 2; --R) {
      const int32_t T = std::min(nsteps, R), M = nsteps - T;
      const int32_t K = M > 0 ? (interval > 0 ? std::min(interval, R) : R) : 1;
      /* checkpoints of the replayed steps, and one of the tail's first state when both exist */
      const int64_t need = fixed + (int64_t)R * rec + (int64_t)((M + K - 1) / K + (M > 0 ? 1 : 0)) * st4;
      if (need <= budget) {
        best = R;
        break;
      }
    }
    if (best == 0) {
      a->bytes = fixed + 2 * rec + (int64_t)((nsteps + 1) / 2) * st4;
      adj_free(a);
      delete a;
      return fail(c, CF_ENOMEM, "adjoint memory budget of " + std::to_string(budget) +
                                    " bytes is below this run's smallest schedule");
    }
    a->nseg_states = std::max(best, 2);
    a->T = std::min(nsteps, best);
    const int32_t M = nsteps - a->T;
    a->K = M > 0 ? (interval > 0 ? std::min(interval, best) : best) : std::max(1, std::min(nsteps, best));
  }
  a->Mc = nsteps - a->T;
  a->nseg = a->Mc > 0 ? (a->Mc + a->K - 1) / a->K : 0;
  /* checkpoint nseg (when the run has both parts) keeps U^Mc, the tail's first state */
  const int32_t nck = a->nseg + ((a->T > 0 && a->Mc > 0) ? 1 : 0);
  a->bytes = fixed + (int64_t)a->nseg_states * rec + (int64_t)nck * st4;
  int rc;
  if ((rc = dalloc(c, &a->pp, 2 * np)) || (rc = dalloc(c, &a->ckpt, (size_t)std::max(nck, 1) * np)) ||
      (rc = dalloc(c, &a->seg, (size_t)a->nseg_states * np)) ||
      (rc = dalloc(c, &a->mst, (size_t)nm)) || (rc = dalloc(c, &a->dt_hist, (size_t)nsteps * nm)) ||
      (rc = dalloc(c, &a->t_hist, (size_t)nsteps * nm)) || (rc = dalloc(c, &a->eta, (size_t)nsteps * ngauges)) ||
      (rc = dalloc(c, &a->wbuf, (size_t)nsteps * ngauges)) || (rc = dalloc(c, &a->gcell, (size_t)ngauges)) ||
      (rc = dalloc(c, &a->goff, np + 1)) || (rc = dalloc(c, &a->gidx, (size_t)ngauges)) ||
      (rc = dalloc(c, &a->lam[0], np)) || (rc = dalloc(c, &a->lam[1], np)) || (rc = dalloc(c, &a->cadj, np)) ||
      (rc = dalloc(c, &a->sums, (size_t)a->nseg_states * np)) ||
      (rc = dalloc(c, &a->eadj, 2 * nep)) || (rc = dalloc(c, &a->gman, np)) || (rc = dalloc(c, &a->flag, 1)) ||
      (rc = dalloc(c, &a->pend, nep)) || (rc = dalloc(c, &a->npend, 1)))
    return done(rc);
  /* gauges: new order, and their CSR over the elements */
  {
    std::vector<int32_t> gc(ngauges), ge(ngauges), gi(ngauges), off, idx;
    for (int32_t g = 0; g < ngauges; ++g) {
      const Member& M = c->mem[gauge_member ? gauge_member[g] : 0];
      gc[g] = M.cell_off + M.prep.iperm[gauges[g]];
      ge[g] = g;
    }
    build_csr(c->n_pad, gc, ge, off, idx);
    if ((rc = put(c, a->gcell, gc.data(), gc.size())) || (rc = put(c, a->goff, off.data(), off.size())) ||
        (rc = put(c, a->gidx, idx.data(), idx.size())))
      return done(rc);
  }
  /* second order: which edge entries each element is an upwind element of */
  if (second) {
    if ((rc = dalloc(c, &a->uadj, 4 * nep)) || (rc = dalloc(c, &a->uoff, np + 1))) return done(rc);
    std::vector<int2> ecell(nep);
    std::vector<int4> up(nep);
    std::vector<double4> dw(nep);
    if ((rc = get(c, ecell.data(), c->ecell, nep)) || (rc = get(c, up.data(), c->eupw, nep)) ||
        (rc = get(c, dw.data(), c->ewts, nep)))
      return done(rc);
    std::vector<int32_t> el, en, off, idx;
    for (const Member& M : c->mem)   /* the members' real edges (not the tile padding) */
      for (int32_t e = M.edge_off; e < M.edge_off + M.ne; ++e) {
        if (ecell[e].y < 0) continue;
        el.push_back(up[e].x);
        en.push_back(4 * e);
        if (dw[e].x >= 0.0) { el.push_back(up[e].y); en.push_back(4 * e + 1); }
        el.push_back(up[e].z);
        en.push_back(4 * e + 2);
        if (dw[e].z >= 0.0) { el.push_back(up[e].w); en.push_back(4 * e + 3); }
      }
    build_csr(c->n_pad, el, en, off, idx);
    if ((rc = dalloc(c, &a->uidx, idx.size())) || (rc = put(c, a->uoff, off.data(), off.size())) ||
        (rc = put(c, a->uidx, idx.data(), idx.size())))
      return done(rc);
  }
  return done(CF_OK);
}

/* copy n doubles to a caller's pointer (host or device) */
int to_user(cf_ctx* c, double* dst, const double* src, size_t count) {
  if (dst && count) CF_CUDA(c, cudaMemcpyAsync(dst, src, count * sizeof(double), cudaMemcpyDefault, c->stream));
  return CF_OK;
}

/* Per member, a device state (comps = 3: double4 states, h hu hv out) or scalar field (comps = 1)
 * in the flat new order -> dst in member order, reference element order within a member. */
int gather_members(cf_adjoint* a, const void* src, double* dst, int comps) {
  cf_ctx* c = a->ctx;
  const stream_t st = reinterpret_cast<stream_t>(c->stream);
  int rc;
  size_t off = 0;
  for (const Member& M : c->mem) {
    if (comps == 3)
      rc = launch_gather_state(static_cast<const double4*>(src) + M.cell_off, c->iperm + M.cell_off, c->staging, M.n, st);
    else
      rc = launch_gather_scalar(static_cast<const double*>(src) + M.cell_off, c->iperm + M.cell_off, c->staging, M.n, st);
    if (rc) return fail(c, rc, "gather launch failed");
    if ((rc = to_user(c, dst + off, c->staging, (size_t)comps * M.n))) return rc;
    off += (size_t)comps * M.n;
  }
  return CF_OK;
}

int forward_impl(cf_adjoint* a, int32_t replay, double* eta_out, double* state_out) {
  cf_ctx* c = a->ctx;
  if (replay && !a->recorded) return fail(c, CF_ESTATE, "replay before a recording forward");
  CF_CUDA(c, cudaSetDevice(c->device));
  int rc;
  if ((rc = read_states(c))) return rc;
  const stream_t st = reinterpret_cast<stream_t>(c->stream);
  const size_t np = (size_t)a->n_pad;
  /* every member's current state into the first segment state, and the adjoint's own member
   * records, all at one buffer parity p0 (members set at different times may differ) */
  const int p0 = (int)(c->launched & 1);
  std::vector<MemberState> ms(c->host_state, c->host_state + a->nm);
  a->have_traj = false;
  for (int32_t i = 0; i < a->nm; ++i) {
    MemberState& s = ms[i];
    const std::string who = a->nm > 1 ? "member " + std::to_string(i) + ": " : std::string();
    if (s.status & STATUS_NO_STATE) return fail(c, CF_ESTATE, who + "no state set");
    if (s.status) {
      const int code = status_code(s.status);
      return fail(c, code != CF_OK ? code : CF_ESTATE, who + "the member is stopped");
    }
    const Member& M = c->mem[i];
    const int cur = (int)((s.base + s.nstep) & 1);
    /* the run starts in a run state, or in the first record when every step is stored */
    double4* X0 = a->Mc > 0 ? a->pp : a->seg;
    CF_CUDA(c, cudaMemcpyAsync(X0 + M.cell_off, c->U[cur] + M.cell_off, (size_t)M.n * sizeof(double4),
                               cudaMemcpyDeviceToDevice, c->stream));
    if (cur != p0) {
      std::swap(s.dt[0], s.dt[1]);
      std::swap(s.t[0], s.t[1]);
      s.base ^= 1;
    }
    s.ts = INFINITY;   /* the adjoint's run has N steps: no end time */
  }
  if (!replay) CF_CUDA(c, cudaMemcpyAsync(a->mst, ms.data(), ms.size() * sizeof(MemberState), cudaMemcpyHostToDevice,
                                          c->stream));
  CF_CUDA(c, cudaMemsetAsync(a->flag, 0, sizeof(uint32_t), c->stream));
  const int32_t Mc = a->Mc;
  double4* X = Mc > 0 ? a->pp : a->seg;
  int p = p0;
  for (int32_t k = 0; k < a->N; ++k) {
    if ((k < Mc && k % a->K == 0) || (k == Mc && k > 0))
      CF_CUDA(c, cudaMemcpyAsync(a->ckpt + (size_t)(k < Mc ? k / a->K : a->nseg) * np, X, np * sizeof(double4),
                                 cudaMemcpyDeviceToDevice, c->stream));
    /* U^{k+1} into its record when that step is stored, else into the other run state */
    double4* Y = (k + 1 >= Mc && k + 1 < a->N) ? a->seg + (size_t)(k + 1 - Mc) * np : (X == a->pp ? a->pp + np : a->pp);
    Slot* sums = k >= Mc ? a->sums + (size_t)(k - Mc) * np : nullptr;
    StepArgs sa = step_args(c, p);
    sa.Uin = X;
    sa.Uout = Y;
    sa.steady = 0;   /* the adjoint's run has N steps: no steady-state stop */
    if (!replay) {
      sa.mst = a->mst;
      sa.sums_out = sums;   /* the element kernel stores the step's sums for the stored records */
      if ((rc = launch_step(sa, st, nullptr, nullptr))) return fail(c, rc, "step launch failed");
      rc = launch_record(Y, c->zcell, a->mst, a->nm, p, k, a->dt_hist, a->t_hist, a->gcell, a->G, a->eta, st);
    } else {
      if ((rc = launch_replay_step(sa, a->dt_hist, a->t_hist, k, a->flag, sums, st)))
        return fail(c, rc, "replay launch failed");
      rc = launch_record(Y, c->zcell, nullptr, a->nm, 0, k, a->dt_hist, a->t_hist, a->gcell, a->G, a->eta, st);
    }
    if (rc) return fail(c, rc, "record launch failed");
    X = Y;
    p ^= 1;
  }
  if (state_out && (rc = gather_members(a, X, state_out, 3))) return rc;
  if ((rc = to_user(c, eta_out, a->eta, (size_t)a->N * a->G))) return rc;
  uint32_t flag = 0;
  CF_CUDA(c, cudaMemcpyAsync(ms.data(), a->mst, ms.size() * sizeof(MemberState), cudaMemcpyDeviceToHost, c->stream));
  CF_CUDA(c, cudaMemcpyAsync(&flag, a->flag, sizeof(flag), cudaMemcpyDeviceToHost, c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  uint32_t bad = flag;
  if (!replay)
    for (const MemberState& s : ms) bad |= s.status;
  if (bad) {
    rc = status_code(bad);
    return fail(c, rc, rc == CF_EDT ? "dt left the range (1e-12, 9999] during the run" : "non-finite value in the state");
  }
  if (!replay) a->recorded = true;
  a->have_traj = true;
  a->tail_valid = true;
  return CF_OK;
}

int backward_impl(cf_adjoint* a, const double* w_eta, const double* w_state, double* g_state0, double* g_manning) {
  cf_ctx* c = a->ctx;
  if (!a->have_traj) return fail(c, CF_ESTATE, "backward before a forward");
  CF_CUDA(c, cudaSetDevice(c->device));
  const stream_t st = reinterpret_cast<stream_t>(c->stream);
  const size_t np = (size_t)a->n_pad;
  const size_t nw = (size_t)a->N * a->G;
  int rc;
  const bool weights = w_eta && nw > 0;
  if (weights) CF_CUDA(c, cudaMemcpyAsync(a->wbuf, w_eta, nw * sizeof(double), cudaMemcpyDefault, c->stream));
  CF_CUDA(c, cudaMemsetAsync(a->lam[0], 0, np * sizeof(double4), c->stream));
  CF_CUDA(c, cudaMemsetAsync(a->lam[1], 0, np * sizeof(double4), c->stream));
  CF_CUDA(c, cudaMemsetAsync(a->gman, 0, np * sizeof(double), c->stream));
  if (w_state) {
    size_t off = 0;
    for (const Member& M : c->mem) {
      CF_CUDA(c, cudaMemcpyAsync(c->staging, w_state + off, 3 * (size_t)M.n * sizeof(double), cudaMemcpyDefault,
                                 c->stream));
      if ((rc = launch_scatter_state(c->staging, c->perm + M.cell_off, c->zcell + M.cell_off, a->lam[0] + M.cell_off,
                                     M.n, st)))
        return fail(c, rc, "scatter launch failed");
      off += 3 * (size_t)M.n;
    }
  }
  if (weights && (rc = launch_add_gauges(a->lam[0], a->goff, a->gidx, a->wbuf + (size_t)(a->N - 1) * a->G, a->n_pad, st)))
    return fail(c, rc, "gauge launch failed");
  /* lam[0] = lambda^N; lam[1] = the own part of lambda^k, carried from reverse step to reverse
   * step (the edge contributions are gathered by the next reverse step, or the final pass). */
  bool first = true;
  AdjArgs A{};
  /* the reverse steps k = k1 - 1 .. k0 whose records r = k - k0 are in the pool */
  auto reverse = [&](int32_t k0, int32_t k1) -> int {
    for (int32_t k = k1 - 1; k >= k0; --k) {
      A = AdjArgs{};
      A.s = step_args(c, 0);
      A.s.Uin = a->seg + (size_t)(k - k0) * np;
      A.s.Uout = nullptr;
      A.dt_hist = a->dt_hist;
      A.t_hist = a->t_hist;
      A.n = k;
      A.gather = first ? 0 : 1;
      A.sums = a->sums + (size_t)(k - k0) * np;
      A.lam_init = a->lam[0];
      A.lam_own = a->lam[1];
      A.cadj = a->cadj;
      A.eadj = a->eadj;
      A.uadj = a->uadj;
      A.uoff = a->uoff;
      A.uidx = a->uidx;
      A.goff = a->goff;
      A.gidx = a->gidx;
      /* the gauges of U^{k+1} (row k); those of U^N are already in lambda^N */
      A.gw = (weights && k + 1 < a->N) ? a->wbuf + (size_t)k * a->G : nullptr;
      A.gman = a->gman;
      A.freeze_r = a->freeze_r;
      A.pend = a->pend;
      A.npend = a->npend;
      const int r = launch_adjoint_step(A, st);
      if (r) return fail(c, r, "adjoint launch failed");
      first = false;
    }
    return CF_OK;
  };
  /* the tail the recording forward stored: no replay (after a backward that replayed segments
   * into the pool, the tail's records are rebuilt from its checkpoint first) */
  if (a->T > 0) {
    if (!a->tail_valid) {
      CF_CUDA(c, cudaMemcpyAsync(a->seg, a->ckpt + (size_t)a->nseg * np, np * sizeof(double4),
                                 cudaMemcpyDeviceToDevice, c->stream));
      for (int32_t i = 0; i < a->T; ++i) {
        StepArgs sa = step_args(c, 0);
        sa.Uin = a->seg + (size_t)i * np;
        sa.Uout = (i + 1 < a->T) ? a->seg + (size_t)(i + 1) * np : nullptr;
        if ((rc = launch_replay_step(sa, a->dt_hist, a->t_hist, a->Mc + i, a->flag, a->sums + (size_t)i * np, st)))
          return fail(c, rc, "replay launch failed");
      }
      a->tail_valid = true;
    }
    if ((rc = reverse(a->Mc, a->N))) return rc;
  }
  if (a->nseg > 0) a->tail_valid = false;   /* the segment replays below reuse the pool */
  for (int32_t j = a->nseg - 1; j >= 0; --j) {
    const int32_t s0 = j * a->K, s1 = std::min(a->Mc, s0 + a->K);
    CF_CUDA(c, cudaMemcpyAsync(a->seg, a->ckpt + (size_t)j * np, np * sizeof(double4), cudaMemcpyDeviceToDevice,
                               c->stream));
    /* replay the segment: its states and, for every step, the flux and bed sums at U^k */
    for (int32_t i = 0; i < s1 - s0; ++i) {
      StepArgs sa = step_args(c, 0);
      sa.Uin = a->seg + (size_t)i * np;
      sa.Uout = (i + 1 < s1 - s0) ? a->seg + (size_t)(i + 1) * np : nullptr;
      if ((rc = launch_replay_step(sa, a->dt_hist, a->t_hist, s0 + i, a->flag, a->sums + (size_t)i * np, st)))
        return fail(c, rc, "replay launch failed");
    }
    if ((rc = reverse(s0, s1))) return rc;
  }
  if ((rc = launch_adjoint_final(A, st))) return fail(c, rc, "adjoint launch failed");
  double4* Lin = a->lam[1];
  if (g_state0 && (rc = gather_members(a, Lin, g_state0, 3))) return rc;
  if (g_manning && (rc = gather_members(a, a->gman, g_manning, 1))) return rc;
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

}  // namespace

extern "C" {

int cf_member_set_manning(cf_ctx* c, int32_t member, const double* n_elt) {
  if (!c) return CF_EINVAL;
  if (!n_elt) return fail(c, CF_EINVAL, "null argument");
  if (member < 0 || member >= (int32_t)c->mem.size()) return fail(c, CF_EINVAL, "member index out of range");
  CF_CUDA(c, cudaSetDevice(c->device));
  const Member& M = c->mem[member];
  CF_CUDA(c, cudaMemcpyAsync(c->staging, n_elt, (size_t)M.n * sizeof(double), cudaMemcpyDefault, c->stream));
  int rc = launch_set_manning(c->cstat + M.cell_off, c->perm + M.cell_off, c->staging, M.n,
                              reinterpret_cast<stream_t>(c->stream));
  if (rc != CF_OK) return fail(c, rc, "manning launch failed");
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_set_manning(cf_ctx* c, const double* n_elt) {
  if (!c) return CF_EINVAL;
  if (c->mem.size() != 1) return fail(c, CF_ENOTSUP, "cf_set_manning takes a context with one member");
  return cf_member_set_manning(c, 0, n_elt);
}

int cf_adjoint_create(cf_ctx* ctx, int32_t nsteps, int32_t checkpoint_interval, const int32_t* gauges,
                      int32_t ngauges, cf_adjoint** out) {
  if (!ctx) return CF_EINVAL;
  return abi_guard(ctx, [&] { return create_impl(ctx, nsteps, checkpoint_interval, nullptr, gauges, ngauges, 0, out); });
}

int cf_adjoint_create_batch(cf_ctx* ctx, int32_t nsteps, int32_t checkpoint_interval, const int32_t* gauge_member,
                            const int32_t* gauges, int32_t ngauges, cf_adjoint** out) {
  if (!ctx) return CF_EINVAL;
  if (ngauges > 0 && !gauge_member) return fail(ctx, CF_EINVAL, "gauge_member is NULL");
  return abi_guard(ctx, [&] {
    return create_impl(ctx, nsteps, checkpoint_interval, gauge_member, gauges, ngauges, 0, out);
  });
}

int cf_adjoint_create_budget(cf_ctx* ctx, int32_t nsteps, int32_t checkpoint_interval, const int32_t* gauge_member,
                             const int32_t* gauges, int32_t ngauges, int64_t budget_bytes, cf_adjoint** out) {
  if (!ctx) return CF_EINVAL;
  if (budget_bytes <= 0) return fail(ctx, CF_EINVAL, "budget_bytes <= 0");
  if (ngauges > 0 && !gauge_member && ctx->mem.size() > 1) return fail(ctx, CF_EINVAL, "gauge_member is NULL");
  return abi_guard(ctx, [&] {
    return create_impl(ctx, nsteps, checkpoint_interval, gauge_member, gauges, ngauges, budget_bytes, out);
  });
}

int cf_adjoint_schedule(cf_adjoint* a, int32_t* stored_steps, int32_t* checkpoint_interval, int32_t* checkpoints,
                        int32_t* records, int64_t* device_bytes) {
  if (!a) return CF_EINVAL;
  if (stored_steps) *stored_steps = a->T;
  if (checkpoint_interval) *checkpoint_interval = a->K;
  if (checkpoints) *checkpoints = a->nseg;
  if (records) *records = a->nseg_states;
  if (device_bytes) *device_bytes = a->bytes;
  return CF_OK;
}

void cf_adjoint_destroy(cf_adjoint* a) {
  if (!a) return;
  cudaSetDevice(a->ctx->device);
  cudaStreamSynchronize(a->ctx->stream);
  adj_free(a);
  delete a;
}

int cf_adjoint_forward(cf_adjoint* a, int32_t replay, double* eta, double* state) {
  if (!a) return CF_EINVAL;
  return forward_impl(a, replay, eta, state);
}

int cf_adjoint_backward(cf_adjoint* a, const double* w_eta, const double* w_state, double* g_state0,
                        double* g_manning) {
  if (!a) return CF_EINVAL;
  return backward_impl(a, w_eta, w_state, g_state0, g_manning);
}

int cf_adjoint_get_dt(cf_adjoint* a, double* dt, double* t) {
  if (!a) return CF_EINVAL;
  cf_ctx* c = a->ctx;
  if (!a->recorded) return fail(c, CF_ESTATE, "no recorded dt sequence");
  CF_CUDA(c, cudaSetDevice(c->device));
  int rc;
  const size_t nh = (size_t)a->N * a->nm;
  if ((rc = to_user(c, dt, a->dt_hist, nh)) || (rc = to_user(c, t, a->t_hist, nh))) return rc;
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_adjoint_set_dt(cf_adjoint* a, const double* dt, const double* t) {
  if (!a || !dt || !t) return a ? fail(a->ctx, CF_EINVAL, "null argument") : CF_EINVAL;
  cf_ctx* c = a->ctx;
  CF_CUDA(c, cudaSetDevice(c->device));
  const size_t nh = (size_t)a->N * a->nm;
  CF_CUDA(c, cudaMemcpyAsync(a->dt_hist, dt, nh * sizeof(double), cudaMemcpyDefault, c->stream));
  CF_CUDA(c, cudaMemcpyAsync(a->t_hist, t, nh * sizeof(double), cudaMemcpyDefault, c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  a->recorded = true;
  a->have_traj = false;
  return CF_OK;
}

int cf_adjoint_set_linearization(cf_adjoint* a, int32_t mode) {
  if (!a) return CF_EINVAL;
  if (mode < 0 || mode > 1) return fail(a->ctx, CF_EINVAL, "linearization mode must be 0 or 1");
  a->freeze_r = mode;
  return CF_OK;
}

int cf_adjoint_sizes(cf_adjoint* a, int32_t* nsteps, int32_t* interval, int32_t* ngauges, int64_t* device_bytes) {
  if (!a) return CF_EINVAL;
  if (nsteps) *nsteps = a->N;
  if (interval) *interval = a->K;
  if (ngauges) *ngauges = a->G;
  if (device_bytes) *device_bytes = a->bytes;
  return CF_OK;
}

/* ---- Manning zones ------------------------------------------------------------------------ */

static int zones_create_impl(cf_ctx* c, const int32_t* zone_of_elem, int32_t nzones, cf_zones** out);

int cf_zones_create(cf_ctx* c, const int32_t* zone_of_elem, int32_t nzones, cf_zones** out) {
  if (!c) return CF_EINVAL;
  return abi_guard(c, [&] { return zones_create_impl(c, zone_of_elem, nzones, out); });
}

static int zones_create_impl(cf_ctx* c, const int32_t* zone_of_elem, int32_t nzones, cf_zones** out) {
  if (!out || !zone_of_elem || nzones < 1) return fail(c, CF_EINVAL, "null argument or nzones < 1");
  *out = nullptr;
  CF_CUDA(c, cudaSetDevice(c->device));
  /* zone of every element in the flat new order; CSR zone -> elements in ascending new order */
  std::vector<int32_t> zone_new((size_t)c->n_pad, -1), el, zn;
  size_t off = 0;
  for (const Member& M : c->mem) {
    for (int32_t o = 0; o < M.n; ++o) {
      const int32_t z = zone_of_elem[off + o];
      if (z < -1 || z >= nzones) return fail(c, CF_EINVAL, "zone id out of range");
      zone_new[(size_t)M.cell_off + M.prep.iperm[o]] = z;
    }
    off += (size_t)M.n;
  }
  for (int32_t i = 0; i < c->n_pad; ++i)
    if (zone_new[i] >= 0) { zn.push_back(zone_new[i]); el.push_back(i); }
  std::vector<int32_t> zoff, zidx;
  build_csr(nzones, zn, el, zoff, zidx);
  cf_zones* z = new (std::nothrow) cf_zones();
  if (!z) return fail(c, CF_ENOMEM, "host allocation failed");
  z->ctx = c;
  z->nz = nzones;
  int rc;
  if ((rc = dalloc(c, &z->zoff, zoff.size())) || (rc = dalloc(c, &z->zidx, zidx.size())) ||
      (rc = dalloc(c, &z->zone_of, zone_new.size())) || (rc = dalloc(c, &z->gz, (size_t)nzones)) ||
      (rc = dalloc(c, &z->vals, (size_t)nzones)) || (rc = put(c, z->zoff, zoff.data(), zoff.size())) ||
      (rc = put(c, z->zidx, zidx.data(), zidx.size())) || (rc = put(c, z->zone_of, zone_new.data(), zone_new.size()))) {
    cf_zones_destroy(z);
    return rc;
  }
  *out = z;
  return CF_OK;
}

void cf_zones_destroy(cf_zones* z) {
  if (!z) return;
  cudaSetDevice(z->ctx->device);
  cudaStreamSynchronize(z->ctx->stream);
  void* ptrs[] = {z->zoff, z->zidx, z->zone_of, z->gz, z->vals};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  delete z;
}

int cf_zones_set(cf_zones* z, const double* values) {
  if (!z) return CF_EINVAL;
  cf_ctx* c = z->ctx;
  if (!values) return fail(c, CF_EINVAL, "null argument");
  CF_CUDA(c, cudaSetDevice(c->device));
  CF_CUDA(c, cudaMemcpyAsync(z->vals, values, (size_t)z->nz * sizeof(double), cudaMemcpyDefault, c->stream));
  int rc = launch_zone_apply(c->cstat, z->zone_of, z->vals, c->n_pad, reinterpret_cast<stream_t>(c->stream));
  if (rc) return fail(c, rc, "zone launch failed");
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_zones_get(cf_zones* z, double* values, double* gradient) {
  if (!z) return CF_EINVAL;
  cf_ctx* c = z->ctx;
  CF_CUDA(c, cudaSetDevice(c->device));
  int rc;
  if ((rc = to_user(c, values, z->vals, (size_t)z->nz)) || (rc = to_user(c, gradient, z->gz, (size_t)z->nz))) return rc;
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_zones_gradient(cf_zones* z, cf_adjoint* a, double* gradient) {
  if (!z || !a) return CF_EINVAL;
  cf_ctx* c = z->ctx;
  if (a->ctx != c) return fail(c, CF_EINVAL, "the zones and the adjoint belong to different contexts");
  CF_CUDA(c, cudaSetDevice(c->device));
  int rc = launch_zone_sum(a->gman, z->zoff, z->zidx, z->gz, z->nz, reinterpret_cast<stream_t>(c->stream));
  if (rc) return fail(c, rc, "zone launch failed");
  if ((rc = to_user(c, gradient, z->gz, (size_t)z->nz))) return rc;
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_zones_descend(cf_zones* z, double lr, double lo, double hi) {
  if (!z) return CF_EINVAL;
  cf_ctx* c = z->ctx;
  if (!(lo <= hi)) return fail(c, CF_EINVAL, "lo > hi");
  CF_CUDA(c, cudaSetDevice(c->device));
  const stream_t st = reinterpret_cast<stream_t>(c->stream);
  int rc = launch_zone_step(z->vals, z->gz, z->nz, lr, lo, hi, st);
  if (rc == CF_OK) rc = launch_zone_apply(c->cstat, z->zone_of, z->vals, c->n_pad, st);
  if (rc) return fail(c, rc, "zone launch failed");
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

}  // extern "C"
