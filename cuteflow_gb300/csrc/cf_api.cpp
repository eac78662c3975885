/*
 * cf_api.cpp -- the C ABI of include/cuteflow_gb300.h.
 *
 * A context holds one or more independent simulations ("members") packed into one flat
 * element/edge space: member m owns the elements [cell_off, cell_off + n) and the edges
 * [edge_off, edge_off + ne), both padded to whole tiles (TILE_C elements, TILE_E edges), so
 * every tile, and every thread block, belongs to one member.  A step is then two kernel
 * launches over all members together, each member with its own parameters, time, dt and
 * status.  The plain API (cf_create, cf_set_state, ...) is the one-member case.
 *
 * Stepping never returns to the host between steps: the next dt of every member is produced on
 * the device by the element kernel and read by the next edge kernel.  The host reads the small
 * per-member records once at the end of a cf_step call.  Runs of steps are replayed from a
 * captured CUDA graph of two steps (even and odd buffer parity).
 */
#include <cuda_runtime.h>

#include <cstddef>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "cf_ctx.h"

using namespace cf;

namespace cf {

thread_local std::string g_create_error;

int fail(cf_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  else g_create_error = msg;
  return code;
}

int cuda_fail(cf_ctx* c, cudaError_t e, const char* what) {
  std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(c, e == cudaErrorMemoryAllocation ? CF_ENOMEM : CF_ECUDA, msg);
}

StepArgs step_args(const cf_ctx* c, int parity) {
  StepArgs a{};
  a.Uin = c->U[parity];
  a.Uout = c->U[1 - parity];
  a.cslot = c->cslot;
  a.cnbr = c->cnbr;
  a.cstat = c->cstat;
  a.ecell = c->ecell;
  a.egeo = c->egeo;
  a.ebid = c->ebid;
  a.ez = c->ez;
  a.eupw = c->eupw;
  a.ewts = c->ewts;
  a.edk = c->edk;
  a.einv = c->einv;
  a.slots = c->slots;
  a.etile_mem = c->etile_mem;
  a.ctile_mem = c->ctile_mem;
  a.mdev = c->mdev;
  a.mst = c->mst;
  a.n_etiles = c->n_etiles;
  a.n_ctiles = c->n_ctiles;
  a.parity = parity;
  a.iflux = c->iflux;
  a.ilimiteur = c->ilimiteur;
  a.flux_mode = c->flux_mode;
  a.inl_cell = c->inl_cell;
  a.inl_len = c->inl_len;
  a.nmembers = (int32_t)c->mem.size();
  a.phys_inflow = c->any_phys_inflow ? 1 : 0;
  a.steady = c->any_steady ? 1 : 0;
  a.xd_cmp = c->xd_cmp;
  a.xd_mul_mask = c->xd_mul_mask;
  a.eblock = c->eblock;
  a.ept = c->ept;
  a.cblock = c->cblock;
  a.c_lo = 0;
  a.c_hi = 0x7fffffff;
  a.bq = c->bq;
  a.sums_out = nullptr;
  return a;
}

void free_all(cf_ctx* c) {
  if (c->graph2) cudaGraphExecDestroy(c->graph2);
  void* ptrs[] = {c->U[0], c->U[1], c->cslot, c->cnbr, c->cstat, c->zcell, c->perm, c->iperm, c->ecell, c->egeo, c->ez,
                  c->ebid, c->eupw, c->ewts, c->edk, c->einv, c->slots, c->etile_mem, c->ctile_mem, c->mdev,
                  c->mst, c->staging, c->inl_cell, c->inl_len, c->ids, c->bq, c->elist1, c->elist2,
                  c->xsend, c->xrecv, c->terms};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->host_state) cudaFreeHost(c->host_state);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->ev_pack) cudaEventDestroy(c->ev_pack);
  if (c->stream) cudaStreamDestroy(c->stream);
}

int read_states(cf_ctx* c) {
  CF_CUDA(c, cudaMemcpyAsync(c->host_state, c->mst, c->mem.size() * sizeof(MemberState), cudaMemcpyDeviceToHost,
                             c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

void fill_info(const MemberState& s, cf_step_info* info) {
  const int cur = (int)((s.base + s.nstep) & 1);
  info->steps = s.nstep;
  info->t = s.t[cur];
  info->dt_next = s.dt[cur];
  info->dt_last = s.nstep > 0 ? s.dt[1 - cur] : 0.0;
  info->q_in = s.q_in;
  info->q_out = s.q_out;
  info->status = s.status & ~STATUS_NO_STATE;
  info->pad_ = 0;
}

int status_code(uint32_t st) {
  if (st & STATUS_NO_STATE) return CF_ESTATE;
  if (st & CF_STATUS_NONFINITE) return CF_ENONFINITE;
  if (st & CF_STATUS_DT_RANGE) return CF_EDT;
  return CF_OK;
}

int enqueue_step(cf_ctx* c, int parity, bool timed) {
  StepArgs a = step_args(c, parity);
  int rc = launch_step(a, reinterpret_cast<stream_t>(c->stream), timed ? c->ev[1] : nullptr,
                       timed ? c->ev[2] : nullptr);
  if (rc != CF_OK) return fail(c, rc, rc == CF_ENOTSUP ? "iflux not supported by the GPU step" : "kernel launch failed");
  return CF_OK;
}

int build_graph(cf_ctx* c) {
  cudaGraph_t g = nullptr;
  CF_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int rc0 = enqueue_step(c, 0, false);
  int rc1 = rc0 == CF_OK ? enqueue_step(c, 1, false) : rc0;
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (rc1 != CF_OK) {
    if (g) cudaGraphDestroy(g);
    return rc1;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&c->graph2, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
  return CF_OK;
}

int check_params(const cf_params* p, std::string& why) {
  if (p->iflux < 1 || p->iflux > 4) { why = "iflux must be 1..4"; return CF_EINVAL; }
  if (p->inlet < 1 || p->inlet > 3 || p->outlet < 1 || p->outlet > 2) { why = "inlet must be 1..3 and outlet 1..2"; return CF_EINVAL; }
  if (p->ilimiteur < 0 || p->ilimiteur > 4) { why = "ilimiteur must be 0..4"; return CF_EINVAL; }
  if (p->flux_mode < 0 || p->flux_mode > 1) { why = "flux_mode must be 0 or 1"; return CF_EINVAL; }
  if (p->fricimplic < 0 || p->fricimplic > 2) { why = "fricimplic must be 0..2"; return CF_EINVAL; }
  if (!(p->gp > 0.0) || !(p->cfl > 0.0) || !(p->tolisec >= 0.0)) { why = "gp and cfl must be positive, tolisec non-negative"; return CF_EINVAL; }
  if (p->ramp_time < 0.0) { why = "ramp_time must be non-negative"; return CF_EINVAL; }
  if (!(p->tol_reg_perm >= 0.0)) { why = "tol_reg_perm must be non-negative"; return CF_EINVAL; }
  if (p->reorder < 0 || p->reorder > 2) { why = "reorder must be 0 (the caller's order), 1 (Hilbert) or 2 (Morton)"; return CF_EINVAL; }
  return CF_OK;
}

MemberDev member_dev(const Member& M) {
  const cf_params* p = &M.params;
  MemberDev D;
  std::memset(&D, 0, sizeof(D));
  D.gp = p->gp;
  D.tolisec = p->tolisec;
  D.tol = p->tol;
  D.constant_dt = p->constant_dt;
  D.ramp_time = p->ramp_time;
  D.dt_reset = ((p->dt_reset_nelt > 0 ? p->dt_reset_nelt : M.n) % 1024 != 0) ? 100000.0 : 1000000.0;
  for (int i = 0; i < CF_MAX_IO; ++i) {
    D.debit_end[i] = p->debitglob[i];
    D.debit_start[i] = p->debitglob_start[i];
    D.long_entree[i] = M.prep.long_entree[i];
    D.h_sortie[i] = p->h_sortie[i];
  }
  D.inlet = p->inlet;
  D.outlet = p->outlet;
  D.friction = p->friction;
  D.fricimplic = p->fricimplic;
  D.is_dt_constant = p->is_dt_constant;
  D.cell_begin = M.cell_off;
  D.cell_end = M.cell_off + M.n;
  D.edge_begin = M.edge_off;
  D.edge_end = M.edge_off + M.ne;
  D.bedge_begin = M.edge_off + M.prep.n_interior;
  D.bedge_end = M.edge_off + M.ne;
  D.inl_begin = M.inl_off;
  D.inl_count = (int32_t)M.prep.inl_cell.size();
  D.nin = M.prep.nin;
  D.tol_reg_perm = p->tol_reg_perm;
  D.steady_count = p->steady_count > 0 ? p->steady_count : 1000;
  return D;
}

/* Build a context of nm members (the meshes are preprocessed in parallel on the host). */
int create_impl(const cf_mesh* meshes, const cf_params* params, int32_t nm, cf_ctx** out,
                const int32_t* elem_class = nullptr) {
  if (!out) return fail(nullptr, CF_EINVAL, "out is NULL");
  *out = nullptr;
  if (!meshes || !params || nm < 1) return fail(nullptr, CF_EINVAL, "meshes/params NULL or no member");
  std::string why;
  for (int i = 0; i < nm; ++i) {
    int rc = check_params(&params[i], why);
    if (rc != CF_OK) return fail(nullptr, rc, "member " + std::to_string(i) + ": " + why);
    if (params[i].iflux != params[0].iflux || params[i].ilimiteur != params[0].ilimiteur ||
        params[i].flux_mode != params[0].flux_mode)
      return fail(nullptr, CF_EINVAL, "all members must share iflux, ilimiteur and flux_mode");
  }
  cf_ctx* c = new (std::nothrow) cf_ctx();
  if (!c) return fail(nullptr, CF_ENOMEM, "host allocation failed");
  c->iflux = params[0].iflux;
  c->ilimiteur = params[0].ilimiteur;
  c->flux_mode = params[0].flux_mode;
  c->mem.resize(nm);
  for (int i = 0; i < nm; ++i) c->mem[i].params = params[i];
  /* host preprocessing, members in parallel */
  std::vector<int> rcs(nm, CF_OK);
  std::vector<std::string> errs(nm);
  {
    std::atomic<int> next(0);
    unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int nth = (int)std::min<unsigned>(hw, (unsigned)nm);
    auto work = [&]() {
      for (int i = next++; i < nm; i = next++)
        rcs[i] = prepare_mesh(&meshes[i], &params[i], c->mem[i].prep, errs[i], elem_class);
    };
    std::vector<std::thread> th;
    for (int t = 1; t < nth; ++t) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
  }
  for (int i = 0; i < nm; ++i)
    if (rcs[i] != CF_OK) {
      std::string msg = (nm > 1 ? "member " + std::to_string(i) + ": " : std::string()) + errs[i];
      delete c;
      return fail(nullptr, rcs[i], msg);
    }
  auto done = [&](int code) {
    if (code != CF_OK) {
      g_create_error = c->err;
      free_all(c);
      delete c;
      return code;
    }
    *out = c;
    return CF_OK;
  };
  /* layout of the flat space */
  int64_t noff = 0, eoff = 0, ioff = 0;
  for (auto& M : c->mem) {
    M.inl_off = (int32_t)ioff;
    ioff += (int64_t)M.prep.inl_cell.size();
    c->any_phys_inflow |= M.params.inlet == 3;
    c->any_steady |= M.params.tol_reg_perm > 0.0;
    M.n = M.prep.nelt;
    M.ne = (int32_t)M.prep.edges.size();
    M.cell_off = (int32_t)noff;
    M.edge_off = (int32_t)eoff;
    M.ctile_begin = (int32_t)(noff / TILE_C);
    noff += (M.n + TILE_C - 1) / TILE_C * (int64_t)TILE_C;
    eoff += (M.ne + TILE_E - 1) / TILE_E * (int64_t)TILE_E;
    M.ctile_end = (int32_t)(noff / TILE_C);
    c->max_n = std::max(c->max_n, M.n);
    M.dev = member_dev(M);
  }
  if (noff > 0x7fffffffLL || 2 * eoff > 0x7fffffffLL) return done(fail(c, CF_EINVAL, "batch too large for 32-bit indices"));
  c->n_pad = (int32_t)noff;
  c->ne_pad = (int32_t)eoff;
  c->n_ctiles = c->n_pad / TILE_C;
  c->n_etiles = c->ne_pad / TILE_E;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaGetDevice"));
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaStreamCreate"));
  for (auto& ev : c->ev) {
    e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaEventCreate"));
  }
  int rc;
  const bool second = c->iflux >= 3;
  if ((rc = dalloc(c, &c->U[0], c->n_pad)) || (rc = dalloc(c, &c->U[1], c->n_pad)) ||
      (rc = dalloc(c, &c->cslot, c->n_pad)) || (rc = dalloc(c, &c->cnbr, c->n_pad)) || (rc = dalloc(c, &c->cstat, c->n_pad)) ||
      (rc = dalloc(c, &c->zcell, c->n_pad)) || (rc = dalloc(c, &c->perm, c->n_pad)) ||
      (rc = dalloc(c, &c->iperm, c->n_pad)) || (rc = dalloc(c, &c->ecell, c->ne_pad)) ||
      (rc = dalloc(c, &c->egeo, c->ne_pad)) || (rc = dalloc(c, &c->ebid, c->ne_pad)) ||
      (rc = dalloc(c, &c->ez, c->ne_pad)) ||
      (rc = dalloc(c, &c->slots, 2 * (size_t)c->ne_pad)) || (rc = dalloc(c, &c->etile_mem, c->n_etiles)) ||
      (rc = dalloc(c, &c->ctile_mem, c->n_ctiles)) || (rc = dalloc(c, &c->mdev, (size_t)nm)) ||
      (rc = dalloc(c, &c->mst, (size_t)nm)) || (rc = dalloc(c, &c->staging, 3 * (size_t)c->max_n)))
    return done(rc);
  c->n_inl = ioff;
  if (c->any_phys_inflow) {
    size_t nl = 0;
    for (auto& M : c->mem) nl += M.prep.inl_len.size();
    if ((rc = dalloc(c, &c->inl_cell, (size_t)ioff)) || (rc = dalloc(c, &c->inl_len, nl))) return done(rc);
  }
  if (second && ((rc = dalloc(c, &c->eupw, c->ne_pad)) || (rc = dalloc(c, &c->ewts, c->ne_pad)) ||
                 (rc = dalloc(c, &c->edk, c->ne_pad)) || (rc = dalloc(c, &c->einv, c->ne_pad))))
    return done(rc);
  /* per-member uploads with the member offsets applied */
  std::vector<int32_t> etm(c->n_etiles), ctm(c->n_ctiles);
  std::vector<MemberDev> mdev(nm);
  for (int i = 0; i < nm; ++i) {
    Member& M = c->mem[i];
    Prep& P = M.prep;
    const int32_t co = M.cell_off, eo = M.edge_off;
    for (int t = M.ctile_begin; t < M.ctile_end; ++t) ctm[t] = i;
    for (int t = eo / TILE_E; t < (eo + (M.ne + TILE_E - 1) / TILE_E * TILE_E) / TILE_E; ++t) etm[t] = i;
    std::vector<int4> cslot(P.cslot);
    for (auto& s : cslot) { s.x += 2 * eo; s.y += 2 * eo; s.z += 2 * eo; }
    std::vector<int2> ecell(P.ecell);
    for (auto& e2 : ecell) { e2.x += co; if (e2.y >= 0) e2.y += co; }
    std::vector<int4> cnbr(P.cnbr);
    for (auto& b : cnbr) {
      if (b.x >= 0) b.x += co;
      if (b.y >= 0) b.y += co;
      if (b.z >= 0) b.z += co;
    }
    if ((rc = put(c, c->cslot + co, cslot.data(), cslot.size())) || (rc = put(c, c->cnbr + co, cnbr.data(), cnbr.size())) || (rc = put(c, c->cstat + co, P.cstat.data(), P.cstat.size())) ||
        (rc = put(c, c->zcell + co, P.zcell.data(), P.zcell.size())) || (rc = put(c, c->perm + co, P.perm.data(), P.perm.size())) ||
        (rc = put(c, c->iperm + co, P.iperm.data(), P.iperm.size())) || (rc = put(c, c->ecell + eo, ecell.data(), ecell.size())) ||
        (rc = put(c, c->egeo + eo, P.egeo.data(), P.egeo.size())) || (rc = put(c, c->ebid + eo, P.ebid.data(), P.ebid.size())) ||
        (rc = put(c, c->ez + eo, P.ez.data(), P.ez.size())))
      return done(rc);
    if (second) {
      std::vector<int4> up(P.eupw);
      for (auto& u : up) { u.x += co; u.y += co; u.z += co; u.w += co; }
      if ((rc = put(c, c->eupw + eo, up.data(), up.size())) || (rc = put(c, c->ewts + eo, P.ewts.data(), P.ewts.size())) ||
          (rc = put(c, c->edk + eo, P.edk.data(), P.edk.size())) || (rc = put(c, c->einv + eo, P.einv.data(), P.einv.size())))
        return done(rc);
      std::vector<int4>().swap(P.eupw);
      std::vector<double4>().swap(P.ewts);
      std::vector<double4>().swap(P.edk);
      std::vector<double4>().swap(P.einv);
    }
    if (!P.inl_cell.empty()) {
      /* entry lengths are stored per member with that member's inlet count */
      std::vector<int32_t> cells(P.inl_cell);
      for (auto& x : cells) x += co;
      size_t loff = 0;
      for (int j = 0; j < i; ++j) loff += c->mem[j].prep.inl_len.size();
      M.dev.inl_len_off = (int32_t)loff;
      if ((rc = put(c, c->inl_cell + M.inl_off, cells.data(), cells.size())) ||
          (rc = put(c, c->inl_len + loff, P.inl_len.data(), P.inl_len.size())))
        return done(rc);
    }
    mdev[i] = M.dev;
    /* the device copies are authoritative; keep the reference-order tables and the permutation */
    std::vector<int4>().swap(P.cslot);
    std::vector<int4>().swap(P.cnbr);
    std::vector<double4>().swap(P.cstat);
    std::vector<int2>().swap(P.ecell);
    std::vector<double4>().swap(P.egeo);
    std::vector<double4>().swap(P.ez);
    std::vector<int32_t>().swap(P.ebid);
    std::vector<HostEdge>().swap(P.edges);
  }
  /* boundary edges in reference order (flat, edge offsets applied) */
  {
    std::vector<int32_t> bq;
    for (int i = 0; i < nm; ++i) {
      Member& M = c->mem[i];
      mdev[i].bq_begin = M.dev.bq_begin = (int32_t)bq.size();
      mdev[i].bq_count = M.dev.bq_count = (int32_t)M.prep.bq_ref.size();
      for (int32_t e : M.prep.bq_ref) bq.push_back(e + M.edge_off);
    }
    if ((rc = dalloc(c, &c->bq, bq.size())) || (rc = put(c, c->bq, bq.data(), bq.size()))) return done(rc);
  }
  /* a part of a decomposed mesh: its phase edge lists */
  if (elem_class) {
    const Prep& P = c->mem[0].prep;
    c->is_part = true;
    c->n_send = P.n_send;
    c->n_own = P.n_own;
    c->nel1 = (int32_t)P.elist1.size();
    c->nel2 = (int32_t)P.elist2.size();
    if ((rc = dalloc(c, &c->elist1, P.elist1.size())) || (rc = dalloc(c, &c->elist2, P.elist2.size())) ||
        (rc = put(c, c->elist1, P.elist1.data(), P.elist1.size())) ||
        (rc = put(c, c->elist2, P.elist2.data(), P.elist2.size())))
      return done(rc);
    e = cudaEventCreateWithFlags(&c->ev_pack, cudaEventDisableTiming);
    if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaEventCreate"));
    const size_t nt = std::max(P.inl_cell.size() * (size_t)std::max(P.nin, 1), P.bq_ref.size());
    if ((rc = dalloc(c, &c->terms, std::max<size_t>(nt, 1)))) return done(rc);
  }
  if ((rc = put(c, c->etile_mem, etm.data(), etm.size())) || (rc = put(c, c->ctile_mem, ctm.data(), ctm.size())) ||
      (rc = put(c, c->mdev, mdev.data(), mdev.size())))
    return done(rc);
  e = cudaMallocHost((void**)&c->host_state, nm * sizeof(MemberState));
  if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaMallocHost"));
  for (int i = 0; i < nm; ++i) {
    std::memset(&c->host_state[i], 0, sizeof(MemberState));
    c->host_state[i].status = STATUS_NO_STATE;
  }
  if ((rc = put(c, c->mst, c->host_state, (size_t)nm))) return done(rc);
  return done(CF_OK);
}

int member_ok(cf_ctx* c, int32_t m) {
  if (!c) return CF_EINVAL;
  if (m < 0 || m >= (int32_t)c->mem.size()) return fail(c, CF_EINVAL, "member index out of range");
  return CF_OK;
}

/* The address through which the kernels on c's device reach the caller's buffer p: p itself for
 * device or managed memory of that device, the mapped address for pinned host memory (GB300 reads
 * and writes it over the coherent CPU link), NULL for anything else (pageable host memory, another
 * device's memory, a pointer not aligned to 8 bytes, or direct access switched off): such buffers
 * go through the staging buffer with a copy. */
void* device_view(cf_ctx* c, const void* p) {
  if (!c->direct_io || !p || ((uintptr_t)p & 7u)) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
    return a.device == c->device ? const_cast<void*>(p) : nullptr;
  if (a.type == cudaMemoryTypeHost) return a.devicePointer;
  return nullptr;
}

/* Set the state of member m, resetting its time and steps: from src (reference order, an address
 * the device reaches, see device_view) or, with src NULL, from c->staging.  Stream-ordered, no
 * wait; c->ev[3] completes once the caller's inputs have been read. */
int enqueue_set_state(cf_ctx* c, int32_t m, double t0, const double* src = nullptr) {
  const Member& M = c->mem[m];
  const int p0 = (int)(c->launched & 1);
  MemberState s;
  std::memset(&s, 0, sizeof(s));
  s.dt[p0] = M.dev.dt_reset;
  s.t[p0] = t0;
  s.tc = t0;
  s.ts = INFINITY;
  s.base = p0;
  c->host_state[m] = s;
  CF_CUDA(c, cudaMemcpyAsync(c->mst + m, c->host_state + m, sizeof(MemberState), cudaMemcpyHostToDevice, c->stream));
  int rc;
  if (src) {
    /* the state, and with it the first dt (the block minima of its CFL dt) */
    rc = launch_load_ref(src, c->iperm + M.cell_off, c->U[p0] + M.cell_off, M.n, reinterpret_cast<stream_t>(c->stream),
                         c->cstat + M.cell_off, c->mdev, c->mst, m, p0);
    if (rc != CF_OK) return fail(c, rc, "state load launch failed");
    CF_CUDA(c, cudaEventRecord(c->ev[3], c->stream));   /* the host inputs (caller's state, member record) read */
    return CF_OK;
  } else {
    CF_CUDA(c, cudaEventRecord(c->ev[3], c->stream));   /* the host inputs (caller's state, member record) read */
    rc = launch_scatter_state(c->staging, c->perm + M.cell_off, c->zcell + M.cell_off, c->U[p0] + M.cell_off, M.n,
                              reinterpret_cast<stream_t>(c->stream));
    if (rc != CF_OK) return fail(c, rc, "state scatter launch failed");
  }
  rc = launch_cfl(c->U[p0], c->cstat, c->ctile_mem, M.ctile_begin, M.ctile_end - M.ctile_begin, c->mdev, c->mst, p0,
                  reinterpret_cast<stream_t>(c->stream));
  if (rc != CF_OK) return fail(c, rc, "cfl launch failed");
  return CF_OK;
}

int set_state_member(cf_ctx* c, int32_t m, double t0, const double* src = nullptr) {
  const int rc = enqueue_set_state(c, m, t0, src);
  if (rc != CF_OK) return rc;
  /* return once the host buffers are consumed; the scatter and the initial dt run on the stream
   * ahead of the next call's work (which every later call orders after) */
  CF_CUDA(c, cudaEventSynchronize(c->ev[3]));
  return CF_OK;
}

int set_state_host(cf_ctx* c, int32_t m, const double* hu3, double t0, cudaMemcpyKind kind) {
  int rc = member_ok(c, m);
  if (rc) return rc;
  if (!hu3) return fail(c, CF_EINVAL, "null state");
  CF_CUDA(c, cudaSetDevice(c->device));
  if (const void* v = device_view(c, hu3)) return set_state_member(c, m, t0, static_cast<const double*>(v));
  CF_CUDA(c, cudaMemcpyAsync(c->staging, hu3, 3 * (size_t)c->mem[m].n * sizeof(double), kind, c->stream));
  return set_state_member(c, m, t0);
}

/* set_initial_condition, initial_condition.cuf:18-79, evaluated on the host (setup only). */
int initial_condition(cf_ctx* c, int32_t m, const cf_ic* ic, double t0) {
  int rc = member_ok(c, m);
  if (rc) return rc;
  if (!ic) return fail(c, CF_EINVAL, "null argument");
  const Member& M = c->mem[m];
  const Prep& P = M.prep;
  std::vector<double> U(3 * (size_t)M.n, 0.0);
  const double tolisec = M.params.tolisec;
  for (int k = 0; k < M.n; ++k) {
    const double zmd = P.zm[k], v1 = P.xc[k], v2 = P.yc[k];
    double* u = &U[3 * (size_t)k];
    if (ic->eqlin_barrage == 1) {
      const double alpha = (ic->y1eqbar - ic->y2eqbar) / (ic->x1eqbar - ic->x2eqbar);
      const double beta = ic->y1eqbar - alpha * ic->x1eqbar;
      const bool up = alpha * v1 - v2 + beta >= 0.00;
      const double h = (up ? ic->h_amont : ic->h_aval) - zmd;
      u[0] = h;
      if (h > tolisec) {
        u[1] = h * (up ? ic->u_amont : ic->u_aval);
        u[2] = h * (up ? ic->v_amont : ic->v_aval);
      } else {
        u[0] = u[1] = u[2] = 0.0;
      }
    }
    if (ic->plan == 1) {
      const double h = (-(ic->xplan * (ic->xpoint - v1)) - ic->yplan * (ic->ypoint - v2)) / ic->zplan + ic->zpoint - zmd;
      u[0] = h;
      if (h > tolisec) {
        u[1] = h * ic->u_aval;
        u[2] = h * ic->v_aval;
      } else {
        u[0] = u[1] = u[2] = 0.0;
      }
    }
  }
  return set_state_host(c, m, U.data(), t0, cudaMemcpyHostToDevice);
}

int get_state_member(cf_ctx* c, int32_t m, double* dst, cudaMemcpyKind kind) {
  int rc = member_ok(c, m);
  if (rc) return rc;
  if (!dst) return fail(c, CF_EINVAL, "null destination");
  CF_CUDA(c, cudaSetDevice(c->device));
  if ((rc = read_states(c))) return rc;
  const MemberState& s = c->host_state[m];
  if (s.status & STATUS_NO_STATE) return fail(c, CF_ESTATE, "no state set");
  const Member& M = c->mem[m];
  const int buf = (int)((s.base + s.nstep) & 1);
  if (void* v = device_view(c, dst)) {
    rc = launch_store_ref(c->U[buf] + M.cell_off, nullptr, nullptr, 0, c->iperm + M.cell_off, static_cast<double*>(v),
                          M.n, reinterpret_cast<stream_t>(c->stream));
    if (rc != CF_OK) return fail(c, rc, "state store launch failed");
    CF_CUDA(c, cudaStreamSynchronize(c->stream));
    return CF_OK;
  }
  rc = launch_gather_state(c->U[buf] + M.cell_off, c->iperm + M.cell_off, c->staging, M.n,
                           reinterpret_cast<stream_t>(c->stream));
  if (rc != CF_OK) return fail(c, rc, "gather launch failed");
  CF_CUDA(c, cudaMemcpyAsync(dst, c->staging, 3 * (size_t)M.n * sizeof(double), kind, c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

/* the launches of nsteps steps and the discharge diagnostics (stream-ordered, no wait) */
int enqueue_steps(cf_ctx* c, int32_t nsteps) {
  if (nsteps < 0) return fail(c, CF_EINVAL, "nsteps < 0");
  CF_CUDA(c, cudaSetDevice(c->device));
  int rc;
  c->flux_ms = c->update_ms = 0.0;
  c->launches = 0;
  int32_t left = nsteps;
  if (c->timing) {
    for (int32_t i = 0; i < nsteps; ++i) {
      CF_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
      if ((rc = enqueue_step(c, (int)((c->launched + i) & 1), true))) return rc;
      CF_CUDA(c, cudaEventSynchronize(c->ev[2]));
      float a = 0.f, b = 0.f;
      cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
      cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
      c->flux_ms += a;
      c->update_ms += b;
      c->launches += 2;
    }
    left = 0;
  } else {
    if (left > 0 && (c->launched & 1)) {
      if ((rc = enqueue_step(c, 1, false))) return rc;
      --left;
    }
    if (c->use_graph && left >= 2) {
      if (!c->graph2 && (rc = build_graph(c))) return rc;
      for (; left >= 2; left -= 2) CF_CUDA(c, cudaGraphLaunch(c->graph2, c->stream));
    }
    while (left > 0) {
      if ((rc = enqueue_step(c, (int)((c->launched + nsteps - left) & 1), false))) return rc;
      --left;
    }
    c->launches = 2 * (int64_t)nsteps;
  }
  c->launched += nsteps;
  rc = launch_discharge(c->slots, c->ecell, c->bq, c->mdev, c->mst, (int32_t)c->mem.size(),
                        reinterpret_cast<stream_t>(c->stream));
  if (rc != CF_OK) return fail(c, rc, "discharge launch failed");
  return CF_OK;
}

/* wait for the stream, read the member records back and report them (info, status code) */
int finish_steps(cf_ctx* c, cf_step_info* infos) {
  int rc;
  if ((rc = read_states(c))) return rc;
  uint32_t any = 0;
  for (size_t i = 0; i < c->mem.size(); ++i) {
    if (infos) fill_info(c->host_state[i], &infos[i]);
    any |= c->host_state[i].status;
  }
  if (c->mem.size() == 1 && (any & STATUS_NO_STATE)) return fail(c, CF_ESTATE, "cf_step before a state was set");
  rc = status_code(any & ~STATUS_NO_STATE);
  if (rc != CF_OK)
    return fail(c, rc, rc == CF_EDT ? "dt left the range (1e-12, 9999]" : "non-finite value in the state");
  return CF_OK;
}

int step_impl(cf_ctx* c, int32_t nsteps, cf_step_info* infos) {
  if (!c) return CF_EINVAL;
  const int rc = enqueue_steps(c, nsteps);
  if (rc != CF_OK) return rc;
  return finish_steps(c, infos);
}

/* The reference's time loop until its end test on ts (finite_volumes_method.cuf:123), the
 * steady-state stop or max_steps: steps in chunks, the device stopping each member at its
 * own step; the host looks between chunks whether any member is still running. */
int run_impl(cf_ctx* c, double ts, int64_t max_steps, cf_step_info* infos) {
  if (!(ts == ts)) return fail(c, CF_EINVAL, "ts is NaN");
  if (max_steps < 0) return fail(c, CF_EINVAL, "max_steps < 0");
  CF_CUDA(c, cudaSetDevice(c->device));
  int rc;
  if ((rc = read_states(c))) return rc;
  const size_t nm = c->mem.size();
  for (size_t i = 0; i < nm; ++i) {
    MemberState& s = c->host_state[i];
    if (s.status & STATUS_NO_STATE) {
      if (nm == 1) return fail(c, CF_ESTATE, "cf_run before a state was set");
      continue;
    }
    if ((s.status & ~CF_STATUS_END) != 0) continue;  /* stopped for another reason */
    if (s.status & CF_STATUS_END) {
      /* steps launched while the member stood still have moved the launch parity: move its
       * state (and dt, t) to the buffer the next launch reads */
      const int cur = (int)((s.base + s.nstep) & 1), want = (int)(c->launched & 1);
      if (cur != want) {
        const Member& M = c->mem[i];
        CF_CUDA(c, cudaMemcpyAsync(c->U[want] + M.cell_off, c->U[cur] + M.cell_off, (size_t)M.n * sizeof(double4),
                                   cudaMemcpyDeviceToDevice, c->stream));
        s.dt[want] = s.dt[cur];
        s.t[want] = s.t[cur];
        s.base ^= 1;
      }
    }
    s.status &= ~CF_STATUS_END;                      /* a later end time continues the run */
    s.ts = ts;
    CF_CUDA(c, cudaMemcpyAsync(c->mst + i, &s, sizeof(MemberState), cudaMemcpyHostToDevice, c->stream));
  }
  const int64_t chunk = 256;
  int64_t done = 0;
  while (done < max_steps) {
    const int32_t k = (int32_t)std::min<int64_t>(chunk, max_steps - done);
    if ((rc = step_impl(c, k, infos)) != CF_OK) return rc;
    done += k;
    bool running = false;
    for (size_t i = 0; i < nm; ++i) running |= c->host_state[i].status == 0;
    if (!running) break;
  }
  if (done == 0 && (rc = step_impl(c, 0, infos)) != CF_OK) return rc;
  return CF_OK;
}

}  // namespace

/* ---- helpers of the static-scratch entry point (cf_noalloc.cu) ---------------------------- */

int cf::ctx_set_device(cf_ctx* c) {
  CF_CUDA(c, cudaSetDevice(c->device));
  return CF_OK;
}

int cf::ctx_error(cf_ctx* c, int code, const std::string& msg) { return fail(c, code, msg); }

int cf::step_with_slots(cf_ctx* c, int32_t nsteps, cf_step_info* infos, Slot* slots, size_t capacity) {
  if (nsteps < 0) return fail(c, CF_EINVAL, "nsteps < 0");
  const size_t need = 2 * (size_t)c->ne_pad;
  if (need > capacity) {
    char msg[256];
    std::snprintf(msg, sizeof(msg),
                  "the context needs %zu edge-flux slots (%zu bytes) but the static scratch holds %zu (%zu bytes)",
                  need, need * sizeof(Slot), capacity, capacity * sizeof(Slot));
    return fail(c, CF_EINVAL, msg);
  }
  int rc;
  const stream_t s = reinterpret_cast<stream_t>(c->stream);
  if (nsteps > 0) {
    /* the scratch keeps whatever the previous call left: start from zero like a new context */
    CF_CUDA(c, cudaMemsetAsync(slots, 0, need * sizeof(Slot), c->stream));
    for (int32_t i = 0; i < nsteps; ++i) {
      StepArgs a = step_args(c, (int)((c->launched + i) & 1));
      a.slots = slots;
      if ((rc = launch_step(a, s, nullptr, nullptr))) return fail(c, rc, "step launch failed");
    }
    c->launched += nsteps;
    rc = launch_discharge(slots, c->ecell, c->bq, c->mdev, c->mst, (int32_t)c->mem.size(), s);
    if (rc != CF_OK) return fail(c, rc, "discharge launch failed");
  }
  c->flux_ms = c->update_ms = 0.0;
  c->launches = 2 * (int64_t)nsteps;
  if ((rc = read_states(c))) return rc;
  uint32_t any = 0;
  for (size_t i = 0; i < c->mem.size(); ++i) {
    if (infos) fill_info(c->host_state[i], &infos[i]);
    any |= c->host_state[i].status;
  }
  if (c->mem.size() == 1 && (any & STATUS_NO_STATE)) return fail(c, CF_ESTATE, "step before a state was set");
  rc = status_code(any & ~STATUS_NO_STATE);
  if (rc != CF_OK)
    return fail(c, rc, rc == CF_EDT ? "dt left the range (1e-12, 9999]" : "non-finite value in the state");
  return CF_OK;
}

extern "C" {

int cf_run(cf_ctx* ctx, double ts, int64_t max_steps, cf_step_info* info) {
  if (!ctx) return CF_EINVAL;
  return run_impl(ctx, ts, max_steps, info);
}

int cf_set_tuning(cf_ctx* ctx, int32_t int_compare, int32_t int_mul_warps) {
  if (!ctx) return CF_EINVAL;
  if (int_compare < 0 || int_compare > 1 || int_mul_warps < 0 || int_mul_warps > 0x1f)
    return fail(ctx, CF_EINVAL, "int_compare must be 0/1 and int_mul_warps a 4-bit warp mask plus bit 4");
  if (int_mul_warps && !int_compare) return fail(ctx, CF_EINVAL, "integer products need int_compare = 1");
  if (ctx->xd_cmp != int_compare || ctx->xd_mul_mask != int_mul_warps) {
    ctx->xd_cmp = int_compare;
    ctx->xd_mul_mask = int_mul_warps;
    if (ctx->graph2) {   /* the captured steps hold the old arguments */
      CF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      cudaGraphExecDestroy(ctx->graph2);
      ctx->graph2 = nullptr;
    }
  }
  return CF_OK;
}

int cf_probe_fp64(cf_ctx* ctx, double* instr_per_s) {
  if (!ctx || !instr_per_s) return CF_EINVAL;
  cf_ctx* c = ctx;
  CF_CUDA(c, cudaSetDevice(c->device));
  int sms = 0;
  CF_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  const int32_t nblocks = 8 * sms;
  const int64_t iters = 4096;
  double* out = nullptr;
  int rc = dalloc(c, &out, (size_t)nblocks * 256);
  if (rc) return rc;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float ms = 0.0f;
  cudaError_t err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  if (err == cudaSuccess) rc = launch_probe_fp64(out, nblocks, iters, reinterpret_cast<stream_t>(c->stream));
  if (err == cudaSuccess && rc == CF_OK) err = cudaEventRecord(e0, c->stream);
  if (err == cudaSuccess && rc == CF_OK) rc = launch_probe_fp64(out, nblocks, iters, reinterpret_cast<stream_t>(c->stream));
  if (err == cudaSuccess && rc == CF_OK) err = cudaEventRecord(e1, c->stream);
  if (err == cudaSuccess && rc == CF_OK) err = cudaEventSynchronize(e1);
  if (err == cudaSuccess && rc == CF_OK) err = cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return cuda_fail(c, err, "cf_probe_fp64");
  if (rc != CF_OK) return fail(c, rc, "cf_probe_fp64 launch failed");
  *instr_per_s = (double)nblocks * 256.0 * 8.0 * (double)iters / (ms * 1e-3);
  return CF_OK;
}

int cf_selftest_xd(cf_ctx* ctx, int64_t n, uint64_t seed, int64_t* mismatches) {
  if (!ctx || !mismatches || n < 0) return CF_EINVAL;
  cf_ctx* c = ctx;
  CF_CUDA(c, cudaSetDevice(c->device));
  int sms = 0;
  CF_CUDA(c, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  unsigned long long* bad = nullptr;
  int rc = dalloc(c, &bad, 1);
  if (rc) return rc;
  unsigned long long h = 0;
  cudaError_t err = cudaMemsetAsync(bad, 0, sizeof(*bad), c->stream);
  if (err == cudaSuccess) rc = launch_selftest_xd(n, seed, bad, 4 * sms, reinterpret_cast<stream_t>(c->stream));
  if (err == cudaSuccess && rc == CF_OK) err = cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, c->stream);
  if (err == cudaSuccess && rc == CF_OK) err = cudaStreamSynchronize(c->stream);
  cudaFree(bad);
  if (err != cudaSuccess) return cuda_fail(c, err, "cf_selftest_xd");
  if (rc != CF_OK) return fail(c, rc, "cf_selftest_xd launch failed");
  *mismatches = (int64_t)h;
  return CF_OK;
}

int cf_get_tuning(cf_ctx* ctx, int32_t* int_compare, int32_t* int_mul_warps) {
  if (!ctx) return CF_EINVAL;
  if (int_compare) *int_compare = ctx->xd_cmp;
  if (int_mul_warps) *int_mul_warps = ctx->xd_mul_mask;
  return CF_OK;
}

int cf_set_launch_shape(cf_ctx* ctx, int32_t edge_block, int32_t edges_per_thread, int32_t cell_block) {
  if (!ctx) return CF_EINVAL;
  if ((edge_block != 64 && edge_block != 128 && edge_block != 256) || (edges_per_thread != 1 && edges_per_thread != 2) ||
      (cell_block != 128 && cell_block != 256))
    return fail(ctx, CF_EINVAL, "launch shape: edge_block 64, 128 or 256, edges_per_thread 1 or 2, cell_block 128 or 256");
  if (ctx->eblock != edge_block || ctx->ept != edges_per_thread || ctx->cblock != cell_block) {
    ctx->eblock = edge_block;
    ctx->ept = edges_per_thread;
    ctx->cblock = cell_block;
    if (ctx->graph2) {   /* the captured steps hold the old launch configuration */
      CF_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      cudaGraphExecDestroy(ctx->graph2);
      ctx->graph2 = nullptr;
    }
  }
  return CF_OK;
}

int cf_get_launch_shape(cf_ctx* ctx, int32_t* edge_block, int32_t* edges_per_thread, int32_t* cell_block) {
  if (!ctx) return CF_EINVAL;
  if (edge_block) *edge_block = ctx->eblock;
  if (edges_per_thread) *edges_per_thread = ctx->ept;
  if (cell_block) *cell_block = ctx->cblock;
  return CF_OK;
}

int cf_autotune(cf_ctx* ctx, int32_t steps_per_trial, int32_t* int_compare, int32_t* int_mul_warps, double* ms_per_step) {
  if (!ctx) return CF_EINVAL;
  cf_ctx* c = ctx;
  if (steps_per_trial < 2) return fail(c, CF_EINVAL, "steps_per_trial < 2");
  CF_CUDA(c, cudaSetDevice(c->device));
  int rc;
  if ((rc = read_states(c))) return rc;
  for (size_t i = 0; i < c->mem.size(); ++i)
    if (c->host_state[i].status) return fail(c, CF_ESTATE, "cf_autotune needs every member set and running");
  /* the trials step the context's own state; it is restored after each one (both buffers,
   * the member records and the launch count), so tuning leaves the simulation unchanged */
  const size_t np = (size_t)c->n_pad, nm = c->mem.size();
  double4* saved = nullptr;
  CF_CUDA(c, cudaMalloc((void**)&saved, 2 * np * sizeof(double4)));
  std::vector<MemberState> ms(c->host_state, c->host_state + nm);
  const int64_t launched0 = c->launched;
  const int32_t cmp0 = c->xd_cmp, mul0 = c->xd_mul_mask, eb0 = c->eblock, ept0 = c->ept, cb0 = c->cblock;
  auto restore = [&]() -> int {
    CF_CUDA(c, cudaMemcpyAsync(c->U[0], saved, np * sizeof(double4), cudaMemcpyDeviceToDevice, c->stream));
    CF_CUDA(c, cudaMemcpyAsync(c->U[1], saved + np, np * sizeof(double4), cudaMemcpyDeviceToDevice, c->stream));
    CF_CUDA(c, cudaMemcpyAsync(c->mst, ms.data(), nm * sizeof(MemberState), cudaMemcpyHostToDevice, c->stream));
    CF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->launched = launched0;
    return CF_OK;
  };
  cudaError_t e = cudaMemcpyAsync(saved, c->U[0], np * sizeof(double4), cudaMemcpyDeviceToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(saved + np, c->U[1], np * sizeof(double4), cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) {
    cudaFree(saved);
    return cuda_fail(c, e, "cudaMemcpyAsync");
  }
  /* one trial: warm-up (and graph build), steps_per_trial timed steps, the state restored */
  auto trial = [&](double& per) -> int {
    int r;
    if ((r = step_impl(c, 2, nullptr))) return r;
    CF_CUDA(c, cudaEventRecord(c->ev[0], c->stream));
    if ((r = step_impl(c, steps_per_trial, nullptr))) return r;
    CF_CUDA(c, cudaEventRecord(c->ev[1], c->stream));
    CF_CUDA(c, cudaEventSynchronize(c->ev[1]));
    float t = 0.f;
    cudaEventElapsedTime(&t, c->ev[0], c->ev[1]);
    if ((r = restore())) return r;
    per = t / steps_per_trial;
    return CF_OK;
  };
  /* 1. how the FP64 work is shared with the integer pipes, at the current launch shape:
   * all on the FP64 pipe; comparisons on the integer pipes; comparisons and the arithmetic of
   * all edge warps, of half of them, of three of four, each without and with the elements, and
   * of the elements alone */
  const int32_t cand[8][2] = {{0, 0}, {1, 0}, {1, 0xf}, {1, 0x5}, {1, 0x1f}, {1, 0x15}, {1, 0x17}, {1, 0x10}};
  double best = 1e300;
  int32_t bc = cmp0, bm = mul0, beb = eb0, bept = ept0, bcb = cb0;
  rc = CF_OK;
  for (const auto& k : cand) {
    double per = 0.0;
    if ((rc = cf_set_tuning(c, k[0], k[1])) || (rc = trial(per))) break;
    if (per < best) {
      best = per;
      bc = k[0];
      bm = k[1];
    }
  }
  /* 2. the edge kernel's launch shape (threads per block, edges per thread), then 3. the element
   * kernel's block, with the setting of 1 */
  if (rc == CF_OK) rc = cf_set_tuning(c, bc, bm);
  const int32_t eshape[6][2] = {{128, 1}, {64, 1}, {256, 1}, {128, 2}, {64, 2}, {256, 2}};
  for (int i = 0; rc == CF_OK && i < 6; ++i) {
    double per = 0.0;
    if ((rc = cf_set_launch_shape(c, eshape[i][0], eshape[i][1], bcb)) || (rc = trial(per))) break;
    if (per < best) {
      best = per;
      beb = eshape[i][0];
      bept = eshape[i][1];
    }
  }
  for (int cb : {256, 128}) {
    if (rc != CF_OK) break;
    double per = 0.0;
    if ((rc = cf_set_launch_shape(c, beb, bept, cb)) || (rc = trial(per))) break;
    if (per < best) {
      best = per;
      bcb = cb;
    }
  }
  cudaFree(saved);
  if (rc != CF_OK) {
    cf_set_tuning(c, cmp0, mul0);
    cf_set_launch_shape(c, eb0, ept0, cb0);
    restore();
    return rc;
  }
  if ((rc = cf_set_tuning(c, bc, bm)) || (rc = cf_set_launch_shape(c, beb, bept, bcb))) return rc;
  if (int_compare) *int_compare = bc;
  if (int_mul_warps) *int_mul_warps = bm;
  if (ms_per_step) *ms_per_step = best;
  return CF_OK;
}

int cf_autotune_order(const cf_mesh* mesh, const cf_params* params, const double* hu3, int32_t steps_per_trial,
                      int32_t* reorder, double* ms_per_step) {
  if (!mesh || !params || !hu3) return CF_EINVAL;
  /* the element orders a context can be created with: Hilbert, Morton, the caller's; each timed
   * with the rest of its tuning (cf_autotune) on the caller's state */
  double best = 1e300;
  int32_t br = -1;
  for (int32_t r : {1, 2, 0}) {
    cf_params q = *params;
    q.reorder = r;
    cf_ctx* c = nullptr;
    int rc = cf_create(mesh, &q, &c);
    if (rc == CF_OK) rc = cf_set_state(c, hu3, 0.0);
    double per = 0.0;
    if (rc == CF_OK) rc = cf_autotune(c, steps_per_trial, nullptr, nullptr, &per);
    if (rc != CF_OK) {
      if (c) g_create_error = c->err;
      cf_destroy(c);
      return rc;
    }
    cf_destroy(c);
    if (per < best) {
      best = per;
      br = r;
    }
  }
  if (reorder) *reorder = br;
  if (ms_per_step) *ms_per_step = best;
  return CF_OK;
}

/* ---- pieces of a decomposed mesh: halo exchange and the global dt ------------------------- */

namespace {

int elements_prep(cf_ctx* c, int32_t member, const int32_t* ids, int32_t n, const void* vals) {
  int rc = member_ok(c, member);
  if (rc) return rc;
  const Member& M = c->mem[member];
  if (n < 0 || n > M.n || (n > 0 && (!ids || !vals))) return fail(c, CF_EINVAL, "bad element list");
  for (int32_t i = 0; i < n; ++i)
    if (ids[i] < 0 || ids[i] >= M.n) return fail(c, CF_EINVAL, "element id out of range");
  CF_CUDA(c, cudaSetDevice(c->device));
  if (!c->ids && (rc = dalloc(c, &c->ids, (size_t)c->max_n))) return rc;
  if ((rc = read_states(c))) return rc;
  if (c->host_state[member].status & STATUS_NO_STATE) return fail(c, CF_ESTATE, "no state set");
  CF_CUDA(c, cudaMemcpyAsync(c->ids, ids, (size_t)n * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
  return CF_OK;
}

}  // namespace

int cf_get_elements(cf_ctx* ctx, int32_t member, const int32_t* ids, int32_t n, double* hu3_out) {
  if (!ctx) return CF_EINVAL;
  cf_ctx* c = ctx;
  int rc = elements_prep(c, member, ids, n, hu3_out);
  if (rc || n == 0) return rc;
  const Member& M = c->mem[member];
  const MemberState& s = c->host_state[member];
  const int cur = (int)((s.base + s.nstep) & 1);
  rc = launch_gather_ids(c->U[cur] + M.cell_off, c->iperm + M.cell_off, c->ids, c->staging, n,
                         reinterpret_cast<stream_t>(c->stream));
  if (rc) return fail(c, rc, "gather launch failed");
  CF_CUDA(c, cudaMemcpyAsync(hu3_out, c->staging, 3 * (size_t)n * sizeof(double), cudaMemcpyDefault, c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_set_elements(cf_ctx* ctx, int32_t member, const int32_t* ids, int32_t n, const double* hu3) {
  if (!ctx) return CF_EINVAL;
  cf_ctx* c = ctx;
  int rc = elements_prep(c, member, ids, n, hu3);
  if (rc) return rc;
  const Member& M = c->mem[member];
  MemberState s = c->host_state[member];
  const int cur = (int)((s.base + s.nstep) & 1);
  const stream_t st = reinterpret_cast<stream_t>(c->stream);
  if (n > 0) {
    CF_CUDA(c, cudaMemcpyAsync(c->staging, hu3, 3 * (size_t)n * sizeof(double), cudaMemcpyDefault, c->stream));
    if ((rc = launch_scatter_ids(c->U[cur] + M.cell_off, c->iperm + M.cell_off, c->ids, c->staging, n, st)))
      return fail(c, rc, "scatter launch failed");
  }
  /* the next dt is the CFL of the state as it now is (as cf_set_state computes it) */
  s.dt[cur] = M.dev.dt_reset;
  c->host_state[member] = s;
  CF_CUDA(c, cudaMemcpyAsync(c->mst + member, &c->host_state[member], sizeof(MemberState), cudaMemcpyHostToDevice,
                             c->stream));
  if ((rc = launch_cfl(c->U[cur], c->cstat, c->ctile_mem, M.ctile_begin, M.ctile_end - M.ctile_begin, c->mdev, c->mst,
                       cur, st)))
    return fail(c, rc, "cfl launch failed");
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_set_dt(cf_ctx* ctx, int32_t member, double dt) {
  if (!ctx) return CF_EINVAL;
  cf_ctx* c = ctx;
  int rc = member_ok(c, member);
  if (rc) return rc;
  if (!(dt > 0.0)) return fail(c, CF_EINVAL, "dt must be positive");
  CF_CUDA(c, cudaSetDevice(c->device));
  if ((rc = read_states(c))) return rc;
  MemberState& s = c->host_state[member];
  if (s.status & STATUS_NO_STATE) return fail(c, CF_ESTATE, "no state set");
  s.dt[(s.base + s.nstep) & 1] = dt;
  CF_CUDA(c, cudaMemcpyAsync(c->mst + member, &s, sizeof(MemberState), cudaMemcpyHostToDevice, c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_default_params(cf_params* p) {
  if (!p) return CF_EINVAL;
  std::memset(p, 0, sizeof(*p));
  p->gp = 9.81;
  p->tolisec = 1e-5;
  p->cfl = 0.9;
  p->tol = (double)1e-6f;
  p->iflux = 1;
  p->ilimiteur = 1;
  p->friction = 0;
  p->fricimplic = 1;
  p->inlet = 2;
  p->outlet = 1;
  p->flux_mode = 0;
  p->reorder = 1;
  p->tol_reg_perm = 0.0;
  p->steady_count = 1000;
  return CF_OK;
}

int cf_create(const cf_mesh* mesh, const cf_params* params, cf_ctx** out) {
  return abi_guard(nullptr, [&] { return create_impl(mesh, params, 1, out); });
}

int cf_create_batch(const cf_mesh* meshes, const cf_params* params, int32_t nmembers, cf_ctx** out) {
  return abi_guard(nullptr, [&] { return create_impl(meshes, params, nmembers, out); });
}

void cf_destroy(cf_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_all(c);
  delete c;
}

int cf_get_members(cf_ctx* c) { return c ? (int)c->mem.size() : CF_EINVAL; }

int cf_set_state(cf_ctx* c, const double* hu3, double t0) {
  return set_state_host(c, 0, hu3, t0, cudaMemcpyHostToDevice);
}

int cf_set_state_device(cf_ctx* c, const double* d_hu3, double t0) {
  return set_state_host(c, 0, d_hu3, t0, cudaMemcpyDeviceToDevice);
}

int cf_member_set_state(cf_ctx* c, int32_t member, const double* hu3, double t0) {
  return set_state_host(c, member, hu3, t0, cudaMemcpyHostToDevice);
}

int cf_set_initial_condition(cf_ctx* c, const cf_ic* ic, double t0) {
  return abi_guard(c, [&] { return initial_condition(c, 0, ic, t0); });
}

int cf_member_set_initial_condition(cf_ctx* c, int32_t member, const cf_ic* ic, double t0) {
  return abi_guard(c, [&] { return initial_condition(c, member, ic, t0); });
}

int cf_step(cf_ctx* c, int32_t nsteps, cf_step_info* info) { return step_impl(c, nsteps, info); }

int cf_advance(cf_ctx* c, const double* hu3_in, double t0, int32_t nsteps, double* hu3_out, cf_step_info* info) {
  if (!c) return CF_EINVAL;
  if (c->mem.size() != 1) return fail(c, CF_EINVAL, "cf_advance: a context with one member");
  if (!hu3_in || !hu3_out) return fail(c, CF_EINVAL, "null state");
  if (nsteps < 0) return fail(c, CF_EINVAL, "nsteps < 0");
  CF_CUDA(c, cudaSetDevice(c->device));
  const Member& M = c->mem[0];
  const size_t bytes = 3 * (size_t)M.n * sizeof(double);
  const stream_t st = reinterpret_cast<stream_t>(c->stream);
  /* one stream-ordered sequence, one wait: state in, initial dt, the steps, the current state out
   * (its buffer chosen on the device, so a member that stopped early returns where it stopped) */
  const double* vin = static_cast<const double*>(device_view(c, hu3_in));
  double* vout = static_cast<double*>(device_view(c, hu3_out));
  if (!vin) CF_CUDA(c, cudaMemcpyAsync(c->staging, hu3_in, bytes, cudaMemcpyDefault, c->stream));
  int rc = enqueue_set_state(c, 0, t0, vin);
  if (rc == CF_OK) rc = enqueue_steps(c, nsteps);
  if (rc != CF_OK) {
    cudaStreamSynchronize(c->stream);
    return rc;
  }
  /* the store kernel writes the caller's buffer in its own order with coalesced stores (a step's
   * element kernel writing it through the permutation took 0.33 instead of 0.24 ms per 1M step,
   * its scattered 8-byte stores crossing the CPU link) */
  if (vout)
    rc = launch_store_ref(c->U[0] + M.cell_off, c->U[1] + M.cell_off, c->mst, 0, c->iperm + M.cell_off, vout, M.n, st);
  else
    rc = launch_gather_current(c->U[0] + M.cell_off, c->U[1] + M.cell_off, c->mst, 0, c->iperm + M.cell_off,
                               c->staging, M.n, st);
  if (rc != CF_OK) {
    cudaStreamSynchronize(c->stream);
    return fail(c, rc, "gather launch failed");
  }
  if (!vout) CF_CUDA(c, cudaMemcpyAsync(hu3_out, c->staging, bytes, cudaMemcpyDefault, c->stream));
  return finish_steps(c, info);
}

int cf_get_state(cf_ctx* c, double* hu3) { return get_state_member(c, 0, hu3, cudaMemcpyDeviceToHost); }

int cf_get_state_device(cf_ctx* c, double* d_hu3) { return get_state_member(c, 0, d_hu3, cudaMemcpyDeviceToDevice); }

int cf_member_get_state(cf_ctx* c, int32_t member, double* hu3) {
  return get_state_member(c, member, hu3, cudaMemcpyDeviceToHost);
}

int cf_get_info(cf_ctx* c, cf_step_info* info) { return cf_member_get_info(c, 0, info); }

int cf_member_get_info(cf_ctx* c, int32_t member, cf_step_info* info) {
  int rc = member_ok(c, member);
  if (rc) return rc;
  if (!info) return fail(c, CF_EINVAL, "null argument");
  CF_CUDA(c, cudaSetDevice(c->device));
  if ((rc = read_states(c))) return rc;
  fill_info(c->host_state[member], info);
  return CF_OK;
}

int cf_get_mesh_tables(cf_ctx* c, int32_t* boundary, double* area, double* zm, double* cotemin) {
  return cf_member_get_mesh_tables(c, 0, boundary, area, zm, cotemin);
}

int cf_member_get_mesh_tables(cf_ctx* c, int32_t member, int32_t* boundary, double* area, double* zm, double* cotemin) {
  int rc = member_ok(c, member);
  if (rc) return rc;
  const Prep& P = c->mem[member].prep;
  const size_t n = (size_t)P.nelt;
  if (boundary) std::memcpy(boundary, P.bnd.data(), n * 6 * sizeof(int32_t));
  if (area) std::memcpy(area, P.area.data(), n * sizeof(double));
  if (zm) std::memcpy(zm, P.zm.data(), n * sizeof(double));
  if (cotemin) std::memcpy(cotemin, P.cotemin.data(), n * sizeof(double));
  return CF_OK;
}

static int mesh_tables_impl(const cf_mesh* mesh, const cf_params* params, int32_t* boundary, double* area,
                            double* zm, double* cotemin);

int cf_mesh_tables(const cf_mesh* mesh, const cf_params* params, int32_t* boundary, double* area, double* zm,
                   double* cotemin) {
  return abi_guard(nullptr, [&] { return mesh_tables_impl(mesh, params, boundary, area, zm, cotemin); });
}

static int mesh_tables_impl(const cf_mesh* mesh, const cf_params* params, int32_t* boundary, double* area, double* zm,
                            double* cotemin) {
  Prep P;
  std::string err;
  int rc = prepare_mesh(mesh, params, P, err);
  if (rc != CF_OK) return fail(nullptr, rc, err);
  const size_t n = (size_t)P.nelt;
  if (boundary) std::memcpy(boundary, P.bnd.data(), n * 6 * sizeof(int32_t));
  if (area) std::memcpy(area, P.area.data(), n * sizeof(double));
  if (zm) std::memcpy(zm, P.zm.data(), n * sizeof(double));
  if (cotemin) std::memcpy(cotemin, P.cotemin.data(), n * sizeof(double));
  return CF_OK;
}

int cf_get_sizes(cf_ctx* c, int64_t* nelt, int64_t* nedge) {
  if (!c) return CF_EINVAL;
  int64_t n = 0, e = 0;
  for (const auto& M : c->mem) {
    n += M.n;
    e += M.ne;
  }
  if (nelt) *nelt = n;
  if (nedge) *nedge = e;
  return CF_OK;
}

void* cf_get_stream(cf_ctx* c) { return c ? (void*)c->stream : nullptr; }

const char* cf_last_error(const cf_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

/* ---- a part of a decomposed mesh ----------------------------------------------------------- */

namespace {

int part_ok(cf_ctx* c) {
  if (!c) return CF_EINVAL;
  if (!c->is_part) return fail(c, CF_EINVAL, "not a part context (cf_create_part)");
  return CF_OK;
}

/* terms (device) -> dst (host or device), count doubles, waiting for them */
int part_terms_out(cf_ctx* c, double* dst, size_t count) {
  if (count) CF_CUDA(c, cudaMemcpyAsync(dst, c->terms, count * sizeof(double), cudaMemcpyDefault, c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

}  // namespace

int cf_create_part(const cf_mesh* mesh, const cf_params* params, const int32_t* elem_class, cf_ctx** out) {
  if (!elem_class) return fail(nullptr, CF_EINVAL, "elem_class is NULL");
  return abi_guard(nullptr, [&] { return create_impl(mesh, params, 1, out, elem_class); });
}

int cf_part_sizes(cf_ctx* c, int32_t* n_send, int32_t* n_own, int32_t* inlet_entries, int32_t* boundary_edges) {
  int rc = part_ok(c);
  if (rc) return rc;
  const Member& M = c->mem[0];
  if (n_send) *n_send = c->n_send;
  if (n_own) *n_own = c->n_own;
  if (inlet_entries) *inlet_entries = M.dev.inl_count;
  if (boundary_edges) *boundary_edges = M.dev.bq_count;
  return CF_OK;
}

int cf_part_set_exchange(cf_ctx* c, const int32_t* send_ids, int32_t nsend, const int32_t* recv_ids, int32_t nrecv) {
  int rc = part_ok(c);
  if (rc) return rc;
  if (nsend < 0 || nrecv < 0 || (nsend && !send_ids) || (nrecv && !recv_ids))
    return fail(c, CF_EINVAL, "exchange lists NULL or negative counts");
  const Prep& P = c->mem[0].prep;
  std::vector<int32_t> s(nsend), r(nrecv);
  for (int32_t i = 0; i < nsend; ++i) {
    if (send_ids[i] < 0 || send_ids[i] >= P.nelt || P.iperm[send_ids[i]] >= c->n_send)
      return fail(c, CF_EINVAL, "send element " + std::to_string(send_ids[i]) + " is not a send element of the part");
    s[i] = P.iperm[send_ids[i]];
  }
  for (int32_t i = 0; i < nrecv; ++i) {
    if (recv_ids[i] < 0 || recv_ids[i] >= P.nelt || P.iperm[recv_ids[i]] < c->n_own)
      return fail(c, CF_EINVAL, "receive element " + std::to_string(recv_ids[i]) + " is not a halo element of the part");
    r[i] = P.iperm[recv_ids[i]];
  }
  CF_CUDA(c, cudaSetDevice(c->device));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  if (c->xsend) cudaFree(c->xsend);
  if (c->xrecv) cudaFree(c->xrecv);
  c->xsend = c->xrecv = nullptr;
  c->nxsend = c->nxrecv = 0;
  if ((rc = dalloc(c, &c->xsend, s.size())) || (rc = dalloc(c, &c->xrecv, r.size())) ||
      (rc = put(c, c->xsend, s.data(), s.size())) || (rc = put(c, c->xrecv, r.data(), r.size())))
    return rc;
  c->nxsend = nsend;
  c->nxrecv = nrecv;
  return CF_OK;
}

int cf_part_step_begin(cf_ctx* c, double* send_buf) {
  int rc = part_ok(c);
  if (rc) return rc;
  CF_CUDA(c, cudaSetDevice(c->device));
  double* v = static_cast<double*>(device_view(c, send_buf));
  if (c->nxsend && !v) return fail(c, CF_EINVAL, "the send buffer must be device memory or pinned host memory");
  if (c->any_phys_inflow && !c->external_sums)
    return fail(c, CF_ESTATE, "a phys_inflow part needs the whole mesh's inlet sums (cf_part_set_inlet_sums)");
  const stream_t st = reinterpret_cast<stream_t>(c->stream);
  StepArgs a = step_args(c, (int)(c->launched & 1));
  a.steady = 0;        /* the steady-state test runs on the whole mesh's discharges (cf_part_apply_discharges) */
  a.phys_inflow = 0;   /* the inlet sums are the whole mesh's (cf_part_set_inlet_sums) */
  /* the send elements first, their states out to the other parts, then the interior elements */
  if ((rc = launch_part_phase(a, 1, c->elist1, c->nel1, 0, c->n_send, st))) return fail(c, rc, "step launch failed");
  if ((rc = launch_pack(a.Uout, c->xsend, c->nxsend, v, st))) return fail(c, rc, "pack launch failed");
  CF_CUDA(c, cudaEventRecord(c->ev_pack, c->stream));
  if ((rc = launch_part_phase(a, 2, c->elist2, c->nel2, c->n_send, c->n_own, st))) return fail(c, rc, "step launch failed");
  c->launched += 1;
  return CF_OK;
}

int cf_part_wait_send(cf_ctx* c) {
  int rc = part_ok(c);
  if (rc) return rc;
  CF_CUDA(c, cudaEventSynchronize(c->ev_pack));
  return CF_OK;
}

int cf_part_step_end(cf_ctx* c, const double* recv_buf, cf_step_info* info) {
  int rc = part_ok(c);
  if (rc) return rc;
  CF_CUDA(c, cudaSetDevice(c->device));
  const double* v = static_cast<const double*>(device_view(c, recv_buf));
  if (c->nxrecv && !v) return fail(c, CF_EINVAL, "the receive buffer must be device memory or pinned host memory");
  if ((rc = launch_unpack(c->U[c->launched & 1], c->xrecv, c->nxrecv, v, reinterpret_cast<stream_t>(c->stream))))
    return fail(c, rc, "unpack launch failed");
  return finish_steps(c, info);
}

int cf_part_inlet_terms(cf_ctx* c, double* out) {
  int rc = part_ok(c);
  if (rc) return rc;
  if (!out) return fail(c, CF_EINVAL, "out is NULL");
  CF_CUDA(c, cudaSetDevice(c->device));
  const MemberDev& D = c->mem[0].dev;
  if (!c->any_phys_inflow) return CF_OK;
  if ((rc = launch_inlet_terms(step_args(c, 0), c->U[c->launched & 1], D.inl_count, c->terms,
                               reinterpret_cast<stream_t>(c->stream))))
    return fail(c, rc, "terms launch failed");
  return part_terms_out(c, out, (size_t)D.inl_count * D.nin);
}

int cf_part_set_inlet_sums(cf_ctx* c, const double* surf) {
  int rc = part_ok(c);
  if (rc) return rc;
  if (!surf) return fail(c, CF_EINVAL, "surf is NULL");
  CF_CUDA(c, cudaSetDevice(c->device));
  const int32_t nin = c->mem[0].dev.nin;
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  char* dst = reinterpret_cast<char*>(c->mst) + offsetof(MemberState, surf);
  if (nin > 0) CF_CUDA(c, cudaMemcpy(dst, surf, (size_t)nin * sizeof(double), cudaMemcpyDefault));
  c->external_sums = true;
  return CF_OK;
}

int cf_part_discharge_terms(cf_ctx* c, double* out) {
  int rc = part_ok(c);
  if (rc) return rc;
  if (!out) return fail(c, CF_EINVAL, "out is NULL");
  CF_CUDA(c, cudaSetDevice(c->device));
  const MemberDev& D = c->mem[0].dev;
  if ((rc = launch_bq_terms(c->slots, c->bq, c->mdev, D.bq_count, c->terms, reinterpret_cast<stream_t>(c->stream))))
    return fail(c, rc, "terms launch failed");
  return part_terms_out(c, out, (size_t)D.bq_count);
}

int cf_part_apply_discharges(cf_ctx* c, double q_in, double q_out) {
  int rc = part_ok(c);
  if (rc) return rc;
  CF_CUDA(c, cudaSetDevice(c->device));
  if ((rc = launch_steady_apply(c->mdev, c->mst, q_in, q_out, reinterpret_cast<stream_t>(c->stream))))
    return fail(c, rc, "steady launch failed");
  return finish_steps(c, nullptr);
}

int cf_set_direct_io(cf_ctx* c, int32_t enable) {
  if (!c) return CF_EINVAL;
  c->direct_io = enable != 0;
  return CF_OK;
}

int cf_set_timing(cf_ctx* c, int32_t enable) {
  if (!c) return CF_EINVAL;
  c->timing = enable != 0;
  return CF_OK;
}

int cf_get_timing(cf_ctx* c, double* flux_ms, double* update_ms, int64_t* launches) {
  if (!c) return CF_EINVAL;
  if (flux_ms) *flux_ms = c->flux_ms;
  if (update_ms) *update_ms = c->update_ms;
  if (launches) *launches = c->launches;
  return CF_OK;
}

}  // extern "C"
