/*
 * cf_api.cpp -- the C ABI of include/cuteflow_gb300.h.
 *
 * A context holds one simulation (one "member" of the flat cell/edge space the kernels work
 * on), its device tables, the ping-pong state buffers and one CUDA stream.  Stepping never
 * returns to the host between steps: the next dt is produced on the device by the element
 * kernel and read by the next edge kernel.  The host only reads the small per-member state
 * record at the end of a cf_step call.  Runs of steps are replayed from a captured CUDA
 * graph of two steps (even and odd parity).
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "cf_internal.h"

using namespace cf;

struct cf_ctx {
  int device = 0;
  cf_params params{};
  Prep prep;
  int32_t n = 0, n_pad = 0, ne = 0, ne_pad = 0, n_etiles = 0, n_ctiles = 0;
  cudaStream_t stream = nullptr;
  /* device memory */
  double4* U[2] = {nullptr, nullptr};
  int4* cslot = nullptr;
  double4* cstat = nullptr;
  double* zcell = nullptr;
  int32_t* perm = nullptr;   /* new -> old */
  int32_t* iperm = nullptr;  /* old -> new */
  int2* ecell = nullptr;
  double4* egeo = nullptr;
  int32_t* ebid = nullptr;
  int4* eupw = nullptr;
  double4* ewts = nullptr;
  double2* edk = nullptr;
  Slot* slots = nullptr;
  int32_t* etile_mem = nullptr;
  int32_t* ctile_mem = nullptr;
  MemberDev* mdev = nullptr;
  MemberState* mst = nullptr;
  double* staging = nullptr;      /* 3*n doubles, reference order */
  MemberState* host_state = nullptr; /* pinned */
  MemberDev mhost{};
  /* stepping */
  bool have_state = false;
  int64_t launched = 0;           /* steps launched since the state was set */
  cudaGraphExec_t graph2 = nullptr; /* two steps: parity 0 then 1 */
  bool use_graph = true;
  /* timing */
  bool timing = false;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
  double flux_ms = 0.0, update_ms = 0.0;
  int64_t launches = 0;
  std::string err;
};

namespace {

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

#define CF_CUDA(c, call)                                     \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cuda_fail((c), e_, #call); \
  } while (0)

template <class T>
int upload(cf_ctx* c, T** dst, const std::vector<T>& src, size_t count_pad) {
  size_t bytes = std::max<size_t>(1, count_pad) * sizeof(T);
  CF_CUDA(c, cudaMalloc((void**)dst, bytes));
  CF_CUDA(c, cudaMemset(*dst, 0, bytes));
  if (!src.empty()) CF_CUDA(c, cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return CF_OK;
}

StepArgs step_args(const cf_ctx* c, int parity) {
  StepArgs a{};
  a.Uin = c->U[parity];
  a.Uout = c->U[1 - parity];
  a.cslot = c->cslot;
  a.cstat = c->cstat;
  a.ecell = c->ecell;
  a.egeo = c->egeo;
  a.ebid = c->ebid;
  a.eupw = c->eupw;
  a.ewts = c->ewts;
  a.edk = c->edk;
  a.slots = c->slots;
  a.etile_mem = c->etile_mem;
  a.ctile_mem = c->ctile_mem;
  a.mdev = c->mdev;
  a.mst = c->mst;
  a.n_etiles = c->n_etiles;
  a.n_ctiles = c->n_ctiles;
  a.parity = parity;
  a.iflux = c->params.iflux;
  a.ilimiteur = c->params.ilimiteur;
  a.flux_mode = c->params.flux_mode;
  return a;
}

void free_all(cf_ctx* c) {
  if (c->graph2) cudaGraphExecDestroy(c->graph2);
  void* ptrs[] = {c->U[0], c->U[1], c->cslot, c->cstat, c->zcell, c->perm, c->iperm, c->ecell, c->egeo,
                  c->ebid, c->eupw, c->ewts, c->edk, c->slots, c->etile_mem, c->ctile_mem, c->mdev,
                  c->mst, c->staging};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (c->host_state) cudaFreeHost(c->host_state);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  if (c->stream) cudaStreamDestroy(c->stream);
}

int read_state(cf_ctx* c) {
  CF_CUDA(c, cudaMemcpyAsync(c->host_state, c->mst, sizeof(MemberState), cudaMemcpyDeviceToHost, c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

void fill_info(const cf_ctx* c, cf_step_info* info) {
  const MemberState& s = *c->host_state;
  info->steps = s.nstep;
  info->t = s.t[s.nstep & 1];
  info->dt_next = s.dt[s.nstep & 1];
  info->dt_last = s.nstep > 0 ? s.dt[(s.nstep - 1) & 1] : 0.0;
  info->q_in = s.q_in;
  info->q_out = s.q_out;
  info->status = s.status;
  info->pad_ = 0;
}

int status_code(uint32_t st) {
  if (st & CF_STATUS_NONFINITE) return CF_ENONFINITE;
  if (st & CF_STATUS_DT_RANGE) return CF_EDT;
  return CF_OK;
}

/* one step with explicit parity (also used while capturing the graph) */
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
  if (rc1 != CF_OK) { if (g) cudaGraphDestroy(g); return rc1; }
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&c->graph2, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaGraphInstantiate");
  return CF_OK;
}

}  // namespace

extern "C" {

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
  return CF_OK;
}

int cf_create(const cf_mesh* mesh, const cf_params* params, cf_ctx** out) {
  if (!out) return fail(nullptr, CF_EINVAL, "out is NULL");
  *out = nullptr;
  if (!mesh || !params) return fail(nullptr, CF_EINVAL, "mesh or params is NULL");
  if (params->iflux < 1 || params->iflux > 3)
    return fail(nullptr, CF_ENOTSUP, "iflux must be 1 (HLLC), 2 (HLLC, star states) or 3 (WAF)");
  if (params->inlet == 3) return fail(nullptr, CF_ENOTSUP, "inlet 'phys_inflow' is not supported");
  if (params->inlet < 1 || params->inlet > 3 || params->outlet < 1 || params->outlet > 2)
    return fail(nullptr, CF_EINVAL, "inlet must be 1..3 and outlet 1..2");
  if (params->ilimiteur < 0 || params->ilimiteur > 4) return fail(nullptr, CF_EINVAL, "ilimiteur must be 0..4");
  if (params->flux_mode < 0 || params->flux_mode > 1) return fail(nullptr, CF_EINVAL, "flux_mode must be 0 or 1");
  if (!(params->gp > 0.0) || !(params->cfl > 0.0) || !(params->tolisec >= 0.0))
    return fail(nullptr, CF_EINVAL, "gp and cfl must be positive, tolisec non-negative");
  cf_ctx* c = new (std::nothrow) cf_ctx();
  if (!c) return fail(nullptr, CF_ENOMEM, "host allocation failed");
  c->params = *params;
  std::string err;
  int rc = prepare_mesh(mesh, params, c->prep, err);
  if (rc != CF_OK) { delete c; return fail(nullptr, rc, err); }
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
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaGetDevice"));
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaStreamCreate"));
  for (auto& ev : c->ev) {
    e = cudaEventCreate(&ev);
    if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaEventCreate"));
  }
  const Prep& P = c->prep;
  c->n = P.nelt;
  c->ne = (int32_t)P.edges.size();
  c->n_ctiles = (c->n + TILE_C - 1) / TILE_C;
  c->n_etiles = (c->ne + TILE_E - 1) / TILE_E;
  c->n_pad = c->n_ctiles * TILE_C;
  c->ne_pad = c->n_etiles * TILE_E;
  if ((rc = upload(c, &c->cslot, P.cslot, c->n_pad)) || (rc = upload(c, &c->cstat, P.cstat, c->n_pad)) ||
      (rc = upload(c, &c->zcell, P.zcell, c->n_pad)) || (rc = upload(c, &c->perm, P.perm, c->n_pad)) ||
      (rc = upload(c, &c->iperm, P.iperm, c->n_pad)) || (rc = upload(c, &c->ecell, P.ecell, c->ne_pad)) ||
      (rc = upload(c, &c->egeo, P.egeo, c->ne_pad)) || (rc = upload(c, &c->ebid, P.ebid, c->ne_pad)))
    return done(rc);
  if (params->iflux >= 3) {
    if ((rc = upload(c, &c->eupw, P.eupw, c->ne_pad)) || (rc = upload(c, &c->ewts, P.ewts, c->ne_pad)) ||
        (rc = upload(c, &c->edk, P.edk, c->ne_pad)))
      return done(rc);
  }
  std::vector<double4> none;
  if ((rc = upload(c, &c->U[0], none, c->n_pad)) || (rc = upload(c, &c->U[1], none, c->n_pad))) return done(rc);
  std::vector<Slot> noslot;
  if ((rc = upload(c, &c->slots, noslot, 2 * (size_t)c->ne_pad))) return done(rc);
  std::vector<int32_t> tm_e(c->n_etiles, 0), tm_c(c->n_ctiles, 0);
  if ((rc = upload(c, &c->etile_mem, tm_e, c->n_etiles)) || (rc = upload(c, &c->ctile_mem, tm_c, c->n_ctiles)))
    return done(rc);
  std::vector<double> none_d;
  if ((rc = upload(c, &c->staging, none_d, 3 * (size_t)c->n))) return done(rc);
  /* member constants */
  MemberDev& M = c->mhost;
  std::memset(&M, 0, sizeof(M));
  M.gp = params->gp;
  M.tolisec = params->tolisec;
  M.tol = params->tol;
  M.constant_dt = params->constant_dt;
  M.ramp_time = params->ramp_time;
  M.dt_reset = (c->n % 1024 != 0) ? 100000.0 : 1000000.0;
  for (int i = 0; i < CF_MAX_IO; ++i) {
    M.debit_end[i] = params->debitglob[i];
    M.debit_start[i] = params->debitglob_start[i];
    M.long_entree[i] = P.long_entree[i];
    M.h_sortie[i] = params->h_sortie[i];
  }
  M.inlet = params->inlet;
  M.outlet = params->outlet;
  M.friction = params->friction;
  M.fricimplic = params->fricimplic;
  M.is_dt_constant = params->is_dt_constant;
  M.cell_begin = 0;
  M.cell_end = c->n;
  M.edge_begin = 0;
  M.edge_end = c->ne;
  M.bedge_begin = P.n_interior;
  M.bedge_end = c->ne;
  std::vector<MemberDev> mv(1, M);
  if ((rc = upload(c, &c->mdev, mv, 1))) return done(rc);
  std::vector<MemberState> ms(1);
  std::memset(ms.data(), 0, sizeof(MemberState));
  if ((rc = upload(c, &c->mst, ms, 1))) return done(rc);
  e = cudaMallocHost((void**)&c->host_state, sizeof(MemberState));
  if (e != cudaSuccess) return done(cuda_fail(c, e, "cudaMallocHost"));
  std::memset(c->host_state, 0, sizeof(MemberState));
  return done(CF_OK);
}

void cf_destroy(cf_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  free_all(c);
  delete c;
}

static int set_state_common(cf_ctx* c, double t0) {
  MemberState s;
  std::memset(&s, 0, sizeof(s));
  s.dt[0] = c->mhost.dt_reset;
  s.t[0] = t0;
  *c->host_state = s;
  CF_CUDA(c, cudaMemcpyAsync(c->mst, c->host_state, sizeof(MemberState), cudaMemcpyHostToDevice, c->stream));
  int rc = launch_scatter_state(c->staging, c->perm, c->zcell, c->U[0], c->n, reinterpret_cast<stream_t>(c->stream));
  if (rc != CF_OK) return fail(c, rc, "state scatter launch failed");
  rc = launch_cfl(c->U[0], c->cstat, c->ctile_mem, c->n_ctiles, c->mdev, c->mst, 0, reinterpret_cast<stream_t>(c->stream));
  if (rc != CF_OK) return fail(c, rc, "cfl launch failed");
  /* the host record is reused below; wait for the copy and the kernels */
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_state = true;
  c->launched = 0;
  return CF_OK;
}

int cf_set_state(cf_ctx* c, const double* hu3, double t0) {
  if (!c || !hu3) return fail(c, CF_EINVAL, "null argument");
  CF_CUDA(c, cudaSetDevice(c->device));
  CF_CUDA(c, cudaMemcpyAsync(c->staging, hu3, 3 * (size_t)c->n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  return set_state_common(c, t0);
}

int cf_set_state_device(cf_ctx* c, const double* d_hu3, double t0) {
  if (!c || !d_hu3) return fail(c, CF_EINVAL, "null argument");
  CF_CUDA(c, cudaSetDevice(c->device));
  CF_CUDA(c, cudaMemcpyAsync(c->staging, d_hu3, 3 * (size_t)c->n * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
  return set_state_common(c, t0);
}

/* set_initial_condition, initial_condition.cuf:18-79, evaluated on the host (setup only). */
int cf_set_initial_condition(cf_ctx* c, const cf_ic* ic, double t0) {
  if (!c || !ic) return fail(c, CF_EINVAL, "null argument");
  const Prep& P = c->prep;
  std::vector<double> U(3 * (size_t)c->n, 0.0);
  const double tolisec = c->params.tolisec;
  for (int k = 0; k < c->n; ++k) {
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
  return cf_set_state(c, U.data(), t0);
}

int cf_step(cf_ctx* c, int32_t nsteps, cf_step_info* info) {
  if (!c) return CF_EINVAL;
  if (nsteps < 0) return fail(c, CF_EINVAL, "nsteps < 0");
  if (!c->have_state) return fail(c, CF_ESTATE, "cf_step before a state was set");
  CF_CUDA(c, cudaSetDevice(c->device));
  if (c->host_state->status) {
    if (info) fill_info(c, info);
    return fail(c, status_code(c->host_state->status), "the run is stopped (status latched on the device)");
  }
  int rc;
  const bool timed = c->timing;
  c->flux_ms = c->update_ms = 0.0;
  c->launches = 0;
  int32_t left = nsteps;
  if (timed) {
    /* per-step events: edge kernel [ev0, ev1), element kernel [ev1, ev2) */
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
  }
  c->launched += nsteps;
  rc = launch_discharge(c->slots, c->ecell, c->mdev, c->mst, 1, reinterpret_cast<stream_t>(c->stream));
  if (rc != CF_OK) return fail(c, rc, "discharge launch failed");
  if ((rc = read_state(c))) return rc;
  if (info) fill_info(c, info);
  rc = status_code(c->host_state->status);
  if (rc != CF_OK) return fail(c, rc, rc == CF_EDT ? "dt left the range (1e-12, 9999]" : "non-finite value in the state");
  return CF_OK;
}

static int gather_common(cf_ctx* c, double* dst, cudaMemcpyKind kind) {
  if (!c->have_state) return fail(c, CF_ESTATE, "no state set");
  int rc = read_state(c);
  if (rc) return rc;
  const int buf = (int)(c->host_state->nstep & 1);
  rc = launch_gather_state(c->U[buf], c->iperm, c->staging, c->n, reinterpret_cast<stream_t>(c->stream));
  if (rc != CF_OK) return fail(c, rc, "gather launch failed");
  CF_CUDA(c, cudaMemcpyAsync(dst, c->staging, 3 * (size_t)c->n * sizeof(double), kind, c->stream));
  CF_CUDA(c, cudaStreamSynchronize(c->stream));
  return CF_OK;
}

int cf_get_state(cf_ctx* c, double* hu3) {
  if (!c || !hu3) return fail(c, CF_EINVAL, "null argument");
  CF_CUDA(c, cudaSetDevice(c->device));
  return gather_common(c, hu3, cudaMemcpyDeviceToHost);
}

int cf_get_state_device(cf_ctx* c, double* d_hu3) {
  if (!c || !d_hu3) return fail(c, CF_EINVAL, "null argument");
  CF_CUDA(c, cudaSetDevice(c->device));
  return gather_common(c, d_hu3, cudaMemcpyDeviceToDevice);
}

int cf_get_info(cf_ctx* c, cf_step_info* info) {
  if (!c || !info) return fail(c, CF_EINVAL, "null argument");
  CF_CUDA(c, cudaSetDevice(c->device));
  int rc = read_state(c);
  if (rc) return rc;
  fill_info(c, info);
  return CF_OK;
}

int cf_get_mesh_tables(cf_ctx* c, int32_t* boundary, double* area, double* zm, double* cotemin) {
  if (!c) return CF_EINVAL;
  const Prep& P = c->prep;
  const size_t n = (size_t)P.nelt;
  if (boundary) std::memcpy(boundary, P.bnd.data(), n * 6 * sizeof(int32_t));
  if (area) std::memcpy(area, P.area.data(), n * sizeof(double));
  if (zm) std::memcpy(zm, P.zm.data(), n * sizeof(double));
  if (cotemin) std::memcpy(cotemin, P.cotemin.data(), n * sizeof(double));
  return CF_OK;
}

int cf_mesh_tables(const cf_mesh* mesh, const cf_params* params, int32_t* boundary, double* area,
                   double* zm, double* cotemin) {
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
  if (nelt) *nelt = c->n;
  if (nedge) *nedge = c->ne;
  return CF_OK;
}

void* cf_get_stream(cf_ctx* c) { return c ? (void*)c->stream : nullptr; }

const char* cf_last_error(const cf_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

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
