/*
 * cf_internal.h -- data layout shared by the host preprocessing (cf_mesh.cpp), the C ABI
 * (cf_api.cpp) and the sm_103a kernels (cf_kernels.cu).
 *
 * Device layout (all arrays in space-filling-curve order, see cf_mesh.cpp):
 *   cells  U[2]  : double4 {h, hu, hv, RN(1/h) (0 where h = 0)} per element, ping-pong (state n in
 *                  U[n & 1]); the bed elevations live in zcell and, per edge, in ez
 *          cslot : int4 {slot of local edge 0, 1, 2, -}   (local edges in the reference's order)
 *          cnbr  : int4 {element across local edge 0, 1, 2 (-1: boundary), 1 when all three edges
 *                  are interior with finite normals and lengths and the area passes area_ok,
 *                  else 0}
 *          cstat : double4 {area, Manning n, cfl*L_cfl, RN(1/area)}
 *   edges  ecell : int2 {A, B}; B >= 0 another element, B < 0 the boundary kind (-1/-2/-3)
 *          egeo  : double4 {nx, ny, len, d_AB}, normal pointing out of A, centroid distance
 *          ebid  : int32 inlet/outlet number of a boundary edge
 *          eupw  : int4 {A-side upwind 1, 2, B-side upwind 1, 2}          (second order only)
 *          ewts  : double4 {A distances d1, d2, B distances d1, d2}; d1 < 0: copy element 1
 *          edk   : double4 {d_mkvol, d_mkvoisin, RN(1/d_mkvol), RN(1/d_mkvoisin)}  (second order)
 *          einv  : double4 {RN(1/d_AB), RN(1/(d1+d2)) of A, of B, -}          (second order only)
 *   slots  Slot  : 48 bytes per (edge, side): flux*len of that side's own evaluation and
 *                  the bed-slope source of that side.  Slot 2e is side A, 2e+1 side B.
 *   inlet  inl_cell, inl_len : phys_inflow only, the entries of the reference's list of inflow
 *                  elements (one per (element, inflow edge), reference order) with, per inlet
 *                  number, the length the entry contributes to calcul_surf_entree.
 * Several independent simulations ("members") can share one flat cell/edge space; each
 * member owns whole tiles of TILE_C cells and TILE_E edges so every tile belongs to one
 * member and the per-member dt minimum is a tile reduction plus one atomic.
 */
#ifndef CF_INTERNAL_H
#define CF_INTERNAL_H

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/cuteflow_gb300.h"

#include <vector_types.h>
#include <vector_functions.h>

namespace cf {

constexpr int TILE_E = 128;  /* edges per tile (= edge-kernel block) */
constexpr int TILE_C = 256;  /* cells per tile (= cell-kernel block) */
constexpr int32_t XD_CELLS = 0x10;  /* tuning-mask bit of the element kernel */

/* Fortran default-real literals of the reference, rounded to single precision. */
constexpr double EPS_HLLC = (double)1e-8f;    /* flux_riemann.cuf:926 */
constexpr double EPS_RIADH = (double)1e-6f;   /* flux_riemann.cuf:1051 */
constexpr double EPS_SECOND = (double)1e-16f; /* flux_riemann.cuf:555, :749 */
constexpr double EPS_VLEER = (double)1e-12f;  /* flux_riemann.cuf:454 */
constexpr double DT_LOW = (double)1e-12f;     /* cfl_condition.cuf:129 */
constexpr double TOL_LOOP = (double)1e-6f;    /* tol, global_data.cuf:59, in the loop test :123 */

struct Slot {
  double f1, f2, f3;   /* flux*len as evaluated by this side, global frame */
  double bx, by;       /* bed-slope source of this side (source_terms.cuf:90-97) */
  double q;            /* boundary discharge diagnostic (boundary edges, side A) */
};

/* Per-member constants. */
struct MemberDev {
  double gp, tolisec, tol, constant_dt, ramp_time, dt_reset;
  double debit_end[CF_MAX_IO];
  double debit_start[CF_MAX_IO];
  double long_entree[CF_MAX_IO];
  double h_sortie[CF_MAX_IO];
  int32_t inlet, outlet, friction, fricimplic, is_dt_constant, pad_;
  int32_t cell_begin, cell_end;   /* real elements [begin, end) of the flat space */
  int32_t edge_begin, edge_end;   /* real edges */
  int32_t bedge_begin, bedge_end; /* boundary edges (a sub-range of the edges) */
  int32_t inl_begin, inl_count;   /* phys_inflow entries [begin, begin + count) */
  int32_t inl_len_off;            /* first entry length: inl_len[inl_len_off + entry * nin + id - 1] */
  int32_t nin;                    /* inlets (nombre_entrees) of the entry table */
  int32_t steady_count;           /* steady-state stop after more than this many qualifying steps */
  int32_t bq_begin;               /* boundary edges in reference order: bq[bq_begin, + bq_count) */
  int32_t bq_count;
  int32_t pad2_;
  double tol_reg_perm;            /* steady-state tolerance; 0: no test */
};

/* Per-member mutable device state.  dt[p] and t[p] belong to the step with parity p; the
 * step with parity p folds the next dt into dt[1-p] with an ordered-integer atomicMin. */
struct MemberState {
  double dt[2];
  double t[2];
  double q_in, q_out;
  long long nstep;   /* steps completed since the state was set */
  uint32_t status;   /* CF_STATUS_* bits; a member with a non-zero status does not step */
  int32_t base;      /* buffer parity at which the state was set: the state is in U[(base + nstep) & 1] */
  int32_t steady_iter;  /* consecutive steps that met the steady-state test */
  int32_t pad_;
  double surf[CF_MAX_IO];  /* phys_inflow: sum of length * depth over each inlet, at the step's start */
  double tc;         /* the reference's loop time: t0, then + the dt computed after every step */
  double ts;         /* cf_run's end time; the member stops when (tc - ts + 2 tol) < tol fails */
};

/* status bit of a member whose state has not been set yet */
constexpr uint32_t STATUS_NO_STATE = 0x80000000u;

/* Everything a step kernel needs, passed by value. */
struct StepArgs {
  const double4* Uin;
  double4* Uout;
  const int4* cslot;
  const int4* cnbr;
  const double4* cstat;
  const double4* ez;       /* per edge: bed of A, of B, of the upwind reconstructions of A and B */
  const int2* ecell;
  const double4* egeo;
  const int32_t* ebid;
  const int4* eupw;
  const double4* ewts;
  const double4* edk;
  const double4* einv;
  Slot* slots;
  const int32_t* etile_mem;
  const int32_t* ctile_mem;
  const MemberDev* mdev;
  MemberState* mst;
  const int32_t* inl_cell;   /* phys_inflow entry tables (NULL without phys_inflow) */
  const double* inl_len;
  int32_t n_etiles, n_ctiles;
  int32_t parity;
  int32_t iflux, ilimiteur, flux_mode;
  int32_t nmembers;
  int32_t phys_inflow;       /* some member uses inlet 3: k_surf runs before the edges */
  int32_t steady;            /* some member tests for steady state: k_steady runs after the cells */
  int32_t xd_cmp;            /* edge kernel: 1 = comparisons on integer keys (cf_xd.h) */
  int32_t xd_mul_mask;       /* with xd_cmp: the edges of warp w (0-3) of an edge tile with bit w set,
                                and with bit 4 (XD_CELLS) the element kernel, form products,
                                quotients and roots on the integer pipes */
  int32_t eblock, ept;       /* launch shape of the edge kernel: threads per block (64, 128, 256) and
                                edges per thread (1, 2) */
  int32_t cblock;            /* threads per block of the element kernel (128, 256) */
  int32_t c_lo, c_hi;        /* elements the element kernel updates: [c_lo, c_hi) of the flat space */
  const int32_t* bq;         /* boundary edges of every member in reference order (MemberDev.bq_*) */
  Slot* sums_out;            /* the adjoint's recording forward: every element's flux and bed sums of the
                                step (the expressions k_rep_cells stores), or NULL */
};

/* ---- host preprocessing (cf_mesh.cpp) ---------------------------------------------- */

struct HostEdge {
  int32_t a, b;      /* new element ids; b < 0: boundary kind */
  int32_t ka, kb;    /* local edge index in a and b */
  int32_t id;        /* inlet/outlet number of a boundary edge */
};

struct Prep {
  int32_t nelt = 0, nnt = 0;
  /* reference-order tables */
  std::vector<int32_t> bnd;       /* nelt*3*2 (boundary(:,:,1:2)) */
  std::vector<int32_t> nbr_k;     /* nelt*3: local edge index in the neighbour */
  std::vector<double> area, zm, cotemin, xc, yc;
  double long_entree[CF_MAX_IO] = {0};
  /* renumbering */
  std::vector<int32_t> perm;      /* new -> old */
  std::vector<int32_t> iperm;     /* old -> new */
  /* device tables in new order (unpadded) */
  std::vector<HostEdge> edges;    /* interior edges, then boundary edges */
  int32_t n_interior = 0;
  std::vector<int4> cslot;
  std::vector<int4> cnbr;
  std::vector<double4> cstat;
  std::vector<double> zcell;      /* new order */
  std::vector<int2> ecell;
  std::vector<double4> egeo;
  std::vector<int32_t> ebid;
  std::vector<int4> eupw;
  std::vector<double4> ewts;
  std::vector<double4> edk;
  std::vector<double4> einv;
  std::vector<double4> ez;        /* per edge: zA, zB, upwind bed of A and of B (second order) */
  /* phys_inflow: one entry per (element, inflow edge) in reference order (compute_input_elems,
   * maillage.cuf:1333-1363): its element (new order) and, per inlet number 1..nin, the length
   * of the element's last inflow edge of that number (0 if none), as calcul_surf_entree
   * (maillage.cuf:1368-1421) weighs the element's depth */
  std::vector<int32_t> inl_cell;
  std::vector<double> inl_len;    /* [entries * nin] */
  int32_t nin = 0;
  /* boundary edges (device edge index) in reference order: element, then local edge; the
   * discharge sums run over this list (so that a decomposed mesh can reproduce them) */
  std::vector<int32_t> bq_ref;
  /* a part of a decomposed mesh (element classes given): the elements are ordered send, interior,
   * halo; elist1 holds the edges of the send elements, elist2 those of the interior ones that
   * are not in elist1 (the halo's other edges are not evaluated) */
  int32_t n_send = 0, n_own = 0;
  std::vector<int32_t> elist1, elist2;
};

/* Build every host table from the reference mesh inputs.  elem_class (NULL: a whole mesh) gives,
 * for a part of a decomposed mesh, each element's class: 0 owned interior, 1 owned and read by
 * another part (send), 2 halo.  Returns CF_OK or CF_EINVAL with a message in err. */
int prepare_mesh(const cf_mesh* m, const cf_params* p, Prep& out, std::string& err,
                 const int32_t* elem_class = nullptr);

/* ---- kernel launchers (cf_kernels.cu) ---------------------------------------------- */

typedef struct CUstream_st* stream_t;

int launch_step(const StepArgs& a, stream_t s, void* ev_mid, void* ev_end);
/* the edge kernel of one scheme in the shape a.eblock x a.ept (cf_edges_<IFLUX>.cu) */
int launch_edges_1(const StepArgs& a, stream_t s);
int launch_edges_2(const StepArgs& a, stream_t s);
int launch_edges_3(const StepArgs& a, stream_t s);
int launch_edges_4(const StepArgs& a, stream_t s);
int launch_probe_fp64(double* out, int32_t nblocks, int64_t iters, stream_t s);  /* nblocks x 256 outputs */
int launch_selftest_xd(int64_t n, uint64_t seed, unsigned long long* bad, int32_t nblocks, stream_t s);
int launch_cfl(const double4* U, const double4* cstat, const int32_t* ctile_mem, int32_t tile_begin,
               int32_t n_tiles, const MemberDev* mdev, MemberState* mst, int32_t slot, stream_t s);
int launch_discharge(const Slot* slots, const int2* ecell, const int32_t* bq, const MemberDev* mdev, MemberState* mst,
                     int32_t nmembers, stream_t s);
/* A part of a decomposed mesh.  One phase of its step: phase 1 first makes every member's step
 * start (k_begin_step); then the edges of elist and the element update of [c_lo, c_hi). */
int launch_part_phase(const StepArgs& a, int phase, const int32_t* elist, int32_t nel, int32_t c_lo, int32_t c_hi,
                      stream_t s);
int launch_edges_list_1(const StepArgs& a, const int32_t* list, int32_t n, stream_t s);
int launch_edges_list_2(const StepArgs& a, const int32_t* list, int32_t n, stream_t s);
int launch_edges_list_3(const StepArgs& a, const int32_t* list, int32_t n, stream_t s);
int launch_edges_list_4(const StepArgs& a, const int32_t* list, int32_t n, stream_t s);
/* (h, hu, hv) of the listed elements (device order) into / out of buf (device or pinned host) */
int launch_pack(const double4* U, const int32_t* ids, int32_t n, double* buf, stream_t s);
int launch_unpack(double4* U, const int32_t* ids, int32_t n, const double* buf, stream_t s);
/* member 0's phys_inflow terms of U (entries x inlets) and boundary discharges (reference order) */
int launch_inlet_terms(const StepArgs& a, const double4* U, int32_t count, double* out, stream_t s);
int launch_bq_terms(const Slot* slots, const int32_t* bq, const MemberDev* mdev, int32_t count, double* out, stream_t s);
/* member 0's discharges and steady-state test with given (whole-mesh) discharges */
int launch_steady_apply(const MemberDev* mdev, MemberState* mst, double qi, double qo, stream_t s);
/* phys_inflow inlet sums of the state U into mst[m].surf (every member with inlet 3) */
int launch_surf(const StepArgs& a, const double4* U, stream_t s);
/* hu3 (reference order, one member) <-> U (new order); perm/iperm/zcell/U point at the member's
 * first element, the permutations hold member-local indices. */
int launch_scatter_state(const double* hu3, const int32_t* perm_new2old, const double* zcell,
                         double4* U, int32_t n, stream_t s);
int launch_gather_state(const double4* U, const int32_t* iperm_old2new, double* hu3, int32_t n,
                        stream_t s);
/* launch_gather_state out of member m's current buffer, chosen on the device from mst[m] */
int launch_gather_current(const double4* U0, const double4* U1, const MemberState* mst, int32_t m,
                          const int32_t* iperm, double* hu3, int32_t n, stream_t s);
/* The same directly between a buffer the GPU can address (device memory, or pinned host memory over
 * the CPU link) and U, coalesced on the buffer's side: load writes U[iperm[o]] from hu3[3 o ..];
 * store reads U0 (or, with mst, member m's current buffer of U0 / U1) into hu3. */
int launch_load_ref(const double* hu3, const int32_t* iperm_old2new, double4* U, int32_t n, stream_t s,
                    const double4* cstat = nullptr, const MemberDev* mdev = nullptr, MemberState* mst = nullptr,
                    int32_t m = 0, int32_t slot = 0);   /* with mst: also the state's CFL dt into mst[m].dt[slot] */
int launch_store_ref(const double4* U0, const double4* U1, const MemberState* mst, int32_t m,
                     const int32_t* iperm_old2new, double* hu3, int32_t n, stream_t s);
/* (h, hu, hv) of listed elements (member-local reference ids, iperm member-local) */
int launch_gather_ids(const double4* U, const int32_t* iperm, const int32_t* ids, double* out, int32_t n, stream_t s);
int launch_scatter_ids(double4* U, const int32_t* iperm, const int32_t* ids, const double* in, int32_t n, stream_t s);

/* ---- discrete adjoint (cf_adjoint.cu) ------------------------------------------------- */

/* One reverse step n: s holds the step's buffers with s.Uin = U^n. */
struct AdjArgs {
  StepArgs s;
  const double* dt_hist;   /* dt of every step and member (frozen), [N][members] */
  const double* t_hist;    /* start time of every step and member */
  int32_t n;
  int32_t gather;          /* 1: lambda^{n+1} = lam_own + the edge contributions; 0: lam_init */
  const Slot* sums;        /* per element: its flux sums (f1..f3) and bed sums (bx, by) at U^n */
  const double4* lam_init; /* lambda^N */
  double4* lam_own;        /* in: the element's own part of lambda^{n+1}; out: of lambda^n */
  Slot* cadj;              /* per element: adjoint of its flux sums (f1..f3) and bed sums (bx, by) */
  double4* eadj;           /* per edge side: contribution to the side's element */
  double4* uadj;           /* per edge, 4: contributions to the upwind elements (second order) */
  const int32_t* uoff;     /* per element: its entries in uidx (second order; NULL otherwise) */
  const int32_t* uidx;
  const int32_t* goff;     /* per element: its gauges in gidx */
  const int32_t* gidx;
  const double* gw;        /* objective weights of the gauge elevations after step n+1, or NULL */
  double* gman;            /* dJ/dn, accumulated */
  int32_t freeze_r;        /* 1: WAF limiter ratios held constant in the linearization */
  int32_t* pend;           /* first-order HLLC: interior edges left to the six-lane kernel */
  int32_t* npend;          /* their count (zeroed before each reverse step) */
};

/* Step n with the recorded dt / time: edge stage, then element stage writing a.Uout (if not
 * NULL) and, if sums is not NULL, every element's flux and bed sums; non-finite results are
 * OR-ed into *flag. */
int launch_replay_step(const StepArgs& a, const double* dt_hist, const double* t_hist, int n, uint32_t* flag,
                       Slot* sums, stream_t s);
/* gauge elevations h + z of Unew into eta row n; with S, also dt / t of parity p into the histories */
int launch_record(const double4* Unew, const double* zcell, const MemberState* S, int nm, int p, int n, double* dt_hist,
                  double* t_hist, const int32_t* gcell, int G, double* eta, stream_t s);
int launch_adjoint_step(const AdjArgs& A, stream_t s);
/* lambda^0 = lam_own + the edge contributions of the last reverse step, into lam_own */
int launch_adjoint_final(const AdjArgs& A, stream_t s);
int launch_add_gauges(double4* lam, const int32_t* goff, const int32_t* gidx, const double* gw, int32_t n, stream_t s);
int launch_gather_scalar(const double* x, const int32_t* iperm, double* out, int32_t n, stream_t s);
int launch_set_manning(double4* cstat, const int32_t* perm, const double* nref, int32_t n, stream_t s);
/* Manning zones: fixed-order zone sums of dJ/dn (CSR zone -> elements, new order), a projected
 * gradient step on the zone values, and the zone values into every element's n */
int launch_zone_sum(const double* gman, const int32_t* zoff, const int32_t* zidx, double* gz, int32_t nz, stream_t s);
int launch_zone_step(double* v, const double* g, int32_t nz, double lr, double lo, double hi, stream_t s);
int launch_zone_apply(double4* cstat, const int32_t* zone_of, const double* v, int32_t n, stream_t s);

/* ---- context helpers for the static-scratch entry point (cf_api.cpp) ---------------- */

int ctx_set_device(cf_ctx* c);                                /* the context's device current */
int ctx_error(cf_ctx* c, int code, const std::string& msg);  /* record msg, return code */
/* The steps of cf_step with the edge-flux slots at `slots` (room for `capacity` slots) in
 * place of the context's own slot buffer: direct launches, no graph, no allocation. */
int step_with_slots(cf_ctx* c, int32_t nsteps, cf_step_info* infos, Slot* slots, size_t capacity);

/* lec_mail_cgns (maillage.cuf:398-778) for one process, without libcgns (cf_cgns.cpp): a CGNS/HDF5
 * triangle mesh with its inflow/outflow node lists (numbered by inlet_name / outlet_name) and, when
 * want_manning, the per-element "Manning" user data.  Returns a CF_* code; err says why. */
struct CgnsMesh {
  std::vector<double> x, y, z, manning_elt;
  std::vector<int32_t> tri, ndinput, numero_ndinput, ndoutput, numero_ndoutput;
  bool has_manning = false;
};
int read_cgns_mesh(const std::string& path, const std::vector<std::string>& inlet_names,
                   const std::vector<std::string>& outlet_names, bool want_manning, CgnsMesh& M, std::string& err);

}  // namespace cf

#endif
