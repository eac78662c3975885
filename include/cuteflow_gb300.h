/*
 * cuteflow_gb300.h -- C ABI of the GB300-native CuteFlow time step (libcfgb.so).
 *
 * The reference has no library API: its hot path is the body of solve_finite_volumes
 * (finite_volumes_method.cuf:123-242), which reaches the kernels through module globals
 * (global_data_device.cuf:8-76) filled by the host setup (data_transfer.cuf:4-100,
 * maillage.cuf:4-166, main.cuf:124-169).  This header replaces that surface with plain
 * C entry points a Fortran ISO_C_BINDING module (or ctypes, cgo, JNI) binds directly.
 *
 * Conventions
 *  - Every call returns 0 or a negative CF_E* code; nothing calls exit().  The text of the
 *    last error of a context is available from cf_last_error().
 *  - Host arrays passed in are borrowed for the duration of the call only.
 *  - Element order and indexing at the boundary are the reference's: element k of the mesh
 *    tables is element k everywhere (any internal renumbering is undone on output), node
 *    and element ids inside the mesh tables are 1-based, and states are element-major
 *    (h, hu, hv) triples exactly like vdlg(3, nelt).
 *  - A context owns all of its device memory and one CUDA stream; it is used by one host
 *    thread at a time.  Separate contexts are independent.
 *  - Arithmetic is IEEE FP64 throughout.
 */
#ifndef CUTEFLOW_GB300_H
#define CUTEFLOW_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CF_MAX_IO 20

/* Error codes */
#define CF_OK 0
#define CF_EINVAL -1     /* bad argument or inconsistent input */
#define CF_ECUDA -2      /* CUDA runtime error (message in cf_last_error) */
#define CF_ENOMEM -3     /* device or host allocation failed */
#define CF_EDT -4        /* time step left the range (1e-12, 9999] (cfl_condition.cuf:129-132) */
#define CF_ENONFINITE -5 /* a NaN or Inf appeared in the state */
#define CF_ESTATE -6     /* call out of order (e.g. stepping before a state was set) */
#define CF_ENOTSUP -7    /* option not implemented */

/* Device status bits reported in cf_step_info.status */
#define CF_STATUS_DT_RANGE 1u
#define CF_STATUS_NONFINITE 2u
#define CF_STATUS_STEADY 4u      /* steady state reached (check_steady_state,
                                    finite_volumes_method.cuf:370-393): the member stops, no error */
#define CF_STATUS_END 8u         /* cf_run reached its end time ts: the member stops, no error */

/* Mesh tables, as lec_mail_tri reads them (maillage.cuf:196-313). */
typedef struct cf_mesh {
  int32_t nnt;                     /* number of nodes (nnt) */
  int32_t nelt;                    /* number of triangles (nelt) */
  const double* x;                 /* [nnt] coordonnees(:,1) */
  const double* y;                 /* [nnt] coordonnees(:,2) */
  const double* z;                 /* [nnt] coordonnees(:,3): bed elevation at the nodes */
  const int32_t* tri;              /* [3*nelt] 1-based node ids, tri[3*k+j] = connectivite(k+1,j+1);
                                      edge j joins node j and node j+1 (mod 3) */
  const double* manning_elt;       /* [nelt] manning_nelt; may be NULL with is_override_manning */
  const int32_t* ndinput;          /* [ndi] inflow nodes (ndinput) */
  const int32_t* numero_ndinput;   /* [ndi] inlet number of each inflow node (numero_ndinput) */
  const int32_t* ndoutput;         /* [ndo] outflow nodes (ndoutput) */
  const int32_t* numero_ndoutput;  /* [ndo] outlet number of each outflow node (numero_ndoutput) */
  const int32_t* ndwall;           /* [ndw] wall nodes (ndwall) */
  int32_t ndi, ndo, ndw;
  int32_t nombre_entrees;          /* number of inlets (nombre_entrees) */
  int32_t nombre_sorties;          /* number of outlets (nombre_sorties) */
  int32_t pad_;
} cf_mesh;

/* The used subset of the donnees_namelist (global_data.cuf:31-94) plus extensions. */
typedef struct cf_params {
  double gp;                       /* gravity (gp) */
  double tolisec;                  /* dry threshold (tolisec) */
  double cfl;                      /* CFL number (cfl) */
  double tol;                      /* friction velocity floor; the reference's tol is the
                                      single-precision literal 1e-6 (global_data.cuf:59) */
  double override_manning;         /* (override_manning) */
  double constant_dt;              /* (constant_dt) */
  double debitglob[CF_MAX_IO];     /* inflow discharge per inlet, m^3/s (debitglob) */
  double h_sortie[CF_MAX_IO];      /* water level per outlet (h_sortie) */
  double debitglob_start[CF_MAX_IO]; /* extension: discharge at t = 0 of a linear ramp */
  double ramp_time;                /* extension: ramp duration in s; 0 keeps debitglob constant */
  int32_t iflux;                   /* 1 HLLC, 2 HLLC (Ata et al. star states), 3 WAF, 4 MUSCL */
  int32_t ilimiteur;               /* limiter (ilimiteur), default 1 */
  int32_t friction;                /* 1: Manning friction (friction) */
  int32_t fricimplic;              /* 0 explicit, 1 (I - dt/2 J)^-1, 2 diagonal (fricimplic) */
  int32_t is_override_manning;     /* (is_override_manning) */
  int32_t is_dt_constant;          /* (is_dt_constant) */
  int32_t inlet;                   /* 1 'transm', 2 'inflow', 3 'phys_inflow' (data_transfer.cuf:43-55):
                                      3 spreads debitglob over the inlet in proportion to the
                                      depth of its elements (flux_riemann.cuf:127-138,
                                      calcul_surf_entree maillage.cuf:1368-1421) */
  int32_t outlet;                  /* 1 'fixedheight', 2 'transm' (data_transfer.cuf:57-66) */
  int32_t flux_mode;               /* extension: 0 (default) = the reference's semantics, the flux of
                                      every (element, edge) as that element evaluates it
                                      (flux_riemann.cuf:33-426); 1 = conservative, one evaluation
                                      per edge with the opposite sign for the neighbour */
  int32_t reorder;                 /* extension: element order on the device: 1 = along a Hilbert curve of the
                                      centroids (default), 2 = along a Morton curve, 0 = the caller's
                                      order (results are identical; cf_autotune_order picks one) */
  int32_t pad_;
  double tol_reg_perm;             /* steady-state stop (tol_reg_perm): after a step whose inflow
                                      Q_in > 1e-8 and |Q_in - Q_out| / Q_in < tol_reg_perm for
                                      more than steady_count consecutive steps the member stops
                                      with CF_STATUS_STEADY; 0 (default) disables the test */
  int32_t steady_count;            /* 1000 in the reference (finite_volumes_method.cuf:380) */
  int32_t dt_reset_nelt;           /* extension: the element count whose remainder mod 1024 selects the
                                      dt minimum's start value 1e5 / 1e6 (cfl_condition.cuf:86); 0 = the
                                      mesh's own (a part of a decomposed mesh passes the whole mesh's) */
  double long_entree[CF_MAX_IO];   /* extension: inlet lengths; 0 = measured on the mesh (a part of a
                                      decomposed mesh passes the whole mesh's, calcul_long_entree) */
} cf_params;

/* set_initial_condition inputs (initial_condition.cuf:4-80, namelist global_data.cuf:40-44). */
typedef struct cf_ic {
  double x1eqbar, x2eqbar, y1eqbar, y2eqbar;
  double h_amont, u_amont, v_amont, h_aval, u_aval, v_aval;
  double xplan, yplan, zplan, xpoint, ypoint, zpoint;
  int32_t eqlin_barrage;
  int32_t plan;
} cf_ic;

/* Result of cf_step. */
typedef struct cf_step_info {
  double t;                        /* time after the last step: t0 + sum of the dt used */
  double dt_last;                  /* dt used by the last step */
  double dt_next;                  /* dt the next step will use (CFL of the current state) */
  double q_in;                     /* inflow discharge of the last step (debit_entree_sum) */
  double q_out;                    /* outflow discharge of the last step (debit_sortie) */
  int64_t steps;                   /* steps taken since the state was set */
  uint32_t status;                 /* CF_STATUS_* bits latched on the device */
  int32_t pad_;
} cf_step_info;

typedef struct cf_ctx cf_ctx;

/* Fill p with the reference's namelist defaults (global_data.cuf:31-62) and the values the
 * reference's own cases set (gp = 9.81, tolisec = 1e-5, cfl = 0.9, iflux = 1). */
int cf_default_params(cf_params* p);

/* Build a context: boundary tagging and adjacency (replaces tab_bound_tri / boundary_kind,
 * maillage.cuf:781-1110, and set_undefined_boudaries_as_walls, :1454-1471), geometry
 * (compute_surface_and_bathy :1284-1331, the CFL length :132-165, inlet lengths
 * :1423-1452), upwind tables (find_upwind_cells :954-978), renumbering and upload. */
int cf_create(const cf_mesh* mesh, const cf_params* params, cf_ctx** out);

/* Destroy a context and release its device memory (NULL is accepted). */
void cf_destroy(cf_ctx* ctx);

/* Set U^0 from host memory: hu3[3*k+c] = vdlg0(c+1, k+1) (read_initial_condition,
 * initial_condition.cuf:82-102).  Resets the time to t0 and the step count, and computes
 * the first dt (finite_volumes_method.cuf:113-116).  Returns once hu3 has been read (the
 * caller may reuse it); the state's device-side setup runs ahead of the context's next call. */
int cf_set_state(cf_ctx* ctx, const double* hu3, double t0);

/* Same with a device pointer (3*nelt doubles, reference element order). */
int cf_set_state_device(cf_ctx* ctx, const double* d_hu3, double t0);

/* Initial condition by dam line or plane (set_initial_condition, initial_condition.cuf:4-80),
 * then as cf_set_state. */
int cf_set_initial_condition(cf_ctx* ctx, const cf_ic* ic, double t0);

/* Advance nsteps steps of the time loop (finite_volumes_method.cuf:123-242 without file
 * output).  Each step: fluxes, sources and friction, update with the wet/dry clamp, and the
 * CFL dt of the new state for the next step, all on the device with no host round trip.
 * info is NULL or an array of cf_get_members(ctx) records (one for a plain context).
 * Returns CF_EDT / CF_ENONFINITE when a member has stopped (that member no longer steps; the
 * others do), CF_ESTATE for a plain context without a state. */
int cf_step(cf_ctx* ctx, int32_t nsteps, cf_step_info* info);

/* A host-held state advanced by nsteps steps in one call: cf_set_state(hu3_in, t0), cf_step(nsteps),
 * cf_get_state(hu3_out), with the copies, the steps and the read-back in one stream-ordered sequence
 * and a single wait (for a caller that keeps the state itself, e.g. a coupled model exchanging it
 * every step).  hu3_in and hu3_out may be the same buffer.  Contexts with one member; the result
 * and the return code are those of the three calls. */
int cf_advance(cf_ctx* ctx, const double* hu3_in, double t0, int32_t nsteps, double* hu3_out, cf_step_info* info);

/* The reference's time loop (solve_finite_volumes, finite_volumes_method.cuf:123-242): steps
 * every member until the loop test (tc - ts + 2 tol) < tol fails (tol = 1e-6 in single
 * precision, tc = the state's t0 plus the dt computed after every step, :232), the
 * steady-state test stops it (tol_reg_perm), or max_steps steps have run.  Members that
 * reach ts stop with CF_STATUS_END; a later cf_run with a larger ts continues them.  The
 * test runs on the device, so every member stops at its own step.  Returns as cf_step. */
int cf_run(cf_ctx* ctx, double ts, int64_t max_steps, cf_step_info* info);

/* Copy U^n to host memory in reference order (3*nelt doubles). */
int cf_get_state(cf_ctx* ctx, double* hu3_out);

/* Copy U^n to device memory in reference order (3*nelt doubles). */
int cf_get_state_device(cf_ctx* ctx, double* d_hu3_out);

/* Current time, dt and status without stepping. */
int cf_get_info(cf_ctx* ctx, cf_step_info* info);

/* ---- The reference's input files -------------------------------------------------------
 * A case directory as the reference's main program reads it (main.cuf:48-182): the
 * donnees_namelist file (lec_donnees, maillage.cuf:168-193; keys of global_data.cuf:65-94,
 * unknown keys are an error as in a Fortran namelist read), the ASCII mesh it names
 * (meshfile_path // meshfile, lec_mail_tri, maillage.cuf:196-313; is_cgns = 1 gives
 * CF_ENOTSUP) and, with solinit = 1, the element initial-condition file fich_sol_init
 * (read_initial_condition, initial_condition.cuf:82-102).  Relative paths are taken from dir.
 * The mesh and params pointers stay valid until cf_case_free. */
typedef struct cf_case cf_case;
int cf_case_read(const char* dir, const char* namelist_file /* NULL: "donnees.f" */, cf_case** out);
void cf_case_free(cf_case* c);
/* Text of the last failed cf_case_* / cf_write_state_file call of this thread. */
const char* cf_case_last_error(void);
/* Mesh and parameters for cf_create, the dam line / plane of the namelist (cf_ic), its end time
 * ts and solinit; any pointer may be NULL. */
int cf_case_get(const cf_case* c, const cf_mesh** mesh, const cf_params** params, cf_ic* ic, double* ts,
                int32_t* solinit);
/* solinit = 1: the state of fich_sol_init (3*nelt doubles) and the time written on its first
 * line (which the reference reads but does not use: main.cuf:182 starts at tc = 0). */
int cf_case_initial_state(const cf_case* c, double* hu3, double* t_file);
/* Write a state in the layout of save_sol_for_restart (pre_post_traitement.cuf:498-512): the
 * time, then h, hu, hv of every element in fields '(4f16.6)', which keep 6 decimals. */
int cf_write_state_file(const char* path, const double* hu3, int32_t nelt, double t);

/* ---- Batched ensembles (no reference counterpart: the reference runs ensemble members as
 * separate processes, scripts/array.sh:8-11, Calibration_manning/scripts/calib_array.sh:8-11).
 * A batch context holds nmembers independent simulations of uneven size in one flat
 * element/edge space; every cf_step advances all of them in the same kernel launches, each
 * with its own parameters, dt, time and status.  All members share iflux, ilimiteur and
 * flux_mode.  Member indices are 0-based; the plain functions above act on member 0. */
int cf_create_batch(const cf_mesh* meshes, const cf_params* params, int32_t nmembers, cf_ctx** out);
int cf_get_members(cf_ctx* ctx);
int cf_member_set_state(cf_ctx* ctx, int32_t member, const double* hu3, double t0);
int cf_member_set_initial_condition(cf_ctx* ctx, int32_t member, const cf_ic* ic, double t0);
int cf_member_get_state(cf_ctx* ctx, int32_t member, double* hu3_out);
int cf_member_get_info(cf_ctx* ctx, int32_t member, cf_step_info* info);
int cf_member_get_mesh_tables(cf_ctx* ctx, int32_t member, int32_t* boundary, double* area, double* zm,
                              double* cotemin);

/* Preprocessing results in reference order, for comparison with the reference's own
 * boundary table file (maillage.cuf:62-68).  boundary: [nelt*3*2] int32 with
 * boundary[(k*3+j)*2+0] = neighbour id (1-based) or -1 inflow / -2 outflow / -3 wall and
 * boundary[(k*3+j)*2+1] = inlet/outlet number (the element's own id elsewhere).
 * area, zm, cotemin: [nelt] each; any pointer may be NULL. */
int cf_get_mesh_tables(cf_ctx* ctx, int32_t* boundary, double* area, double* zm, double* cotemin);

/* The same tables computed from the mesh alone, without a context or a GPU (the host
 * preprocessing of cf_create).  Lets a caller check its inputs on a machine without a GPU. */
int cf_mesh_tables(const cf_mesh* mesh, const cf_params* params, int32_t* boundary, double* area,
                   double* zm, double* cotemin);

/* Number of elements and edges of the context (all members); edges counts each shared edge
 * once. */
int cf_get_sizes(cf_ctx* ctx, int64_t* nelt, int64_t* nedge);

/* The CUDA stream (cudaStream_t) the context launches on. */
void* cf_get_stream(cf_ctx* ctx);

/* Text of the last error of ctx (or of the last failed cf_create when ctx is NULL). */
const char* cf_last_error(const cf_ctx* ctx);

/* ---- Pieces of a decomposed mesh (the reference's MPI decomposition, memory_exchange_functions.cuf,
 * finite_volumes_method.cuf:141-171): each part is its own context over its elements and a halo of
 * the neighbours' elements (one ring of neighbours; two for iflux 3 and 4, whose upwind states read
 * the neighbours' neighbours).  After every step the caller copies the owners' states into the
 * halos and applies the minimum dt over all parts (the reference's MPI_ALLREDUCE MIN).  With the
 * whole mesh's inlet lengths and element count in cf_params (long_entree, dt_reset_nelt), every
 * element evolves bit for bit as in the undivided mesh.
 * cf_get_elements / cf_set_elements read / write (h, hu, hv) of listed elements (0-based, member-local
 * reference order) of the current state; cf_set_elements then recomputes the member's next dt from
 * the CFL of the state as it now is.  cf_set_dt sets the member's next dt. */
int cf_get_elements(cf_ctx* ctx, int32_t member, const int32_t* ids, int32_t n, double* hu3_out);
int cf_set_elements(cf_ctx* ctx, int32_t member, const int32_t* ids, int32_t n, const double* hu3);
int cf_set_dt(cf_ctx* ctx, int32_t member, double dt);

/* A part as its own rank, with the reference's send-cells-first step (finite_volumes_method.cuf:141-171;
 * update_send_cells and gpu_echange_cgns, memory_exchange_functions.cuf:129-172).
 * cf_create_part: as cf_create for one mesh (a part: own elements and halo), with elem_class[k] the
 *   class of element k: 0 owned interior, 1 owned and held in another part's halo (send), 2 halo.
 * cf_part_set_exchange: the send elements (class 1) whose states go out, and the halo elements
 *   (class 2) whose states come in, each in the order of the caller's buffers (0-based ids).
 * cf_part_step_begin: enqueues one step: its start (dt test, next time), the send elements' edges
 *   and update, their new states packed into send_buf (3 per element, in the exchange order; device
 *   memory or pinned host memory, written by the kernel over the CPU link), then the interior
 *   elements' edges and update; returns without waiting.
 * cf_part_wait_send: waits until send_buf is complete (the interior may still be running).
 * cf_part_step_end: unpacks recv_buf (the halo states, exchange order) into the new state, waits,
 *   and reports the step (info.dt_next: the part's own elements' minimum; the caller applies the
 *   minimum over the parts with cf_set_dt, the reference's MPI_ALLREDUCE MIN).
 * The whole mesh's sums (MPI_ALLREDUCE SUM, finite_volumes_method.cuf:133-138, :218-219):
 * cf_part_inlet_terms: before a phys_inflow step, the part's inlet terms (length * depth, entries x
 *   inlets, its inlet entries in element then local-edge order); the caller sums the whole mesh's
 *   entries in the step's order and passes the sums per inlet to cf_part_set_inlet_sums (required
 *   before every step of a phys_inflow part).
 * cf_part_discharge_terms: after a step, the part's boundary discharges (its boundary edges in element
 *   then local-edge order); the caller sums the whole mesh's and passes them to
 *   cf_part_apply_discharges, which sets info.q_in / q_out and applies the steady-state test.
 * cf_part_sizes: send and own element counts, inlet entries and boundary edges of the part. */
int cf_create_part(const cf_mesh* mesh, const cf_params* params, const int32_t* elem_class, cf_ctx** out);
int cf_part_sizes(cf_ctx* ctx, int32_t* n_send, int32_t* n_own, int32_t* inlet_entries, int32_t* boundary_edges);
int cf_part_set_exchange(cf_ctx* ctx, const int32_t* send_ids, int32_t nsend, const int32_t* recv_ids, int32_t nrecv);
int cf_part_step_begin(cf_ctx* ctx, double* send_buf);
int cf_part_wait_send(cf_ctx* ctx);
int cf_part_step_end(cf_ctx* ctx, const double* recv_buf, cf_step_info* info);
int cf_part_inlet_terms(cf_ctx* ctx, double* out);
int cf_part_set_inlet_sums(cf_ctx* ctx, const double* surf);
int cf_part_discharge_terms(cf_ctx* ctx, double* out);
int cf_part_apply_discharges(cf_ctx* ctx, double q_in, double q_out);

/* How the step shares its FP64 work between GB300's FP64 pipe and its integer pipes (results
 * are identical bit for bit in every setting): int_compare 1 evaluates the edge kernel's
 * comparisons on integer keys of the bit patterns; bits 0-3 of int_mul_warps are a mask over
 * the 4 warps of an edge block, and the warps whose bit is set form products, quotients, square
 * roots and scalings by 2^k in exact integer arithmetic on the significands (correctly rounded,
 * the IEEE results); bit 4 does the same for the element kernel.  Default (0, 0): every
 * operation on the FP64 pipe.  cf_autotune picks a setting by timing. */
int cf_set_tuning(cf_ctx* ctx, int32_t int_compare, int32_t int_mul_warps);
int cf_get_tuning(cf_ctx* ctx, int32_t* int_compare, int32_t* int_mul_warps);
/* Launch shape of the step (no counterpart in the reference, whose launch shapes are fixed,
 * finite_volumes_method.cuf:85-109): threads per block of the edge kernel (64, 128 or 256), edges
 * each of its threads evaluates (1 or 2), threads per block of the element kernel (128 or 256).
 * Default (256, 1, 128).  Results are identical bit for bit in every shape. */
int cf_set_launch_shape(cf_ctx* ctx, int32_t edge_block, int32_t edges_per_thread, int32_t cell_block);
int cf_get_launch_shape(cf_ctx* ctx, int32_t* edge_block, int32_t* edges_per_thread, int32_t* cell_block);
/* Autotuner: times steps_per_trial steps on the context's own state and keeps the fastest
 * setting (the state, time and step count are restored after each trial, so the simulation is
 * unchanged): first the integer-pipe setting (8 candidates), then the edge kernel's launch shape
 * (6) and the element kernel's block (2).  Returns the integer-pipe setting and the best time per
 * step; cf_get_launch_shape reports the shape.  Every member must have a state and be running.
 * Outputs may be NULL. */
int cf_autotune(cf_ctx* ctx, int32_t steps_per_trial, int32_t* int_compare, int32_t* int_mul_warps,
                double* ms_per_step);
/* The element order (params->reorder 1 Hilbert, 2 Morton, 0 the caller's) with which a context of
 * this mesh steps fastest: creates a context per order, sets the state hu3, runs cf_autotune on
 * it, and destroys it.  The caller then creates its context with that order.  Outputs may be
 * NULL. */
int cf_autotune_order(const cf_mesh* mesh, const cf_params* params, const double* hu3, int32_t steps_per_trial,
                      int32_t* reorder, double* ms_per_step);

/* Diagnostic: the FP64 pipe's throughput on the context's device in FP64 instructions per second
 * (independent FMA chains on every SM, timed with CUDA events), the denominator of the step's
 * roofline: the step is bound by FP64 instruction issue, not by HBM.  Allocates and frees a
 * scratch buffer of 2 KB per block. */
int cf_probe_fp64(cf_ctx* ctx, double* instr_per_s);

/* Diagnostic: checks the integer-pipe arithmetic the tuned step uses (products, quotients,
 * scalings by 2^k, negation and comparisons of doubles in integer instructions) against the
 * device's FP64 unit on n adversarial operand pairs generated on the device from seed, and
 * stores in *mismatches how many results differ in any bit (0 expected).  Allocates and frees
 * 8 bytes of device memory. */
int cf_selftest_xd(cf_ctx* ctx, int64_t n, uint64_t seed, int64_t* mismatches);

/* How cf_set_state, cf_get_state and cf_advance move a caller's state (no counterpart in the
 * reference, which keeps the state on the device).  enable = 1 (the default): a state buffer
 * the device can address (device memory, or pinned host memory, which GB300 reaches over its
 * coherent CPU link) is read and written by the state kernels themselves, coalesced in the
 * caller's element order, with no staging copy; pageable host memory is still copied through a
 * device staging buffer.  enable = 0: every buffer goes through the staging copy.  The results
 * are the same bytes either way. */
int cf_set_direct_io(cf_ctx* ctx, int32_t enable);

/* Kernel timing of the last cf_step call: total device milliseconds of the edge-flux and
 * cell-update kernels measured with CUDA events when timing is enabled. */
int cf_set_timing(cf_ctx* ctx, int32_t enable);
int cf_get_timing(cf_ctx* ctx, double* flux_ms, double* update_ms, int64_t* launches);

/* ---- discrete adjoint (new: the reference has no gradients) ----------------------------
 *
 * For Manning calibration: gradients of an objective on gauge elevations and on the final
 * state with respect to the per-element Manning n and the initial state, by the discrete
 * adjoint of the step (the dt of every step held at its recorded value).  Contexts with one
 * member, or the members of a batch (cf_adjoint_create_batch).
 *
 *   J = sum_{k=1..N} sum_g w_eta[(k-1)*G + g] * eta^k_g  +  sum_e w_state[3e..3e+2] . U^N_e
 *
 * eta^k_g = h + z of gauge element g (0-based, reference order) after step k of a run of N
 * steps from the context's current state.  Pointers of the run functions may be host or
 * device memory. */
typedef struct cf_adjoint cf_adjoint;

/* Per-element Manning n [nelt], reference order (replaces the mesh's values and the override);
 * cf_set_manning for a one-member context, cf_member_set_manning for member m of a batch. */
int cf_set_manning(cf_ctx* ctx, const double* n_elt);
int cf_member_set_manning(cf_ctx* ctx, int32_t member, const double* n_elt);

/* An adjoint of N steps with G gauges; checkpoint_interval K (0: ceil(sqrt(N))): the state is
 * kept every K steps, ceil(N/K) + max(K, 2) states of device memory. */
int cf_adjoint_create(cf_ctx* ctx, int32_t nsteps, int32_t checkpoint_interval, const int32_t* gauges,
                      int32_t ngauges, cf_adjoint** out);
/* The adjoint of a batch: every member runs the same N steps with its own dt, in the same
 * launches.  Gauge g is element gauges[g] (0-based, reference order) of member gauge_member[g].
 * States, weights and gradients of the run functions are concatenated in member order
 * ([sum of nelt] elements); the dt / time histories are [N][members]. */
int cf_adjoint_create_batch(cf_ctx* ctx, int32_t nsteps, int32_t checkpoint_interval, const int32_t* gauge_member,
                            const int32_t* gauges, int32_t ngauges, cf_adjoint** out);
/* The adjoint (one member: gauge_member may be NULL; a batch: as cf_adjoint_create_batch) with
 * its memory schedule chosen to fit budget_bytes of device memory (no counterpart in the
 * reference).  A reverse step needs the state and every element's flux and bed sums of its
 * forward step (a record, 80 bytes per element); the recording forward keeps the records of the
 * last steps itself, as many as fit, so that the backward pass replays only the steps before
 * them, from checkpoints every checkpoint_interval steps (0: as long as the record pool).  When
 * the whole run fits nothing is replayed.  CF_ENOMEM when no schedule fits.  The gradient is the
 * same, bit for bit, under every schedule. */
int cf_adjoint_create_budget(cf_ctx* ctx, int32_t nsteps, int32_t checkpoint_interval, const int32_t* gauge_member,
                             const int32_t* gauges, int32_t ngauges, int64_t budget_bytes, cf_adjoint** out);
/* The schedule: steps whose records the recording forward keeps (the last stored_steps), the
 * checkpoint interval and count of the steps before them, the record pool, device bytes. */
int cf_adjoint_schedule(cf_adjoint* adj, int32_t* stored_steps, int32_t* checkpoint_interval, int32_t* checkpoints,
                        int32_t* records, int64_t* device_bytes);
void cf_adjoint_destroy(cf_adjoint* adj);

/* N steps from the context's current state (which is left unchanged).  replay 0: the dt of
 * every step comes from the CFL condition, as in cf_step (bit-identical results), and is
 * recorded; replay 1: the recorded dt and times are used (for finite differences at frozen
 * dt).  eta [N*G] and state [nelt*3] (the state after step N) may be NULL. */
int cf_adjoint_forward(cf_adjoint* adj, int32_t replay, double* eta, double* state);

/* dJ/dU^0 [nelt*3] and dJ/dn [nelt] of the last forward run; w_eta [N*G] and w_state
 * [nelt*3] may be NULL (zero), g_state0 and g_manning may be NULL (not returned). */
int cf_adjoint_backward(cf_adjoint* adj, const double* w_eta, const double* w_state, double* g_state0,
                        double* g_manning);

/* The recorded dt and start time of every step [N]; set_dt installs a sequence to replay. */
int cf_adjoint_get_dt(cf_adjoint* adj, double* dt, double* t);
int cf_adjoint_set_dt(cf_adjoint* adj, const double* dt, const double* t);
/* Linearization of the WAF limiter (iflux 3): mode 0 (default) differentiates everything, the
 * exact derivative of the step along the branches the forward took; mode 1 holds the limiter
 * ratios r = dupw / (dloc + eps) constant.  Over long runs the WAF objective is not
 * differentiable (the limiter jumps when dloc changes sign, superbee also at r = 0.5, 1, 2,
 * and r divides round-off in still water, where its exact derivative ~1/eps overflows).
 * Mode 1 is an approximate gradient for those runs: on a 10,000-triangle flooding case over
 * 2000 steps its tangent stays bounded with the van Albada limiter (ilimiteur 3), while the
 * exact one grows by 1e133; with superbee (ilimiteur 1), whose frozen weights are
 * anti-diffusive, it still grows (1e18 against 1e290).  First-order schemes need neither. */
int cf_adjoint_set_linearization(cf_adjoint* adj, int32_t mode);
int cf_adjoint_sizes(cf_adjoint* adj, int32_t* nsteps, int32_t* checkpoint_interval, int32_t* ngauges,
                     int64_t* device_bytes);

/* Manning zones for calibration on the device.  zone_of_elem [sum of nelt] (member order,
 * reference order within a member) gives every element's zone in 0..nzones-1, or -1 for an
 * element whose n is not a parameter.  cf_zones_set writes zone values (host or device
 * memory) into every zoned element's n; cf_zones_gradient sums the adjoint's last dJ/dn over
 * each zone in a fixed order (deterministic); cf_zones_descend takes the projected gradient
 * step v = min(hi, max(lo, v - lr g)) on the device and writes the new n, so that a
 * calibration loop (forward, backward, gradient, descend) needs no host round trip. */
typedef struct cf_zones cf_zones;
int cf_zones_create(cf_ctx* ctx, const int32_t* zone_of_elem, int32_t nzones, cf_zones** out);
void cf_zones_destroy(cf_zones* z);
int cf_zones_set(cf_zones* z, const double* values);
int cf_zones_get(cf_zones* z, double* values, double* gradient);
int cf_zones_gradient(cf_zones* z, cf_adjoint* adj, double* gradient /* may be NULL */);
int cf_zones_descend(cf_zones* z, double lr, double lo, double hi);

/* ---- stepping without allocation (no counterpart in the reference) --------------------
 *
 * For callers that may not allocate device memory once their time loop runs: a coupled host
 * model whose GPU memory is budgeted among its components at start-up, or a process under a
 * fixed device-memory limit (a CUDA MPS client limit) where an allocation in mid-run could
 * fail and lose the simulation.  cf_step allocates nothing per step either, but on its first
 * call with two or more steps it instantiates a CUDA graph, which takes resources of its own.
 *
 * cf_step_noalloc advances exactly like cf_step (same kernels, bit-identical results), with
 * two differences: it launches the kernels one by one, and the per-edge flux slots that the
 * edge kernel hands to the element kernel live in one fixed array inside the library
 * (CF_NOALLOC_SCRATCH_SLOTS slots of 48 bytes, 16 MiB, held on every GPU that loads the
 * library until the process exits) instead of the context's buffer.  It calls no cudaMalloc,
 * cudaFree or allocating library routine.
 *   - Limit: contexts whose edges need at most CF_NOALLOC_SCRATCH_SLOTS slots (two per edge,
 *     each member's edges rounded up to a multiple of 128): about 116,000 triangles in one
 *     member.  A larger context is rejected with CF_EINVAL, the sizes in cf_last_error, and
 *     nothing is launched.
 *   - Every call looks up the array's address in the current device context (a lookup that
 *     allocates nothing); the first call on a device can load the library's device code there,
 *     so make that first call before any stream capture.
 *   - Every call on a device shares the one array, which keeps the last call's contents; a
 *     call clears the part it uses before its first step.  Calls whose work overlaps on the
 *     GPU (contexts stepped at the same time from several host threads) race on the array:
 *     serialise them.  A call returns after its work has finished, so calls from one host
 *     thread never overlap.
 *   - Kernel timing is not collected (cf_get_timing reports zero times); a member whose
 *     status was already set before the call reports q_in = q_out = 0. */
#define CF_NOALLOC_SCRATCH_SLOTS 349525
int cf_step_noalloc(cf_ctx* ctx, int32_t nsteps, cf_step_info* info);

#ifdef __cplusplus
}
#endif
#endif
