/*
 * cf_oracle.h -- CPU restatement of the CuteFlow explicit finite-volume St-Venant step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness checker for the GPU
 * implementation in cuteflow_gb300/.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py may load it.  The product never links,
 * calls or falls back to it.
 *
 * The structs below are laid out field-for-field like cf_mesh / cf_params in
 * include/cuteflow_gb300.h so that one ctypes description serves both libraries.
 * They are declared here independently: the oracle shares no source with the product.
 */
#ifndef CF_ORACLE_H
#define CF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAX_IO 20

typedef struct orc_mesh {
  int32_t nnt;                     /* nodes (nnt) */
  int32_t nelt;                    /* triangles (nelt) */
  const double* x;                 /* coordonnees(:,1) */
  const double* y;                 /* coordonnees(:,2) */
  const double* z;                 /* coordonnees(:,3), bed elevation at nodes */
  const int32_t* tri;              /* 3*nelt, 1-based: tri[3*k+j] = connectivite(k+1, j+1) */
  const double* manning_elt;       /* nelt (manning_nelt), may be NULL when overridden */
  const int32_t* ndinput;          /* ndi inflow nodes (1-based) */
  const int32_t* numero_ndinput;   /* ndi inlet numbers (1-based) */
  const int32_t* ndoutput;         /* ndo outflow nodes */
  const int32_t* numero_ndoutput;  /* ndo outlet numbers */
  const int32_t* ndwall;           /* ndw wall nodes */
  int32_t ndi, ndo, ndw;
  int32_t nombre_entrees, nombre_sorties;
  int32_t pad_;
} orc_mesh;

typedef struct orc_params {
  double gp;
  double tolisec;
  double cfl;
  double tol;                      /* friction velocity floor (tol) */
  double override_manning;
  double constant_dt;
  double debitglob[ORC_MAX_IO];
  double h_sortie[ORC_MAX_IO];
  double debitglob_start[ORC_MAX_IO];
  double ramp_time;
  int32_t iflux;
  int32_t ilimiteur;
  int32_t friction;
  int32_t fricimplic;
  int32_t is_override_manning;
  int32_t is_dt_constant;
  int32_t inlet;                   /* 1 transm, 2 inflow, 3 phys_inflow */
  int32_t outlet;                  /* 1 fixedheight, 2 transm */
  int32_t flux_mode;               /* 0: per (cell, edge) like the reference; 1: once per edge */
  int32_t reorder;                 /* ignored by the oracle */
  int32_t pad_;
  double tol_reg_perm;             /* steady-state stop; 0 disables */
  int32_t steady_count;            /* consecutive qualifying steps before the stop (1000) */
  int32_t dt_reset_nelt;           /* element count selecting the dt sentinel (0: the mesh's) */
  double long_entree[ORC_MAX_IO];  /* inlet lengths (0: measured on the mesh) */
} orc_params;

typedef struct orc_ic {
  double x1eqbar, x2eqbar, y1eqbar, y2eqbar;
  double h_amont, u_amont, v_amont, h_aval, u_aval, v_aval;
  double xplan, yplan, zplan, xpoint, ypoint, zpoint;
  int32_t eqlin_barrage;
  int32_t plan;
} orc_ic;

/* Mesh preprocessing in the reference's semantics.  Any output pointer may be NULL.
 * boundary: nelt*3*2 int32, [(k*3+j)*2 + 0] = neighbour (1-based) or -1/-2/-3,
 *           [(k*3+j)*2 + 1] = inlet/outlet number (cell id for other edges),
 *           with unmatched edges already turned into walls (-3). */
int orc_setup(const orc_mesh* m, int32_t* boundary, double* area, double* zm,
              double* cotemin, double* xc, double* yc);

/* set_initial_condition (dam line / plane) into U0 (3*nelt, element-major h,hu,hv). */
int orc_initial_condition(const orc_mesh* m, const orc_params* p, const orc_ic* ic, double* U0);

/* Run nsteps of the time loop from U0 at time t0.
 *   U_out    : 3*nelt, state after the last step
 *   dt_hist  : nsteps+1 or NULL; dt_hist[0] = dt(U0), dt_hist[n] = dt computed after step n
 *   dt_replay: nsteps or NULL; when given, step n uses dt_replay[n-1] instead of the CFL dt
 *   t_out    : time after the last step (t0 + sum of the dt used)
 *   q_out    : 2 or NULL; inflow and outflow discharge of the last step
 *   nthreads : OpenMP threads (<=0: library default)
 *   loop_seconds: NULL or the wall time of the time loop alone (setup excluded)
 *   steps_out: NULL or the number of steps taken
 * Returns 0, 1 when the steady-state test stopped the run (tol_reg_perm > 0), or a negative
 * code: -1 bad input, -2 dt out of the reference's sane range. */
int orc_run(const orc_mesh* m, const orc_params* p, const double* U0, double t0, int32_t nsteps,
            double* U_out, double* dt_hist, const double* dt_replay, double* t_out, double* q_out,
            int32_t nthreads, double* loop_seconds, int32_t* steps_out);

/* flux*len of edge tj (0..2) of element gi (0-based) for state U (3 doubles out). */
int orc_edge_flux(const orc_mesh* m, const orc_params* p, const double* U, double dt, double t,
                  int32_t gi, int32_t tj, double* fl_out);

/* flux*len of every (element, edge): fl_out[(gi*3+tj)*3+c]. */
int orc_all_edge_fluxes(const orc_mesh* m, const orc_params* p, const double* U, double dt,
                        double t, double* fl_out);

/* Number of OpenMP threads the library would use by default. */
/* x^(-1/3) as the friction term evaluates it, elementwise. */
void orc_rcbrt(const double* x, double* y, int64_t n);
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
