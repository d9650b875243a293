/* CPU oracle for the DG Euler RHS + SSPRK3 step — TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load the libraries built from this directory.  The product path
 * (airfoil-op2-fem_gb300/) never links or calls them.
 *
 * Two implementations export this same C API:
 *   liboracle.so        ("port")      a line-by-line C++ restatement of the
 *                                     reference's user kernels, generic in the
 *                                     polynomial order N (1..6), OpenMP-parallel
 *                                     in the style of OP2's openmp backend;
 *   _ref/libref.so      ("reference") the reference's own kernel headers
 *                                     (the src, src/constants and vortex/src headers)
 *                                     compiled unmodified from the reference tree
 *                                     with the 4-routine CBLAS shim; N=4 only;
 *                                     built only where the reference tree exists.
 * The driver loop both share (oracle/driver.h) follows src/airfoil.cpp:204-334
 * and vortex/src/vortex.cpp:186-306.
 *
 * Data layouts are the reference's: per cell, node-major with the four
 * conserved variables interleaved, q[c*4*Np + node*4 + var]
 * (src/airfoil.cpp:126,171); face arrays [c*3*Nfp + face*Nfp + k]. */
#ifndef DG_ORACLE_H
#define DG_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int N;                  /* polynomial order; Np=(N+1)(N+2)/2, Nfp=N+1 */
  const double *r, *s;    /* Np each */
  const double *Dr, *Ds;  /* Np*Np, row-major */
  const double *Drw, *Dsw;/* Np*Np */
  const double *LIFT;     /* Np*3Nfp */
  const int *FMASK;       /* 3*Nfp */
} orc_ops;

typedef struct {
  double gam, bc_mach, bc_alpha, bc_p, bc_r, bc_u, bc_v, bc_e;
  double vortex_x0, vortex_y0, vortex_beta;
} orc_phys;

typedef struct {
  int n_nodes, n_cells, n_edges, n_bedges;
  const double *coords;   /* 2*n_nodes {x,y} */
  const int *cell2nodes;  /* 3*n_cells, counter-clockwise */
  const int *edge2cells;  /* 2*n_edges */
  const int *edgeNum;     /* 2*n_edges: local face of each side */
  const int *bedge2cell;  /* n_bedges */
  const int *bedgeNum;    /* n_bedges */
  const int *bedge_type;  /* n_bedges: 0 inflow, 1 outflow, 2 wall, 3 characteristic farfield (port only) */
} orc_mesh;

enum { ORC_APP_AIRFOIL = 0, ORC_APP_VORTEX = 1 };
enum { ORC_DT_EVERY_STEP = 0, ORC_DT_FROZEN = 1 };

/* Create an instance; copies the mesh.  NULL on bad input (see orc_last_error). */
void *orc_create(const orc_ops *ops, const orc_phys *phys, const orc_mesh *mesh, int app);
void orc_destroy(void *h);
const char *orc_last_error(void);
const char *orc_kind(void); /* "port" or "reference" */

/* init_grid + set_ic + neighbour_zero + calc_dt (src/airfoil.cpp:204-237).
 * cfl scales dt: dt = (1/dt1) * cfl  (cfl=1 for the airfoil app, 0.1 for vortex.cpp:223-224). */
int orc_init(void *h, double cfl);
/* Copy a dat out / in by its reference name (q, workingQ, rk1, rk2, rk3, exteriorQ,
 * nodeX, nodeY, x, y, xr, yr, xs, ys, rx, ry, sx, sy, nx, ny, fscale). */
int orc_get(void *h, const char *name, double *out);
int orc_set(void *h, const char *name, const double *in);
/* One stage's RHS of workingQ into rk[stage] (get_neighbour_q, get_bedge_q, euler_rhs);
 * t_stage is the boundary time for the vortex app. */
int orc_rhs(void *h, int stage, double t_stage);
/* iters SSPRK3 steps.  dt_mode ORC_DT_EVERY_STEP recomputes dt after every step
 * (src/airfoil.cpp:321-331); ORC_DT_FROZEN keeps it (vortex.cpp:296-305).
 * nthreads<=0 uses all OpenMP threads.  dt_hist (may be NULL) receives the dt of each step. */
int orc_run(void *h, int iters, int dt_mode, int nthreads, double *dt_hist);
double orc_dt(void *h);
double orc_time(void *h);
/* Vortex: per-variable sums of squared nodal errors vs the analytic state at the current time
 * (vortex/src/l2_error.h:3-29). err4 = {rho, rhou, rhov, E}. */
int orc_l2_error(void *h, double *err4);
/* Recompute dt = (1/dt1)*cfl from the current q and fscale (after geometry was replaced with orc_set). */
int orc_refresh_dt(void *h);

/* Scalar advection app (advec/src/advec.cpp): one value per node, q[c*Np + node].
 * adv_init runs init_grid and set_ic and fixes dt; adv_rhs evaluates one stage's right-hand
 * side of workingQ into rk<stage+1>; adv_run takes classical RK4 steps (advec.cpp:202-262).
 * Dats by name: q, workingQ, rk1..rk4, exteriorQ and the geometry dats of orc_get. */
void *adv_create(const orc_ops *ops, const orc_mesh *mesh, double vel_x, double vel_y);
void adv_destroy(void *h);
int adv_init(void *h, double dt);
int adv_get(void *h, const char *name, double *out);
int adv_set(void *h, const char *name, const double *in);
int adv_rhs(void *h, int stage);
int adv_run(void *h, int iters, int nthreads);
double adv_time(void *h);

#ifdef __cplusplus
}
#endif
#endif
