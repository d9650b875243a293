/* dg_gb300 — native C ABI of the GB300 DG Euler solver (plain fused path).
 *
 * The reference runs its hot path as OP2 loops driven from main()
 * (src/airfoil.cpp:204-334).  This header is the fused, device-resident form
 * of the same computation: a mesh handle (the tables src/load_mesh.cpp
 * produces), a solver handle owning the dats on the GPU, and a step call that
 * advances whole SSPRK3 steps without returning to the host.  The drop-in
 * OP2 surface is in op2_gb300.h.
 *
 * Conventions: every function returns 0 on success or a negative code, with
 * a message in dg_last_error() (thread-local).  Host arrays are plain C
 * arrays in the reference's layouts:
 *   q, workingQ   [n_cells][Np][4] doubles (src/airfoil.cpp:126,171)
 *   maps          row-major int32, 0-based (src/load_mesh.cpp:112-146).
 * Nothing here takes ownership of caller memory. */
#ifndef DG_GB300_H
#define DG_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  DG_OK = 0,
  DG_ERR_ARG = -1,
  DG_ERR_CUDA = -100,
  DG_ERR_NONPHYSICAL = -200, /* a kernel saw a non-positive or non-finite density */
  DG_ERR_TIMEOUT = -300      /* a bounded wait in a batched or element kernel gave up (that step is invalid) */
};

const char *dg_last_error(void);

/* ------------------------------------------------------------------ meshes */
typedef struct dg_mesh_t dg_mesh_t;

/* Cells + coordinates -> edge tables with the conventions of tools/vtk2CGNS.cpp:112-199
 * (counter-clockwise fix, face j = (v_j, v_j+1), edges in sorted-vertex-pair order). */
int dg_mesh_from_cells(int n_nodes, const double *coords, int n_cells, const int *cell2nodes,
                       dg_mesh_t **out);
/* The same tables built on the GPU (orientation fix, radix sort of the half-edges, run
 * detection, scan, scatter), bit-identical to dg_mesh_from_cells; device_ms (may be NULL)
 * receives the device time of the build, host<->device copies excluded. */
int dg_mesh_from_cells_device(int n_nodes, const double *coords, int n_cells, const int *cell2nodes,
                              dg_mesh_t **out, float *device_ms);
/* Tables as src/load_mesh.cpp:36-192 returns them (replaces load_mesh's outputs). */
int dg_mesh_from_tables(int n_nodes, const double *coords, int n_cells, const int *cell2nodes,
                        int n_edges, const int *edge2cells, const int *edgeNum, int n_bedges,
                        const int *bedge2cell, const int *bedgeNum, const int *bedge_type,
                        dg_mesh_t **out);
/* Gmsh legacy VTK (the reference's naca0012.vtk); classify_box=1 applies
 * src/load_mesh.cpp:147-171's boundary typing. */
int dg_mesh_read_vtk(const char *path, int classify_box, dg_mesh_t **out);
/* O-grid around NACA 0012; farfield 0: inflow/outflow by face-midpoint x<0, 1: characteristic. */
int dg_mesh_naca_ogrid(int n_theta, int n_r, double stretch, double radius, int farfield,
                       dg_mesh_t **out);
/* [lo,hi]^2 in n x n squares cut along diagonals drawn from std::mt19937_64(seed). */
int dg_mesh_vortex_square(int n, double lo, double hi, unsigned long long seed, dg_mesh_t **out);
enum { DG_MESH_NODES = 0, DG_MESH_CELLS = 1, DG_MESH_EDGES = 2, DG_MESH_BEDGES = 3 };
int dg_mesh_size(const dg_mesh_t *m, int what);
/* name: coords (double), cell2nodes, edge2nodes, edge2cells, edgeNum, bedge2nodes,
 * bedge2cell, bedgeNum, bedge_type (int). */
int dg_mesh_get(const dg_mesh_t *m, const char *name, void *out);
int dg_mesh_set_bedge_type(dg_mesh_t *m, const int *types);
void dg_mesh_free(dg_mesh_t *m);

/* Nodal operators of order N (1..6) on the reference triangle, the tables of
 * src/constants/constant_*.h for N=4.  Any output pointer may be NULL. */
int dg_operators(int N, double *r, double *s, double *Dr, double *Ds, double *Drw, double *Dsw,
                 double *LIFT, int *FMASK);

/* ------------------------------------------------------------------ solver */
typedef struct {
  int N;          /* polynomial order 1..6 */
  int app;        /* 0: airfoil boundary types (src/get_bedge_q.h); 1: isentropic vortex */
  int dt_mode;    /* 0: dt recomputed after every step (src/airfoil.cpp:321-331); 1: frozen */
  double cfl;     /* dt = (1/dt1) * cfl; 1.0 in src/airfoil.cpp:237, 0.1 in vortex.cpp:223 */
  double gam, mach, alpha_deg, p_inf, rho_inf; /* freestream (src/airfoil.cpp:79-99) */
  double vortex_x0, vortex_y0, vortex_beta;    /* vortex/src/constants/constant_util.h:6-8 */
} dg_config_t;

typedef struct dg_solver_t dg_solver_t;

int dg_solver_create(const dg_config_t *cfg, const dg_mesh_t *mesh, dg_solver_t **out);
/* set_ic + calc_dt (src/airfoil.cpp:224-237). */
int dg_solver_init(dg_solver_t *s);
/* Enqueue nsteps SSPRK3 steps (src/airfoil.cpp:252-334) on the solver's stream; returns
 * without waiting.  Each step is one launch of a captured CUDA graph (built on the first call):
 * the face and element kernels of the three stages over P ranges of cells (dg_set_step_parts),
 * each range's launches depending only on the launches whose cells they share, so that ranges
 * in different stages overlap on the GPU; bitwise the same result for every P. */
int dg_solver_run(dg_solver_t *s, int nsteps);
/* Kernel launches of one dg_solver_run step for this solver (7 with one range). */
int dg_solver_kernels_per_step(dg_solver_t *s);
/* Wait for the solver's stream; DG_ERR_NONPHYSICAL if the density guard fired. */
int dg_solver_sync(dg_solver_t *s);
/* Copy a dat to/from the host: "q", "workingQ" ([K][Np][4]), "geo" ([K][16], get only). */
int dg_solver_get(dg_solver_t *s, const char *name, double *host);
int dg_solver_set(dg_solver_t *s, const char *name, const double *host);
/* One right-hand side L(W) (get_neighbour_q + get_bedge_q + euler_rhs of one stage) for the
 * given stage state; the vortex boundary uses the current time. */
int dg_solver_rhs(dg_solver_t *s, const double *host_W, double *host_rhs);
int dg_solver_time(dg_solver_t *s, double *t, double *dt, unsigned long long *step);
/* Vortex: per-variable sums of squared nodal errors vs the analytic state (vortex/src/l2_error.h). */
int dg_solver_l2_error(dg_solver_t *s, double *err4);
/* Record the dt of each of the next max_steps steps; read them with dg_solver_dt_history. */
int dg_solver_record_dt(dg_solver_t *s, int max_steps);
int dg_solver_dt_history(dg_solver_t *s, double *out, int n);
/* End-to-end call with host buffers: q_in -> device, nsteps steps, device -> q_out.
 * Either pointer may be NULL to skip that copy.  Synchronous.  With pinned buffers on a mesh that
 * runs the step graph over cell ranges, a one-step call is one captured graph: each range's q is
 * uploaded on its own stream before the range's first face launch, and each range's new q is
 * downloaded as soon as its last element launch is done, while the other ranges compute; otherwise
 * the last step's final element kernel runs as four ranges of cells and each range is copied
 * back while the later ones compute.  Results equal dg_solver_run's bit for bit. */
int dg_solver_step_host(dg_solver_t *s, const double *q_in, int nsteps, double *q_out);
void *dg_solver_device_ptr(dg_solver_t *s, const char *name);
void *dg_solver_stream(dg_solver_t *s);
/* Launch one step as separate kernels with an event between each, wait, and write the seven
 * kernel durations (face, elem x 3 stages, finalize) in milliseconds. */
int dg_solver_step_timed(dg_solver_t *s, float *ms7);
/* Per mesh vertex rho, u, v, p (host arrays of n_nodes) sampled as src/save_solution.cpp:13-46
 * does (the vertex nodes of the last cell containing the vertex), and the same fields written as
 * a legacy-VTK file (the reference writes them to CGNS, :48-98). */
int dg_solver_vertex_fields(dg_solver_t *s, const dg_mesh_t *mesh, double *rho, double *u, double *v, double *p);
int dg_solver_write_vtk(dg_solver_t *s, const dg_mesh_t *mesh, const char *path);
/* ------------------------------------------------------------------ scalar advection app
 * advec/src/advec.cpp: one scalar per node (q [n_cells][Np] doubles), flux (vx q, vy q) with the
 * Lax-Friedrichs face flux of advec/src/advec_rhs.h:36-63, the constant ghost value 4.5e-5 on
 * every boundary face (advec/src/get_bedge_q.h), the Gaussian pulse of advec/src/set_ic.h and
 * classical RK4 with a fixed dt (advec.cpp:197-262; -vx/-vy/-iter there are vel_x, vel_y and the
 * step count here).  Same operators, geometry and edge records as the Euler solver; order 1..6. */
typedef struct dg_advec_t dg_advec_t;
int dg_advec_create(const dg_mesh_t *mesh, int order, double vel_x, double vel_y, double dt, dg_advec_t **out);
int dg_advec_init(dg_advec_t *a);                 /* set_ic, t = 0 */
int dg_advec_run(dg_advec_t *a, int nsteps);      /* enqueue nsteps RK4 steps (a CUDA graph) */
int dg_advec_sync(dg_advec_t *a);
int dg_advec_get(dg_advec_t *a, const char *name, double *host);        /* q, workingQ, geo */
int dg_advec_set(dg_advec_t *a, const char *name, const double *host);  /* q, workingQ */
/* One right-hand side of W (advec_rhs after the face loops); overwrites workingQ. */
int dg_advec_rhs(dg_advec_t *a, const double *W, double *rhs);
int dg_advec_time(dg_advec_t *a, double *t, unsigned long long *steps);
/* One step as separate launches with per-kernel times (face, element) x 4 stages, in ms. */
int dg_advec_step_timed(dg_advec_t *a, float *ms8);
/* q per mesh vertex as advec/src/save_solution.cpp:13-52 samples it, and as a legacy-VTK file. */
int dg_advec_vertex_values(dg_advec_t *a, const dg_mesh_t *mesh, double *out);
int dg_advec_write_vtk(dg_advec_t *a, const dg_mesh_t *mesh, const char *path);
void *dg_advec_stream(dg_advec_t *a);
void dg_advec_free(dg_advec_t *a);

/* The writer alone (host only): per-vertex fields given by the caller. */
int dg_mesh_write_vtk(const dg_mesh_t *mesh, const char *path, const double *rho, const double *u,
                      const double *v, const double *p);
void dg_solver_free(dg_solver_t *s);

/* ------------------------------------------------------------------ batched instances
 * Many instances (airfoil or vortex, any size, order 1..6, Mach, alpha) advanced together:
 * each RK stage of the whole batch is one persistent kernel (cooperative launch: face phase,
 * grid barrier, element phase over all instances' tiles), a step is three of them plus one
 * finalize, captured in a CUDA graph.  Each instance computes exactly what dg_solver would.
 * A grid barrier wait is bounded (about 2 s); if one gives up, dg_batch_sync reports it. */
typedef struct dg_batch_t dg_batch_t;
int dg_batch_create(int n, const dg_config_t *cfgs, const dg_mesh_t *const *meshes, dg_batch_t **out);
int dg_batch_init(dg_batch_t *b);
/* Time every launch shape over `steps` steps, keep the fastest; the instances' state is
 * restored afterwards.  Shapes: the persistent cooperative kernel (variants 0..2: 512 threads x
 * 1 or 2 resident blocks, 1024 x 1) with face tiles of 1, 2 or 4 blocks' worth of nodes, and
 * grouped launches (variant 99: per stage one face launch over all instances and one element
 * launch per order) with face tiles of 64, 128 or 256 nodes. */
int dg_batch_autotune(dg_batch_t *b, int steps, double *best_ms_per_step);
int dg_batch_run(dg_batch_t *b, int nsteps);
int dg_batch_sync(dg_batch_t *b);
int dg_batch_get(dg_batch_t *b, int instance, const char *name, double *host);
int dg_batch_time(dg_batch_t *b, int instance, double *t, double *dt, unsigned long long *step);
int dg_batch_shape(dg_batch_t *b, int *variant, int *block, int *face_tile, int *grid);
/* Host-side fault injection for tests: record a grid-barrier timeout as a kernel whose bounded
 * wait gave up would; the next dg_batch_sync reports DG_ERR_TIMEOUT and clears it. */
int dg_batch_inject_barrier_timeout(dg_batch_t *b);
/* The persistent kernel's grid barrier waits at most `cycles` SM clocks (0: the default, 2^32,
 * about 2 s at 2 GHz) before recording a timeout and returning; applies to launches from now on. */
int dg_batch_set_barrier_limit(dg_batch_t *b, unsigned long long cycles);
/* Device-side check of that bounded wait: one cooperative launch (one 64-thread block per SM) that
 * runs only the grid barrier, with block 0 held back before it by a bounded delay of hold_cycles
 * SM clocks (at most 2^40).  With hold_cycles above the limit the other blocks' waits run out and
 * the next dg_batch_sync reports DG_ERR_TIMEOUT; with 0 the barrier completes normally.  No wait is
 * unbounded either way. */
int dg_batch_barrier_check(dg_batch_t *b, unsigned long long hold_cycles);
/* Use one launch shape (variant as above) without timing. */
int dg_batch_use_shape(dg_batch_t *b, int variant, int face_tile);
/* The shapes the last dg_batch_autotune timed: with i < 0 returns their count; else shape i's
 * variant (99: grouped launches), face tile and ms per step, and the count. */
int dg_batch_tried(dg_batch_t *b, int i, int *variant, int *face_tile, double *ms_per_step);
int dg_batch_uses_graph(dg_batch_t *b);
void *dg_batch_stream(dg_batch_t *b);
void dg_batch_free(dg_batch_t *b);
const char *dg_batch_last_error(void);
/* The batched sweep's instances: alpha ~ U[-4,8] deg, Mach ~ U[0.3,0.6] from
 * std::mt19937_64(seed); O-grids 128x32 .. 384x96 linearly; order 3 even / 4 odd. */
int dg_sweep_config(int n, unsigned long long seed, int *n_theta, int *n_r, int *order, double *alpha_deg,
                    double *mach);

/* ------------------------------------------------------------------ adjoint (lift gradient)
 * J = mean over the last navg of nsteps SSPRK3 steps of the lift coefficient
 *   C_l = sum over wall face nodes of w_k sJ p (n . (-sin a, cos a)) / (1/2 rho |V|^2 c), c = 1
 * (airfoil boundary types 0, 1, 2).  dg_adjoint_forward runs the solver from its initial state
 * recording the dt sequence and checkpointing q every checkpoint_every steps;
 * dg_adjoint_backward runs the discrete adjoint (hand-written reverse kernels of the Roe flux,
 * boundary states, volume and lift operators; SSPRK3 reversed segment by segment with
 * recomputation from the checkpoints) and returns grad_J * dJ/dalpha (alpha in degrees) and
 * grad_J * dJ/dq0 ([K][Np][4], may be NULL), with the dt sequence frozen.
 * dg_adjoint_evaluate gives J for another alpha / initial state with that frozen sequence (the
 * function backward differentiates), for finite-difference checks.
 *
 * Isentropic vortex (cfg->app = 1; navg unused but must be in 1..nsteps): J is the final-time sum
 * over nodes and variables of the squared error against the analytic vortex (the four sums of
 * vortex/src/l2_error.h:3-29 added) and the scalar parameter is the vortex strength beta: the
 * grad_alpha / alpha_deg / alpha_part arguments then carry dJ/dbeta, beta and v . dL/dbeta.
 * The dt sequence (cfg->dt_mode 1: frozen at the initial state's value) is held fixed. */
typedef struct dg_adjoint_t dg_adjoint_t;
int dg_adjoint_create(const dg_config_t *cfg, const dg_mesh_t *mesh, int nsteps, int navg, int checkpoint_every,
                      dg_adjoint_t **out);
int dg_adjoint_forward(dg_adjoint_t *a, double *J);
int dg_adjoint_backward(dg_adjoint_t *a, double grad_J, double *grad_alpha, double *grad_q0);
int dg_adjoint_evaluate(dg_adjoint_t *a, double alpha_deg, const double *q0, double *J);
int dg_adjoint_dt_sequence(dg_adjoint_t *a, double *out, int n);
/* Tangent-linear FP64 run (forward mode, independent of the reverse kernels), after
 * dg_adjoint_forward: dJ = dJ/dparam * d_param + dJ/dq0 . dq0 (dq0 [K][Np][4] or NULL) along the
 * same frozen dt sequence; equals the adjoint's gradient applied to that direction. */
int dg_adjoint_tangent(dg_adjoint_t *a, double d_param, const double *dq0, double *dJ);
/* (dL/dW at W)^T v and v . dL/dalpha of one right-hand side (host arrays [K][Np][4]). */
int dg_adjoint_rhs_vjp(dg_adjoint_t *a, const double *W, const double *v, double *out, double *alpha_part);
/* Many instances at once (for example 16 vortex strengths on one mesh): every instance's
 * forward, or backward, runs concurrently on its own stream from its own host thread; one call
 * returns all J / all gradients (grad_q0 may be NULL, else n pointers, each may be NULL). */
int dg_adjoint_batch_forward(dg_adjoint_t *const *a, int n, double *J);
int dg_adjoint_batch_backward(dg_adjoint_t *const *a, int n, double grad_J, double *grad_param, double *const *grad_q0);
void *dg_adjoint_stream(dg_adjoint_t *a);
void dg_adjoint_free(dg_adjoint_t *a);
const char *dg_adjoint_last_error(void);

/* ------------------------------------------------------------------ allocation-free RHS
 * No counterpart in the reference.  For callers that cannot call cudaMalloc — the device
 * memory belongs to another runtime's pool or budget, or the call may happen while another
 * library is capturing a CUDA graph: one right-hand side L(W) of the airfoil case
 * (app 0 boundary types), as dg_solver_rhs computes it, that allocates nothing.  Inputs and
 * output are device arrays the caller owns, in dg_solver's layouts:
 *   W, rhs  [n_cells][Np][4] doubles;  geo [n_cells][16] (rx, ry, sx, sy, then nx, ny, fscale
 *   of faces 0..2; dg_solver_get(s, "geo") gives it);  edges [n_edges][4] ints
 *   {cL, cR, fL | fR << 2 | reverse << 4, 0};  bedges [n_bedges][4] ints {cell, face, type, 0};
 *   all 16-byte aligned; every cell face covered by exactly one edge or boundary edge.
 * The face-flux scratch is a file-scope device array of 32 MiB that every GPU loading the
 * library holds until the process exits: meshes needing more (n_cells * 3 * (N+1) * 32 bytes)
 * are rejected with DG_ERR_ARG, and so are counts with 2 n_edges + n_bedges != 3 n_cells.  The
 * first call on each device, with that device current, looks up the scratch's device address
 * there and uploads the operator tables of every order 1..6 (synchronous copies); make that
 * first call on each device before any stream capture.  Later calls on that device, of any
 * order, make no synchronous call.  The set-up is guarded by a lock, so host threads may make
 * their first calls concurrently.  All calls on a device share its scratch (cleared at the start
 * of each call): calls that overlap on the GPU race.  stream may be NULL (the legacy default
 * stream).
 * Errors: dg_rhs_noalloc_error(). */
int dg_rhs_noalloc(const dg_config_t *cfg, int n_cells, int n_edges, int n_bedges, const double *W,
                   const double *geo, const int *edges, const int *bedges, double *rhs, void *stream);
const char *dg_rhs_noalloc_error(void);

/* ------------------------------------------------------------------ diagnostics
 * The device's boundary ghost state (src/get_bedge_q.h types 0 inflow, 1 outflow, 2 wall, and 3
 * the characteristic farfield, which has no reference counterpart) for n interior states qi
 * [n][4] and unit normals nrm [n][2], host arrays in and out (qb [n][4]); the freestream comes
 * from cfg (gam, mach, alpha_deg, p_inf, rho_inf).  The same device function the face kernels
 * call, so tests can check its physics directly.  Errors: dg_boundary_state_error(). */
int dg_boundary_state(const dg_config_t *cfg, int type, int n, const double *qi, const double *nrm, double *qb);
const char *dg_boundary_state_error(void);

/* Set-up bookkeeping queries (host only, no device call): 1 if order N's operator tables (and its
 * kernels' shared-memory limits) are uploaded to device `device`, 0 if not, -1 out of range.
 * The tables are per device; every solver, batch, adjoint or allocation-free call uploads them
 * once per (device, order). */
int dg_order_tables_loaded(int device, int N);
/* 1 if dg_rhs_noalloc has set itself up on device `device`, 0 if not, -1 out of range. */
int dg_rhs_noalloc_ready(int device);
/* Host-only check of the once-per-(device, slot) table behind both: `threads` host threads race
 * through every pair of `devices` devices x 7 slots three times, with a fake upload that fails on
 * its first attempt for every third pair.  uploads[d * 7 + s] receives the successful uploads
 * of each pair (1 when the bookkeeping is right), attempts[] every attempt (2 for the pairs
 * that failed once).  0 on success. */
int dg_once_table_selftest(int threads, int devices, int *uploads, int *attempts);

/* ------------------------------------------------------------------ measurement helpers */
void *dg_host_alloc(size_t bytes); /* pinned */
void dg_host_free(void *p);
void *dg_event_create(void);
int dg_event_record(void *ev, void *stream);
float dg_event_elapsed_ms(void *start, void *stop);
void dg_event_destroy(void *ev);
int dg_stream_sync(void *stream);
/* Overwrite a device buffer larger than L2 on the stream (cache flush between timed steps). */
int dg_l2_flush(void *stream);
/* Measured FP64 DFMA throughput of this GPU, GFLOP/s (FMA = 2 flops). */
double dg_fp64_peak_gflops(void);
/* Measured FP64 tensor-core (mma.sync m8n8k4 f64) throughput of this GPU, GFLOP/s. */
double dg_fp64_mma_peak_gflops(void);
/* Measured fp16 tensor-core throughput of this GPU for mma.sync.m16n8k16 with FP32 accumulation
 * (the element kernel's contraction instruction), GFLOP/s. */
double dg_f16_mma_peak_gflops(void);
/* Number of kernels one dg_solver_run step launches. */
int dg_kernels_per_step(void);
/* Element-kernel form for launches and graphs built from now on: 3 (default) the dense rows
 * [Drw | Dsw | -LIFT] on the tensor cores as an exact integer product at orders N = 1, 2 and
 * form 2 at the other orders; 2 the even/odd split of those rows with its contraction on the
 * tensor cores at orders N = 3, 4, 5 and in FP64 at the other orders; 1 the even/odd split in
 * FP64; 0 dense FP64 rows.  All compute the same right-hand side to rounding (the tensor-core
 * contraction is the correctly rounded dot product of the 56-bit truncated inputs). */
void dg_set_elem_variant(int variant);
/* The current element-kernel form. */
int dg_elem_variant(void);
/* How the tensor-core element form runs at order 3, for launches and graphs built from now
 * on: 0 (default) one block per 32-cell tile; 1 a warp-specialised persistent kernel, one block per SM walking a contiguous range
 * of 32-cell tiles, node warps staging the next tile and combining the previous one while
 * contraction warps run the current tile's tensor-core product (triple-buffered shared memory,
 * bounded mbarrier waits: a wait that runs out makes dg_solver_sync report DG_ERR_TIMEOUT);
 * 2 the same with a launch over a range of tiles taking that range's share of the SMs.  All
 * compute the same bits; the persistent kernel measured slower on the benchmark mesh. */
void dg_set_elem_ws(int mode);
int dg_elem_ws(void);
/* Resident blocks per SM the order-3 tensor-core element kernel (one block per tile) is compiled
 * for: 3 (default; 64 registers) or 2 (more registers, and room for face-kernel blocks of other
 * cell ranges beside it in the step graph); other values select 3.  Same bits either way. */
void dg_set_elem_blocks_per_sm(int blocks);
int dg_elem_blocks_per_sm(void);
/* Host-only (no GPU needed): the tables of the tensor-core contraction of order N (3..5).
 * dims[4] receives NUe, NUo, NRe, NRo; S (NRe*NUe + NRo*NUo doubles, may be NULL) the even then
 * odd operator blocks row-major; fexp (2 x 32 ints, may be NULL) each row's biased binary
 * exponent F; digits (2 x 7 x 32 x 32 ints, may be NULL) [parity][digit s][slot k][row n], with
 * S[n][k] = sum_s digit * 256^(6-s) * 2^(F-1023-55) up to the cut bits below 2^(F-1023-55). */
int dg_tc_operator_digits(int N, int *dims, double *S, int *fexp, int *digits);
/* Host-only (no GPU needed): the final rounding of the tensor-core contraction, the same code the
 * device runs.  *out = (th * 2^32 + tl) * 2^sc rounded to the nearest double, ties to even, for
 * |th| < 2^41, |tl| < 2^49 (the joined level sums) and -1022 <= sc <= 900; DG_ERR_ARG outside. */
int dg_tc_round(long long th, long long tl, int sc, double *out);
/* Cell ranges of the step graph for solvers whose graph is built from now on: 0 automatic (the
 * default: ranges of at least 128 tiles of 32 cells, at most 4), 1 a single range (the seven
 * launches as one chain), 2..32 that many ranges (fewer if the mesh has fewer tiles). */
void dg_set_step_parts(int parts);
int dg_step_parts(void);
/* Steps in one launch of that graph (1..8, default 8; other values select 8), for graphs built from
 * now on: the next step's first face launches of a range then wait only for the element launches
 * whose cells they read (its first element launches for the new dt), so they overlap the previous
 * step's last element launches.  dg_solver_run launches it as often as it fits, then one-step
 * graphs.  Same bits. */
void dg_set_steps_per_graph(int steps);
int dg_steps_per_graph(void);
/* Tuning of that graph (more than one range) for graphs built from now on: bit 0 launches its
 * kernels without programmatic dependent launch, bit 1 gives range p's launches a scheduling
 * priority falling with p (earlier ranges scheduled first), bit 2 gives element launches a higher
 * priority than face launches (when bit 1 is clear).  1 by default.  Results are bitwise the
 * same. */
void dg_set_step_graph_flags(int flags);
int dg_step_graph_flags(void);
/* Threads per face-kernel block of the plain path (32..256, multiple of 32; default 64). */
void dg_set_face_block(int threads);
/* 64-thread face blocks compiled for at most 64 registers (1; one fits beside three order-3 element
 * blocks on an SM) or without a bound (0, default).  Same bits. */
void dg_set_face_regs64(int on);
int dg_face_regs64(void);
/* Launch the plain path's face and element kernels with programmatic dependent launch (1, the
 * default: each may start while its predecessor drains) or in plain stream order (0).  Both give
 * bit-identical results; applies to launches and graphs built from now on. */
void dg_set_pdl(int on);

#ifdef __cplusplus
}
#endif
#endif
