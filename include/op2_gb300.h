/* op2_gb300 — drop-in OP2 surface for the Airfoil-OP2-FEM hot path, on one GB300.
 *
 * An application translated by op2.py (src/airfoil_op.cpp) declares its sets,
 * maps, dats and constants and calls one op_par_loop_<kernel> per loop.  This
 * header declares exactly that surface with OP2's argument meanings, so the
 * application links against libdg_gb300.so in place of an OP2 backend
 * (seq/openmp/cuda).  Every loop runs as a hand-written sm_103a kernel on
 * device copies of the dats; results equal the reference's user kernels
 * bit for bit when given the same constant tables (the kernels keep the
 * reference's operation order and are compiled without FMA contraction).
 *
 * Semantics follow OP2:
 *  - op_decl_dat copies the caller's array to the device; op_fetch_data
 *    copies it back.  Caller arrays are never written otherwise.
 *  - op_arg_gbl OP_READ values are read when the loop is called; OP_MAX
 *    results are written to the caller's variable before the loop returns.
 *  - each loop returns when its kernel has finished (as OP2's CUDA backend
 *    synchronises after every loop), so op_timing_output reports device times.
 *  - errors print a message and exit(1), as OP2 does
 *    (src/cuda/airfoil_kernels.cu:105); op2_gb300_set_exit_on_error(0) makes
 *    them return silently with the message in op2_gb300_last_error().
 *
 * The loop kernels of the airfoil application are provided with the argument
 * lists of src/airfoil.cpp:204-331, those of the vortex application
 * (vortex/src/vortex.cpp:210-318) as C++ overloads and op_par_loop_l2_error, and
 * those of the scalar advection application (advec/src/advec.cpp:191-260) as C++
 * overloads and op_par_loop_advec_rhs.
 *
 * For C++ callers that include the reference's generated declarations
 * (src/airfoil_op.cpp:17-94 declare the loops with C++ linkage unless
 * OPENACC is defined), compile with -DOPENACC or include op_lib_cpp.h. */
#ifndef OP2_GB300_H
#define OP2_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Handles (OP2: op_lib_core.h op_set_core/op_map_core/op_dat_core pointers). */
typedef struct op_set_core *op_set;
typedef struct op_map_core *op_map;
typedef struct op_dat_core *op_dat;

typedef enum { OP_READ = 0, OP_WRITE = 1, OP_RW = 2, OP_INC = 3, OP_MIN = 4, OP_MAX = 5 } op_access;

enum { OP_ARG_DAT = 0, OP_ARG_GBL = 1 };

/* One loop argument, built by op_arg_dat / op_arg_gbl and passed by value. */
typedef struct {
  op_dat dat;        /* OP_ARG_DAT: the dataset */
  op_map map;        /* OP_ID (NULL) for direct access */
  int idx;           /* map column, -1 for direct */
  int dim;           /* values per set element (dat) or count (gbl) */
  int size;          /* bytes per element */
  op_access acc;
  int argtype;       /* OP_ARG_DAT or OP_ARG_GBL */
  char *data;        /* OP_ARG_GBL: the caller's variable */
  const char *type;  /* "double" or "int" */
} op_arg;

#define OP_ID ((op_map)0)
#define OP_GBL ((op_map)0)

/* Runtime (OP2 op_init/op_exit; diags as op_init's third argument). */
void op_init(int argc, char **argv, int diags);
void op_exit(void);

/* Declarations: src/airfoil.cpp:135-201 (the translated form uses op_decl_const2,
 * src/airfoil_op.cpp:144-160). */
op_set op_decl_set(int size, char const *name);
op_map op_decl_map(op_set from, op_set to, int dim, int *imap, char const *name);
op_dat op_decl_dat(op_set set, int dim, char const *type, void *data, char const *name);
void op_decl_const2(char const *name, int dim, char const *type, void *data);

op_arg op_arg_dat(op_dat dat, int idx, op_map map, int dim, char const *type, op_access acc);
op_arg op_arg_gbl(void *data, int dim, char const *type, op_access acc);

void op_fetch_data(op_dat dat, void *data);
int op_get_size(op_set set);
void op_timers(double *cpu, double *wall);
void op_timing_output(void);

/* The loops, with the arities and argument orders of src/airfoil_op.cpp:17-94 and the
 * argument meanings of src/airfoil.cpp:204-331. */
void op_par_loop_init_grid(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                           op_arg a3, op_arg a4, op_arg a5, op_arg a6, op_arg a7, op_arg a8,
                           op_arg a9, op_arg a10, op_arg a11, op_arg a12, op_arg a13,
                           op_arg a14, op_arg a15, op_arg a16, op_arg a17);
void op_par_loop_set_ic(char const *name, op_set set, op_arg a0, op_arg a1);
void op_par_loop_neighbour_zero(char const *name, op_set set, op_arg a0);
void op_par_loop_calc_dt(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2);
void op_par_loop_get_neighbour_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                                 op_arg a3, op_arg a4, op_arg a5, op_arg a6, op_arg a7,
                                 op_arg a8);
void op_par_loop_get_bedge_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                             op_arg a3, op_arg a4, op_arg a5);
void op_par_loop_euler_rhs(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                           op_arg a3, op_arg a4, op_arg a5, op_arg a6, op_arg a7, op_arg a8,
                           op_arg a9);
void op_par_loop_set_workingQ(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                              op_arg a3, op_arg a4, op_arg a5);
void op_par_loop_update_Q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                          op_arg a3, op_arg a4, op_arg a5);
/* vortex/src/vortex.cpp:308-318: l2_error(x, y, q, t, 4 x OP_INC error sums, error dat).  The
 * reference kernel zeroes its accumulators on entry (vortex/src/l2_error.h:6-9); here the
 * per-cell sums are added to the globals, as a device backend's reduction does. */
void op_par_loop_l2_error(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3,
                          op_arg a4, op_arg a5, op_arg a6, op_arg a7, op_arg a8);
/* advec/src/advec.cpp:232-242: advec_rhs(q, exteriorQ, rx, ry, sx, sy, fscale, nx, ny, rk), one
 * value per node; reads the constants velX, velY. */
void op_par_loop_advec_rhs(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3,
                           op_arg a4, op_arg a5, op_arg a6, op_arg a7, op_arg a8, op_arg a9);

/* Extensions (no OP2 counterpart). */
const char *op2_gb300_last_error(void);
void op2_gb300_clear_error(void);
void op2_gb300_set_exit_on_error(int on);
/* Wait for all enqueued loops; 0 or -1 with the CUDA error in op2_gb300_last_error(). */
int op2_gb300_sync(void);
/* Drop every declaration and free device memory (op_exit does the same). */
void op2_gb300_reset(void);
/* The loop of user kernel `kernel` ("euler_rhs", ...) with its arguments in an array: the same
 * call as op_par_loop_<kernel>(name, set, args[0], ..., args[nargs-1]) for bindings that cannot
 * pass structures by value (foreign-function layers). */
void op2_gb300_par_loop(char const *kernel, char const *name, op_set set, int nargs, const op_arg *args);

#ifdef __cplusplus
}
#endif
#ifdef __cplusplus
/* The vortex app's loops that share a name with an airfoil loop but take other arguments
 * (vortex/src/vortex.cpp:210-260), as C++ overloads:
 *   set_ic(t, x, y, q, workingQ)                                    vortex/src/set_ic.h:3-28
 *   get_neighbour_q(edgeNum, n0, n1, nodeX L, nodeY L, nodeX R, nodeY R, W L, W R, ext L, ext R)
 *   get_bedge_q(bedgeNum, n0, n1, nodeX, nodeY, x, y, t, exteriorQ)  vortex/src/get_bedge_q.h:3-40
 * The vortex euler_rhs is op_par_loop_euler_rhs with exteriorQ OP_READ (not zeroed). */
void op_par_loop_set_ic(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4);
void op_par_loop_get_neighbour_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3,
                                 op_arg a4, op_arg a5, op_arg a6, op_arg a7, op_arg a8, op_arg a9, op_arg a10);
void op_par_loop_get_bedge_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4,
                             op_arg a5, op_arg a6, op_arg a7, op_arg a8);
/* The advection app's loops (advec/src/advec.cpp:191-260), one value per node, as C++ overloads:
 *   set_ic(x, y, q, workingQ)                                        advec/src/set_ic.h:3-10
 *   get_neighbour_q: the 11-argument overload above, taken when q has Np values per cell
 *   get_bedge_q(bedgeNum, n0, n1, nodeX, nodeY, x, y, exteriorQ)     advec/src/get_bedge_q.h:3-13
 *   set_workingQ(dt, q, rk, rk_frac, workingQ)                       advec/src/set_workingQ.h:1-6
 *   update_Q(dt, q, rk1, rk2, rk3, rk4, workingQ)                    advec/src/update_Q.h:1-8 */
void op_par_loop_set_ic(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3);
void op_par_loop_get_bedge_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4,
                             op_arg a5, op_arg a6, op_arg a7);
void op_par_loop_set_workingQ(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4);
void op_par_loop_update_Q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4,
                          op_arg a5, op_arg a6);
#endif

#endif
