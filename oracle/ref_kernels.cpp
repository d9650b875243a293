/* Oracle "reference" library: the reference's own user kernels and N=4
 * operator tables, compiled unmodified from the reference tree
 * (the src, src/constants and vortex/src headers) with the CBLAS shim of
 * oracle/shim/cblas.h, driven by the shared oracle driver (driver.h).
 * TEST INFRASTRUCTURE ONLY (see dg_oracle.h).  Built by oracle/Makefile
 * into oracle/_ref/ only where the reference tree is present.
 *
 * The airfoil and vortex headers define the same names, so each set is
 * included inside its own namespace; their include guards are reset between
 * the two.  Deviations from the vortex app, all in the driver rather than in
 * the kernels:
 *  - set_workingQ: the airfoil copy is used (vortex/src/set_workingQ.h:6 tests
 *    the stage pointer, not its value);
 *  - calc_dt: the airfoil copy, seeded per cell, reduced with a max
 *    (vortex/src/calc_dt.h:15 seeds from its own first value, so under OP2's
 *    seq backend the "max" is the last cell's);
 *  - l2_error: each cell's sums go into zeroed locals that the driver adds
 *    (vortex/src/l2_error.h:6-9 zero the OP_INC accumulators on every call). */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <iostream>
#include <string>

#include <cblas.h>

#include "driver.h"

namespace refa {
#include "src/constants/constant_r.h"
#include "src/constants/constant_s.h"
#include "src/constants/constant_Dr.h"
#include "src/constants/constant_Ds.h"
#include "src/constants/constant_Drw.h"
#include "src/constants/constant_Dsw.h"
#include "src/constants/constant_LIFT.h"
#include "src/constants/constant_util.h"
#include "src/init_grid.h"
#include "src/euler_rhs.h"
#include "src/get_neighbour_q.h"
#include "src/get_bedge_q.h"
#include "src/set_ic.h"
#include "src/set_workingQ.h"
#include "src/update_Q.h"
#include "src/calc_dt.h"
#include "src/neighbour_zero.h"
}  // namespace refa

#undef __CONSTANTS_R_H
#undef __CONSTANTS_S_H
#undef __CONSTANTS_DR_H
#undef __CONSTANTS_DS_H
#undef __CONSTANTS_DRW_H
#undef __CONSTANTS_DSW_H
#undef __CONSTANTS_LIFT_H
#undef __CONSTANTS_UTIL_H

namespace refv {
#define NUM_SOLUTION_PTS 15
#define NUM_FACE_PTS 5
#define ORDER 4
#include "vortex/src/constants/constant_r.h"
#include "vortex/src/constants/constant_s.h"
#include "vortex/src/constants/constant_Dr.h"
#include "vortex/src/constants/constant_Ds.h"
#include "vortex/src/constants/constant_Drw.h"
#include "vortex/src/constants/constant_Dsw.h"
#include "vortex/src/constants/constant_LIFT.h"
#include "vortex/src/constants/constant_util.h"
#include "vortex/src/euler_rhs.h"
#include "vortex/src/get_bedge_q.h"
#include "vortex/src/set_ic.h"
#include "vortex/src/l2_error.h"
}  // namespace refv

namespace {

struct RefPolicy {
  static constexpr int Np = 15, Nfp = 5;
  static void bind(void *c) {
    const orc_phys *p = (const orc_phys *)c;
    refa::gam = p->gam; refa::bc_mach = p->bc_mach; refa::bc_alpha = p->bc_alpha;
    refa::bc_p = p->bc_p; refa::bc_r = p->bc_r; refa::bc_u = p->bc_u; refa::bc_v = p->bc_v;
    refa::bc_e = p->bc_e;
    refv::gam = p->gam; refv::vortex_x0 = p->vortex_x0; refv::vortex_y0 = p->vortex_y0;
    refv::vortex_beta = p->vortex_beta;
  }
  static void free_ctx(void *c) { delete (orc_phys *)c; }
  static void init_grid(const double *n0, const double *n1, const double *n2, double *nodeX,
                        double *nodeY, double *x, double *y, double *xr, double *yr, double *xs,
                        double *ys, double *rx, double *ry, double *sx, double *sy, double *nx,
                        double *ny, double *fscale) {
    refa::init_grid(n0, n1, n2, nodeX, nodeY, x, y, xr, yr, xs, ys, rx, ry, sx, sy, nx, ny, fscale);
  }
  static void set_ic(double *q, double *W) { refa::set_ic(q, W); }
  static void set_ic_vortex(const double *t, const double *x, const double *y, double *q, double *W) {
    refv::set_ic(t, x, y, q, W);
  }
  static void neighbour_zero(double *e) { refa::neighbour_zero(e); }
  static void calc_dt(const double *q, const double *fscale, double *dt1) { refa::calc_dt(q, fscale, dt1); }
  static void get_neighbour_q(const int *en, const double *xL, const double *yL, const double *xR,
                              const double *yR, const double *qL, const double *qR, double *eL,
                              double *eR) {
    refa::get_neighbour_q(en, xL, yL, xR, yR, qL, qR, eL, eR);
  }
  static void get_bedge_q(const int *ty, const int *bn, const double *nx, const double *ny,
                          const double *q, double *e) {
    refa::get_bedge_q(ty, bn, nx, ny, q, e);
  }
  static void get_bedge_q_vortex(const int *bn, const double *x, const double *y, const double *t,
                                 double *e) {
    refv::get_bedge_q(bn, nullptr, nullptr, nullptr, nullptr, x, y, t, e);
  }
  static void euler_rhs(const double *q, double *e, const double *rx, const double *ry,
                        const double *sx, const double *sy, const double *fs, const double *nx,
                        const double *ny, double *rhs, bool zero_ext) {
    if (zero_ext) refa::euler_rhs(q, e, rx, ry, sx, sy, fs, nx, ny, rhs);
    else refv::euler_rhs(q, e, rx, ry, sx, sy, fs, nx, ny, rhs);
  }
  static void set_workingQ(const double *dt, const int *st, const double *q, const double *k1,
                           const double *k2, double *W) {
    refa::set_workingQ(dt, st, q, k1, k2, W);
  }
  static void update_Q(const double *dt, double *q, const double *k1, const double *k2,
                       const double *k3, double *W) {
    refa::update_Q(dt, q, k1, k2, k3, W);
  }
  static void l2_error(const double *x, const double *y, const double *q, const double *t,
                       double *e0, double *e1, double *e2, double *e3) {
    double a, b, c, d, err[4 * Np];
    refv::l2_error(x, y, q, t, &a, &b, &c, &d, err);
    *e0 += a; *e1 += b; *e2 += c; *e3 += d;
  }
};

}  // namespace

static void *orc_make(const orc_ops *ops, const orc_phys *phys, const orc_mesh *mesh, int app) {
  if (!ops || !phys || !mesh) { orc::g_err = "null argument"; return nullptr; }
  if (ops->N != 4) { orc::g_err = "the reference build is N=4 only"; return nullptr; }
  return new orc::Instance<RefPolicy>(mesh, app, new orc_phys(*phys));
}

ORC_DEFINE_C_API("reference")
