/* Oracle "reference" library, scalar advection part: the advection app's own
 * user kernels and N=4 operator tables (the advec/src and advec/src/constants
 * headers), compiled unmodified from the reference tree with the CBLAS shim
 * and driven by advec_driver.h — TEST INFRASTRUCTURE ONLY (see dg_oracle.h).
 * Linked into _ref/libref.so beside ref_kernels.cpp. */
#include <algorithm>
#include <cmath>
#include <cstring>
#include <iostream>
#include <string>

#include <cblas.h>

#include "advec_driver.h"

namespace refadv {
#define NUM_SOLUTION_PTS 15
#define NUM_FACE_PTS 5
#define ORDER 4
#include "advec/src/constants/constant_r.h"
#include "advec/src/constants/constant_s.h"
#include "advec/src/constants/constant_Dr.h"
#include "advec/src/constants/constant_Ds.h"
#include "advec/src/constants/constant_Drw.h"
#include "advec/src/constants/constant_Dsw.h"
#include "advec/src/constants/constant_LIFT.h"
#include "advec/src/constants/constant_util.h"
#include "advec/src/init_grid.h"
#include "advec/src/advec_rhs.h"
#include "advec/src/get_neighbour_q.h"
#include "advec/src/get_bedge_q.h"
#include "advec/src/set_ic.h"
#include "advec/src/set_workingQ.h"
#include "advec/src/update_Q.h"
#include "advec/src/neighbour_zero.h"
}  // namespace refadv

namespace {

struct AdvRefPolicy {
  static constexpr int Np = 15, Nfp = 5;
  static void bind(void *c) {
    const double *v = (const double *)c;
    refadv::velX = v[0];
    refadv::velY = v[1];
  }
  static void free_ctx(void *c) { delete[] (double *)c; }
  static void init_grid(const double *n0, const double *n1, const double *n2, double *nodeX,
                        double *nodeY, double *x, double *y, double *xr, double *yr, double *xs,
                        double *ys, double *rx, double *ry, double *sx, double *sy, double *nx,
                        double *ny, double *fscale) {
    refadv::init_grid(n0, n1, n2, nodeX, nodeY, x, y, xr, yr, xs, ys, rx, ry, sx, sy, nx, ny, fscale);
  }
  static void adv_set_ic(const double *x, const double *y, double *q, double *W) { refadv::set_ic(x, y, q, W); }
  static void adv_neighbour_zero(double *e) { refadv::neighbour_zero(e); }
  static void adv_get_neighbour_q(const int *en, const double *xL, const double *yL, const double *xR,
                                  const double *yR, const double *qL, const double *qR, double *eL,
                                  double *eR) {
    refadv::get_neighbour_q(en, nullptr, nullptr, xL, yL, xR, yR, qL, qR, eL, eR);
  }
  static void adv_get_bedge_q(const int *bn, double *e) {
    refadv::get_bedge_q(bn, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, e);
  }
  static void advec_rhs(const double *q, const double *e, const double *rx, const double *ry,
                        const double *sx, const double *sy, const double *fs, const double *nx,
                        const double *ny, double *rhs) {
    refadv::advec_rhs(q, e, rx, ry, sx, sy, fs, nx, ny, rhs);
  }
  static void adv_set_workingQ(const double *dt, const double *q, const double *rk, const double *f, double *W) {
    refadv::set_workingQ(dt, q, rk, f, W);
  }
  static void adv_update_Q(const double *dt, double *q, const double *k1, const double *k2, const double *k3,
                           const double *k4, double *W) {
    refadv::update_Q(dt, q, k1, k2, k3, k4, W);
  }
};

}  // namespace

static void *adv_make(const orc_ops *ops, const orc_mesh *mesh, double vel_x, double vel_y) {
  if (!ops || !mesh) { orc::g_err = "null argument"; return nullptr; }
  if (ops->N != 4) { orc::g_err = "the reference build is N=4 only"; return nullptr; }
  return new orc::AdvInstance<AdvRefPolicy>(mesh, new double[2]{vel_x, vel_y});
}

ADV_DEFINE_C_API
