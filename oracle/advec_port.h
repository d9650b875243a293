/* Oracle restatement of the scalar advection app's OP2 user kernels
 * (the advec/src headers), generic in the order N — TEST INFRASTRUCTURE ONLY (see
 * dg_oracle.h).  Same rules as port_kernels.h: the reference's argument
 * lists, layouts and floating-point operation order, cblas calls as
 * ascending-index loops; Np and Nfp replace the hard-coded 15 and 5.
 * init_grid is the airfoil app's (advec/src/init_grid.h differs from
 * src/init_grid.h only in spelling 15 as NUM_SOLUTION_PTS). */
#ifndef ORACLE_ADVEC_PORT_H
#define ORACLE_ADVEC_PORT_H

#include "port_kernels.h"

namespace port {

template <int N>
struct A : K<N> {
  using K<N>::Np;
  using K<N>::Nfp;

  /* Names carry an adv_ prefix where the airfoil app has a kernel of the same name. */

  /* advec/src/set_ic.h:3-10: a Gaussian pulse centred on (0.5, 0.5) */
  static void adv_set_ic(const double *x, const double *y, double *q, double *workingQ) {
    for (int i = 0; i < Np; i++) {
      q[i] = std::exp(-40.0 * (x[i] - 0.5) * (x[i] - 0.5)) * std::exp(-40.0 * (y[i] - 0.5) * (y[i] - 0.5));
      workingQ[i] = q[i];
    }
  }

  /* advec/src/neighbour_zero.h:1-5 */
  static void adv_neighbour_zero(double *exQ) {
    for (int i = 0; i < 3 * Nfp; i++) exQ[i] = 0.0;
  }

  /* advec/src/get_neighbour_q.h:3-87: the traces of each side, one value per face node; the
   * far side is read backwards when vertex edgeL of L is not vertex edgeR of R. */
  static void adv_get_neighbour_q(const int *edgeNum, const double *xL, const double *yL,
                                  const double *xR, const double *yR, const double *qL,
                                  const double *qR, double *exteriorQL, double *exteriorQR) {
    const int *FMASK = g.FMASK.data();
    const int edgeL = edgeNum[0], edgeR = edgeNum[1];
    const bool reverse = !(xL[edgeL] == xR[edgeR] && yL[edgeL] == yR[edgeR]);
    for (int i = 0; i < Nfp; i++) {
      const int k = reverse ? Nfp - i - 1 : i;
      exteriorQL[edgeL * Nfp + i] += qR[FMASK[edgeR * Nfp + k]];
      exteriorQR[edgeR * Nfp + i] += qL[FMASK[edgeL * Nfp + k]];
    }
  }

  /* advec/src/get_bedge_q.h:3-13: a constant ghost value on every boundary face */
  static void adv_get_bedge_q(const int *bedgeNum, double *exteriorQ) {
    for (int i = 0; i < Nfp; i++) exteriorQ[*bedgeNum * Nfp + i] += 4.5e-5;
  }

  /* advec/src/advec_rhs.h:7-67 */
  static void advec_rhs(const double *q, const double *exteriorQ, const double *rx,
                        const double *ry, const double *sx, const double *sy,
                        const double *fscale, const double *nx, const double *ny, double *qRHS) {
    const double velX = g.velX, velY = g.velY;
    double F[Np], G[Np], dFdr[Np], dFds[Np], dGdr[Np], dGds[Np];
    for (int i = 0; i < Np; i++) {
      F[i] = velX * q[i];
      G[i] = velY * q[i];
    }
    gemv(Np, Np, 1.0, g.Drw.data(), Np, F, 1, 0.0, dFdr, 1);
    gemv(Np, Np, 1.0, g.Dsw.data(), Np, F, 1, 0.0, dFds, 1);
    gemv(Np, Np, 1.0, g.Drw.data(), Np, G, 1, 0.0, dGdr, 1);
    gemv(Np, Np, 1.0, g.Dsw.data(), Np, G, 1, 0.0, dGds, 1);
    for (int i = 0; i < Np; i++)
      qRHS[i] = rx[i] * dFdr[i] + sx[i] * dFds[i] + ry[i] * dGdr[i] + sy[i] * dGds[i];
    // Lax-Friedrichs flux with the speed |v| at each face point
    const double a = std::sqrt(velX * velX + velY * velY);
    double nflux[3 * Nfp];
    for (int j = 0; j < 3 * Nfp; j++) {
      const double mQ = q[g.FMASK[j]], pQ = exteriorQ[j];
      const double mF = velX * mQ, mG = velY * mQ, pF = velX * pQ, pG = velY * pQ;
      nflux[j] = nx[j] * (mF + pF) + ny[j] * (mG + pG) + a * (mQ - pQ);
      nflux[j] *= 0.5 * fscale[j];
    }
    gemv(Np, 3 * Nfp, -1.0, g.LIFT.data(), 3 * Nfp, nflux, 1, 1.0, qRHS, 1);
  }

  /* advec/src/set_workingQ.h:1-6 */
  static void adv_set_workingQ(const double *dt, const double *q, const double *rk,
                               const double *rk_frac, double *workingQ) {
    for (int i = 0; i < Np; i++) workingQ[i] = q[i] + (*dt) * (*rk_frac) * rk[i];
  }

  /* advec/src/update_Q.h:1-8: classical RK4 */
  static void adv_update_Q(const double *dt, double *q, const double *rk1, const double *rk2,
                           const double *rk3, const double *rk4, double *workingQ) {
    for (int i = 0; i < Np; i++) {
      q[i] = q[i] + (1.0 / 6.0) * (*dt) * (rk1[i] + 2 * rk2[i] + 2 * rk3[i] + rk4[i]);
      workingQ[i] = q[i];
    }
  }
};

}  // namespace port
#endif
