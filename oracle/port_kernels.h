/* Oracle restatement of the reference's OP2 user kernels, generic in the
 * polynomial order N — TEST INFRASTRUCTURE ONLY (see dg_oracle.h).
 *
 * Every function keeps the reference's argument list, data layout and the
 * order of its floating-point operations, so that with the same operator
 * tables it reproduces the reference kernels bit for bit (both are compiled
 * with -ffp-contract=off).  The reference hard-codes N=4 (15 volume nodes,
 * 5 face nodes); here Np=(N+1)(N+2)/2 and Nfp=N+1 take their place.
 * Each cblas call of the reference is restated as the ascending-index loop
 * of oracle/shim/cblas.h. */
#ifndef ORACLE_PORT_KERNELS_H
#define ORACLE_PORT_KERNELS_H

#include <cmath>
#include <vector>

#include "dg_oracle.h"

namespace port {

struct Ctx {
  int N = 0;
  std::vector<double> r, s, Dr, Ds, Drw, Dsw, LIFT, ones;
  std::vector<int> FMASK;
  double gam, bc_mach, bc_alpha, bc_p, bc_r, bc_u, bc_v, bc_e;
  double vortex_x0, vortex_y0, vortex_beta;
  double velX = 1.0, velY = 1.0;  // scalar advection velocity (advec/src/constants/constant_util.h:9-10)
};
extern Ctx g;

/* y = alpha*A*x + beta*y, row-major, ascending j (oracle/shim/cblas.h). */
inline void gemv(int m, int n, double alpha, const double *a, int lda, const double *x, int incx,
                 double beta, double *y, int incy) {
  for (int i = 0; i < m; i++) {
    double acc = 0.0;
    for (int j = 0; j < n; j++) acc += a[i * lda + j] * x[j * incx];
    if (beta == 0.0) y[i * incy] = alpha * acc;
    else y[i * incy] = alpha * acc + beta * y[i * incy];
  }
}

template <int N>
struct K {
  static constexpr int Np = (N + 1) * (N + 2) / 2;
  static constexpr int Nfp = N + 1;

  /* src/init_grid.h:3-106 */
  static void init_grid(const double *n0, const double *n1, const double *n2, double *nodeX,
                        double *nodeY, double *x, double *y, double *xr, double *yr, double *xs,
                        double *ys, double *rx, double *ry, double *sx, double *sy, double *nx,
                        double *ny, double *fscale) {
    const double *r = g.r.data(), *s = g.s.data();
    const int *FMASK = g.FMASK.data();
    nodeX[0] = n0[0]; nodeX[1] = n1[0]; nodeX[2] = n2[0];
    nodeY[0] = n0[1]; nodeY[1] = n1[1]; nodeY[2] = n2[1];
    double temp[Np];
    // x = 0.5*n1_x*(1+r) + 0.5*n2_x*(1+s) - 0.5*n0_x*(r+s), as the cblas sequence of :25-37
    for (int i = 0; i < Np; i++) x[i] = 1.0;
    for (int i = 0; i < Np; i++) x[i] = x[i] + 1.0 * r[i];
    for (int i = 0; i < Np; i++) x[i] = (0.5 * n1[0]) * x[i];
    for (int i = 0; i < Np; i++) temp[i] = 1.0;
    for (int i = 0; i < Np; i++) temp[i] = temp[i] + 1.0 * s[i];
    for (int i = 0; i < Np; i++) x[i] = x[i] + (0.5 * n2[0]) * temp[i];
    for (int i = 0; i < Np; i++) temp[i] = s[i];
    for (int i = 0; i < Np; i++) temp[i] = temp[i] + 1.0 * r[i];
    for (int i = 0; i < Np; i++) x[i] = x[i] + (-0.5 * n0[0]) * temp[i];
    // y, :42-54
    for (int i = 0; i < Np; i++) y[i] = 1.0;
    for (int i = 0; i < Np; i++) y[i] = y[i] + 1.0 * r[i];
    for (int i = 0; i < Np; i++) y[i] = (0.5 * n1[1]) * y[i];
    for (int i = 0; i < Np; i++) temp[i] = 1.0;
    for (int i = 0; i < Np; i++) temp[i] = temp[i] + 1.0 * s[i];
    for (int i = 0; i < Np; i++) y[i] = y[i] + (0.5 * n2[1]) * temp[i];
    for (int i = 0; i < Np; i++) temp[i] = s[i];
    for (int i = 0; i < Np; i++) temp[i] = temp[i] + 1.0 * r[i];
    for (int i = 0; i < Np; i++) y[i] = y[i] + (-0.5 * n0[1]) * temp[i];
    // :58-65
    gemv(Np, Np, 1.0, g.Dr.data(), Np, x, 1, 0.0, xr, 1);
    gemv(Np, Np, 1.0, g.Ds.data(), Np, x, 1, 0.0, xs, 1);
    gemv(Np, Np, 1.0, g.Dr.data(), Np, y, 1, 0.0, yr, 1);
    gemv(Np, Np, 1.0, g.Ds.data(), Np, y, 1, 0.0, ys, 1);
    double J[Np];
    for (int i = 0; i < Np; i++) J[i] = -xs[i] * yr[i] + xr[i] * ys[i];
    for (int i = 0; i < Np; i++) {
      rx[i] = ys[i] / J[i];
      sx[i] = -yr[i] / J[i];
      ry[i] = -xs[i] / J[i];
      sy[i] = xr[i] / J[i];
    }
    // normals :81-97
    for (int i = 0; i < Nfp; i++) {
      nx[i] = yr[FMASK[i]];
      ny[i] = -xr[FMASK[i]];
    }
    for (int i = 0; i < Nfp; i++) {
      nx[Nfp + i] = ys[FMASK[Nfp + i]] - yr[FMASK[Nfp + i]];
      ny[Nfp + i] = xr[FMASK[Nfp + i]] - xs[FMASK[Nfp + i]];
    }
    for (int i = 0; i < Nfp; i++) {
      nx[2 * Nfp + i] = -ys[FMASK[2 * Nfp + i]];
      ny[2 * Nfp + i] = xs[FMASK[2 * Nfp + i]];
    }
    // :100-105
    for (int i = 0; i < 3 * Nfp; i++) {
      double sJ = std::sqrt(nx[i] * nx[i] + ny[i] * ny[i]);
      nx[i] = nx[i] / sJ;
      ny[i] = ny[i] / sJ;
      fscale[i] = sJ / J[FMASK[i]];
    }
  }

  /* src/set_ic.h:1-12 */
  static void set_ic(double *q, double *workingQ) {
    for (int i = 0; i < Np; i++) {
      q[i * 4] = g.bc_r;
      q[i * 4 + 1] = g.bc_r * g.bc_u;
      q[i * 4 + 2] = g.bc_r * g.bc_v;
      q[i * 4 + 3] = g.bc_e;
      for (int k = 0; k < 4; k++) workingQ[i * 4 + k] = q[i * 4 + k];
    }
  }

  /* Analytic isentropic vortex state at (x,y,t): vortex/src/set_ic.h:6-22 */
  static void vortex_state(double x, double y, double t, double *rho_o, double *u_o, double *v_o,
                           double *ener_o) {
    const double gam = g.gam, x0 = g.vortex_x0, y0 = g.vortex_y0, beta = g.vortex_beta;
    double r = (x - t - x0) * (x - t - x0) + (y - y0) * (y - y0);
    r = std::sqrt(r);
    double u = 1.0 - beta * std::exp(1.0 - r * r) * ((y - y0) / (2 * M_PI));
    double v = beta * std::exp(1.0 - r * r) * ((x - x0) / (2 * M_PI));
    double rho = 1.0 - ((gam - 1) / (16 * gam * M_PI * M_PI)) * beta * beta * std::exp(2 * (1.0 - r * r));
    rho = std::pow(rho, 1.0 / (gam - 1));
    double p = std::pow(rho, gam);
    *rho_o = rho;
    *u_o = u;
    *v_o = v;
    *ener_o = (p / (gam - 1)) + 0.5 * rho * (u * u + v * v);
  }

  /* vortex/src/set_ic.h:3-28 */
  static void set_ic_vortex(const double *t, const double *x, const double *y, double *q,
                            double *workingQ) {
    for (int i = 0; i < Np; i++) {
      double rho, u, v, ener;
      vortex_state(x[i], y[i], *t, &rho, &u, &v, &ener);
      q[i * 4] = rho;
      q[i * 4 + 1] = rho * u;
      q[i * 4 + 2] = rho * v;
      q[i * 4 + 3] = ener;
      for (int k = 0; k < 4; k++) workingQ[i * 4 + k] = q[i * 4 + k];
    }
  }

  /* src/neighbour_zero.h:1-5 */
  static void neighbour_zero(double *exQ) {
    for (int i = 0; i < 4 * 3 * Nfp; i++) exQ[i] = 0.0;
  }

  /* fscale index used by calc_dt: the reference reads fscale[FMASK[i]] (src/calc_dt.h:11), a
   * volume-node id used as a face-point index.  That is in range only while Np <= 3*Nfp
   * (N <= 4); for N >= 5 the face point's own fscale[i] is used. */
  static int dt_fscale_index(int i) { return (Np <= 3 * Nfp) ? g.FMASK[i] : i; }

  /* src/calc_dt.h:3-22, with (4+1)^2 generalised to (N+1)^2 */
  static void calc_dt(const double *q, const double *fscale, double *dt1) {
    const int *FMASK = g.FMASK.data();
    const double gam = g.gam;
    double dt1_arr[3 * Nfp];
    for (int i = 0; i < 3 * Nfp; i++) {
      double rho = q[FMASK[i] * 4];
      double u = q[FMASK[i] * 4 + 1] / rho;
      double v = q[FMASK[i] * 4 + 2] / rho;
      double p = (gam - 1.0) * (q[FMASK[i] * 4 + 3] - rho * (u * u + v * v) * 0.5);
      double c = std::sqrt(std::abs(gam * p / rho));
      dt1_arr[i] = ((N + 1) * (N + 1)) * 0.5 * fscale[dt_fscale_index(i)] * (std::sqrt(u * u + v * v) + c);
    }
    double max = *dt1;
    for (int i = 0; i < 3 * Nfp; i++)
      if (dt1_arr[i] > max) max = dt1_arr[i];
    *dt1 = max;
  }

  /* src/get_neighbour_q.h:1-89 */
  static void get_neighbour_q(const int *edgeNum, const double *xL, const double *yL,
                              const double *xR, const double *yR, const double *qL,
                              const double *qR, double *exteriorQL, double *exteriorQR) {
    const int *FMASK = g.FMASK.data();
    int edgeL = edgeNum[0];
    int edgeR = edgeNum[1];
    // :10-34 — vertex edgeL of L against vertex edgeR of R, exact compare
    bool reverse = !(xL[edgeL] == xR[edgeR] && yL[edgeL] == yR[edgeR]);
    int exInd = edgeL * 4 * Nfp;
    const int *fmask = &FMASK[edgeR * Nfp];
    for (int i = 0; i < Nfp; i++) {
      int rInd = reverse ? 4 * fmask[Nfp - i - 1] : 4 * fmask[i];
      for (int k = 0; k < 4; k++) exteriorQL[exInd + 4 * i + k] += qR[rInd + k];
    }
    exInd = edgeR * 4 * Nfp;
    fmask = &FMASK[edgeL * Nfp];
    for (int i = 0; i < Nfp; i++) {
      int lInd = reverse ? 4 * fmask[Nfp - i - 1] : 4 * fmask[i];
      for (int k = 0; k < 4; k++) exteriorQR[exInd + 4 * i + k] += qL[lInd + k];
    }
  }

  /* Characteristic (Riemann-invariant) farfield ghost state: bedge_type 3.  This has no
   * counterpart in the reference (which has inflow/outflow/wall only); it is the build's
   * extension for the farfield of the O-grid airfoil case.  Subsonic: R+ from the interior,
   * R- from the freestream; entropy and tangential velocity from the upwind side.
   * Supersonic inflow takes the freestream, supersonic outflow the interior state. */
  static void farfield_state(const double *qi, double nx, double ny, double *qb) {
    const double gam = g.gam;
    double rhoi = qi[0], ui = qi[1] / rhoi, vi = qi[2] / rhoi;
    double pi = (gam - 1.0) * (qi[3] - 0.5 * rhoi * (ui * ui + vi * vi));
    double ci = std::sqrt(std::abs(gam * pi / rhoi));
    double vni = ui * nx + vi * ny;
    double rinf = g.bc_r, uinf = g.bc_u, vinf = g.bc_v, pinf = g.bc_p;
    double cinf = std::sqrt(gam * pinf / rinf);
    double vninf = uinf * nx + vinf * ny;
    if (vni <= -ci) {  // supersonic inflow
      qb[0] = rinf; qb[1] = rinf * uinf; qb[2] = rinf * vinf; qb[3] = g.bc_e;
      return;
    }
    if (vni >= ci) {  // supersonic outflow
      for (int k = 0; k < 4; k++) qb[k] = qi[k];
      return;
    }
    double rp = vni + 2.0 * ci / (gam - 1.0);
    double rm = vninf - 2.0 * cinf / (gam - 1.0);
    double vnb = 0.5 * (rp + rm);
    double cb = 0.25 * (gam - 1.0) * (rp - rm);
    double sref, ut, vt;
    if (vnb > 0.0) {  // outflow: entropy and tangential velocity from the interior
      sref = pi / std::pow(rhoi, gam);
      ut = ui - vni * nx;
      vt = vi - vni * ny;
    } else {
      sref = pinf / std::pow(rinf, gam);
      ut = uinf - vninf * nx;
      vt = vinf - vninf * ny;
    }
    double rhob = std::pow(cb * cb / (gam * sref), 1.0 / (gam - 1.0));
    double ub = ut + vnb * nx, vb = vt + vnb * ny;
    double pb = rhob * cb * cb / gam;
    qb[0] = rhob;
    qb[1] = rhob * ub;
    qb[2] = rhob * vb;
    qb[3] = pb / (gam - 1.0) + 0.5 * rhob * (ub * ub + vb * vb);
  }

  /* src/get_bedge_q.h:1-51 (+ type 3, see farfield_state) */
  static void get_bedge_q(const int *bedge_type, const int *bedgeNum, const double *nx,
                          const double *ny, const double *q, double *exteriorQ) {
    int exInd = *bedgeNum * 4 * Nfp;
    int nInd = *bedgeNum * Nfp;
    const int *fmask = &g.FMASK[*bedgeNum * Nfp];
    if (*bedge_type == 0) {
      for (int i = 0; i < Nfp; i++) {
        exteriorQ[exInd + i * 4] += g.bc_r;
        exteriorQ[exInd + i * 4 + 1] += g.bc_r * g.bc_u;
        exteriorQ[exInd + i * 4 + 2] += g.bc_r * g.bc_v;
        exteriorQ[exInd + i * 4 + 3] += g.bc_e;
      }
    } else if (*bedge_type == 1) {
      for (int i = 0; i < Nfp; i++) {
        int qInd = fmask[i] * 4;
        exteriorQ[exInd + i * 4] += g.bc_r;
        exteriorQ[exInd + i * 4 + 1] += g.bc_r * g.bc_u;
        exteriorQ[exInd + i * 4 + 2] += g.bc_r * g.bc_v;
        exteriorQ[exInd + i * 4 + 3] += q[qInd + 3];
      }
    } else if (*bedge_type == 3) {
      for (int i = 0; i < Nfp; i++) {
        double qb[4];
        farfield_state(&q[fmask[i] * 4], nx[nInd + i], ny[nInd + i], qb);
        for (int k = 0; k < 4; k++) exteriorQ[exInd + i * 4 + k] += qb[k];
      }
    } else {
      for (int i = 0; i < Nfp; i++) {
        int qInd = fmask[i] * 4;
        exteriorQ[exInd + i * 4] += q[qInd];
        exteriorQ[exInd + i * 4 + 1] += q[qInd + 1] - 2 * (nx[nInd + i] * q[qInd + 1] + ny[nInd + i] * q[qInd + 2]) * nx[nInd + i];
        exteriorQ[exInd + i * 4 + 2] += q[qInd + 2] - 2 * (nx[nInd + i] * q[qInd + 1] + ny[nInd + i] * q[qInd + 2]) * ny[nInd + i];
        exteriorQ[exInd + i * 4 + 3] += q[qInd + 3];
      }
    }
  }

  /* vortex/src/get_bedge_q.h:3-40 — analytic state at the stage time */
  static void get_bedge_q_vortex(const int *bedgeNum, const double *x, const double *y,
                                 const double *t, double *exteriorQ) {
    int exInd = *bedgeNum * 4 * Nfp;
    const int *fmask = &g.FMASK[*bedgeNum * Nfp];
    for (int i = 0; i < Nfp; i++) {
      double rho, u, v, ener;
      vortex_state(x[fmask[i]], y[fmask[i]], *t, &rho, &u, &v, &ener);
      exteriorQ[exInd + i * 4] += rho;
      exteriorQ[exInd + i * 4 + 1] += rho * u;
      exteriorQ[exInd + i * 4 + 2] += rho * v;
      exteriorQ[exInd + i * 4 + 3] += ener;
    }
  }

  /* src/euler_rhs.h:7-23 */
  static void euler_flux(const double *q, double *F, double *G, double *rho, double *u, double *v,
                         double *p) {
    const double gam = g.gam;
    *rho = q[0];
    *u = q[1] / (*rho);
    *v = q[2] / (*rho);
    *p = (gam - 1) * (q[3] - 0.5 * (q[1] * (*u) + q[2] * (*v)));
    F[0] = q[1];
    F[1] = q[1] * (*u) + (*p);
    F[2] = q[2] * (*u);
    F[3] = (*u) * (q[3] + (*p));
    G[0] = q[2];
    G[1] = q[1] * (*v);
    G[2] = q[2] * (*v) + (*p);
    G[3] = (*v) * (q[3] + (*p));
  }

  /* src/euler_rhs.h:120-220 */
  static void roe(double *flux, const double *nx, const double *ny, const double *fscale,
                  const double *q, const double *pQ) {
    const double gam = g.gam;
    const int *FMASK = g.FMASK.data();
    for (int i = 0; i < 3 * Nfp; i++) {
      double mQ[4];
      int ind = FMASK[i] * 4;
      for (int k = 0; k < 4; k++) mQ[k] = q[ind + k];
      const double *pq = &pQ[i * 4];
      double mRoeQ[4], pRoeQ[4];
      mRoeQ[0] = mQ[0];
      mRoeQ[1] = nx[i] * mQ[1] + ny[i] * mQ[2];
      mRoeQ[2] = -ny[i] * mQ[1] + nx[i] * mQ[2];
      mRoeQ[3] = mQ[3];
      pRoeQ[0] = pq[0];
      pRoeQ[1] = nx[i] * pq[1] + ny[i] * pq[2];
      pRoeQ[2] = -ny[i] * pq[1] + nx[i] * pq[2];
      pRoeQ[3] = pq[3];
      double fxMQ[4], fyMQ[4], mRoeRho, mRoeU, mRoeV, mRoeP;
      euler_flux(mRoeQ, fxMQ, fyMQ, &mRoeRho, &mRoeU, &mRoeV, &mRoeP);
      double fxPQ[4], fyPQ[4], pRoeRho, pRoeU, pRoeV, pRoeP;
      euler_flux(pRoeQ, fxPQ, fyPQ, &pRoeRho, &pRoeU, &pRoeV, &pRoeP);
      double mH = (mRoeQ[3] + mRoeP) / mRoeRho;
      double pH = (pRoeQ[3] + pRoeP) / pRoeRho;
      double mRoeRhoSqrt = std::sqrt(mRoeRho);
      double pRoeRhoSqrt = std::sqrt(pRoeRho);
      double rho = mRoeRhoSqrt * pRoeRhoSqrt;
      double u = (mRoeRhoSqrt * mRoeU + pRoeRhoSqrt * pRoeU) / (mRoeRhoSqrt + pRoeRhoSqrt);
      double v = (mRoeRhoSqrt * mRoeV + pRoeRhoSqrt * pRoeV) / (mRoeRhoSqrt + pRoeRhoSqrt);
      double H = (mRoeRhoSqrt * mH + pRoeRhoSqrt * pH) / (mRoeRhoSqrt + pRoeRhoSqrt);
      double c2 = (gam - 1) * (H - 0.5 * (u * u + v * v));
      double c = std::sqrt(c2);
      double dW1 = -0.5 * rho * (pRoeU - mRoeU) / c + 0.5 * (pRoeP - mRoeP) / c2;
      double dW2 = (pRoeRho - mRoeRho) - (pRoeP - mRoeP) / c2;
      double dW3 = rho * (pRoeV - mRoeV);
      double dW4 = 0.5 * rho * (pRoeU - mRoeU) / c + 0.5 * (pRoeP - mRoeP) / c2;
      dW1 = std::abs(u - c) * dW1;
      dW2 = std::abs(u) * dW2;
      dW3 = std::abs(u) * dW3;
      dW4 = std::abs(u + c) * dW4;
      double fx[4];
      for (int k = 0; k < 4; k++) fx[k] = (fxMQ[k] + fxPQ[k]) / 2.0;
      fx[0] = fx[0] - (dW1 + dW2 + dW4) / 2.0;
      fx[1] = fx[1] - (dW1 * (u - c) + dW2 * u + dW4 * (u + c)) / 2.0;
      fx[2] = fx[2] - (dW1 * v + dW2 * v + dW3 + dW4 * v) / 2.0;
      fx[3] = fx[3] - (dW1 * (H - u * c) + dW2 * (u * u + v * v) + dW3 * v + dW4 * (H + u * c)) / 2.0;
      flux[i * 4] = fx[0];
      flux[i * 4 + 1] = nx[i] * fx[1] - ny[i] * fx[2];
      flux[i * 4 + 2] = ny[i] * fx[1] + nx[i] * fx[2];
      flux[i * 4 + 3] = fx[3];
      for (int k = 0; k < 4; k++) flux[i * 4 + k] *= fscale[i];
    }
  }

  /* src/euler_rhs.h:222-291.  zero_ext=false gives the vortex variant
   * (vortex/src/euler_rhs.h: exteriorQ is OP_READ and is cleared by neighbour_zero). */
  static void euler_rhs(const double *q, double *exteriorQ, const double *rx, const double *ry,
                        const double *sx, const double *sy, const double *fscale, const double *nx,
                        const double *ny, double *qRHS, bool zero_ext = true) {
    double F[4 * Np], G[4 * Np];
    for (int i = 0; i < Np; i++) {
      double rho, u, v, p;
      euler_flux(&q[i * 4], &F[i * 4], &G[i * 4], &rho, &u, &v, &p);
    }
    for (int i = 0; i < 4; i++) {
      double dFdr[Np], dFds[Np], dGdr[Np], dGds[Np];
      gemv(Np, Np, 1.0, g.Drw.data(), Np, &F[i], 4, 0.0, dFdr, 1);
      gemv(Np, Np, 1.0, g.Dsw.data(), Np, &F[i], 4, 0.0, dFds, 1);
      gemv(Np, Np, 1.0, g.Drw.data(), Np, &G[i], 4, 0.0, dGdr, 1);
      gemv(Np, Np, 1.0, g.Dsw.data(), Np, &G[i], 4, 0.0, dGds, 1);
      for (int j = 0; j < Np; j++)
        qRHS[i + j * 4] = (rx[j] * dFdr[j] + sx[j] * dFds[j]) + (ry[j] * dGdr[j] + sy[j] * dGds[j]);
    }
    // The reference recomputes mF/pF here (:250-278) without using them; roe recomputes them.
    double flux[4 * 3 * Nfp];
    roe(flux, nx, ny, fscale, q, exteriorQ);
    for (int i = 0; i < 4; i++)
      gemv(Np, 3 * Nfp, -1.0, g.LIFT.data(), 3 * Nfp, &flux[i], 4, 1.0, qRHS + i, 4);
    if (zero_ext)
      for (int i = 0; i < 4 * 3 * Nfp; i++) exteriorQ[i] = 0.0;
  }

  /* src/set_workingQ.h:1-12 (the airfoil copy; the vortex copy's stage test is on the pointer,
   * vortex/src/set_workingQ.h:6, and is not reproduced). */
  static void set_workingQ(const double *dt, const int *stage, const double *q, const double *k1,
                           const double *k2, double *workingQ) {
    if (*stage == 0) {
      for (int i = 0; i < 4 * Np; i++) workingQ[i] = q[i] + (*dt) * k1[i];
    } else {
      for (int i = 0; i < 4 * Np; i++) workingQ[i] = q[i] + (*dt) * (k1[i] / 4.0 + k2[i] / 4.0);
    }
  }

  /* src/update_Q.h:1-12 */
  static void update_Q(const double *dt, double *q, const double *rk1, const double *rk2,
                       const double *rk3, double *workingQ) {
    for (int i = 0; i < 4 * Np; i++) {
      q[i] = q[i] + (*dt) * (rk1[i] / 6.0 + rk2[i] / 6.0 + 2.0 * rk3[i] / 3.0);
      workingQ[i] = q[i];
    }
  }

  /* vortex/src/l2_error.h:3-29 (OP_INC sums; the per-node error dat is not kept) */
  static void l2_error(const double *x, const double *y, const double *q, const double *t,
                       double *error_r, double *error_ru, double *error_rv, double *error_ener) {
    double er = 0.0, eru = 0.0, erv = 0.0, ee = 0.0;
    for (int i = 0; i < Np; i++) {
      double rho, u, v, ener;
      vortex_state(x[i], y[i], *t, &rho, &u, &v, &ener);
      er += (q[i * 4] - rho) * (q[i * 4] - rho);
      eru += (q[i * 4 + 1] - rho * u) * (q[i * 4 + 1] - rho * u);
      erv += (q[i * 4 + 2] - rho * v) * (q[i * 4 + 2] - rho * v);
      ee += (q[i * 4 + 3] - ener) * (q[i * 4 + 3] - ener);
    }
    *error_r += er;
    *error_ru += eru;
    *error_rv += erv;
    *error_ener += ee;
  }
};

}  // namespace port
#endif
