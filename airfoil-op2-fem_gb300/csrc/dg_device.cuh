// Device physics shared by the native solver kernels: the Roe numerical flux and the boundary
// ghost states, written to spend as few FP64 instructions as possible.  On GB300 the FP64 pipe
// issues about 1.9 DFMA per clock per SM (1.2 TFLOP/s for the chip), some 60x below FP32, and
// a correctly rounded divide or square root costs about ten DFMA slots; so every division of
// the reference's formulas is turned into a reciprocal or reciprocal square root that is
// reused, and constant factors are folded.  The results equal the reference's expressions up
// to rounding.
#pragma once
#include <cstdint>

namespace dg {

struct Phys {
  double gam, gm1;               // gamma, gamma - 1
  double rinf, uinf, vinf, pinf, einf;  // freestream (src/airfoil.cpp:79-99)
  double vx0, vy0, vbeta;        // isentropic vortex centre and strength
  float gamf, gm1f;              // gamma, gamma - 1 in single precision (the dt estimate)
};

__device__ __forceinline__ double rcp(double x) { return __drcp_rn(x); }

// Roe flux across a face with unit normal (nx, ny) from the interior state qm to the exterior
// state qp, in the global frame and not yet scaled by fscale.  Restates src/euler_rhs.h:120-220
// per face node: rotation into the normal frame, Roe averages with sqrt(rho) weights, wave
// strengths dW1..dW4 with |lambda| weights, flux average minus dissipation, rotation back.
// The result is multiplied by 0.5 (the /2.0 of the reference) only at the end, by the caller's
// scale factor: out = scale * 2 * roe.
__device__ __forceinline__ void roe_flux2(const double qm[4], const double qp[4], double nx,
                                          double ny, const Phys &P, double f2[4]) {
  // rotate momenta: m = n.(rho u), t = n x (rho u)
  const double mL = fma(nx, qm[1], ny * qm[2]);
  const double tL = fma(nx, qm[2], -ny * qm[1]);
  const double mR = fma(nx, qp[1], ny * qp[2]);
  const double tR = fma(nx, qp[2], -ny * qp[1]);
  const double rsL = rsqrt(qm[0]), rsR = rsqrt(qp[0]);
  const double sL = qm[0] * rsL, sR = qp[0] * rsR;     // sqrt(rho)
  const double irL = rsL * rsL, irR = rsR * rsR;       // 1/rho
  const double uL = mL * irL, vL = tL * irL;
  const double uR = mR * irR, vR = tR * irR;
  const double pL = P.gm1 * fma(-0.5, fma(mL, uL, tL * vL), qm[3]);
  const double pR = P.gm1 * fma(-0.5, fma(mR, uR, tR * vR), qp[3]);
  const double EpL = qm[3] + pL, EpR = qp[3] + pR;
  const double HL = EpL * irL, HR = EpR * irR;
  // Roe averages
  const double rho = sL * sR;
  const double isum = rcp(sL + sR);
  const double u = fma(sL, uL, sR * uR) * isum;
  const double v = fma(sL, vL, sR * vR) * isum;
  const double H = fma(sL, HL, sR * HR) * isum;
  const double q2 = fma(u, u, v * v);
  const double c2 = P.gm1 * fma(-0.5, q2, H);
  const double rc = rsqrt(c2);
  const double c = c2 * rc;
  const double ic2 = rc * rc;
  // wave strengths
  const double dp = pR - pL;
  const double a = (rho * (uR - uL)) * rc;
  const double dpc2 = dp * ic2;
  double dW1 = 0.5 * (dpc2 - a);
  double dW4 = 0.5 * (dpc2 + a);
  double dW2 = (qp[0] - qm[0]) - dpc2;
  double dW3 = rho * (vR - vL);
  dW1 *= fabs(u - c);
  dW4 *= fabs(u + c);
  const double au = fabs(u);
  dW2 *= au;
  dW3 *= au;
  // dissipation, reference :205-208 regrouped
  const double d14 = dW1 + dW4, e14 = dW4 - dW1;
  const double d0 = d14 + dW2;
  const double d1 = fma(u, d0, c * e14);
  const double d2 = fma(v, d0, dW3);
  const double d3 = fma(H, d14, fma(u * c, e14, fma(dW2, q2, dW3 * v)));
  // 2 * rotated flux = FL + FR - d
  const double g0 = (mL + mR) - d0;
  const double g1 = (fma(mL, uL, pL) + fma(mR, uR, pR)) - d1;
  const double g2 = fma(tL, uL, tR * uR) - d2;
  const double g3 = fma(uL, EpL, uR * EpR) - d3;
  f2[0] = g0;
  f2[1] = fma(nx, g1, -ny * g2);
  f2[2] = fma(ny, g1, nx * g2);
  f2[3] = g3;
}

// Isentropic vortex state at (x, y, t): vortex/src/set_ic.h:6-22.
__device__ __forceinline__ void vortex_state(double x, double y, double t, const Phys &P,
                                             double q[4]) {
  const double dx = x - t - P.vx0, dy = y - P.vy0;
  const double r2 = dx * dx + dy * dy;
  const double e1 = exp(1.0 - r2);
  const double u = 1.0 - P.vbeta * e1 * (dy / (2 * M_PI));
  const double v = P.vbeta * e1 * ((x - P.vx0) / (2 * M_PI));
  double rho = 1.0 - (P.gm1 / (16 * P.gam * M_PI * M_PI)) * P.vbeta * P.vbeta * exp(2 * (1.0 - r2));
  rho = pow(rho, 1.0 / P.gm1);
  const double p = pow(rho, P.gam);
  q[0] = rho;
  q[1] = rho * u;
  q[2] = rho * v;
  q[3] = p / P.gm1 + 0.5 * rho * (u * u + v * v);
}

// Characteristic farfield ghost state (boundary type 3).  No reference counterpart: Riemann
// invariants R+ from the interior and R- from the freestream; entropy and tangential velocity
// from the upwind side; supersonic inflow/outflow take freestream/interior.
__device__ __forceinline__ void farfield_state(const double qi[4], double nx, double ny,
                                               const Phys &P, double qb[4]) {
  const double rhoi = qi[0], ui = qi[1] / rhoi, vi = qi[2] / rhoi;
  const double pi = P.gm1 * (qi[3] - 0.5 * rhoi * (ui * ui + vi * vi));
  const double ci = sqrt(fabs(P.gam * pi / rhoi));
  const double vni = ui * nx + vi * ny;
  if (vni <= -ci) {
    qb[0] = P.rinf; qb[1] = P.rinf * P.uinf; qb[2] = P.rinf * P.vinf; qb[3] = P.einf;
    return;
  }
  if (vni >= ci) {
    qb[0] = qi[0]; qb[1] = qi[1]; qb[2] = qi[2]; qb[3] = qi[3];
    return;
  }
  const double cinf = sqrt(P.gam * P.pinf / P.rinf);
  const double vninf = P.uinf * nx + P.vinf * ny;
  const double rp = vni + 2.0 * ci / P.gm1;
  const double rm = vninf - 2.0 * cinf / P.gm1;
  const double vnb = 0.5 * (rp + rm);
  const double cb = 0.25 * P.gm1 * (rp - rm);
  double sref, ut, vt;
  if (vnb > 0.0) {
    sref = pi / pow(rhoi, P.gam);
    ut = ui - vni * nx;
    vt = vi - vni * ny;
  } else {
    sref = P.pinf / pow(P.rinf, P.gam);
    ut = P.uinf - vninf * nx;
    vt = P.vinf - vninf * ny;
  }
  const double rhob = pow(cb * cb / (P.gam * sref), 1.0 / P.gm1);
  const double ub = ut + vnb * nx, vb = vt + vnb * ny;
  const double pb = rhob * cb * cb / P.gam;
  qb[0] = rhob;
  qb[1] = rhob * ub;
  qb[2] = rhob * vb;
  qb[3] = pb / P.gm1 + 0.5 * rhob * (ub * ub + vb * vb);
}

// Ghost state of src/get_bedge_q.h:23-50 (types 0 inflow, 1 outflow, 2 wall) and type 3.
__device__ __forceinline__ void bc_state(int type, const double qi[4], double nx, double ny,
                                         const Phys &P, double qb[4]) {
  if (type == 0) {
    qb[0] = P.rinf; qb[1] = P.rinf * P.uinf; qb[2] = P.rinf * P.vinf; qb[3] = P.einf;
  } else if (type == 1) {
    qb[0] = P.rinf; qb[1] = P.rinf * P.uinf; qb[2] = P.rinf * P.vinf; qb[3] = qi[3];
  } else if (type == 3) {
    farfield_state(qi, nx, ny, P, qb);
  } else {
    const double mn = 2.0 * fma(nx, qi[1], ny * qi[2]);
    qb[0] = qi[0];
    qb[1] = fma(-mn, nx, qi[1]);
    qb[2] = fma(-mn, ny, qi[2]);
    qb[3] = qi[3];
  }
}

// A density that is not a positive finite double: sign bit set, zero/subnormal, inf or NaN.
// Integer test on the bit pattern, so it costs no FP64 instruction.
__device__ __forceinline__ bool bad_density(double rho) {
  const uint64_t b = (uint64_t)__double_as_longlong(rho);
  return ((b >> 52) - 1ull) >= 0x7FEull;
}

}  // namespace dg
