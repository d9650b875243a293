// Device physics shared by the native solver kernels: the Roe numerical flux and the boundary
// ghost states, written to spend as few FP64 instructions as possible.  On GB300 the FP64 pipe
// issues about 1.9 DFMA per clock per SM (1.2 TFLOP/s for the chip), some 60x below FP32, and
// a correctly rounded divide or square root costs about ten DFMA slots; so every division of
// the reference's formulas is turned into a reciprocal or reciprocal square root that is
// reused, and constant factors are folded.  The results equal the reference's expressions up
// to rounding.
#pragma once
#include <cmath>
#include <cstdint>

namespace dg {

struct Phys {
  double gam, gm1;               // gamma, gamma - 1
  double rinf, uinf, vinf, pinf, einf;  // freestream (src/airfoil.cpp:79-99)
  double vx0, vy0, vbeta;        // isentropic vortex centre and strength
  // Set by derive(): freestream sound speed and its reciprocal, 2/(gamma-1), 1/gamma,
  // 1/(gamma-1), and the vortex's density coefficient (gamma-1)/(16 gamma pi^2).
  double cinf, rcinf, tgm1, igam, igm1, kvort;
  float gamf, gm1f;              // gamma, gamma - 1 in single precision (the dt estimate)
  // 2/(gamma-1) is 5 (gamma = 1.4; 5 + 9e-16 after the rounding of gamma - 1 in double): the
  // powers x^(2/(gamma-1)) and x^(1/(gamma-1)) are taken as x^5 and x^2 sqrt(x).
  int pow5;

  void derive() {
    gamf = (float)gam;
    gm1f = (float)gm1;
    cinf = sqrt(gam * pinf / rinf);
    rcinf = 1.0 / cinf;
    tgm1 = 2.0 / gm1;
    igam = 1.0 / gam;
    igm1 = 1.0 / gm1;
    kvort = gm1 / (16 * gam * M_PI * M_PI);
    pow5 = fabs(tgm1 - 5.0) < 1e-12 ? 1 : 0;
  }
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
  // One reciprocal square root serves both sides: with r = 1/sqrt(rho_L rho_R),
  // 1/rho_L = rho_R r^2, 1/rho_R = rho_L r^2, sqrt(rho_R / rho_L) = rho_R r and the Roe density
  // sqrt(rho_L rho_R) = rho_L rho_R r.
  const double PLR = qm[0] * qp[0];
  const double r = rsqrt(PLR);
  const double r2 = r * r;
  const double irL = qp[0] * r2, irR = qm[0] * r2;   // 1/rho
  const double uL = mL * irL, vL = tL * irL;
  const double uR = mR * irR, vR = tR * irR;
  const double pL = P.gm1 * fma(-0.5, fma(mL, uL, tL * vL), qm[3]);
  const double pR = P.gm1 * fma(-0.5, fma(mR, uR, tR * vR), qp[3]);
  const double EpL = qm[3] + pL, EpR = qp[3] + pR;
  const double HL = EpL * irL, HR = EpR * irR;
  // Roe averages (sqrt(rho_L) x_L + sqrt(rho_R) x_R) / (sqrt(rho_L) + sqrt(rho_R)), divided through
  // by sqrt(rho_L): (x_L + R x_R) / (1 + R), R = sqrt(rho_R / rho_L)
  const double rho = PLR * r;
  const double R = qp[0] * r;
  const double isum = rcp(1.0 + R);
  const double u = fma(R, uR, uL) * isum;
  const double v = fma(R, vR, vL) * isum;
  const double H = fma(R, HR, HL) * isum;
  const double q2 = fma(u, u, v * v);
  const double c2 = P.gm1 * fma(-0.5, q2, H);
  const double rc = rsqrt(c2);
  const double c = c2 * rc;
  // wave strengths, with the 1/2 of dW1 and dW4 carried by rch = rc / 2: scaling by a power of
  // two is exact, so dpc2h = dp / (2 c^2) and ah = a / 2 round exactly as dp / c^2 and a do, and
  // dW1 = dpc2h - ah is the reference's (dp / c^2 - a) / 2 bit for bit, one multiply fewer
  const double rch = 0.5 * rc;
  const double dp = pR - pL;
  const double ah = (rho * (uR - uL)) * rch;
  const double dpc2h = dp * (rc * rch);
  double dW1 = dpc2h - ah;
  double dW4 = dpc2h + ah;
  double dW2 = fma(-2.0, dpc2h, qp[0] - qm[0]);
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
  // b = 1 - k beta^2 exp(2 (1 - r2)), rho = b^(1/(gamma-1)), p = rho^gamma = b^(gamma/(gamma-1)),
  // which is rho * b: one exp and at most one pow instead of two and two.
  const double b = 1.0 - P.kvort * P.vbeta * P.vbeta * (e1 * e1);
  const double rho = P.pow5 ? b * b * sqrt(b) : pow(b, P.igm1);
  const double p = rho * b;
  q[0] = rho;
  q[1] = rho * u;
  q[2] = rho * v;
  q[3] = fma(p, P.igm1, 0.5 * rho * (u * u + v * v));
}

// Characteristic farfield ghost state (boundary type 3).  No reference counterpart: Riemann
// invariants R+ from the interior and R- from the freestream; entropy and tangential velocity
// from the upwind side; supersonic inflow/outflow take freestream/interior.
__device__ __forceinline__ void farfield_state(const double qi[4], double nx, double ny,
                                               const Phys &P, double qb[4]) {
  const double rhoi = qi[0], ir = rcp(rhoi);
  const double ui = qi[1] * ir, vi = qi[2] * ir;
  const double pi = P.gm1 * fma(-0.5, fma(qi[1], ui, qi[2] * vi), qi[3]);
  const double c2i = fabs(P.gam * pi * ir);
  const double rci = rsqrt(c2i), ci = c2i * rci;
  const double vni = fma(ui, nx, vi * ny);
  if (vni <= -ci) {
    qb[0] = P.rinf; qb[1] = P.rinf * P.uinf; qb[2] = P.rinf * P.vinf; qb[3] = P.einf;
    return;
  }
  if (vni >= ci) {
    qb[0] = qi[0]; qb[1] = qi[1]; qb[2] = qi[2]; qb[3] = qi[3];
    return;
  }
  const double vninf = fma(P.uinf, nx, P.vinf * ny);
  const double rp = fma(P.tgm1, ci, vni);
  const double rm = fma(-P.tgm1, P.cinf, vninf);
  const double vnb = 0.5 * (rp + rm);
  const double cb = 0.25 * P.gm1 * (rp - rm);
  // Entropy s = p_u / rho_u^gamma and tangential velocity from the upwind side u (interior for
  // outflow, freestream for inflow).  rho_b = (cb^2 / (gamma s))^(1/(gamma-1)) is, since
  // c_u^2 = gamma p_u / rho_u, rho_u (|cb| / c_u)^(2/(gamma-1)): no pow for gamma = 1.4.
  const bool out = vnb > 0.0;
  const double rho_u = out ? rhoi : P.rinf;
  const double ratio = fabs(cb) * (out ? rci : P.rcinf);
  double rhob;
  if (P.pow5) {
    const double r2 = ratio * ratio;
    rhob = rho_u * (r2 * r2 * ratio);
  } else {
    rhob = rho_u * pow(ratio, P.tgm1);
  }
  const double ut = out ? fma(-vni, nx, ui) : fma(-vninf, nx, P.uinf);
  const double vt = out ? fma(-vni, ny, vi) : fma(-vninf, ny, P.vinf);
  const double ub = fma(vnb, nx, ut), vb = fma(vnb, ny, vt);
  const double pb = rhob * cb * cb * P.igam;
  qb[0] = rhob;
  qb[1] = rhob * ub;
  qb[2] = rhob * vb;
  qb[3] = fma(pb, P.igm1, 0.5 * rhob * fma(ub, ub, vb * vb));
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
