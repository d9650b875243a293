// Discrete adjoint of the plain fused path (included at the end of dg_solver.cu: it shares the
// per-order constant-memory operators and the forward device functions).
//
// Objective: the mean, over the last `navg` of `nsteps` SSPRK3 steps, of the lift coefficient
//   C_l(q) = (1 / (1/2 rho_inf |V_inf|^2 c)) * sum over wall faces, face nodes k of
//            w_k sJ p_k (n . e_lift),   e_lift = (-sin alpha, cos alpha), c = 1,
// with n the cell's outward normal (pointing into the body: the pressure force on the body) and
// w_k the 1-D face quadrature weights of the face nodes (row sums of the face mass matrix).
// Gradients with respect to alpha (degrees; through the boundary states and the initial state)
// and the initial field q0, with the dt sequence frozen from the forward run.
//
// Objective (isentropic vortex, app 1): the final-time sum over nodes and variables of the
// squared error against the analytic vortex (the four sums of vortex/src/l2_error.h:3-29
// added), J = sum (q_N - q_ex(t_N; beta))^2.  The scalar parameter is then the vortex strength
// beta, entering through the initial state, the analytic boundary states of every stage and
// the exact solution in J; the gradient with respect to q0 is as above.
//
// One reverse SSPRK3 step (Shu-Osher form: W1 = q + dt L(q); W2 = 3/4 q + 1/4 (W1 + dt L(W1));
// q' = 1/3 q + 2/3 (W2 + dt L(W2))), with G(W, v) = (dL/dW at W)^T v:
//   lW2 = 2/3 l' + 2/3 dt G(W2, l')
//   lW1 = 1/4 lW2 + 1/4 dt G(W1, lW2)
//   l   = 1/3 l' + 3/4 lW2 + lW1 + dt G(q, lW1)
// G is three kernels: adj_elem (transposed contraction of [Drw | Dsw | -LIFT] and the nodal
// flux Jacobians), adj_face (reverse of the Roe flux and of the ghost states, once per face node)
// and adj_combine (gathers the face-trace adjoints onto the nodes and forms the combination).
// Every adjoint slot has one writer, so the gradient is deterministic.
//
// Stage states come from recomputation: q is checkpointed every C steps in the forward run;
// going backwards, each segment is re-run from its checkpoint with the frozen dt sequence,
// keeping q, W1, W2 of each of its steps.
#pragma once

namespace dg {

__constant__ double c_wq[7][8];    // face quadrature weights per order
__constant__ int c_fpt[7][28 * 2]; // face points k with FMASK[k] == node (up to two; -1 none)

// ---------------------------------------------------------------- reverse of roe_flux2
// Adds to qmb, qpb the adjoints of qm, qp given fb, the adjoint of roe_flux2's output f2.  The
// forward sweep is roe_flux2's (one reciprocal square root of rho_L rho_R for both sides).
__device__ __forceinline__ void roe_flux2_adj(const double qm[4], const double qp[4], const double nx,
                                              const double ny, const Phys &P, const double fb[4], double qmb[4],
                                              double qpb[4]) {
  // forward sweep
  const double mL = fma(nx, qm[1], ny * qm[2]);
  const double tL = fma(nx, qm[2], -ny * qm[1]);
  const double mR = fma(nx, qp[1], ny * qp[2]);
  const double tR = fma(nx, qp[2], -ny * qp[1]);
  const double PLR = qm[0] * qp[0];
  const double r = rsqrt(PLR);
  const double r2 = r * r;
  const double irL = qp[0] * r2, irR = qm[0] * r2;
  const double uL = mL * irL, vL = tL * irL;
  const double uR = mR * irR, vR = tR * irR;
  const double pL = P.gm1 * fma(-0.5, fma(mL, uL, tL * vL), qm[3]);
  const double pR = P.gm1 * fma(-0.5, fma(mR, uR, tR * vR), qp[3]);
  const double EpL = qm[3] + pL, EpR = qp[3] + pR;
  const double HL = EpL * irL, HR = EpR * irR;
  const double rho = PLR * r;
  const double R = qp[0] * r;
  const double isum = rcp(1.0 + R);
  const double us = fma(R, uR, uL), vs = fma(R, vR, vL), Hs = fma(R, HR, HL);
  const double u = us * isum, v = vs * isum, H = Hs * isum;
  const double q2 = fma(u, u, v * v);
  const double c2 = P.gm1 * fma(-0.5, q2, H);
  const double rc = rsqrt(c2);
  const double c = c2 * rc;
  const double ic2 = rc * rc;
  const double dp = pR - pL;
  const double du = uR - uL;
  const double a = (rho * du) * rc;
  const double dpc2 = dp * ic2;
  const double dW1 = 0.5 * (dpc2 - a), dW4 = 0.5 * (dpc2 + a);
  const double dW2 = (qp[0] - qm[0]) - dpc2;
  const double dW3 = rho * (vR - vL);
  const double lam1 = fabs(u - c), lam4 = fabs(u + c), au = fabs(u);
  const double W1 = dW1 * lam1, W4 = dW4 * lam4, W2 = dW2 * au, W3 = dW3 * au;
  const double d14 = W1 + W4, e14 = W4 - W1;
  const double d0 = d14 + W2;
  // reverse sweep
  const double gb0 = fb[0], gb1 = fma(nx, fb[1], ny * fb[2]), gb2 = fma(nx, fb[2], -ny * fb[1]), gb3 = fb[3];
  double mLb = gb0 + gb1 * uL, mRb = gb0 + gb1 * uR;
  double uLb = gb1 * mL + gb2 * tL + gb3 * EpL;
  double uRb = gb1 * mR + gb2 * tR + gb3 * EpR;
  double pLb = gb1, pRb = gb1;
  double tLb = gb2 * uL, tRb = gb2 * uR;
  double EpLb = gb3 * uL, EpRb = gb3 * uR;
  const double d0b0 = -gb0, d1b = -gb1, d2b = -gb2, d3b = -gb3;
  // d3 = H d14 + (u c) e14 + W2 q2 + W3 v
  double Hb = d3b * d14;
  double d14b = d3b * H;
  const double ucb = d3b * e14;
  double ub = ucb * c, cb = ucb * u;
  double e14b = d3b * (u * c);
  double W2b = d3b * q2, q2b = d3b * W2, W3b = d3b * v, vb = d3b * W3;
  // d2 = v d0 + W3
  vb += d2b * d0;
  double d0b = d0b0 + d2b * v;
  W3b += d2b;
  // d1 = u d0 + c e14
  ub += d1b * d0;
  d0b += d1b * u;
  cb += d1b * e14;
  e14b += d1b * c;
  // d0 = d14 + W2
  d14b += d0b;
  W2b += d0b;
  const double W1b = d14b - e14b, W4b = d14b + e14b;
  const double dW3b = W3b * au, dW2b = W2b * au, dW4b = W4b * lam4, dW1b = W1b * lam1;
  const double aub = W3b * dW3 + W2b * dW2, lam4b = W4b * dW4, lam1b = W1b * dW1;
  const double s_u = copysign(1.0, u), s4 = copysign(1.0, u + c), s1 = copysign(1.0, u - c);
  ub += aub * s_u + lam4b * s4 + lam1b * s1;
  cb += lam4b * s4 - lam1b * s1;
  double rhob = dW3b * (vR - vL);
  double vRb = dW3b * rho, vLb = -dW3b * rho;
  double q0pb = dW2b, q0mb = -dW2b;
  double dpc2b = -dW2b + 0.5 * (dW1b + dW4b);
  const double ab = 0.5 * (dW4b - dW1b);
  double dpb = dpc2b * ic2;
  double ic2b = dpc2b * dp;
  rhob += ab * du * rc;
  uRb += ab * rho * rc;
  uLb -= ab * rho * rc;
  double rcb = ab * rho * du;
  pRb += dpb;
  pLb -= dpb;
  rcb += 2.0 * rc * ic2b;
  double c2b = cb * rc;
  rcb += cb * c2;
  c2b += rcb * (-0.5) * rc * ic2;
  Hb += c2b * P.gm1;
  q2b -= 0.5 * c2b * P.gm1;
  ub += 2.0 * u * q2b;
  vb += 2.0 * v * q2b;
  // u, v, H = (x_L + R x_R) * isum, isum = 1 / (1 + R)
  const double isumb = Hb * Hs + ub * us + vb * vs;
  const double Hsb = Hb * isum, usb = ub * isum, vsb = vb * isum;
  const double Rb = Hsb * HR + usb * uR + vsb * vR - isumb * isum * isum;
  const double HLb = Hsb, HRb = Hsb * R;
  uLb += usb;
  uRb += usb * R;
  vLb += vsb;
  vRb += vsb * R;
  // rho = PLR r, R = rho_R r
  double rb = rhob * PLR + Rb * qp[0];
  double PLRb = rhob * r;
  q0pb += Rb * r;
  // H = Ep * ir
  EpLb += HLb * irL;
  double irLb = HLb * EpL;
  EpRb += HRb * irR;
  double irRb = HRb * EpR;
  // Ep = q3 + p
  double q3mb = EpLb, q3pb = EpRb;
  pLb += EpLb;
  pRb += EpRb;
  // p = gm1 (q3 - 0.5 (m u + t v))
  q3mb += pLb * P.gm1;
  q3pb += pRb * P.gm1;
  const double kL = -0.5 * P.gm1 * pLb, kR = -0.5 * P.gm1 * pRb;
  mLb += kL * uL;
  uLb += kL * mL;
  tLb += kL * vL;
  vLb += kL * tL;
  mRb += kR * uR;
  uRb += kR * mR;
  tRb += kR * vR;
  vRb += kR * tR;
  // u = m ir, v = t ir
  mLb += uLb * irL;
  irLb += uLb * mL + vLb * tL;
  tLb += vLb * irL;
  mRb += uRb * irR;
  irRb += uRb * mR + vRb * tR;
  tRb += vRb * irR;
  // irL = rho_R r^2, irR = rho_L r^2, r = PLR^(-1/2), PLR = rho_L rho_R
  q0pb += irLb * r2;
  q0mb += irRb * r2;
  rb += 2.0 * r * (irLb * qp[0] + irRb * qm[0]);
  PLRb += rb * (-0.5) * r * r2;
  q0mb += PLRb * qp[0];
  q0pb += PLRb * qm[0];
  // m = nx q1 + ny q2, t = nx q2 - ny q1
  qmb[0] += q0mb;
  qmb[1] += mLb * nx - tLb * ny;
  qmb[2] += mLb * ny + tLb * nx;
  qmb[3] += q3mb;
  qpb[0] += q0pb;
  qpb[1] += mRb * nx - tRb * ny;
  qpb[2] += mRb * ny + tRb * nx;
  qpb[3] += q3pb;
}

// Freestream momenta' sensitivities to alpha in degrees (src/airfoil.cpp:85-88:
// u = sin(pi/2 - a) |V|, v = cos(pi/2 - a) |V|, a in radians).
struct AlphaSens {
  double dru, drv, dE;  // d(rho u)/d alpha, d(rho v)/d alpha, dE/d alpha
};

// Reverse sweep of the characteristic farfield ghost state (farfield_state, dg_device.cuh):
// adds (d qb / d qi)^T qbb to qmb and returns qbb . d qb / d alpha (alpha enters through the
// freestream velocity (u_inf, v_inf) = |V| (cos a, sin a); rho_inf, p_inf, c_inf and E_inf do not
// depend on it).  The branch (supersonic inflow / outflow, subsonic outflow or inflow) is the one
// the forward evaluation took at qi.
__device__ __forceinline__ double farfield_state_adj(const double qi[4], const double nx, const double ny,
                                                     const Phys &P, const double qbb[4], const AlphaSens &S,
                                                     double qmb[4]) {
  // forward sweep (farfield_state, same operations)
  const double rhoi = qi[0], ir = rcp(rhoi);
  const double ui = qi[1] * ir, vi = qi[2] * ir;
  const double pi = P.gm1 * fma(-0.5, fma(qi[1], ui, qi[2] * vi), qi[3]);
  const double c2s = P.gam * pi * ir;
  const double c2i = fabs(c2s);
  const double rci = rsqrt(c2i), ci = c2i * rci;
  const double vni = fma(ui, nx, vi * ny);
  const double irinf = rcp(P.rinf);
  const double duinf = S.dru * irinf, dvinf = S.drv * irinf;  // d u_inf / d alpha, d v_inf / d alpha
  if (vni <= -ci) return qbb[1] * S.dru + qbb[2] * S.drv + qbb[3] * S.dE;
  if (vni >= ci) {
    for (int k = 0; k < 4; k++) qmb[k] += qbb[k];
    return 0.0;
  }
  const double vninf = fma(P.uinf, nx, P.vinf * ny);
  const double rp = fma(P.tgm1, ci, vni);
  const double rm = fma(-P.tgm1, P.cinf, vninf);
  const double vnb = 0.5 * (rp + rm);
  const double cb = 0.25 * P.gm1 * (rp - rm);
  const bool out = vnb > 0.0;
  const double rho_u = out ? rhoi : P.rinf;
  const double rc_u = out ? rci : P.rcinf;
  const double acb = fabs(cb);
  const double ratio = acb * rc_u;
  double pw, dpow;  // ratio^k (k = 2 / (gam - 1)) and its derivative
  if (P.pow5) {
    const double r2 = ratio * ratio, r4 = r2 * r2;
    pw = r4 * ratio;
    dpow = 5.0 * r4;
  } else {
    pw = pow(ratio, P.tgm1);
    dpow = P.tgm1 * pow(ratio, P.tgm1 - 1.0);
  }
  const double rhob = rho_u * pw;
  const double ut = out ? fma(-vni, nx, ui) : fma(-vninf, nx, P.uinf);
  const double vt = out ? fma(-vni, ny, vi) : fma(-vninf, ny, P.vinf);
  const double ub = fma(vnb, nx, ut), vb = fma(vnb, ny, vt);
  // reverse sweep
  // qb = (rhob, rhob ub, rhob vb, pb / (gam - 1) + rhob (ub^2 + vb^2) / 2), pb = rhob cb^2 / gam
  double rhobb = qbb[0] + qbb[1] * ub + qbb[2] * vb + qbb[3] * 0.5 * fma(ub, ub, vb * vb);
  const double ubb = (qbb[1] + qbb[3] * ub) * rhob, vbb = (qbb[2] + qbb[3] * vb) * rhob;
  const double pbb = qbb[3] * P.igm1;
  rhobb += pbb * cb * cb * P.igam;
  double cbb = pbb * 2.0 * rhob * cb * P.igam;
  // ub = vnb nx + ut, vb = vnb ny + vt
  double vnbb = ubb * nx + vbb * ny;
  const double utb = ubb, vtb = vbb;
  // rhob = rho_u ratio^k, ratio = |cb| rc_u
  const double rho_ub = rhobb * pw;
  const double ratiob = rhobb * rho_u * dpow;
  cbb += ratiob * rc_u * (cb < 0.0 ? -1.0 : 1.0);
  const double rc_ub = ratiob * acb;
  double rhoib = 0.0, uib = 0.0, vib = 0.0, vnib = 0.0, rcib = 0.0, uinfb = 0.0, vinfb = 0.0, vninfb = 0.0;
  if (out) {
    rhoib += rho_ub;
    rcib += rc_ub;
    uib += utb;
    vib += vtb;
    vnib -= utb * nx + vtb * ny;
  } else {
    uinfb += utb;
    vinfb += vtb;
    vninfb -= utb * nx + vtb * ny;
  }
  // vnb = (rp + rm) / 2, cb = (gam - 1) (rp - rm) / 4
  const double rpb = 0.5 * vnbb + 0.25 * P.gm1 * cbb;
  const double rmb = 0.5 * vnbb - 0.25 * P.gm1 * cbb;
  vninfb += rmb;                          // rm = vninf - 2 c_inf / (gam - 1)
  const double cib = P.tgm1 * rpb;        // rp = vni + 2 ci / (gam - 1)
  vnib += rpb;
  uinfb += vninfb * nx;
  vinfb += vninfb * ny;
  uib += vnib * nx;
  vib += vnib * ny;
  // ci = c2i rci = sqrt(c2i), rci = c2i^(-1/2), c2i = |gam pi / rhoi|
  //   d ci / d c2i = rci / 2, d rci / d c2i = -rci^3 / 2
  const double c2ib = 0.5 * (cib - rcib * rci * rci) * rci * (c2s < 0.0 ? -1.0 : 1.0);
  const double pib = c2ib * P.gam * ir;
  double irb = c2ib * P.gam * pi;
  // pi = (gam - 1) (q3 - (q1 ui + q2 vi) / 2)
  double q1b = 0.0, q2b = 0.0, q3b = pib * P.gm1;
  const double kk = -0.5 * P.gm1 * pib;
  q1b += kk * ui;
  uib += kk * qi[1];
  q2b += kk * vi;
  vib += kk * qi[2];
  // ui = q1 ir, vi = q2 ir, ir = 1 / rhoi
  q1b += uib * ir;
  q2b += vib * ir;
  irb += uib * qi[1] + vib * qi[2];
  rhoib -= irb * ir * ir;
  qmb[0] += rhoib;
  qmb[1] += q1b;
  qmb[2] += q2b;
  qmb[3] += q3b;
  return uinfb * duinf + vinfb * dvinf;
}

// Adds to qmb the adjoint of the interior state qi through the ghost state of types 0..2
// (src/get_bedge_q.h:23-50) and 3 (the characteristic farfield) and returns
// qbb . d(ghost)/d(alpha).
__device__ __forceinline__ double bc_state_adj(const int type, const double qi[4], const double nx, const double ny,
                                               const double qbb[4], const Phys &P, const AlphaSens &S,
                                               double qmb[4]) {
  if (type == 3) return farfield_state_adj(qi, nx, ny, P, qbb, S, qmb);
  if (type == 0) return qbb[1] * S.dru + qbb[2] * S.drv + qbb[3] * S.dE;
  if (type == 1) {
    qmb[3] += qbb[3];
    return qbb[1] * S.dru + qbb[2] * S.drv;
  }
  // wall: qb = (q0, q1 - 2 (n.q) nx, q2 - 2 (n.q) ny, q3)
  const double mnb = -2.0 * fma(qbb[1], nx, qbb[2] * ny);
  qmb[0] += qbb[0];
  qmb[1] += qbb[1] + mnb * nx;
  qmb[2] += qbb[2] + mnb * ny;
  qmb[3] += qbb[3];
  return 0.0;
}

// ---------------------------------------------------------------- adjoint element kernel
// Transposed Jacobian of one node's metric-combined fluxes (Fr = rx F + ry G, Fs = sx F + sy G)
// applied to their adjoints (r, s), written to out[4].
__device__ __forceinline__ void nodal_flux_adj(const double gm1, const double w0, const double w1, const double w2,
                                               const double w3, const double rx, const double ry, const double sx,
                                               const double sy, const double2 r01, const double2 r23,
                                               const double2 s01, const double2 s23, double *out) {
  const double ir = rcp(w0);
  const double u = w1 * ir, v = w2 * ir;
  const double p = gm1 * fma(-0.5, fma(w1, u, w2 * v), w3);
  const double ep = w3 + p;
  const double U = fma(rx, u, ry * v), V = fma(sx, u, sy * v);
  double w1b = rx * r01.x + sx * s01.x, w2b = ry * r01.x + sy * s01.x;
  w1b += r01.y * U + s01.y * V;
  w2b += r23.x * U + s23.x * V;
  const double Ub = r01.y * w1 + r23.x * w2 + r23.y * ep;
  const double Vb = s01.y * w1 + s23.x * w2 + s23.y * ep;
  double pb = rx * r01.y + ry * r23.x + sx * s01.y + sy * s23.x;
  const double epb = r23.y * U + s23.y * V;
  double w3b = epb;
  pb += epb;
  double ub = rx * Ub + sx * Vb, vb = ry * Ub + sy * Vb;
  w3b += gm1 * pb;
  const double kk = -0.5 * gm1 * pb;
  w1b += kk * u;
  ub += kk * w1;
  w2b += kk * v;
  vb += kk * w2;
  w1b += ub * ir;
  w2b += vb * ir;
  const double irb = ub * w1 + vb * w2;
  const double w0b = -irb * ir * ir;
  st2(out, w0b, w1b);
  st2(out + 2, w2b, w3b);
}

// mu: adjoint of L (per node); W: the primal state L was evaluated at.  Writes wbar (the volume
// part of G) and fluxbar (adjoint of each face slot's scaled flux).
template <int N>
__global__ void __launch_bounds__(32 * np_of(N)) adj_elem_kernel(const Inst d, const double *mu, double *wbar,
                                                                  double *fluxbar) {
  constexpr int Np = np_of(N), Nfp = N + 1, NK = nk_of(N);
  extern __shared__ double2 sm[];
  double2 *M = sm;                 // [Np][32] x 4 doubles
  double2 *Xb = sm + Np * 32 * 2;  // [NK][32] x 4 doubles
  const int lane = threadIdx.x, i = threadIdx.y;
  const int e0 = blockIdx.x * 32, e = e0 + lane;
  const bool live = e < d.K;
  double2 m01 = make_double2(0.0, 0.0), m23 = make_double2(0.0, 0.0);
  if (live) {
    m01 = ld2(mu + ((size_t)e * Np + i) * 4);
    m23 = ld2(mu + ((size_t)e * Np + i) * 4 + 2);
  }
  M[(i * 32 + lane) * 2] = m01;
  M[(i * 32 + lane) * 2 + 1] = m23;
  __syncthreads();
  // transposed contraction: Xb[k] = sum_i A[i][k] mu_i, column k handled by warp k mod Np
  for (int k = i; k < NK; k += Np) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
#pragma unroll
    for (int r = 0; r < Np; r++) {
      const double cc = opA<N>(r * NK + k);
      const double2 x01 = M[(r * 32 + lane) * 2], x23 = M[(r * 32 + lane) * 2 + 1];
      a0 = fma(cc, x01.x, a0);
      a1 = fma(cc, x01.y, a1);
      a2 = fma(cc, x23.x, a2);
      a3 = fma(cc, x23.y, a3);
    }
    Xb[(k * 32 + lane) * 2] = make_double2(a0, a1);
    Xb[(k * 32 + lane) * 2 + 1] = make_double2(a2, a3);
  }
  __syncthreads();
  // face-slot adjoints, contiguous per block of cells
  for (int j = i * 32 + lane; j < 3 * Nfp * 32; j += 32 * Np) {
    const int f = j >> 5, el = j & 31;
    if (e0 + el < d.K) {
      double *o = fluxbar + (((size_t)(e0 + el)) * 3 * Nfp + f) * 4;
      const double2 a = Xb[((2 * Np + f) * 32 + el) * 2], b = Xb[((2 * Np + f) * 32 + el) * 2 + 1];
      st2(o, a.x, a.y);
      st2(o + 2, b.x, b.y);
    }
  }
  if (!live) return;
  // nodal flux Jacobians transposed: Fr = rx F + ry G, Fs = sx F + sy G of node i
  const double *wp = d.W + ((size_t)e * Np + i) * 4;
  const double2 wa = ld2(wp), wb = ld2(wp + 2);
  const double w0 = wa.x, w1 = wa.y, w2 = wb.x, w3 = wb.y;
  const double2 ga = ld2(d.geo + (size_t)e * 16), gb = ld2(d.geo + (size_t)e * 16 + 2);
  const double rx = ga.x, ry = ga.y, sx = gb.x, sy = gb.y;
  const double2 r01 = Xb[(i * 32 + lane) * 2], r23 = Xb[(i * 32 + lane) * 2 + 1];
  const double2 s01 = Xb[((Np + i) * 32 + lane) * 2], s23 = Xb[((Np + i) * 32 + lane) * 2 + 1];
  nodal_flux_adj(d.P.gm1, w0, w1, w2, w3, rx, ry, sx, sy, r01, r23, s01, s23,
                 wbar + ((size_t)e * Np + i) * 4);
}


// adj_elem_kernel in even/odd form.  The forward operator factors as A = R S B (B: input
// butterfly, S: the even and odd blocks, R: output recombination), so A^T = B^T S^T R^T: the
// node adjoints are combined pairwise into even and odd rows (R^T), the blocks are applied
// transposed (about half the multiply-adds of the dense columns) and each original column is
// read back as a sum or difference of an even and an odd column (B^T).  TC: S^T on the tensor
// cores as the exact integer product of dg_ozaki.cuh (element-kernel form 2, at N = 3).
template <int N, bool TC>
__global__ void __launch_bounds__(32 * np_of(N), oz_used_t(N, TC) ? 3 : 1)
    adj_elem_kernel_sym(const Inst d, const double *mu, double *wbar, double *fluxbar) {
  constexpr int Np = np_of(N), Nfp = N + 1, NK = nk_of(N);
  constexpr int NUe = Sym<N>::NUe, NUo = Sym<N>::NUo, NRe = Sym<N>::NRe;
  extern __shared__ double2 sm[];
  // rows of 32 cells x 4 doubles, kElemSlot doubles apart (the padding keeps the tensor-core
  // fragment loads free of bank conflicts)
  constexpr int kS2 = kElemSlot / 2;
  double2 *M = sm;                 // [Np] rows: mu per node
  double2 *MS = sm + Np * kS2;     // [Np] rows: even rows, then odd rows
  double2 *XS = sm + 2 * Np * kS2; // [NK] rows: even columns, then odd columns
  const int lane = threadIdx.x, i = threadIdx.y;
  const int e0 = blockIdx.x * 32, e = e0 + lane;
  const bool live = e < d.K;
  {
    double2 m01 = make_double2(0.0, 0.0), m23 = make_double2(0.0, 0.0);
    if (live) {
      m01 = ld2(mu + ((size_t)e * Np + i) * 4);
      m23 = ld2(mu + ((size_t)e * Np + i) * 4 + 2);
    }
    M[i * kS2 + lane * 2] = m01;
    M[i * kS2 + lane * 2 + 1] = m23;
  }
  __syncthreads();
  {  // R^T: row i of the split from its node pair
    const int a = c_rin[N][2 * i], b = c_rin[N][2 * i + 1];
    double2 v01 = M[a * kS2 + lane * 2], v23 = M[a * kS2 + lane * 2 + 1];
    if (b >= 0) {
      const double2 w01 = M[b * kS2 + lane * 2], w23 = M[b * kS2 + lane * 2 + 1];
      if (i < NRe) {
        v01.x += w01.x; v01.y += w01.y; v23.x += w23.x; v23.y += w23.y;
      } else {
        v01.x -= w01.x; v01.y -= w01.y; v23.x -= w23.x; v23.y -= w23.y;
      }
    }
    MS[i * kS2 + lane * 2] = v01;
    MS[i * kS2 + lane * 2 + 1] = v23;
  }
  __syncthreads();
  // S^T: column k of the even block (k < NUe) or of the odd block
  if constexpr (oz_used_t(N, TC)) {
    oz_contract_t<N, NUe, NUo, NRe, Sym<N>::NRo, kElemSlot>(reinterpret_cast<const double *>(MS),
                                                            reinterpret_cast<double *>(XS), i, Np, lane);
  } else
  for (int k = i; k < NK; k += Np) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (k < NUe) {
#pragma unroll
      for (int r = 0; r < NRe; r++) {
        const double cc = opS<N>(r * NUe + k);
        const double2 x01 = MS[r * kS2 + lane * 2], x23 = MS[r * kS2 + lane * 2 + 1];
        a0 = fma(cc, x01.x, a0); a1 = fma(cc, x01.y, a1); a2 = fma(cc, x23.x, a2); a3 = fma(cc, x23.y, a3);
      }
    } else {
      const int kk = k - NUe;
#pragma unroll
      for (int q = 0; q < Np - NRe; q++) {
        const double cc = opS<N>(NRe * NUe + q * NUo + kk);
        const double2 x01 = MS[(NRe + q) * kS2 + lane * 2], x23 = MS[(NRe + q) * kS2 + lane * 2 + 1];
        a0 = fma(cc, x01.x, a0); a1 = fma(cc, x01.y, a1); a2 = fma(cc, x23.x, a2); a3 = fma(cc, x23.y, a3);
      }
    }
    XS[k * kS2 + lane * 2] = make_double2(a0, a1);
    XS[k * kS2 + lane * 2 + 1] = make_double2(a2, a3);
  }
  __syncthreads();
  // B^T: the adjoint of original input column c for cell el
  auto col = [&](const int c, const int el, double2 &o01, double2 &o23) {
    const int pos = c_pos[N][c];
    if (pos >= NUo && pos < NUe) {  // a column fixed by the reflection
      o01 = XS[pos * kS2 + el * 2];
      o23 = XS[pos * kS2 + el * 2 + 1];
      return;
    }
    const int p = pos < NUo ? pos : pos - NUe;
    const double2 e01 = XS[p * kS2 + el * 2], e23 = XS[p * kS2 + el * 2 + 1];
    const double2 d01 = XS[(NUe + p) * kS2 + el * 2], d23 = XS[(NUe + p) * kS2 + el * 2 + 1];
    if (pos < NUo) {
      o01 = make_double2(e01.x + d01.x, e01.y + d01.y);
      o23 = make_double2(e23.x + d23.x, e23.y + d23.y);
    } else {
      o01 = make_double2(e01.x - d01.x, e01.y - d01.y);
      o23 = make_double2(e23.x - d23.x, e23.y - d23.y);
    }
  };
  for (int j = i * 32 + lane; j < 3 * Nfp * 32; j += 32 * Np) {
    const int f = j >> 5, el = j & 31;
    if (e0 + el < d.K) {
      double2 a, b;
      col(2 * Np + f, el, a, b);
      double *o = fluxbar + (((size_t)(e0 + el)) * 3 * Nfp + f) * 4;
      st2(o, a.x, a.y);
      st2(o + 2, b.x, b.y);
    }
  }
  if (!live) return;
  double2 r01, r23, s01, s23;
  col(i, lane, r01, r23);
  col(Np + i, lane, s01, s23);
  const double *wp = d.W + ((size_t)e * Np + i) * 4;
  const double2 wa = ld2(wp), wb = ld2(wp + 2);
  const double w0 = wa.x, w1 = wa.y, w2 = wb.x, w3 = wb.y;
  const double2 ga = ld2(d.geo + (size_t)e * 16), gb = ld2(d.geo + (size_t)e * 16 + 2);
  const double rx = ga.x, ry = ga.y, sx = gb.x, sy = gb.y;
  nodal_flux_adj(d.P.gm1, w0, w1, w2, w3, rx, ry, sx, sy, r01, r23, s01, s23,
                 wbar + ((size_t)e * Np + i) * 4);
}

// The vortex state and its derivative with respect to beta (vortex_state with P.vbeta):
// rho = s^(1/(g-1)), s = 1 - k beta^2, u = 1 + beta cu, v = beta cv.
__device__ __forceinline__ void vortex_state_dbeta(double x, double y, double t, const Phys &P, double dq[4]) {
  const double dx = x - t - P.vx0, dy = y - P.vy0;
  const double r2 = dx * dx + dy * dy;
  const double e1 = exp(1.0 - r2);
  const double b = P.vbeta;
  const double cu = -e1 * (dy / (2 * M_PI)), cv = e1 * ((x - P.vx0) / (2 * M_PI));
  const double u = 1.0 + b * cu, v = b * cv;
  const double k = (P.gm1 / (16 * P.gam * M_PI * M_PI)) * exp(2 * (1.0 - r2));
  const double sb = 1.0 - k * b * b;
  const double rho = pow(sb, 1.0 / P.gm1);
  const double p = pow(rho, P.gam);
  const double drho = rho / (P.gm1 * sb) * (-2.0 * k * b);
  const double dp = P.gam * (p / rho) * drho;
  dq[0] = drho;
  dq[1] = drho * u + rho * cu;
  dq[2] = drho * v + rho * cv;
  dq[3] = dp / P.gm1 + 0.5 * drho * (u * u + v * v) + rho * (u * cu + v * cv);
}

// ---------------------------------------------------------------- adjoint face kernel
// Reverse of face_node: writes the adjoint of each cell face-node trace into tracebar slots
// [K][3][Nfp][4] (one writer each) and adds scale * (qbb . d ghost / d alpha) to galpha[tid].
template <int N>
__global__ void __launch_bounds__(256) adj_face_kernel(const Inst d, const double *fluxbar, double *tracebar,
                                                        double *galpha, const double ascale, const AlphaSens S,
                                                        const double t_stage) {
  constexpr int Np = np_of(N), Nfp = N + 1;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = (d.nE + d.nB) * Nfp;
  if (tid >= total) return;
  const int nbf = d.nB * Nfp;
  const Phys &P = d.P;
  double qm[4], qp[4], fb[4], qmb[4] = {0, 0, 0, 0}, qpb[4] = {0, 0, 0, 0};
  if (tid >= nbf) {
    const int e = (tid - nbf) / Nfp, i = (tid - nbf) - e * Nfp;
    const int4 ed = __ldg(&d.edges[e]);
    const int cL = ed.x, cR = ed.y, fL = ed.z & 3, fR = (ed.z >> 2) & 3;
    const int iR = (ed.z >> 4) ? Nfp - 1 - i : i;
    const int nodeL = __ldg(&d.fmask[fL * Nfp + i]), nodeR = __ldg(&d.fmask[fR * Nfp + iR]);
    const double *wl = d.W + ((size_t)cL * Np + nodeL) * 4;
    const double *wr = d.W + ((size_t)cR * Np + nodeR) * 4;
    double2 a = ld2(wl), b = ld2(wl + 2), c = ld2(wr), dd = ld2(wr + 2);
    qm[0] = a.x; qm[1] = a.y; qm[2] = b.x; qm[3] = b.y;
    qp[0] = c.x; qp[1] = c.y; qp[2] = dd.x; qp[3] = dd.y;
    const double *gl = d.geo + (size_t)cL * 16 + 4 + 3 * fL;
    const double nx = gl[0], ny = gl[1];
    const double sL = gl[2];
    const double sR = -d.geo[(size_t)cR * 16 + 4 + 3 * fR + 2];
    const size_t sl = (((size_t)cL * 3 + fL) * Nfp + i) * 4, sr = (((size_t)cR * 3 + fR) * Nfp + iR) * 4;
    const double2 la = ld2(fluxbar + sl), lb = ld2(fluxbar + sl + 2);
    const double2 ra = ld2(fluxbar + sr), rb = ld2(fluxbar + sr + 2);
    fb[0] = fma(sL, la.x, sR * ra.x);
    fb[1] = fma(sL, la.y, sR * ra.y);
    fb[2] = fma(sL, lb.x, sR * rb.x);
    fb[3] = fma(sL, lb.y, sR * rb.y);
    roe_flux2_adj(qm, qp, nx, ny, P, fb, qmb, qpb);
    st2(tracebar + sl, qmb[0], qmb[1]);
    st2(tracebar + sl + 2, qmb[2], qmb[3]);
    st2(tracebar + sr, qpb[0], qpb[1]);
    st2(tracebar + sr + 2, qpb[2], qpb[3]);
  } else {
    const int b = tid / Nfp, i = tid - b * Nfp;
    const int4 bd = __ldg(&d.bedges[b]);
    const int c = bd.x, f = bd.y, type = bd.z;
    const int node = __ldg(&d.fmask[f * Nfp + i]);
    const double *w = d.W + ((size_t)c * Np + node) * 4;
    double2 a = ld2(w), bb = ld2(w + 2);
    qm[0] = a.x; qm[1] = a.y; qm[2] = bb.x; qm[3] = bb.y;
    const double *g = d.geo + (size_t)c * 16 + 4 + 3 * f;
    const double nx = g[0], ny = g[1], s = g[2];
    const size_t sl = (((size_t)c * 3 + f) * Nfp + i) * 4;
    const double2 la = ld2(fluxbar + sl), lb = ld2(fluxbar + sl + 2);
    fb[0] = s * la.x; fb[1] = s * la.y; fb[2] = s * lb.x; fb[3] = s * lb.y;
    if (d.app == 1) {
      // analytic ghost state: no dependence on the interior; its beta sensitivity
      const double *xy = d.bxy + ((size_t)b * Nfp + i) * 2;
      double dqp[4];
      vortex_state(xy[0], xy[1], t_stage, P, qp);
      vortex_state_dbeta(xy[0], xy[1], t_stage, P, dqp);
      roe_flux2_adj(qm, qp, nx, ny, P, fb, qmb, qpb);
      galpha[tid] += ascale * (qpb[0] * dqp[0] + qpb[1] * dqp[1] + qpb[2] * dqp[2] + qpb[3] * dqp[3]);
    } else {
      bc_state(type, qm, nx, ny, P, qp);
      roe_flux2_adj(qm, qp, nx, ny, P, fb, qmb, qpb);
      galpha[tid] += ascale * bc_state_adj(type, qm, nx, ny, qpb, P, S, qmb);
    }
    st2(tracebar + sl, qmb[0], qmb[1]);
    st2(tracebar + sl + 2, qmb[2], qmb[3]);
  }
}

// out = ca*la + cb*lb + cc*lc + cg*(wbar + gather(tracebar)) per node (lb, lc may be null).
template <int N>
__global__ void adj_combine_kernel(const int K, double *out, const double *la, const double ca, const double *lb,
                                   const double cb, const double *lc, const double cc, const double *wbar,
                                   const double *tracebar, const double cg) {
  constexpr int Np = np_of(N), Nfp = N + 1;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)K * Np) return;
  const int e = (int)(t / Np), i = (int)(t - (long long)e * Np);
  double g[4];
  for (int v = 0; v < 4; v++) g[v] = wbar[4 * t + v];
  for (int j = 0; j < 2; j++) {
    const int k = c_fpt[N][2 * i + j];
    if (k >= 0)
      for (int v = 0; v < 4; v++) g[v] += tracebar[(((size_t)e * 3 * Nfp) + k) * 4 + v];
  }
  for (int v = 0; v < 4; v++) {
    double r = ca * la[4 * t + v] + cg * g[v];
    if (lb) r = fma(cb, lb[4 * t + v], r);
    if (lc) r = fma(cc, lc[4 * t + v], r);
    out[4 * t + v] = r;
  }
}

// Lift coefficient parts per boundary face node (0 off the wall) and their alpha derivative;
// with lam non-null, adds wscale * dC_l/dq at the wall face nodes.
template <int N>
__global__ void cl_kernel(const Inst d, const double *q, double *parts, double *dparts, double *lam,
                          const double wscale, const double inv_qinf, const double elx, const double ely,
                          const double delx, const double dely) {
  constexpr int Np = np_of(N), Nfp = N + 1;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= d.nB * Nfp) return;
  const int b = tid / Nfp, i = tid - b * Nfp;
  const int4 bd = d.bedges[b];
  double val = 0.0, dval = 0.0;
  if (bd.z == 2) {
    const int c = bd.x, f = bd.y;
    const int node = d.fmask[f * Nfp + i];
    const double *qq = q + ((size_t)c * Np + node) * 4;
    const double *g = d.geo + (size_t)c * 16;
    const double nx = g[4 + 3 * f], ny = g[5 + 3 * f], sJ = g[6 + 3 * f] * g[13];
    const double w = c_wq[N][i] * sJ * inv_qinf;
    const double ir = 1.0 / qq[0], u = qq[1] * ir, v = qq[2] * ir;
    const double p = d.P.gm1 * (qq[3] - 0.5 * (qq[1] * u + qq[2] * v));
    const double ne = nx * elx + ny * ely;
    val = w * p * ne;
    dval = w * p * (nx * delx + ny * dely);
    if (lam) {
      const double k = wscale * w * ne * d.P.gm1;
      double *l = lam + ((size_t)c * Np + node) * 4;
      atomicAdd(l + 0, k * 0.5 * (u * u + v * v));
      atomicAdd(l + 1, -k * u);
      atomicAdd(l + 2, -k * v);
      atomicAdd(l + 3, k);
    }
  }
  parts[tid] = val;
  dparts[tid] = dval;
}

// Sum of a double array in a fixed order (deterministic): one block.
__global__ void det_sum_kernel(const double *x, const int n, double *out) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int k = threadIdx.x; k < n; k += 256) acc += x[k];
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

// sum over nodes of lam . dq0/dalpha for the freestream initial state, per cell (one writer each).
template <int N>
__global__ void ic_alpha_kernel(const int K, const double *lam, const AlphaSens S, double *parts) {
  constexpr int Np = np_of(N);
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= K) return;
  double acc = 0.0;
  for (int i = 0; i < Np; i++) {
    const double *l = lam + ((size_t)e * Np + i) * 4;
    acc += l[1] * S.dru + l[2] * S.drv + l[3] * S.dE;
  }
  parts[e] = acc;
}

// Vortex objective per cell: sum over nodes and variables of (q - q_ex(t))^2 and its explicit
// beta derivative; with lam non-null adds dJ/dq = 2 (q - q_ex) (one writer per node).
template <int N>
__global__ void vortex_obj_kernel(const Inst d, const double *coords, const int *cells, const double *q,
                                  const double t, double *parts, double *dparts, double *lam) {
  constexpr int Np = np_of(N);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.K) return;
  const int a = cells[3 * c], b = cells[3 * c + 1], e = cells[3 * c + 2];
  double acc = 0.0, dacc = 0.0;
  for (int i = 0; i < Np; i++) {
    const double r = c_rs[N][i], s = c_rs[N][Np + i];
    const double x = node_coord(coords[2 * a], coords[2 * b], coords[2 * e], r, s);
    const double y = node_coord(coords[2 * a + 1], coords[2 * b + 1], coords[2 * e + 1], r, s);
    double ex[4], dex[4];
    vortex_state(x, y, t, d.P, ex);
    vortex_state_dbeta(x, y, t, d.P, dex);
    const size_t o = ((size_t)c * Np + i) * 4;
    for (int k = 0; k < 4; k++) {
      const double err = q[o + k] - ex[k];
      acc += err * err;
      dacc -= 2.0 * err * dex[k];
      if (lam) lam[o + k] += 2.0 * err;
    }
  }
  parts[c] = acc;
  dparts[c] = dacc;
}

// sum over nodes of lam . dq0/dbeta for the vortex initial state, per cell.
template <int N>
__global__ void ic_beta_kernel(const Inst d, const double *coords, const int *cells, const double *lam,
                               double *parts) {
  constexpr int Np = np_of(N);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.K) return;
  const int a = cells[3 * c], b = cells[3 * c + 1], e = cells[3 * c + 2];
  double acc = 0.0;
  for (int i = 0; i < Np; i++) {
    const double r = c_rs[N][i], s = c_rs[N][Np + i];
    const double x = node_coord(coords[2 * a], coords[2 * b], coords[2 * e], r, s);
    const double y = node_coord(coords[2 * a + 1], coords[2 * b + 1], coords[2 * e + 1], r, s);
    double dq[4];
    vortex_state_dbeta(x, y, 0.0, d.P, dq);
    const double *l = lam + ((size_t)c * Np + i) * 4;
    acc += l[0] * dq[0] + l[1] * dq[1] + l[2] * dq[2] + l[3] * dq[3];
  }
  parts[c] = acc;
}

__global__ void set_dt_kernel(StepState *st, const double *dts) {
  if (threadIdx.x | blockIdx.x) return;
  st->dt = dts[st->step];
}

// ---------------------------------------------------------------- host driver
struct Adjoint {
  Mesh mesh;
  Config cfg;
  int nsteps = 0, navg = 0, C = 0;
  Solver *fwd = nullptr;  // the forward / recompute solver (dt frozen after the recording run)
  std::vector<double> dts;
  double *d_dts = nullptr, *ckpt = nullptr, *seg = nullptr;  // checkpoints; segment q, W1, W2
  double *lam = nullptr, *lW2 = nullptr, *lW1 = nullptr, *lnew = nullptr, *wbar = nullptr;
  double *fluxbar = nullptr, *tracebar = nullptr, *galpha = nullptr, *parts = nullptr, *dparts = nullptr;
  double *scal = nullptr;  // device scalars
  double J = 0.0, dJ_dalpha = 0.0;
  bool have_forward = false;
  std::vector<void *> allocs;

  ~Adjoint() {
    for (void *p : allocs) cudaFree(p);
    delete fwd;
  }
  double *dalloc(size_t n) {
    void *p = nullptr;
    if (cudaMalloc(&p, n ? n * 8 : 16) != cudaSuccess) return nullptr;
    allocs.push_back(p);
    return (double *)p;
  }
  size_t nq() const { return fwd->q_count(); }
  size_t nslot() const { return (size_t)fwd->K * 3 * (cfg.N + 1) * 4; }
  int nbf() const { return fwd->d.nB * (cfg.N + 1); }

  AlphaSens sens() const {
    // d/d(alpha deg) of rho u = rho cos(a) V, rho v = rho sin(a) V with a = alpha * pi / 180
    const double V = std::sqrt(cfg.gam * cfg.p_inf / cfg.rho_inf) * cfg.mach;
    const double a = cfg.alpha_deg * M_PI / 180.0, k = M_PI / 180.0;
    AlphaSens S;
    S.dru = -cfg.rho_inf * V * std::sin(a) * k;
    S.drv = cfg.rho_inf * V * std::cos(a) * k;
    S.dE = 0.0;  // |V| does not change with alpha
    return S;
  }
  void lift_dirs(double &elx, double &ely, double &delx, double &dely, double &inv_qinf) const {
    const double a = cfg.alpha_deg * M_PI / 180.0, k = M_PI / 180.0;
    elx = -std::sin(a);
    ely = std::cos(a);
    delx = -std::cos(a) * k;
    dely = -std::sin(a) * k;
    const double V = std::sqrt(cfg.gam * cfg.p_inf / cfg.rho_inf) * cfg.mach;
    inv_qinf = 1.0 / (0.5 * cfg.rho_inf * V * V);
  }

  int create(const Config &c, const Mesh &m, int nsteps_, int navg_, int C_, std::string &err) {
    if (c.app != 0 && c.app != 1) { err = "app must be 0 (airfoil) or 1 (vortex)"; return -1; }
    if (nsteps_ < 1 || navg_ < 1 || navg_ > nsteps_ || C_ < 1) { err = "bad step counts"; return -1; }
    cfg = c;
    mesh = m;
    nsteps = nsteps_;
    navg = navg_;
    C = C_;
    fwd = new Solver();
    if (int rc = fwd->create(cfg, mesh, err)) return rc;
    const int nck = (nsteps + C - 1) / C + 1;
    d_dts = dalloc(nsteps + 1);
    ckpt = dalloc((size_t)nck * nq());
    seg = dalloc((size_t)3 * C * nq());
    lam = dalloc(nq()); lW2 = dalloc(nq()); lW1 = dalloc(nq()); lnew = dalloc(nq()); wbar = dalloc(nq());
    fluxbar = dalloc(nslot()); tracebar = dalloc(nslot());
    galpha = dalloc(std::max(nbf(), fwd->K));
    parts = dalloc(std::max(nbf(), fwd->K)); dparts = dalloc(std::max(nbf(), fwd->K));
    scal = dalloc(16);
    for (void *p : allocs)
      if (!p) { err = "cudaMalloc failed"; return -100; }
    // per-order tables: face quadrature weights and node -> face points
    Operators o;
    build_operators(cfg.N, o);
    const int Np = o.Np, Nfp = o.Nfp;
    double wq[8] = {0};
    {
      // weights = row sums of the 1-D face mass matrix inv(V1 V1^T) on the face-node coordinates
      std::vector<double> x(Nfp);
      for (int k = 0; k < Nfp; k++) x[k] = o.r[o.FMASK[k]];
      // Legendre-normalised Vandermonde and its Gram inverse, small dense solve
      std::vector<double> V((size_t)Nfp * Nfp), G((size_t)Nfp * Nfp, 0.0);
      for (int k = 0; k < Nfp; k++) {
        double p0 = 1.0 / std::sqrt(2.0), p1 = std::sqrt(1.5) * x[k];
        for (int j = 0; j < Nfp; j++) {
          double pj;
          if (j == 0) pj = p0;
          else if (j == 1) pj = p1;
          else {
            double pm2 = 1.0 / std::sqrt(2.0), pm1 = std::sqrt(1.5) * x[k];
            for (int n = 1; n < j; n++) {
              const double an = n / std::sqrt((2.0 * n - 1) * (2.0 * n + 1));
              const double an1 = (n + 1) / std::sqrt((2.0 * n + 1) * (2.0 * n + 3));
              const double pn1 = (x[k] * pm1 - an * pm2) / an1;
              pm2 = pm1;
              pm1 = pn1;
            }
            pj = pm1;
          }
          V[(size_t)k * Nfp + j] = pj;
        }
      }
      // mass = (V V^T)^-1, weights w = mass * 1  <=>  (V V^T) w = 1
      for (int r = 0; r < Nfp; r++)
        for (int s2 = 0; s2 < Nfp; s2++) {
          double acc = 0.0;
          for (int j = 0; j < Nfp; j++) acc += V[(size_t)r * Nfp + j] * V[(size_t)s2 * Nfp + j];
          G[(size_t)r * Nfp + s2] = acc;
        }
      std::vector<double> rhs(Nfp, 1.0);
      for (int col = 0; col < Nfp; col++) {  // Gaussian elimination with partial pivoting
        int piv = col;
        for (int r = col + 1; r < Nfp; r++)
          if (std::fabs(G[(size_t)r * Nfp + col]) > std::fabs(G[(size_t)piv * Nfp + col])) piv = r;
        for (int j = 0; j < Nfp; j++) std::swap(G[(size_t)col * Nfp + j], G[(size_t)piv * Nfp + j]);
        std::swap(rhs[col], rhs[piv]);
        for (int r = col + 1; r < Nfp; r++) {
          const double f = G[(size_t)r * Nfp + col] / G[(size_t)col * Nfp + col];
          for (int j = col; j < Nfp; j++) G[(size_t)r * Nfp + j] -= f * G[(size_t)col * Nfp + j];
          rhs[r] -= f * rhs[col];
        }
      }
      for (int r = Nfp - 1; r >= 0; r--) {
        double acc = rhs[r];
        for (int j = r + 1; j < Nfp; j++) acc -= G[(size_t)r * Nfp + j] * wq[j];
        wq[r] = acc / G[(size_t)r * Nfp + r];
      }
    }
    int fpt[28 * 2];
    for (int k = 0; k < 56; k++) fpt[k] = -1;
    for (int k = 0; k < 3 * Nfp; k++) {
      const int node = o.FMASK[k];
      if (fpt[2 * node] < 0) fpt[2 * node] = k;
      else fpt[2 * node + 1] = k;
    }
    (void)Np;
    cudaError_t ce = cudaMemcpyToSymbol(c_wq, wq, sizeof(wq), (size_t)cfg.N * sizeof(wq));
    if (ce == cudaSuccess) ce = cudaMemcpyToSymbol(c_fpt, fpt, sizeof(fpt), (size_t)cfg.N * sizeof(fpt));
    if (ce == cudaSuccess) {
      DG_DISPATCH(cfg.N, {
        const size_t sm = (size_t)(np_of(NN) + nk_of(NN)) * 32 * 4 * sizeof(double);
        ce = cudaFuncSetAttribute(adj_elem_kernel<NN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        for (auto k : {adj_elem_kernel_sym<NN, false>, adj_elem_kernel_sym<NN, true>})
          if (ce == cudaSuccess)
            ce = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)((size_t)(2 * np_of(NN) + nk_of(NN)) * kElemSlot * sizeof(double)));
      });
    }
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    return fwd->init(err);  // a defined state (t = 0, dt) for rhs_vjp before any forward run
  }

  // Vortex objective of q at time t with the solver s's parameters: J and its explicit beta part.
  cudaError_t vortex_objective(const Solver &s, const double *q, double t, double *lamacc, double *J_out,
                               double *dJ_out) {
    DG_DISPATCH(cfg.N, (vortex_obj_kernel<NN><<<(s.K + 127) / 128, 128, 0, s.stream>>>(
                           s.d, s.coords_d, s.cells_d, q, t, parts, dparts, lamacc)));
    det_sum_kernel<<<1, 256, 0, s.stream>>>(parts, s.K, scal + 6);
    det_sum_kernel<<<1, 256, 0, s.stream>>>(dparts, s.K, scal + 7);
    double h[2];
    cudaError_t ce = cudaMemcpyAsync(h, scal + 6, 16, cudaMemcpyDeviceToHost, s.stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s.stream);
    if (J_out) *J_out = h[0];
    if (dJ_out) *dJ_out = h[1];
    return ce;
  }

  // Times at the start of each step (t_n, accumulated in the device's order: t += dt).
  std::vector<double> step_times() const {
    std::vector<double> t(nsteps + 1, 0.0);
    for (int n = 0; n < nsteps; n++) t[n + 1] = t[n] + dts[n];
    return t;
  }

  // C_l of the solver's current q (device), optional gradient accumulation into lam.
  cudaError_t lift(const Solver &s, double *lamacc, double wscale, double *cl_out, double *dcl_out) {
    double elx, ely, delx, dely, iq;
    lift_dirs(elx, ely, delx, dely, iq);
    const int n = nbf();
    if (n == 0) {
      *cl_out = 0.0;
      *dcl_out = 0.0;
      return cudaSuccess;
    }
    DG_DISPATCH(cfg.N, (cl_kernel<NN><<<(n + 127) / 128, 128, 0, s.stream>>>(s.d, s.d.q, parts, dparts, lamacc,
                                                                            wscale, iq, elx, ely, delx, dely)));
    det_sum_kernel<<<1, 256, 0, s.stream>>>(parts, n, scal);
    det_sum_kernel<<<1, 256, 0, s.stream>>>(dparts, n, scal + 1);
    double h[2];
    cudaError_t ce = cudaMemcpyAsync(h, scal, 16, cudaMemcpyDeviceToHost, s.stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s.stream);
    *cl_out = h[0];
    *dcl_out = h[1];
    return ce;
  }

  // The recording forward run from the solver's initial state: real dt sequence, checkpoints.
  int forward(std::string &err) {
    Solver &s = *fwd;
    if (int rc = s.init(err)) return rc;
    s.d.dt_mode = cfg.app == 1 ? cfg.dt_mode : 0;
    s.d.dt_hist = d_dts;
    s.d.dt_hist_len = (unsigned long long)nsteps + 1;
    double acc = 0.0, dacc = 0.0;
    for (int n = 0; n < nsteps; n++) {
      if (n % C == 0)
        if (cudaMemcpyAsync(ckpt + (size_t)(n / C) * nq(), s.d.q, nq() * 8, cudaMemcpyDeviceToDevice, s.stream) !=
            cudaSuccess) { err = "checkpoint copy"; return -100; }
      s.enqueue_step(s.stream);
      if (cfg.app == 0 && n + 1 > nsteps - navg) {
        double cl, dcl;
        if (lift(s, nullptr, 0.0, &cl, &dcl) != cudaSuccess) { err = "lift"; return -100; }
        acc += cl;
        dacc += dcl;
      }
    }
    dts.assign(nsteps, 0.0);
    cudaError_t ce = cudaMemcpyAsync(dts.data(), d_dts, nsteps * 8, cudaMemcpyDeviceToHost, s.stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s.stream);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    StepState st;
    if (s.state(st, err)) return -100;
    if (st.err & 1u) { err = "non-positive or non-finite density in the forward run"; return -200; }
    s.d.dt_hist = nullptr;
    s.d.dt_hist_len = 0;
    if (cfg.app == 1) {
      if (vortex_objective(s, s.d.q, step_times()[nsteps], nullptr, &J, &dJ_dalpha) != cudaSuccess) {
        err = "vortex objective";
        return -100;
      }
    } else {
      J = acc / navg;
      dJ_dalpha = dacc / navg;  // explicit part; completed in backward()
    }
    have_forward = true;
    return 0;
  }

  // Re-run step n from the state in s (frozen dt), keeping q, W1, W2 in seg slot j.
  void recompute_step(int n, int j, cudaStream_t st) {
    Solver &s = *fwd;
    double *qj = seg + (size_t)(3 * j) * nq(), *w1 = qj + nq(), *w2 = w1 + nq();
    set_dt_kernel<<<1, 32, 0, st>>>(s.d.st, d_dts);
    cudaMemcpyAsync(qj, s.d.q, nq() * 8, cudaMemcpyDeviceToDevice, st);
    DG_DISPATCH(cfg.N, {
      launch_stage<NN>(s.d, 0, st);
      cudaMemcpyAsync(w1, s.d.W, nq() * 8, cudaMemcpyDeviceToDevice, st);
      launch_stage<NN>(s.d, 1, st);
      cudaMemcpyAsync(w2, s.d.W, nq() * 8, cudaMemcpyDeviceToDevice, st);
      launch_stage<NN>(s.d, 2, st);
    });
    finalize_kernel<<<1, 32, 0, st>>>(s.d.st, 1, nullptr, 0);
    (void)n;
  }

  // G(W, v) into wbar/tracebar, then out = combination (see adj_combine_kernel).
  void apply_G(const double *W, const double *v, double ascale, cudaStream_t st, double t_stage) {
    Inst d = fwd->d;
    d.W = const_cast<double *>(W);
    const AlphaSens S = sens();
    const int total = (d.nE + d.nB) * (cfg.N + 1);
    DG_DISPATCH(cfg.N, {
      if (g_elem_variant) {
        const size_t sm = (size_t)(2 * np_of(NN) + nk_of(NN)) * kElemSlot * sizeof(double);
        if (g_elem_variant >= 2 && oz_used_t(NN, true))
          adj_elem_kernel_sym<NN, true><<<(d.K + 31) / 32, dim3(32, np_of(NN)), sm, st>>>(d, v, wbar, fluxbar);
        else
          adj_elem_kernel_sym<NN, false><<<(d.K + 31) / 32, dim3(32, np_of(NN)), sm, st>>>(d, v, wbar, fluxbar);
      } else {
        const size_t sm = (size_t)(np_of(NN) + nk_of(NN)) * 32 * 4 * sizeof(double);
        adj_elem_kernel<NN><<<(d.K + 31) / 32, dim3(32, np_of(NN)), sm, st>>>(d, v, wbar, fluxbar);
      }
      // 124 registers: 64-thread blocks (8 per SM) balance the last wave better than 256
      adj_face_kernel<NN><<<(total + 63) / 64, 64, 0, st>>>(d, fluxbar, tracebar, galpha, ascale, S, t_stage);
    });
  }

  void combine(double *out, const double *la, double ca, const double *lb, double cb, const double *lc, double cc,
               double cg, cudaStream_t st) {
    const long long n = (long long)fwd->K * np_of(cfg.N);
    DG_DISPATCH(cfg.N, (adj_combine_kernel<NN><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
                           fwd->K, out, la, ca, lb, cb, lc, cc, wbar, tracebar, cg)));
  }

  int backward(double *dq0_host, std::string &err) {
    if (!have_forward) { err = "call forward first"; return -1; }
    Solver &s = *fwd;
    cudaStream_t st = s.stream;
    s.d.dt_mode = 1;  // recomputation uses the recorded dt sequence
    cudaMemsetAsync(lam, 0, nq() * 8, st);
    cudaMemsetAsync(galpha, 0, (size_t)std::max(nbf(), fwd->K) * 8, st);
    double dcl_unused;
    const int nseg = (nsteps + C - 1) / C;
    const std::vector<double> tn = step_times();
    for (int sg = nseg - 1; sg >= 0; sg--) {
      const int n0 = sg * C, n1 = std::min(nsteps, n0 + C);
      // restore the checkpoint and recompute the segment with the frozen dt sequence
      StepState s0;
      std::memset(&s0, 0, sizeof(s0));
      s0.cfl = cfg.cfl;
      s0.step = (unsigned long long)n0;
      s0.t = tn[n0];
      cudaMemcpyAsync(s.d.st, &s0, sizeof(s0), cudaMemcpyHostToDevice, st);
      cudaMemcpyAsync(s.d.q, ckpt + (size_t)sg * nq(), nq() * 8, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(s.d.W, s.d.q, nq() * 8, cudaMemcpyDeviceToDevice, st);
      for (int n = n0; n < n1; n++) recompute_step(n, n - n0, st);
      for (int n = n1 - 1; n >= n0; n--) {
        // objective term of q_{n+1}
        if (cfg.app == 1) {
          if (n + 1 == nsteps) {
            Inst dq = s.d;
            DG_DISPATCH(cfg.N, (vortex_obj_kernel<NN><<<(s.K + 127) / 128, 128, 0, st>>>(
                                   dq, s.coords_d, s.cells_d, s.d.q, tn[nsteps], parts, dparts, lam)));
          }
        } else if (n + 1 > nsteps - navg) {
          // C_l gradient needs q_{n+1}: the next slot's q, or the final state for the last step
          const double *qn1 = (n + 1 < n1) ? seg + (size_t)(3 * (n + 1 - n0)) * nq() : s.d.q;
          Inst dq = s.d;
          dq.q = const_cast<double *>(qn1);
          double elx, ely, delx, dely, iq;
          lift_dirs(elx, ely, delx, dely, iq);
          const int nb = nbf();
          if (nb) DG_DISPATCH(cfg.N, (cl_kernel<NN><<<(nb + 127) / 128, 128, 0, st>>>(
                                         dq, qn1, parts, dparts, lam, 1.0 / navg, iq, elx, ely, delx, dely)));
        }
        const double dt = dts[n];
        const double *qj = seg + (size_t)(3 * (n - n0)) * nq(), *w1 = qj + nq(), *w2 = w1 + nq();
        // stage boundary times as the forward face kernel forms them: t, t + dt, t + dt/2
        apply_G(w2, lam, (2.0 / 3.0) * dt, st, tn[n] + 0.5 * dt);
        combine(lW2, lam, 2.0 / 3.0, nullptr, 0.0, nullptr, 0.0, (2.0 / 3.0) * dt, st);
        apply_G(w1, lW2, 0.25 * dt, st, tn[n] + 1.0 * dt);
        combine(lW1, lW2, 0.25, nullptr, 0.0, nullptr, 0.0, 0.25 * dt, st);
        apply_G(qj, lW1, dt, st, tn[n] + 0.0 * dt);
        combine(lnew, lam, 1.0 / 3.0, lW2, 0.75, lW1, 1.0, dt, st);
        std::swap(lam, lnew);
      }
    }
    (void)dcl_unused;
    // parameter: boundary terms (galpha, per boundary face node) + initial state + explicit part
    if (cfg.app == 1) {
      DG_DISPATCH(cfg.N, (ic_beta_kernel<NN><<<(fwd->K + 127) / 128, 128, 0, st>>>(fwd->d, fwd->coords_d,
                                                                                  fwd->cells_d, lam, parts)));
    } else {
      const AlphaSens S = sens();
      DG_DISPATCH(cfg.N, (ic_alpha_kernel<NN><<<(fwd->K + 127) / 128, 128, 0, st>>>(fwd->K, lam, S, parts)));
    }
    det_sum_kernel<<<1, 256, 0, st>>>(parts, fwd->K, scal + 2);
    det_sum_kernel<<<1, 256, 0, st>>>(galpha, nbf(), scal + 3);
    double h[2];
    cudaError_t ce = cudaMemcpyAsync(h, scal + 2, 16, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess && dq0_host) ce = cudaMemcpyAsync(dq0_host, lam, nq() * 8, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    grad_alpha = dJ_dalpha + h[0] + h[1];
    return 0;
  }
  double grad_alpha = 0.0;

  // out = (dL/dW at W)^T v and v . dL/dalpha for one right-hand side (host arrays).
  int rhs_vjp(const double *W_host, const double *v_host, double *out_host, double *alpha_part, std::string &err) {
    Solver &s = *fwd;
    cudaStream_t st = s.stream;
    double *dW = seg, *dv = seg + nq();  // scratch: the segment buffers are free outside backward()
    cudaMemcpyAsync(dW, W_host, nq() * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(dv, v_host, nq() * 8, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(galpha, 0, (size_t)std::max(nbf(), fwd->K) * 8, st);
    StepState cur;
    if (fwd->state(cur, err)) return -100;
    apply_G(dW, dv, 1.0, st, cur.t + 0.5 * cur.dt);  // the boundary time of Solver::rhs
    cudaMemsetAsync(lW1, 0, nq() * 8, st);
    combine(lnew, lW1, 0.0, nullptr, 0.0, nullptr, 0.0, 1.0, st);
    det_sum_kernel<<<1, 256, 0, st>>>(galpha, nbf(), scal + 5);
    cudaError_t ce = cudaMemcpyAsync(out_host, lnew, nq() * 8, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(alpha_part, scal + 5, 8, cudaMemcpyDeviceToHost, st);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    return 0;
  }

  // J for a given parameter (alpha in degrees, or beta for the vortex) and initial state (host
  // q0, or the app's initial state if null), with the dt sequence of the recording run: the
  // function whose derivatives backward() returns.
  int evaluate(double alpha_deg, const double *q0_host, double *J_out, std::string &err) {
    if (!have_forward) { err = "call forward first"; return -1; }
    Config c2 = cfg;
    if (cfg.app == 1) c2.vortex_beta = alpha_deg;
    else c2.alpha_deg = alpha_deg;
    c2.dt_mode = 1;
    Solver s;
    if (int rc = s.create(c2, mesh, err)) return rc;
    if (int rc = s.init(err)) return rc;
    if (q0_host) {
      cudaMemcpyAsync(s.d.q, q0_host, nq() * 8, cudaMemcpyHostToDevice, s.stream);
      cudaMemcpyAsync(s.d.W, s.d.q, nq() * 8, cudaMemcpyDeviceToDevice, s.stream);
    }
    Adjoint tmp;  // lift() helper state for this alpha
    tmp.cfg = c2;
    tmp.fwd = nullptr;
    double acc = 0.0;
    for (int n = 0; n < nsteps; n++) {
      set_dt_kernel<<<1, 32, 0, s.stream>>>(s.d.st, d_dts);
      s.enqueue_step(s.stream);
      if (cfg.app == 0 && n + 1 > nsteps - navg) {
        double elx, ely, delx, dely, iq;
        tmp.lift_dirs(elx, ely, delx, dely, iq);
        const int nb = s.d.nB * (cfg.N + 1);
        if (nb) {
          DG_DISPATCH(cfg.N, (cl_kernel<NN><<<(nb + 127) / 128, 128, 0, s.stream>>>(
                                 s.d, s.d.q, parts, dparts, nullptr, 0.0, iq, elx, ely, delx, dely)));
          det_sum_kernel<<<1, 256, 0, s.stream>>>(parts, nb, scal + 4);
          double h;
          cudaMemcpyAsync(&h, scal + 4, 8, cudaMemcpyDeviceToHost, s.stream);
          cudaStreamSynchronize(s.stream);
          acc += h;
        }
      }
    }
    cudaError_t ce = cudaStreamSynchronize(s.stream);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    if (ce == cudaSuccess && cfg.app == 1) {
      // s carries this evaluation's beta; the scratch (parts, scal) is this instance's
      ce = vortex_objective(s, s.d.q, step_times()[nsteps], nullptr, J_out, nullptr);
      if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
      return 0;
    }
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    *J_out = acc / navg;
    return 0;
  }
};

// C++ interface shaped like torch.autograd.Function: forward(ctx, alpha, q0) -> J saves what
// backward needs in ctx; backward(ctx, dL/dJ) -> (dL/dalpha, dL/dq0).
struct LiftObjective {
  struct Context {
    Adjoint adj;
  };
  static int forward(Context &ctx, std::string &err, double *J) {
    if (int rc = ctx.adj.forward(err)) return rc;
    *J = ctx.adj.J;
    return 0;
  }
  static int backward(Context &ctx, double grad_J, double *grad_alpha, double *grad_q0_host, std::string &err) {
    if (int rc = ctx.adj.backward(grad_q0_host, err)) return rc;
    *grad_alpha = grad_J * ctx.adj.grad_alpha;
    if (grad_q0_host && grad_J != 1.0)
      for (size_t k = 0; k < ctx.adj.nq(); k++) grad_q0_host[k] *= grad_J;
    return 0;
  }
};

}  // namespace dg

// ---------------------------------------------------------------- adjoint C ABI
#include <thread>

#include "dg_handles.h"
struct dg_adjoint_t {
  dg::LiftObjective::Context ctx;
};

namespace {
thread_local std::string g_adj_err;
int adj_fail(int code, const std::string &m) {
  g_adj_err = m;
  return code;
}
}  // namespace

extern "C" const char *dg_adjoint_last_error(void) { return g_adj_err.c_str(); }

extern "C" int dg_adjoint_create(const dg_config_t *c, const dg_mesh_t *mesh, int nsteps, int navg,
                                 int checkpoint_every, dg_adjoint_t **out) {
  if (!c || !mesh || !out) return adj_fail(DG_ERR_ARG, "bad arguments");
  if (c->N < 1 || c->N > 6 || !(c->cfl > 0.0) || !(c->gam > 1.0) || !(c->rho_inf > 0.0) || !(c->p_inf > 0.0))
    return adj_fail(DG_ERR_ARG, "bad configuration");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return adj_fail(DG_ERR_CUDA, "no CUDA device");
  dg::Config cfg;
  cfg.N = c->N; cfg.app = c->app; cfg.dt_mode = c->app == 1 ? c->dt_mode : 0; cfg.cfl = c->cfl; cfg.gam = c->gam;
  cfg.mach = c->mach; cfg.alpha_deg = c->alpha_deg; cfg.p_inf = c->p_inf; cfg.rho_inf = c->rho_inf;
  cfg.vortex_x0 = c->vortex_x0; cfg.vortex_y0 = c->vortex_y0; cfg.vortex_beta = c->vortex_beta;
  auto *h = new (std::nothrow) dg_adjoint_t();
  if (!h) return adj_fail(DG_ERR_ARG, "out of host memory");
  std::string err;
  if (int rc = h->ctx.adj.create(cfg, mesh->m, nsteps, navg, checkpoint_every, err)) {
    delete h;
    return adj_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  }
  *out = h;
  return 0;
}

extern "C" int dg_adjoint_forward(dg_adjoint_t *h, double *J) {
  if (!h || !J) return adj_fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  const int rc = dg::LiftObjective::forward(h->ctx, err, J);
  if (rc == -200) return adj_fail(DG_ERR_NONPHYSICAL, err);
  if (rc) return adj_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  return 0;
}

extern "C" int dg_adjoint_backward(dg_adjoint_t *h, double grad_J, double *grad_alpha, double *grad_q0) {
  if (!h || !grad_alpha) return adj_fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (int rc = dg::LiftObjective::backward(h->ctx, grad_J, grad_alpha, grad_q0, err))
    return adj_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  return 0;
}

// Runs job(i) for every instance in its own host thread on the caller's device; returns the
// first failing instance's code and message.
template <class F>
static int adj_for_each(int n, F job) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return adj_fail(DG_ERR_CUDA, "no current device");
  std::vector<int> rc(n, 0);
  std::vector<std::string> errs(n);
  std::vector<std::thread> th;
  th.reserve(n);
  for (int i = 0; i < n; i++)
    th.emplace_back([&, i] {
      if (cudaSetDevice(dev) != cudaSuccess) {
        rc[i] = -100;
        errs[i] = "cudaSetDevice";
        return;
      }
      rc[i] = job(i, errs[i]);
    });
  for (auto &t : th) t.join();
  for (int i = 0; i < n; i++)
    if (rc[i]) {
      const int code = rc[i] == -200 ? DG_ERR_NONPHYSICAL : rc[i] <= -100 ? DG_ERR_CUDA : DG_ERR_ARG;
      return adj_fail(code, "instance " + std::to_string(i) + ": " + errs[i]);
    }
  return 0;
}

extern "C" int dg_adjoint_batch_forward(dg_adjoint_t *const *hs, int n, double *J) {
  if (!hs || n < 1 || !J) return adj_fail(DG_ERR_ARG, "bad arguments");
  for (int i = 0; i < n; i++)
    if (!hs[i]) return adj_fail(DG_ERR_ARG, "null instance");
  return adj_for_each(n, [&](int i, std::string &err) { return dg::LiftObjective::forward(hs[i]->ctx, err, &J[i]); });
}

extern "C" int dg_adjoint_batch_backward(dg_adjoint_t *const *hs, int n, double grad_J, double *grad_param,
                                         double *const *grad_q0) {
  if (!hs || n < 1 || !grad_param) return adj_fail(DG_ERR_ARG, "bad arguments");
  for (int i = 0; i < n; i++)
    if (!hs[i]) return adj_fail(DG_ERR_ARG, "null instance");
  return adj_for_each(n, [&](int i, std::string &err) {
    return dg::LiftObjective::backward(hs[i]->ctx, grad_J, &grad_param[i], grad_q0 ? grad_q0[i] : nullptr, err);
  });
}

extern "C" int dg_adjoint_evaluate(dg_adjoint_t *h, double alpha_deg, const double *q0, double *J) {
  if (!h || !J) return adj_fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (int rc = h->ctx.adj.evaluate(alpha_deg, q0, J, err)) return adj_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  return 0;
}

extern "C" int dg_adjoint_dt_sequence(dg_adjoint_t *h, double *out, int n) {
  if (!h || !out || n < 0 || n > (int)h->ctx.adj.dts.size()) return adj_fail(DG_ERR_ARG, "bad arguments");
  for (int k = 0; k < n; k++) out[k] = h->ctx.adj.dts[k];
  return 0;
}

extern "C" int dg_adjoint_rhs_vjp(dg_adjoint_t *h, const double *W, const double *v, double *out, double *alpha_part) {
  if (!h || !W || !v || !out || !alpha_part) return adj_fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (int rc = h->ctx.adj.rhs_vjp(W, v, out, alpha_part, err)) return adj_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  return 0;
}

extern "C" void *dg_adjoint_stream(dg_adjoint_t *h) { return h && h->ctx.adj.fwd ? (void *)h->ctx.adj.fwd->stream : nullptr; }
extern "C" void dg_adjoint_free(dg_adjoint_t *h) { delete h; }

