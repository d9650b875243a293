// Tangent-linear (forward-mode) model of the plain path, the independent check of the discrete
// adjoint: for a direction (d_param, dq0) it propagates dq through the SSPRK3 steps with the
// recorded dt sequence and returns dJ = dJ/dparam d_param + dJ/dq0 . dq0 directly, without the
// adjoint's reverse sweep.  The derivative of the Roe flux and of the nodal Euler fluxes comes
// from forward-mode dual numbers run through generic copies of the forward formulas (the same
// operation sequence as roe_flux2 and the element kernel's flux block); the ghost states, the
// stage combination and the objectives are differentiated by hand.  Included at the end of
// dg_solver.cu after the adjoint (it reuses the adjoint's buffers, kernels and parameters).
#pragma once

namespace dg {
namespace tl {

using ::fabs;
using ::fma;
using ::rsqrt;
using dg::rcp;

// value and derivative
struct Dual {
  double v, d;
};

__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, fma(a.d, b.v, a.v * b.d)}; }
__device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__device__ __forceinline__ Dual &operator*=(Dual &a, Dual b) { return a = a * b; }
__device__ __forceinline__ Dual fma(Dual a, Dual b, Dual c) {
  return {fma(a.v, b.v, c.v), fma(a.d, b.v, fma(a.v, b.d, c.d))};
}
__device__ __forceinline__ Dual fma(double a, Dual b, Dual c) { return {fma(a, b.v, c.v), fma(a, b.d, c.d)}; }
__device__ __forceinline__ Dual fma(Dual a, double b, Dual c) { return {fma(a.v, b, c.v), fma(a.d, b, c.d)}; }
__device__ __forceinline__ Dual rsqrt(Dual a) {
  const double r = rsqrt(a.v);
  return {r, -0.5 * r * r * r * a.d};
}
__device__ __forceinline__ Dual rcp(Dual a) {
  const double r = rcp(a.v);
  return {r, -r * r * a.d};
}
__device__ __forceinline__ Dual fabs(Dual a) { return a.v < 0.0 ? -a : a; }
__device__ __forceinline__ Dual pow(Dual a, double k) { return {::pow(a.v, k), k * ::pow(a.v, k - 1.0) * a.d}; }
__device__ __forceinline__ double val(double a) { return a; }
__device__ __forceinline__ double val(Dual a) { return a.v; }

// farfield_state (dg_device.cuh) for a generic scalar, line for line, with the freestream
// velocity and energy as arguments (they carry the alpha derivative).
template <class T>
__device__ __forceinline__ void farfield_state_t(const T qi[4], double nx, double ny, const Phys &P, const T uinf,
                                                 const T vinf, const T einf, T qb[4]) {
  const T rhoi = qi[0], ir = rcp(rhoi);
  const T ui = qi[1] * ir, vi = qi[2] * ir;
  const T pi = P.gm1 * fma(-0.5, fma(qi[1], ui, qi[2] * vi), qi[3]);
  const T c2i = fabs(P.gam * pi * ir);
  const T rci = rsqrt(c2i), ci = c2i * rci;
  const T vni = fma(ui, nx, vi * ny);
  if (val(vni) <= -val(ci)) {
    qb[0] = T{P.rinf}; qb[1] = P.rinf * uinf; qb[2] = P.rinf * vinf; qb[3] = einf;
    return;
  }
  if (val(vni) >= val(ci)) {
    qb[0] = qi[0]; qb[1] = qi[1]; qb[2] = qi[2]; qb[3] = qi[3];
    return;
  }
  const T vninf = fma(uinf, nx, vinf * ny);
  const T rp = fma(P.tgm1, ci, vni);
  const T rm = fma(-P.tgm1, T{P.cinf}, vninf);
  const T vnb = 0.5 * (rp + rm);
  const T cb = (0.25 * P.gm1) * (rp - rm);
  const bool out = val(vnb) > 0.0;
  const T rho_u = out ? rhoi : T{P.rinf};
  const T ratio = fabs(cb) * (out ? rci : T{P.rcinf});
  T rhob;
  if (P.pow5) {
    const T r2 = ratio * ratio;
    rhob = rho_u * (r2 * r2 * ratio);
  } else {
    rhob = rho_u * pow(ratio, P.tgm1);
  }
  const T ut = out ? fma(-vni, nx, ui) : fma(-vninf, nx, uinf);
  const T vt = out ? fma(-vni, ny, vi) : fma(-vninf, ny, vinf);
  const T ub = fma(vnb, nx, ut), vb = fma(vnb, ny, vt);
  const T pb = rhob * cb * cb * P.igam;
  qb[0] = rhob;
  qb[1] = rhob * ub;
  qb[2] = rhob * vb;
  qb[3] = fma(pb, P.igm1, 0.5 * rhob * fma(ub, ub, vb * vb));
}

// roe_flux2 (dg_device.cuh) for a generic scalar, line for line.
template <class T>
__device__ __forceinline__ void roe_flux2_t(const T qm[4], const T qp[4], double nx, double ny, const Phys &P,
                                            T f2[4]) {
  const T mL = fma(nx, qm[1], ny * qm[2]);
  const T tL = fma(nx, qm[2], -ny * qm[1]);
  const T mR = fma(nx, qp[1], ny * qp[2]);
  const T tR = fma(nx, qp[2], -ny * qp[1]);
  const T PLR = qm[0] * qp[0];
  const T r = rsqrt(PLR);
  const T r2 = r * r;
  const T irL = qp[0] * r2, irR = qm[0] * r2;
  const T uL = mL * irL, vL = tL * irL;
  const T uR = mR * irR, vR = tR * irR;
  const T pL = P.gm1 * fma(-0.5, fma(mL, uL, tL * vL), qm[3]);
  const T pR = P.gm1 * fma(-0.5, fma(mR, uR, tR * vR), qp[3]);
  const T EpL = qm[3] + pL, EpR = qp[3] + pR;
  const T HL = EpL * irL, HR = EpR * irR;
  const T rho = PLR * r;
  const T R = qp[0] * r;
  const T isum = rcp(1.0 + R);
  const T u = fma(R, uR, uL) * isum;
  const T v = fma(R, vR, vL) * isum;
  const T H = fma(R, HR, HL) * isum;
  const T q2 = fma(u, u, v * v);
  const T c2 = P.gm1 * fma(-0.5, q2, H);
  const T rc = rsqrt(c2);
  const T c = c2 * rc;
  const T ic2 = rc * rc;
  const T dp = pR - pL;
  const T a = (rho * (uR - uL)) * rc;
  const T dpc2 = dp * ic2;
  T dW1 = 0.5 * (dpc2 - a);
  T dW4 = 0.5 * (dpc2 + a);
  T dW2 = (qp[0] - qm[0]) - dpc2;
  T dW3 = rho * (vR - vL);
  dW1 *= fabs(u - c);
  dW4 *= fabs(u + c);
  const T au = fabs(u);
  dW2 *= au;
  dW3 *= au;
  const T d14 = dW1 + dW4, e14 = dW4 - dW1;
  const T d0 = d14 + dW2;
  const T d1 = fma(u, d0, c * e14);
  const T d2 = fma(v, d0, dW3);
  const T d3 = fma(H, d14, fma(u * c, e14, fma(dW2, q2, dW3 * v)));
  const T g0 = (mL + mR) - d0;
  const T g1 = (fma(mL, uL, pL) + fma(mR, uR, pR)) - d1;
  const T g2 = fma(tL, uL, tR * uR) - d2;
  const T g3 = fma(uL, EpL, uR * EpR) - d3;
  f2[0] = g0;
  f2[1] = fma(nx, g1, -ny * g2);
  f2[2] = fma(ny, g1, nx * g2);
  f2[3] = g3;
}

// The element kernel's nodal fluxes with the metric terms: Fr = rx F + ry G, Fs = sx F + sy G.
template <class T>
__device__ __forceinline__ void nodal_flux_t(const T w[4], double rx, double ry, double sx, double sy, double gm1,
                                             T fr[4], T fs[4]) {
  const T ir = rcp(w[0]);
  const T u = w[1] * ir, v = w[2] * ir;
  const T p = gm1 * fma(-0.5, fma(w[1], u, w[2] * v), w[3]);
  const T ep = w[3] + p;
  const T U = fma(rx, u, ry * v), V = fma(sx, u, sy * v);
  fr[0] = fma(rx, w[1], ry * w[2]);
  fr[1] = fma(w[1], U, rx * p);
  fr[2] = fma(w[2], U, ry * p);
  fr[3] = U * ep;
  fs[0] = fma(sx, w[1], sy * w[2]);
  fs[1] = fma(w[1], V, sx * p);
  fs[2] = fma(w[2], V, sy * p);
  fs[3] = V * ep;
}

__device__ __forceinline__ void load_dual(const double *w, const double *dw, Dual q[4]) {
  for (int k = 0; k < 4; k++) q[k] = {w[k], dw[k]};
}

}  // namespace tl

// Face fluxes' derivative dflux (slot layout of Inst::flux) at W in the direction dW, d_param.
template <int N>
__global__ void __launch_bounds__(256) tlm_face_kernel(const Inst d, const double *dW, double *dflux,
                                                        const double dpar, const AlphaSens S, const double t_stage) {
  using tl::Dual;
  constexpr int Np = np_of(N), Nfp = N + 1;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (d.nE + d.nB) * Nfp) return;
  const int nbf = d.nB * Nfp;
  const Phys &P = d.P;
  Dual qm[4], qp[4], f2[4];
  if (tid >= nbf) {
    const int e = (tid - nbf) / Nfp, i = (tid - nbf) - e * Nfp;
    const int4 ed = d.edges[e];
    const int cL = ed.x, cR = ed.y, fL = ed.z & 3, fR = (ed.z >> 2) & 3;
    const int iR = (ed.z >> 4) ? Nfp - 1 - i : i;
    const size_t oL = ((size_t)cL * Np + d.fmask[fL * Nfp + i]) * 4, oR = ((size_t)cR * Np + d.fmask[fR * Nfp + iR]) * 4;
    tl::load_dual(d.W + oL, dW + oL, qm);
    tl::load_dual(d.W + oR, dW + oR, qp);
    const double *gl = d.geo + (size_t)cL * 16 + 4 + 3 * fL;
    const double sL = gl[2], sR = -d.geo[(size_t)cR * 16 + 6 + 3 * fR];
    tl::roe_flux2_t(qm, qp, gl[0], gl[1], P, f2);
    double *ol = dflux + (((size_t)cL * 3 + fL) * Nfp + i) * 4, *orr = dflux + (((size_t)cR * 3 + fR) * Nfp + iR) * 4;
    for (int k = 0; k < 4; k++) {
      ol[k] = sL * f2[k].d;
      orr[k] = sR * f2[k].d;
    }
  } else {
    const int b = tid / Nfp, i = tid - b * Nfp;
    const int4 bd = d.bedges[b];
    const int c = bd.x, f = bd.y, type = bd.z;
    const size_t o = ((size_t)c * Np + d.fmask[f * Nfp + i]) * 4;
    tl::load_dual(d.W + o, dW + o, qm);
    const double *g = d.geo + (size_t)c * 16 + 4 + 3 * f;
    const double nx = g[0], ny = g[1], s = g[2];
    if (d.app == 1) {
      const double *xy = d.bxy + ((size_t)b * Nfp + i) * 2;
      double v[4], dv[4];
      vortex_state(xy[0], xy[1], t_stage, P, v);
      vortex_state_dbeta(xy[0], xy[1], t_stage, P, dv);
      for (int k = 0; k < 4; k++) qp[k] = {v[k], dv[k] * dpar};
    } else if (type == 0) {
      qp[0] = {P.rinf, 0.0};
      qp[1] = {P.rinf * P.uinf, S.dru * dpar};
      qp[2] = {P.rinf * P.vinf, S.drv * dpar};
      qp[3] = {P.einf, S.dE * dpar};
    } else if (type == 1) {
      qp[0] = {P.rinf, 0.0};
      qp[1] = {P.rinf * P.uinf, S.dru * dpar};
      qp[2] = {P.rinf * P.vinf, S.drv * dpar};
      qp[3] = qm[3];
    } else if (type == 3) {  // characteristic farfield
      const double irinf = 1.0 / P.rinf;
      const Dual uinf = {P.uinf, S.dru * irinf * dpar}, vinf = {P.vinf, S.drv * irinf * dpar};
      tl::farfield_state_t(qm, nx, ny, P, uinf, vinf, Dual{P.einf, S.dE * dpar}, qp);
    } else {  // wall mirror (bc_state type 2)
      const Dual mn = 2.0 * tl::fma(nx, qm[1], ny * qm[2]);
      qp[0] = qm[0];
      qp[1] = tl::fma(-mn, nx, qm[1]);
      qp[2] = tl::fma(-mn, ny, qm[2]);
      qp[3] = qm[3];
    }
    tl::roe_flux2_t(qm, qp, nx, ny, P, f2);
    double *out = dflux + (((size_t)c * 3 + f) * Nfp + i) * 4;
    for (int k = 0; k < 4; k++) out[k] = s * f2[k].d;
  }
}

// dL = derivative of the right-hand side at W in the direction (dW, dflux): the nodal fluxes'
// derivatives, then the forward contraction [Drw | Dsw | -LIFT] (it is linear).
template <int N>
__global__ void __launch_bounds__(32 * np_of(N)) tlm_elem_kernel(const Inst d, const double *dW,
                                                                  const double *dflux, double *dL) {
  using tl::Dual;
  constexpr int Np = np_of(N), Nfp = N + 1, NK = nk_of(N);
  extern __shared__ double2 X[];  // [NK][32][2] double2
  const int lane = threadIdx.x, i = threadIdx.y;
  const int e0 = blockIdx.x * 32, e = e0 + lane;
  const bool live = e < d.K;
  {
    Dual fr[4] = {}, fs[4] = {};
    if (live) {
      const size_t o = ((size_t)e * Np + i) * 4;
      Dual w[4];
      tl::load_dual(d.W + o, dW + o, w);
      const double *g = d.geo + (size_t)e * 16;
      tl::nodal_flux_t(w, g[0], g[1], g[2], g[3], d.P.gm1, fr, fs);
    }
    X[(i * 32 + lane) * 2] = make_double2(fr[0].d, fr[1].d);
    X[(i * 32 + lane) * 2 + 1] = make_double2(fr[2].d, fr[3].d);
    X[((Np + i) * 32 + lane) * 2] = make_double2(fs[0].d, fs[1].d);
    X[((Np + i) * 32 + lane) * 2 + 1] = make_double2(fs[2].d, fs[3].d);
  }
  {
    const int nthr = 32 * Np, tid = i * 32 + lane;
    const size_t base = (size_t)e0 * 3 * Nfp;
    for (int j = tid; j < 32 * 3 * Nfp * 2; j += nthr) {
      const int slot = j >> 1, h = j & 1;
      const int el = slot / (3 * Nfp), f = slot - el * (3 * Nfp);
      double2 v = make_double2(0.0, 0.0);
      if (e0 + el < d.K) v = ld2(dflux + (base + slot) * 4 + 2 * h);
      X[((2 * Np + f) * 32 + el) * 2 + h] = v;
    }
  }
  __syncthreads();
  double r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0;
  for (int k = 0; k < NK; k++) {
    const double c = opA<N>(i * NK + k);
    const double2 x01 = X[(k * 32 + lane) * 2], x23 = X[(k * 32 + lane) * 2 + 1];
    r0 = fma(c, x01.x, r0);
    r1 = fma(c, x01.y, r1);
    r2 = fma(c, x23.x, r2);
    r3 = fma(c, x23.y, r3);
  }
  if (live) {
    double *o = dL + ((size_t)e * Np + i) * 4;
    st2(o, r0, r1);
    st2(o + 2, r2, r3);
  }
}

// The SSPRK3 stage of the tangent (Shu-Osher, as stage_combine):
//   0: dW = dq + dt dL;  1: dW = 3/4 dq + 1/4 (dW + dt dL);  2: dq = dW = 1/3 dq + 2/3 (dW + dt dL)
__global__ void tlm_combine_kernel(const long long n, const int stage, const double dt, double *dq, double *dW,
                                   const double *dL) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double nw = fma(dt, dL[t], stage == 0 ? dq[t] : dW[t]);
  if (stage == 0) dW[t] = nw;
  else if (stage == 1) dW[t] = fma(0.25, nw, 0.75 * dq[t]);
  else {
    const double q = fma(2.0 / 3.0, nw, (1.0 / 3.0) * dq[t]);
    dq[t] = q;
    dW[t] = q;
  }
}

// Initial-state derivative: the freestream's alpha sensitivity (airfoil) or the vortex's beta
// sensitivity, times d_param, added to dq.
template <int N>
__global__ void tlm_ic_kernel(const Inst d, const double *coords, const int *cells, const AlphaSens S,
                              const double dpar, double *dq) {
  constexpr int Np = np_of(N);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)d.K * Np) return;
  double g[4];
  if (d.app == 1) {
    const int c = (int)(t / Np), i = (int)(t - (long long)c * Np);
    const int a = cells[3 * c], b = cells[3 * c + 1], e = cells[3 * c + 2];
    const double r = c_rs[N][i], s = c_rs[N][Np + i];
    vortex_state_dbeta(node_coord(coords[2 * a], coords[2 * b], coords[2 * e], r, s),
                       node_coord(coords[2 * a + 1], coords[2 * b + 1], coords[2 * e + 1], r, s), 0.0, d.P, g);
  } else {
    g[0] = 0.0;
    g[1] = S.dru;
    g[2] = S.drv;
    g[3] = S.dE;
  }
  for (int k = 0; k < 4; k++) dq[4 * t + k] += g[k] * dpar;
}

// Lift-coefficient derivative parts per boundary face node (cl_kernel's formula differentiated).
template <int N>
__global__ void tlm_cl_kernel(const Inst d, const double *q, const double *dq, const double dpar, double *parts,
                              const double inv_qinf, const double elx, const double ely, const double delx,
                              const double dely) {
  constexpr int Np = np_of(N), Nfp = N + 1;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= d.nB * Nfp) return;
  const int b = tid / Nfp, i = tid - b * Nfp;
  const int4 bd = d.bedges[b];
  double val = 0.0;
  if (bd.z == 2) {
    const int c = bd.x, f = bd.y;
    const size_t o = ((size_t)c * Np + d.fmask[f * Nfp + i]) * 4;
    const double *qq = q + o, *dqq = dq + o;
    const double *g = d.geo + (size_t)c * 16;
    const double nx = g[4 + 3 * f], ny = g[5 + 3 * f], sJ = g[6 + 3 * f] * g[13];
    const double w = c_wq[N][i] * sJ * inv_qinf;
    const double ir = 1.0 / qq[0], u = qq[1] * ir, v = qq[2] * ir;
    const double p = d.P.gm1 * (qq[3] - 0.5 * (qq[1] * u + qq[2] * v));
    const double dp = d.P.gm1 * (dqq[3] - (u * dqq[1] + v * dqq[2]) + 0.5 * (u * u + v * v) * dqq[0]);
    val = w * (nx * elx + ny * ely) * dp + w * p * (nx * delx + ny * dely) * dpar;
  }
  parts[tid] = val;
}

// Vortex objective derivative per cell: sum 2 (q - q_ex) . (dq - dq_ex/dbeta d_param).
template <int N>
__global__ void tlm_vortex_obj_kernel(const Inst d, const double *coords, const int *cells, const double *q,
                                      const double *dq, const double t, const double dpar, double *parts) {
  constexpr int Np = np_of(N);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.K) return;
  const int a = cells[3 * c], b = cells[3 * c + 1], e = cells[3 * c + 2];
  double acc = 0.0;
  for (int i = 0; i < Np; i++) {
    const double r = c_rs[N][i], s = c_rs[N][Np + i];
    const double x = node_coord(coords[2 * a], coords[2 * b], coords[2 * e], r, s);
    const double y = node_coord(coords[2 * a + 1], coords[2 * b + 1], coords[2 * e + 1], r, s);
    double ex[4], dex[4];
    vortex_state(x, y, t, d.P, ex);
    vortex_state_dbeta(x, y, t, d.P, dex);
    const size_t o = ((size_t)c * Np + i) * 4;
    for (int k = 0; k < 4; k++) acc += 2.0 * (q[o + k] - ex[k]) * (dq[o + k] - dex[k] * dpar);
  }
  parts[c] = acc;
}

// The tangent run (after Adjoint::forward, which recorded the dt sequence): returns
// dJ = dJ/dparam d_param + dJ/dq0 . dq0 (dq0 host [K][Np][4] or null).
inline int adjoint_tangent(Adjoint &A, double dpar, const double *dq0_host, double *dJ, std::string &err) {
  if (!A.have_forward) { err = "call forward first"; return -1; }
  Solver &s = *A.fwd;
  cudaStream_t st = s.stream;
  if (int rc = s.init(err)) return rc;
  s.d.dt_mode = 1;
  const int N = A.cfg.N;
  const size_t nq = A.nq();
  double *dq = A.lam, *dW = A.lW1, *dL = A.lW2, *dflux = A.fluxbar;
  const AlphaSens S = A.sens();
  const std::vector<double> tn = A.step_times();
  cudaError_t ce = cudaSuccess;
  DG_DISPATCH(N, ce = cudaFuncSetAttribute(tlm_elem_kernel<NN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)((size_t)nk_of(NN) * 32 * 4 * sizeof(double))));
  if (ce == cudaSuccess)
    ce = dq0_host ? cudaMemcpyAsync(dq, dq0_host, nq * 8, cudaMemcpyHostToDevice, st) : cudaMemsetAsync(dq, 0, nq * 8, st);
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
  const long long nn = (long long)s.K * np_of(N);
  DG_DISPATCH(N, (tlm_ic_kernel<NN><<<(unsigned)((nn + 255) / 256), 256, 0, st>>>(s.d, s.coords_d, s.cells_d, S,
                                                                                   dpar, dq)));
  cudaMemcpyAsync(dW, dq, nq * 8, cudaMemcpyDeviceToDevice, st);
  const int total = (s.d.nE + s.d.nB) * (N + 1), nbf = A.nbf();
  const unsigned gq = (unsigned)((nq + 255) / 256);
  double elx, ely, delx, dely, iq;
  A.lift_dirs(elx, ely, delx, dely, iq);
  double acc = 0.0;
  for (int n = 0; n < A.nsteps; n++) {
    const double dt = A.dts[n];
    set_dt_kernel<<<1, 32, 0, st>>>(s.d.st, A.d_dts);
    const double ts[3] = {tn[n] + 0.0 * dt, tn[n] + 1.0 * dt, tn[n] + 0.5 * dt};
    for (int stage = 0; stage < 3; stage++) {
      DG_DISPATCH(N, {
        tlm_face_kernel<NN><<<(total + 255) / 256, 256, 0, st>>>(s.d, dW, dflux, dpar, S, ts[stage]);
        const size_t sm = (size_t)nk_of(NN) * 32 * 4 * sizeof(double);
        tlm_elem_kernel<NN><<<(s.K + 31) / 32, dim3(32, np_of(NN)), sm, st>>>(s.d, dW, dflux, dL);
      });
      tlm_combine_kernel<<<gq, 256, 0, st>>>((long long)nq, stage, dt, dq, dW, dL);
      DG_DISPATCH(N, launch_stage<NN>(s.d, stage, st));
    }
    finalize_kernel<<<1, 32, 0, st>>>(s.d.st, 1, nullptr, 0);
    if (A.cfg.app == 0 && n + 1 > A.nsteps - A.navg && nbf) {
      DG_DISPATCH(N, (tlm_cl_kernel<NN><<<(nbf + 127) / 128, 128, 0, st>>>(s.d, s.d.q, dq, dpar, A.parts, iq, elx,
                                                                          ely, delx, dely)));
      det_sum_kernel<<<1, 256, 0, st>>>(A.parts, nbf, A.scal + 8);
      double h;
      ce = cudaMemcpyAsync(&h, A.scal + 8, 8, cudaMemcpyDeviceToHost, st);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
      if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
      acc += h;
    }
  }
  if (A.cfg.app == 1) {
    DG_DISPATCH(N, (tlm_vortex_obj_kernel<NN><<<(s.K + 127) / 128, 128, 0, st>>>(
                       s.d, s.coords_d, s.cells_d, s.d.q, dq, tn[A.nsteps], dpar, A.parts)));
    det_sum_kernel<<<1, 256, 0, st>>>(A.parts, s.K, A.scal + 8);
    ce = cudaMemcpyAsync(&acc, A.scal + 8, 8, cudaMemcpyDeviceToHost, st);
  }
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
  *dJ = A.cfg.app == 1 ? acc : acc / A.navg;
  return 0;
}

}  // namespace dg

extern "C" int dg_adjoint_tangent(dg_adjoint_t *h, double d_param, const double *dq0, double *dJ) {
  if (!h || !dJ) return adj_fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (int rc = dg::adjoint_tangent(h->ctx.adj, d_param, dq0, dJ, err))
    return adj_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  return 0;
}
