// Native DG Euler solver on one GPU: the plain fused path.
//
// One SSPRK3 stage is two kernels:
//   face_kernel  one thread per face node of every interior and boundary edge: gathers both
//                traces (src/get_neighbour_q.h), builds the boundary ghost state
//                (src/get_bedge_q.h), evaluates the Roe flux once per face node
//                (src/euler_rhs.h:120-220) and writes twice it (the 1/2 is in the LIFT
//                columns), scaled by each side's fscale, into both cells' face slots.  Each
//                slot has exactly one writer: no atomics.
//   elem_kernel  32 cells x Np node-warps per block: nodal Euler fluxes combined with the
//                (affine, per-cell) metric terms, one contraction of [Drw | Dsw | -LIFT/2]
//                (operators in constant memory, warp-uniform rows) against
//                [Fr ; Fs ; flux] staged in shared memory (src/euler_rhs.h:226-247,284-286),
//                then the SSPRK3 stage combine in registers (src/set_workingQ.h,
//                src/update_Q.h, in Shu-Osher form) and, in the last stage, single-precision
//                calc_dt estimates (src/calc_dt.h) on the new state, one maximum per node-warp.
// plus a finalize kernel per step: the exact FP64 calc_dt maximum over the candidate nodes the
// estimates single out (dt_finalize_kernel), then t += dt; dt = (1/dt1)*cfl.  dt never leaves the
// device, so a whole step is a fixed launch sequence that is captured once in a CUDA graph.
//
// Data layout in HBM (K cells, order N, Np=(N+1)(N+2)/2, Nfp=N+1):
//   q, W   [K][Np][4] doubles (the reference's AoS, src/airfoil.cpp:171)
//   flux   [K][3][Nfp][4]
//   geo    [K][16]: rx, ry, sx, sy, then (nx, ny, fscale) of faces 0..2, J, and the three
//                    fscale again as floats in the last 16 bytes (the dt estimate)
//   edges  int4 {cL, cR, fL | fR << 2 | reverse << 4, 0};  bedges int4 {cell, face, type, 0}
//   bxy    [nB][Nfp][2] boundary face-node coordinates (vortex boundary)
//   dt_est [tiles][Np] floats: each node-warp's largest calc_dt estimate of the last stage
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstddef>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "dg_device.cuh"
#include "dg_mesh.h"
#include "dg_once.h"
#include "dg_ops.h"
#include "dg_solver.h"
#include "../../include/dg_gb300.h"

#define DG_DISPATCH(N_, ...)                                 \
  switch (N_) {                                              \
    case 1: { constexpr int NN = 1; __VA_ARGS__; } break;   \
    case 2: { constexpr int NN = 2; __VA_ARGS__; } break;   \
    case 3: { constexpr int NN = 3; __VA_ARGS__; } break;   \
    case 4: { constexpr int NN = 4; __VA_ARGS__; } break;   \
    case 5: { constexpr int NN = 5; __VA_ARGS__; } break;   \
    default: { constexpr int NN = 6; __VA_ARGS__; } break;  \
  }

namespace dg {

constexpr int np_of(int n) { return (n + 1) * (n + 2) / 2; }
constexpr int nk_of(int n) { return 2 * np_of(n) + 3 * (n + 1); }

// ---------------------------------------------------------------- operators in constant memory
__constant__ double c_A1[np_of(1) * nk_of(1)];
__constant__ double c_A2[np_of(2) * nk_of(2)];
__constant__ double c_A3[np_of(3) * nk_of(3)];
__constant__ double c_A4[np_of(4) * nk_of(4)];
// Orders 5 and 6 live in global memory (read-only path; warp-uniform reads): constant memory
// (64 KB) holds the other tables.
__device__ double c_A5[np_of(5) * nk_of(5)];
__device__ double c_A6[np_of(6) * nk_of(6)];
// Even/odd (reflection r <-> s) form of the same operator, per order: even rows (NRe x NUe)
// then odd rows (NRo x NUo); staging slot of each input column; per node its even row, odd
// row (-1 if on the symmetry axis) and sign.  See sym_tables().
template <int N> struct Sym;
template <> struct Sym<1> { static constexpr int NUe = 6, NUo = 6, NRe = 2, NRo = 1; };
template <> struct Sym<2> { static constexpr int NUe = 11, NUo = 10, NRe = 4, NRo = 2; };
template <> struct Sym<3> { static constexpr int NUe = 16, NUo = 16, NRe = 6, NRo = 4; };
template <> struct Sym<4> { static constexpr int NUe = 23, NUo = 22, NRe = 9, NRo = 6; };
template <> struct Sym<5> { static constexpr int NUe = 30, NUo = 30, NRe = 12, NRo = 9; };
template <> struct Sym<6> { static constexpr int NUe = 39, NUo = 38, NRe = 16, NRo = 12; };
constexpr int sym_size(int NUe, int NUo, int NRe, int NRo) { return NRe * NUe + NRo * NUo; }
__constant__ double c_S1[sym_size(6, 6, 2, 1)];
__constant__ double c_S2[sym_size(11, 10, 4, 2)];
__constant__ double c_S3[sym_size(16, 16, 6, 4)];
__constant__ double c_S4[sym_size(23, 22, 9, 6)];
__constant__ double c_S5[sym_size(30, 30, 12, 9)];
__constant__ double c_S6[sym_size(39, 38, 16, 12)];
__constant__ int c_pos[7][77];      // staging slot of input column k (Fr 0..Np-1, Fs Np.., faces 2Np..)
__constant__ int c_out[7][28 * 3];  // per node: even row, odd row or -1, sign (+1 / -1)
__constant__ int c_rin[7][28 * 2];  // per row (even rows, then odd rows): its node pair (a, b or -1)

// calc_dt face points of each volume node: up to two faces whose fscale multiplies the node's
// wave speed (-1 = none), after the index rule of src/calc_dt.h:11.
__constant__ int c_dtf[7][28 * 2];
// reference-node coordinates (r, s) per order, for node positions.
__constant__ double c_rs[7][2 * 28];

template <int N>
__device__ __forceinline__ double opA(int idx) {
  if constexpr (N == 1) return c_A1[idx];
  else if constexpr (N == 2) return c_A2[idx];
  else if constexpr (N == 3) return c_A3[idx];
  else if constexpr (N == 4) return c_A4[idx];
  else if constexpr (N == 5) return __ldg(&c_A5[idx]);
  else return __ldg(&c_A6[idx]);
}

template <int N>
__device__ __forceinline__ double opS(int idx) {
  if constexpr (N == 1) return c_S1[idx];
  else if constexpr (N == 2) return c_S2[idx];
  else if constexpr (N == 3) return c_S3[idx];
  else if constexpr (N == 4) return c_S4[idx];
  else if constexpr (N == 5) return c_S5[idx];
  else return c_S6[idx];
}

__device__ __forceinline__ double2 ld2(const double *p) { return *reinterpret_cast<const double2 *>(p); }

// Programmatic dependent launch (griddepcontrol): a kernel launched with programmatic stream
// serialisation may start while its predecessor drains.  pdl_wait() returns once the
// predecessor grid has completed and its writes are visible (a no-op without that launch
// attribute); pdl_trigger() lets this grid's successor be scheduled once every block of this
// grid has issued it or exited.  The waits are the hardware's, not spins of ours.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void st2(double *p, double a, double b) {
  *reinterpret_cast<double2 *>(p) = make_double2(a, b);
}

// Asynchronous 16-byte global -> shared copies (cp.async, completion per thread by
// cp.async.wait_all, then a block barrier for the other threads' copies).  valid = false fills
// the 16 bytes with zeros and reads nothing.
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, const bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(sa), "l"(gmem), "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

#include "dg_ozaki.cuh"

// ---------------------------------------------------------------- face kernel
// One face node (tid in [0, (nB + nE) * Nfp)): boundary face nodes come first.  PDL: the kernel
// was launched with programmatic dependent launch; the edge records, node indices and face
// geometry (fixed for the run) are loaded before waiting for the previous kernel, W and the step
// state after.  Only after that wait may the next kernel be scheduled: the element kernel reads
// W before its own wait, so it must not start while the previous element kernel still writes W.
template <int N, bool PDL = false>
__device__ __forceinline__ void face_node(const Inst &d, const int stage, const int tid) {
  constexpr int Np = np_of(N), Nfp = N + 1;
  // Boundary face nodes come first: their ghost states (characteristic farfield, vortex exp) cost
  // several times an interior node, and last they would leave a tail on a near-idle GPU.
  const int nbf = d.nB * Nfp;
  const Phys &P = d.P;
  double qm[4], qp[4], f2[4];
  if (tid >= nbf) {
    const int e = (tid - nbf) / Nfp, i = (tid - nbf) - e * Nfp;
    const int4 ed = __ldg(&d.edges[e]);
    const int cL = ed.x, cR = ed.y, fL = ed.z & 3, fR = (ed.z >> 2) & 3;
    const int iR = (ed.z >> 4) ? Nfp - 1 - i : i;
    const int nodeL = __ldg(&d.fmask[fL * Nfp + i]), nodeR = __ldg(&d.fmask[fR * Nfp + iR]);
    const double *gl = d.geo + (size_t)cL * 16 + 4 + 3 * fL;
    const double nx = __ldg(gl), ny = __ldg(gl + 1);
    const double sL = __ldg(gl + 2);
    const double sR = -__ldg(d.geo + (size_t)cR * 16 + 4 + 3 * fR + 2);
    if constexpr (PDL) {
      pdl_wait();
      pdl_trigger();
    }
    const double *wl = d.W + ((size_t)cL * Np + nodeL) * 4;
    const double *wr = d.W + ((size_t)cR * Np + nodeR) * 4;
    double2 a = ld2(wl), b = ld2(wl + 2), c = ld2(wr), dd = ld2(wr + 2);
    qm[0] = a.x; qm[1] = a.y; qm[2] = b.x; qm[3] = b.y;
    qp[0] = c.x; qp[1] = c.y; qp[2] = dd.x; qp[3] = dd.y;
    roe_flux2(qm, qp, nx, ny, P, f2);
    double *ol = d.flux + (((size_t)cL * 3 + fL) * Nfp + i) * 4;
    double *orr = d.flux + (((size_t)cR * 3 + fR) * Nfp + iR) * 4;
    st2(ol, sL * f2[0], sL * f2[1]);
    st2(ol + 2, sL * f2[2], sL * f2[3]);
    st2(orr, sR * f2[0], sR * f2[1]);
    st2(orr + 2, sR * f2[2], sR * f2[3]);
  } else {
    const int b = tid / Nfp, i = tid - b * Nfp;
    const int4 bd = __ldg(&d.bedges[b]);
    const int c = bd.x, f = bd.y, type = bd.z;
    const int node = __ldg(&d.fmask[f * Nfp + i]);
    const double *g = d.geo + (size_t)c * 16 + 4 + 3 * f;
    const double nx = __ldg(g), ny = __ldg(g + 1), s = __ldg(g + 2);
    if constexpr (PDL) {
      pdl_wait();
      pdl_trigger();
    }
    const double *w = d.W + ((size_t)c * Np + node) * 4;
    double2 a = ld2(w), bb = ld2(w + 2);
    qm[0] = a.x; qm[1] = a.y; qm[2] = bb.x; qm[3] = bb.y;
    if (d.app == 1) {
      const double frac = stage == 0 ? 0.0 : (stage == 1 ? 1.0 : 0.5);
      const double tst = d.st->t + frac * d.st->dt;
      const double *xy = d.bxy + ((size_t)b * Nfp + i) * 2;
      vortex_state(xy[0], xy[1], tst, P, qp);
    } else {
      bc_state(type, qm, nx, ny, P, qp);
    }
    roe_flux2(qm, qp, nx, ny, P, f2);
    double *o = d.flux + (((size_t)c * 3 + f) * Nfp + i) * 4;
    st2(o, s * f2[0], s * f2[1]);
    st2(o + 2, s * f2[2], s * f2[3]);
  }
}

template <int N>
__global__ void __launch_bounds__(256) face_kernel(const Inst d, const int stage) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (d.nE + d.nB) * (N + 1)) return;
  // waits for W (and the step state) of the previous kernel, then lets the element kernel start
  // its face-independent part
  face_node<N, true>(d, stage, tid);
}

// The same in 64-thread blocks compiled for 16 resident blocks per SM (at most 64 registers):
// one such block fits on an SM beside three order-3 element blocks (3 x 20,480 + 4,096 = 65,536
// registers), so face blocks of one cell range can run next to element blocks of another.
template <int N>
__global__ void __launch_bounds__(64, 16) face_kernel_r64(const Inst d, const int stage) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (d.nE + d.nB) * (N + 1)) return;
  face_node<N, true>(d, stage, tid);
}

// double -> float by truncation of the bit pattern, with integer instructions only (the
// conversion instruction occupies the FP64 pipe).  Relative error below 2^-23; magnitudes below
// 2^-126 give +-0, above the float range (and inf, NaN) +-inf.  For the dt estimate only.
__device__ __forceinline__ float f32_trunc(const double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const int e = (int)((hi >> 20) & 0x7FF) - (1023 - 127);
  const uint32_t sign = hi & 0x80000000u;
  const uint32_t mag = e <= 0 ? 0u : (e >= 255 ? 0x7F800000u : (((uint32_t)e << 23) | ((hi & 0xFFFFFu) << 3) | (lo >> 29)));
  return __uint_as_float(sign | mag);
}

// src/calc_dt.h for one node in FP64: (N+1)^2 / 2 (|v| + c) fs as the bit pattern of a
// non-negative double (fs the larger fscale of the node's faces).  The element kernel and
// dt_finalize_kernel evaluate it with the same operations, so either gives the same maximum.
template <int N>
__device__ __forceinline__ unsigned long long dt_speed_bits(const double n0, const double n1, const double n2,
                                                            const double n3, const double fs, const Phys &P) {
  const double ir = rcp(n0);
  const double u = n1 * ir, v = n2 * ir;
  const double v2 = fma(u, u, v * v);
  const double p = P.gm1 * fma(-0.5 * n0, v2, n3);
  const double cs = sqrt(fabs(P.gam * p * ir));
  const double spd = ((N + 1) * (N + 1) * 0.5) * (sqrt(v2) + cs);
  return (unsigned long long)__double_as_longlong(spd * fs);
}

// SSPRK3 stage combine of one node's right-hand side (r0..r3), and in the last stage each
// node-warp's largest single-precision calc_dt estimate (Inst::dt_est; the step's finalize takes
// the FP64 maximum).  Every thread of the node-warps calls it: `active` is false for warps beyond
// the Np node-warps of a wider block, `live` is false for lanes past the last cell (they take part
// in the warp reductions).  qs: this node's q staged in shared memory (qs[0] variables 0, 1 and
// qs[qstride] variables 2, 3; the warp-specialised kernel) or null to read it from q.
template <int N>
__device__ __forceinline__ void stage_combine(const Inst &d, const int stage, const int e, const bool active,
                                              const bool live, const int i, const int lane, const double w[4],
                                              double r0, double r1, double r2, double r3,
                                              const double2 *qs = nullptr, const int qstride = 0) {
  constexpr int Np = np_of(N);
  const Phys &P = d.P;
  const size_t off = ((size_t)(live ? e : 0) * Np + (active ? i : 0)) * 4;
  double *wp = d.W + off;
  if (stage == 3) {
    if (live) {
      double *o = d.rhs_out + off;
      st2(o, r0, r1);
      st2(o + 2, r2, r3);
    }
    return;
  }
  const double dt = d.st->dt;
  double n0 = fma(dt, r0, w[0]), n1 = fma(dt, r1, w[1]), n2 = fma(dt, r2, w[2]), n3 = fma(dt, r3, w[3]);
  if (stage == 0) {
    if (live) {
      st2(wp, n0, n1);
      st2(wp + 2, n2, n3);
    }
    return;
  }
  double *qp = d.q + off;
  double2 qa = make_double2(0.0, 0.0), qb = make_double2(0.0, 0.0);
  if (live) {
    if (qs) {
      qa = qs[0];
      qb = qs[qstride];
    } else {
      qa = ld2(qp);
      qb = ld2(qp + 2);
    }
  }
  if (stage == 1) {
    if (live) {
      n0 = fma(0.25, n0, 0.75 * qa.x);
      n1 = fma(0.25, n1, 0.75 * qa.y);
      n2 = fma(0.25, n2, 0.75 * qb.x);
      n3 = fma(0.25, n3, 0.75 * qb.y);
      st2(wp, n0, n1);
      st2(wp + 2, n2, n3);
    }
    return;
  }
  const double third = 1.0 / 3.0, two_third = 2.0 / 3.0;
  n0 = fma(two_third, n0, third * qa.x);
  n1 = fma(two_third, n1, third * qa.y);
  n2 = fma(two_third, n2, third * qb.x);
  n3 = fma(two_third, n3, third * qb.y);
  if (live) {
    st2(qp, n0, n1);
    st2(qp + 2, n2, n3);
    st2(wp, n0, n1);
    st2(wp + 2, n2, n3);
    if (bad_density(n0)) atomicOr(&d.st->err, 1u);
  }
  if (d.dt_mode == 0 && d.dt_est) {
    // src/calc_dt.h: (N+1)^2 * 0.5 * fscale * (|v| + c) at the face points of this node, maximised
    // over the mesh.  Here only a single-precision estimate (from bit-truncated copies of the
    // state, f32_trunc, and single-precision copies of fscale and gamma), within ~1e-6 of the FP64
    // value: each node-warp stores its largest estimate and combines it into the step state's
    // maximum estimate; the step's finalize (dt_finalize_kernel, batch_dt_finalize_kernel)
    // evaluates in FP64 the nodes whose estimate is within 1e-4 of that maximum, among them the
    // node of the FP64 maximum.  No barrier and no FP64 instruction here: evaluating a block's
    // candidates in this kernel (a barrier, a ~35-long FP64 chain waiting behind the other blocks'
    // FP64 work, a second barrier) held every stage-2 tile ~9k clocks.
    const int fa = active ? c_dtf[N][2 * i] : -1, fb = active ? c_dtf[N][2 * i + 1] : -1;
    float est = 0.0f;
    if (live && fa >= 0) {
      const float *gf = reinterpret_cast<const float *>(d.geo + (size_t)e * 16 + 14);  // fscale, f32
      const float fsf = fb >= 0 ? fmaxf(gf[fa], gf[fb]) : gf[fa];
      const float rho = f32_trunc(n0), ir = 1.0f / rho, u = f32_trunc(n1) * ir, v = f32_trunc(n2) * ir;
      const float v2 = u * u + v * v;
      const float p = P.gm1f * (f32_trunc(n3) - 0.5f * rho * v2);
      const float cs = sqrtf(fabsf(P.gamf * p * ir));
      est = ((N + 1) * (N + 1) * 0.5f) * (sqrtf(v2) + cs) * fsf;
      if (!(est == est) || est > 3.0e38f) est = 3.0e38f;  // non-finite: always a candidate
    }
    if (active) {
      float wm = est;
      for (int o = 16; o > 0; o >>= 1) wm = fmaxf(wm, __shfl_xor_sync(0xffffffffu, wm, o));
      if (lane == 0) {
        d.dt_est[(size_t)(e >> 5) * Np + i] = wm;
        atomicMax(&d.st->dt_est_max, __float_as_uint(wm));  // non-negative: ordered as integers
      }
    }
  }
}

// ---------------------------------------------------------------- element kernel
// stage 0: W = W + dt*L           (W holds q at the start of a step)
// stage 1: W = 3/4 q + 1/4 (W + dt*L)
// stage 2: q = W = 1/3 q + 2/3 (W + dt*L), then the calc_dt estimates of the new q
// stage 3: rhs_out = L (one right-hand side, no combine)
template <int N>
__global__ void __launch_bounds__(32 * np_of(N)) elem_kernel(const Inst d, const int stage) {
  constexpr int Np = np_of(N), Nfp = N + 1, NK = nk_of(N);
  extern __shared__ double2 X[];  // [NK][32][2] double2 = [NK][32] x 4 doubles
  const int lane = threadIdx.x, i = threadIdx.y;
  const int e0 = blockIdx.x * 32;
  const int e = e0 + lane;
  const bool live = e < d.K;
  const Phys &P = d.P;
  pdl_trigger();

  double w[4] = {0.0, 0.0, 0.0, 0.0};
  double g[4] = {0.0, 0.0, 0.0, 0.0};
  if (live) {
    const double *wp = d.W + ((size_t)e * Np + i) * 4;
    double2 a = ld2(wp), b = ld2(wp + 2);
    w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
    double2 ga = ld2(d.geo + (size_t)e * 16), gb = ld2(d.geo + (size_t)e * 16 + 2);
    g[0] = ga.x; g[1] = ga.y; g[2] = gb.x; g[3] = gb.y;
  }
  // Nodal fluxes (src/euler_rhs.h:7-23) combined with the metric terms:
  //   Fr = rx F + ry G,  Fs = sx F + sy G   (rhs = Drw Fr + Dsw Fs - LIFT flux)
  {
    const double rx = g[0], ry = g[1], sx = g[2], sy = g[3];
    double fr0 = 0, fr1 = 0, fr2 = 0, fr3 = 0, fs0 = 0, fs1 = 0, fs2 = 0, fs3 = 0;
    if (live) {
      const double ir = rcp(w[0]);
      const double u = w[1] * ir, v = w[2] * ir;
      const double p = P.gm1 * fma(-0.5, fma(w[1], u, w[2] * v), w[3]);
      const double ep = w[3] + p;
      const double U = fma(rx, u, ry * v), V = fma(sx, u, sy * v);
      fr0 = w[0] * U;  // = rx w1 + ry w2 (U = rx u + ry v), one multiply
      fr1 = fma(w[1], U, rx * p);
      fr2 = fma(w[2], U, ry * p);
      fr3 = U * ep;
      fs0 = w[0] * V;
      fs1 = fma(w[1], V, sx * p);
      fs2 = fma(w[2], V, sy * p);
      fs3 = V * ep;
    }
    X[(i * 32 + lane) * 2] = make_double2(fr0, fr1);
    X[(i * 32 + lane) * 2 + 1] = make_double2(fr2, fr3);
    X[((Np + i) * 32 + lane) * 2] = make_double2(fs0, fs1);
    X[((Np + i) * 32 + lane) * 2 + 1] = make_double2(fs2, fs3);
  }
  pdl_wait();  // the face fluxes are the face kernel's output
  // Face fluxes of the block's 32 cells: contiguous in HBM, scattered into [k][cell] order.
  {
    const int nthr = 32 * Np, tid = i * 32 + lane;
    const size_t base = (size_t)e0 * 3 * Nfp;
    for (int j = tid; j < 32 * 3 * Nfp * 2; j += nthr) {
      const int slot = j >> 1, h = j & 1;
      const int el = slot / (3 * Nfp), f = slot - el * (3 * Nfp);
      double2 v = make_double2(0.0, 0.0);
      if (e0 + el < d.K) v = ld2(d.flux + (base + slot) * 4 + 2 * h);
      X[((2 * Np + f) * 32 + el) * 2 + h] = v;
    }
  }
  __syncthreads();
  // Contraction: row i of [Drw | Dsw | -LIFT] against the staged columns.
  double r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0;
#pragma unroll
  for (int k = 0; k < NK; k++) {
    const double c = opA<N>(i * NK + k);
    const double2 x01 = X[(k * 32 + lane) * 2], x23 = X[(k * 32 + lane) * 2 + 1];
    r0 = fma(c, x01.x, r0);
    r1 = fma(c, x01.y, r1);
    r2 = fma(c, x23.x, r2);
    r3 = fma(c, x23.y, r3);
  }
  stage_combine<N>(d, stage, e, true, live, i, lane, w, r0, r1, r2, r3);
}

// The element kernel in even/odd form.  The reflection sigma: (r,s) -> (s,r) of the reference
// triangle permutes the nodes (P) and the face points (Q: face 0 <-> face 2 reversed, face 1
// reversed), maps Drw to Dsw (P Drw P = Dsw) and leaves LIFT invariant (P LIFT Q = LIFT).  So
// A = [Drw | Dsw | -LIFT] commutes with the input permutation Pi = (Fr_i <-> Fs_P(i), Q):
// P A = A Pi.  Splitting the staged inputs into sums and differences over the Pi-pairs
// ("butterfly") makes A block-diagonal: even rows on the sums give y_i + y_P(i), odd rows on the
// differences give y_i - y_P(i).  The contraction shrinks to 0.55-0.62 of the dense one.
// One tile of 32 cells starting at e0, thread (lane, node i) of a block with at least Np
// node-warps (warps with i >= Np only take part in the barriers).
// TC: 0 the even/odd contraction in FP64, 1 the even/odd blocks on the tensor cores (N = 3-5; the
// butterfly and the operand alignment by oz_prep), 2 the dense rows on the tensor cores at N = 1, 2
// (no butterfly) and form 1 at N = 3-5.
template <int N, bool PDL = false, int TC = 0>
__device__ __forceinline__ void elem_tile_sym(const Inst &d, const int stage, const int e0, const int lane,
                                              const int i, double2 *X) {
  constexpr int Np = np_of(N), Nfp = N + 1, NK = nk_of(N);
  constexpr int NUe = Sym<N>::NUe, NUo = Sym<N>::NUo, NRe = Sym<N>::NRe;
  constexpr int NPin = NUo;  // input pairs
  constexpr int kS2 = kElemSlot / 2;  // double2 per staged slot
  constexpr bool DENSE = ozd_used(N, TC);           // dense rows, slots in natural order
  constexpr bool SYMTC = !DENSE && oz_used(N, TC != 0);  // even/odd blocks on the tensor cores
  double2 *Y = X + NK * kS2;
  int *Ems = reinterpret_cast<int *>(Y + Np * kS2);  // column exponents of the prepared operands
  const int nthr = 32 * Np, tid = i * 32 + lane;
  const bool active = i < Np;
  const int e = e0 + lane;
  const bool live = active && e < d.K;
  const Phys &P = d.P;
  // the tile's face fluxes (contiguous in HBM) go straight into their slots by asynchronous
  // copies: j = tid + m*nthr, so the face point f = j / 32 is uniform in a warp
  auto stage_face_fluxes = [&]() {
    for (int j = active ? tid : 3 * Nfp * 32; j < 3 * Nfp * 32; j += nthr) {
      const int f = j >> 5, el = j & 31;
      const bool ok = e0 + el < d.K;
      const double *fp = d.flux + (((size_t)(ok ? e0 + el : 0)) * 3 * Nfp + f) * 4;
      const int pf = DENSE ? 2 * Np + f : c_pos[N][2 * Np + f];
      cp_async16(X + pf * kS2 + el * 2, fp, ok);
      cp_async16(X + pf * kS2 + el * 2 + 1, fp + 2, ok);
    }
  };

  double w[4] = {0.0, 0.0, 0.0, 0.0};
  double g[4] = {0.0, 0.0, 0.0, 0.0};
  if (live) {
    const double *wp = d.W + ((size_t)e * Np + i) * 4;
    double2 a = ld2(wp), b = ld2(wp + 2);
    w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
    double2 ga = ld2(d.geo + (size_t)e * 16), gb = ld2(d.geo + (size_t)e * 16 + 2);
    g[0] = ga.x; g[1] = ga.y; g[2] = gb.x; g[3] = gb.y;
  }
  // Without programmatic launch the face fluxes are ready: their copies overlap the nodal fluxes.
  if constexpr (!PDL) stage_face_fluxes();
  {
    const double rx = g[0], ry = g[1], sx = g[2], sy = g[3];
    double fr0 = 0, fr1 = 0, fr2 = 0, fr3 = 0, fs0 = 0, fs1 = 0, fs2 = 0, fs3 = 0;
    if (live) {
      const double ir = rcp(w[0]);
      const double u = w[1] * ir, v = w[2] * ir;
      const double p = P.gm1 * fma(-0.5, fma(w[1], u, w[2] * v), w[3]);
      const double ep = w[3] + p;
      const double U = fma(rx, u, ry * v), V = fma(sx, u, sy * v);
      fr0 = w[0] * U;  // = rx w1 + ry w2 (U = rx u + ry v), one multiply
      fr1 = fma(w[1], U, rx * p);
      fr2 = fma(w[2], U, ry * p);
      fr3 = U * ep;
      fs0 = w[0] * V;
      fs1 = fma(w[1], V, sx * p);
      fs2 = fma(w[2], V, sy * p);
      fs3 = V * ep;
    }
    if (active) {
      const int pr = DENSE ? i : c_pos[N][i], ps = DENSE ? Np + i : c_pos[N][Np + i];
      X[pr * kS2 + lane * 2] = make_double2(fr0, fr1);
      X[pr * kS2 + lane * 2 + 1] = make_double2(fr2, fr3);
      X[ps * kS2 + lane * 2] = make_double2(fs0, fs1);
      X[ps * kS2 + lane * 2 + 1] = make_double2(fs2, fs3);
    }
  }
  // Everything above reads only W, q and the metrics (written before the face kernel ran); the
  // face fluxes are the face kernel's output.
  if constexpr (PDL) {
    pdl_wait();
    stage_face_fluxes();
  }
  cp_async_wait_all();  // this thread's copies; the barrier publishes everyone's
  __syncthreads();
  if constexpr (SYMTC) {
    // the butterfly in integers and the operand alignment, once per value
    oz_prep<NUe, NUo, kElemSlot>(reinterpret_cast<double *>(X), Ems, tid);
    __syncthreads();
  } else if constexpr (!DENSE) {
    // butterfly over the input pairs: slot p <- x_a + x_b, slot NUe + p <- x_a - x_b (the
    // tensor-core form does it exactly in integers instead)
    for (int j = active ? tid : NPin * 32; j < NPin * 32; j += nthr) {
      const int p = j >> 5, el = j & 31;
      double2 *xa = X + p * kS2 + el * 2, *xb = X + (NUe + p) * kS2 + el * 2;
      const double2 a0 = xa[0], a1 = xa[1], b0 = xb[0], b1 = xb[1];
      xa[0] = make_double2(a0.x + b0.x, a0.y + b0.y);
      xa[1] = make_double2(a1.x + b1.x, a1.y + b1.y);
      xb[0] = make_double2(a0.x - b0.x, a0.y - b0.y);
      xb[1] = make_double2(a1.x - b1.x, a1.y - b1.y);
    }
    __syncthreads();
  }
  double r0 = 0.0, r1 = 0.0, r2 = 0.0, r3 = 0.0;
  if constexpr (DENSE) {
    // the dense rows on the tensor cores: Y row i is node i's right-hand side
    oz_contract_dense<N, NK, Np>(reinterpret_cast<const double *>(X), reinterpret_cast<double *>(Y), i,
                                 (int)(blockDim.x * blockDim.y) >> 5, lane);
  } else if constexpr (SYMTC) {
    // the contraction on the tensor cores (dg_ozaki.cuh), every warp of the block taking part
    oz_contract<N, NUe, NUo, NRe, Sym<N>::NRo>(reinterpret_cast<const double *>(X),
                                                     reinterpret_cast<double *>(Y), i,
                                                     (int)(blockDim.x * blockDim.y) >> 5, lane, Ems);
  } else if (!active) {
  } else if (i < NRe) {
#pragma unroll
    for (int k = 0; k < NUe; k++) {
      const double c = opS<N>(i * NUe + k);
      const double2 x01 = X[k * kS2 + lane * 2], x23 = X[k * kS2 + lane * 2 + 1];
      r0 = fma(c, x01.x, r0);
      r1 = fma(c, x01.y, r1);
      r2 = fma(c, x23.x, r2);
      r3 = fma(c, x23.y, r3);
    }
  } else {
#pragma unroll
    for (int k = 0; k < NUo; k++) {
      const double c = opS<N>(NRe * NUe + (i - NRe) * NUo + k);
      const double2 x01 = X[(NUe + k) * kS2 + lane * 2], x23 = X[(NUe + k) * kS2 + lane * 2 + 1];
      r0 = fma(c, x01.x, r0);
      r1 = fma(c, x01.y, r1);
      r2 = fma(c, x23.x, r2);
      r3 = fma(c, x23.y, r3);
    }
  }
  if (active && !DENSE && !SYMTC) {
    Y[i * kS2 + lane * 2] = make_double2(r0, r1);
    Y[i * kS2 + lane * 2 + 1] = make_double2(r2, r3);
  }
  __syncthreads();
  if (DENSE && active) {
    const double2 y01 = Y[i * kS2 + lane * 2], y23 = Y[i * kS2 + lane * 2 + 1];
    r0 = y01.x; r1 = y01.y; r2 = y23.x; r3 = y23.y;
  } else if (active) {
    const int re = c_out[N][3 * i], ro = c_out[N][3 * i + 1], sg = c_out[N][3 * i + 2];
    const double2 e01 = Y[re * kS2 + lane * 2], e23 = Y[re * kS2 + lane * 2 + 1];
    r0 = e01.x; r1 = e01.y; r2 = e23.x; r3 = e23.y;
    if (ro >= 0) {
      const double2 o01 = Y[ro * kS2 + lane * 2], o23 = Y[ro * kS2 + lane * 2 + 1];
      if (sg > 0) {
        r0 += o01.x; r1 += o01.y; r2 += o23.x; r3 += o23.y;
      } else {
        r0 -= o01.x; r1 -= o01.y; r2 -= o23.x; r3 -= o23.y;
      }
    }
  }
  if constexpr (DENSE || SYMTC) {
    // this node's W again from HBM (L2) rather than held in registers through the contraction
    // (the node is written only below, by this thread).  Keeping W and q of every node of the
    // tile in shared memory instead (+20.5 KB per block at N = 3) measured slightly slower in the
    // step graph over cell ranges (N = 3 / 4 / 5: 234.6 / 382.2 / 611 against 232.3 / 380.2 / 607 us
    // per step in runs of 40 steps; same bits).
    if (live) {
      const double *wp = d.W + ((size_t)e * Np + i) * 4;
      const double2 a = ld2(wp), b = ld2(wp + 2);
      w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
    }
  }
  stage_combine<N>(d, stage, e, active, live, i, lane, w, r0, r1, r2, r3);
  // X and Y are rewritten by the next tile only after every warp is past this point
  __syncthreads();
}

// Dynamic shared memory of the even/odd element kernels: NK staged slots, Np output rows and the
// 128 column exponents of the prepared tensor-core operands.
constexpr size_t elem_sym_smem(int N) {
  return (size_t)(nk_of(N) + np_of(N)) * kElemSlot * sizeof(double) + 128 * sizeof(int);
}

// MB: minimum resident blocks per SM the register allocation must allow (oz_min_blocks for the
// tensor-core form; at N = 3 without the bound it takes ~95 registers and runs two blocks per SM,
// measured slower).
// tile0: first 32-cell tile of this launch (a launch may cover a range of the tiles).
// PW: launched with programmatic dependence on the face kernel (its fluxes are read after the
// launch wait) or not (they are complete when the kernel starts).
template <int N, int TC, int MB = 1, bool PW = true>
__global__ void __launch_bounds__(32 * np_of(N), MB) elem_kernel_sym(const Inst d, const int stage, const int tile0) {
  extern __shared__ double2 Xs[];  // [NK][32] x 4 doubles, then [Np][32] x 4 doubles
  pdl_trigger();  // the next face kernel may be scheduled (it waits for this grid's writes)
  elem_tile_sym<N, PW, TC>(d, stage, (tile0 + (int)blockIdx.x) * 32, threadIdx.x, threadIdx.y, Xs);
}

#include "dg_elem_ws.cuh"

// ---------------------------------------------------------------- per-step finalize
// Launched with programmatic dependent launch in the step graph: it waits for the last element
// kernel (whose dt maximum it reads) and lets the next step's face kernel be scheduled meanwhile.
__global__ void finalize_kernel(StepState *st, int dt_mode, double *dt_hist, unsigned long long dt_hist_len) {
  pdl_wait();
  pdl_trigger();
  if (threadIdx.x | blockIdx.x) return;
  if (dt_hist && st->step < dt_hist_len) dt_hist[st->step] = st->dt;
  st->t += st->dt;
  st->step += 1;
  st->dt_est_max = 0u;  // a stage-2 element kernel with deferred estimates may have run (dt frozen)
  if (dt_mode == 0) {
    const double dt1 = __longlong_as_double((long long)st->dt1_bits);
    st->dt = (1.0 / dt1) * st->cfl;
    st->dt1_bits = 0ull;
  }
}

// The per-step finalize with the deferred calc_dt maximum (Inst::dt_est): with M the largest
// single-precision estimate of the mesh (the element kernel's node-warps combine theirs into the
// step state by atomicMax), the grid's warps share the node-warps whose estimate is within 1e-4
// of M and evaluate those
// nodes in FP64 from the new q (the estimates are within ~1e-6 of the FP64 values, so the node
// of the FP64 maximum is always among them and the result is the exact maximum, the same as the
// element kernel's per-block evaluation gives), combined with atomicMax; the last block to finish
// (a counter in the step state, no waiting) then advances t and sets the new dt.
// calc_dt of node i of cell e (src/calc_dt.h) in FP64 from q, as the bit pattern of a non-negative
// double; 0 for a cell past the last or a node without face points.
template <int N>
__device__ __forceinline__ unsigned long long dt_node_bits(const Inst &d, const int e, const int i) {
  constexpr int Np = np_of(N);
  const int fa = c_dtf[N][2 * i], fb = c_dtf[N][2 * i + 1];
  if (e >= d.K || fa < 0) return 0ull;
  const double *ge = d.geo + (size_t)e * 16;
  const double fs = fb >= 0 ? fmax(ge[6 + 3 * fa], ge[6 + 3 * fb]) : ge[6 + 3 * fa];
  const double *qp = d.q + ((size_t)e * Np + i) * 4;
  const double2 a = ld2(qp), b = ld2(qp + 2);
  return dt_speed_bits<N>(a.x, a.y, b.x, b.y, fs, d.P);
}

// The end of a finalize block: its warps' FP64 maxima go into the step state by atomicMax, and the
// last of the nblocks blocks of this instance's finalize (a counter in the step state, no waiting)
// advances t and the step count, records the step's dt, and sets the new dt from the maximum
// (dt recomputed) or leaves it (frozen).  The step state's other fields are not written by any
// block before that last block's update, so every block reads them first.
__device__ __forceinline__ void finalize_block_end(const Inst &d, unsigned long long best, const unsigned nblocks) {
  StepState *st = d.st;
  __shared__ int s_last;
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, best, o);
    best = x > best ? x : best;
  }
  if ((threadIdx.x & 31) == 0 && best) atomicMax(&st->dt1_bits, best);
  const double dt0 = st->dt, t0 = st->t, cfl = st->cfl;
  const unsigned long long step0 = st->step;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&st->dt_blocks, 1u) == nblocks - 1u;
  __syncthreads();
  if (!s_last || threadIdx.x) return;
  __threadfence();
  st->dt_blocks = 0u;
  st->dt_est_max = 0u;
  if (d.dt_hist && step0 < d.dt_hist_len) d.dt_hist[step0] = dt0;
  st->t = t0 + dt0;
  st->step = step0 + 1;
  if (d.dt_mode == 0) {
    const double dt1 = __longlong_as_double((long long)atomicAdd(&st->dt1_bits, 0ull));
    st->dt = (1.0 / dt1) * cfl;
    st->dt1_bits = 0ull;
  }
}

template <int N>
__global__ void __launch_bounds__(256) dt_finalize_kernel(const Inst d) {
  constexpr int Np = np_of(N);
  pdl_wait();
  pdl_trigger();
  const int n = ((d.K + 31) >> 5) * Np;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const float thr = __uint_as_float(d.st->dt_est_max) * 0.9999f;
  // warp w of the grid takes the estimates w, w + G, w + 2G, ... (G warps in the grid): its lanes
  // read 32 of them at once, and the candidates among them are evaluated one after the other,
  // each by the whole warp (lane = cell of the tile)
  unsigned long long best = 0ull;
  const int gs = gridDim.x * nw;
  for (int base = blockIdx.x * nw + warp; base < n; base += 32 * gs) {
    const int jl = base + lane * gs;
    unsigned cand = __ballot_sync(0xffffffffu, jl < n && d.dt_est[jl] >= thr);
    while (cand) {
      const int k = __ffs((int)cand) - 1;
      cand &= cand - 1u;
      const int j = base + k * gs, tile = j / Np;
      const unsigned long long v = dt_node_bits<N>(d, tile * 32 + lane, j - tile * Np);
      best = v > best ? v : best;
    }
  }
  finalize_block_end(d, best, gridDim.x);
}

// ---------------------------------------------------------------- set-up kernels
// Affine geometry from the vertices: x = -(r+s)/2 x0 + (1+r)/2 x1 + (1+s)/2 x2, so
// xr = (x1-x0)/2, xs = (x2-x0)/2; J = xr ys - xs yr; rx = ys/J, sx = -yr/J, ry = -xs/J,
// sy = xr/J; face normals as src/init_grid.h:81-105 with fscale = sJ/J.  Explicit rounding
// intrinsics keep the result independent of FMA contraction.
__global__ void geometry_kernel(int K, const double *coords, const int *cells, double *geo) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= K) return;
  const int a = cells[3 * c], b = cells[3 * c + 1], e = cells[3 * c + 2];
  const double x0 = coords[2 * a], y0 = coords[2 * a + 1];
  const double xr = __dmul_rn(0.5, __dsub_rn(coords[2 * b], x0));
  const double yr = __dmul_rn(0.5, __dsub_rn(coords[2 * b + 1], y0));
  const double xs = __dmul_rn(0.5, __dsub_rn(coords[2 * e], x0));
  const double ys = __dmul_rn(0.5, __dsub_rn(coords[2 * e + 1], y0));
  const double J = __dadd_rn(__dmul_rn(-xs, yr), __dmul_rn(xr, ys));
  double *g = geo + (size_t)c * 16;
  g[0] = __ddiv_rn(ys, J);
  g[1] = __ddiv_rn(-xs, J);
  g[2] = __ddiv_rn(-yr, J);
  g[3] = __ddiv_rn(xr, J);
  const double fnx[3] = {yr, __dsub_rn(ys, yr), -ys};
  const double fny[3] = {-xr, __dsub_rn(xr, xs), xs};
  for (int f = 0; f < 3; f++) {
    const double sJ = __dsqrt_rn(__dadd_rn(__dmul_rn(fnx[f], fnx[f]), __dmul_rn(fny[f], fny[f])));
    g[4 + 3 * f] = __ddiv_rn(fnx[f], sJ);
    g[5 + 3 * f] = __ddiv_rn(fny[f], sJ);
    g[6 + 3 * f] = __ddiv_rn(sJ, J);
  }
  g[13] = J;  // cell Jacobian: face arc-length element sJ = fscale * J
  // fscale of the three faces again in single precision (the dt estimate), in the padding
  float *gf = reinterpret_cast<float *>(g + 14);
  gf[0] = (float)g[6];
  gf[1] = (float)g[9];
  gf[2] = (float)g[12];
  gf[3] = 0.0f;
}

// Node position with the operation order of src/init_grid.h:19-54 (cblas dcopy/daxpy/dscal).
__device__ __forceinline__ double node_coord(double v0, double v1, double v2, double r, double s) {
  double x = __dmul_rn(__dmul_rn(0.5, v1), __dadd_rn(1.0, r));
  x = __dadd_rn(x, __dmul_rn(__dmul_rn(0.5, v2), __dadd_rn(1.0, s)));
  x = __dadd_rn(x, __dmul_rn(__dmul_rn(-0.5, v0), __dadd_rn(s, r)));
  return x;
}

// Initial state: freestream (src/set_ic.h) or the isentropic vortex at t=0
// (vortex/src/set_ic.h).  One thread per (cell, node).
template <int N>
__global__ void set_ic_kernel(const Inst d, const double *coords, const int *cells) {
  constexpr int Np = np_of(N);
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (long long)d.K * Np) return;
  const int c = (int)(tid / Np), i = (int)(tid - (long long)c * Np);
  double q[4];
  if (d.app == 1) {
    const int a = cells[3 * c], b = cells[3 * c + 1], e = cells[3 * c + 2];
    const double r = c_rs[N][i], s = c_rs[N][Np + i];
    const double x = node_coord(coords[2 * a], coords[2 * b], coords[2 * e], r, s);
    const double y = node_coord(coords[2 * a + 1], coords[2 * b + 1], coords[2 * e + 1], r, s);
    vortex_state(x, y, 0.0, d.P, q);
  } else {
    q[0] = d.P.rinf;
    q[1] = d.P.rinf * d.P.uinf;
    q[2] = d.P.rinf * d.P.vinf;
    q[3] = d.P.einf;
  }
  double *qp = d.q + (size_t)tid * 4, *wp = d.W + (size_t)tid * 4;
  st2(qp, q[0], q[1]); st2(qp + 2, q[2], q[3]);
  st2(wp, q[0], q[1]); st2(wp + 2, q[2], q[3]);
}

// Boundary face-node coordinates for the vortex boundary state.
template <int N>
__global__ void bxy_kernel(const Inst d, const double *coords, const int *cells, double *bxy) {
  constexpr int Nfp = N + 1, Np = np_of(N);
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= d.nB * Nfp) return;
  const int b = tid / Nfp, i = tid - b * Nfp;
  const int4 bd = d.bedges[b];
  const int c = bd.x, node = d.fmask[bd.y * Nfp + i];
  const int a = cells[3 * c], bb = cells[3 * c + 1], e = cells[3 * c + 2];
  const double r = c_rs[N][node], s = c_rs[N][Np + node];
  bxy[2 * tid] = node_coord(coords[2 * a], coords[2 * bb], coords[2 * e], r, s);
  bxy[2 * tid + 1] = node_coord(coords[2 * a + 1], coords[2 * bb + 1], coords[2 * e + 1], r, s);
}

// calc_dt over the current q into st->dt1_bits (src/calc_dt.h, seeded from 0 as
// src/airfoil.cpp:231).
template <int N>
__global__ void calc_dt_kernel(const Inst d) {
  constexpr int Np = np_of(N);
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long best = 0ull;
  if (tid < (long long)d.K * Np) {
    const int c = (int)(tid / Np), i = (int)(tid - (long long)c * Np);
    const int fa = c_dtf[N][2 * i], fb = c_dtf[N][2 * i + 1];
    if (fa >= 0) {
      const double *qp = d.q + (size_t)tid * 4;
      const double ir = rcp(qp[0]);
      const double u = qp[1] * ir, v = qp[2] * ir;
      const double v2 = fma(u, u, v * v);
      const double p = d.P.gm1 * fma(-0.5 * qp[0], v2, qp[3]);
      const double cs = sqrt(fabs(d.P.gam * p * ir));
      const double spd = ((N + 1) * (N + 1) * 0.5) * (sqrt(v2) + cs);
      const double fs = fb >= 0 ? fmax(d.geo[(size_t)c * 16 + 6 + 3 * fa], d.geo[(size_t)c * 16 + 6 + 3 * fb])
                                : d.geo[(size_t)c * 16 + 6 + 3 * fa];
      best = (unsigned long long)__double_as_longlong(spd * fs);
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_xor_sync(0xffffffffu, best, off);
    best = o > best ? o : best;
  }
  if ((threadIdx.x & 31) == 0 && best) atomicMax(&d.st->dt1_bits, best);
}

// Sums of squared nodal errors against the analytic vortex (vortex/src/l2_error.h:3-29),
// one partial per cell so the host can add them in cell order.
template <int N>
__global__ void l2_error_kernel(const Inst d, const double *coords, const int *cells, double *part) {
  constexpr int Np = np_of(N);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.K) return;
  const int a = cells[3 * c], b = cells[3 * c + 1], e = cells[3 * c + 2];
  double acc[4] = {0, 0, 0, 0};
  const double t = d.st->t;
  for (int i = 0; i < Np; i++) {
    const double r = c_rs[N][i], s = c_rs[N][Np + i];
    const double x = node_coord(coords[2 * a], coords[2 * b], coords[2 * e], r, s);
    const double y = node_coord(coords[2 * a + 1], coords[2 * b + 1], coords[2 * e + 1], r, s);
    double ex[4];
    vortex_state(x, y, t, d.P, ex);
    const double *qp = d.q + ((size_t)c * Np + i) * 4;
    for (int k = 0; k < 4; k++) acc[k] += (qp[k] - ex[k]) * (qp[k] - ex[k]);
  }
  for (int k = 0; k < 4; k++) part[4 * (size_t)c + k] = acc[k];
}

// ---------------------------------------------------------------- solution output
// src/save_solution.cpp:13-46: per mesh vertex, rho, u, v, p from the cell's vertex node (local
// nodes 0, N, Np-1 for vertices 0, 1, 2); cells are visited in ascending order there, so the last
// cell containing a vertex wins.  Here pass 1 finds that cell (atomicMax of the cell index per
// vertex), pass 2 lets it write: the same values, independent of thread order.
__global__ void vertex_owner_kernel(int K, const int *cells, int *owner) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= K) return;
  for (int v = 0; v < 3; v++) atomicMax(&owner[cells[3 * c + v]], c);
}

template <int N>
__global__ void vertex_fields_kernel(int K, const int *cells, const int *owner, const double *q, double gam,
                                     double *rho, double *u, double *v, double *p) {
  constexpr int Np = np_of(N);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= K) return;
  const int local[3] = {0, N, Np - 1};
  for (int k = 0; k < 3; k++) {
    const int node = cells[3 * c + k];
    if (owner[node] != c) continue;
    const double *qq = q + ((size_t)c * Np + local[k]) * 4;
    const double r = qq[0], uu = qq[1] / r, vv = qq[2] / r;  // IEEE division, as on the host
    rho[node] = r;
    u[node] = uu;
    v[node] = vv;
    // unfused products in the reference's order, so the fields are bit-identical to it
    p[node] = __dmul_rn(gam - 1, __dsub_rn(qq[3], __dmul_rn(0.5, __dadd_rn(__dmul_rn(qq[1], uu), __dmul_rn(qq[2], vv)))));
  }
}

// ---------------------------------------------------------------- launch helpers
// Threads per face-kernel block (a multiple of 32, at most 256).  The 68-register face blocks
// fill an SM with ~30 warps; with 256-thread blocks the last of ~1.7 waves leaves SMs idle
// (SM active 70 % of the launch).  Small blocks let the block scheduler balance that tail:
// 64 threads measured 58.5 / 61.8 us per stage at N=3 / N=4 on the K=32768 O-grid against
// 65.9 / 74.0 us with 256.
static std::atomic<int> g_face_block{64};
// 1: 64-thread face blocks use face_kernel_r64 (at most 64 registers).
static std::atomic<int> g_face_r64{0};

// 1: face and element kernels of the plain path are launched with programmatic stream
// serialisation (each may start while its predecessor drains), 0: plain stream order.
static std::atomic<int> g_pdl{1};
// Set by this thread while it enqueues the step graph over cell ranges without programmatic
// launch (the process-wide setting stays as it is for other threads).
static thread_local int t_no_pdl = 0;
static inline bool pdl_on() { return g_pdl.load(std::memory_order_relaxed) && !t_no_pdl; }

// Scheduling priority given to the launches this thread makes while g_launch_prio_on is set (the
// step graph over cell ranges sets it per range; lower numbers are scheduled first).
static thread_local int g_launch_prio_on = 0, g_launch_prio = 0;

template <class... KArgs, class... Args>
static void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  int na = 0;
  if (pdl_on()) {
    attr[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[na].val.programmaticStreamSerializationAllowed = 1;
    na++;
  }
  if (g_launch_prio_on) {
    attr[na].id = cudaLaunchAttributePriority;
    attr[na].val.priority = g_launch_prio;
    na++;
  }
  cfg.attrs = attr;
  cfg.numAttrs = na;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

template <int N>
static void launch_face(const Inst &d, int stage, cudaStream_t s) {
  const long long nf = ((long long)d.nE + d.nB) * (N + 1);
  const int bs = g_face_block;
  if (g_face_r64 && bs == 64)
    launch_pdl(face_kernel_r64<N>, dim3((unsigned)((nf + bs - 1) / bs)), dim3(bs), 0, s, d, stage);
  else
    launch_pdl(face_kernel<N>, dim3((unsigned)((nf + bs - 1) / bs)), dim3(bs), 0, s, d, stage);
}

// 3: dense rows on the tensor cores at N = 1, 2 (dg_ozaki.cuh), form 2 at the other orders
// (default);
// 2: even/odd with the contraction on the tensor cores (at N = 3, 4, 5, the even/odd FP64
// kernel at the other orders), 1: even/odd element kernel, 0: dense FP64.
static std::atomic<int> g_elem_variant{3};

// The even/odd element kernel instance for form TC at order N, launched over tiles [t0, t1):
// with the launch attributes of launch_pdl (attr true) or as a plain launch.  The instance
// knows whether it was launched with programmatic dependence (PW): without it the face fluxes
// are complete at the start and their copies are issued first.
template <int N, int TC, int MB>
static void elem_sym_launch(const Inst &d, int stage, int t0, int t1, cudaStream_t s, bool attr) {
  constexpr int Np = np_of(N);
  const size_t smem = elem_sym_smem(N);
  if (attr && pdl_on())
    launch_pdl(elem_kernel_sym<N, TC, MB, true>, dim3(t1 - t0), dim3(32, Np), smem, s, d, stage, t0);
  else if (attr)
    launch_pdl(elem_kernel_sym<N, TC, MB, false>, dim3(t1 - t0), dim3(32, Np), smem, s, d, stage, t0);
  else
    elem_kernel_sym<N, TC, MB, false><<<t1 - t0, dim3(32, Np), smem, s>>>(d, stage, t0);
}

// 1: the tensor-core element form at N = 3 runs as the warp-specialised persistent kernel
// (dg_elem_ws.cuh) over one block per SM; 2: the same, a launch over a range of tiles taking the
// range's share of the SMs; 0 (default): one block per tile (elem_kernel_sym).  Bitwise the same
// results.  On the K = 32768 O-grid the warp-specialised kernel measured slower (stages 0 / 1 / 2:
// 61 / 57 / 74 us against 46 / 51 / 61 us): its 8 contraction warps per SM run the integer-heavy
// product with too little parallelism, where the one-tile blocks bring 30 warps per SM to it.
static std::atomic<int> g_elem_ws{0};

// Resident blocks per SM that the order-3 tensor-core element kernel is compiled for: 3 (the
// default: 64 registers, a small spill) or 2 (more registers, no spill, and room beside two
// element blocks for face-kernel blocks of another cell range in the step graph).
static std::atomic<int> g_elem_mb{3};

static int ws_sm_count() {
  static int sms[kMaxDevices] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return 1;
  if (!sms[dev]) cudaDeviceGetAttribute(&sms[dev], cudaDevAttrMultiProcessorCount, dev);
  return sms[dev] > 0 ? sms[dev] : 1;
}

template <int N>
static void elem_ws_launch(const Inst &d, int stage, int t0, int t1, cudaStream_t s, bool attr) {
  const int T = (d.K + 31) / 32, sms = ws_sm_count();
  int grid = g_elem_ws == 2 ? (int)(((long long)sms * (t1 - t0) + T - 1) / T) : sms;
  grid = std::max(1, std::min(grid, t1 - t0));
  const size_t smem = ws_smem(N);
  if (attr && pdl_on())
    launch_pdl(elem_kernel_ws<N, true>, dim3(grid), dim3(ws_threads(N)), smem, s, d, stage, t0, t1);
  else if (attr)
    launch_pdl(elem_kernel_ws<N, false>, dim3(grid), dim3(ws_threads(N)), smem, s, d, stage, t0, t1);
  else
    elem_kernel_ws<N, false><<<grid, ws_threads(N), smem, s>>>(d, stage, t0, t1);
}

// Element tiles [t0, t1) of one stage in the current form (the even/odd forms; form 0, dense FP64,
// only as a whole-mesh launch with attr).
template <int N>
static void launch_elem_form(const Inst &d, int stage, int t0, int t1, cudaStream_t s, bool attr) {
  if (t1 <= t0) return;
  if constexpr (ws_used(N)) {
    if (g_elem_ws && g_elem_variant >= 2) return elem_ws_launch<N>(d, stage, t0, t1, s, attr);
  }
  if constexpr (ozd_used(N, 2)) {
    if (g_elem_variant == 3) return elem_sym_launch<N, 2, oz_min_blocks(N)>(d, stage, t0, t1, s, attr);
  }
  if constexpr (oz_used(N, true)) {
    if constexpr (N == 3) {
      // the register budget of two resident blocks per SM instead of three (g_elem_mb)
      if (g_elem_variant >= 2 && g_elem_mb == 2) return elem_sym_launch<N, 1, 2>(d, stage, t0, t1, s, attr);
    }
    if (g_elem_variant >= 2) return elem_sym_launch<N, 1, oz_min_blocks(N)>(d, stage, t0, t1, s, attr);
  }
  elem_sym_launch<N, 0, 1>(d, stage, t0, t1, s, attr);
}

template <int N>
static void launch_elem(const Inst &d, int stage, cudaStream_t s) {
  constexpr int Np = np_of(N), NK = nk_of(N);
  if (g_elem_variant) {
    launch_elem_form<N>(d, stage, 0, (d.K + 31) / 32, s, true);
  } else {
    const size_t smem = (size_t)NK * 32 * 4 * sizeof(double);
    launch_pdl(elem_kernel<N>, dim3((d.K + 31) / 32), dim3(32, Np), smem, s, d, stage);
  }
}

// Element tiles [t0, t1) of one stage with the launch attributes of launch_elem.
template <int N>
static void launch_elem_range(const Inst &d, int stage, int t0, int t1, cudaStream_t s) {
  launch_elem_form<N>(d, stage, t0, t1, s, true);
}

// Element tiles [t0, t1) of one stage, in plain stream order on s (the even/odd forms only).
template <int N>
static void launch_elem_tiles(const Inst &d, int stage, int t0, int t1, cudaStream_t s) {
  launch_elem_form<N>(d, stage, t0, t1, s, false);
}

template <int N>
static void launch_stage(const Inst &d, int stage, cudaStream_t s) {
  launch_face<N>(d, stage, s);
  launch_elem<N>(d, stage, s);
}

template <int N>
static cudaError_t set_smem_attr() {
  const size_t smem = (size_t)nk_of(N) * 32 * 4 * sizeof(double);
  cudaError_t e = cudaFuncSetAttribute(elem_kernel<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const size_t smem_sym = elem_sym_smem(N);
  auto both = [&](auto k_pdl, auto k_plain) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_pdl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_sym);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_plain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_sym);
  };
  both(elem_kernel_sym<N, 0, 1, true>, elem_kernel_sym<N, 0, 1, false>);
  if constexpr (oz_used(N, true))
    both(elem_kernel_sym<N, 1, oz_min_blocks(N), true>, elem_kernel_sym<N, 1, oz_min_blocks(N), false>);
  if constexpr (N == 3) both(elem_kernel_sym<N, 1, 2, true>, elem_kernel_sym<N, 1, 2, false>);
  if constexpr (ozd_used(N, 2))
    both(elem_kernel_sym<N, 2, oz_min_blocks(N), true>, elem_kernel_sym<N, 2, oz_min_blocks(N), false>);
  if constexpr (ws_used(N)) {
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(elem_kernel_ws<N, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ws_smem(N));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(elem_kernel_ws<N, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ws_smem(N));
  }
  return e;
}

template <int N>
static void sym_dims(int &NUe, int &NUo, int &NRe, int &NRo) {
  NUe = Sym<N>::NUe; NUo = Sym<N>::NUo; NRe = Sym<N>::NRe; NRo = Sym<N>::NRo;
}

// Tables of the even/odd form (see elem_kernel_sym) from the dense rows A = [Drw | Dsw | -LIFT].
struct SymHost {
  int NUe = 0, NUo = 0, NRe = 0, NRo = 0;
  std::vector<double> S;  // even rows NRe x NUe, then odd rows NRo x NUo
  int pos[77], out[28 * 3], rin[28 * 2];
};

static int sym_build(const Operators &o, const std::vector<double> &A, SymHost &t, std::string &err) {
  const int N = o.N, Np = o.Np, Nfp = o.Nfp, NK = 2 * Np + 3 * Nfp;
  std::vector<int> Pn(Np, -1), Pi(NK);
  for (int i = 0; i < Np; i++)
    for (int j = 0; j < Np; j++)
      if (std::fabs(o.r[j] - o.s[i]) + std::fabs(o.s[j] - o.r[i]) < 1e-10) Pn[i] = j;
  for (int i = 0; i < Np; i++)
    if (Pn[i] < 0) { err = "node set is not symmetric under r <-> s"; return -4; }
  for (int i = 0; i < Np; i++) {
    Pi[i] = Np + Pn[i];
    Pi[Np + i] = Pn[i];
  }
  for (int k = 0; k < Nfp; k++) {
    Pi[2 * Np + k] = 2 * Np + 2 * Nfp + (Nfp - 1 - k);
    Pi[2 * Np + 2 * Nfp + k] = 2 * Np + (Nfp - 1 - k);
    Pi[2 * Np + Nfp + k] = 2 * Np + Nfp + (Nfp - 1 - k);
  }
  std::vector<std::pair<int, int>> inp, outp;
  std::vector<int> infix, outfix;
  for (int a = 0; a < NK; a++) {
    if (a < Pi[a]) inp.push_back({a, Pi[a]});
    else if (a == Pi[a]) infix.push_back(a);
  }
  for (int i = 0; i < Np; i++) {
    if (i < Pn[i]) outp.push_back({i, Pn[i]});
    else if (i == Pn[i]) outfix.push_back(i);
  }
  const int NPin = (int)inp.size(), NUe = NPin + (int)infix.size(), NUo = NPin;
  const int NPo = (int)outp.size(), NRe = NPo + (int)outfix.size(), NRo = NPo;
  int cNUe, cNUo, cNRe, cNRo;
  DG_DISPATCH(N, sym_dims<NN>(cNUe, cNUo, cNRe, cNRo));
  if (NUe != cNUe || NUo != cNUo || NRe != cNRe || NRo != cNRo) { err = "unexpected symmetry dimensions"; return -4; }
  int *pos = t.pos, *out = t.out, *rin = t.rin;
  for (int k = 0; k < 77; k++) pos[k] = 0;
  for (int k = 0; k < 28 * 3; k++) out[k] = 0;
  for (int p = 0; p < NPin; p++) {
    pos[inp[p].first] = p;
    pos[inp[p].second] = NUe + p;
  }
  for (size_t j = 0; j < infix.size(); j++) pos[infix[j]] = NPin + (int)j;
  std::vector<double> &S = t.S;
  S.assign((size_t)NRe * NUe + (size_t)NRo * NUo, 0.0);
  for (int r = 0; r < NRe; r++) {
    const int i = r < NPo ? outp[r].first : outfix[r - NPo];
    for (int k = 0; k < NUe; k++)
      S[(size_t)r * NUe + k] = k < NPin ? 0.5 * (A[(size_t)i * NK + inp[k].first] + A[(size_t)i * NK + inp[k].second])
                                        : A[(size_t)i * NK + infix[k - NPin]];
  }
  for (int q = 0; q < NRo; q++) {
    const int i = outp[q].first;
    for (int k = 0; k < NUo; k++)
      S[(size_t)NRe * NUe + (size_t)q * NUo + k] =
          0.5 * (A[(size_t)i * NK + inp[k].first] - A[(size_t)i * NK + inp[k].second]);
  }
  for (int q = 0; q < NPo; q++) {
    const int a = outp[q].first, b = outp[q].second;
    out[3 * a] = q; out[3 * a + 1] = NRe + q; out[3 * a + 2] = 1;
    out[3 * b] = q; out[3 * b + 1] = NRe + q; out[3 * b + 2] = -1;
  }
  for (size_t j = 0; j < outfix.size(); j++) {
    const int a = outfix[j];
    out[3 * a] = NPo + (int)j; out[3 * a + 1] = -1; out[3 * a + 2] = 1;
  }
  // rows -> nodes, for transposed products: even row r is the pair outp[r] (or a fixed node),
  // odd row NRe + q the pair outp[q]
  for (int k = 0; k < 56; k++) rin[k] = -1;
  for (int r = 0; r < NRe; r++) {
    rin[2 * r] = r < NPo ? outp[r].first : outfix[r - NPo];
    rin[2 * r + 1] = r < NPo ? outp[r].second : -1;
  }
  for (int q = 0; q < NRo; q++) {
    rin[2 * (NRe + q)] = outp[q].first;
    rin[2 * (NRe + q) + 1] = outp[q].second;
  }
  t.NUe = NUe; t.NUo = NUo; t.NRe = NRe; t.NRo = NRo;
  return 0;
}

static int sym_tables(const Operators &o, const std::vector<double> &A, std::string &err) {
  const int N = o.N;
  SymHost t;
  if (int rc = sym_build(o, A, t, err)) return rc;
  const void *syms[7] = {nullptr, c_S1, c_S2, c_S3, c_S4, c_S5, c_S6};
  cudaError_t ce = cudaMemcpyToSymbol(syms[N], t.S.data(), t.S.size() * sizeof(double));
  if (ce == cudaSuccess) ce = cudaMemcpyToSymbol(c_rin, t.rin, sizeof(t.rin), (size_t)N * sizeof(t.rin));
  if (ce == cudaSuccess) ce = cudaMemcpyToSymbol(c_pos, t.pos, sizeof(t.pos), (size_t)N * sizeof(t.pos));
  if (ce == cudaSuccess) ce = cudaMemcpyToSymbol(c_out, t.out, sizeof(t.out), (size_t)N * sizeof(t.out));
  if (ce != cudaSuccess) { err = std::string("constant upload: ") + cudaGetErrorString(ce); return -3; }
  return oz_upload(N, t.S, t.NUe, t.NUo, t.NRe, t.NRo, A, o.Np, 2 * o.Np + 3 * o.Nfp, err);
}

// Dense rows [Drw | Dsw | -LIFT/2] of order N.  The 1/2 of the reference's flux
// (src/euler_rhs.h:217, the average of the two sides' fluxes) is taken here, exactly (a power of
// two), instead of in every face kernel: the face kernels store fscale * (F_L + F_R - dissipation).
static void dense_rows(const Operators &o, std::vector<double> &A) {
  const int Np = o.Np, Nfp = o.Nfp, NK = 2 * Np + 3 * Nfp;
  A.assign((size_t)Np * NK, 0.0);
  for (int i = 0; i < Np; i++) {
    for (int k = 0; k < Np; k++) {
      A[(size_t)i * NK + k] = o.Drw[(size_t)i * Np + k];
      A[(size_t)i * NK + Np + k] = o.Dsw[(size_t)i * Np + k];
    }
    for (int k = 0; k < 3 * Nfp; k++) A[(size_t)i * NK + 2 * Np + k] = -0.5 * o.LIFT[(size_t)i * 3 * Nfp + k];
  }
}

// Host-only view of the tensor-core operator tables of order N (for tests): the parity
// dimensions, the even/odd operator blocks S, the row exponents and the digits.
int tc_operator_tables(int N, int dims[4], std::vector<double> &S, int fexp[2][kOzRows], std::vector<int> &dig,
                       std::string &err) {
  if (!oz_used(N, true)) { err = "no tensor-core contraction at this order"; return -1; }
  Operators o;
  if (build_operators(N, o)) { err = "operator construction failed"; return -2; }
  std::vector<double> A;
  dense_rows(o, A);
  SymHost t;
  if (int rc = sym_build(o, A, t, err)) return rc;
  dims[0] = t.NUe; dims[1] = t.NUo; dims[2] = t.NRe; dims[3] = t.NRo;
  S = t.S;
  return oz_digits(t.S, t.NUe, t.NUo, t.NRe, t.NRo, fexp, dig, err);
}

// Host-only: the tensor-core contraction's final rounding, (th 2^32 + tl) 2^sc to the nearest
// double, exactly as the device computes it.
double tc_round(long long th, long long tl, int sc) { return oz_round(th, tl, sc); }

// ---------------------------------------------------------------- operator upload
// The order's tables go to the device that is current; g_order_table records which (device,
// order) pairs are uploaded.
static OnceTable g_order_table;

static int upload_order_constants(int N, std::string &err) {
  Operators o;
  if (build_operators(N, o)) { err = "operator construction failed"; return -2; }
  const int Np = o.Np, Nfp = o.Nfp;
  std::vector<double> A;
  dense_rows(o, A);
  const void *syms[7] = {nullptr, c_A1, c_A2, c_A3, c_A4, c_A5, c_A6};
  cudaError_t ce = cudaMemcpyToSymbol(syms[N], A.data(), A.size() * sizeof(double));
  if (ce == cudaSuccess) {
    if (int rc = sym_tables(o, A, err)) return rc;
  }
  // calc_dt face points: for node i, the faces f of face points k with FMASK[k] == i; the
  // fscale index follows src/calc_dt.h:11 (fscale[FMASK[k]], read as face FMASK[k] / Nfp while
  // Np <= 3 Nfp, i.e. N <= 4) or the face point's own face k / Nfp for N >= 5.
  int dtf[28 * 2];
  for (int i = 0; i < 28 * 2; i++) dtf[i] = -1;
  for (int k = 0; k < 3 * Nfp; k++) {
    const int node = o.FMASK[k];
    const int face = (Np <= 3 * Nfp) ? node / Nfp : k / Nfp;
    if (dtf[2 * node] < 0) dtf[2 * node] = face;
    else if (dtf[2 * node] != face && dtf[2 * node + 1] < 0) dtf[2 * node + 1] = face;
  }
  if (ce == cudaSuccess) ce = cudaMemcpyToSymbol(c_dtf, dtf, sizeof(dtf), (size_t)N * sizeof(dtf));
  double rs[2 * 28] = {0};
  for (int i = 0; i < Np; i++) {
    rs[i] = o.r[i];
    rs[Np + i] = o.s[i];
  }
  if (ce == cudaSuccess) ce = cudaMemcpyToSymbol(c_rs, rs, sizeof(rs), (size_t)N * sizeof(rs));
  if (ce == cudaSuccess) {
    DG_DISPATCH(N, ce = set_smem_attr<NN>());
  }
  if (ce != cudaSuccess) { err = std::string("constant upload: ") + cudaGetErrorString(ce); return -3; }
  return 0;
}

int load_order_constants(int N, std::string &err) {
  if (N < 1 || N > 6) { err = "order N must be in 1..6"; return -1; }
  int dev = 0;
  const cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) { err = std::string("cudaGetDevice: ") + cudaGetErrorString(ce); return -100; }
  if (dev >= kMaxDevices) { err = "device ordinal beyond the library's table"; return -1; }
  return g_order_table.ensure(dev, N, [&] { return upload_order_constants(N, err); });
}

int order_constants_loaded(int dev, int N) { return (N < 1 || N > 6) ? -1 : g_order_table.done(dev, N); }

void set_elem_variant(int v) { g_elem_variant = (v >= 0 && v <= 3) ? v : 3; }
void set_elem_ws(int m) { g_elem_ws = (m >= 0 && m <= 2) ? m : 0; }
void set_elem_blocks_per_sm(int b) { g_elem_mb = (b == 2) ? 2 : 3; }
int elem_blocks_per_sm() { return g_elem_mb; }
int elem_ws() { return g_elem_ws; }
int elem_variant() { return g_elem_variant; }
void set_pdl(int on) { g_pdl = on ? 1 : 0; }
void set_face_regs64(int on) { g_face_r64 = on ? 1 : 0; }
int face_regs64() { return g_face_r64; }
void set_face_block(int b) { g_face_block = (b >= 32 && b <= 256 && b % 32 == 0) ? b : 64; }

// ---------------------------------------------------------------- Solver (host)
#define CK(x)                                                                  \
  do {                                                                         \
    cudaError_t e_ = (x);                                                      \
    if (e_ != cudaSuccess) {                                                   \
      err = std::string(#x) + ": " + cudaGetErrorString(e_);                   \
      return -100;                                                             \
    }                                                                          \
  } while (0)

Solver::~Solver() {
  for (int c = 0; c < kOutChunks; c++) {
    if (io_streams[c]) cudaStreamDestroy(io_streams[c]);
    if (io_kern[c]) cudaEventDestroy(io_kern[c]);
    if (io_copy[c]) cudaEventDestroy(io_copy[c]);
  }
  if (io_fork) cudaEventDestroy(io_fork);
  for (cudaStream_t st : pstreams) cudaStreamDestroy(st);
  for (cudaEvent_t ev : pevents) cudaEventDestroy(ev);
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
  if (io_graph_exec) cudaGraphExecDestroy(io_graph_exec);
  if (io_graph) cudaGraphDestroy(io_graph);
  if (graphG_exec) cudaGraphExecDestroy(graphG_exec);
  if (graphG) cudaGraphDestroy(graphG);
  for (void *p : allocs) cudaFree(p);
  if (stream) cudaStreamDestroy(stream);
}

void *Solver::dalloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
  allocs.push_back(p);
  return p;
}

// Device edge records: {cL, cR, fL | fR << 2 | reverse << 4, 0} and {cell, face, type, 0}.
static void edge_records(const Mesh &m, std::vector<int4> &edges, std::vector<int4> &bedges) {
  edges.resize(m.n_edges());
  bedges.resize(m.n_bedges());
  for (int i = 0; i < m.n_edges(); i++) {
    const int cL = m.edge2cells[2 * i], cR = m.edge2cells[2 * i + 1];
    const int fL = m.edgeNum[2 * i], fR = m.edgeNum[2 * i + 1];
    // src/get_neighbour_q.h:10-34: vertex fL of L against vertex fR of R, exact comparison
    const int vL = m.cell2nodes[3 * cL + fL], vR = m.cell2nodes[3 * cR + fR];
    const bool rev = !(m.coords[2 * vL] == m.coords[2 * vR] && m.coords[2 * vL + 1] == m.coords[2 * vR + 1]);
    edges[i] = make_int4(cL, cR, fL | (fR << 2) | ((rev ? 1 : 0) << 4), 0);
  }
  for (int i = 0; i < m.n_bedges(); i++)
    bedges[i] = make_int4(m.bedge2cell[i], m.bedgeNum[i], m.bedge_type.empty() ? 2 : m.bedge_type[i], 0);
}

// Freestream and gas constants of a configuration, as src/airfoil.cpp:79-99 computes them.
Phys make_phys(const Config &c) {
  Phys P{};
  const double gam = c.gam;
  P.gam = gam;
  P.gm1 = gam - 1.0;
  double u, v, e;
  if (c.alpha_deg != 0.0) {
    u = std::sin((M_PI / 2.0) - (c.alpha_deg * M_PI / 180.0)) * std::sqrt(gam * c.p_inf / c.rho_inf) * c.mach;
    v = std::cos((M_PI / 2.0) - (c.alpha_deg * M_PI / 180.0)) * std::sqrt(gam * c.p_inf / c.rho_inf) * c.mach;
    e = c.p_inf / (gam - 1.0) + 0.5 * c.rho_inf * (u * u + v * v);
  } else {
    u = std::sqrt(gam * c.p_inf / c.rho_inf) * c.mach;
    v = 0.0;
    e = c.p_inf / (gam - 1.0) + 0.5 * c.rho_inf * (u * u);
  }
  P.rinf = c.rho_inf;
  P.uinf = u;
  P.vinf = v;
  P.pinf = c.p_inf;
  P.einf = e;
  P.vx0 = c.vortex_x0;
  P.vy0 = c.vortex_y0;
  P.vbeta = c.vortex_beta;
  P.derive();
  return P;
}

int Solver::create(const Config &c, const Mesh &m, std::string &err) {
  cfg = c;
  if (int rc = validate(m, err)) return rc;
  if (int rc = load_order_constants(c.N, err)) return rc;
  CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  const int N = c.N, Np = np_of(N), Nfp = N + 1;
  Operators o;
  build_operators(N, o);
  K = m.n_cells();
  d = Inst();
  d.N = N;
  d.K = K;
  d.nE = m.n_edges();
  d.nB = m.n_bedges();
  d.app = c.app;
  d.dt_mode = c.dt_mode;
  d.P = make_phys(c);  // freestream as src/airfoil.cpp:79-99

  edge_records(m, h_edges, h_bedges);
  const std::vector<int4> &edges = h_edges, &bedges = h_bedges;

  const size_t nq = (size_t)K * Np * 4;
  d.q = (double *)dalloc(nq * 8);
  d.W = (double *)dalloc(nq * 8);
  d.flux = (double *)dalloc((size_t)K * 3 * Nfp * 4 * 8);
  double *geo = (double *)dalloc((size_t)K * 16 * 8);
  d.geo = geo;
  int4 *de = (int4 *)dalloc(sizeof(int4) * d.nE), *db = (int4 *)dalloc(sizeof(int4) * d.nB);
  d.edges = de;
  d.bedges = db;
  int *fm = (int *)dalloc(sizeof(int) * 3 * Nfp);
  d.fmask = fm;
  d.st = (StepState *)dalloc(sizeof(StepState));
  d.dt_est = (float *)dalloc((size_t)((K + 31) / 32) * Np * sizeof(float));
  {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev));
  }
  coords_d = (double *)dalloc(m.coords.size() * 8);
  cells_d = (int *)dalloc(m.cell2nodes.size() * 4);
  double *bxy = (double *)dalloc((size_t)d.nB * Nfp * 2 * 8);
  d.bxy = bxy;
  for (void *p : allocs)
    if (!p) { err = "cudaMalloc failed"; return -101; }
  CK(cudaMemcpyAsync(de, edges.data(), sizeof(int4) * d.nE, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(db, bedges.data(), sizeof(int4) * d.nB, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(fm, o.FMASK.data(), sizeof(int) * 3 * Nfp, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(coords_d, m.coords.data(), m.coords.size() * 8, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(cells_d, m.cell2nodes.data(), m.cell2nodes.size() * 4, cudaMemcpyHostToDevice, stream));
  CK(cudaMemsetAsync(d.flux, 0, (size_t)K * 3 * Nfp * 4 * 8, stream));
  geometry_kernel<<<(K + 127) / 128, 128, 0, stream>>>(K, coords_d, cells_d, geo);
  if (d.nB) DG_DISPATCH(N, (bxy_kernel<NN><<<(d.nB * Nfp + 127) / 128, 128, 0, stream>>>(d, coords_d, cells_d, bxy)));
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(stream));
  return 0;
}

int Solver::init(std::string &err) {
  const int Np = np_of(cfg.N);
  StepState s0;
  std::memset(&s0, 0, sizeof(s0));
  s0.cfl = cfg.cfl;
  CK(cudaMemcpyAsync(d.st, &s0, sizeof(s0), cudaMemcpyHostToDevice, stream));
  const long long n = (long long)K * Np;
  DG_DISPATCH(cfg.N, (set_ic_kernel<NN><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(d, coords_d, cells_d)));
  DG_DISPATCH(cfg.N, (calc_dt_kernel<NN><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(d)));
  CK(cudaGetLastError());
  return set_dt_from_max(err);
}

// dt = (1/dt1)*cfl from the accumulated maximum, then clear it (src/airfoil.cpp:237).
int Solver::set_dt_from_max(std::string &err) {
  StepState s;
  CK(cudaMemcpyAsync(&s, d.st, sizeof(s), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  const double dt1 = __builtin_bit_cast(double, s.dt1_bits);
  if (!(dt1 > 0.0) || !std::isfinite(dt1)) { err = "calc_dt produced a non-positive maximum"; return -5; }
  s.dt = (1.0 / dt1) * cfg.cfl;
  s.dt1_bits = 0ull;
  CK(cudaMemcpyAsync(d.st, &s, sizeof(s), cudaMemcpyHostToDevice, stream));
  CK(cudaStreamSynchronize(stream));
  return 0;
}

void Solver::enqueue_step(cudaStream_t s) {
  DG_DISPATCH(cfg.N, (launch_stage<NN>(d, 0, s), launch_stage<NN>(d, 1, s), launch_stage<NN>(d, 2, s)));
  enqueue_finalize(s, true);
}

void Solver::enqueue_finalize(cudaStream_t s, bool pdl) {
  if (d.dt_mode == 0 && d.dt_est) {
    // one block per SM at most, at least 8 estimates per block
    const int n = ((K + 31) / 32) * np_of(cfg.N);
    const int g = std::max(1, std::min(sm_count > 0 ? sm_count : 1, (n + 7) / 8));
    DG_DISPATCH(cfg.N, pdl ? launch_pdl(dt_finalize_kernel<NN>, dim3(g), dim3(256), 0, s, d)
                           : (dt_finalize_kernel<NN><<<g, 256, 0, s>>>(d), void()));
  } else if (pdl) {
    launch_pdl(finalize_kernel, dim3(1), dim3(32), 0, s, d.st, d.dt_mode, d.dt_hist, d.dt_hist_len);
  } else {
    finalize_kernel<<<1, 32, 0, s>>>(d.st, d.dt_mode, d.dt_hist, d.dt_hist_len);
  }
}

// One step with an event recorded after each of its seven kernels (ev[0] is recorded by the
// caller before the step).
void Solver::enqueue_step_events(cudaStream_t s, cudaEvent_t *ev) {
  for (int stage = 0; stage < 3; stage++) {
    DG_DISPATCH(cfg.N, launch_face<NN>(d, stage, s));
    cudaEventRecord(ev[1 + 2 * stage], s);
    DG_DISPATCH(cfg.N, launch_elem<NN>(d, stage, s));
    cudaEventRecord(ev[2 + 2 * stage], s);
  }
  enqueue_finalize(s, false);
  cudaEventRecord(ev[7], s);
}

int Solver::build_graph(std::string &err) {
  if (graph_exec) return 0;
  const int P = g_elem_variant ? step_parts_for(K) : 1;  // the dense FP64 form has no tile ranges
  if (P > 1) {
    if (int rc = build_parts(P, err)) return rc;
  } else {
    parts = 1;
  }
  const unsigned long long flags = (parts > 1 && (step_graph_flags() & 6)) ? cudaGraphInstantiateFlagUseNodePriority : 0;
  // one step, and (over cell ranges) graph_steps steps in one graph
  graph_steps = parts > 1 ? steps_per_graph() : 1;
  for (int k = 0; k < (graph_steps > 1 ? 2 : 1); k++) {
    const int G = k == 0 ? 1 : graph_steps;
    cudaGraph_t &gr = k == 0 ? graph : graphG;
    cudaGraphExec_t &ex = k == 0 ? graph_exec : graphG_exec;
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    if (parts > 1) enqueue_step_parts(stream, nullptr, nullptr, G);
    else enqueue_step(stream);
    cudaError_t ce = cudaStreamEndCapture(stream, &gr);
    if (ce != cudaSuccess) { err = std::string("graph capture: ") + cudaGetErrorString(ce); return -6; }
    CK(cudaGraphInstantiate(&ex, gr, flags));
  }
  return 0;
}

// ---------------------------------------------------------------- the step as a DAG of cell ranges
// The cells are cut into P ranges of whole 32-cell tiles; every face goes to the range of its
// higher cell (a boundary face to its cell's).  Per stage, range p has a face launch F_p (its
// faces, boundary faces first) and an element launch E_p (its tiles).  F_p reads W of ranges
// lo_p..p and writes face slots of the same cells; E_p reads the face slots of its cells, written
// by F_p..F_hi_p, and writes W (and q) of its own cells.  So
//   F_p(s) after E_q(s-1), q in lo_p..p  (W it reads is final; the slots it writes are consumed)
//   E_p(s) after F_q(s),   q in p..hi_p  (its slots are written; nobody still reads its old W)
// and nothing else: E_p of stage s can run while later ranges are still in their face launches,
// and F_p of stage s+1 while later ranges are still in their element launches.  The face kernel
// is FP64 bound and the element kernel latency bound, so the two overlap on the SMs.  Each
// launch computes exactly what the one-range step computes for its faces and tiles (every face
// slot has one writer), so the result is bitwise the same for every P.  With a mesh numbered
// with locality (O-grid rings, square rows) lo_p and hi_p are p-1 and p+1.
static std::atomic<int> g_step_parts{0};  // 0: automatic (step_parts_for), 1: the single-range chain
// bit 2: element launches get a higher scheduling priority than face launches.
// bit 0: launch the ranges' kernels without programmatic dependent launch (the default: with it,
// dependent launches start early and their waiting blocks hold SM slots the other ranges' kernels
// could use: 300 vs 267 us per step at 4 ranges); bit 1: give range p's launches a scheduling
// priority that falls with p (earlier ranges first; measured no faster).
static std::atomic<int> g_step_graph_flags{1};
void set_step_graph_flags(int f) { g_step_graph_flags = f & 7; }
int step_graph_flags() { return g_step_graph_flags; }

int step_parts_for(int K) {
  const int T = (K + 31) / 32, sp = g_step_parts.load();
  if (sp >= 1) return std::max(1, std::min(sp, std::min(kMaxStepParts, T)));
  // automatic: ranges of at least 128 tiles, at most 4 (on the K = 32768 O-grid at N = 3, steps of
  // 290 / 267 / 269 / 271 us with 1 / 4 / 8 / 16 ranges; more ranges add launches and edges)
  return std::max(1, std::min(4, T / 128));
}

// Steps in one launch of the step graph over cell ranges (run() launches it as often as it fits,
// then the one-step graph for the rest).  On the K = 32768 O-grid at N = 3, 40 steps in one run():
// 254.3 / 245.9 / 241.6 / 239.4 us per step with 1 / 2 / 4 / 8 steps per graph.
static std::atomic<int> g_steps_per_graph{8};
void set_steps_per_graph(int g) { g_steps_per_graph = (g >= 1 && g <= 8) ? g : 8; }
int steps_per_graph() { return g_steps_per_graph; }

void set_step_parts(int p) { g_step_parts = (p >= 0 && p <= kMaxStepParts) ? p : 0; }
int step_parts() { return g_step_parts; }

int Solver::build_parts(int P, std::string &err) {
  const int T = (K + 31) / 32, N = cfg.N, Nfp = N + 1;
  ptile0.assign(P + 1, 0);
  for (int p = 0; p <= P; p++) ptile0[p] = (int)((long long)T * p / P);
  auto part_of = [&](int c) {  // the range holding cell c
    const int t = c / 32;
    int p = (int)((long long)t * P / T);
    while (p + 1 <= P - 1 && ptile0[p + 1] <= t) p++;
    while (p > 0 && ptile0[p] > t) p--;
    return p;
  };
  std::vector<std::vector<int4>> eb(P), bb(P);
  plo.assign(P, 0);
  phi.assign(P, 0);
  for (int p = 0; p < P; p++) plo[p] = phi[p] = p;
  for (const int4 &e : h_edges) {
    const int pl = part_of(e.x), pr = part_of(e.y), q = std::max(pl, pr);
    eb[q].push_back(e);
    plo[q] = std::min(plo[q], std::min(pl, pr));
    phi[pl] = std::max(phi[pl], q);
    phi[pr] = std::max(phi[pr], q);
  }
  for (const int4 &b : h_bedges) bb[part_of(b.x)].push_back(b);
  std::vector<int4> es, bs;
  pe0.assign(P + 1, 0);
  pb0.assign(P + 1, 0);
  for (int p = 0; p < P; p++) {
    pe0[p] = (int)es.size();
    pb0[p] = (int)bs.size();
    es.insert(es.end(), eb[p].begin(), eb[p].end());
    bs.insert(bs.end(), bb[p].begin(), bb[p].end());
  }
  pe0[P] = (int)es.size();
  pb0[P] = (int)bs.size();
  if (!pedges) {
    pedges = (int4 *)dalloc(sizeof(int4) * std::max<size_t>(1, es.size()));
    pbedges = (int4 *)dalloc(sizeof(int4) * std::max<size_t>(1, bs.size()));
    pbxy = (double *)dalloc((size_t)std::max<size_t>(1, bs.size()) * Nfp * 2 * 8);
    if (!pedges || !pbedges || !pbxy) { err = "cudaMalloc failed"; return -101; }
  }
  if (!es.empty()) CK(cudaMemcpyAsync(pedges, es.data(), sizeof(int4) * es.size(), cudaMemcpyHostToDevice, stream));
  if (!bs.empty()) {
    CK(cudaMemcpyAsync(pbedges, bs.data(), sizeof(int4) * bs.size(), cudaMemcpyHostToDevice, stream));
    Inst db = d;
    db.bedges = pbedges;
    DG_DISPATCH(N, (bxy_kernel<NN><<<(db.nB * Nfp + 127) / 128, 128, 0, stream>>>(db, coords_d, cells_d, pbxy)));
    CK(cudaGetLastError());
  }
  while ((int)pstreams.size() < P) {
    cudaStream_t st = nullptr;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    pstreams.push_back(st);
  }
  while ((int)pevents.size() < 7 * P + 2) {
    cudaEvent_t ev = nullptr;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    pevents.push_back(ev);
  }
  CK(cudaStreamSynchronize(stream));
  parts = P;
  return 0;
}

// Kernel launches of one step of the graph built (or to be built) for this solver.
int Solver::kernels_per_step() const {
  const int P = parts ? parts : step_parts_for(K);
  if (P <= 1) return 7;
  if (!parts) return 6 * P + 1;  // every range has faces on any mesh of this size
  int n = 3 * P + 1;
  for (int p = 0; p < P; p++) n += (pe0[p + 1] - pe0[p] + pb0[p + 1] - pb0[p] > 0) ? 3 : 0;
  return n;
}

void Solver::enqueue_step_parts(cudaStream_t s, const double *q_in, double *q_out, int nsteps) {
  const int P = parts, Nfp = cfg.N + 1;
  const size_t cell_bytes = (size_t)np_of(cfg.N) * 4 * sizeof(double);
  auto cells_of = [&](int p, size_t &c0, size_t &nc) {
    c0 = (size_t)ptile0[p] * 32;
    nc = std::min((size_t)ptile0[p + 1] * 32, (size_t)K) - c0;
  };
  t_no_pdl = (g_step_graph_flags & 1) ? 1 : 0;
  int prio_lo = 0, prio_hi = 0;  // least and greatest priority (numerically: hi <= lo)
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  // bit 1: earlier ranges first; bit 2: element launches before face launches
  auto set_prio = [&](int p, bool elem) {
    if (g_step_graph_flags & 2) {
      g_launch_prio_on = 1;
      g_launch_prio = prio_hi + (int)((long long)(prio_lo - prio_hi) * p / std::max(1, P - 1));
    } else if (g_step_graph_flags & 4) {
      g_launch_prio_on = 1;
      g_launch_prio = elem ? prio_hi : prio_lo;
    }
  };
  cudaEvent_t fork = pevents[6 * P];
  auto evF = [&](int st, int p) { return pevents[(2 * st) * P + p]; };
  auto evE = [&](int st, int p) { return pevents[(2 * st + 1) * P + p]; };
  auto evU = [&](int p) { return pevents[6 * P + 1 + p]; };
  cudaEvent_t fin = pevents[7 * P + 1];  // after the previous step's finalize
  cudaEventRecord(fork, s);
  for (int p = 0; p < P; p++) cudaStreamWaitEvent(pstreams[p], fork, 0);
  if (q_in) {
    // the input range by range: q, then W = q, on the range's own stream
    for (int p = 0; p < P; p++) {
      size_t c0, nc;
      cells_of(p, c0, nc);
      cudaMemcpyAsync(d.q + c0 * cell_bytes / 8, q_in + c0 * cell_bytes / 8, nc * cell_bytes, cudaMemcpyHostToDevice,
                      pstreams[p]);
      cudaMemcpyAsync(d.W + c0 * cell_bytes / 8, d.q + c0 * cell_bytes / 8, nc * cell_bytes,
                      cudaMemcpyDeviceToDevice, pstreams[p]);
      cudaEventRecord(evU(p), pstreams[p]);
    }
  }
  // Steps after the first in this graph: the first face launch of range p needs only the previous
  // step's last element launches of the ranges whose W it reads (and, in the vortex app, the time
  // the finalize kernel advanced); the first element launch also needs the new dt.  So the next
  // step's face launches overlap the previous step's last element launches.
  for (int step = 0; step < nsteps; step++) {
  for (int stage = 0; stage < 3; stage++) {
    for (int p = 0; p < P; p++) {
      cudaStream_t ps = pstreams[p];
      if (stage > 0 || step > 0)
        for (int q = plo[p]; q < p; q++) cudaStreamWaitEvent(ps, evE(stage > 0 ? stage - 1 : 2, q), 0);
      else if (q_in)
        for (int q = plo[p]; q < p; q++) cudaStreamWaitEvent(ps, evU(q), 0);  // the W it reads
      if (stage == 0 && step > 0 && d.app == 1) cudaStreamWaitEvent(ps, fin, 0);
      Inst dp = d;
      dp.edges = pedges + pe0[p];
      dp.nE = pe0[p + 1] - pe0[p];
      dp.bedges = pbedges + pb0[p];
      dp.nB = pb0[p + 1] - pb0[p];
      dp.bxy = pbxy + (size_t)pb0[p] * Nfp * 2;
      set_prio(p, false);
      if (dp.nE + dp.nB > 0) DG_DISPATCH(cfg.N, launch_face<NN>(dp, stage, ps));
      g_launch_prio_on = 0;
      cudaEventRecord(evF(stage, p), ps);
    }
    for (int p = 0; p < P; p++) {
      cudaStream_t ps = pstreams[p];
      for (int q = p + 1; q <= phi[p]; q++) cudaStreamWaitEvent(ps, evF(stage, q), 0);
      if (stage == 0 && step > 0) cudaStreamWaitEvent(ps, fin, 0);  // this step's dt
      set_prio(p, true);
      DG_DISPATCH(cfg.N, launch_elem_range<NN>(d, stage, ptile0[p], ptile0[p + 1], ps));
      g_launch_prio_on = 0;
      cudaEventRecord(evE(stage, p), ps);
      if (stage == 2 && q_out) {  // this range's result leaves while the others compute
        size_t c0, nc;
        cells_of(p, c0, nc);
        cudaMemcpyAsync(q_out + c0 * cell_bytes / 8, d.q + c0 * cell_bytes / 8, nc * cell_bytes,
                        cudaMemcpyDeviceToHost, ps);
      }
    }
  }
  for (int p = 0; p < P; p++) {
    cudaEventRecord(evE(2, p), pstreams[p]);  // after the range's copy too
    cudaStreamWaitEvent(s, evE(2, p), 0);
  }
  enqueue_finalize(s, true);
  cudaEventRecord(fin, s);
  }
  t_no_pdl = 0;
}

// One step with host buffers through a captured graph over the cell ranges: each range's input
// is uploaded on its own stream before its first face launch (which also waits for the ranges
// whose W it reads), and each range's result is downloaded as soon as its last element launch is
// done.  The graph is kept for the last pair of host pointers; host buffers that are not pinned
// (or registered) take the single-range path below.
int Solver::step_io_parts(const double *q_in, double *q_out, bool &done, std::string &err) {
  done = false;
  if (int rc = build_graph(err)) return rc;
  if (parts <= 1) return 0;
  for (const void *hp : {(const void *)q_in, (const void *)q_out}) {
    if (!hp) continue;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, hp) != cudaSuccess || at.type != cudaMemoryTypeHost) {
      cudaGetLastError();
      return 0;
    }
  }
  if (!io_graph_exec || io_in != q_in || io_out != q_out) {
    if (io_graph_exec) { cudaGraphExecDestroy(io_graph_exec); io_graph_exec = nullptr; }
    if (io_graph) { cudaGraphDestroy(io_graph); io_graph = nullptr; }
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step_parts(stream, q_in, q_out);
    cudaError_t ce = cudaStreamEndCapture(stream, &io_graph);
    if (ce != cudaSuccess) { err = std::string("io graph capture: ") + cudaGetErrorString(ce); return -6; }
    CK(cudaGraphInstantiate(&io_graph_exec, io_graph, 0));
    io_in = q_in;
    io_out = q_out;
  }
  CK(cudaGraphLaunch(io_graph_exec, stream));
  done = true;
  return 0;
}

int Solver::step_io(const double *q_in, double *q_out, std::string &err) {
  if (g_elem_variant) {
    bool done = false;
    if (int rc = step_io_parts(q_in, q_out, done, err)) return rc;
    if (done) return 0;
  }
  if (!g_elem_variant) {  // the dense form has no tile ranges: plain copies around a whole step
    const size_t n = q_count() * 8;
    if (q_in) {
      CK(cudaMemcpyAsync(d.q, q_in, n, cudaMemcpyHostToDevice, stream));
      CK(cudaMemcpyAsync(d.W, d.q, n, cudaMemcpyDeviceToDevice, stream));
    }
    enqueue_step(stream);
    if (q_out) CK(cudaMemcpyAsync(q_out, d.q, n, cudaMemcpyDeviceToHost, stream));
    return 0;
  }
  if (!io_fork) {
    int lo = 0, hi = 0;
    CK(cudaDeviceGetStreamPriorityRange(&lo, &hi));  // hi: the highest priority (numerically least)
    for (int c = 0; c < kOutChunks; c++) {
      const int prio = hi + (lo - hi) * c / (kOutChunks - 1);
      CK(cudaStreamCreateWithPriority(&io_streams[c], cudaStreamNonBlocking, prio));
      CK(cudaEventCreateWithFlags(&io_kern[c], cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&io_copy[c], cudaEventDisableTiming));
    }
    CK(cudaEventCreateWithFlags(&io_fork, cudaEventDisableTiming));
  }
  const int N = cfg.N, Np = (N + 1) * (N + 2) / 2, T = (K + 31) / 32;
  const size_t cell_doubles = (size_t)Np * 4;
  if (q_in) {
    // one upload: split into ranges and overlapped with the first face kernel it saved ~4 us of
    // 52, since host<->device copies slow the running kernels by about two thirds of their
    // own time on this part
    CK(cudaMemcpyAsync(d.q, q_in, q_count() * 8, cudaMemcpyHostToDevice, stream));
    CK(cudaMemcpyAsync(d.W, d.q, q_count() * 8, cudaMemcpyDeviceToDevice, stream));
  }
  DG_DISPATCH(N, launch_stage<NN>(d, 0, stream));
  DG_DISPATCH(N, (launch_stage<NN>(d, 1, stream), launch_face<NN>(d, 2, stream)));
  if (!q_out) {
    DG_DISPATCH(N, launch_elem<NN>(d, 2, stream));
    enqueue_finalize(stream, true);
    CK(cudaGetLastError());
    return 0;
  }
  CK(cudaEventRecord(io_fork, stream));
  // The last element kernel as ranges of tiles on streams of falling priority: the block
  // scheduler runs the first range's tiles first, so its q is final (and on its way to the host)
  // while the later ranges compute.
  for (int c = 0; c < kOutChunks; c++) {
    const int t0 = (int)((long long)T * c / kOutChunks), t1 = (int)((long long)T * (c + 1) / kOutChunks);
    cudaStream_t cs = io_streams[c];
    CK(cudaStreamWaitEvent(cs, io_fork, 0));
    if (t1 > t0) {
      DG_DISPATCH(N, launch_elem_tiles<NN>(d, 2, t0, t1, cs));
      CK(cudaGetLastError());
    }
    CK(cudaEventRecord(io_kern[c], cs));
    const size_t e0 = (size_t)t0 * 32, e1 = std::min((size_t)t1 * 32, (size_t)K);
    if (e1 > e0)
      CK(cudaMemcpyAsync(q_out + e0 * cell_doubles, d.q + e0 * cell_doubles, (e1 - e0) * cell_doubles * 8,
                         cudaMemcpyDeviceToHost, cs));
    CK(cudaEventRecord(io_copy[c], cs));
  }
  for (int c = 0; c < kOutChunks; c++) CK(cudaStreamWaitEvent(stream, io_kern[c], 0));
  enqueue_finalize(stream, false);
  CK(cudaGetLastError());
  for (int c = 0; c < kOutChunks; c++) CK(cudaStreamWaitEvent(stream, io_copy[c], 0));
  return 0;
}

int Solver::step(int nsteps, bool use_graph, std::string &err) {
  if (use_graph) {
    if (int rc = build_graph(err)) return rc;
    int i = 0;
    if (graph_steps > 1 && graphG_exec)
      for (; i + graph_steps <= nsteps; i += graph_steps) CK(cudaGraphLaunch(graphG_exec, stream));
    for (; i < nsteps; i++) CK(cudaGraphLaunch(graph_exec, stream));
  } else {
    for (int i = 0; i < nsteps; i++) enqueue_step(stream);
    CK(cudaGetLastError());
  }
  return 0;
}

int Solver::rhs(double *out_dev, std::string &err) {
  d.rhs_out = out_dev;
  DG_DISPATCH(cfg.N, (launch_stage<NN>(d, 3, stream)));
  d.rhs_out = nullptr;
  CK(cudaGetLastError());
  return 0;
}

int Solver::l2_error(double err4[4], std::string &err) {
  double *part = nullptr;
  CK(cudaMallocAsync((void **)&part, (size_t)K * 4 * 8, stream));
  DG_DISPATCH(cfg.N, (l2_error_kernel<NN><<<(K + 127) / 128, 128, 0, stream>>>(d, coords_d, cells_d, part)));
  std::vector<double> h((size_t)K * 4);
  cudaError_t ce = cudaMemcpyAsync(h.data(), part, h.size() * 8, cudaMemcpyDeviceToHost, stream);
  cudaFreeAsync(part, stream);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream);
  if (ce != cudaSuccess) { err = std::string("l2_error: ") + cudaGetErrorString(ce); return -100; }
  for (int k = 0; k < 4; k++) err4[k] = 0.0;
  for (int c = 0; c < K; c++)
    for (int k = 0; k < 4; k++) err4[k] += h[4 * (size_t)c + k];
  return 0;
}

int Solver::vertex_fields(int n_nodes, double *rho, double *u, double *v, double *p, std::string &err) {
  int *owner = nullptr;
  double *buf = nullptr;
  CK(cudaMallocAsync((void **)&owner, (size_t)n_nodes * 4, stream));
  CK(cudaMallocAsync((void **)&buf, (size_t)n_nodes * 4 * 8, stream));
  CK(cudaMemsetAsync(owner, 0xff, (size_t)n_nodes * 4, stream));  // -1: vertex of no cell
  CK(cudaMemsetAsync(buf, 0, (size_t)n_nodes * 4 * 8, stream));
  vertex_owner_kernel<<<(K + 127) / 128, 128, 0, stream>>>(K, cells_d, owner);
  DG_DISPATCH(cfg.N, (vertex_fields_kernel<NN><<<(K + 127) / 128, 128, 0, stream>>>(
                         K, cells_d, owner, d.q, cfg.gam, buf, buf + n_nodes, buf + 2 * n_nodes, buf + 3 * n_nodes)));
  double *outs[4] = {rho, u, v, p};
  for (int k = 0; k < 4; k++)
    CK(cudaMemcpyAsync(outs[k], buf + (size_t)k * n_nodes, (size_t)n_nodes * 8, cudaMemcpyDeviceToHost, stream));
  CK(cudaFreeAsync(owner, stream));
  CK(cudaFreeAsync(buf, stream));
  CK(cudaStreamSynchronize(stream));
  return 0;
}

int Solver::state(StepState &s, std::string &err) {
  CK(cudaMemcpyAsync(&s, d.st, sizeof(s), cudaMemcpyDeviceToHost, stream));
  CK(cudaStreamSynchronize(stream));
  return 0;
}

}  // namespace dg

// ---------------------------------------------------------------- allocation-free RHS
// dg_rhs_noalloc (include/dg_gb300.h): one right-hand side with no device allocation, for
// callers that must not call cudaMalloc (a memory pool owned by another runtime, a fixed
// budget, code that may run while another library is capturing a CUDA graph).  The face-flux
// scratch that Solver allocates per mesh lives here in one file-scope device array instead:
// kNoAllocScratchBytes (32 MiB) on every GPU that loads this library, held until the process
// exits.  Every call shares it, so calls that overlap on the GPU race; the used part is
// cleared at the start of each call.
namespace dg {

constexpr size_t kNoAllocScratchBytes = 32ull << 20;
static __device__ __align__(256) double g_noalloc_flux[kNoAllocScratchBytes / sizeof(double)];
static __device__ __align__(256) int g_noalloc_fmask[7][3 * 7];

// Device addresses of the two arrays on each device (a host-side name of a __device__ array is
// not a device address); written once per device under g_noalloc_table's lock, read after it.
struct NoAllocDevice {
  double *flux = nullptr;
  int *fmask = nullptr;  // [7][21]
};
static NoAllocDevice g_noalloc[kMaxDevices];
static OnceTable g_noalloc_table;  // slot 0: this device's addresses, every order's tables, fmasks

// Once per device, with that device current: the scratch addresses, and the operator tables and
// face masks of every order 1..6, so that only the first call on a device makes synchronous
// uploads (whatever its order).
static int noalloc_setup(int dev, std::string &err) {
  if (dev < 0 || dev >= kMaxDevices) { err = "device ordinal out of range"; return -1; }
  return g_noalloc_table.ensure(dev, 0, [&]() -> int {
    NoAllocDevice nd;
    cudaError_t ce = cudaGetSymbolAddress((void **)&nd.flux, g_noalloc_flux);
    if (ce != cudaSuccess) { err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(ce); return -100; }
    ce = cudaGetSymbolAddress((void **)&nd.fmask, g_noalloc_fmask);
    if (ce != cudaSuccess) { err = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(ce); return -100; }
    for (int N = 1; N <= 6; N++) {
      if (int rc = load_order_constants(N, err)) return rc;
      Operators o;
      if (build_operators(N, o)) { err = "operator construction failed"; return -2; }
      ce = cudaMemcpyToSymbol(g_noalloc_fmask, o.FMASK.data(), o.FMASK.size() * sizeof(int),
                              (size_t)N * 3 * 7 * sizeof(int));
      if (ce != cudaSuccess) { err = std::string("cudaMemcpyToSymbol: ") + cudaGetErrorString(ce); return -100; }
    }
    g_noalloc[dev] = nd;
    return 0;
  });
}

int noalloc_ready(int dev) { return g_noalloc_table.done(dev, 0); }

int rhs_noalloc(const Config &c, int K, int nE, int nB, const double *W, const double *geo,
                const int4 *edges, const int4 *bedges, double *rhs, cudaStream_t stream,
                std::string &err) {
  const int N = c.N, Nfp = N + 1;
  const size_t need = (size_t)K * 3 * Nfp * 4 * sizeof(double);
  if (need > kNoAllocScratchBytes) {
    err = "mesh too large for the allocation-free path: " + std::to_string(need) + " bytes of face-flux scratch > " +
          std::to_string(kNoAllocScratchBytes);
    return -3;
  }
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess) { err = std::string("cudaGetDevice: ") + cudaGetErrorString(ce); return -100; }
  if (int rc = noalloc_setup(dev, err)) return rc;
  const NoAllocDevice nd = g_noalloc[dev];
  Inst d{};
  d.N = N;
  d.K = K;
  d.nE = nE;
  d.nB = nB;
  d.app = 0;
  d.dt_mode = 1;
  d.edges = edges;
  d.bedges = bedges;
  d.fmask = nd.fmask + N * 3 * 7;
  d.geo = geo;
  d.W = const_cast<double *>(W);  // read only in the RHS stage
  d.flux = nd.flux;
  d.rhs_out = rhs;
  const double gam = c.gam;
  double u, v, e;
  if (c.alpha_deg != 0.0) {
    u = std::sin((M_PI / 2.0) - (c.alpha_deg * M_PI / 180.0)) * std::sqrt(gam * c.p_inf / c.rho_inf) * c.mach;
    v = std::cos((M_PI / 2.0) - (c.alpha_deg * M_PI / 180.0)) * std::sqrt(gam * c.p_inf / c.rho_inf) * c.mach;
    e = c.p_inf / (gam - 1.0) + 0.5 * c.rho_inf * (u * u + v * v);
  } else {
    u = std::sqrt(gam * c.p_inf / c.rho_inf) * c.mach;
    v = 0.0;
    e = c.p_inf / (gam - 1.0) + 0.5 * c.rho_inf * (u * u);
  }
  d.P.gam = gam;
  d.P.gm1 = gam - 1.0;
  d.P.rinf = c.rho_inf;
  d.P.uinf = u;
  d.P.vinf = v;
  d.P.pinf = c.p_inf;
  d.P.einf = e;
  d.P.derive();
  ce = cudaMemsetAsync(nd.flux, 0, need, stream);
  if (ce != cudaSuccess) { err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(ce); return -100; }
  DG_DISPATCH(N, (launch_stage<NN>(d, 3, stream)));
  ce = cudaGetLastError();
  if (ce != cudaSuccess) { err = std::string("launch: ") + cudaGetErrorString(ce); return -100; }
  return 0;
}

}  // namespace dg

namespace {
thread_local std::string g_noalloc_err;
}

extern "C" const char *dg_rhs_noalloc_error(void) { return g_noalloc_err.c_str(); }

extern "C" int dg_rhs_noalloc(const dg_config_t *cfg, int n_cells, int n_edges, int n_bedges,
                              const double *W, const double *geo, const int *edges,
                              const int *bedges, double *rhs, void *stream) {
  if (!cfg || n_cells <= 0 || n_edges < 0 || n_bedges < 0 || !W || !geo || !rhs || (n_edges && !edges) ||
      (n_bedges && !bedges)) {
    g_noalloc_err = "bad arguments";
    return DG_ERR_ARG;
  }
  // every cell face is one side of exactly one edge or boundary edge; checked here in 64 bits, so
  // that inconsistent counts never reach the face kernel
  if (2ll * n_edges + n_bedges != 3ll * n_cells) {
    g_noalloc_err = "inconsistent mesh counts: 2 n_edges + n_bedges must equal 3 n_cells";
    return DG_ERR_ARG;
  }
  if (cfg->N < 1 || cfg->N > 6 || cfg->app != 0 || !(cfg->gam > 1.0) || !(cfg->rho_inf > 0.0) || !(cfg->p_inf > 0.0)) {
    g_noalloc_err = "config: N must be 1..6, app 0 (airfoil boundary types), gam > 1, rho_inf and p_inf > 0";
    return DG_ERR_ARG;
  }
  if (((uintptr_t)W | (uintptr_t)geo | (uintptr_t)rhs | (uintptr_t)edges | (uintptr_t)bedges) & 15u) {
    g_noalloc_err = "device arrays must be 16-byte aligned";
    return DG_ERR_ARG;
  }
  dg::Config c;
  c.N = cfg->N;
  c.gam = cfg->gam;
  c.mach = cfg->mach;
  c.alpha_deg = cfg->alpha_deg;
  c.p_inf = cfg->p_inf;
  c.rho_inf = cfg->rho_inf;
  std::string err;
  const int rc = dg::rhs_noalloc(c, n_cells, n_edges, n_bedges, W, geo, (const int4 *)edges,
                                 (const int4 *)bedges, rhs, (cudaStream_t)stream, err);
  if (rc) {
    g_noalloc_err = err;
    return rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG;
  }
  return 0;
}

// ---------------------------------------------------------------- boundary ghost states
// dg_boundary_state (include/dg_gb300.h): the device's ghost-state function bc_state applied to
// n given interior states and unit normals, so that tests can check its physics (Riemann
// invariants, entropy, tangential velocity of the characteristic farfield) independently of
// any restatement of the formula.
namespace dg {
__global__ void boundary_state_kernel(int n, int type, const double *qi, const double *nrm, Phys P, double *qb) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  double a[4], b[4];
  for (int j = 0; j < 4; j++) a[j] = qi[4 * k + j];
  bc_state(type, a, nrm[2 * k], nrm[2 * k + 1], P, b);
  for (int j = 0; j < 4; j++) qb[4 * k + j] = b[j];
}
}  // namespace dg

namespace {
thread_local std::string g_bstate_err;
}
extern "C" const char *dg_boundary_state_error(void) { return g_bstate_err.c_str(); }

extern "C" int dg_boundary_state(const dg_config_t *cfg, int type, int n, const double *qi, const double *nrm,
                                 double *qb) {
  if (!cfg || n <= 0 || !qi || !nrm || !qb || type < 0 || type > 3 || !(cfg->gam > 1.0) || !(cfg->rho_inf > 0.0) ||
      !(cfg->p_inf > 0.0)) {
    g_bstate_err = "bad arguments";
    return DG_ERR_ARG;
  }
  dg::Config c;
  c.gam = cfg->gam;
  c.mach = cfg->mach;
  c.alpha_deg = cfg->alpha_deg;
  c.p_inf = cfg->p_inf;
  c.rho_inf = cfg->rho_inf;
  const dg::Phys P = dg::make_phys(c);
  double *d = nullptr;
  const size_t bytes = (size_t)n * 10 * sizeof(double);
  cudaError_t ce = cudaMalloc(&d, bytes);
  if (ce == cudaSuccess) ce = cudaMemcpy(d, qi, (size_t)n * 4 * sizeof(double), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) ce = cudaMemcpy(d + 4 * (size_t)n, nrm, (size_t)n * 2 * sizeof(double), cudaMemcpyHostToDevice);
  if (ce == cudaSuccess) {
    dg::boundary_state_kernel<<<(n + 127) / 128, 128>>>(n, type, d, d + 4 * (size_t)n, P, d + 6 * (size_t)n);
    ce = cudaGetLastError();
  }
  if (ce == cudaSuccess) ce = cudaMemcpy(qb, d + 6 * (size_t)n, (size_t)n * 4 * sizeof(double), cudaMemcpyDeviceToHost);
  if (d) cudaFree(d);
  if (ce != cudaSuccess) {
    g_bstate_err = std::string("dg_boundary_state: ") + cudaGetErrorString(ce);
    return DG_ERR_CUDA;
  }
  return 0;
}

#include "dg_batch.cuh"
#include "dg_adjoint.cuh"
#include "dg_tangent.cuh"
#include "dg_advec.cuh"

// ---------------------------------------------------------------- batched C ABI
#include "dg_handles.h"

struct dg_batch_t {
  dg::Batch b;
};

namespace {
thread_local std::string g_batch_err;
int batch_fail(int code, const std::string &m) {
  g_batch_err = m;
  return code;
}
}  // namespace

extern "C" const char *dg_batch_last_error(void) { return g_batch_err.c_str(); }

extern "C" int dg_batch_create(int n, const dg_config_t *cfgs, const dg_mesh_t *const *meshes, dg_batch_t **out) {
  if (n <= 0 || !cfgs || !meshes || !out) return batch_fail(DG_ERR_ARG, "bad arguments");
  std::vector<dg::Config> cs(n);
  std::vector<const dg::Mesh *> ms(n);
  for (int k = 0; k < n; k++) {
    const dg_config_t &c = cfgs[k];
    if (c.N < 1 || c.N > 6 || !(c.cfl > 0.0) || !(c.gam > 1.0) || !(c.rho_inf > 0.0) || !(c.p_inf > 0.0) ||
        (c.app != 0 && c.app != 1) || !meshes[k])
      return batch_fail(DG_ERR_ARG, "instance " + std::to_string(k) + ": bad configuration");
    cs[k].N = c.N; cs[k].app = c.app; cs[k].dt_mode = c.dt_mode; cs[k].cfl = c.cfl; cs[k].gam = c.gam;
    cs[k].mach = c.mach; cs[k].alpha_deg = c.alpha_deg; cs[k].p_inf = c.p_inf; cs[k].rho_inf = c.rho_inf;
    cs[k].vortex_x0 = c.vortex_x0; cs[k].vortex_y0 = c.vortex_y0; cs[k].vortex_beta = c.vortex_beta;
    ms[k] = &meshes[k]->m;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return batch_fail(DG_ERR_CUDA, "no CUDA device");
  auto *h = new (std::nothrow) dg_batch_t();
  if (!h) return batch_fail(DG_ERR_ARG, "out of host memory");
  std::string err;
  if (int rc = h->b.create(cs, ms, err)) {
    delete h;
    return batch_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  }
  *out = h;
  return 0;
}

extern "C" int dg_batch_init(dg_batch_t *h) {
  if (!h) return batch_fail(DG_ERR_ARG, "null batch");
  std::string err;
  if (int rc = h->b.init(err)) return batch_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  return 0;
}

extern "C" int dg_batch_autotune(dg_batch_t *h, int steps, double *best_ms_per_step) {
  if (!h || steps <= 0) return batch_fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (int rc = h->b.autotune(steps, err)) return batch_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  if (best_ms_per_step) *best_ms_per_step = h->b.shape.ms_per_step;
  return 0;
}

extern "C" int dg_batch_run(dg_batch_t *h, int nsteps) {
  if (!h || nsteps < 0) return batch_fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (int rc = h->b.run(nsteps, err)) return batch_fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  return 0;
}

extern "C" int dg_batch_sync(dg_batch_t *h) {
  if (!h) return batch_fail(DG_ERR_ARG, "null batch");
  std::string err;
  const int rc = h->b.sync(err);
  if (rc == -200) return batch_fail(DG_ERR_NONPHYSICAL, err);
  if (rc == -8) return batch_fail(DG_ERR_TIMEOUT, err);
  if (rc) return batch_fail(DG_ERR_CUDA, err);
  return 0;
}

// Host-side fault injection for tests: mark the grid barrier as timed out, as a kernel whose
// bounded wait gave up would (no kernel is made to wait).
extern "C" int dg_batch_inject_barrier_timeout(dg_batch_t *h) {
  if (!h) return batch_fail(DG_ERR_ARG, "null batch");
  const unsigned e = 2u;
  if (cudaStreamSynchronize(h->b.stream) != cudaSuccess ||
      cudaMemcpy((char *)h->b.d_bar + offsetof(dg::GridBarrier, err), &e, sizeof(e), cudaMemcpyHostToDevice) != cudaSuccess)
    return batch_fail(DG_ERR_CUDA, "cudaMemcpy");
  return 0;
}

extern "C" int dg_batch_set_barrier_limit(dg_batch_t *h, unsigned long long cycles) {
  if (!h) return batch_fail(DG_ERR_ARG, "null batch");
  std::string err;
  if (h->b.set_barrier_limit(cycles, err)) return batch_fail(DG_ERR_CUDA, err);
  return 0;
}

extern "C" int dg_batch_barrier_check(dg_batch_t *h, unsigned long long hold_cycles) {
  if (!h || hold_cycles > (1ull << 40)) return batch_fail(DG_ERR_ARG, "bad arguments (hold at most 2^40 clocks)");
  std::string err;
  if (h->b.barrier_check(hold_cycles, err)) return batch_fail(DG_ERR_CUDA, err);
  return 0;
}

extern "C" int dg_batch_get(dg_batch_t *h, int k, const char *name, double *host) {
  if (!h || !name || !host || k < 0 || k >= (int)h->b.solvers.size()) return batch_fail(DG_ERR_ARG, "bad arguments");
  dg::Solver *s = h->b.solvers[k];
  const std::string n(name);
  const double *p = n == "q" ? s->d.q : (n == "workingQ" ? s->d.W : nullptr);
  if (!p) return batch_fail(DG_ERR_ARG, "unknown dat " + n);
  cudaError_t ce = cudaStreamSynchronize(h->b.stream);
  if (ce == cudaSuccess) ce = cudaMemcpy(host, p, s->q_count() * 8, cudaMemcpyDeviceToHost);
  if (ce != cudaSuccess) return batch_fail(DG_ERR_CUDA, cudaGetErrorString(ce));
  return 0;
}

extern "C" int dg_batch_time(dg_batch_t *h, int k, double *t, double *dt, unsigned long long *step) {
  if (!h || k < 0 || k >= (int)h->b.solvers.size()) return batch_fail(DG_ERR_ARG, "bad arguments");
  dg::StepState st;
  std::string err;
  if (cudaStreamSynchronize(h->b.stream) != cudaSuccess || h->b.solvers[k]->state(st, err))
    return batch_fail(DG_ERR_CUDA, err);
  if (t) *t = st.t;
  if (dt) *dt = st.dt;
  if (step) *step = st.step;
  return 0;
}

extern "C" int dg_batch_shape(dg_batch_t *h, int *variant, int *block, int *face_tile, int *grid) {
  if (!h) return batch_fail(DG_ERR_ARG, "null batch");
  std::string err;
  if (h->b.ensure_shape(err)) return batch_fail(DG_ERR_ARG, err);
  const auto vs = dg::batch_variants();
  const bool grouped = h->b.shape.variant == dg::kGroupedVariant;
  if (variant) *variant = h->b.shape.variant;
  // grouped launches: the element block of the highest order, and the face-kernel grid
  if (block) *block = grouped ? 32 * dg::np_of(h->b.maxN) : vs[h->b.shape.variant].bs;
  if (face_tile) *face_tile = h->b.shape.face_tile;
  if (grid) *grid = grouped ? h->b.nft : h->b.shape.grid;
  return 0;
}

extern "C" int dg_batch_use_shape(dg_batch_t *h, int variant, int face_tile) {
  if (!h) return batch_fail(DG_ERR_ARG, "null batch");
  std::string err;
  dg::BatchShape sh;
  if (h->b.set_shape(variant, face_tile, sh, err)) return batch_fail(DG_ERR_ARG, err);
  h->b.shape = sh;
  if (h->b.graph_exec) { cudaGraphExecDestroy(h->b.graph_exec); h->b.graph_exec = nullptr; }
  if (h->b.graph) { cudaGraphDestroy(h->b.graph); h->b.graph = nullptr; }
  h->b.graph_ok = true;
  return 0;
}

extern "C" int dg_batch_tried(dg_batch_t *h, int i, int *variant, int *face_tile, double *ms_per_step) {
  if (!h) return batch_fail(DG_ERR_ARG, "null batch");
  const int n = (int)h->b.tried.size();
  if (i < 0) return n;
  if (i >= n) return batch_fail(DG_ERR_ARG, "no such shape");
  const dg::BatchShape &sh = h->b.tried[i];
  if (variant) *variant = sh.variant;
  if (face_tile) *face_tile = sh.face_tile;
  if (ms_per_step) *ms_per_step = sh.ms_per_step;
  return n;
}

extern "C" int dg_batch_uses_graph(dg_batch_t *h) { return h && h->b.graph_exec ? 1 : 0; }
extern "C" void *dg_batch_stream(dg_batch_t *h) { return h ? (void *)h->b.stream : nullptr; }
extern "C" void dg_batch_free(dg_batch_t *h) { delete h; }

