// OP2 drop-in: the op_decl_* / op_arg_* / op_par_loop_<kernel> surface of include/op2_gb300.h.
//
// Each loop is one sm_103a kernel over the loop's set, one thread per set element, that
// restates the reference's user kernel on device copies of the dats in the reference's own
// layout.  The restatements keep the reference's operation order and this file is compiled
// with --fmad=false, so with the same constant tables the results equal the reference's
// (src/*.h with the ascending-index dgemv) bit for bit.  Increments (OP_INC) use atomicAdd,
// which equals OP2's colouring when each slot has a single writer (it does in a valid mesh).
#include <cuda_runtime.h>
#include <sys/time.h>
#include <time.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/op2_gb300.h"

struct op_set_core {
  int size;
  std::string name;
};
struct op_map_core {
  op_set from, to;
  int dim;
  int *d_data;
  std::string name;
};
struct op_dat_core {
  op_set set;
  int dim;
  bool is_double;
  void *d_data;
  std::string name;
};

namespace op2g {

// Device copies of the constants the loops read (names as src/airfoil_op.cpp:144-160).
struct Consts {
  const double *r, *s, *Dr, *Ds, *Drw, *Dsw, *LIFT, *ones;
  const int *FMASK;
  double gam, bc_r, bc_u, bc_v, bc_e;
  double vortex_x0, vortex_y0, vortex_beta;  // the vortex app's constants (vortex.cpp op_decl_const)
  double velX, velY;                         // the advection app's (advec/src/advec.cpp:156-157)
};

struct LoopStat {
  int count = 0;
  double ms = 0.0;
};

struct State {
  std::vector<std::unique_ptr<op_set_core>> sets;
  std::vector<std::unique_ptr<op_map_core>> maps;
  std::vector<std::unique_ptr<op_dat_core>> dats;
  std::map<std::string, std::pair<std::vector<char>, void *>> consts;  // host copy, device copy
  std::map<std::string, LoopStat> stats;
  cudaStream_t stream = nullptr;
  double *d_red = nullptr;  // reduction scratch
  int diags = 0;
  bool exit_on_error = true;
};
State &S() {
  static State s;
  return s;
}
thread_local std::string g_err;

bool fail(const std::string &msg) {
  g_err = msg;
  if (S().exit_on_error) {
    fprintf(stderr, "op2_gb300 error: %s\n", msg.c_str());
    exit(1);
  }
  return false;
}

bool ck(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return true;
  return fail(std::string(what) + ": " + cudaGetErrorString(e));
}

bool ensure_stream() {
  if (S().stream) return true;
  return ck(cudaStreamCreateWithFlags(&S().stream, cudaStreamNonBlocking), "cudaStreamCreate");
}

// ------------------------------------------------------------------ device restatements
template <int N>
struct Ord {
  static constexpr int Np = (N + 1) * (N + 2) / 2, Nfp = N + 1;
};

// y = alpha*A*x + beta*y, row-major, ascending j (the dgemv of the reference's call sites).
__device__ __forceinline__ void gemv(int m, int n, double alpha, const double *a, int lda,
                                     const double *x, int incx, double beta, double *y, int incy) {
  for (int i = 0; i < m; i++) {
    double acc = 0.0;
    for (int j = 0; j < n; j++) acc += a[i * lda + j] * x[j * incx];
    if (beta == 0.0) y[i * incy] = alpha * acc;
    else y[i * incy] = alpha * acc + beta * y[i * incy];
  }
}

// src/init_grid.h:3-106
template <int N>
__global__ void k_init_grid(int n, const double *coords, const int *map, int mdim, int i0, int i1,
                            int i2, double *nodeX, double *nodeY, double *x, double *y, double *xr,
                            double *yr, double *xs, double *ys, double *rx, double *ry, double *sx,
                            double *sy, double *nx, double *ny, double *fscale, const Consts C) {
  constexpr int Np = Ord<N>::Np, Nfp = Ord<N>::Nfp;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double *n0 = coords + 2 * map[c * mdim + i0];
  const double *n1 = coords + 2 * map[c * mdim + i1];
  const double *n2 = coords + 2 * map[c * mdim + i2];
  nodeX += 3 * c; nodeY += 3 * c;
  x += Np * c; y += Np * c; xr += Np * c; yr += Np * c; xs += Np * c; ys += Np * c;
  rx += Np * c; ry += Np * c; sx += Np * c; sy += Np * c;
  nx += 3 * Nfp * c; ny += 3 * Nfp * c; fscale += 3 * Nfp * c;
  nodeX[0] = n0[0]; nodeX[1] = n1[0]; nodeX[2] = n2[0];
  nodeY[0] = n0[1]; nodeY[1] = n1[1]; nodeY[2] = n2[1];
  double temp[Np];
  for (int d = 0; d < 2; d++) {
    double *o = d == 0 ? x : y;
    for (int i = 0; i < Np; i++) o[i] = C.ones[i];
    for (int i = 0; i < Np; i++) o[i] = o[i] + 1.0 * C.r[i];
    for (int i = 0; i < Np; i++) o[i] = (0.5 * n1[d]) * o[i];
    for (int i = 0; i < Np; i++) temp[i] = C.ones[i];
    for (int i = 0; i < Np; i++) temp[i] = temp[i] + 1.0 * C.s[i];
    for (int i = 0; i < Np; i++) o[i] = o[i] + (0.5 * n2[d]) * temp[i];
    for (int i = 0; i < Np; i++) temp[i] = C.s[i];
    for (int i = 0; i < Np; i++) temp[i] = temp[i] + 1.0 * C.r[i];
    for (int i = 0; i < Np; i++) o[i] = o[i] + (-0.5 * n0[d]) * temp[i];
  }
  gemv(Np, Np, 1.0, C.Dr, Np, x, 1, 0.0, xr, 1);
  gemv(Np, Np, 1.0, C.Ds, Np, x, 1, 0.0, xs, 1);
  gemv(Np, Np, 1.0, C.Dr, Np, y, 1, 0.0, yr, 1);
  gemv(Np, Np, 1.0, C.Ds, Np, y, 1, 0.0, ys, 1);
  double J[Np];
  for (int i = 0; i < Np; i++) J[i] = -xs[i] * yr[i] + xr[i] * ys[i];
  for (int i = 0; i < Np; i++) {
    rx[i] = ys[i] / J[i];
    sx[i] = -yr[i] / J[i];
    ry[i] = -xs[i] / J[i];
    sy[i] = xr[i] / J[i];
  }
  const int *F = C.FMASK;
  for (int i = 0; i < Nfp; i++) {
    nx[i] = yr[F[i]];
    ny[i] = -xr[F[i]];
    nx[Nfp + i] = ys[F[Nfp + i]] - yr[F[Nfp + i]];
    ny[Nfp + i] = xr[F[Nfp + i]] - xs[F[Nfp + i]];
    nx[2 * Nfp + i] = -ys[F[2 * Nfp + i]];
    ny[2 * Nfp + i] = xs[F[2 * Nfp + i]];
  }
  for (int i = 0; i < 3 * Nfp; i++) {
    double sJ = sqrt(nx[i] * nx[i] + ny[i] * ny[i]);
    nx[i] = nx[i] / sJ;
    ny[i] = ny[i] / sJ;
    fscale[i] = sJ / J[F[i]];
  }
}

// src/set_ic.h:1-12, one thread per node
__global__ void k_set_ic(long long n_nodes, double *q, double *W, const Consts C) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= n_nodes) return;
  double v[4] = {C.bc_r, C.bc_r * C.bc_u, C.bc_r * C.bc_v, C.bc_e};
  for (int k = 0; k < 4; k++) {
    q[4 * t + k] = v[k];
    W[4 * t + k] = v[k];
  }
}

// The analytic vortex of vortex/src/set_ic.h:6-21 (also get_bedge_q.h, l2_error.h), in their
// operation order.
__device__ void vortex_ref(double x, double y, double t, const Consts &C, double &rho, double &u, double &v,
                           double &ener) {
  const double gam = C.gam, x0 = C.vortex_x0, y0 = C.vortex_y0, beta = C.vortex_beta;
  double r = (x - t - x0) * (x - t - x0) + (y - y0) * (y - y0);
  r = sqrt(r);
  u = 1.0 - beta * exp(1.0 - r * r) * ((y - y0) / (2 * M_PI));
  v = beta * exp(1.0 - r * r) * ((x - x0) / (2 * M_PI));
  rho = 1.0 - ((gam - 1) / (16 * gam * M_PI * M_PI)) * beta * beta * exp(2 * (1.0 - r * r));
  rho = pow(rho, 1.0 / (gam - 1));
  const double p = pow(rho, gam);
  ener = (p / (gam - 1)) + 0.5 * rho * (u * u + v * v);
}

// vortex/src/set_ic.h:3-28, one thread per node
__global__ void k_set_ic_vortex(long long n_nodes, double t, const double *x, const double *y, double *q, double *W,
                                const Consts C) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n_nodes) return;
  double rho, u, v, ener;
  vortex_ref(x[i], y[i], t, C, rho, u, v, ener);
  const double val[4] = {rho, rho * u, rho * v, ener};
  for (int k = 0; k < 4; k++) {
    q[4 * i + k] = val[k];
    W[4 * i + k] = val[k];
  }
}

// vortex/src/get_bedge_q.h:3-40
template <int N>
__global__ void k_get_bedge_q_vortex(int n, const int *bnum, const int *map, int mdim, int i0, const double *xa,
                                     const double *ya, double t, double *exQ, const Consts C) {
  constexpr int Np = Ord<N>::Np, Nfp = Ord<N>::Nfp;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const int c = map[b * mdim + i0], f = bnum[b];
  const double *x = xa + (size_t)Np * c, *y = ya + (size_t)Np * c;
  double *e = exQ + (size_t)12 * Nfp * c + f * 4 * Nfp;
  const int *fm = C.FMASK + f * Nfp;
  for (int i = 0; i < Nfp; i++) {
    double rho, u, v, ener;
    vortex_ref(x[fm[i]], y[fm[i]], t, C, rho, u, v, ener);
    atomicAdd(&e[i * 4], rho);
    atomicAdd(&e[i * 4 + 1], rho * u);
    atomicAdd(&e[i * 4 + 2], rho * v);
    atomicAdd(&e[i * 4 + 3], ener);
  }
}

// vortex/src/l2_error.h:3-29: per-cell sums (the kernel zeroes its accumulators on entry, so the
// cell sums are what OP2's device backends reduce) and the per-node error dat.
template <int N>
__global__ void k_l2_error(int n, const double *xa, const double *ya, const double *qa, double t, double *part,
                           double *err, const Consts C) {
  constexpr int Np = Ord<N>::Np;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const double *x = xa + (size_t)Np * c, *y = ya + (size_t)Np * c, *q = qa + (size_t)4 * Np * c;
  double *error = err + (size_t)4 * Np * c;
  double e0 = 0.0, e1 = 0.0, e2 = 0.0, e3 = 0.0;
  for (int i = 0; i < Np; i++) {
    double rho, u, v, ener;
    vortex_ref(x[i], y[i], t, C, rho, u, v, ener);
    e0 += (q[i * 4] - rho) * (q[i * 4] - rho);
    e1 += (q[i * 4 + 1] - rho * u) * (q[i * 4 + 1] - rho * u);
    e2 += (q[i * 4 + 2] - rho * v) * (q[i * 4 + 2] - rho * v);
    e3 += (q[i * 4 + 3] - ener) * (q[i * 4 + 3] - ener);
    error[i * 4] = (q[i * 4] - rho) * (q[i * 4] - rho);
    error[i * 4 + 1] = (q[i * 4 + 1] - rho * u) * (q[i * 4 + 1] - rho * u);
    error[i * 4 + 2] = (q[i * 4 + 2] - rho * v) * (q[i * 4 + 2] - rho * v);
    error[i * 4 + 3] = (q[i * 4 + 3] - ener) * (q[i * 4 + 3] - ener);
  }
  part[4 * (size_t)c] = e0;
  part[4 * (size_t)c + 1] = e1;
  part[4 * (size_t)c + 2] = e2;
  part[4 * (size_t)c + 3] = e3;
}

// ------------------------------------------------------------------ advection app (advec/src)
// advec/src/set_ic.h:3-10, one thread per node
__global__ void k_adv_set_ic(long long n, const double *x, const double *y, double *q, double *W) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  q[i] = exp(-40.0 * (x[i] - 0.5) * (x[i] - 0.5)) * exp(-40.0 * (y[i] - 0.5) * (y[i] - 0.5));
  W[i] = q[i];
}

// advec/src/get_neighbour_q.h:3-87
template <int N>
__global__ void k_adv_get_neighbour_q(int n, const int *edgeNum, const int *map, int mdim, int iL, int iR,
                                      const double *nodeX, const double *nodeY, const double *W, double *exQ,
                                      const Consts C) {
  constexpr int Np = Ord<N>::Np, Nfp = Ord<N>::Nfp;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int cL = map[e * mdim + iL], cR = map[e * mdim + iR];
  const int edgeL = edgeNum[2 * e], edgeR = edgeNum[2 * e + 1];
  const double *xL = nodeX + 3 * cL, *yL = nodeY + 3 * cL, *xR = nodeX + 3 * cR, *yR = nodeY + 3 * cR;
  const bool reverse = !(xL[edgeL] == xR[edgeR] && yL[edgeL] == yR[edgeR]);
  const double *qL = W + (size_t)Np * cL, *qR = W + (size_t)Np * cR;
  double *eL = exQ + (size_t)3 * Nfp * cL, *eR = exQ + (size_t)3 * Nfp * cR;
  const int *fR = C.FMASK + edgeR * Nfp, *fL = C.FMASK + edgeL * Nfp;
  for (int i = 0; i < Nfp; i++) {
    atomicAdd(&eL[edgeL * Nfp + i], qR[reverse ? fR[Nfp - i - 1] : fR[i]]);
    atomicAdd(&eR[edgeR * Nfp + i], qL[reverse ? fL[Nfp - i - 1] : fL[i]]);
  }
}

// advec/src/get_bedge_q.h:3-13
template <int N>
__global__ void k_adv_get_bedge_q(int n, const int *bnum, const int *map, int mdim, int i0, double *exQ) {
  constexpr int Nfp = Ord<N>::Nfp;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  double *e = exQ + (size_t)3 * Nfp * map[b * mdim + i0] + bnum[b] * Nfp;
  for (int i = 0; i < Nfp; i++) atomicAdd(&e[i], 4.5e-5);
}

// advec/src/advec_rhs.h:7-67, one thread per (cell, node) for the volume and lift dot products
// (each in ascending order) and per (cell, face point) for the face flux, T cells per block.
template <int N>
__global__ void __launch_bounds__(128) k_advec_rhs(int n, const double *qa, const double *exQa, const double *rxa,
                                                    const double *rya, const double *sxa, const double *sya,
                                                    const double *fsa, const double *nxa, const double *nya,
                                                    double *rhsa, const Consts C) {
  constexpr int Np = Ord<N>::Np, Nfp = Ord<N>::Nfp, T = 16;
  __shared__ double F[T * Np], G[T * Np], FL[T * 3 * Nfp];
  const int c0 = blockIdx.x * T;
  const int nc = min(T, n - c0);
  const double velX = C.velX, velY = C.velY;
  for (int t = threadIdx.x; t < nc * Np; t += blockDim.x) {
    const double q = qa[(size_t)Np * c0 + t];
    F[t] = velX * q;
    G[t] = velY * q;
  }
  const double a = sqrt(velX * velX + velY * velY);
  for (int t = threadIdx.x; t < nc * 3 * Nfp; t += blockDim.x) {
    const int cl = t / (3 * Nfp), j = t - cl * 3 * Nfp;
    const size_t c = c0 + cl;
    const double mQ = qa[(size_t)Np * c + C.FMASK[j]], pQ = exQa[(size_t)3 * Nfp * c + j];
    const double mF = velX * mQ, mG = velY * mQ, pF = velX * pQ, pG = velY * pQ;
    const size_t f = (size_t)3 * Nfp * c + j;
    double nf = nxa[f] * (mF + pF) + nya[f] * (mG + pG) + a * (mQ - pQ);
    nf *= 0.5 * fsa[f];
    FL[t] = nf;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nc * Np; t += blockDim.x) {
    const int cl = t / Np, i = t - cl * Np;
    const double *Fc = F + cl * Np, *Gc = G + cl * Np;
    double dFdr = 0.0, dFds = 0.0, dGdr = 0.0, dGds = 0.0;
    for (int k = 0; k < Np; k++) dFdr += C.Drw[i * Np + k] * Fc[k];
    for (int k = 0; k < Np; k++) dFds += C.Dsw[i * Np + k] * Fc[k];
    for (int k = 0; k < Np; k++) dGdr += C.Drw[i * Np + k] * Gc[k];
    for (int k = 0; k < Np; k++) dGds += C.Dsw[i * Np + k] * Gc[k];
    dFdr = 1.0 * dFdr; dFds = 1.0 * dFds; dGdr = 1.0 * dGdr; dGds = 1.0 * dGds;
    const size_t o = (size_t)Np * c0 + t;
    const double vol = rxa[o] * dFdr + sxa[o] * dFds + rya[o] * dGdr + sya[o] * dGds;
    double lift = 0.0;
    for (int k = 0; k < 3 * Nfp; k++) lift += C.LIFT[i * 3 * Nfp + k] * FL[cl * 3 * Nfp + k];
    rhsa[o] = -1.0 * lift + 1.0 * vol;
  }
}

// advec/src/set_workingQ.h:1-6, one thread per value
__global__ void k_adv_set_workingQ(long long n, double dt, double frac, const double *q, const double *rk, double *W) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i < n) W[i] = q[i] + dt * frac * rk[i];
}

// advec/src/update_Q.h:1-8, one thread per value
__global__ void k_adv_update_Q(long long n, double dt, double *q, const double *k1, const double *k2, const double *k3,
                               const double *k4, double *W) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  q[i] = q[i] + (1.0 / 6.0) * dt * (k1[i] + 2 * k2[i] + 2 * k3[i] + k4[i]);
  W[i] = q[i];
}

__global__ void k_zero(long long n, double *p) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t < n) p[t] = 0.0;
}

// src/calc_dt.h:3-22, the OP_MAX combined on the bit patterns of non-negative doubles
template <int N>
__global__ void k_calc_dt(int n, const double *q, const double *fscale, double seed,
                          unsigned long long *red, const Consts C) {
  constexpr int Np = Ord<N>::Np, Nfp = Ord<N>::Nfp;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  double max = seed;
  if (c < n) {
    const double *qc = q + (size_t)4 * Np * c;
    const double *fs = fscale + (size_t)3 * Nfp * c;
    const int *F = C.FMASK;
    const double gam = C.gam;
    for (int i = 0; i < 3 * Nfp; i++) {
      double rho = qc[F[i] * 4];
      double u = qc[F[i] * 4 + 1] / rho;
      double v = qc[F[i] * 4 + 2] / rho;
      double p = (gam - 1.0) * (qc[F[i] * 4 + 3] - rho * (u * u + v * v) * 0.5);
      double cs = sqrt(fabs(gam * p / rho));
      const int fi = (Np <= 3 * Nfp) ? F[i] : i;
      double val = ((N + 1) * (N + 1)) * 0.5 * fs[fi] * (sqrt(u * u + v * v) + cs);
      if (val > max) max = val;
    }
  }
  unsigned long long b = max > 0.0 ? (unsigned long long)__double_as_longlong(max) : 0ull;
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xffffffffu, b, o);
    b = x > b ? x : b;
  }
  if ((threadIdx.x & 31) == 0 && b) atomicMax(red, b);
}

// src/get_neighbour_q.h:1-89
template <int N>
__global__ void k_get_neighbour_q(int n, const int *edgeNum, const int *map, int mdim, int iL,
                                  int iR, const double *nodeX, const double *nodeY, const double *W,
                                  double *exQ, const Consts C) {
  constexpr int Np = Ord<N>::Np, Nfp = Ord<N>::Nfp;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  const int cL = map[e * mdim + iL], cR = map[e * mdim + iR];
  const int edgeL = edgeNum[2 * e], edgeR = edgeNum[2 * e + 1];
  const double *xL = nodeX + 3 * cL, *yL = nodeY + 3 * cL, *xR = nodeX + 3 * cR, *yR = nodeY + 3 * cR;
  const bool reverse = !(xL[edgeL] == xR[edgeR] && yL[edgeL] == yR[edgeR]);
  const double *qL = W + (size_t)4 * Np * cL, *qR = W + (size_t)4 * Np * cR;
  double *eL = exQ + (size_t)12 * Nfp * cL, *eR = exQ + (size_t)12 * Nfp * cR;
  const int *fR = C.FMASK + edgeR * Nfp, *fL = C.FMASK + edgeL * Nfp;
  for (int i = 0; i < Nfp; i++) {
    const int ri = 4 * (reverse ? fR[Nfp - i - 1] : fR[i]);
    for (int k = 0; k < 4; k++) atomicAdd(&eL[edgeL * 4 * Nfp + 4 * i + k], qR[ri + k]);
  }
  for (int i = 0; i < Nfp; i++) {
    const int li = 4 * (reverse ? fL[Nfp - i - 1] : fL[i]);
    for (int k = 0; k < 4; k++) atomicAdd(&eR[edgeR * 4 * Nfp + 4 * i + k], qL[li + k]);
  }
}

// src/get_bedge_q.h:1-51
template <int N>
__global__ void k_get_bedge_q(int n, const int *btype, const int *bnum, const int *map, int mdim,
                              int i0, const double *nxa, const double *nya, const double *W,
                              double *exQ, const Consts C) {
  constexpr int Np = Ord<N>::Np, Nfp = Ord<N>::Nfp;
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  const int c = map[b * mdim + i0];
  const int f = bnum[b];
  const double *q = W + (size_t)4 * Np * c;
  const double *nx = nxa + (size_t)3 * Nfp * c, *ny = nya + (size_t)3 * Nfp * c;
  double *e = exQ + (size_t)12 * Nfp * c;
  const int exInd = f * 4 * Nfp, nInd = f * Nfp;
  const int *fm = C.FMASK + f * Nfp;
  for (int i = 0; i < Nfp; i++) {
    const int qi = fm[i] * 4;
    double v[4];
    if (btype[b] == 0) {
      v[0] = C.bc_r; v[1] = C.bc_r * C.bc_u; v[2] = C.bc_r * C.bc_v; v[3] = C.bc_e;
    } else if (btype[b] == 1) {
      v[0] = C.bc_r; v[1] = C.bc_r * C.bc_u; v[2] = C.bc_r * C.bc_v; v[3] = q[qi + 3];
    } else {
      v[0] = q[qi];
      v[1] = q[qi + 1] - 2 * (nx[nInd + i] * q[qi + 1] + ny[nInd + i] * q[qi + 2]) * nx[nInd + i];
      v[2] = q[qi + 2] - 2 * (nx[nInd + i] * q[qi + 1] + ny[nInd + i] * q[qi + 2]) * ny[nInd + i];
      v[3] = q[qi + 3];
    }
    for (int k = 0; k < 4; k++) atomicAdd(&e[exInd + i * 4 + k], v[k]);
  }
}

// src/euler_rhs.h:7-23
__device__ __forceinline__ void euler_flux(const double *q, double *F, double *G, double &rho,
                                           double &u, double &v, double &p, double gam) {
  rho = q[0];
  u = q[1] / rho;
  v = q[2] / rho;
  p = (gam - 1) * (q[3] - 0.5 * (q[1] * u + q[2] * v));
  F[0] = q[1];
  F[1] = q[1] * u + p;
  F[2] = q[2] * u;
  F[3] = u * (q[3] + p);
  G[0] = q[2];
  G[1] = q[1] * v;
  G[2] = q[2] * v + p;
  G[3] = v * (q[3] + p);
}

// src/euler_rhs.h:120-220: the Roe flux at face point i of a cell, times fscale, into out[4].
template <int N>
__device__ __forceinline__ void roe_point(const double *q, const double *exQ, const double *nx, const double *ny,
                                          const double *fscale, const int i, const Consts &C, double *out) {
  const double gam = C.gam;
  const int ind = C.FMASK[i] * 4;
  const double *pq = &exQ[i * 4];
  double mRoeQ[4], pRoeQ[4];
  mRoeQ[0] = q[ind];
  mRoeQ[1] = nx[i] * q[ind + 1] + ny[i] * q[ind + 2];
  mRoeQ[2] = -ny[i] * q[ind + 1] + nx[i] * q[ind + 2];
  mRoeQ[3] = q[ind + 3];
  pRoeQ[0] = pq[0];
  pRoeQ[1] = nx[i] * pq[1] + ny[i] * pq[2];
  pRoeQ[2] = -ny[i] * pq[1] + nx[i] * pq[2];
  pRoeQ[3] = pq[3];
  double fxMQ[4], fyMQ[4], mRoeRho, mRoeU, mRoeV, mRoeP;
  euler_flux(mRoeQ, fxMQ, fyMQ, mRoeRho, mRoeU, mRoeV, mRoeP, gam);
  double fxPQ[4], fyPQ[4], pRoeRho, pRoeU, pRoeV, pRoeP;
  euler_flux(pRoeQ, fxPQ, fyPQ, pRoeRho, pRoeU, pRoeV, pRoeP, gam);
  double mH = (mRoeQ[3] + mRoeP) / mRoeRho;
  double pH = (pRoeQ[3] + pRoeP) / pRoeRho;
  double mS = sqrt(mRoeRho), pS = sqrt(pRoeRho);
  double rho = mS * pS;
  double u = (mS * mRoeU + pS * pRoeU) / (mS + pS);
  double v = (mS * mRoeV + pS * pRoeV) / (mS + pS);
  double H = (mS * mH + pS * pH) / (mS + pS);
  double c2 = (gam - 1) * (H - 0.5 * (u * u + v * v));
  double cc = sqrt(c2);
  double dW1 = -0.5 * rho * (pRoeU - mRoeU) / cc + 0.5 * (pRoeP - mRoeP) / c2;
  double dW2 = (pRoeRho - mRoeRho) - (pRoeP - mRoeP) / c2;
  double dW3 = rho * (pRoeV - mRoeV);
  double dW4 = 0.5 * rho * (pRoeU - mRoeU) / cc + 0.5 * (pRoeP - mRoeP) / c2;
  dW1 = fabs(u - cc) * dW1;
  dW2 = fabs(u) * dW2;
  dW3 = fabs(u) * dW3;
  dW4 = fabs(u + cc) * dW4;
  double fx[4];
  for (int k = 0; k < 4; k++) fx[k] = (fxMQ[k] + fxPQ[k]) / 2.0;
  fx[0] = fx[0] - (dW1 + dW2 + dW4) / 2.0;
  fx[1] = fx[1] - (dW1 * (u - cc) + dW2 * u + dW4 * (u + cc)) / 2.0;
  fx[2] = fx[2] - (dW1 * v + dW2 * v + dW3 + dW4 * v) / 2.0;
  fx[3] = fx[3] - (dW1 * (H - u * cc) + dW2 * (u * u + v * v) + dW3 * v + dW4 * (H + u * cc)) / 2.0;
  out[0] = fx[0] * fscale[i];
  out[1] = (nx[i] * fx[1] - ny[i] * fx[2]) * fscale[i];
  out[2] = (ny[i] * fx[1] + nx[i] * fx[2]) * fscale[i];
  out[3] = fx[3] * fscale[i];
}

// src/euler_rhs.h:222-291 for a tile of T cells per block, work spread over the tile's nodes and
// face points: (1) nodal fluxes F, G (:226-229), (2) the Roe flux of every face point
// (:281-282), (3) per node and variable the four weak-derivative dot products (:240-243, each in
// ascending order, as the ascending-index dgemv), their metric combination (:245-247) and the
// LIFT dot product (:284-286), (4) exteriorQ zeroed when the loop has it OP_RW (:288-290).  Every
// value is formed by the same operations in the same order as the one-cell kernel.
template <int N>
__global__ void __launch_bounds__(128) k_euler_rhs(int n, int T, const double *Wa, double *exQa,
                                                    const double *rxa, const double *rya,
                                                    const double *sxa, const double *sya,
                                                    const double *fsa, const double *nxa,
                                                    const double *nya, double *rhsa, const Consts C,
                                                    const bool zero_ext) {
  constexpr int Np = Ord<N>::Np, Nfp = Ord<N>::Nfp;
  extern __shared__ double sh[];
  double *F = sh, *G = sh + (size_t)T * 4 * Np, *FL = sh + (size_t)T * 8 * Np;  // [T][4Np], [T][4Np], [T][12Nfp]
  const int c0 = blockIdx.x * T;
  const int nc = min(T, n - c0);
  for (int t = threadIdx.x; t < nc * Np; t += blockDim.x) {
    const int cl = t / Np, j = t - cl * Np;
    double rho, u, v, p;
    euler_flux(Wa + (size_t)4 * Np * (c0 + cl) + 4 * j, F + (size_t)cl * 4 * Np + 4 * j, G + (size_t)cl * 4 * Np + 4 * j,
               rho, u, v, p, C.gam);
  }
  for (int t = threadIdx.x; t < nc * 3 * Nfp; t += blockDim.x) {
    const int cl = t / (3 * Nfp), i = t - cl * 3 * Nfp;
    const size_t c = c0 + cl;
    roe_point<N>(Wa + 4 * Np * c, exQa + 12 * Nfp * c, nxa + 3 * Nfp * c, nya + 3 * Nfp * c, fsa + 3 * Nfp * c, i, C,
                 FL + (size_t)cl * 12 * Nfp + 4 * i);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nc * Np * 4; t += blockDim.x) {
    const int cl = t / (4 * Np), r = t - cl * 4 * Np, j = r >> 2, var = r & 3;
    const size_t c = c0 + cl;
    const double *Fc = F + (size_t)cl * 4 * Np, *Gc = G + (size_t)cl * 4 * Np;
    double dFdr = 0.0, dFds = 0.0, dGdr = 0.0, dGds = 0.0;
    for (int k = 0; k < Np; k++) dFdr += C.Drw[j * Np + k] * Fc[k * 4 + var];
    for (int k = 0; k < Np; k++) dFds += C.Dsw[j * Np + k] * Fc[k * 4 + var];
    for (int k = 0; k < Np; k++) dGdr += C.Drw[j * Np + k] * Gc[k * 4 + var];
    for (int k = 0; k < Np; k++) dGds += C.Dsw[j * Np + k] * Gc[k * 4 + var];
    dFdr = 1.0 * dFdr; dFds = 1.0 * dFds; dGdr = 1.0 * dGdr; dGds = 1.0 * dGds;
    const size_t o = (size_t)Np * c + j;
    const double vol = (rxa[o] * dFdr + sxa[o] * dFds) + (rya[o] * dGdr + sya[o] * dGds);
    const double *fl = FL + (size_t)cl * 12 * Nfp;
    double lift = 0.0;
    for (int k = 0; k < 3 * Nfp; k++) lift += C.LIFT[j * 3 * Nfp + k] * fl[k * 4 + var];
    rhsa[4 * Np * c + 4 * j + var] = -1.0 * lift + 1.0 * vol;
  }
  if (zero_ext) {  // the airfoil copy zeroes exteriorQ (OP_RW); the vortex copy reads it (OP_READ)
    __syncthreads();
    for (int t = threadIdx.x; t < nc * 12 * Nfp; t += blockDim.x) exQa[(size_t)12 * Nfp * c0 + t] = 0.0;
  }
}

// src/set_workingQ.h:1-12, one thread per value
__global__ void k_set_workingQ(long long n, double dt, int stage, const double *q, const double *k1,
                               const double *k2, double *W) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (stage == 0) W[i] = q[i] + dt * k1[i];
  else W[i] = q[i] + dt * (k1[i] / 4.0 + k2[i] / 4.0);
}

// src/update_Q.h:1-12, one thread per value
__global__ void k_update_Q(long long n, double dt, double *q, const double *k1, const double *k2,
                           const double *k3, double *W) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  q[i] = q[i] + dt * (k1[i] / 6.0 + k2[i] / 6.0 + 2.0 * k3[i] / 3.0);
  W[i] = q[i];
}

// ------------------------------------------------------------------ host helpers
#define DISPATCH_N(NN_, ...)                           \
  switch (NN_) {                                       \
    case 1: { constexpr int N = 1; __VA_ARGS__; } break; \
    case 2: { constexpr int N = 2; __VA_ARGS__; } break; \
    case 3: { constexpr int N = 3; __VA_ARGS__; } break; \
    case 4: { constexpr int N = 4; __VA_ARGS__; } break; \
    case 5: { constexpr int N = 5; __VA_ARGS__; } break; \
    default: { constexpr int N = 6; __VA_ARGS__; } break; \
  }

int order_from_np(int np) {
  for (int n = 1; n <= 6; n++)
    if ((n + 1) * (n + 2) / 2 == np) return n;
  return -1;
}

template <class T>
const T *cdev(const char *name, size_t count) {
  auto it = S().consts.find(name);
  if (it == S().consts.end()) return nullptr;
  if (it->second.first.size() < count * sizeof(T)) return nullptr;
  return (const T *)it->second.second;
}

double chost(const char *name, bool &ok) {
  auto it = S().consts.find(name);
  if (it == S().consts.end() || it->second.first.size() < sizeof(double)) {
    ok = false;
    return 0.0;
  }
  double v;
  std::memcpy(&v, it->second.first.data(), sizeof(double));
  return v;
}

// Constants a loop of order N needs; fails with a message naming the first missing one.
// Which scalar constants a loop reads: the airfoil freestream (bc_*), the vortex parameters, or
// only gam (geometry, dt, RHS and update loops are shared by both apps).
enum Need { kFreestream, kVortex, kGamOnly, kNone, kAdvec };

bool consts_for(int N, bool need_ops, Consts &c, Need need = kGamOnly) {
  const int Np = (N + 1) * (N + 2) / 2, Nfp = N + 1;
  std::memset(&c, 0, sizeof(c));
  bool ok = true;
  if (need == kAdvec) {  // the advection app declares no gam
    c.velX = chost("velX", ok);
    c.velY = chost("velY", ok);
    if (!ok) return fail("constants velX, velY must be declared with op_decl_const2");
  } else if (need != kNone) {
    c.gam = chost("gam", ok);
    if (!ok) return fail("constant gam must be declared with op_decl_const2");
  }
  if (need == kVortex) {
    c.vortex_x0 = chost("vortex_x0", ok);
    c.vortex_y0 = chost("vortex_y0", ok);
    c.vortex_beta = chost("vortex_beta", ok);
    if (!ok) return fail("constants vortex_x0, vortex_y0, vortex_beta must be declared with op_decl_const2");
  } else if (need == kFreestream) {
    c.bc_r = chost("bc_r", ok);
    c.bc_u = chost("bc_u", ok);
    c.bc_v = chost("bc_v", ok);
    c.bc_e = chost("bc_e", ok);
    if (!ok) return fail("constants bc_r, bc_u, bc_v, bc_e must be declared with op_decl_const2");
  }
  c.FMASK = cdev<int>("FMASK", 3 * Nfp);
  if (!c.FMASK) return fail("constant FMASK (3*Nfp ints) not declared");
  if (need_ops) {
    c.r = cdev<double>("r", Np);
    c.s = cdev<double>("s", Np);
    c.ones = cdev<double>("ones", Np);
    c.Dr = cdev<double>("Dr", Np * Np);
    c.Ds = cdev<double>("Ds", Np * Np);
    c.Drw = cdev<double>("Drw", Np * Np);
    c.Dsw = cdev<double>("Dsw", Np * Np);
    c.LIFT = cdev<double>("LIFT", Np * 3 * Nfp);
    if (!c.r || !c.s || !c.ones || !c.Dr || !c.Ds || !c.Drw || !c.Dsw || !c.LIFT)
      return fail("constants r, s, ones, Dr, Ds, Drw, Dsw, LIFT of order " + std::to_string(N) +
                  " must be declared with op_decl_const2");
  }
  return true;
}

// Argument checks against the reference's call sites.
bool arg_dat(const op_arg &a, op_set loop_set, bool direct, int dim, bool dbl, const char *what) {
  if (a.argtype != OP_ARG_DAT || !a.dat) return fail(std::string(what) + ": expected op_arg_dat");
  if (a.dat->dim != dim || a.dim != dim) return fail(std::string(what) + ": dat " + a.dat->name + " has the wrong dim");
  if (a.dat->is_double != dbl) return fail(std::string(what) + ": dat " + a.dat->name + " has the wrong type");
  if (direct) {
    if (a.map || a.dat->set != loop_set) return fail(std::string(what) + ": expected a direct argument on the loop set");
  } else {
    if (!a.map || a.map->from != loop_set || a.map->to != a.dat->set || a.idx < 0 || a.idx >= a.map->dim)
      return fail(std::string(what) + ": expected an indirect argument through a map from the loop set");
  }
  return true;
}
bool arg_gbl(const op_arg &a, int dim, bool dbl, const char *what) {
  if (a.argtype != OP_ARG_GBL || !a.data || a.dim != dim || (std::strcmp(a.type, dbl ? "double" : "int") != 0))
    return fail(std::string(what) + ": expected op_arg_gbl of " + std::to_string(dim) + (dbl ? " double" : " int"));
  return true;
}

template <class T>
T *dptr(const op_arg &a) {
  return (T *)a.dat->d_data;
}

struct Timed {
  cudaEvent_t a = nullptr, b = nullptr;
  std::string name;
  explicit Timed(const char *n) : name(n) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, S().stream);
  }
  void done() {
    cudaEventRecord(b, S().stream);
    cudaEventSynchronize(b);  // loops are short; timing every one matches op_timers in the driver
    float ms = 0;
    cudaEventElapsedTime(&ms, a, b);
    LoopStat &st = S().stats[name];
    st.count++;
    st.ms += ms;
  }
  ~Timed() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

unsigned blocks(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace op2g

using namespace op2g;

extern "C" {

const char *op2_gb300_last_error(void) { return g_err.c_str(); }
void op2_gb300_clear_error(void) { g_err.clear(); }
void op2_gb300_set_exit_on_error(int on) { S().exit_on_error = on != 0; }

int op2_gb300_sync(void) {
  if (!S().stream) return 0;
  cudaError_t e = cudaStreamSynchronize(S().stream);
  if (e != cudaSuccess) {
    g_err = cudaGetErrorString(e);
    return -1;
  }
  return 0;
}

void op2_gb300_reset(void) {
  State &s = S();
  if (s.stream) cudaStreamSynchronize(s.stream);
  for (auto &m : s.maps) cudaFree(m->d_data);
  for (auto &d : s.dats) cudaFree(d->d_data);
  for (auto &c : s.consts) cudaFree(c.second.second);
  if (s.d_red) cudaFree(s.d_red);
  s.d_red = nullptr;
  s.maps.clear();
  s.dats.clear();
  s.sets.clear();
  s.consts.clear();
  s.stats.clear();
}

void op_init(int argc, char **argv, int diags) {
  (void)argc;
  (void)argv;
  S().diags = diags;
  ensure_stream();
}

void op_exit(void) { op2_gb300_reset(); }

op_set op_decl_set(int size, char const *name) {
  if (size < 0) { fail("op_decl_set: negative size"); return nullptr; }
  auto s = std::make_unique<op_set_core>();
  s->size = size;
  s->name = name ? name : "";
  S().sets.push_back(std::move(s));
  return S().sets.back().get();
}

op_map op_decl_map(op_set from, op_set to, int dim, int *imap, char const *name) {
  if (!from || !to || dim <= 0 || (!imap && from->size)) { fail("op_decl_map: bad arguments"); return nullptr; }
  for (long long i = 0; i < (long long)from->size * dim; i++)
    if (imap[i] < 0 || imap[i] >= to->size) {
      fail(std::string("op_decl_map ") + (name ? name : "") + ": entry out of range");
      return nullptr;
    }
  if (!ensure_stream()) return nullptr;
  auto m = std::make_unique<op_map_core>();
  m->from = from;
  m->to = to;
  m->dim = dim;
  m->name = name ? name : "";
  const size_t bytes = (size_t)from->size * dim * sizeof(int);
  m->d_data = nullptr;
  if (!ck(cudaMalloc(&m->d_data, bytes ? bytes : 4), "cudaMalloc")) return nullptr;
  if (bytes && !ck(cudaMemcpy(m->d_data, imap, bytes, cudaMemcpyHostToDevice), "cudaMemcpy")) return nullptr;
  S().maps.push_back(std::move(m));
  return S().maps.back().get();
}

op_dat op_decl_dat(op_set set, int dim, char const *type, void *data, char const *name) {
  if (!set || dim <= 0 || !type) { fail("op_decl_dat: bad arguments"); return nullptr; }
  const bool dbl = std::strcmp(type, "double") == 0;
  if (!dbl && std::strcmp(type, "int") != 0) { fail(std::string("op_decl_dat: unsupported type ") + type); return nullptr; }
  if (!ensure_stream()) return nullptr;
  auto d = std::make_unique<op_dat_core>();
  d->set = set;
  d->dim = dim;
  d->is_double = dbl;
  d->name = name ? name : "";
  const size_t bytes = (size_t)set->size * dim * (dbl ? 8 : 4);
  d->d_data = nullptr;
  if (!ck(cudaMalloc(&d->d_data, bytes ? bytes : 8), "cudaMalloc")) return nullptr;
  if (bytes) {
    if (data) {
      if (!ck(cudaMemcpy(d->d_data, data, bytes, cudaMemcpyHostToDevice), "cudaMemcpy")) return nullptr;
    } else if (!ck(cudaMemset(d->d_data, 0, bytes), "cudaMemset")) {
      return nullptr;
    }
  }
  S().dats.push_back(std::move(d));
  return S().dats.back().get();
}

void op_decl_const2(char const *name, int dim, char const *type, void *data) {
  if (!name || !data || dim <= 0 || !type) { fail("op_decl_const2: bad arguments"); return; }
  const bool dbl = std::strcmp(type, "double") == 0;
  if (!dbl && std::strcmp(type, "int") != 0) { fail(std::string("op_decl_const2: unsupported type ") + type); return; }
  if (!ensure_stream()) return;
  const size_t bytes = (size_t)dim * (dbl ? 8 : 4);
  auto &slot = S().consts[name];
  if (slot.second) cudaFree(slot.second);
  slot.first.assign((const char *)data, (const char *)data + bytes);
  slot.second = nullptr;
  if (!ck(cudaMalloc(&slot.second, bytes), "cudaMalloc")) return;
  ck(cudaMemcpy(slot.second, data, bytes, cudaMemcpyHostToDevice), "cudaMemcpy");
}

op_arg op_arg_dat(op_dat dat, int idx, op_map map, int dim, char const *type, op_access acc) {
  op_arg a;
  std::memset(&a, 0, sizeof(a));
  a.dat = dat;
  a.map = map;
  a.idx = map ? idx : -1;
  a.dim = dim;
  a.size = dim * ((type && std::strcmp(type, "int") == 0) ? 4 : 8);
  a.acc = acc;
  a.argtype = OP_ARG_DAT;
  a.type = type;
  return a;
}

op_arg op_arg_gbl(void *data, int dim, char const *type, op_access acc) {
  op_arg a;
  std::memset(&a, 0, sizeof(a));
  a.dim = dim;
  a.size = dim * ((type && std::strcmp(type, "int") == 0) ? 4 : 8);
  a.acc = acc;
  a.argtype = OP_ARG_GBL;
  a.data = (char *)data;
  a.type = type;
  a.idx = -1;
  return a;
}

void op_fetch_data(op_dat dat, void *data) {
  if (!dat || !data) { fail("op_fetch_data: bad arguments"); return; }
  const size_t bytes = (size_t)dat->set->size * dat->dim * (dat->is_double ? 8 : 4);
  if (!ck(cudaMemcpyAsync(data, dat->d_data, bytes, cudaMemcpyDeviceToHost, S().stream), "cudaMemcpyAsync")) return;
  ck(cudaStreamSynchronize(S().stream), "cudaStreamSynchronize");
}

int op_get_size(op_set set) { return set ? set->size : 0; }

void op_timers(double *cpu, double *wall) {
  struct timeval t;
  gettimeofday(&t, nullptr);
  if (wall) *wall = t.tv_sec + t.tv_usec * 1e-6;
  if (cpu) *cpu = (double)clock() / CLOCKS_PER_SEC;
}

void op_timing_output(void) {
  printf("\n  count   device time (ms)   kernel\n");
  for (auto &kv : S().stats)
    printf(" %6d  %16.4f   %s\n", kv.second.count, kv.second.ms, kv.first.c_str());
}

// ------------------------------------------------------------------ loops
// src/airfoil.cpp:204-222
void op_par_loop_init_grid(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                           op_arg a3, op_arg a4, op_arg a5, op_arg a6, op_arg a7, op_arg a8,
                           op_arg a9, op_arg a10, op_arg a11, op_arg a12, op_arg a13,
                           op_arg a14, op_arg a15, op_arg a16, op_arg a17) {
  if (!set) { fail("init_grid: null set"); return; }
  const int Np = a5.dim, N = order_from_np(Np);
  if (N < 0) { fail("init_grid: x dim is not a triangle node count of order 1..6"); return; }
  const int Nfp = N + 1;
  if (!arg_dat(a0, set, false, 2, true, "init_grid arg0") || !arg_dat(a1, set, false, 2, true, "init_grid arg1") ||
      !arg_dat(a2, set, false, 2, true, "init_grid arg2") || a0.map != a1.map || a0.map != a2.map ||
      a0.dat != a1.dat || a0.dat != a2.dat)
    return (void)fail("init_grid: args 0-2 must read one coordinate dat through one map");
  if (!arg_dat(a3, set, true, 3, true, "init_grid nodeX") || !arg_dat(a4, set, true, 3, true, "init_grid nodeY")) return;
  const op_arg *np_args[10] = {&a5, &a6, &a7, &a8, &a9, &a10, &a11, &a12, &a13, &a14};
  for (auto *a : np_args)
    if (!arg_dat(*a, set, true, Np, true, "init_grid node dat")) return;
  const op_arg *f_args[3] = {&a15, &a16, &a17};
  for (auto *a : f_args)
    if (!arg_dat(*a, set, true, 3 * Nfp, true, "init_grid face dat")) return;
  Consts C;
  if (!consts_for(N, true, C, kNone)) return;
  Timed t(name ? name : "init_grid");
  DISPATCH_N(N, (k_init_grid<N><<<blocks(set->size, 128), 128, 0, S().stream>>>(
                    set->size, dptr<double>(a0), a0.map->d_data, a0.map->dim, a0.idx, a1.idx, a2.idx,
                    dptr<double>(a3), dptr<double>(a4), dptr<double>(a5), dptr<double>(a6), dptr<double>(a7),
                    dptr<double>(a8), dptr<double>(a9), dptr<double>(a10), dptr<double>(a11), dptr<double>(a12),
                    dptr<double>(a13), dptr<double>(a14), dptr<double>(a15), dptr<double>(a16),
                    dptr<double>(a17), C)));
  if (!ck(cudaGetLastError(), "init_grid launch")) return;
  t.done();
}

// src/airfoil.cpp:224-226
void op_par_loop_set_ic(char const *name, op_set set, op_arg a0, op_arg a1) {
  if (!set) { fail("set_ic: null set"); return; }
  const int dim = a0.dim;
  if (order_from_np(dim / 4) < 0 || dim % 4) { fail("set_ic: q dim must be 4*Np"); return; }
  if (!arg_dat(a0, set, true, dim, true, "set_ic q") || !arg_dat(a1, set, true, dim, true, "set_ic workingQ")) return;
  Consts C;
  if (!consts_for(order_from_np(dim / 4), false, C, kFreestream)) return;
  Timed t(name ? name : "set_ic");
  const long long n = (long long)set->size * dim / 4;
  k_set_ic<<<blocks(n, 256), 256, 0, S().stream>>>(n, dptr<double>(a0), dptr<double>(a1), C);
  if (!ck(cudaGetLastError(), "set_ic launch")) return;
  t.done();
}

// src/airfoil.cpp:228-229
void op_par_loop_neighbour_zero(char const *name, op_set set, op_arg a0) {
  if (!set) { fail("neighbour_zero: null set"); return; }
  if (!arg_dat(a0, set, true, a0.dim, true, "neighbour_zero")) return;
  Timed t(name ? name : "neighbour_zero");
  const long long n = (long long)set->size * a0.dim;
  k_zero<<<blocks(n, 256), 256, 0, S().stream>>>(n, dptr<double>(a0));
  if (!ck(cudaGetLastError(), "neighbour_zero launch")) return;
  t.done();
}

// src/airfoil.cpp:232-235, 324-327
void op_par_loop_calc_dt(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2) {
  if (!set) { fail("calc_dt: null set"); return; }
  const int N = order_from_np(a0.dim / 4);
  if (N < 0 || a0.dim % 4) { fail("calc_dt: q dim must be 4*Np"); return; }
  if (!arg_dat(a0, set, true, a0.dim, true, "calc_dt q") || !arg_dat(a1, set, true, 3 * (N + 1), true, "calc_dt fscale") ||
      !arg_gbl(a2, 1, true, "calc_dt dt1"))
    return;
  if (a2.acc != OP_MAX) { fail("calc_dt: the global must be OP_MAX"); return; }
  Consts C;
  if (!consts_for(N, false, C)) return;
  if (!S().d_red && !ck(cudaMalloc(&S().d_red, 8), "cudaMalloc")) return;
  Timed t(name ? name : "calc_dt");
  double seed;
  std::memcpy(&seed, a2.data, 8);
  unsigned long long seed_bits = seed > 0.0 ? (unsigned long long)__builtin_bit_cast(long long, seed) : 0ull;
  if (!ck(cudaMemcpyAsync(S().d_red, &seed_bits, 8, cudaMemcpyHostToDevice, S().stream), "cudaMemcpyAsync")) return;
  DISPATCH_N(N, (k_calc_dt<N><<<blocks(set->size, 128), 128, 0, S().stream>>>(
                    set->size, dptr<double>(a0), dptr<double>(a1), seed, (unsigned long long *)S().d_red, C)));
  if (!ck(cudaGetLastError(), "calc_dt launch")) return;
  unsigned long long bits = 0;
  if (!ck(cudaMemcpyAsync(&bits, S().d_red, 8, cudaMemcpyDeviceToHost, S().stream), "cudaMemcpyAsync")) return;
  if (!ck(cudaStreamSynchronize(S().stream), "calc_dt sync")) return;
  double out = seed > 0.0 ? seed : 0.0;
  if (bits) out = __builtin_bit_cast(double, bits);
  if (seed > out) out = seed;
  std::memcpy(a2.data, &out, 8);
  t.done();
}

// src/airfoil.cpp:256-265
void op_par_loop_get_neighbour_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                                 op_arg a3, op_arg a4, op_arg a5, op_arg a6, op_arg a7,
                                 op_arg a8) {
  if (!set) { fail("get_neighbour_q: null set"); return; }
  const int N = order_from_np(a5.dim / 4);
  if (N < 0 || a5.dim % 4) { fail("get_neighbour_q: workingQ dim must be 4*Np"); return; }
  const int Nfp = N + 1;
  if (!arg_dat(a0, set, true, 2, false, "get_neighbour_q edgeNum")) return;
  if (!arg_dat(a1, set, false, 3, true, "get_neighbour_q nodeX L") || !arg_dat(a2, set, false, 3, true, "get_neighbour_q nodeY L") ||
      !arg_dat(a3, set, false, 3, true, "get_neighbour_q nodeX R") || !arg_dat(a4, set, false, 3, true, "get_neighbour_q nodeY R") ||
      !arg_dat(a5, set, false, a5.dim, true, "get_neighbour_q q L") || !arg_dat(a6, set, false, a5.dim, true, "get_neighbour_q q R") ||
      !arg_dat(a7, set, false, 12 * Nfp, true, "get_neighbour_q ext L") || !arg_dat(a8, set, false, 12 * Nfp, true, "get_neighbour_q ext R"))
    return;
  const op_arg *all[8] = {&a1, &a2, &a3, &a4, &a5, &a6, &a7, &a8};
  for (auto *a : all)
    if (a->map != a1.map) return (void)fail("get_neighbour_q: all indirect args must use one map");
  if (a1.idx != a2.idx || a3.idx != a4.idx || a5.idx != a1.idx || a7.idx != a1.idx || a6.idx != a3.idx || a8.idx != a3.idx ||
      a1.dat != a3.dat || a2.dat != a4.dat || a5.dat != a6.dat || a7.dat != a8.dat)
    return (void)fail("get_neighbour_q: arguments do not follow src/airfoil.cpp:256-265");
  if (a7.acc != OP_INC || a8.acc != OP_INC) return (void)fail("get_neighbour_q: exteriorQ must be OP_INC");
  Consts C;
  if (!consts_for(N, false, C, kNone)) return;
  Timed t(name ? name : "get_neighbour_q");
  DISPATCH_N(N, (k_get_neighbour_q<N><<<blocks(set->size, 128), 128, 0, S().stream>>>(
                    set->size, dptr<int>(a0), a1.map->d_data, a1.map->dim, a1.idx, a3.idx, dptr<double>(a1),
                    dptr<double>(a2), dptr<double>(a5), dptr<double>(a7), C)));
  if (!ck(cudaGetLastError(), "get_neighbour_q launch")) return;
  t.done();
}

// src/airfoil.cpp:271-277
void op_par_loop_get_bedge_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                             op_arg a3, op_arg a4, op_arg a5) {
  if (!set) { fail("get_bedge_q: null set"); return; }
  const int N = order_from_np(a4.dim / 4);
  if (N < 0 || a4.dim % 4) { fail("get_bedge_q: workingQ dim must be 4*Np"); return; }
  const int Nfp = N + 1;
  if (!arg_dat(a0, set, true, 1, false, "get_bedge_q bedge_type") || !arg_dat(a1, set, true, 1, false, "get_bedge_q bedgeNum") ||
      !arg_dat(a2, set, false, 3 * Nfp, true, "get_bedge_q nx") || !arg_dat(a3, set, false, 3 * Nfp, true, "get_bedge_q ny") ||
      !arg_dat(a4, set, false, a4.dim, true, "get_bedge_q q") || !arg_dat(a5, set, false, 12 * Nfp, true, "get_bedge_q ext"))
    return;
  if (a2.map != a3.map || a2.map != a4.map || a2.map != a5.map || a2.idx != a3.idx || a2.idx != a4.idx || a2.idx != a5.idx)
    return (void)fail("get_bedge_q: indirect args must use one map column");
  if (a5.acc != OP_INC) return (void)fail("get_bedge_q: exteriorQ must be OP_INC");
  Consts C;
  if (!consts_for(N, false, C, kFreestream)) return;
  Timed t(name ? name : "get_bedge_q");
  DISPATCH_N(N, (k_get_bedge_q<N><<<blocks(set->size, 128), 128, 0, S().stream>>>(
                    set->size, dptr<int>(a0), dptr<int>(a1), a2.map->d_data, a2.map->dim, a2.idx, dptr<double>(a2),
                    dptr<double>(a3), dptr<double>(a4), dptr<double>(a5), C)));
  if (!ck(cudaGetLastError(), "get_bedge_q launch")) return;
  t.done();
}

// src/airfoil.cpp:283-293
void op_par_loop_euler_rhs(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                           op_arg a3, op_arg a4, op_arg a5, op_arg a6, op_arg a7, op_arg a8,
                           op_arg a9) {
  if (!set) { fail("euler_rhs: null set"); return; }
  const int N = order_from_np(a0.dim / 4);
  if (N < 0 || a0.dim % 4) { fail("euler_rhs: workingQ dim must be 4*Np"); return; }
  const int Np = a0.dim / 4, Nfp = N + 1;
  if (!arg_dat(a0, set, true, 4 * Np, true, "euler_rhs q") || !arg_dat(a1, set, true, 12 * Nfp, true, "euler_rhs exteriorQ") ||
      !arg_dat(a2, set, true, Np, true, "euler_rhs rx") || !arg_dat(a3, set, true, Np, true, "euler_rhs ry") ||
      !arg_dat(a4, set, true, Np, true, "euler_rhs sx") || !arg_dat(a5, set, true, Np, true, "euler_rhs sy") ||
      !arg_dat(a6, set, true, 3 * Nfp, true, "euler_rhs fscale") || !arg_dat(a7, set, true, 3 * Nfp, true, "euler_rhs nx") ||
      !arg_dat(a8, set, true, 3 * Nfp, true, "euler_rhs ny") || !arg_dat(a9, set, true, 4 * Np, true, "euler_rhs rk"))
    return;
  if (a9.dat == a0.dat) return (void)fail("euler_rhs: output aliases the input state");
  if (a1.acc != OP_RW && a1.acc != OP_READ) return (void)fail("euler_rhs: exteriorQ must be OP_RW or OP_READ");
  const bool zero_ext = a1.acc == OP_RW;  // src/airfoil.cpp:285 (OP_RW) vs vortex/src/vortex.cpp:268 (OP_READ)
  Consts C;
  if (!consts_for(N, true, C)) return;
  Timed t(name ? name : "euler_rhs");
  // tile of T cells per 128-thread block, T chosen so that the tile's fluxes fit in 48 KB
  const int per_cell = (12 * Np + 12 * Nfp) * 8;
  const int T = std::max(1, std::min(32, 49152 / per_cell));
  const size_t smem = (size_t)T * per_cell;
  DISPATCH_N(N, (k_euler_rhs<N><<<blocks(set->size, T), 128, smem, S().stream>>>(
                    set->size, T, dptr<double>(a0), dptr<double>(a1), dptr<double>(a2), dptr<double>(a3),
                    dptr<double>(a4), dptr<double>(a5), dptr<double>(a6), dptr<double>(a7), dptr<double>(a8),
                    dptr<double>(a9), C, zero_ext)));
  if (!ck(cudaGetLastError(), "euler_rhs launch")) return;
  t.done();
}

// src/airfoil.cpp:299-305
void op_par_loop_set_workingQ(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                              op_arg a3, op_arg a4, op_arg a5) {
  if (!set) { fail("set_workingQ: null set"); return; }
  const int dim = a2.dim;
  if (!arg_gbl(a0, 1, true, "set_workingQ dt") || !arg_gbl(a1, 1, false, "set_workingQ stage") ||
      !arg_dat(a2, set, true, dim, true, "set_workingQ q") || !arg_dat(a3, set, true, dim, true, "set_workingQ k1") ||
      !arg_dat(a4, set, true, dim, true, "set_workingQ k2") || !arg_dat(a5, set, true, dim, true, "set_workingQ W"))
    return;
  double dt;
  int stage;
  std::memcpy(&dt, a0.data, 8);
  std::memcpy(&stage, a1.data, 4);
  Timed t(name ? name : "set_workingQ");
  const long long n = (long long)set->size * dim;
  k_set_workingQ<<<blocks(n, 256), 256, 0, S().stream>>>(n, dt, stage, dptr<double>(a2), dptr<double>(a3),
                                                         dptr<double>(a4), dptr<double>(a5));
  if (!ck(cudaGetLastError(), "set_workingQ launch")) return;
  t.done();
}

// src/airfoil.cpp:311-317
void op_par_loop_update_Q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2,
                          op_arg a3, op_arg a4, op_arg a5) {
  if (!set) { fail("update_Q: null set"); return; }
  const int dim = a1.dim;
  if (!arg_gbl(a0, 1, true, "update_Q dt") || !arg_dat(a1, set, true, dim, true, "update_Q q") ||
      !arg_dat(a2, set, true, dim, true, "update_Q k1") || !arg_dat(a3, set, true, dim, true, "update_Q k2") ||
      !arg_dat(a4, set, true, dim, true, "update_Q k3") || !arg_dat(a5, set, true, dim, true, "update_Q W"))
    return;
  double dt;
  std::memcpy(&dt, a0.data, 8);
  Timed t(name ? name : "update_Q");
  const long long n = (long long)set->size * dim;
  k_update_Q<<<blocks(n, 256), 256, 0, S().stream>>>(n, dt, dptr<double>(a1), dptr<double>(a2), dptr<double>(a3),
                                                     dptr<double>(a4), dptr<double>(a5));
  if (!ck(cudaGetLastError(), "update_Q launch")) return;
  t.done();
}

// advec/src/advec.cpp:232-242
void op_par_loop_advec_rhs(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4,
                           op_arg a5, op_arg a6, op_arg a7, op_arg a8, op_arg a9) {
  if (!set) { fail("advec_rhs: null set"); return; }
  const int Np = a0.dim, N = order_from_np(Np);
  if (N < 0) { fail("advec_rhs: q dim is not a triangle node count of order 1..6"); return; }
  const int Nfp = N + 1;
  if (!arg_dat(a0, set, true, Np, true, "advec_rhs q") || !arg_dat(a1, set, true, 3 * Nfp, true, "advec_rhs exteriorQ") ||
      !arg_dat(a2, set, true, Np, true, "advec_rhs rx") || !arg_dat(a3, set, true, Np, true, "advec_rhs ry") ||
      !arg_dat(a4, set, true, Np, true, "advec_rhs sx") || !arg_dat(a5, set, true, Np, true, "advec_rhs sy") ||
      !arg_dat(a6, set, true, 3 * Nfp, true, "advec_rhs fscale") || !arg_dat(a7, set, true, 3 * Nfp, true, "advec_rhs nx") ||
      !arg_dat(a8, set, true, 3 * Nfp, true, "advec_rhs ny") || !arg_dat(a9, set, true, Np, true, "advec_rhs rk"))
    return;
  if (a9.dat == a0.dat) return (void)fail("advec_rhs: output aliases the input state");
  Consts C;
  if (!consts_for(N, true, C, kAdvec)) return;
  Timed t(name ? name : "advec_rhs");
  DISPATCH_N(N, (k_advec_rhs<N><<<blocks(set->size, 16), 128, 0, S().stream>>>(
                    set->size, dptr<double>(a0), dptr<double>(a1), dptr<double>(a2), dptr<double>(a3),
                    dptr<double>(a4), dptr<double>(a5), dptr<double>(a6), dptr<double>(a7), dptr<double>(a8),
                    dptr<double>(a9), C)));
  if (!ck(cudaGetLastError(), "advec_rhs launch")) return;
  t.done();
}

// vortex/src/vortex.cpp:308-318 (the per-cell error sums are added to the four globals, OP_INC)
void op_par_loop_l2_error(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4,
                          op_arg a5, op_arg a6, op_arg a7, op_arg a8) {
  if (!set) { fail("l2_error: null set"); return; }
  const int N = order_from_np(a0.dim);
  if (N < 0) { fail("l2_error: x dim is not a triangle node count of order 1..6"); return; }
  const int Np = a0.dim;
  if (!arg_dat(a0, set, true, Np, true, "l2_error x") || !arg_dat(a1, set, true, Np, true, "l2_error y") ||
      !arg_dat(a2, set, true, 4 * Np, true, "l2_error q") || !arg_gbl(a3, 1, true, "l2_error t") ||
      !arg_gbl(a4, 1, true, "l2_error rho") || !arg_gbl(a5, 1, true, "l2_error rhou") ||
      !arg_gbl(a6, 1, true, "l2_error rhov") || !arg_gbl(a7, 1, true, "l2_error ener") ||
      !arg_dat(a8, set, true, 4 * Np, true, "l2_error error"))
    return;
  if (a4.acc != OP_INC || a5.acc != OP_INC || a6.acc != OP_INC || a7.acc != OP_INC)
    return (void)fail("l2_error: the error sums must be OP_INC");
  Consts C;
  if (!consts_for(N, false, C, kVortex)) return;
  double t;
  std::memcpy(&t, a3.data, 8);
  double *part = nullptr;
  if (!ck(cudaMallocAsync((void **)&part, (size_t)set->size * 4 * 8 + 8, S().stream), "cudaMallocAsync")) return;
  Timed tm(name ? name : "l2_error");
  DISPATCH_N(N, (k_l2_error<N><<<blocks(set->size, 128), 128, 0, S().stream>>>(
                    set->size, dptr<double>(a0), dptr<double>(a1), dptr<double>(a2), t, part, dptr<double>(a8), C)));
  std::vector<double> h((size_t)set->size * 4);
  bool good = ck(cudaGetLastError(), "l2_error launch") &&
              ck(cudaMemcpyAsync(h.data(), part, h.size() * 8, cudaMemcpyDeviceToHost, S().stream), "cudaMemcpyAsync");
  cudaFreeAsync(part, S().stream);
  if (!good || !ck(cudaStreamSynchronize(S().stream), "l2_error sync")) return;
  double *out[4] = {(double *)a4.data, (double *)a5.data, (double *)a6.data, (double *)a7.data};
  for (int k = 0; k < 4; k++) {
    double acc = 0.0;
    for (int c = 0; c < set->size; c++) acc += h[4 * (size_t)c + k];
    *out[k] += acc;
  }
  tm.done();
}

void op2_gb300_par_loop(char const *kernel, char const *name, op_set set, int nargs, const op_arg *a) {
  if (!kernel || (nargs && !a)) { fail("op2_gb300_par_loop: bad arguments"); return; }
  const std::string k(kernel);
  auto need = [&](int n) {
    if (nargs == n) return true;
    return fail("op_par_loop_" + k + " takes " + std::to_string(n) + " arguments");
  };
  if (k == "init_grid") {
    if (need(18))
      op_par_loop_init_grid(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10], a[11],
                            a[12], a[13], a[14], a[15], a[16], a[17]);
  } else if (k == "set_ic") {
    if (nargs == 5) op_par_loop_set_ic(name, set, a[0], a[1], a[2], a[3], a[4]);
    else if (nargs == 4) op_par_loop_set_ic(name, set, a[0], a[1], a[2], a[3]);
    else if (need(2)) op_par_loop_set_ic(name, set, a[0], a[1]);
  } else if (k == "neighbour_zero") {
    if (need(1)) op_par_loop_neighbour_zero(name, set, a[0]);
  } else if (k == "calc_dt") {
    if (need(3)) op_par_loop_calc_dt(name, set, a[0], a[1], a[2]);
  } else if (k == "get_neighbour_q") {
    if (nargs == 11)
      op_par_loop_get_neighbour_q(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9], a[10]);
    else if (need(9)) op_par_loop_get_neighbour_q(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]);
  } else if (k == "get_bedge_q") {
    if (nargs == 9) op_par_loop_get_bedge_q(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]);
    else if (nargs == 8) op_par_loop_get_bedge_q(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7]);
    else if (need(6)) op_par_loop_get_bedge_q(name, set, a[0], a[1], a[2], a[3], a[4], a[5]);
  } else if (k == "l2_error") {
    if (need(9)) op_par_loop_l2_error(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]);
  } else if (k == "euler_rhs") {
    if (need(10)) op_par_loop_euler_rhs(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9]);
  } else if (k == "set_workingQ") {
    if (nargs == 5) op_par_loop_set_workingQ(name, set, a[0], a[1], a[2], a[3], a[4]);
    else if (need(6)) op_par_loop_set_workingQ(name, set, a[0], a[1], a[2], a[3], a[4], a[5]);
  } else if (k == "update_Q") {
    if (nargs == 7) op_par_loop_update_Q(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6]);
    else if (need(6)) op_par_loop_update_Q(name, set, a[0], a[1], a[2], a[3], a[4], a[5]);
  } else if (k == "advec_rhs") {
    if (need(10)) op_par_loop_advec_rhs(name, set, a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8], a[9]);
  } else {
    fail("unknown user kernel " + k);
  }
}

}  // extern "C"

// ------------------------------------------------------------------ vortex app loops
// vortex/src/vortex.cpp calls set_ic, get_neighbour_q and get_bedge_q with other argument lists
// than the airfoil app; a translated vortex driver binds these C++ overloads (the FFI reaches them
// through op2_gb300_par_loop by argument count).

// vortex/src/vortex.cpp:210-215: set_ic(t, x, y, q, workingQ)
void op_par_loop_set_ic(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4) {
  if (!set) { fail("set_ic: null set"); return; }
  const int Np = a1.dim, N = order_from_np(Np);
  if (N < 0) { fail("set_ic: x dim is not a triangle node count of order 1..6"); return; }
  if (!arg_gbl(a0, 1, true, "set_ic t") || !arg_dat(a1, set, true, Np, true, "set_ic x") ||
      !arg_dat(a2, set, true, Np, true, "set_ic y") || !arg_dat(a3, set, true, 4 * Np, true, "set_ic q") ||
      !arg_dat(a4, set, true, 4 * Np, true, "set_ic workingQ"))
    return;
  Consts C;
  if (!consts_for(N, false, C, kVortex)) return;
  double t;
  std::memcpy(&t, a0.data, 8);
  Timed tm(name ? name : "set_ic");
  const long long n = (long long)set->size * Np;
  k_set_ic_vortex<<<blocks(n, 256), 256, 0, S().stream>>>(n, t, dptr<double>(a1), dptr<double>(a2), dptr<double>(a3),
                                                         dptr<double>(a4), C);
  if (!ck(cudaGetLastError(), "set_ic launch")) return;
  tm.done();
}

// vortex/src/vortex.cpp:235-246: get_neighbour_q(edgeNum, n0, n1, nodeX L, nodeY L, nodeX R, nodeY R,
// W L, W R, exteriorQ L, exteriorQ R); the edge's two vertex coordinates are not used by the kernel.
void op_par_loop_get_neighbour_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3,
                                 op_arg a4, op_arg a5, op_arg a6, op_arg a7, op_arg a8, op_arg a9, op_arg a10) {
  if (!set) { fail("get_neighbour_q: null set"); return; }
  if (!arg_dat(a1, set, false, 2, true, "get_neighbour_q n0") || !arg_dat(a2, set, false, 2, true, "get_neighbour_q n1"))
    return;
  const int Nq = order_from_np(a7.dim);
  if (Nq < 0 || a9.dim != 3 * (Nq + 1)) {  // the vortex app's (4 variables per node)
    op_par_loop_get_neighbour_q(name, set, a0, a3, a4, a5, a6, a7, a8, a9, a10);
    return;
  }
  // the advection app's (advec/src/advec.cpp:207-218): one value per node
  const int N = Nq, Np = a7.dim, Nfp = N + 1;
  if (!arg_dat(a0, set, true, 2, false, "get_neighbour_q edgeNum")) return;
  if (!arg_dat(a3, set, false, 3, true, "get_neighbour_q nodeX L") || !arg_dat(a4, set, false, 3, true, "get_neighbour_q nodeY L") ||
      !arg_dat(a5, set, false, 3, true, "get_neighbour_q nodeX R") || !arg_dat(a6, set, false, 3, true, "get_neighbour_q nodeY R") ||
      !arg_dat(a7, set, false, Np, true, "get_neighbour_q q L") || !arg_dat(a8, set, false, Np, true, "get_neighbour_q q R") ||
      !arg_dat(a9, set, false, 3 * Nfp, true, "get_neighbour_q ext L") || !arg_dat(a10, set, false, 3 * Nfp, true, "get_neighbour_q ext R"))
    return;
  const op_arg *all[8] = {&a3, &a4, &a5, &a6, &a7, &a8, &a9, &a10};
  for (auto *a : all)
    if (a->map != a3.map) return (void)fail("get_neighbour_q: all indirect args must use one map");
  if (a3.idx != a4.idx || a5.idx != a6.idx || a7.idx != a3.idx || a9.idx != a3.idx || a8.idx != a5.idx ||
      a10.idx != a5.idx || a3.dat != a5.dat || a4.dat != a6.dat || a7.dat != a8.dat || a9.dat != a10.dat)
    return (void)fail("get_neighbour_q: arguments do not follow advec/src/advec.cpp:207-218");
  if (a9.acc != OP_INC || a10.acc != OP_INC) return (void)fail("get_neighbour_q: exteriorQ must be OP_INC");
  Consts C;
  if (!consts_for(N, false, C, kNone)) return;
  Timed t(name ? name : "get_neighbour_q");
  DISPATCH_N(N, (k_adv_get_neighbour_q<N><<<blocks(set->size, 128), 128, 0, S().stream>>>(
                    set->size, dptr<int>(a0), a3.map->d_data, a3.map->dim, a3.idx, a5.idx, dptr<double>(a3),
                    dptr<double>(a4), dptr<double>(a7), dptr<double>(a9), C)));
  if (!ck(cudaGetLastError(), "get_neighbour_q launch")) return;
  t.done();
}

// advec/src/advec.cpp:191-195: set_ic(x, y, q, workingQ), one value per node
void op_par_loop_set_ic(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3) {
  if (!set) { fail("set_ic: null set"); return; }
  const int Np = a0.dim;
  if (order_from_np(Np) < 0) { fail("set_ic: x dim is not a triangle node count of order 1..6"); return; }
  if (!arg_dat(a0, set, true, Np, true, "set_ic x") || !arg_dat(a1, set, true, Np, true, "set_ic y") ||
      !arg_dat(a2, set, true, Np, true, "set_ic q") || !arg_dat(a3, set, true, Np, true, "set_ic workingQ"))
    return;
  Timed tm(name ? name : "set_ic");
  const long long n = (long long)set->size * Np;
  k_adv_set_ic<<<blocks(n, 256), 256, 0, S().stream>>>(n, dptr<double>(a0), dptr<double>(a1), dptr<double>(a2),
                                                       dptr<double>(a3));
  if (!ck(cudaGetLastError(), "set_ic launch")) return;
  tm.done();
}

// advec/src/advec.cpp:221-229: get_bedge_q(bedgeNum, n0, n1, nodeX, nodeY, x, y, exteriorQ)
void op_par_loop_get_bedge_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4,
                             op_arg a5, op_arg a6, op_arg a7) {
  if (!set) { fail("get_bedge_q: null set"); return; }
  const int Np = a5.dim, N = order_from_np(Np);
  if (N < 0) { fail("get_bedge_q: x dim is not a triangle node count of order 1..6"); return; }
  const int Nfp = N + 1;
  if (!arg_dat(a0, set, true, 1, false, "get_bedge_q bedgeNum") || !arg_dat(a1, set, false, 2, true, "get_bedge_q n0") ||
      !arg_dat(a2, set, false, 2, true, "get_bedge_q n1") || !arg_dat(a3, set, false, 3, true, "get_bedge_q nodeX") ||
      !arg_dat(a4, set, false, 3, true, "get_bedge_q nodeY") || !arg_dat(a5, set, false, Np, true, "get_bedge_q x") ||
      !arg_dat(a6, set, false, Np, true, "get_bedge_q y") || !arg_dat(a7, set, false, 3 * Nfp, true, "get_bedge_q ext"))
    return;
  if (a5.map != a7.map || a5.idx != a7.idx) return (void)fail("get_bedge_q: x and exteriorQ must use one map column");
  if (a7.acc != OP_INC) return (void)fail("get_bedge_q: exteriorQ must be OP_INC");
  Timed tm(name ? name : "get_bedge_q");
  DISPATCH_N(N, (k_adv_get_bedge_q<N><<<blocks(set->size, 128), 128, 0, S().stream>>>(
                    set->size, dptr<int>(a0), a7.map->d_data, a7.map->dim, a7.idx, dptr<double>(a7))));
  if (!ck(cudaGetLastError(), "get_bedge_q launch")) return;
  tm.done();
}

// advec/src/advec.cpp:245-250: set_workingQ(dt, q, rk, rk_frac, workingQ)
void op_par_loop_set_workingQ(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4) {
  if (!set) { fail("set_workingQ: null set"); return; }
  const int dim = a1.dim;
  if (!arg_gbl(a0, 1, true, "set_workingQ dt") || !arg_dat(a1, set, true, dim, true, "set_workingQ q") ||
      !arg_dat(a2, set, true, dim, true, "set_workingQ rk") || !arg_gbl(a3, 1, true, "set_workingQ rk_frac") ||
      !arg_dat(a4, set, true, dim, true, "set_workingQ W"))
    return;
  double dt, frac;
  std::memcpy(&dt, a0.data, 8);
  std::memcpy(&frac, a3.data, 8);
  Timed tm(name ? name : "set_workingQ");
  const long long n = (long long)set->size * dim;
  k_adv_set_workingQ<<<blocks(n, 256), 256, 0, S().stream>>>(n, dt, frac, dptr<double>(a1), dptr<double>(a2),
                                                             dptr<double>(a4));
  if (!ck(cudaGetLastError(), "set_workingQ launch")) return;
  tm.done();
}

// advec/src/advec.cpp:253-260: update_Q(dt, q, rk1, rk2, rk3, rk4, workingQ)
void op_par_loop_update_Q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4,
                          op_arg a5, op_arg a6) {
  if (!set) { fail("update_Q: null set"); return; }
  const int dim = a1.dim;
  if (!arg_gbl(a0, 1, true, "update_Q dt") || !arg_dat(a1, set, true, dim, true, "update_Q q") ||
      !arg_dat(a2, set, true, dim, true, "update_Q k1") || !arg_dat(a3, set, true, dim, true, "update_Q k2") ||
      !arg_dat(a4, set, true, dim, true, "update_Q k3") || !arg_dat(a5, set, true, dim, true, "update_Q k4") ||
      !arg_dat(a6, set, true, dim, true, "update_Q W"))
    return;
  double dt;
  std::memcpy(&dt, a0.data, 8);
  Timed tm(name ? name : "update_Q");
  const long long n = (long long)set->size * dim;
  k_adv_update_Q<<<blocks(n, 256), 256, 0, S().stream>>>(n, dt, dptr<double>(a1), dptr<double>(a2), dptr<double>(a3),
                                                         dptr<double>(a4), dptr<double>(a5), dptr<double>(a6));
  if (!ck(cudaGetLastError(), "update_Q launch")) return;
  tm.done();
}

// vortex/src/vortex.cpp:249-260: get_bedge_q(bedgeNum, n0, n1, nodeX, nodeY, x, y, t, exteriorQ)
void op_par_loop_get_bedge_q(char const *name, op_set set, op_arg a0, op_arg a1, op_arg a2, op_arg a3, op_arg a4,
                             op_arg a5, op_arg a6, op_arg a7, op_arg a8) {
  if (!set) { fail("get_bedge_q: null set"); return; }
  const int Np = a5.dim, N = order_from_np(Np);
  if (N < 0) { fail("get_bedge_q: x dim is not a triangle node count of order 1..6"); return; }
  const int Nfp = N + 1;
  if (!arg_dat(a0, set, true, 1, false, "get_bedge_q bedgeNum") || !arg_dat(a1, set, false, 2, true, "get_bedge_q n0") ||
      !arg_dat(a2, set, false, 2, true, "get_bedge_q n1") || !arg_dat(a3, set, false, 3, true, "get_bedge_q nodeX") ||
      !arg_dat(a4, set, false, 3, true, "get_bedge_q nodeY") || !arg_dat(a5, set, false, Np, true, "get_bedge_q x") ||
      !arg_dat(a6, set, false, Np, true, "get_bedge_q y") || !arg_gbl(a7, 1, true, "get_bedge_q t") ||
      !arg_dat(a8, set, false, 12 * Nfp, true, "get_bedge_q ext"))
    return;
  if (a5.map != a6.map || a5.map != a8.map || a5.idx != a6.idx || a5.idx != a8.idx)
    return (void)fail("get_bedge_q: x, y and exteriorQ must use one map column");
  if (a8.acc != OP_INC) return (void)fail("get_bedge_q: exteriorQ must be OP_INC");
  Consts C;
  if (!consts_for(N, false, C, kVortex)) return;
  double t;
  std::memcpy(&t, a7.data, 8);
  Timed tm(name ? name : "get_bedge_q");
  DISPATCH_N(N, (k_get_bedge_q_vortex<N><<<blocks(set->size, 128), 128, 0, S().stream>>>(
                    set->size, dptr<int>(a0), a5.map->d_data, a5.map->dim, a5.idx, dptr<double>(a5), dptr<double>(a6),
                    t, dptr<double>(a8), C)));
  if (!ck(cudaGetLastError(), "get_bedge_q launch")) return;
  tm.done();
}
