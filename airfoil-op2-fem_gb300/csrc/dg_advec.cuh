// Scalar advection app (advec/src/advec.cpp:171-262) on the device.  Included at the end of
// dg_solver.cu: it shares the per-order operators [Drw | Dsw | -LIFT/2] in constant memory, the
// reference-node coordinates, the affine geometry kernel and the edge records of the Euler path.
//
// One classical RK4 stage is two kernels:
//   advec_face_kernel  one thread per face node (boundary faces first): the Lax-Friedrichs flux
//                      n.(F- + F+)/2 + |v|(q- - q+)/2 of advec/src/advec_rhs.h:36-63 once per
//                      face node, with the trace of the neighbour (advec/src/get_neighbour_q.h)
//                      or the constant ghost value 4.5e-5 (advec/src/get_bedge_q.h), written
//                      into both cells' face slots scaled by each side's fscale (twice the flux:
//                      the 1/2 is in the operator's LIFT columns);
//   advec_elem_kernel  32 cells x Np node-warps (even/odd form by default, advec_elem_kernel_sym):
//                      rhs = cr Drw q + cs Dsw q - LIFT flux with
//                      cr = vx rx + vy ry, cs = vx sx + vy sy (F = vx q, G = vy q on affine
//                      cells; advec_rhs.h:11-34), then the RK4 combine: W = q + dt frac k for
//                      stages 0-2 (advec/src/set_workingQ.h) with frac {1/2, 1/2, 1}, and
//                      q += dt/6 (k1 + 2 k2 + 2 k3 + k4) in the last (advec/src/update_Q.h).
//                      k1 + 2 k2 + 2 k3 is accumulated in one array in the reference's order.
// Layout: q, W, acc [K][Np]; flux [K][3][Nfp].  dt is fixed; t is kept on the host.
#pragma once

#include "dg_advec.h"

namespace dg {

constexpr double kAdvecGhost = 4.5e-5;  // advec/src/get_bedge_q.h:10

template <int N>
__global__ void __launch_bounds__(256) advec_face_kernel(const AdvInst d) {
  constexpr int Np = np_of(N), Nfp = N + 1;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nbf = d.nB * Nfp;
  if (tid >= nbf + d.nE * Nfp) return;
  const double vx = d.vx, vy = d.vy, a = d.speed;
  if (tid >= nbf) {
    const int e = (tid - nbf) / Nfp, i = (tid - nbf) - e * Nfp;
    const int4 ed = __ldg(&d.edges[e]);
    const int cL = ed.x, cR = ed.y, fL = ed.z & 3, fR = (ed.z >> 2) & 3;
    const int iR = (ed.z >> 4) ? Nfp - 1 - i : i;
    const double qm = d.W[(size_t)cL * Np + __ldg(&d.fmask[fL * Nfp + i])];
    const double qp = d.W[(size_t)cR * Np + __ldg(&d.fmask[fR * Nfp + iR])];
    const double *gl = d.geo + (size_t)cL * 16 + 4 + 3 * fL;
    const double nx = __ldg(gl), ny = __ldg(gl + 1);
    const double f = nx * (vx * qm + vx * qp) + ny * (vy * qm + vy * qp) + a * (qm - qp);
    d.flux[((size_t)cL * 3 + fL) * Nfp + i] = __ldg(gl + 2) * f;
    d.flux[((size_t)cR * 3 + fR) * Nfp + iR] = -__ldg(d.geo + (size_t)cR * 16 + 6 + 3 * fR) * f;
  } else {
    const int b = tid / Nfp, i = tid - b * Nfp;
    const int4 bd = __ldg(&d.bedges[b]);
    const int c = bd.x, fc = bd.y;
    const double qm = d.W[(size_t)c * Np + __ldg(&d.fmask[fc * Nfp + i])], qp = kAdvecGhost;
    const double *g = d.geo + (size_t)c * 16 + 4 + 3 * fc;
    const double nx = __ldg(g), ny = __ldg(g + 1);
    const double f = nx * (vx * qm + vx * qp) + ny * (vy * qm + vy * qp) + a * (qm - qp);
    d.flux[((size_t)c * 3 + fc) * Nfp + i] = __ldg(g + 2) * f;
  }
}

// stage 0..3: RK4 stage; stage 4: rhs_out = L(W) only.
template <int N>
__global__ void __launch_bounds__(32 * np_of(N)) advec_elem_kernel(const AdvInst d, const int stage) {
  constexpr int Np = np_of(N), NF = 3 * (N + 1), NK = nk_of(N), LD = 33;
  __shared__ double X[(Np + NF) * LD];  // [k][cell]: the tile's W, then its face fluxes
  __shared__ double R[32 * Np];         // right-hand sides, [cell][node] as in HBM
  const int t = threadIdx.x;
  const int e0 = blockIdx.x * 32;
  const int nc = min(32, d.K - e0);
  const size_t base = (size_t)e0 * Np;
  // coalesced loads of the tile's contiguous W and flux ranges
  {
    const int el = t / Np, k = t - el * Np;
    X[k * LD + el] = el < nc ? d.W[base + t] : 0.0;
    for (int j = t; j < 32 * NF; j += 32 * Np) {
      const int ef = j / NF, f = j - ef * NF;
      X[(Np + f) * LD + ef] = ef < nc ? d.flux[(size_t)e0 * NF + j] : 0.0;
    }
  }
  __syncthreads();
  {
    const int lane = t & 31, i = t >> 5;
    double ar = 0.0, as = 0.0, al = 0.0;
#pragma unroll
    for (int k = 0; k < Np; k++) {
      const double x = X[k * LD + lane];
      ar = fma(opA<N>(i * NK + k), x, ar);
      as = fma(opA<N>(i * NK + Np + k), x, as);
    }
#pragma unroll
    for (int f = 0; f < NF; f++) al = fma(opA<N>(i * NK + 2 * Np + f), X[(Np + f) * LD + lane], al);
    double cr = 0.0, cs = 0.0;
    if (lane < nc) {
      const double *g = d.geo + (size_t)(e0 + lane) * 16;
      cr = d.vx * g[0] + d.vy * g[1];
      cs = d.vx * g[2] + d.vy * g[3];
    }
    R[lane * Np + i] = fma(cr, ar, fma(cs, as, al));
  }
  __syncthreads();
  const int el = t / Np;
  if (el >= nc) return;
  const size_t o = base + t;
  const double r = R[t];
  if (stage == 4) {
    d.rhs_out[o] = r;
    return;
  }
  const double q = d.q[o], dt = d.dt;
  // the reference's operation order: q + (dt * frac) * k and q + ((1/6) dt) (((k1 + 2 k2) + 2 k3) + k4)
  if (stage == 0) {
    d.acc[o] = r;
    d.W[o] = __dadd_rn(q, __dmul_rn(dt * 0.5, r));
  } else if (stage < 3) {
    d.acc[o] = __dadd_rn(d.acc[o], 2.0 * r);
    d.W[o] = __dadd_rn(q, __dmul_rn(stage == 1 ? dt * 0.5 : dt, r));
  } else {
    const double qn = __dadd_rn(q, __dmul_rn((1.0 / 6.0) * dt, __dadd_rn(d.acc[o], r)));
    d.q[o] = qn;
    d.W[o] = qn;
  }
}

// The element kernel in even/odd form (the reflection r <-> s splits [Drw | Dsw | -LIFT] into an
// even and an odd block; see elem_tile_sym in dg_solver.cu): the inputs [cr q; cs q; flux] are
// staged in the pair order of that split, added and subtracted pairwise, contracted with the
// even and odd blocks (about half the multiply-adds of the dense rows) and recombined.  Same
// right-hand side as advec_elem_kernel up to rounding; the RK4 combine is the same.
template <int N>
__global__ void __launch_bounds__(32 * np_of(N)) advec_elem_kernel_sym(const AdvInst d, const int stage) {
  constexpr int Np = np_of(N), NF = 3 * (N + 1), NK = nk_of(N), LD = 33;
  constexpr int NUe = Sym<N>::NUe, NUo = Sym<N>::NUo, NRe = Sym<N>::NRe;
  __shared__ double X[NK * LD];   // [slot][cell]
  __shared__ double Y[Np * LD];   // even / odd row results [row][cell]
  __shared__ double R[32 * Np];   // right-hand sides [cell][node]
  const int t = threadIdx.x;
  const int e0 = blockIdx.x * 32;
  const int nc = min(32, d.K - e0);
  const size_t base = (size_t)e0 * Np;
  {
    const int el = t / Np, k = t - el * Np;
    double cr = 0.0, cs = 0.0, w = 0.0;
    if (el < nc) {
      const double *g = d.geo + (size_t)(e0 + el) * 16;
      cr = d.vx * g[0] + d.vy * g[1];
      cs = d.vx * g[2] + d.vy * g[3];
      w = d.W[base + t];
    }
    X[c_pos[N][k] * LD + el] = cr * w;
    X[c_pos[N][Np + k] * LD + el] = cs * w;
    for (int j = t; j < 32 * NF; j += 32 * Np) {
      const int ef = j / NF, f = j - ef * NF;
      X[c_pos[N][2 * Np + f] * LD + ef] = ef < nc ? d.flux[(size_t)e0 * NF + j] : 0.0;
    }
  }
  __syncthreads();
  for (int j = t; j < NUo * 32; j += 32 * Np) {  // butterfly over the input pairs
    const int p = j >> 5, el = j & 31;
    const double a = X[p * LD + el], b = X[(NUe + p) * LD + el];
    X[p * LD + el] = a + b;
    X[(NUe + p) * LD + el] = a - b;
  }
  __syncthreads();
  const int lane = t & 31, i = t >> 5;
  {
    double acc = 0.0;
    if (i < NRe) {
#pragma unroll
      for (int k = 0; k < NUe; k++) acc = fma(opS<N>(i * NUe + k), X[k * LD + lane], acc);
    } else {
#pragma unroll
      for (int k = 0; k < NUo; k++) acc = fma(opS<N>(NRe * NUe + (i - NRe) * NUo + k), X[(NUe + k) * LD + lane], acc);
    }
    Y[i * LD + lane] = acc;
  }
  __syncthreads();
  {
    const int re = c_out[N][3 * i], ro = c_out[N][3 * i + 1], sg = c_out[N][3 * i + 2];
    double r = Y[re * LD + lane];
    if (ro >= 0) r = sg > 0 ? r + Y[ro * LD + lane] : r - Y[ro * LD + lane];
    R[lane * Np + i] = r;
  }
  __syncthreads();
  const int el = t / Np;
  if (el >= nc) return;
  const size_t o = base + t;
  const double r = R[t];
  if (stage == 4) {
    d.rhs_out[o] = r;
    return;
  }
  const double q = d.q[o], dt = d.dt;
  if (stage == 0) {
    d.acc[o] = r;
    d.W[o] = __dadd_rn(q, __dmul_rn(dt * 0.5, r));
  } else if (stage < 3) {
    d.acc[o] = __dadd_rn(d.acc[o], 2.0 * r);
    d.W[o] = __dadd_rn(q, __dmul_rn(stage == 1 ? dt * 0.5 : dt, r));
  } else {
    const double qn = __dadd_rn(q, __dmul_rn((1.0 / 6.0) * dt, __dadd_rn(d.acc[o], r)));
    d.q[o] = qn;
    d.W[o] = qn;
  }
}

// The element kernel with the even/odd contraction on the tensor cores (the exact integer
// product of dg_ozaki.cuh): one variable per column, so a 32-cell tile is two row tiles of 16
// cells and the units are (row tile, n-tile of outputs).  Staging, butterfly and alignment
// (oz_prep over 64 threads), the contraction, the recombination and the RK4 combine follow
// advec_elem_kernel_sym; the right-hand side equals it to rounding.  Used at N = 3 (K = 524288:
// 0.304 -> 0.254 ms per stage, step 1.45 -> 1.20 ms); at N = 4, 5 a tile has only 6 or 8
// contraction units for 15 or 21 warps and measured slower than the FP64 kernel (0.562 vs 0.537,
// 0.931 vs 0.885 ms per stage), so those orders keep it.
constexpr bool advec_tc(int N) { return N == 3; }
template <int N>
__global__ void __launch_bounds__(32 * np_of(N), oz_min_blocks(N)) advec_elem_kernel_tc(const AdvInst d,
                                                                                         const int stage) {
  constexpr int Np = np_of(N), NF = 3 * (N + 1), NK = nk_of(N);
  constexpr int NUe = Sym<N>::NUe, NUo = Sym<N>::NUo, NRe = Sym<N>::NRe, NRo = Sym<N>::NRo;
  // 32 cells + 4 doubles of padding per slot: the fragment loads' four k-rows fall on different banks
  constexpr int XS = 36;
  constexpr int NTT = (NRe + 7) / 8 + (NRo + 7) / 8;  // n-tiles of outputs
  __shared__ __align__(16) double X[NK * XS];  // [slot][cell]
  __shared__ __align__(16) double Y[Np * XS];  // even / odd row results [row][cell]
  __shared__ double R[32 * Np];                // right-hand sides [cell][node]
  __shared__ int Ems[32];                      // column exponents of the prepared operands
  const int t = threadIdx.x;
  const int e0 = blockIdx.x * 32;
  const int nc = min(32, d.K - e0);
  const size_t base = (size_t)e0 * Np;
  {
    const int el = t / Np, k = t - el * Np;
    double cr = 0.0, cs = 0.0, w = 0.0;
    if (el < nc) {
      const double *g = d.geo + (size_t)(e0 + el) * 16;
      cr = d.vx * g[0] + d.vy * g[1];
      cs = d.vx * g[2] + d.vy * g[3];
      w = d.W[base + t];
    }
    X[c_pos[N][k] * XS + el] = cr * w;
    X[c_pos[N][Np + k] * XS + el] = cs * w;
    for (int j = t; j < 32 * NF; j += 32 * Np) {
      const int ef = j / NF, f = j - ef * NF;
      X[c_pos[N][2 * Np + f] * XS + ef] = ef < nc ? d.flux[(size_t)e0 * NF + j] : 0.0;
    }
  }
  __syncthreads();
  oz_prep<NUe, NUo, XS, 32>(X, Ems, t);
  __syncthreads();
  const int lane = t & 31, i = t >> 5;
  // unit u: n-tile u >> 1 of the outputs (even rows first), cells 16 (u & 1) .. + 15
  for (int u = i; u < 2 * NTT; u += Np)
    oz_unit<N, 0, NUe, NRe, NUo, NRo, NUe, NRe, 0, true, XS>(X, Y, u >> 1, (u & 1) * 4, lane, Ems);
  __syncthreads();
  {
    const int re = c_out[N][3 * i], ro = c_out[N][3 * i + 1], sg = c_out[N][3 * i + 2];
    double r = Y[re * XS + lane];
    if (ro >= 0) r = sg > 0 ? r + Y[ro * XS + lane] : r - Y[ro * XS + lane];
    R[lane * Np + i] = r;
  }
  __syncthreads();
  const int el = t / Np;
  if (el >= nc) return;
  const size_t o = base + t;
  const double r = R[t];
  if (stage == 4) {
    d.rhs_out[o] = r;
    return;
  }
  const double q = d.q[o], dt = d.dt;
  if (stage == 0) {
    d.acc[o] = r;
    d.W[o] = __dadd_rn(q, __dmul_rn(dt * 0.5, r));
  } else if (stage < 3) {
    d.acc[o] = __dadd_rn(d.acc[o], 2.0 * r);
    d.W[o] = __dadd_rn(q, __dmul_rn(stage == 1 ? dt * 0.5 : dt, r));
  } else {
    const double qn = __dadd_rn(q, __dmul_rn((1.0 / 6.0) * dt, __dadd_rn(d.acc[o], r)));
    d.q[o] = qn;
    d.W[o] = qn;
  }
}

// advec/src/set_ic.h:3-10 at the node positions of src/init_grid.h.
template <int N>
__global__ void advec_ic_kernel(const AdvInst d, const double *coords, const int *cells) {
  constexpr int Np = np_of(N);
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= (long long)d.K * Np) return;
  const int c = (int)(tid / Np), i = (int)(tid - (long long)c * Np);
  const int a = cells[3 * c], b = cells[3 * c + 1], e = cells[3 * c + 2];
  const double r = c_rs[N][i], s = c_rs[N][Np + i];
  const double x = node_coord(coords[2 * a], coords[2 * b], coords[2 * e], r, s);
  const double y = node_coord(coords[2 * a + 1], coords[2 * b + 1], coords[2 * e + 1], r, s);
  const double dx = __dsub_rn(x, 0.5), dy = __dsub_rn(y, 0.5);
  const double q = __dmul_rn(exp(__dmul_rn(__dmul_rn(-40.0, dx), dx)), exp(__dmul_rn(__dmul_rn(-40.0, dy), dy)));
  d.q[tid] = q;
  d.W[tid] = q;
}

// advec/src/save_solution.cpp:13-52: q at local nodes 0, N, Np-1 of the winning cell.
template <int N>
__global__ void advec_vertex_kernel(int K, const int *cells, const int *owner, const double *q, double *out) {
  constexpr int Np = np_of(N);
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= K) return;
  const int local[3] = {0, N, Np - 1};
  for (int k = 0; k < 3; k++) {
    const int node = cells[3 * c + k];
    if (owner[node] == c) out[node] = q[(size_t)c * Np + local[k]];
  }
}

// Element-kernel forms 2 and 3 use the tensor-core contraction where advec_tc says, form 1 (and
// forms 2, 3 at the other orders) the even/odd FP64 kernel, form 0 the dense FP64 kernel.
template <int N>
static void advec_launch_elem(const AdvInst &d, int stage, cudaStream_t s) {
  if constexpr (advec_tc(N)) {
    if (g_elem_variant >= 2) {
      advec_elem_kernel_tc<N><<<(d.K + 31) / 32, 32 * np_of(N), 0, s>>>(d, stage);
      return;
    }
  }
  if (g_elem_variant) advec_elem_kernel_sym<N><<<(d.K + 31) / 32, 32 * np_of(N), 0, s>>>(d, stage);
  else advec_elem_kernel<N><<<(d.K + 31) / 32, 32 * np_of(N), 0, s>>>(d, stage);
}

template <int N>
static void advec_launch_stage(const AdvInst &d, int stage, cudaStream_t s) {
  const int nf = (d.nE + d.nB) * (N + 1);
  if (nf) advec_face_kernel<N><<<(nf + 255) / 256, 256, 0, s>>>(d);
  advec_launch_elem<N>(d, stage, s);
}

Advection::~Advection() {
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  if (graph) cudaGraphDestroy(graph);
  for (void *p : allocs) cudaFree(p);
  if (stream) cudaStreamDestroy(stream);
}

int Advection::create(const Mesh &m, int order, double vel_x, double vel_y, double dt, std::string &err) {
  if (int rc = validate(m, err)) return rc;
  if (int rc = load_order_constants(order, err)) return rc;
  if (!(dt > 0.0) || !std::isfinite(dt) || !std::isfinite(vel_x) || !std::isfinite(vel_y)) {
    err = "dt must be positive and the velocity finite";
    return -4;
  }
  CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  N = order;
  K = m.n_cells();
  const int Np = np_of(N), Nfp = N + 1;
  Operators o;
  build_operators(N, o);
  d = AdvInst();
  d.N = N;
  d.K = K;
  d.nE = m.n_edges();
  d.nB = m.n_bedges();
  d.vx = vel_x;
  d.vy = vel_y;
  d.speed = std::sqrt(vel_x * vel_x + vel_y * vel_y);  // advec/src/advec_rhs.h:57
  d.dt = dt;
  std::vector<int4> edges, bedges;
  edge_records(m, edges, bedges);
  auto alloc = [&](size_t bytes) {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return (void *)nullptr;
    allocs.push_back(p);
    return p;
  };
  const size_t nq = (size_t)K * Np;
  d.q = (double *)alloc(nq * 8);
  d.W = (double *)alloc(nq * 8);
  d.acc = (double *)alloc(nq * 8);
  d.flux = (double *)alloc((size_t)K * 3 * Nfp * 8);
  double *geo = (double *)alloc((size_t)K * 16 * 8);
  d.geo = geo;
  int4 *de = (int4 *)alloc(sizeof(int4) * d.nE), *db = (int4 *)alloc(sizeof(int4) * d.nB);
  d.edges = de;
  d.bedges = db;
  int *fm = (int *)alloc(sizeof(int) * 3 * Nfp);
  d.fmask = fm;
  coords_d = (double *)alloc(m.coords.size() * 8);
  cells_d = (int *)alloc(m.cell2nodes.size() * 4);
  for (void *p : {(void *)d.q, (void *)d.W, (void *)d.acc, (void *)d.flux, (void *)geo, (void *)de, (void *)db,
                  (void *)fm, (void *)coords_d, (void *)cells_d})
    if (!p) { err = "cudaMalloc failed"; return -101; }
  CK(cudaMemcpyAsync(de, edges.data(), sizeof(int4) * d.nE, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(db, bedges.data(), sizeof(int4) * d.nB, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(fm, o.FMASK.data(), sizeof(int) * 3 * Nfp, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(coords_d, m.coords.data(), m.coords.size() * 8, cudaMemcpyHostToDevice, stream));
  CK(cudaMemcpyAsync(cells_d, m.cell2nodes.data(), m.cell2nodes.size() * 4, cudaMemcpyHostToDevice, stream));
  CK(cudaMemsetAsync(d.flux, 0, (size_t)K * 3 * Nfp * 8, stream));
  CK(cudaMemsetAsync(d.acc, 0, nq * 8, stream));
  geometry_kernel<<<(K + 127) / 128, 128, 0, stream>>>(K, coords_d, cells_d, geo);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(stream));
  return 0;
}

int Advection::init(std::string &err) {
  const long long n = (long long)K * np_of(N);
  DG_DISPATCH(N, (advec_ic_kernel<NN><<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(d, coords_d, cells_d)));
  CK(cudaGetLastError());
  t = 0.0;
  steps = 0;
  return 0;
}

void Advection::enqueue_step(cudaStream_t s) {
  DG_DISPATCH(N, (advec_launch_stage<NN>(d, 0, s), advec_launch_stage<NN>(d, 1, s),
                  advec_launch_stage<NN>(d, 2, s), advec_launch_stage<NN>(d, 3, s)));
}

void Advection::enqueue_step_events(cudaStream_t s, cudaEvent_t *ev) {
  const int nf = (d.nE + d.nB) * (N + 1);
  for (int stage = 0; stage < 4; stage++) {
    DG_DISPATCH(N, (advec_face_kernel<NN><<<(nf + 255) / 256, 256, 0, s>>>(d)));
    cudaEventRecord(ev[1 + 2 * stage], s);
    DG_DISPATCH(N, advec_launch_elem<NN>(d, stage, s));
    cudaEventRecord(ev[2 + 2 * stage], s);
  }
}

int Advection::step(int nsteps, bool use_graph, std::string &err) {
  if (use_graph && !graph_exec) {
    CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step(stream);
    cudaError_t ce = cudaStreamEndCapture(stream, &graph);
    if (ce != cudaSuccess) { err = std::string("graph capture: ") + cudaGetErrorString(ce); return -6; }
    CK(cudaGraphInstantiate(&graph_exec, graph, 0));
  }
  for (int i = 0; i < nsteps; i++) {
    if (use_graph) CK(cudaGraphLaunch(graph_exec, stream));
    else enqueue_step(stream);
    t += d.dt;  // advec/src/advec.cpp:262
    steps++;
  }
  CK(cudaGetLastError());
  return 0;
}

int Advection::rhs(double *out_dev, std::string &err) {
  AdvInst r = d;
  r.rhs_out = out_dev;
  DG_DISPATCH(N, (advec_launch_stage<NN>(r, 4, stream)));
  CK(cudaGetLastError());
  return 0;
}

int Advection::vertex_values(int n_nodes, double *out_host, std::string &err) {
  int *owner = nullptr;
  double *buf = nullptr;
  CK(cudaMallocAsync((void **)&owner, (size_t)n_nodes * 4, stream));
  CK(cudaMallocAsync((void **)&buf, (size_t)n_nodes * 8, stream));
  CK(cudaMemsetAsync(owner, 0xff, (size_t)n_nodes * 4, stream));
  CK(cudaMemsetAsync(buf, 0, (size_t)n_nodes * 8, stream));
  vertex_owner_kernel<<<(K + 127) / 128, 128, 0, stream>>>(K, cells_d, owner);
  DG_DISPATCH(N, (advec_vertex_kernel<NN><<<(K + 127) / 128, 128, 0, stream>>>(K, cells_d, owner, d.q, buf)));
  CK(cudaMemcpyAsync(out_host, buf, (size_t)n_nodes * 8, cudaMemcpyDeviceToHost, stream));
  CK(cudaFreeAsync(owner, stream));
  CK(cudaFreeAsync(buf, stream));
  CK(cudaStreamSynchronize(stream));
  return 0;
}

}  // namespace dg
