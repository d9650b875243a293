// Warp-specialised persistent element kernel of the plain path (included by dg_solver.cu inside
// namespace dg, after the element kernels it shares its device functions with).
//
// In the one-tile-per-block element kernel every block runs the same phases in the same order
// (loads, FP64 nodal fluxes, the integer operand pre-pass, the tensor-core contraction and its
// integer rounding, the FP64 stage combine), and the blocks of a wave start together: the FP64
// pipe idles while they are all in the integer phases and is oversubscribed when they are all in
// the FP64 ones.  Here one block per SM walks a contiguous range of 32-cell tiles with two groups
// of warps working on different tiles at the same time:
//   node warps (Np warps, one thread per cell lane and node, as in elem_tile_sym): the tile's
//     loads and nodal fluxes into a staging buffer ("fill"), and later the same tile's
//     recombination and stage combine ("combine");
//   contraction warps (8 warps, 256 threads): the operand pre-pass and the contraction of a filled
//     buffer into its output rows.
// The staging (X, Y, column exponents, staged W and q) is triple-buffered.  In their step j the
// node warps load tile j+1's W and metrics into registers, compute tile j's nodal fluxes (its face
// fluxes and q were copied in during step j-1), start the asynchronous copies of tile j+1's face
// fluxes and q, and combine tile j-1, while the contraction warps work on the tile filled last: the
// node warps' loads are in flight while they compute.  The two groups
// hand buffers over through mbarriers (full / empty per buffer); every wait is bounded (about
// 2^28 SM clocks), after which the thread records an error bit in the step state and goes on, so
// the kernel always ends.  The arithmetic of every tile is that of elem_tile_sym in its
// tensor-core form (same functions, same operation order): the results are bitwise the same.
#pragma once

constexpr int kWsCtrWarps = 8;  // contraction warps: oz_prep's 256 threads, 2 or 3 units each
constexpr long long kWsWaitLimit = 1ll << 28;

// Orders with a warp-specialised kernel: the even/odd blocks on the tensor cores at N = 3 (three
// buffers of 64 KB; at N = 4 three buffers would exceed the 227 KB of shared memory, and with two
// the node warps cannot load ahead: measured no faster than one block per tile there).
constexpr bool ws_used(int N) { return N == 3; }
constexpr int kWsBufs = 3;
constexpr int ws_threads(int N) { return 32 * (np_of(N) + kWsCtrWarps); }
// one staging buffer: X (NK slots), Y (Np rows), 128 column exponents, W and q of every node
constexpr size_t ws_buf_bytes(int N) {
  return (size_t)(nk_of(N) + np_of(N)) * kElemSlot * sizeof(double) + 128 * sizeof(int) +
         (size_t)4 * 32 * np_of(N) * sizeof(double2);
}
constexpr int kWsBars = 16;
constexpr size_t ws_smem(int N) { return kWsBufs * ws_buf_bytes(N) + kWsBars * sizeof(unsigned long long); }

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile(
      "{\n\t.reg .b64 st;\n\t"
      "mbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
      : "memory");
}

// Waits until the barrier's phase of the given parity has completed, at most `limit` SM clocks;
// false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, long long limit) {
  const unsigned a = smem_u32(bar);
  const long long t0 = clock64();
  while (true) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > limit) return false;
  }
}

// Error bit 2 of the step state: a wait of the warp-specialised element kernel gave up.
__device__ __forceinline__ void ws_fail(const Inst &d) {
  if (d.st) atomicOr(&d.st->err, 4u);
}

// The copies of a tile's face fluxes (into their slots) and, in stages 1 and 2, of q (into the
// staged W / q area), as one cp.async group of this thread.
template <int N>
__device__ __forceinline__ void ws_issue(const Inst &d, const int stage, const int e0, const int lane, const int i,
                                         double2 *X, double2 *WQ) {
  constexpr int Np = np_of(N), Nfp = N + 1;
  constexpr int kS2 = kElemSlot / 2;
  constexpr int nthr = 32 * Np;
  const int tid = i * 32 + lane;
  const int e = e0 + lane;
  if ((stage == 1 || stage == 2) && e < d.K) {
    const double *qp = d.q + ((size_t)e * Np + i) * 4;
    cp_async16(WQ + 2 * nthr + tid, qp, true);
    cp_async16(WQ + 3 * nthr + tid, qp + 2, true);
  }
  for (int j = tid; j < 3 * Nfp * 32; j += nthr) {
    const int f = j >> 5, el = j & 31;
    const bool ok = e0 + el < d.K;
    const double *fp = d.flux + (((size_t)(ok ? e0 + el : 0)) * 3 * Nfp + f) * 4;
    const int pf = c_pos[N][2 * Np + f];
    cp_async16(X + pf * kS2 + el * 2, fp, ok);
    cp_async16(X + pf * kS2 + el * 2 + 1, fp + 2, ok);
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}

// This node's W and the cell's metrics, into registers (loaded a tile ahead of their use).
template <int N>
__device__ __forceinline__ void ws_load(const Inst &d, const int e0, const int lane, const int i, double2 w[2],
                                        double2 g[2]) {
  constexpr int Np = np_of(N);
  const int e = e0 + lane;
  if (e < d.K) {
    const double *wp = d.W + ((size_t)e * Np + i) * 4;
    w[0] = ld2(wp);
    w[1] = ld2(wp + 2);
    g[0] = ld2(d.geo + (size_t)e * 16);
    g[1] = ld2(d.geo + (size_t)e * 16 + 2);
  } else {
    w[0] = w[1] = g[0] = g[1] = make_double2(0.0, 0.0);
  }
}

// The nodal fluxes into the slots and W into the staged area (the first part of elem_tile_sym in
// its tensor-core form), then the wait for this thread's copies of the tile.
template <int N>
__device__ __forceinline__ void ws_compute(const Inst &d, const int e0, const int lane, const int i,
                                           const double2 wv[2], const double2 gv[2], double2 *X, double2 *WQ) {
  constexpr int Np = np_of(N);
  constexpr int kS2 = kElemSlot / 2;
  constexpr int nthr = 32 * Np;
  const int tid = i * 32 + lane;
  const bool live = e0 + lane < d.K;
  const Phys &P = d.P;
  const double w[4] = {wv[0].x, wv[0].y, wv[1].x, wv[1].y};
  if (live) {
    WQ[tid] = wv[0];
    WQ[nthr + tid] = wv[1];
  }
  const double rx = gv[0].x, ry = gv[0].y, sx = gv[1].x, sy = gv[1].y;
  double fr0 = 0, fr1 = 0, fr2 = 0, fr3 = 0, fs0 = 0, fs1 = 0, fs2 = 0, fs3 = 0;
  if (live) {
    const double ir = rcp(w[0]);
    const double u = w[1] * ir, v = w[2] * ir;
    const double p = P.gm1 * fma(-0.5, fma(w[1], u, w[2] * v), w[3]);
    const double ep = w[3] + p;
    const double U = fma(rx, u, ry * v), V = fma(sx, u, sy * v);
    fr0 = w[0] * U;
    fr1 = fma(w[1], U, rx * p);
    fr2 = fma(w[2], U, ry * p);
    fr3 = U * ep;
    fs0 = w[0] * V;
    fs1 = fma(w[1], V, sx * p);
    fs2 = fma(w[2], V, sy * p);
    fs3 = V * ep;
  }
  const int pr = c_pos[N][i], ps = c_pos[N][Np + i];
  X[pr * kS2 + lane * 2] = make_double2(fr0, fr1);
  X[pr * kS2 + lane * 2 + 1] = make_double2(fr2, fr3);
  X[ps * kS2 + lane * 2] = make_double2(fs0, fs1);
  X[ps * kS2 + lane * 2 + 1] = make_double2(fs2, fs3);
  cp_async_wait_all();
}

// Combine: the node's right-hand side from the even and odd output rows, then the stage combine
// with the staged W and q (the last part of elem_tile_sym).  Arrives on yempty once Y is read.
template <int N>
__device__ __forceinline__ void ws_combine(const Inst &d, const int stage, const int e0, const int lane, const int i,
                                           const double2 *Y, double2 *WQ, unsigned long long *yempty) {
  constexpr int Np = np_of(N);
  constexpr int kS2 = kElemSlot / 2;
  constexpr int nthr = 32 * Np;
  const int tid = i * 32 + lane;
  const int e = e0 + lane;
  const bool live = e < d.K;
  const int re = c_out[N][3 * i], ro = c_out[N][3 * i + 1], sg = c_out[N][3 * i + 2];
  const double2 e01 = Y[re * kS2 + lane * 2], e23 = Y[re * kS2 + lane * 2 + 1];
  double r0 = e01.x, r1 = e01.y, r2 = e23.x, r3 = e23.y;
  if (ro >= 0) {
    const double2 o01 = Y[ro * kS2 + lane * 2], o23 = Y[ro * kS2 + lane * 2 + 1];
    if (sg > 0) {
      r0 += o01.x; r1 += o01.y; r2 += o23.x; r3 += o23.y;
    } else {
      r0 -= o01.x; r1 -= o01.y; r2 -= o23.x; r3 -= o23.y;
    }
  }
  mbar_arrive(yempty);
  double w[4] = {0.0, 0.0, 0.0, 0.0};
  if (live) {
    const double2 a = WQ[tid], b = WQ[nthr + tid];
    w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
  }
  stage_combine<N>(d, stage, e, true, live, i, lane, w, r0, r1, r2, r3,
                   (stage == 1 || stage == 2) ? WQ + 2 * nthr + tid : nullptr, nthr);
}

// Tiles [t0, t1) of one stage over the grid's blocks, each block a contiguous range of tiles.
// PW: launched with programmatic dependence on the face kernel (the node warps wait for it
// before their first copy of face fluxes).
template <int N, bool PW>
__global__ void __launch_bounds__(ws_threads(N), 1) elem_kernel_ws(const Inst d, const int stage, const int t0,
                                                                    const int t1) {
  constexpr int Np = np_of(N), NK = nk_of(N);
  constexpr int NUe = Sym<N>::NUe, NUo = Sym<N>::NUo, NRe = Sym<N>::NRe, NRo = Sym<N>::NRo;
  constexpr int kS2 = kElemSlot / 2;
  constexpr int B = kWsBufs;
  constexpr unsigned NN = 32 * Np, NC = 32 * kWsCtrWarps;
  extern __shared__ __align__(16) unsigned char ws_sm[];
  double2 *X[B], *Y[B], *WQ[B];
  int *Ems[B];
  for (int b = 0; b < B; b++) {
    X[b] = reinterpret_cast<double2 *>(ws_sm + b * ws_buf_bytes(N));
    Y[b] = X[b] + NK * kS2;
    Ems[b] = reinterpret_cast<int *>(Y[b] + Np * kS2);
    WQ[b] = reinterpret_cast<double2 *>(Ems[b] + 128);
  }
  // per buffer b: X full (b), X empty (B + b), Y full (2B + b), Y empty (3B + b); then the
  // contraction warps' pre-pass barrier (4B)
  unsigned long long *bars = reinterpret_cast<unsigned long long *>(ws_sm + B * ws_buf_bytes(N));
  unsigned long long *xfull = bars, *xempty = bars + B, *yfull = bars + 2 * B, *yempty = bars + 3 * B;
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int b = 0; b < B; b++) {
      mbar_init(&xfull[b], NN);
      mbar_init(&xempty[b], NC);
      mbar_init(&yfull[b], NC);
      mbar_init(&yempty[b], NN);
    }
    mbar_init(&bars[4 * B], NC);
  }
  __syncthreads();
  pdl_trigger();
  const int nt = t1 - t0, G = (int)gridDim.x;
  const int tb = t0 + (int)((long long)nt * blockIdx.x / G);
  const int n = t0 + (int)((long long)nt * (blockIdx.x + 1) / G) - tb;
  if (tid < (int)NN) {
    const int i = tid >> 5, lane = tid & 31;
    // tile j uses buffer j % B for the (j / B)-th time; before its copies start, the contraction of
    // the buffer's previous tile (j - B) must be done with X
    auto issue = [&](int j) {
      const int b = j % B, k = j / B;
      if (k >= 1 && !mbar_wait(&xempty[b], (unsigned)(k - 1) & 1u, kWsWaitLimit)) ws_fail(d);
      ws_issue<N>(d, stage, (tb + j) * 32, lane, i, X[b], WQ[b]);
    };
    double2 wc[2], gc[2], wn[2], gn[2];
    wn[0] = wn[1] = gn[0] = gn[1] = make_double2(0.0, 0.0);
    if (n > 0) ws_load<N>(d, tb * 32, lane, i, wc, gc);
    if constexpr (PW) pdl_wait();
    if (n > 0) issue(0);
    for (int j = 0; j <= n; j++) {
      if (j < n) {
        const int b = j % B;
        if (j + 1 < n) ws_load<N>(d, (tb + j + 1) * 32, lane, i, wn, gn);
        ws_compute<N>(d, (tb + j) * 32, lane, i, wc, gc, X[b], WQ[b]);
        mbar_arrive(&xfull[b]);
        if (j + 1 < n) issue(j + 1);
      }
      if (j >= 1) {
        const int jj = j - 1, b = jj % B, k = jj / B;
        if (!mbar_wait(&yfull[b], (unsigned)k & 1u, kWsWaitLimit)) ws_fail(d);
        ws_combine<N>(d, stage, (tb + jj) * 32, lane, i, Y[b], WQ[b], &yempty[b]);
      }
      wc[0] = wn[0]; wc[1] = wn[1]; gc[0] = gn[0]; gc[1] = gn[1];
    }
  } else {
    const int ct = tid - (int)NN, cw = ct >> 5, lane = ct & 31;
    for (int j = 0; j < n; j++) {
      const int b = j % B, k = j / B;
      if (!mbar_wait(&xfull[b], (unsigned)k & 1u, kWsWaitLimit)) ws_fail(d);
      oz_prep<NUe, NUo, kElemSlot>(reinterpret_cast<double *>(X[b]), Ems[b], ct);
      mbar_arrive(&bars[4 * B]);
      if (!mbar_wait(&bars[4 * B], (unsigned)j & 1u, kWsWaitLimit)) ws_fail(d);
      if (k >= 1 && !mbar_wait(&yempty[b], (unsigned)(k - 1) & 1u, kWsWaitLimit)) ws_fail(d);
      oz_contract<N, NUe, NUo, NRe, NRo>(reinterpret_cast<const double *>(X[b]), reinterpret_cast<double *>(Y[b]), cw,
                                         kWsCtrWarps, lane, Ems[b]);
      mbar_arrive(&yfull[b]);
      mbar_arrive(&xempty[b]);
    }
  }
}
