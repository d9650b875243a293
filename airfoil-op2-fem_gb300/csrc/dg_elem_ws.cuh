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
// The staging (X, Y, column exponents, staged W and q) is double-buffered: while the contraction
// warps work on tile j, the node warps fill tile j+1 and then combine tile j-1.  The two groups
// hand buffers over through mbarriers (full / empty per buffer); every wait is bounded (about
// 2^28 SM clocks), after which the thread records an error bit in the step state and goes on, so
// the kernel always ends.  The arithmetic of every tile is that of elem_tile_sym in its
// tensor-core form (same functions, same operation order): the results are bitwise the same.
#pragma once

constexpr int kWsCtrWarps = 8;  // contraction warps: oz_prep's 256 threads, 2 or 3 units each
constexpr long long kWsWaitLimit = 1ll << 28;

// Orders with a warp-specialised kernel: the even/odd blocks on the tensor cores at N = 3, 4 (at
// N = 5 the block would need 29 warps and two buffers of 150 KB).
constexpr bool ws_used(int N) { return N == 3 || N == 4; }
constexpr int ws_threads(int N) { return 32 * (np_of(N) + kWsCtrWarps); }
// one staging buffer: X (NK slots), Y (Np rows), 128 column exponents, W and q of every node
constexpr size_t ws_buf_bytes(int N) {
  return (size_t)(nk_of(N) + np_of(N)) * kElemSlot * sizeof(double) + 128 * sizeof(int) +
         (size_t)4 * 32 * np_of(N) * sizeof(double2);
}
constexpr int kWsBars = 12;
constexpr size_t ws_smem(int N) { return 2 * ws_buf_bytes(N) + kWsBars * sizeof(unsigned long long); }

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

// The node warps' barrier inside the stage combine (the dt maximum of the last stage): an
// mbarrier over the node threads, bounded like the others.
struct WsNodeSync {
  unsigned long long *bar;
  unsigned *phase;
  const Inst *d;
  __device__ __forceinline__ void operator()() const {
    mbar_arrive(bar);
    if (!mbar_wait(bar, *phase & 1u, kWsWaitLimit)) ws_fail(*d);
    (*phase)++;
  }
};

// Fill: the tile's W, metrics, q and face fluxes, and the nodal fluxes into the slots (the first
// part of elem_tile_sym in its tensor-core form).
template <int N>
__device__ __forceinline__ void ws_fill(const Inst &d, const int stage, const int e0, const int lane, const int i,
                                        double2 *X, double2 *WQ) {
  constexpr int Np = np_of(N), Nfp = N + 1;
  constexpr int kS2 = kElemSlot / 2;
  constexpr int nthr = 32 * Np;
  const int tid = i * 32 + lane;
  const int e = e0 + lane;
  const bool live = e < d.K;
  const Phys &P = d.P;
  double w[4] = {0.0, 0.0, 0.0, 0.0};
  double g[4] = {0.0, 0.0, 0.0, 0.0};
  if (live) {
    const double *wp = d.W + ((size_t)e * Np + i) * 4;
    const double2 a = ld2(wp), b = ld2(wp + 2);
    w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
    const double2 ga = ld2(d.geo + (size_t)e * 16), gb = ld2(d.geo + (size_t)e * 16 + 2);
    g[0] = ga.x; g[1] = ga.y; g[2] = gb.x; g[3] = gb.y;
    WQ[tid] = a;
    WQ[nthr + tid] = b;
    if (stage == 1 || stage == 2) {
      const double *qp = d.q + ((size_t)e * Np + i) * 4;
      cp_async16(WQ + 2 * nthr + tid, qp, true);
      cp_async16(WQ + 3 * nthr + tid, qp + 2, true);
    }
  }
  for (int j = tid; j < 3 * Nfp * 32; j += nthr) {
    const int f = j >> 5, el = j & 31;
    const bool ok = e0 + el < d.K;
    const double *fp = d.flux + (((size_t)(ok ? e0 + el : 0)) * 3 * Nfp + f) * 4;
    const int pf = c_pos[N][2 * Np + f];
    cp_async16(X + pf * kS2 + el * 2, fp, ok);
    cp_async16(X + pf * kS2 + el * 2 + 1, fp + 2, ok);
  }
  const double rx = g[0], ry = g[1], sx = g[2], sy = g[3];
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
                                           const double2 *Y, double2 *WQ, unsigned long long *yempty,
                                           const WsNodeSync &sync) {
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
  // the candidates of the last stage's dt maximum go to this buffer's W / q area: every node thread
  // has read its W and q before the combine's first barrier
  stage_combine<N, WsNodeSync>(d, stage, e, true, live, i, lane, w, r0, r1, r2, r3, WQ,
                               (stage == 1 || stage == 2) ? WQ + 2 * nthr + tid : nullptr, nthr, sync);
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
  constexpr unsigned NN = 32 * Np, NC = 32 * kWsCtrWarps;
  extern __shared__ __align__(16) unsigned char ws_sm[];
  double2 *X[2], *Y[2], *WQ[2];
  int *Ems[2];
  for (int b = 0; b < 2; b++) {
    X[b] = reinterpret_cast<double2 *>(ws_sm + b * ws_buf_bytes(N));
    Y[b] = X[b] + NK * kS2;
    Ems[b] = reinterpret_cast<int *>(Y[b] + Np * kS2);
    WQ[b] = reinterpret_cast<double2 *>(Ems[b] + 128);
  }
  // 0, 1 X full; 2, 3 X empty; 4, 5 Y full; 6, 7 Y empty; 8 pre-pass done; 9 node barrier
  unsigned long long *bars = reinterpret_cast<unsigned long long *>(ws_sm + 2 * ws_buf_bytes(N));
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int b = 0; b < 2; b++) {
      mbar_init(&bars[0 + b], NN);
      mbar_init(&bars[2 + b], NC);
      mbar_init(&bars[4 + b], NC);
      mbar_init(&bars[6 + b], NN);
    }
    mbar_init(&bars[8], NC);
    mbar_init(&bars[9], NN);
  }
  __syncthreads();
  pdl_trigger();
  const int nt = t1 - t0, G = (int)gridDim.x;
  const int tb = t0 + (int)((long long)nt * blockIdx.x / G);
  const int n = t0 + (int)((long long)nt * (blockIdx.x + 1) / G) - tb;
  if (tid < (int)NN) {
    const int i = tid >> 5, lane = tid & 31;
    unsigned nphase = 0;
    const WsNodeSync sync{&bars[9], &nphase, &d};
    if constexpr (PW) pdl_wait();
    for (int j = 0; j <= n; j++) {
      if (j < n) {
        const int b = j & 1, k = j >> 1;
        if (k >= 1 && !mbar_wait(&bars[2 + b], (unsigned)(k - 1) & 1u, kWsWaitLimit)) ws_fail(d);
        ws_fill<N>(d, stage, (tb + j) * 32, lane, i, X[b], WQ[b]);
        mbar_arrive(&bars[0 + b]);
      }
      if (j >= 1) {
        const int jj = j - 1, b = jj & 1, k = jj >> 1;
        if (!mbar_wait(&bars[4 + b], (unsigned)k & 1u, kWsWaitLimit)) ws_fail(d);
        ws_combine<N>(d, stage, (tb + jj) * 32, lane, i, Y[b], WQ[b], &bars[6 + b], sync);
      }
    }
  } else {
    const int ct = tid - (int)NN, cw = ct >> 5, lane = ct & 31;
    for (int j = 0; j < n; j++) {
      const int b = j & 1, k = j >> 1;
      if (!mbar_wait(&bars[0 + b], (unsigned)k & 1u, kWsWaitLimit)) ws_fail(d);
      oz_prep<NUe, NUo, kElemSlot>(reinterpret_cast<double *>(X[b]), Ems[b], ct);
      mbar_arrive(&bars[8]);
      if (!mbar_wait(&bars[8], (unsigned)j & 1u, kWsWaitLimit)) ws_fail(d);
      if (k >= 1 && !mbar_wait(&bars[6 + b], (unsigned)(k - 1) & 1u, kWsWaitLimit)) ws_fail(d);
      oz_contract<N, NUe, NUo, NRe, NRo>(reinterpret_cast<const double *>(X[b]), reinterpret_cast<double *>(Y[b]), cw,
                                         kWsCtrWarps, lane, Ems[b]);
      mbar_arrive(&bars[4 + b]);
      mbar_arrive(&bars[2 + b]);
    }
  }
}
