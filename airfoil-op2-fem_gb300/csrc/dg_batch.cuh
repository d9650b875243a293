// Batched path: many instances (airfoil or vortex; any K, order 1..6, Mach, alpha) advanced
// together.  Included at the end of dg_solver.cu so that it shares the per-order constant-memory
// operators and the device functions face_node<N> / elem_tile_sym<N> with the plain path: a
// batched instance computes exactly what its own Solver would, bit for bit.
//
// One RK stage of the whole batch is ONE persistent kernel (cooperative launch, all blocks
// resident):
//   phase 1  face tiles of every instance (a tile = up to FT face nodes of one instance)
//   grid barrier
//   phase 2  element tiles of every instance (32 cells of one instance; order-4 tiles first)
// Blocks walk the tile lists with a grid stride.  A step is three such launches and one
// finalize launch over the instances, captured once in a CUDA graph.  The launch shape (block
// size, resident blocks per SM, face tile size) is chosen per batch by a timing autotuner.
#pragma once

namespace dg {

struct GridBarrier {
  unsigned count;
  unsigned gen;
  unsigned err;  // bit 1: a barrier wait gave up (the stage's results are then invalid)
  unsigned pad;
  unsigned long long limit;  // longest wait in SM clocks; 0: 2^32 (about 2 s)
};

// Generation barrier over all blocks of a cooperative launch.  The wait is bounded by b->limit
// SM clocks: on timeout the block records the error and the caller stops.
__device__ __forceinline__ bool grid_barrier(GridBarrier *b, const unsigned nblocks) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned *vgen = &b->gen;
    const unsigned gen = *vgen;
    const long long limit = b->limit ? (long long)b->limit : (1ll << 32);
    __threadfence();
    if (atomicAdd(&b->count, 1u) == nblocks - 1) {
      b->count = 0;
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      const long long start = clock64();
      while (*vgen == gen) {
        if (clock64() - start > limit) {
          atomicOr(&b->err, 2u);
          ok = 0;
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Check of the barrier's bounded wait: one cooperative launch that runs only a grid barrier, with
// block 0 held back before it by a bounded delay of `hold` SM clocks.  With hold above the
// barrier's limit the other blocks' waits run out (the error is recorded and they return), and
// block 0 then arrives last and completes the barrier alone: every wait ends.
__global__ void barrier_check_kernel(GridBarrier *b, const long long hold) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && hold > 0) {
    const long long t0 = clock64();
    while (clock64() - t0 < hold) __nanosleep(256);
  }
  grid_barrier(b, gridDim.x);
}

#define DG_DISPATCH_RT(N_, CALL)                             \
  switch (N_) {                                              \
    case 1: { constexpr int NN = 1; CALL; } break;          \
    case 2: { constexpr int NN = 2; CALL; } break;          \
    case 3: { constexpr int NN = 3; CALL; } break;          \
    case 4: { constexpr int NN = 4; CALL; } break;          \
    case 5: { constexpr int NN = 5; CALL; } break;          \
    case 6: { constexpr int NN = 6; CALL; } break;          \
    default: break;                                          \
  }

// ftiles: {instance, first face node, count, order}; etiles: {instance, first cell, 0, order}.
// TC: the element contraction's form as in elem_tile_sym (0 FP64, 1 even/odd blocks on the tensor
// cores, 2 dense rows on the tensor cores), the one the plain path uses.
template <int BS, int MINB, int TC>
__global__ void __launch_bounds__(BS, MINB) batch_stage_kernel(const Inst *insts, const int4 *ftiles, const int nft,
                                                                const int4 *etiles, const int net, const int stage,
                                                                GridBarrier *bar) {
  extern __shared__ double2 Xb[];
  for (int t = blockIdx.x; t < nft; t += gridDim.x) {
    const int4 ft = ftiles[t];
    const Inst &d = insts[ft.x];
    for (int k = threadIdx.x; k < ft.z; k += BS) DG_DISPATCH_RT(ft.w, face_node<NN>(d, stage, ft.y + k));
  }
  if (!grid_barrier(bar, gridDim.x)) return;
  for (int t = blockIdx.x; t < net; t += gridDim.x) {
    const int4 et = etiles[t];
    const Inst &d = insts[et.x];
    DG_DISPATCH_RT(et.w, (elem_tile_sym<NN, false, TC>(d, stage, et.y, threadIdx.x & 31, threadIdx.x >> 5, Xb)));
  }
}

// The grouped alternative the autotuner also times: per stage one ordinary launch over every
// instance's face tiles, then one launch per order over that order's element tiles (no grid
// barrier: the kernel boundary orders the two phases).  Same device functions, same results.
__global__ void __launch_bounds__(256) batch_face_kernel(const Inst *insts, const int4 *ftiles, const int stage) {
  const int4 ft = ftiles[blockIdx.x];
  if ((int)threadIdx.x >= ft.z) return;
  DG_DISPATCH_RT(ft.w, face_node<NN>(insts[ft.x], stage, ft.y + threadIdx.x));
}

template <int N, int TC>
__global__ void __launch_bounds__(32 * np_of(N), elem_min_blocks(N, TC)) batch_elem_kernel(const Inst *insts, const int4 *etiles,
                                                                                const int first, const int stage) {
  extern __shared__ double2 Xg[];
  const int4 et = etiles[first + blockIdx.x];
  elem_tile_sym<N, false, TC>(insts[et.x], stage, et.y, threadIdx.x & 31, threadIdx.x >> 5, Xg);
}

// The step's finalize of every instance, with the calc_dt maximum taken from the element
// kernels' single-precision estimates as dt_finalize_kernel does for one solver: fblocks[b] =
// {instance k, first estimate of the block, blocks of instance k, 0}; each block's 8 warps read
// 32 estimates each (one ballot), evaluate the candidates within 1e-4 of the instance's largest
// estimate in FP64 (each by the whole warp), combine them by atomicMax, and the instance's last
// block (the counter in its step state, no waiting) advances its t and sets its dt.  Instances
// with a frozen dt get one block that advances t.
__global__ void __launch_bounds__(256) batch_dt_finalize_kernel(const Inst *insts, const int4 *fblocks) {
  const int4 fb = fblocks[blockIdx.x];
  const Inst &d = insts[fb.x];
  unsigned long long best = 0ull;
  if (d.dt_mode == 0) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int Np = np_of(d.N), n = ((d.K + 31) >> 5) * Np;
    const float thr = __uint_as_float(d.st->dt_est_max) * 0.9999f;
    const int base = fb.y + warp * 32;
    unsigned cand = __ballot_sync(0xffffffffu, base + lane < n && d.dt_est[base + lane] >= thr);
    while (cand) {
      const int k = __ffs((int)cand) - 1;
      cand &= cand - 1u;
      const int j = base + k, tile = j / Np;
      unsigned long long v = 0ull;
      DG_DISPATCH_RT(d.N, (v = dt_node_bits<NN>(d, tile * 32 + lane, j - tile * Np)));
      best = v > best ? v : best;
    }
  }
  finalize_block_end(d, best, (unsigned)fb.z);
}

// Kernel variants the autotuner chooses among: block size x minimum resident blocks (the
// register budget follows from both).
struct BatchVariant {
  int bs, minb;
  const void *fn;
};

template <int BS, int MINB, int TC>
static BatchVariant batch_variant() {
  return BatchVariant{BS, MINB, (const void *)batch_stage_kernel<BS, MINB, TC>};
}

// The persistent kernels of the current element-kernel form (the batch computes exactly what the
// plain solvers compute).
static std::vector<BatchVariant> batch_variants() {
  if (g_elem_variant == 3)
    return {batch_variant<512, 1, 2>(), batch_variant<512, 2, 2>(), batch_variant<1024, 1, 2>()};
  if (g_elem_variant == 2)
    return {batch_variant<512, 1, 1>(), batch_variant<512, 2, 1>(), batch_variant<1024, 1, 1>()};
  return {batch_variant<512, 1, 0>(), batch_variant<512, 2, 0>(), batch_variant<1024, 1, 0>()};
}

// Variant id of the grouped launches (not a persistent kernel).
constexpr int kGroupedVariant = 99;

struct BatchShape {
  int variant = -1;  // index into batch_variants(), or kGroupedVariant
  int face_tile = 0; // face nodes per face tile
  int grid = 0;      // blocks
  size_t smem = 0;
  float ms_per_step = 0.0f;
};

struct Batch {
  std::vector<Solver *> solvers;  // owned
  std::vector<Config> cfgs;
  std::vector<BatchShape> tried;
  BatchShape shape;
  int maxN = 0, maxNp = 0;
  cudaStream_t stream = nullptr;
  Inst *d_insts = nullptr;
  int4 *d_ftiles = nullptr, *d_etiles = nullptr;
  int nft = 0, net = 0;
  int4 *d_fblocks = nullptr;  // blocks of batch_dt_finalize_kernel
  int nfb = 0;
  int ord_first[7] = {0}, ord_count[7] = {0};  // element tiles of each order (contiguous)
  GridBarrier *d_bar = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  cudaGraph_t graph = nullptr;
  bool graph_ok = true;

  ~Batch() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    if (graph) cudaGraphDestroy(graph);
    if (d_insts) cudaFree(d_insts);
    if (d_ftiles) cudaFree(d_ftiles);
    if (d_etiles) cudaFree(d_etiles);
    if (d_fblocks) cudaFree(d_fblocks);
    if (d_bar) cudaFree(d_bar);
    for (Solver *s : solvers) delete s;
    if (stream) cudaStreamDestroy(stream);
  }

  int create(const std::vector<Config> &cs, const std::vector<const Mesh *> &meshes, std::string &err) {
    if (cs.empty() || cs.size() != meshes.size()) { err = "empty batch"; return -1; }
    cudaError_t ce = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    cfgs = cs;
    for (size_t k = 0; k < cs.size(); k++) {
      auto *s = new Solver();
      solvers.push_back(s);
      if (int rc = s->create(cs[k], *meshes[k], err)) {
        err = "instance " + std::to_string(k) + ": " + err;
        return rc;
      }
      maxN = std::max(maxN, cs[k].N);
    }
    maxNp = np_of(maxN);
    std::vector<Inst> insts;
    std::vector<int4> fbs;  // the finalize's blocks: 256 estimates each, one for a frozen dt
    for (size_t k = 0; k < solvers.size(); k++) {
      const Inst &d = solvers[k]->d;
      insts.push_back(d);
      const int n = ((d.K + 31) / 32) * np_of(d.N);
      const int g = d.dt_mode == 0 ? std::max(1, (n + 255) / 256) : 1;
      for (int b = 0; b < g; b++) fbs.push_back(make_int4((int)k, 256 * b, g, 0));
    }
    nfb = (int)fbs.size();
    if (cudaMalloc(&d_fblocks, sizeof(int4) * fbs.size()) != cudaSuccess ||
        cudaMemcpy(d_fblocks, fbs.data(), sizeof(int4) * fbs.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
      err = "cudaMalloc failed";
      return -100;
    }
    if (cudaMalloc(&d_insts, sizeof(Inst) * insts.size()) != cudaSuccess ||
        cudaMalloc(&d_bar, sizeof(GridBarrier)) != cudaSuccess) {
      err = "cudaMalloc failed";
      return -100;
    }
    ce = cudaMemcpy(d_insts, insts.data(), sizeof(Inst) * insts.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemset(d_bar, 0, sizeof(GridBarrier));
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    return 0;
  }

  // Element tiles (32 cells of one instance), higher orders first; face tiles of ft nodes.
  int build_tiles(int ft, std::string &err) {
    std::vector<int4> et, fts;
    for (int n = 6; n >= 1; n--) {
      ord_first[n] = (int)et.size();
      for (size_t k = 0; k < solvers.size(); k++) {
        if (cfgs[k].N != n) continue;
        const int K = solvers[k]->K;
        for (int e0 = 0; e0 < K; e0 += 32) et.push_back(make_int4((int)k, e0, 0, n));
      }
      ord_count[n] = (int)et.size() - ord_first[n];
    }
    for (size_t k = 0; k < solvers.size(); k++) {
      const Inst &d = solvers[k]->d;
      const int total = (d.nE + d.nB) * (d.N + 1);
      for (int f0 = 0; f0 < total; f0 += ft) fts.push_back(make_int4((int)k, f0, std::min(ft, total - f0), d.N));
    }
    if (d_ftiles) cudaFree(d_ftiles);
    if (d_etiles) cudaFree(d_etiles);
    d_ftiles = d_etiles = nullptr;
    if (cudaMalloc(&d_ftiles, sizeof(int4) * fts.size()) != cudaSuccess ||
        cudaMalloc(&d_etiles, sizeof(int4) * et.size()) != cudaSuccess) {
      err = "cudaMalloc failed";
      return -100;
    }
    cudaError_t ce = cudaMemcpy(d_ftiles, fts.data(), sizeof(int4) * fts.size(), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemcpy(d_etiles, et.data(), sizeof(int4) * et.size(), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    nft = (int)fts.size();
    net = (int)et.size();
    return 0;
  }

  int init(std::string &err) {
    for (Solver *s : solvers)
      if (int rc = s->init(err)) return rc;
    return 0;
  }

  // Configure one launch shape; grid = resident blocks (cooperative launches need all resident).
  int set_shape(int variant, int ft, BatchShape &out, std::string &err) {
    if (variant == kGroupedVariant) {
      if (ft < 32 || ft > 256 || ft % 32) { err = "grouped face tiles are 32..256 nodes, a multiple of 32"; return -1; }
      for (int n = 1; n <= 6; n++) {
        const size_t sm = elem_sym_smem(n);
        cudaError_t ce = cudaSuccess;
        DG_DISPATCH(n, ce = cudaFuncSetAttribute(batch_elem_kernel<NN, 0>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        if (ce == cudaSuccess) {
          DG_DISPATCH(n, ce = cudaFuncSetAttribute(batch_elem_kernel<NN, 1>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        }
        if (ce == cudaSuccess) {
          DG_DISPATCH(n, ce = cudaFuncSetAttribute(batch_elem_kernel<NN, 2>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        }
        if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
      }
      if (int rc = build_tiles(ft, err)) return rc;
      out.variant = variant;
      out.face_tile = ft;
      out.grid = 0;
      out.smem = 0;
      return 0;
    }
    const auto vs = batch_variants();
    if (variant < 0 || variant >= (int)vs.size()) { err = "bad variant"; return -1; }
    const BatchVariant &v = vs[variant];
    if (v.bs < 32 * maxNp) { err = "block too small for the batch's highest order"; return -1; }
    const size_t smem = elem_sym_smem(maxN);
    cudaError_t ce = cudaFuncSetAttribute(v.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0, dev = 0, sms = 0;
    if (ce == cudaSuccess) ce = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, v.fn, v.bs, smem);
    if (ce == cudaSuccess) ce = cudaGetDevice(&dev);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    if (per_sm < 1) { err = "batched kernel does not fit on an SM"; return -1; }
    if (int rc = build_tiles(ft, err)) return rc;
    out.variant = variant;
    out.face_tile = ft;
    out.grid = per_sm * sms;
    out.smem = smem;
    return 0;
  }

  cudaError_t launch_stage(const BatchShape &sh, int stage, cudaStream_t s) {
    const BatchVariant v = batch_variants()[sh.variant];
    cudaLaunchConfig_t lc = {};
    lc.gridDim = dim3(sh.grid);
    lc.blockDim = dim3(v.bs);
    lc.dynamicSmemBytes = sh.smem;
    lc.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    lc.attrs = at;
    lc.numAttrs = 1;
    const Inst *a0 = d_insts;
    const int4 *a1 = d_ftiles;
    int a2 = nft;
    const int4 *a3 = d_etiles;
    int a4 = net;
    int a5 = stage;
    GridBarrier *a6 = d_bar;
    void *args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6};
    return cudaLaunchKernelExC(&lc, v.fn, args);
  }

  cudaError_t launch_grouped(const BatchShape &sh, int stage, cudaStream_t s) {
    batch_face_kernel<<<nft, sh.face_tile, 0, s>>>(d_insts, d_ftiles, stage);
    for (int n = 6; n >= 1; n--) {
      if (!ord_count[n]) continue;
      const size_t sm = elem_sym_smem(n);
      if (g_elem_variant == 3) {
        DG_DISPATCH(n, (batch_elem_kernel<NN, 2><<<ord_count[n], 32 * np_of(NN), sm, s>>>(d_insts, d_etiles,
                                                                                          ord_first[n], stage)));
      } else if (g_elem_variant == 2) {
        DG_DISPATCH(n, (batch_elem_kernel<NN, 1><<<ord_count[n], 32 * np_of(NN), sm, s>>>(d_insts, d_etiles,
                                                                                          ord_first[n], stage)));
      } else {
        DG_DISPATCH(n, (batch_elem_kernel<NN, 0><<<ord_count[n], 32 * np_of(NN), sm, s>>>(d_insts, d_etiles,
                                                                                          ord_first[n], stage)));
      }
    }
    return cudaGetLastError();
  }

  cudaError_t enqueue_step(const BatchShape &sh, cudaStream_t s) {
    for (int stage = 0; stage < 3; stage++) {
      cudaError_t ce = sh.variant == kGroupedVariant ? launch_grouped(sh, stage, s) : launch_stage(sh, stage, s);
      if (ce != cudaSuccess) return ce;
    }
    batch_dt_finalize_kernel<<<nfb, 256, 0, s>>>(d_insts, d_fblocks);
    return cudaGetLastError();
  }

  // Time each candidate shape over a few steps on copies of the current state, keep the best,
  // and restore the state.  Candidates: every kernel variant that fits x face tiles of 1, 2
  // and 4 blocks' worth of nodes.
  int autotune(int steps, std::string &err) {
    std::vector<std::vector<double>> q0(solvers.size()), w0(solvers.size());
    std::vector<StepState> s0(solvers.size());
    for (size_t k = 0; k < solvers.size(); k++) {
      Solver *s = solvers[k];
      q0[k].resize(s->q_count());
      w0[k].resize(s->q_count());
      cudaError_t ce = cudaMemcpy(q0[k].data(), s->d.q, q0[k].size() * 8, cudaMemcpyDeviceToHost);
      if (ce == cudaSuccess) ce = cudaMemcpy(w0[k].data(), s->d.W, w0[k].size() * 8, cudaMemcpyDeviceToHost);
      if (ce == cudaSuccess) ce = cudaMemcpy(&s0[k], s->d.st, sizeof(StepState), cudaMemcpyDeviceToHost);
      if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    }
    tried.clear();
    BatchShape best;
    const auto vs = batch_variants();
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    std::vector<std::pair<int, int>> cands;
    for (int v = 0; v < (int)vs.size(); v++)
      if (vs[v].bs >= 32 * maxNp)
        for (int mult : {1, 2, 4}) cands.push_back({v, vs[v].bs * mult});
    for (int ft : {64, 128, 256}) cands.push_back({kGroupedVariant, ft});
    for (const auto &cand : cands) {
      const int v = cand.first;
      {
        BatchShape sh;
        std::string e2;
        if (set_shape(v, cand.second, sh, e2)) continue;
        if (enqueue_step(sh, stream) != cudaSuccess) { cudaGetLastError(); continue; }  // warm-up
        cudaEventRecord(a, stream);
        bool ok = true;
        for (int i = 0; i < steps && ok; i++) ok = enqueue_step(sh, stream) == cudaSuccess;
        cudaEventRecord(b, stream);
        if (!ok || cudaEventSynchronize(b) != cudaSuccess) { cudaGetLastError(); continue; }
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        sh.ms_per_step = ms / steps;
        tried.push_back(sh);
        if (best.variant < 0 || sh.ms_per_step < best.ms_per_step) best = sh;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    for (size_t k = 0; k < solvers.size(); k++) {
      Solver *s = solvers[k];
      cudaError_t ce = cudaMemcpy(s->d.q, q0[k].data(), q0[k].size() * 8, cudaMemcpyHostToDevice);
      if (ce == cudaSuccess) ce = cudaMemcpy(s->d.W, w0[k].data(), w0[k].size() * 8, cudaMemcpyHostToDevice);
      if (ce == cudaSuccess) ce = cudaMemcpy(s->d.st, &s0[k], sizeof(StepState), cudaMemcpyHostToDevice);
      if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    }
    if (best.variant < 0) { err = "no batched launch shape ran"; return -7; }
    if (int rc = set_shape(best.variant, best.face_tile, shape, err)) return rc;
    shape.ms_per_step = best.ms_per_step;
    if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
    return 0;
  }

  int ensure_shape(std::string &err) {
    if (shape.variant >= 0) return 0;
    const auto vs = batch_variants();
    for (int v = 0; v < (int)vs.size(); v++)
      if (vs[v].bs >= 32 * maxNp) return set_shape(v, vs[v].bs, shape, err);
    err = "no kernel variant fits the batch's highest order";
    return -1;
  }

  // The step graph.  Grouped launches are stream-captured; the persistent kernel's graph is
  // built node by node: stream capture does not take cooperative launches, a kernel node with
  // the cooperative attribute does.
  int build_graph(std::string &err) {
    if (shape.variant == kGroupedVariant) {
      cudaError_t ce = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
      if (ce == cudaSuccess) enqueue_step(shape, stream);
      cudaGraph_t g = nullptr;
      const cudaError_t ce2 = cudaStreamEndCapture(stream, &g);
      if (ce == cudaSuccess) ce = ce2;
      if (ce == cudaSuccess) ce = cudaGraphInstantiate(&graph_exec, g, 0);
      if (ce != cudaSuccess) {
        cudaGetLastError();
        if (g) cudaGraphDestroy(g);
        graph_exec = nullptr;
        err = cudaGetErrorString(ce);
        return -1;
      }
      graph = g;
      return 0;
    }
    const BatchVariant v = batch_variants()[shape.variant];
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaGraphCreate(&g, 0);
    cudaGraphNode_t prev = nullptr;
    static int stages[3] = {0, 1, 2};
    void *args[3][7];
    const Inst *a0 = d_insts;
    const int4 *a1 = d_ftiles, *a3 = d_etiles;
    int a2 = nft, a4 = net;
    GridBarrier *a6 = d_bar;
    for (int st = 0; st < 3 && ce == cudaSuccess; st++) {
      void *arr[7] = {(void *)&a0, (void *)&a1, (void *)&a2, (void *)&a3, (void *)&a4, (void *)&stages[st], (void *)&a6};
      for (int k = 0; k < 7; k++) args[st][k] = arr[k];
      cudaKernelNodeParams kp = {};
      kp.func = (void *)v.fn;
      kp.gridDim = dim3(shape.grid);
      kp.blockDim = dim3(v.bs);
      kp.sharedMemBytes = (unsigned)shape.smem;
      kp.kernelParams = args[st];
      cudaGraphNode_t node;
      ce = cudaGraphAddKernelNode(&node, g, prev ? &prev : nullptr, prev ? 1 : 0, &kp);
      if (ce == cudaSuccess) {
        cudaKernelNodeAttrValue av = {};
        av.cooperative = 1;
        ce = cudaGraphKernelNodeSetAttribute(node, cudaKernelNodeAttributeCooperative, &av);
      }
      prev = node;
    }
    if (ce == cudaSuccess) {
      const int4 *fbp = d_fblocks;
      void *fargs[2] = {(void *)&a0, (void *)&fbp};
      cudaKernelNodeParams kp = {};
      kp.func = (void *)batch_dt_finalize_kernel;
      kp.gridDim = dim3(nfb);
      kp.blockDim = dim3(256);
      kp.kernelParams = fargs;
      cudaGraphNode_t node;
      ce = cudaGraphAddKernelNode(&node, g, &prev, 1, &kp);
    }
    if (ce == cudaSuccess) ce = cudaGraphInstantiate(&graph_exec, g, 0);
    if (ce != cudaSuccess) {
      cudaGetLastError();
      if (g) cudaGraphDestroy(g);
      graph_exec = nullptr;
      err = cudaGetErrorString(ce);
      return -1;
    }
    graph = g;
    return 0;
  }

  int run(int nsteps, std::string &err) {
    if (int rc = ensure_shape(err)) return rc;
    if (!graph_exec && graph_ok) {
      std::string gerr;
      if (build_graph(gerr)) graph_ok = false;  // launch directly instead
    }
    for (int i = 0; i < nsteps; i++) {
      cudaError_t ce = graph_exec ? cudaGraphLaunch(graph_exec, stream) : enqueue_step(shape, stream);
      if (ce != cudaSuccess) { err = std::string("batched step: ") + cudaGetErrorString(ce); return -100; }
    }
    return 0;
  }

  // The grid barrier's longest wait, SM clocks (0: the default, 2^32).
  int set_barrier_limit(unsigned long long cycles, std::string &err) {
    cudaError_t ce = cudaStreamSynchronize(stream);
    if (ce == cudaSuccess)
      ce = cudaMemcpy((char *)d_bar + offsetof(GridBarrier, limit), &cycles, sizeof(cycles), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    return 0;
  }

  // One launch of barrier_check_kernel over one block per SM on the batch's stream and barrier
  // (its outcome is read by sync()).
  int barrier_check(unsigned long long hold, std::string &err) {
    int dev = 0, sms = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sms);
    cfg.blockDim = dim3(64);
    cfg.stream = stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    ce = cudaLaunchKernelEx(&cfg, barrier_check_kernel, d_bar, (long long)hold);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    return 0;
  }

  int sync(std::string &err) {
    cudaError_t ce = cudaStreamSynchronize(stream);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    GridBarrier b;
    ce = cudaMemcpy(&b, d_bar, sizeof(b), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return -100; }
    if (b.err) {
      // report once: the flag is cleared so that the batch can be re-initialised and run again
      GridBarrier z = {};
      z.limit = b.limit;
      cudaMemcpy(d_bar, &z, sizeof(z), cudaMemcpyHostToDevice);
      err = "a grid barrier wait timed out: results of that step are invalid";
      return -8;
    }
    for (size_t k = 0; k < solvers.size(); k++) {
      StepState st;
      if (solvers[k]->state(st, err)) return -100;
      if (st.err & 1u) { err = "instance " + std::to_string(k) + ": non-positive or non-finite density"; return -200; }
    }
    return 0;
  }
};

}  // namespace dg
