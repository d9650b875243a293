// Native DG Euler solver (host side of dg_solver.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dg_device.cuh"
#include "dg_mesh.h"

namespace dg {

struct Config {
  int N = 3;
  int app = 0;      // 0 airfoil boundary types, 1 isentropic vortex (analytic boundary and IC)
  int dt_mode = 0;  // 0 recompute dt after every step (src/airfoil.cpp:321-331), 1 frozen
  double cfl = 1.0; // dt = (1/dt1) * cfl
  double gam = 1.4, mach = 0.4, alpha_deg = 0.0, p_inf = 1.0, rho_inf = 1.0;
  double vortex_x0 = 5.0, vortex_y0 = 0.0, vortex_beta = 5.0;
};

// Device step state of one instance.
struct StepState {
  double dt;                    // current time step
  double t;                     // current time
  unsigned long long dt1_bits;  // running calc_dt maximum (bits of a non-negative double)
  double cfl;
  unsigned long long step;      // completed steps
  unsigned err;                 // bit 0: a non-positive or non-finite density was produced;
                                // bit 2: a bounded wait of the element kernel ran out
  unsigned dt_blocks;           // blocks of the step's dt kernel that are done (reset by the last)
  unsigned dt_est_max;          // bits of the largest dt estimate of the step (Inst::dt_est)
  unsigned pad;
};

// Everything a kernel needs about one instance, passed by value.
struct Inst {
  int N, K, nE, nB;
  int app, dt_mode;
  const int4 *edges;
  const int4 *bedges;
  const int *fmask;
  const double *bxy;
  const double *geo;
  double *q, *W, *flux;
  double *rhs_out;
  StepState *st;
  double *dt_hist;
  unsigned long long dt_hist_len;
  // Per 32-cell tile and node, the largest single-precision calc_dt estimate of the node-warp
  // ([tiles][Np]), written by the last stage's element kernel when non-null: the FP64 maximum is
  // then taken over the candidates by dt_finalize_kernel.  Null: the element kernel takes it.
  float *dt_est;
  Phys P;
};

// Uploads order N's operator tables and sets its kernels' shared-memory limits on the current
// device, once per (device, order); thread-safe.
int load_order_constants(int N, std::string &err);
// Freestream and gas constants of a configuration (src/airfoil.cpp:79-99), derived terms set.
Phys make_phys(const Config &c);
// 1 if order N's tables are on device dev, 0 if not, -1 for an argument out of range.
int order_constants_loaded(int dev, int N);
// 1 if the allocation-free entry point is set up on device dev, 0 if not, -1 out of range.
int noalloc_ready(int dev);
// Element kernel form for launches enqueued from now on: 3 (default) tensor cores (dense rows at
// N = 1, 2, even/odd blocks at N = 3-5), 2 even/odd blocks on the tensor cores at N = 3-5,
// 1 even/odd FP64, 0 dense FP64.
void set_elem_variant(int v);
int elem_variant();
// The tensor-core element form at N = 3 as the warp-specialised persistent kernel: 1 one block
// per SM for every launch, 2 a range launch takes its share of the SMs, 0 (default) off (one block
// per tile).
void set_elem_ws(int m);
int elem_ws();
// Resident blocks per SM the order-3 tensor-core element kernel is compiled for (3 default, or 2).
void set_elem_blocks_per_sm(int b);
int elem_blocks_per_sm();
// Host-only: parity dimensions {NUe, NUo, NRe, NRo}, even/odd operator blocks, row exponents
// [parity][32] and signed base-256 digits [parity][digit][slot 32][row 32] of the tensor-core
// contraction of order N.
int tc_operator_tables(int N, int dims[4], std::vector<double> &S, int fexp[2][32], std::vector<int> &dig,
                       std::string &err);
// Host-only: (th 2^32 + tl) 2^sc rounded to the nearest double as the tensor-core contraction
// rounds its level sums (valid for -1022 <= sc <= 900).
double tc_round(long long th, long long tl, int sc);
// Threads per face-kernel block for launches enqueued from now on (32..256, multiple of 32).
void set_face_block(int b);
// 64-thread face blocks compiled for at most 64 registers (1) or unbounded (0, default).
void set_face_regs64(int on);
int face_regs64();
// Programmatic dependent launch of the plain path's face and element kernels (default on).
void set_pdl(int on);
// Cell ranges of the step graph (Solver::build_graph): 0 automatic, 1 one range (a chain of
// launches), P > 1 a DAG of P ranges whose face and element launches overlap.  Applies to
// graphs built from now on.
constexpr int kMaxStepParts = 32;
void set_step_parts(int p);
// Steps per launch of the step graph over cell ranges (1..8, default 8).
void set_steps_per_graph(int g);
int steps_per_graph();
// Tuning of that graph: bit 0 no programmatic dependent launch between its kernels, bit 1
// per-range scheduling priorities (earlier ranges first).
void set_step_graph_flags(int f);
int step_graph_flags();
int step_parts();
int step_parts_for(int K);

struct Solver {
  Config cfg;
  Inst d{};
  int K = 0;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  double *coords_d = nullptr;
  int *cells_d = nullptr;
  std::vector<void *> allocs;

  ~Solver();
  void *dalloc(size_t bytes);
  int create(const Config &c, const Mesh &m, std::string &err);
  int init(std::string &err);
  int set_dt_from_max(std::string &err);
  void enqueue_step(cudaStream_t s);
  // The step's last launch: t += dt, step += 1 and, with dt recomputed, the new dt (pdl: with
  // programmatic dependence on the last element kernel).
  void enqueue_finalize(cudaStream_t s, bool pdl);
  int sm_count = 0;
  void enqueue_step_events(cudaStream_t s, cudaEvent_t *ev);
  int build_graph(std::string &err);
  // The step graph as a DAG of cell ranges (build_graph with more than one range).
  std::vector<int4> h_edges, h_bedges;  // device edge records in mesh order (host copy)
  int parts = 0;                         // ranges of the graph built (0: none yet)
  int4 *pedges = nullptr, *pbedges = nullptr;  // edge records sorted by range
  double *pbxy = nullptr;                // boundary node coordinates in that order
  std::vector<int> ptile0, pe0, pb0, plo, phi;
  std::vector<cudaStream_t> pstreams;
  std::vector<cudaEvent_t> pevents;
  int build_parts(int P, std::string &err);
  // One step of the ranges' DAG on s; with q_in, the input is uploaded range by range first, with
  // q_out the result is downloaded range by range (host buffers, pinned).
  void enqueue_step_parts(cudaStream_t s, const double *q_in = nullptr, double *q_out = nullptr, int nsteps = 1);
  cudaGraph_t graphG = nullptr;  // graph_steps steps in one graph (over cell ranges)
  cudaGraphExec_t graphG_exec = nullptr;
  int graph_steps = 1;
  int step_io_parts(const double *q_in, double *q_out, bool &done, std::string &err);
  // Forget the captured step graphs (rebuilt on the next run), e.g. after a pointer they hold
  // changed.
  void drop_graphs() {
    if (graph_exec) { cudaGraphExecDestroy(graph_exec); graph_exec = nullptr; }
    if (graph) { cudaGraphDestroy(graph); graph = nullptr; }
    if (graphG_exec) { cudaGraphExecDestroy(graphG_exec); graphG_exec = nullptr; }
    if (graphG) { cudaGraphDestroy(graphG); graphG = nullptr; }
    if (io_graph_exec) { cudaGraphExecDestroy(io_graph_exec); io_graph_exec = nullptr; }
    if (io_graph) { cudaGraphDestroy(io_graph); io_graph = nullptr; }
    io_in = nullptr;
    io_out = nullptr;
  }
  cudaGraph_t io_graph = nullptr;
  cudaGraphExec_t io_graph_exec = nullptr;
  const double *io_in = nullptr;
  double *io_out = nullptr;
  int kernels_per_step() const;
  int step(int nsteps, bool use_graph, std::string &err);
  // One step with host buffers at either end (either may be null): q_in is uploaded first; the
  // last element kernel runs as kOutChunks ranges of tiles on streams of falling priority and
  // each range's new q goes to q_out as soon as it is written.  Enqueues only (wait on
  // `stream`); bitwise the same step as enqueue_step.
  int step_io(const double *q_in, double *q_out, std::string &err);
  static constexpr int kOutChunks = 4;
  cudaStream_t io_streams[kOutChunks] = {};
  cudaEvent_t io_fork = nullptr, io_kern[kOutChunks] = {}, io_copy[kOutChunks] = {};
  int rhs(double *out_dev, std::string &err);
  int l2_error(double err4[4], std::string &err);
  int state(StepState &s, std::string &err);
  // rho, u, v, p per mesh vertex as src/save_solution.cpp:13-46 samples them.
  int vertex_fields(int n_nodes, double *rho, double *u, double *v, double *p, std::string &err);
  size_t q_count() const { return (size_t)K * (cfg.N + 1) * (cfg.N + 2) / 2 * 4; }
};

}  // namespace dg
