// Scalar advection app (advec/src/advec.cpp) on the device: host side.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "dg_mesh.h"

namespace dg {

// Everything the advection kernels need about one instance, passed by value.
struct AdvInst {
  int N, K, nE, nB;
  const int4 *edges;   // {cL, cR, fL | fR << 2 | reverse << 4, 0}
  const int4 *bedges;  // {cell, face, type, 0}
  const int *fmask;
  const double *geo;   // [K][16]: rx, ry, sx, sy, (nx, ny, fscale) x 3, J, pad
  double *q, *W, *acc, *flux, *rhs_out;
  double vx, vy, speed, dt;
};

struct Advection {
  AdvInst d{};
  int K = 0, N = 0;
  double t = 0.0;
  unsigned long long steps = 0;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  double *coords_d = nullptr;
  int *cells_d = nullptr;
  std::vector<void *> allocs;

  ~Advection();
  int create(const Mesh &m, int order, double vel_x, double vel_y, double dt, std::string &err);
  int init(std::string &err);
  void enqueue_step(cudaStream_t s);
  // One step with an event after each of its eight kernels (ev[0] recorded by the caller).
  void enqueue_step_events(cudaStream_t s, cudaEvent_t *ev);
  int step(int nsteps, bool use_graph, std::string &err);
  int rhs(double *out_dev, std::string &err);
  // q at each mesh vertex as advec/src/save_solution.cpp:13-52 samples it (last cell wins).
  int vertex_values(int n_nodes, double *out_host, std::string &err);
  size_t q_count() const { return (size_t)K * (N + 1) * (N + 2) / 2; }
};

}  // namespace dg
