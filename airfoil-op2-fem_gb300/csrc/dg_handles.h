// Opaque handle types of include/dg_gb300.h (shared by the translation units that implement it).
#pragma once
#include <cuda_runtime.h>

#include "dg_advec.h"
#include "dg_mesh.h"
#include "dg_solver.h"

struct dg_mesh_t {
  dg::Mesh m;
};
struct dg_solver_t {
  dg::Solver s;
  double *dt_hist = nullptr;
  int dt_hist_len = 0;
  double *rhs_buf = nullptr;
  cudaEvent_t ev[8] = {};
};
struct dg_advec_t {
  dg::Advection a;
  double *rhs_buf = nullptr;
  cudaEvent_t ev[9] = {};
};
