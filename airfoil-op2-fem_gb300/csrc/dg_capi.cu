// extern "C" implementation of include/dg_gb300.h.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <new>
#include <vector>
#include <string>

#include "../../include/dg_gb300.h"
#include "dg_mesh.h"
#include "dg_ops.h"
#include "dg_handles.h"
#include "dg_once.h"
#include "dg_solver.h"

#include <atomic>
#include <chrono>
#include <thread>

namespace {
thread_local std::string g_err;
int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}
#define CKC(x)                                                              \
  do {                                                                      \
    cudaError_t e_ = (x);                                                   \
    if (e_ != cudaSuccess) return fail(DG_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int finish_mesh(dg::Mesh &m, dg_mesh_t **out) {
  std::string err;
  if (int rc = dg::validate(m, err)) return fail(DG_ERR_ARG, "mesh: " + err + " (" + std::to_string(rc) + ")");
  *out = new (std::nothrow) dg_mesh_t{std::move(m)};
  return *out ? 0 : fail(DG_ERR_ARG, "out of host memory");
}

__global__ void flush_kernel(double2 *p, size_t n, double v) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    p[i] = make_double2(v, v);
}

__global__ void dfma_peak_kernel(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
         x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// FP64 tensor-core (DMMA) throughput probe: mma.sync m8n8k4 f64, four independent accumulator
// chains per thread.  512 flops per warp-level mma.
__global__ void dmma_peak_kernel(double *out, int iters, double a, double b) {
  double c[4][2];
  for (int k = 0; k < 4; k++) c[k][0] = c[k][1] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; k++)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  double acc = 0.0;
  for (int k = 0; k < 4; k++) acc += c[k][0] + c[k][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

// fp16 tensor-core throughput probe for the warp-level mma.sync.m16n8k16 (f32 accumulate) the
// element kernel's contraction issues: four independent accumulator chains per warp.  4096 flops
// per mma.
__global__ void f16_mma_peak_kernel(float *out, int iters, uint32_t a0, uint32_t b0) {
  float c[4][4];
  for (int k = 0; k < 4; k++)
    for (int j = 0; j < 4; j++) c[k][j] = 0.0f;
  const uint32_t a[4] = {a0, a0 ^ threadIdx.x, a0, a0 ^ 1u};
  const uint32_t b[2] = {b0, b0 ^ threadIdx.x};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; k++)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
          "{%0,%1,%2,%3};"
          : "+f"(c[k][0]), "+f"(c[k][1]), "+f"(c[k][2]), "+f"(c[k][3])
          : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
  }
  float acc = 0.0f;
  for (int k = 0; k < 4; k++) acc += c[k][0] + c[k][1] + c[k][2] + c[k][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = acc;
}

template <class F>
double time_peak(F launch, double flops) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  launch();
  cudaEventRecord(a);
  launch();
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms > 0 ? flops / (ms * 1e-3) * 1e-9 : -1.0;
}

void *g_flush_buf = nullptr;
const size_t kFlushBytes = 512ull << 20;  // 4x the 129 MB L2
}  // namespace

extern "C" {

const char *dg_last_error(void) { return g_err.c_str(); }

int dg_mesh_from_cells(int n_nodes, const double *coords, int n_cells, const int *cell2nodes,
                       dg_mesh_t **out) {
  if (!out || !coords || !cell2nodes || n_nodes <= 0 || n_cells <= 0) return fail(DG_ERR_ARG, "bad arguments");
  dg::Mesh m;
  m.coords.assign(coords, coords + 2 * (size_t)n_nodes);
  m.cell2nodes.assign(cell2nodes, cell2nodes + 3 * (size_t)n_cells);
  std::string err;
  if (dg::build_tables(m, err)) return fail(DG_ERR_ARG, "mesh: " + err);
  return finish_mesh(m, out);
}

int dg_mesh_from_cells_device(int n_nodes, const double *coords, int n_cells, const int *cell2nodes,
                              dg_mesh_t **out, float *device_ms) {
  if (!out || !coords || !cell2nodes || n_nodes <= 0 || n_cells <= 0) return fail(DG_ERR_ARG, "bad arguments");
  if ((long long)n_nodes * n_nodes >= (1ll << 62) || 3ll * n_cells >= (1ll << 31)) return fail(DG_ERR_ARG, "mesh too large");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(DG_ERR_CUDA, "no CUDA device");
  dg::Mesh m;
  m.coords.assign(coords, coords + 2 * (size_t)n_nodes);
  m.cell2nodes.assign(cell2nodes, cell2nodes + 3 * (size_t)n_cells);
  std::string err;
  if (int rc = dg::build_tables_device(m, device_ms, err)) return fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, "mesh: " + err);
  return finish_mesh(m, out);
}

int dg_mesh_from_tables(int n_nodes, const double *coords, int n_cells, const int *cell2nodes,
                        int n_edges, const int *edge2cells, const int *edgeNum, int n_bedges,
                        const int *bedge2cell, const int *bedgeNum, const int *bedge_type,
                        dg_mesh_t **out) {
  if (!out || !coords || !cell2nodes || n_nodes <= 0 || n_cells <= 0 || n_edges < 0 || n_bedges < 0 ||
      (n_edges && (!edge2cells || !edgeNum)) || (n_bedges && (!bedge2cell || !bedgeNum)))
    return fail(DG_ERR_ARG, "bad arguments");
  dg::Mesh m;
  m.coords.assign(coords, coords + 2 * (size_t)n_nodes);
  m.cell2nodes.assign(cell2nodes, cell2nodes + 3 * (size_t)n_cells);
  m.edge2cells.assign(edge2cells, edge2cells + 2 * (size_t)n_edges);
  m.edgeNum.assign(edgeNum, edgeNum + 2 * (size_t)n_edges);
  m.bedge2cell.assign(bedge2cell, bedge2cell + n_bedges);
  m.bedgeNum.assign(bedgeNum, bedgeNum + n_bedges);
  if (bedge_type) m.bedge_type.assign(bedge_type, bedge_type + n_bedges);
  else m.bedge_type.assign(n_bedges, 2);
  return finish_mesh(m, out);
}

int dg_mesh_read_vtk(const char *path, int classify_box, dg_mesh_t **out) {
  if (!path || !out) return fail(DG_ERR_ARG, "bad arguments");
  dg::Mesh m;
  std::string err;
  if (dg::read_vtk(path, m.coords, m.cell2nodes, err)) return fail(DG_ERR_ARG, err);
  if (dg::build_tables(m, err)) return fail(DG_ERR_ARG, "mesh: " + err);
  if (classify_box && dg::classify_box(m, err)) return fail(DG_ERR_ARG, err);
  return finish_mesh(m, out);
}

int dg_mesh_naca_ogrid(int n_theta, int n_r, double stretch, double radius, int farfield, dg_mesh_t **out) {
  if (!out) return fail(DG_ERR_ARG, "bad arguments");
  dg::Mesh m;
  std::string err;
  if (dg::naca_ogrid(n_theta, n_r, stretch, radius, farfield, m, err)) return fail(DG_ERR_ARG, err);
  return finish_mesh(m, out);
}

int dg_mesh_vortex_square(int n, double lo, double hi, unsigned long long seed, dg_mesh_t **out) {
  if (!out) return fail(DG_ERR_ARG, "bad arguments");
  dg::Mesh m;
  std::string err;
  if (dg::vortex_square(n, lo, hi, seed, m, err)) return fail(DG_ERR_ARG, err);
  return finish_mesh(m, out);
}

int dg_mesh_size(const dg_mesh_t *m, int what) {
  if (!m) return fail(DG_ERR_ARG, "null mesh");
  switch (what) {
    case DG_MESH_NODES: return m->m.n_nodes();
    case DG_MESH_CELLS: return m->m.n_cells();
    case DG_MESH_EDGES: return m->m.n_edges();
    case DG_MESH_BEDGES: return m->m.n_bedges();
  }
  return fail(DG_ERR_ARG, "unknown size query");
}

int dg_mesh_get(const dg_mesh_t *mh, const char *name, void *out) {
  if (!mh || !name || !out) return fail(DG_ERR_ARG, "bad arguments");
  const dg::Mesh &m = mh->m;
  std::string n(name);
  if (n == "coords") { std::memcpy(out, m.coords.data(), m.coords.size() * 8); return 0; }
  const std::vector<int> *v = nullptr;
  if (n == "cell2nodes") v = &m.cell2nodes;
  else if (n == "edge2nodes") v = &m.edge2nodes;
  else if (n == "edge2cells") v = &m.edge2cells;
  else if (n == "edgeNum") v = &m.edgeNum;
  else if (n == "bedge2nodes") v = &m.bedge2nodes;
  else if (n == "bedge2cell") v = &m.bedge2cell;
  else if (n == "bedgeNum") v = &m.bedgeNum;
  else if (n == "bedge_type") v = &m.bedge_type;
  if (!v) return fail(DG_ERR_ARG, "unknown mesh array " + n);
  std::memcpy(out, v->data(), v->size() * 4);
  return 0;
}

int dg_mesh_set_bedge_type(dg_mesh_t *m, const int *types) {
  if (!m || !types) return fail(DG_ERR_ARG, "bad arguments");
  for (int i = 0; i < m->m.n_bedges(); i++)
    if (types[i] < 0 || types[i] > 3) return fail(DG_ERR_ARG, "boundary type out of range");
  m->m.bedge_type.assign(types, types + m->m.n_bedges());
  return 0;
}

void dg_mesh_free(dg_mesh_t *m) { delete m; }

int dg_sweep_config(int n, unsigned long long seed, int *n_theta, int *n_r, int *order, double *alpha_deg,
                    double *mach) {
  if (n < 2 || !n_theta || !n_r || !order || !alpha_deg || !mach) return fail(DG_ERR_ARG, "bad arguments");
  dg::sweep_config(n, seed, n_theta, n_r, order, alpha_deg, mach);
  return 0;
}

int dg_operators(int N, double *r, double *s, double *Dr, double *Ds, double *Drw, double *Dsw,
                 double *LIFT, int *FMASK) {
  dg::Operators o;
  if (dg::build_operators(N, o)) return fail(DG_ERR_ARG, "order N must be in 1..6");
  auto cp = [](double *dst, const std::vector<double> &v) {
    if (dst) std::memcpy(dst, v.data(), v.size() * 8);
  };
  cp(r, o.r); cp(s, o.s); cp(Dr, o.Dr); cp(Ds, o.Ds); cp(Drw, o.Drw); cp(Dsw, o.Dsw); cp(LIFT, o.LIFT);
  if (FMASK) std::memcpy(FMASK, o.FMASK.data(), o.FMASK.size() * 4);
  return 0;
}

int dg_solver_create(const dg_config_t *cfg, const dg_mesh_t *mesh, dg_solver_t **out) {
  if (!cfg || !mesh || !out) return fail(DG_ERR_ARG, "bad arguments");
  if (cfg->N < 1 || cfg->N > 6) return fail(DG_ERR_ARG, "order N must be in 1..6");
  if (!(cfg->cfl > 0.0) || !(cfg->gam > 1.0) || !(cfg->rho_inf > 0.0) || !(cfg->p_inf > 0.0))
    return fail(DG_ERR_ARG, "cfl, gam-1, rho_inf and p_inf must be positive");
  if (cfg->app != 0 && cfg->app != 1) return fail(DG_ERR_ARG, "app must be 0 (airfoil) or 1 (vortex)");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(DG_ERR_CUDA, "no CUDA device");
  dg::Config c;
  c.N = cfg->N; c.app = cfg->app; c.dt_mode = cfg->dt_mode; c.cfl = cfg->cfl; c.gam = cfg->gam;
  c.mach = cfg->mach; c.alpha_deg = cfg->alpha_deg; c.p_inf = cfg->p_inf; c.rho_inf = cfg->rho_inf;
  c.vortex_x0 = cfg->vortex_x0; c.vortex_y0 = cfg->vortex_y0; c.vortex_beta = cfg->vortex_beta;
  auto *h = new (std::nothrow) dg_solver_t();
  if (!h) return fail(DG_ERR_ARG, "out of host memory");
  std::string err;
  if (int rc = h->s.create(c, mesh->m, err)) {
    delete h;
    return fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  }
  *out = h;
  return 0;
}

int dg_solver_init(dg_solver_t *h) {
  if (!h) return fail(DG_ERR_ARG, "null solver");
  std::string err;
  if (int rc = h->s.init(err)) return fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  return 0;
}

int dg_solver_run(dg_solver_t *h, int nsteps) {
  if (!h || nsteps < 0) return fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (h->s.step(nsteps, true, err)) return fail(DG_ERR_CUDA, err);
  return 0;
}

int dg_solver_kernels_per_step(dg_solver_t *h) { return h ? h->s.kernels_per_step() : -1; }

int dg_solver_sync(dg_solver_t *h) {
  if (!h) return fail(DG_ERR_ARG, "null solver");
  dg::StepState st;
  std::string err;
  if (h->s.state(st, err)) return fail(DG_ERR_CUDA, err);
  if (st.err & 1u) return fail(DG_ERR_NONPHYSICAL, "non-positive or non-finite density");
  if (st.err & 4u) return fail(DG_ERR_TIMEOUT, "a bounded wait of the element kernel ran out: results are invalid");
  return 0;
}

static double *dat_ptr(dg_solver_t *h, const std::string &n, size_t &count) {
  count = h->s.q_count();
  if (n == "q") return h->s.d.q;
  if (n == "workingQ") return h->s.d.W;
  if (n == "geo") { count = (size_t)h->s.K * 16; return const_cast<double *>(h->s.d.geo); }
  if (n == "flux") { count = (size_t)h->s.K * 3 * (h->s.cfg.N + 1) * 4; return h->s.d.flux; }
  return nullptr;
}

int dg_solver_get(dg_solver_t *h, const char *name, double *host) {
  if (!h || !name || !host) return fail(DG_ERR_ARG, "bad arguments");
  size_t n;
  double *p = dat_ptr(h, name, n);
  if (!p) return fail(DG_ERR_ARG, std::string("unknown dat ") + name);
  CKC(cudaMemcpyAsync(host, p, n * 8, cudaMemcpyDeviceToHost, h->s.stream));
  CKC(cudaStreamSynchronize(h->s.stream));
  return 0;
}

int dg_solver_set(dg_solver_t *h, const char *name, const double *host) {
  if (!h || !name || !host) return fail(DG_ERR_ARG, "bad arguments");
  std::string n(name);
  if (n != "q" && n != "workingQ") return fail(DG_ERR_ARG, "only q and workingQ can be set");
  size_t cnt;
  double *p = dat_ptr(h, n, cnt);
  CKC(cudaMemcpyAsync(p, host, cnt * 8, cudaMemcpyHostToDevice, h->s.stream));
  CKC(cudaStreamSynchronize(h->s.stream));
  return 0;
}

int dg_solver_rhs(dg_solver_t *h, const double *host_W, double *host_rhs) {
  if (!h || !host_W || !host_rhs) return fail(DG_ERR_ARG, "bad arguments");
  const size_t n = h->s.q_count();
  if (!h->rhs_buf && cudaMalloc(&h->rhs_buf, n * 8) != cudaSuccess) return fail(DG_ERR_CUDA, "cudaMalloc failed");
  CKC(cudaMemcpyAsync(h->s.d.W, host_W, n * 8, cudaMemcpyHostToDevice, h->s.stream));
  std::string err;
  if (h->s.rhs(h->rhs_buf, err)) return fail(DG_ERR_CUDA, err);
  CKC(cudaMemcpyAsync(host_rhs, h->rhs_buf, n * 8, cudaMemcpyDeviceToHost, h->s.stream));
  CKC(cudaStreamSynchronize(h->s.stream));
  return 0;
}

int dg_solver_time(dg_solver_t *h, double *t, double *dt, unsigned long long *step) {
  if (!h) return fail(DG_ERR_ARG, "null solver");
  dg::StepState st;
  std::string err;
  if (h->s.state(st, err)) return fail(DG_ERR_CUDA, err);
  if (t) *t = st.t;
  if (dt) *dt = st.dt;
  if (step) *step = st.step;
  return 0;
}

int dg_solver_l2_error(dg_solver_t *h, double *err4) {
  if (!h || !err4) return fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (h->s.l2_error(err4, err)) return fail(DG_ERR_CUDA, err);
  return 0;
}

int dg_solver_record_dt(dg_solver_t *h, int max_steps) {
  if (!h || max_steps < 0) return fail(DG_ERR_ARG, "bad arguments");
  if (h->dt_hist) { cudaFree(h->dt_hist); h->dt_hist = nullptr; }
  dg::StepState st;
  std::string err;
  if (h->s.state(st, err)) return fail(DG_ERR_CUDA, err);
  if (max_steps > 0) {
    CKC(cudaMalloc(&h->dt_hist, (size_t)(st.step + max_steps) * 8));
    CKC(cudaMemset(h->dt_hist, 0, (size_t)(st.step + max_steps) * 8));
  }
  h->dt_hist_len = (int)(st.step + max_steps);
  h->s.d.dt_hist = h->dt_hist;
  h->s.d.dt_hist_len = h->dt_hist ? (unsigned long long)h->dt_hist_len : 0ull;
  // the captured graphs hold the old pointer: rebuild on next run
  h->s.drop_graphs();
  return 0;
}

int dg_solver_dt_history(dg_solver_t *h, double *out, int n) {
  if (!h || !out || n < 0 || n > h->dt_hist_len) return fail(DG_ERR_ARG, "bad arguments");
  CKC(cudaMemcpyAsync(out, h->dt_hist, (size_t)n * 8, cudaMemcpyDeviceToHost, h->s.stream));
  CKC(cudaStreamSynchronize(h->s.stream));
  return 0;
}

int dg_solver_step_host(dg_solver_t *h, const double *q_in, int nsteps, double *q_out) {
  if (!h || nsteps < 0) return fail(DG_ERR_ARG, "bad arguments");
  const size_t n = h->s.q_count() * 8;
  std::string err;
  if (nsteps == 0) {
    if (q_in) {
      CKC(cudaMemcpyAsync(h->s.d.q, q_in, n, cudaMemcpyHostToDevice, h->s.stream));
      CKC(cudaMemcpyAsync(h->s.d.W, h->s.d.q, n, cudaMemcpyDeviceToDevice, h->s.stream));
    }
    if (q_out) CKC(cudaMemcpyAsync(q_out, h->s.d.q, n, cudaMemcpyDeviceToHost, h->s.stream));
  } else {
    // the first step takes the input range by range, the last hands out its result range by
    // range (one step: both); the steps between are graph launches
    int rc = 0;
    if (nsteps == 1) {
      rc = h->s.step_io(q_in, q_out, err);
    } else {
      rc = (q_in ? h->s.step_io(q_in, nullptr, err) : h->s.step(1, true, err));
      if (!rc) rc = h->s.step(nsteps - 2, true, err);
      if (!rc) rc = (q_out ? h->s.step_io(nullptr, q_out, err) : h->s.step(1, true, err));
    }
    if (rc) return fail(DG_ERR_CUDA, err);
  }
  CKC(cudaStreamSynchronize(h->s.stream));
  return 0;
}

void *dg_solver_device_ptr(dg_solver_t *h, const char *name) {
  if (!h || !name) return nullptr;
  size_t n;
  return dat_ptr(h, name, n);
}

void *dg_solver_stream(dg_solver_t *h) { return h ? (void *)h->s.stream : nullptr; }

int dg_solver_step_timed(dg_solver_t *h, float *ms7) {
  if (!h || !ms7) return fail(DG_ERR_ARG, "bad arguments");
  for (auto &e : h->ev)
    if (!e) CKC(cudaEventCreate(&e));
  cudaStream_t s = h->s.stream;
  CKC(cudaEventRecord(h->ev[0], s));
  h->s.enqueue_step_events(s, h->ev);
  CKC(cudaGetLastError());
  CKC(cudaEventSynchronize(h->ev[7]));
  for (int k = 0; k < 7; k++) CKC(cudaEventElapsedTime(&ms7[k], h->ev[k], h->ev[k + 1]));
  return 0;
}

// ---------------------------------------------------------------- scalar advection app
int dg_advec_create(const dg_mesh_t *mesh, int order, double vel_x, double vel_y, double dt, dg_advec_t **out) {
  if (!mesh || !out) return fail(DG_ERR_ARG, "bad arguments");
  *out = nullptr;
  int ndev = 0;
  if (order < 1 || order > 6) return fail(DG_ERR_ARG, "order N must be in 1..6");
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(DG_ERR_CUDA, "no CUDA device");
  auto *h = new (std::nothrow) dg_advec_t();
  if (!h) return fail(DG_ERR_ARG, "out of host memory");
  std::string err;
  if (int rc = h->a.create(mesh->m, order, vel_x, vel_y, dt, err)) {
    delete h;
    return fail(rc <= -100 ? DG_ERR_CUDA : DG_ERR_ARG, err);
  }
  *out = h;
  return 0;
}

int dg_advec_init(dg_advec_t *h) {
  if (!h) return fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (h->a.init(err)) return fail(DG_ERR_CUDA, err);
  return 0;
}

int dg_advec_run(dg_advec_t *h, int nsteps) {
  if (!h || nsteps < 0) return fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (h->a.step(nsteps, true, err)) return fail(DG_ERR_CUDA, err);
  return 0;
}

int dg_advec_sync(dg_advec_t *h) {
  if (!h) return fail(DG_ERR_ARG, "bad arguments");
  CKC(cudaStreamSynchronize(h->a.stream));
  return 0;
}

static double *advec_dat(dg_advec_t *h, const std::string &n, size_t &cnt) {
  cnt = h->a.q_count();
  if (n == "q") return h->a.d.q;
  if (n == "workingQ") return h->a.d.W;
  if (n == "geo") { cnt = (size_t)h->a.K * 16; return const_cast<double *>(h->a.d.geo); }
  return nullptr;
}

int dg_advec_get(dg_advec_t *h, const char *name, double *host) {
  if (!h || !name || !host) return fail(DG_ERR_ARG, "bad arguments");
  size_t n;
  double *p = advec_dat(h, name, n);
  if (!p) return fail(DG_ERR_ARG, std::string("unknown dat ") + name);
  CKC(cudaMemcpyAsync(host, p, n * 8, cudaMemcpyDeviceToHost, h->a.stream));
  CKC(cudaStreamSynchronize(h->a.stream));
  return 0;
}

int dg_advec_set(dg_advec_t *h, const char *name, const double *host) {
  if (!h || !name || !host) return fail(DG_ERR_ARG, "bad arguments");
  std::string n(name);
  if (n != "q" && n != "workingQ") return fail(DG_ERR_ARG, "only q and workingQ can be set");
  size_t cnt;
  double *p = advec_dat(h, n, cnt);
  CKC(cudaMemcpyAsync(p, host, cnt * 8, cudaMemcpyHostToDevice, h->a.stream));
  CKC(cudaStreamSynchronize(h->a.stream));
  return 0;
}

int dg_advec_rhs(dg_advec_t *h, const double *host_W, double *host_rhs) {
  if (!h || !host_W || !host_rhs) return fail(DG_ERR_ARG, "bad arguments");
  const size_t n = h->a.q_count();
  if (!h->rhs_buf && cudaMalloc(&h->rhs_buf, n * 8) != cudaSuccess) return fail(DG_ERR_CUDA, "cudaMalloc failed");
  CKC(cudaMemcpyAsync(h->a.d.W, host_W, n * 8, cudaMemcpyHostToDevice, h->a.stream));
  std::string err;
  if (h->a.rhs(h->rhs_buf, err)) return fail(DG_ERR_CUDA, err);
  CKC(cudaMemcpyAsync(host_rhs, h->rhs_buf, n * 8, cudaMemcpyDeviceToHost, h->a.stream));
  CKC(cudaStreamSynchronize(h->a.stream));
  return 0;
}

int dg_advec_time(dg_advec_t *h, double *t, unsigned long long *steps) {
  if (!h || !t) return fail(DG_ERR_ARG, "bad arguments");
  *t = h->a.t;
  if (steps) *steps = h->a.steps;
  return 0;
}

int dg_advec_step_timed(dg_advec_t *h, float *ms) {
  if (!h || !ms) return fail(DG_ERR_ARG, "bad arguments");
  if (!h->ev[0])
    for (auto &e : h->ev) CKC(cudaEventCreate(&e));
  CKC(cudaEventRecord(h->ev[0], h->a.stream));
  h->a.enqueue_step_events(h->a.stream, h->ev);
  CKC(cudaGetLastError());
  CKC(cudaEventSynchronize(h->ev[8]));
  for (int k = 0; k < 8; k++) CKC(cudaEventElapsedTime(&ms[k], h->ev[k], h->ev[k + 1]));
  h->a.t += h->a.d.dt;
  h->a.steps++;
  return 0;
}

int dg_advec_vertex_values(dg_advec_t *h, const dg_mesh_t *m, double *out) {
  if (!h || !m || !out) return fail(DG_ERR_ARG, "bad arguments");
  if (m->m.n_cells() != h->a.K) return fail(DG_ERR_ARG, "mesh does not match the instance");
  std::string err;
  if (h->a.vertex_values(m->m.n_nodes(), out, err)) return fail(DG_ERR_CUDA, err);
  return 0;
}

int dg_advec_write_vtk(dg_advec_t *h, const dg_mesh_t *m, const char *path) {
  if (!h || !m || !path) return fail(DG_ERR_ARG, "bad arguments");
  std::vector<double> v(m->m.n_nodes());
  if (int rc = dg_advec_vertex_values(h, m, v.data())) return rc;
  std::string err;
  if (dg::write_vtk_scalar(path, m->m, "q", v.data(), err)) return fail(DG_ERR_ARG, err);
  return 0;
}

void *dg_advec_stream(dg_advec_t *h) { return h ? (void *)h->a.stream : nullptr; }

void dg_advec_free(dg_advec_t *h) {
  if (!h) return;
  if (h->rhs_buf) cudaFree(h->rhs_buf);
  for (auto &e : h->ev)
    if (e) cudaEventDestroy(e);
  delete h;
}

int dg_mesh_write_vtk(const dg_mesh_t *m, const char *path, const double *rho, const double *u, const double *v,
                      const double *p) {
  if (!m || !path || !rho || !u || !v || !p) return fail(DG_ERR_ARG, "bad arguments");
  std::string err;
  if (dg::write_vtk(path, m->m, rho, u, v, p, err)) return fail(DG_ERR_ARG, err);
  return 0;
}

int dg_solver_vertex_fields(dg_solver_t *h, const dg_mesh_t *m, double *rho, double *u, double *v, double *p) {
  if (!h || !m || !rho || !u || !v || !p) return fail(DG_ERR_ARG, "bad arguments");
  if (m->m.n_cells() != h->s.K) return fail(DG_ERR_ARG, "mesh does not match the solver");
  std::string err;
  if (h->s.vertex_fields(m->m.n_nodes(), rho, u, v, p, err)) return fail(DG_ERR_CUDA, err);
  return 0;
}

int dg_solver_write_vtk(dg_solver_t *h, const dg_mesh_t *m, const char *path) {
  if (!h || !m || !path) return fail(DG_ERR_ARG, "bad arguments");
  const int nn = m->m.n_nodes();
  std::vector<double> f((size_t)4 * nn);
  if (int rc = dg_solver_vertex_fields(h, m, f.data(), f.data() + nn, f.data() + 2 * (size_t)nn, f.data() + 3 * (size_t)nn))
    return rc;
  return dg_mesh_write_vtk(m, path, f.data(), f.data() + nn, f.data() + 2 * (size_t)nn, f.data() + 3 * (size_t)nn);
}

void dg_solver_free(dg_solver_t *h) {
  if (!h) return;
  if (h->dt_hist) cudaFree(h->dt_hist);
  if (h->rhs_buf) cudaFree(h->rhs_buf);
  for (auto &e : h->ev)
    if (e) cudaEventDestroy(e);
  delete h;
}

void *dg_host_alloc(size_t bytes) {
  void *p = nullptr;
  if (cudaMallocHost(&p, bytes) != cudaSuccess) return nullptr;
  return p;
}
void dg_host_free(void *p) {
  if (p) cudaFreeHost(p);
}
void *dg_event_create(void) {
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return (void *)e;
}
int dg_event_record(void *ev, void *stream) {
  CKC(cudaEventRecord((cudaEvent_t)ev, (cudaStream_t)stream));
  return 0;
}
float dg_event_elapsed_ms(void *a, void *b) {
  float ms = -1.0f;
  if (cudaEventSynchronize((cudaEvent_t)b) != cudaSuccess) return -1.0f;
  if (cudaEventElapsedTime(&ms, (cudaEvent_t)a, (cudaEvent_t)b) != cudaSuccess) return -1.0f;
  return ms;
}
void dg_event_destroy(void *ev) {
  if (ev) cudaEventDestroy((cudaEvent_t)ev);
}
int dg_stream_sync(void *stream) {
  CKC(cudaStreamSynchronize((cudaStream_t)stream));
  return 0;
}
int dg_l2_flush(void *stream) {
  if (!g_flush_buf) CKC(cudaMalloc(&g_flush_buf, kFlushBytes));
  static double v = 0.0;
  v += 1.0;
  flush_kernel<<<152 * 4, 512, 0, (cudaStream_t)stream>>>((double2 *)g_flush_buf, kFlushBytes / 16, v);
  CKC(cudaGetLastError());
  return 0;
}
double dg_fp64_peak_gflops(void) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 4096;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
  const double g = time_peak([&] { dfma_peak_kernel<<<blocks, threads>>>(out, iters, 0.999, 1e-3); },
                             16.0 * iters * (double)blocks * threads);
  cudaFree(out);
  return g;
}

double dg_fp64_mma_peak_gflops(void) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 8, threads = 256, iters = 2048;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return -1.0;
  const double warps = (double)blocks * threads / 32;
  const double g = time_peak([&] { dmma_peak_kernel<<<blocks, threads>>>(out, iters, 0.999, 1e-3); },
                             512.0 * 4 * iters * warps);
  cudaFree(out);
  return g;
}
double dg_f16_mma_peak_gflops(void) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int blocks = sms * 4, threads = 256, iters = 4096;
  float *out = nullptr;
  if (cudaMalloc(&out, sizeof(float) * blocks * threads) != cudaSuccess) return -1.0;
  const double warps = (double)blocks * threads / 32;
  // fp16 1.0 = 0x3C00 and 2^-7 = 0x2000 in both halves: small values, no overflow over the iterations
  const double g = time_peak([&] { f16_mma_peak_kernel<<<blocks, threads>>>(out, iters, 0x3C003C00u, 0x20002000u); },
                             4096.0 * 4 * iters * warps);
  cudaFree(out);
  return g;
}
int dg_kernels_per_step(void) { return 7; }
void dg_set_step_parts(int parts) { dg::set_step_parts(parts); }
int dg_step_parts(void) { return dg::step_parts(); }
void dg_set_steps_per_graph(int steps) { dg::set_steps_per_graph(steps); }
int dg_steps_per_graph(void) { return dg::steps_per_graph(); }
void dg_set_step_graph_flags(int flags) { dg::set_step_graph_flags(flags); }
int dg_step_graph_flags(void) { return dg::step_graph_flags(); }
void dg_set_elem_variant(int variant) { dg::set_elem_variant(variant); }
int dg_elem_variant(void) { return dg::elem_variant(); }
void dg_set_elem_ws(int mode) { dg::set_elem_ws(mode); }
void dg_set_elem_blocks_per_sm(int blocks) { dg::set_elem_blocks_per_sm(blocks); }
int dg_elem_blocks_per_sm(void) { return dg::elem_blocks_per_sm(); }
int dg_elem_ws(void) { return dg::elem_ws(); }

int dg_tc_operator_digits(int N, int *dims, double *S, int *fexp, int *digits) {
  if (!dims) return fail(DG_ERR_ARG, "bad arguments");
  int d4[4], fe[2][32];
  std::vector<double> Sv;
  std::vector<int> dig;
  std::string err;
  if (dg::tc_operator_tables(N, d4, Sv, fe, dig, err)) return fail(DG_ERR_ARG, err);
  for (int k = 0; k < 4; k++) dims[k] = d4[k];
  if (S) std::copy(Sv.begin(), Sv.end(), S);
  if (fexp) std::copy(&fe[0][0], &fe[0][0] + 64, fexp);
  if (digits) std::copy(dig.begin(), dig.end(), digits);
  return 0;
}
int dg_tc_round(long long th, long long tl, int sc, double *out) {
  if (!out || sc < -1022 || sc > 900) return fail(DG_ERR_ARG, "dg_tc_round: sc outside -1022..900");
  const long long lim_h = 1LL << 41, lim_l = 1LL << 49;
  if (th <= -lim_h || th >= lim_h || tl <= -lim_l || tl >= lim_l)
    return fail(DG_ERR_ARG, "dg_tc_round: |th| < 2^41 and |tl| < 2^49 required");
  *out = dg::tc_round(th, tl, sc);
  return 0;
}
void dg_set_face_block(int threads) { dg::set_face_block(threads); }
void dg_set_face_regs64(int on) { dg::set_face_regs64(on); }
int dg_face_regs64(void) { return dg::face_regs64(); }
void dg_set_pdl(int on) { dg::set_pdl(on); }

int dg_order_tables_loaded(int device, int N) { return dg::order_constants_loaded(device, N); }
int dg_rhs_noalloc_ready(int device) { return dg::noalloc_ready(device); }

int dg_once_table_selftest(int threads, int devices, int *uploads, int *attempts) {
  if (threads < 1 || threads > 64 || devices < 1 || devices > dg::kMaxDevices || !uploads || !attempts)
    return fail(DG_ERR_ARG, "dg_once_table_selftest: 1..64 threads, 1..64 devices, two output arrays");
  constexpr int S = dg::OnceTable::kSlots;
  const int n = devices * S;
  dg::OnceTable table;
  std::vector<std::atomic<int>> ok(n), tries(n);
  for (int k = 0; k < n; k++) { ok[k] = 0; tries[k] = 0; }
  // the fake upload: takes a little time (so that threads meet inside it) and fails on its first
  // attempt for every third pair, which must then be retried by a later call
  auto load = [&](int k) {
    const int t = tries[k]++;
    std::this_thread::sleep_for(std::chrono::microseconds(50));
    if (t == 0 && k % 3 == 0) return -7;
    ok[k]++;
    return 0;
  };
  std::vector<std::thread> pool;
  for (int th = 0; th < threads; th++)
    pool.emplace_back([&, th] {
      for (int round = 0; round < 3; round++)
        for (int j = 0; j < n; j++) {
          const int k = (j * 7 + th * 13 + round * 5) % n;  // a different order in every thread
          table.ensure(k / S, k % S, [&] { return load(k); });
        }
    });
  for (auto &t : pool) t.join();
  for (int k = 0; k < n; k++) {
    if (table.done(k / S, k % S) != 1) return fail(DG_ERR_ARG, "pair left without a successful upload");
    uploads[k] = ok[k];
    attempts[k] = tries[k];
  }
  if (table.done(devices < dg::kMaxDevices ? devices : 0, S) != -1 || table.done(-1, 0) != -1)
    return fail(DG_ERR_ARG, "range check");
  return 0;
}

}  // extern "C"
