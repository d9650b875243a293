/* Oracle driver shared by the port (dg_oracle.cpp) and the reference build
 * (ref_kernels.cpp) — TEST INFRASTRUCTURE ONLY (see dg_oracle.h).
 *
 * Instance<KP> owns the reference's dats (src/airfoil.cpp:111-132) and runs
 * the reference's loop sequence over them (src/airfoil.cpp:204-334 and
 * vortex/src/vortex.cpp:186-306) with the kernel policy KP, which is either
 * the restated kernels (port::K<N>) or the reference's own headers.
 *
 * Loops over cells are "direct" and split across OpenMP threads in static
 * chunks, like OP2's openmp backend (src/openmp/euler_rhs_kernel.cpp:58-74).
 * The edge and boundary-edge loops increment per-cell dats, so they run one
 * colour at a time with the edges of a colour touching disjoint cells — the
 * job of OP2's colour plan in src/openmp/get_neighbour_q_kernel.cpp:58-94.
 * Reductions (calc_dt's OP_MAX) combine per-cell values in a max, which is
 * order-independent; the vortex L2 error is summed cell by cell in order. */
#ifndef ORACLE_DRIVER_H
#define ORACLE_DRIVER_H

#include <omp.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "dg_oracle.h"

namespace orc {

extern thread_local std::string g_err;

struct Base {
  virtual ~Base() {}
  virtual int init(double cfl) = 0;
  virtual int get(const char *name, double *out) = 0;
  virtual int set(const char *name, const double *in) = 0;
  virtual int rhs(int stage, double t_stage) = 0;
  virtual int run(int iters, int dt_mode, int nthreads, double *dt_hist) = 0;
  virtual int l2(double *err4) = 0;
  virtual int refresh_dt() = 0;
  double dt = 0.0, t = 0.0, cfl = 1.0;
};

/* Greedy colouring of a loop whose items each touch one or two cells. */
inline std::vector<std::vector<int>> colour(int n_items, int n_cells, const int *c0, const int *c1) {
  std::vector<std::vector<int>> out;
  std::vector<unsigned long long> used(n_cells, 0ull);
  std::vector<int> col(n_items, 0);
  for (int e = 0; e < n_items; e++) {
    unsigned long long m = used[c0[e]] | (c1 ? used[c1[e]] : 0ull);
    int c = 0;
    while (m & (1ull << c)) c++;
    col[e] = c;
    used[c0[e]] |= 1ull << c;
    if (c1) used[c1[e]] |= 1ull << c;
    if ((int)out.size() <= c) out.resize(c + 1);
    out[c].push_back(e);
  }
  return out;
}

template <class KP>
struct Instance : Base {
  static constexpr int Np = KP::Np, Nfp = KP::Nfp;
  int app;
  int ncell, nedge, nbedge;
  std::vector<double> coords;
  std::vector<int> cell2nodes, edge2cells, edgeNum, bedge2cell, bedgeNum, bedge_type;
  std::vector<std::vector<int>> ecol, bcol;
  std::map<std::string, std::pair<std::vector<double> *, int>> dats;
  std::vector<double> nodeX, nodeY, x, y, xr, yr, xs, ys, rx, ry, sx, sy, nx, ny, fscale, q, W,
      exQ, rk[3];

  void *ctx;  /* policy-owned constants (operators, physics), bound before every call */

  ~Instance() override { KP::free_ctx(ctx); }

  Instance(const orc_mesh *m, int app_, void *ctx_) : app(app_), ctx(ctx_) {
    ncell = m->n_cells;
    nedge = m->n_edges;
    nbedge = m->n_bedges;
    coords.assign(m->coords, m->coords + 2 * m->n_nodes);
    cell2nodes.assign(m->cell2nodes, m->cell2nodes + 3 * ncell);
    edge2cells.assign(m->edge2cells, m->edge2cells + 2 * nedge);
    edgeNum.assign(m->edgeNum, m->edgeNum + 2 * nedge);
    bedge2cell.assign(m->bedge2cell, m->bedge2cell + nbedge);
    bedgeNum.assign(m->bedgeNum, m->bedgeNum + nbedge);
    if (m->bedge_type) bedge_type.assign(m->bedge_type, m->bedge_type + nbedge);
    else bedge_type.assign(nbedge, 2);
    std::vector<int> e0(nedge), e1(nedge);
    for (int e = 0; e < nedge; e++) {
      e0[e] = edge2cells[2 * e];
      e1[e] = edge2cells[2 * e + 1];
    }
    ecol = colour(nedge, ncell, e0.data(), e1.data());
    bcol = colour(nbedge, ncell, bedge2cell.data(), nullptr);
    auto add = [&](const char *nm, std::vector<double> &v, int dim) {
      v.assign((size_t)dim * ncell, 0.0);
      dats[nm] = {&v, dim};
    };
    add("nodeX", nodeX, 3); add("nodeY", nodeY, 3);
    add("x", x, Np); add("y", y, Np);
    add("xr", xr, Np); add("yr", yr, Np); add("xs", xs, Np); add("ys", ys, Np);
    add("rx", rx, Np); add("ry", ry, Np); add("sx", sx, Np); add("sy", sy, Np);
    add("nx", nx, 3 * Nfp); add("ny", ny, 3 * Nfp); add("fscale", fscale, 3 * Nfp);
    add("q", q, 4 * Np); add("workingQ", W, 4 * Np); add("exteriorQ", exQ, 12 * Nfp);
    add("rk1", rk[0], 4 * Np); add("rk2", rk[1], 4 * Np); add("rk3", rk[2], 4 * Np);
  }

  int get(const char *name, double *out) override {
    auto it = dats.find(name);
    if (it == dats.end()) { g_err = std::string("unknown dat ") + name; return -1; }
    std::memcpy(out, it->second.first->data(), it->second.first->size() * sizeof(double));
    return 0;
  }
  int set(const char *name, const double *in) override {
    auto it = dats.find(name);
    if (it == dats.end()) { g_err = std::string("unknown dat ") + name; return -1; }
    std::memcpy(it->second.first->data(), in, it->second.first->size() * sizeof(double));
    return 0;
  }

  /* max over cells of calc_dt, each cell seeded from 0 (src/airfoil.cpp:231-235,322-327) */
  double calc_dt_all(int nt) {
    double dt1 = 0.0;
#pragma omp parallel for num_threads(nt) reduction(max : dt1) schedule(static)
    for (int c = 0; c < ncell; c++) {
      double local = 0.0;
      KP::calc_dt(&q[(size_t)c * 4 * Np], &fscale[(size_t)c * 3 * Nfp], &local);
      dt1 = std::max(dt1, local);
    }
    return dt1;
  }

  int init(double cfl_) override {
    KP::bind(ctx);
    cfl = cfl_;
    const int *cn = cell2nodes.data();
    for (int c = 0; c < ncell; c++) {
      KP::init_grid(&coords[2 * cn[3 * c]], &coords[2 * cn[3 * c + 1]], &coords[2 * cn[3 * c + 2]],
                    &nodeX[3 * c], &nodeY[3 * c], &x[Np * c], &y[Np * c], &xr[Np * c], &yr[Np * c],
                    &xs[Np * c], &ys[Np * c], &rx[Np * c], &ry[Np * c], &sx[Np * c], &sy[Np * c],
                    &nx[3 * Nfp * c], &ny[3 * Nfp * c], &fscale[3 * Nfp * c]);
    }
    double t0 = 0.0;
    for (int c = 0; c < ncell; c++) {
      if (app == ORC_APP_VORTEX)
        KP::set_ic_vortex(&t0, &x[Np * c], &y[Np * c], &q[4 * Np * c], &W[4 * Np * c]);
      else
        KP::set_ic(&q[4 * Np * c], &W[4 * Np * c]);
      KP::neighbour_zero(&exQ[12 * Nfp * c]);
    }
    double dt1 = calc_dt_all(1);
    dt = (1.0 / dt1) * cfl;
    t = 0.0;
    return 0;
  }

  void stage_rhs(int j, double t1, int nt) {
    if (app == ORC_APP_VORTEX) {
#pragma omp parallel for num_threads(nt) schedule(static)
      for (int c = 0; c < ncell; c++) KP::neighbour_zero(&exQ[(size_t)12 * Nfp * c]);
    }
    for (auto &colour_set : ecol) {
      const int ne = (int)colour_set.size();
#pragma omp parallel for num_threads(nt) schedule(static)
      for (int i = 0; i < ne; i++) {
        int e = colour_set[i];
        int cL = edge2cells[2 * e], cR = edge2cells[2 * e + 1];
        KP::get_neighbour_q(&edgeNum[2 * e], &nodeX[3 * cL], &nodeY[3 * cL], &nodeX[3 * cR],
                            &nodeY[3 * cR], &W[(size_t)4 * Np * cL], &W[(size_t)4 * Np * cR],
                            &exQ[(size_t)12 * Nfp * cL], &exQ[(size_t)12 * Nfp * cR]);
      }
    }
    for (auto &colour_set : bcol) {
      const int nb = (int)colour_set.size();
#pragma omp parallel for num_threads(nt) schedule(static)
      for (int i = 0; i < nb; i++) {
        int b = colour_set[i];
        int c = bedge2cell[b];
        if (app == ORC_APP_VORTEX)
          KP::get_bedge_q_vortex(&bedgeNum[b], &x[Np * c], &y[Np * c], &t1, &exQ[(size_t)12 * Nfp * c]);
        else
          KP::get_bedge_q(&bedge_type[b], &bedgeNum[b], &nx[3 * Nfp * c], &ny[3 * Nfp * c],
                          &W[(size_t)4 * Np * c], &exQ[(size_t)12 * Nfp * c]);
      }
    }
    const bool zero_ext = (app != ORC_APP_VORTEX);
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int c = 0; c < ncell; c++) {
      size_t o = (size_t)Np * c, f = (size_t)3 * Nfp * c;
      KP::euler_rhs(&W[4 * o], &exQ[4 * f], &rx[o], &ry[o], &sx[o], &sy[o], &fscale[f], &nx[f],
                    &ny[f], &rk[j][4 * o], zero_ext);
    }
  }

  int rhs(int stage, double t_stage) override {
    if (stage < 0 || stage > 2) { g_err = "stage out of range"; return -1; }
    KP::bind(ctx);
    stage_rhs(stage, t_stage, 1);
    return 0;
  }

  int run(int iters, int dt_mode, int nthreads, double *dt_hist) override {
    KP::bind(ctx);
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
    const double rk_t_frac[3] = {0.0, 1.0, 0.5};
    for (int i = 0; i < iters; i++) {
      for (int j = 0; j < 3; j++) {
        double t1 = t + rk_t_frac[j] * dt;
        stage_rhs(j, t1, nt);
        if (j != 2) {
#pragma omp parallel for num_threads(nt) schedule(static)
          for (int c = 0; c < ncell; c++) {
            size_t o = (size_t)4 * Np * c;
            KP::set_workingQ(&dt, &j, &q[o], &rk[0][o], &rk[1][o], &W[o]);
          }
        }
      }
#pragma omp parallel for num_threads(nt) schedule(static)
      for (int c = 0; c < ncell; c++) {
        size_t o = (size_t)4 * Np * c;
        KP::update_Q(&dt, &q[o], &rk[0][o], &rk[1][o], &rk[2][o], &W[o]);
      }
      if (dt_hist) dt_hist[i] = dt;
      t += dt;
      if (dt_mode == ORC_DT_EVERY_STEP) {
        double dt1 = calc_dt_all(nt);
        dt = (1.0 / dt1) * cfl;
      }
    }
    return 0;
  }

  /* dt = (1/dt1)*cfl from the current q and fscale (after the caller replaced geometry) */
  int refresh_dt() override {
    KP::bind(ctx);
    dt = (1.0 / calc_dt_all(1)) * cfl;
    return 0;
  }

  int l2(double *err4) override {
    KP::bind(ctx);
    double e[4] = {0, 0, 0, 0};
    for (int c = 0; c < ncell; c++)
      KP::l2_error(&x[Np * c], &y[Np * c], &q[4 * Np * c], &t, &e[0], &e[1], &e[2], &e[3]);
    for (int k = 0; k < 4; k++) err4[k] = e[k];
    return 0;
  }
};

}  // namespace orc

/* The C API over Instance<KP>; the including file defines orc_make(). */
#define ORC_DEFINE_C_API(KIND_STRING)                                                      \
  namespace orc { thread_local std::string g_err; }                                         \
  extern "C" {                                                                              \
  const char *orc_last_error(void) { return orc::g_err.c_str(); }                           \
  const char *orc_kind(void) { return KIND_STRING; }                                        \
  void *orc_create(const orc_ops *ops, const orc_phys *phys, const orc_mesh *mesh, int app) { \
    return orc_make(ops, phys, mesh, app);                                                  \
  }                                                                                         \
  void orc_destroy(void *h) { delete (orc::Base *)h; }                                      \
  int orc_init(void *h, double cfl) { return ((orc::Base *)h)->init(cfl); }                 \
  int orc_get(void *h, const char *n, double *o) { return ((orc::Base *)h)->get(n, o); }    \
  int orc_set(void *h, const char *n, const double *i) { return ((orc::Base *)h)->set(n, i); } \
  int orc_rhs(void *h, int s, double t) { return ((orc::Base *)h)->rhs(s, t); }             \
  int orc_run(void *h, int it, int m, int nt, double *d) { return ((orc::Base *)h)->run(it, m, nt, d); } \
  double orc_dt(void *h) { return ((orc::Base *)h)->dt; }                                   \
  double orc_time(void *h) { return ((orc::Base *)h)->t; }                                  \
  int orc_l2_error(void *h, double *e) { return ((orc::Base *)h)->l2(e); }                  \
  int orc_refresh_dt(void *h) { return ((orc::Base *)h)->refresh_dt(); }                    \
  }

#endif
