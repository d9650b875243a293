/* Oracle driver of the scalar advection app — TEST INFRASTRUCTURE ONLY (see
 * dg_oracle.h).  AdvInstance<KP> owns the app's dats (advec/src/advec.cpp:80-153)
 * and runs its loop sequence (advec/src/advec.cpp:171-262): init_grid, set_ic,
 * then per step four stages of neighbour_zero, get_neighbour_q, get_bedge_q,
 * advec_rhs and (stages 0-2) set_workingQ with rk_frac {0.5, 0.5, 1.0},
 * closed by the RK4 update_Q; dt is fixed (advec.cpp:197, 0.001 there).
 * Loops run the way driver.h runs them (direct loops in static OpenMP chunks,
 * edge loops by colour).  Every face slot is written by exactly one edge or
 * boundary edge onto a zeroed slot, so the result is independent of the loop
 * order. */
#ifndef ORACLE_ADVEC_DRIVER_H
#define ORACLE_ADVEC_DRIVER_H

#include "driver.h"

namespace orc {

struct AdvBase {
  virtual ~AdvBase() {}
  virtual int init(double dt) = 0;
  virtual int get(const char *name, double *out) = 0;
  virtual int set(const char *name, const double *in) = 0;
  virtual int rhs(int stage) = 0;
  virtual int run(int iters, int nthreads) = 0;
  double dt = 0.0, t = 0.0;
};

template <class KP>
struct AdvInstance : AdvBase {
  static constexpr int Np = KP::Np, Nfp = KP::Nfp;
  int ncell, nedge, nbedge;
  std::vector<double> coords;
  std::vector<int> cell2nodes, edge2cells, edgeNum, bedge2cell, bedgeNum;
  std::vector<std::vector<int>> ecol, bcol;
  std::map<std::string, std::pair<std::vector<double> *, int>> dats;
  std::vector<double> nodeX, nodeY, x, y, xr, yr, xs, ys, rx, ry, sx, sy, nx, ny, fscale, q, W,
      exQ, rk[4];
  void *ctx;

  ~AdvInstance() override { KP::free_ctx(ctx); }

  AdvInstance(const orc_mesh *m, void *ctx_) : ctx(ctx_) {
    ncell = m->n_cells;
    nedge = m->n_edges;
    nbedge = m->n_bedges;
    coords.assign(m->coords, m->coords + 2 * m->n_nodes);
    cell2nodes.assign(m->cell2nodes, m->cell2nodes + 3 * ncell);
    edge2cells.assign(m->edge2cells, m->edge2cells + 2 * nedge);
    edgeNum.assign(m->edgeNum, m->edgeNum + 2 * nedge);
    bedge2cell.assign(m->bedge2cell, m->bedge2cell + nbedge);
    bedgeNum.assign(m->bedgeNum, m->bedgeNum + nbedge);
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
    add("q", q, Np); add("workingQ", W, Np); add("exteriorQ", exQ, 3 * Nfp);
    add("rk1", rk[0], Np); add("rk2", rk[1], Np); add("rk3", rk[2], Np); add("rk4", rk[3], Np);
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

  int init(double dt_) override {
    KP::bind(ctx);
    const int *cn = cell2nodes.data();
    for (int c = 0; c < ncell; c++) {
      KP::init_grid(&coords[2 * cn[3 * c]], &coords[2 * cn[3 * c + 1]], &coords[2 * cn[3 * c + 2]],
                    &nodeX[3 * c], &nodeY[3 * c], &x[Np * c], &y[Np * c], &xr[Np * c], &yr[Np * c],
                    &xs[Np * c], &ys[Np * c], &rx[Np * c], &ry[Np * c], &sx[Np * c], &sy[Np * c],
                    &nx[3 * Nfp * c], &ny[3 * Nfp * c], &fscale[3 * Nfp * c]);
      KP::adv_set_ic(&x[Np * c], &y[Np * c], &q[Np * c], &W[Np * c]);
    }
    dt = dt_;
    t = 0.0;
    return 0;
  }

  void stage_rhs(int j, int nt) {
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int c = 0; c < ncell; c++) KP::adv_neighbour_zero(&exQ[(size_t)3 * Nfp * c]);
    for (auto &colour_set : ecol) {
      const int ne = (int)colour_set.size();
#pragma omp parallel for num_threads(nt) schedule(static)
      for (int i = 0; i < ne; i++) {
        const int e = colour_set[i];
        const int cL = edge2cells[2 * e], cR = edge2cells[2 * e + 1];
        KP::adv_get_neighbour_q(&edgeNum[2 * e], &nodeX[3 * cL], &nodeY[3 * cL], &nodeX[3 * cR],
                                &nodeY[3 * cR], &W[(size_t)Np * cL], &W[(size_t)Np * cR],
                                &exQ[(size_t)3 * Nfp * cL], &exQ[(size_t)3 * Nfp * cR]);
      }
    }
    for (auto &colour_set : bcol) {
      const int nb = (int)colour_set.size();
#pragma omp parallel for num_threads(nt) schedule(static)
      for (int i = 0; i < nb; i++) {
        const int b = colour_set[i];
        KP::adv_get_bedge_q(&bedgeNum[b], &exQ[(size_t)3 * Nfp * bedge2cell[b]]);
      }
    }
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int c = 0; c < ncell; c++) {
      const size_t o = (size_t)Np * c, f = (size_t)3 * Nfp * c;
      KP::advec_rhs(&W[o], &exQ[f], &rx[o], &ry[o], &sx[o], &sy[o], &fscale[f], &nx[f], &ny[f],
                    &rk[j][o]);
    }
  }

  int rhs(int stage) override {
    if (stage < 0 || stage > 3) { g_err = "stage out of range"; return -1; }
    KP::bind(ctx);
    stage_rhs(stage, 1);
    return 0;
  }

  int run(int iters, int nthreads) override {
    KP::bind(ctx);
    const int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
    double rk_frac[3] = {0.5, 0.5, 1.0};
    for (int i = 0; i < iters; i++) {
      for (int j = 0; j < 4; j++) {
        stage_rhs(j, nt);
        if (j != 3) {
#pragma omp parallel for num_threads(nt) schedule(static)
          for (int c = 0; c < ncell; c++) {
            const size_t o = (size_t)Np * c;
            KP::adv_set_workingQ(&dt, &q[o], &rk[j][o], &rk_frac[j], &W[o]);
          }
        }
      }
#pragma omp parallel for num_threads(nt) schedule(static)
      for (int c = 0; c < ncell; c++) {
        const size_t o = (size_t)Np * c;
        KP::adv_update_Q(&dt, &q[o], &rk[0][o], &rk[1][o], &rk[2][o], &rk[3][o], &W[o]);
      }
      t += dt;
    }
    return 0;
  }
};

}  // namespace orc

/* The advection C API over AdvInstance<KP>; the including file defines adv_make(). */
#define ADV_DEFINE_C_API                                                                   \
  extern "C" {                                                                              \
  void *adv_create(const orc_ops *ops, const orc_mesh *mesh, double vel_x, double vel_y) {  \
    return adv_make(ops, mesh, vel_x, vel_y);                                               \
  }                                                                                         \
  void adv_destroy(void *h) { delete (orc::AdvBase *)h; }                                   \
  int adv_init(void *h, double dt) { return ((orc::AdvBase *)h)->init(dt); }               \
  int adv_get(void *h, const char *n, double *o) { return ((orc::AdvBase *)h)->get(n, o); } \
  int adv_set(void *h, const char *n, const double *i) { return ((orc::AdvBase *)h)->set(n, i); } \
  int adv_rhs(void *h, int s) { return ((orc::AdvBase *)h)->rhs(s); }                       \
  int adv_run(void *h, int it, int nt) { return ((orc::AdvBase *)h)->run(it, nt); }         \
  double adv_time(void *h) { return ((orc::AdvBase *)h)->t; }                               \
  }

#endif
