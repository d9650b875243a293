// Mesh construction on the host (see dg_mesh.h).
#include "dg_mesh.h"

#include <algorithm>
#include <cmath>
#include <fstream>
#include <random>
#include <cstdio>
#include <sstream>

namespace dg {

int read_vtk(const std::string &path, std::vector<double> &coords, std::vector<int> &cells,
             std::string &err) {
  std::ifstream f(path);
  if (!f) { err = "cannot open " + path; return -1; }
  std::string tok;
  long npts = -1;
  while (f >> tok)
    if (tok == "POINTS") { f >> npts >> tok; break; }
  if (npts <= 0) { err = "no POINTS section in " + path; return -2; }
  coords.resize(2 * npts);
  for (long i = 0; i < npts; i++) {
    double z;
    f >> coords[2 * i] >> coords[2 * i + 1] >> z;
  }
  long ncells = -1, total;
  while (f >> tok)
    if (tok == "CELLS") { f >> ncells >> total; break; }
  if (ncells < 0) { err = "no CELLS section in " + path; return -3; }
  cells.clear();
  std::vector<char> used(npts, 0);
  for (long c = 0; c < ncells; c++) {
    int k;
    f >> k;
    std::vector<int> ids(k);
    for (int i = 0; i < k; i++) f >> ids[i];
    if (k == 3) {
      cells.push_back(ids[0]);
      cells.push_back(ids[2]);
      cells.push_back(ids[1]);
      for (int i = 0; i < 3; i++) {
        if (ids[i] < 0 || ids[i] >= npts) { err = "cell vertex out of range"; return -4; }
        used[ids[i]] = 1;
      }
    }
  }
  if (!f) { err = "truncated VTK file " + path; return -5; }
  for (long i = 0; i < npts; i++)
    if (!used[i]) { err = "VTK point not used by any triangle: ids would shift"; return -6; }
  return 0;
}

int build_tables(Mesh &m, std::string &err) {
  const int nc = m.n_cells(), nn = m.n_nodes();
  const double *x = m.coords.data();
  for (int i = 0; i < nc; i++) {
    int *c = &m.cell2nodes[3 * i];
    for (int k = 0; k < 3; k++)
      if (c[k] < 0 || c[k] >= nn) { err = "cell vertex out of range"; return -1; }
    int p1 = c[0], p2 = c[1], p3 = c[2];
    double val = (x[2 * p2] - x[2 * p1]) * (x[2 * p3 + 1] - x[2 * p2 + 1]) -
                 (x[2 * p2 + 1] - x[2 * p1 + 1]) * (x[2 * p3] - x[2 * p2]);
    if (val < 0) std::swap(c[0], c[2]);
  }
  struct Half { int a, b, cell, face; };
  std::vector<Half> h(3 * (size_t)nc);
  for (int i = 0; i < nc; i++)
    for (int j = 0; j < 3; j++) {
      int p1 = m.cell2nodes[3 * i + j], p2 = m.cell2nodes[3 * i + (j + 1) % 3];
      h[3 * (size_t)i + j] = {std::min(p1, p2), std::max(p1, p2), i, j};
    }
  // Stable on equal keys: the earlier (cell, face) stays first, as the reference's map insert.
  std::stable_sort(h.begin(), h.end(), [](const Half &p, const Half &q) {
    return p.a != q.a ? p.a < q.a : p.b < q.b;
  });
  m.edge2nodes.clear(); m.edge2cells.clear(); m.edgeNum.clear();
  m.bedge2nodes.clear(); m.bedge2cell.clear(); m.bedgeNum.clear();
  for (size_t i = 0; i < h.size();) {
    size_t j = i + 1;
    while (j < h.size() && h[j].a == h[i].a && h[j].b == h[i].b) j++;
    if (h[i].a == h[i].b) { err = "degenerate edge"; return -2; }
    if (j - i == 1) {
      m.bedge2nodes.push_back(h[i].a); m.bedge2nodes.push_back(h[i].b);
      m.bedge2cell.push_back(h[i].cell);
      m.bedgeNum.push_back(h[i].face);
    } else if (j - i == 2) {
      if (h[i].cell == h[i + 1].cell) { err = "edge with identical cells"; return -3; }
      m.edge2nodes.push_back(h[i].a); m.edge2nodes.push_back(h[i].b);
      m.edge2cells.push_back(h[i].cell); m.edge2cells.push_back(h[i + 1].cell);
      m.edgeNum.push_back(h[i].face); m.edgeNum.push_back(h[i + 1].face);
    } else {
      err = "edge shared by more than two cells";
      return -4;
    }
    i = j;
  }
  m.bedge_type.assign(m.bedge2cell.size(), 2);
  return 0;
}

int classify_box(Mesh &m, std::string &err) {
  const double *c = m.coords.data();
  for (int i = 0; i < m.n_bedges(); i++) {
    int a = m.bedge2nodes[2 * i], b = m.bedge2nodes[2 * i + 1];
    double x1 = c[2 * a], y1 = c[2 * a + 1], x2 = c[2 * b], y2 = c[2 * b + 1];
    if (x1 > -1.0 && x1 < 2.0 && y1 > -1.0 && y1 < 1.0 && x2 > -1.0 && x2 < 2.0 && y2 > -1.0 &&
        y2 < 1.0)
      m.bedge_type[i] = 2;
    else if (y1 == y2)
      m.bedge_type[i] = 2;
    else if (x1 == x2)
      m.bedge_type[i] = x1 < 0.0 ? 0 : 1;
    else {
      err = "unclassified boundary edge";
      return -1;
    }
  }
  return 0;
}

static double naca_thickness(double x) {
  // Closed-trailing-edge NACA 0012 half thickness (the polynomial of naca0012.geo:14).
  return 0.594689181 * (0.298222773 * std::sqrt(x) - 0.127125232 * x - 0.357907906 * (x * x) +
                        0.291984971 * (x * x * x) - 0.105174696 * (x * x * x * x));
}

int naca_ogrid(int n_theta, int n_r, double stretch, double radius, int farfield, Mesh &m,
               std::string &err) {
  if (n_theta < 8 || n_r < 1 || stretch <= 0.0 || radius <= 1.0) { err = "bad O-grid size"; return -1; }
  m = Mesh();
  m.coords.resize(2 * (size_t)(n_r + 1) * n_theta);
  const double denom = std::pow(stretch, n_r) - 1.0;
  for (int k = 0; k < n_theta; k++) {
    double phi = 2.0 * M_PI * k / n_theta;
    double xs = 0.5 * (1.0 + std::cos(phi));
    double yt = std::max(naca_thickness(xs), 0.0);
    double ys = (k <= n_theta / 2) ? yt : -yt;
    double xf = 0.5 + radius * std::cos(phi), yf = radius * std::sin(phi);
    for (int j = 0; j <= n_r; j++) {
      double d = (std::pow(stretch, j) - 1.0) / denom;
      size_t id = (size_t)j * n_theta + k;
      m.coords[2 * id] = xs + (xf - xs) * d;
      m.coords[2 * id + 1] = ys + (yf - ys) * d;
    }
  }
  m.cell2nodes.reserve(6 * (size_t)n_theta * n_r);
  for (int j = 0; j < n_r; j++)
    for (int k = 0; k < n_theta; k++) {
      int k1 = (k + 1) % n_theta;
      int a = j * n_theta + k, b = j * n_theta + k1, c = (j + 1) * n_theta + k, d = (j + 1) * n_theta + k1;
      int t[6] = {a, c, b, b, c, d};
      m.cell2nodes.insert(m.cell2nodes.end(), t, t + 6);
    }
  if (int rc = build_tables(m, err)) return rc;
  for (int i = 0; i < m.n_bedges(); i++) {
    int p = m.bedge2nodes[2 * i], q = m.bedge2nodes[2 * i + 1];
    if (p < n_theta && q < n_theta) {
      m.bedge_type[i] = 2;
    } else {
      double xm = 0.5 * (m.coords[2 * p] + m.coords[2 * q]);
      m.bedge_type[i] = farfield ? 3 : (xm < 0.0 ? 0 : 1);
    }
  }
  return 0;
}

int vortex_square(int n, double lo, double hi, uint64_t seed, Mesh &m, std::string &err) {
  if (n < 1 || !(hi > lo)) { err = "bad square size"; return -1; }
  m = Mesh();
  std::mt19937_64 rng(seed);
  const int w = n + 1;
  m.coords.resize(2 * (size_t)w * w);
  for (int j = 0; j < w; j++)
    for (int i = 0; i < w; i++) {
      size_t id = (size_t)j * w + i;
      m.coords[2 * id] = lo + (hi - lo) * i / n;
      m.coords[2 * id + 1] = lo + (hi - lo) * j / n;
    }
  m.cell2nodes.reserve(6 * (size_t)n * n);
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      int a = j * w + i, b = a + 1, c = a + w, d = c + 1;
      if ((rng() >> 63) == 0) {
        int t[6] = {a, b, d, a, d, c};
        m.cell2nodes.insert(m.cell2nodes.end(), t, t + 6);
      } else {
        int t[6] = {a, b, c, b, d, c};
        m.cell2nodes.insert(m.cell2nodes.end(), t, t + 6);
      }
    }
  if (int rc = build_tables(m, err)) return rc;
  m.bedge_type.assign(m.n_bedges(), 0);
  return 0;
}

void sweep_config(int n, uint64_t seed, int *n_theta, int *n_r, int *order, double *alpha_deg, double *mach) {
  std::mt19937_64 rng(seed);
  for (int i = 0; i < n; i++) {
    const double u1 = (double)(rng() >> 11) * 0x1.0p-53, u2 = (double)(rng() >> 11) * 0x1.0p-53;
    alpha_deg[i] = -4.0 + 12.0 * u1;
    mach[i] = 0.3 + 0.3 * u2;
    n_theta[i] = (int)std::lround(128.0 + 256.0 * i / (n - 1));
    n_r[i] = (int)std::lround(32.0 + 64.0 * i / (n - 1));
    order[i] = (i % 2) ? 4 : 3;
  }
}

// Legacy-VTK header and grid; the caller appends POINT_DATA.
static FILE *vtk_open_grid(const std::string &path, const Mesh &m, std::string &err) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) { err = "cannot open " + path; return nullptr; }
  const int nn = m.n_nodes(), nc = m.n_cells();
  std::fprintf(f, "# vtk DataFile Version 2.0\nDG solution\nASCII\nDATASET UNSTRUCTURED_GRID\n");
  std::fprintf(f, "POINTS %d double\n", nn);
  for (int i = 0; i < nn; i++) std::fprintf(f, "%.17g %.17g 0\n", m.coords[2 * i], m.coords[2 * i + 1]);
  std::fprintf(f, "CELLS %d %d\n", nc, 4 * nc);
  for (int c = 0; c < nc; c++)
    std::fprintf(f, "3 %d %d %d\n", m.cell2nodes[3 * c], m.cell2nodes[3 * c + 1], m.cell2nodes[3 * c + 2]);
  std::fprintf(f, "CELL_TYPES %d\n", nc);
  for (int c = 0; c < nc; c++) std::fprintf(f, "5\n");
  std::fprintf(f, "POINT_DATA %d\n", nn);
  return f;
}

static void vtk_scalars(FILE *f, const char *name, const double *v, int n) {
  std::fprintf(f, "SCALARS %s double 1\nLOOKUP_TABLE default\n", name);
  for (int i = 0; i < n; i++) std::fprintf(f, "%.17g\n", v[i]);
}

static int vtk_close(FILE *f, const std::string &path, std::string &err) {
  const bool ok = std::ferror(f) == 0;
  if (std::fclose(f) != 0 || !ok) { err = "write error on " + path; return -2; }
  return 0;
}

int write_vtk(const std::string &path, const Mesh &m, const double *rho, const double *u, const double *v,
              const double *p, std::string &err) {
  FILE *f = vtk_open_grid(path, m, err);
  if (!f) return -1;
  const int nn = m.n_nodes();
  vtk_scalars(f, "rho", rho, nn);
  vtk_scalars(f, "p", p, nn);
  std::fprintf(f, "VECTORS velocity double\n");
  for (int i = 0; i < nn; i++) std::fprintf(f, "%.17g %.17g 0\n", u[i], v[i]);
  return vtk_close(f, path, err);
}

int write_vtk_scalar(const std::string &path, const Mesh &m, const char *name, const double *values,
                     std::string &err) {
  FILE *f = vtk_open_grid(path, m, err);
  if (!f) return -1;
  vtk_scalars(f, name, values, m.n_nodes());
  return vtk_close(f, path, err);
}

int validate(const Mesh &m, std::string &err) {
  const int nc = m.n_cells(), nn = m.n_nodes();
  if (nc <= 0) { err = "mesh has no cells"; return -1; }
  for (int v : m.cell2nodes)
    if (v < 0 || v >= nn) { err = "cell vertex out of range"; return -2; }
  std::vector<unsigned char> cover(3 * (size_t)nc, 0);
  for (int e = 0; e < m.n_edges(); e++)
    for (int s = 0; s < 2; s++) {
      int c = m.edge2cells[2 * e + s], f = m.edgeNum[2 * e + s];
      if (c < 0 || c >= nc || f < 0 || f > 2) { err = "edge cell or face out of range"; return -3; }
      cover[3 * (size_t)c + f]++;
    }
  for (int b = 0; b < m.n_bedges(); b++) {
    int c = m.bedge2cell[b], f = m.bedgeNum[b];
    if (c < 0 || c >= nc || f < 0 || f > 2) { err = "boundary edge cell or face out of range"; return -4; }
    int t = m.bedge_type.empty() ? 2 : m.bedge_type[b];
    if (t < 0 || t > 3) { err = "boundary type out of range"; return -5; }
    cover[3 * (size_t)c + f]++;
  }
  for (size_t i = 0; i < cover.size(); i++)
    if (cover[i] != 1) { err = "a cell face is covered by " + std::to_string(cover[i]) + " edges"; return -6; }
  return 0;
}

}  // namespace dg
