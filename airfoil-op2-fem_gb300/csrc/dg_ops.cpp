// Nodal DG operators on the reference triangle, orders N = 1..6.
//
// The reference ships these as literal N=4 tables (src/constants/constant_{r,s,Dr,Ds,Drw,Dsw,
// LIFT}.h and FMASK at src/constants/constant_util.h:15).  They are the published construction
// of Hesthaven & Warburton, "Nodal Discontinuous Galerkin Methods" (2008), ch. 6 / appendix A,
// computed here from that mathematics for any order:
//   nodes   Warp & Blend (Nodes2D) mapped to (r, s) (xytors)
//   V, Vr, Vs  orthonormal simplex basis and its gradients at the nodes
//   Dr = Vr V^-1,  Ds = Vs V^-1
//   Drw = (V Vr^T)(V V^T)^-1,  Dsw = (V Vs^T)(V V^T)^-1     (weak derivative, M^-1 S^T)
//   LIFT = (V V^T) E, E holding the 1-D face mass matrices on r, r, s of faces 0, 1, 2
//   FMASK  face 0: s=-1, r increasing; face 1: r+s=0 from vertex 1 to vertex 2;
//          face 2: r=-1 from vertex 2 back to vertex 0.
// The tables must agree with the reference's N=4 literals to rounding (checked by the tests).
#include "dg_ops.h"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

namespace dg {
namespace {

using Vec = std::vector<double>;

struct Mat {
  int n = 0, m = 0;
  Vec a;
  Mat() {}
  Mat(int n_, int m_) : n(n_), m(m_), a((size_t)n_ * m_, 0.0) {}
  double &operator()(int i, int j) { return a[(size_t)i * m + j]; }
  double operator()(int i, int j) const { return a[(size_t)i * m + j]; }
};

Mat mul(const Mat &x, const Mat &y) {
  Mat z(x.n, y.m);
  for (int i = 0; i < x.n; i++)
    for (int k = 0; k < x.m; k++) {
      double v = x(i, k);
      for (int j = 0; j < y.m; j++) z(i, j) += v * y(k, j);
    }
  return z;
}

Mat transpose(const Mat &x) {
  Mat t(x.m, x.n);
  for (int i = 0; i < x.n; i++)
    for (int j = 0; j < x.m; j++) t(j, i) = x(i, j);
  return t;
}

// Gauss-Jordan inverse with partial pivoting (matrices here are at most 28 x 28).
Mat inverse(const Mat &x) {
  const int n = x.n;
  Mat a = x, inv(n, n);
  for (int i = 0; i < n; i++) inv(i, i) = 1.0;
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int r = c + 1; r < n; r++)
      if (std::fabs(a(r, c)) > std::fabs(a(p, c))) p = r;
    if (a(p, c) == 0.0) throw std::runtime_error("singular matrix in operator construction");
    if (p != c)
      for (int j = 0; j < n; j++) {
        std::swap(a(p, j), a(c, j));
        std::swap(inv(p, j), inv(c, j));
      }
    double d = a(c, c);
    for (int j = 0; j < n; j++) {
      a(c, j) /= d;
      inv(c, j) /= d;
    }
    for (int r = 0; r < n; r++) {
      if (r == c) continue;
      double f = a(r, c);
      if (f == 0.0) continue;
      for (int j = 0; j < n; j++) {
        a(r, j) -= f * a(c, j);
        inv(r, j) -= f * inv(c, j);
      }
    }
  }
  return inv;
}

// Orthonormal Jacobi polynomial P_n^(alpha,beta) at x (three-term recurrence).
Vec jacobi_p(const Vec &x, double alpha, double beta, int n) {
  const size_t m = x.size();
  std::vector<Vec> pl(n + 1, Vec(m));
  double g0 = std::pow(2.0, alpha + beta + 1) / (alpha + beta + 1) * std::tgamma(alpha + 1) *
              std::tgamma(beta + 1) / std::tgamma(alpha + beta + 1);
  for (size_t i = 0; i < m; i++) pl[0][i] = 1.0 / std::sqrt(g0);
  if (n == 0) return pl[0];
  double g1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * g0;
  for (size_t i = 0; i < m; i++)
    pl[1][i] = ((alpha + beta + 2) * x[i] / 2 + (alpha - beta) / 2) / std::sqrt(g1);
  if (n == 1) return pl[1];
  double aold = 2 / (2 + alpha + beta) * std::sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3));
  for (int k = 1; k < n; k++) {
    double h1 = 2 * k + alpha + beta;
    double anew = 2 / (h1 + 2) *
                  std::sqrt((k + 1) * (k + 1 + alpha + beta) * (k + 1 + alpha) * (k + 1 + beta) /
                            (h1 + 1) / (h1 + 3));
    double bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2);
    for (size_t i = 0; i < m; i++)
      pl[k + 1][i] = 1 / anew * (-aold * pl[k - 1][i] + (x[i] - bnew) * pl[k][i]);
    aold = anew;
  }
  return pl[n];
}

Vec grad_jacobi_p(const Vec &x, double alpha, double beta, int n) {
  if (n == 0) return Vec(x.size(), 0.0);
  Vec p = jacobi_p(x, alpha + 1, beta + 1, n - 1);
  double f = std::sqrt(n * (n + alpha + beta + 1));
  for (double &v : p) v *= f;
  return p;
}

// Eigenvalues of a symmetric matrix by cyclic Jacobi rotations (n <= 8 here).
Vec sym_eigenvalues(Mat a) {
  const int n = a.n;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0.0;
    for (int i = 0; i < n; i++)
      for (int j = i + 1; j < n; j++) off += a(i, j) * a(i, j);
    if (off < 1e-60) break;
    for (int p = 0; p < n; p++)
      for (int q = p + 1; q < n; q++) {
        if (a(p, q) == 0.0) continue;
        double theta = (a(q, q) - a(p, p)) / (2 * a(p, q));
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1));
        double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; k++) {
          double akp = a(k, p), akq = a(k, q);
          a(k, p) = c * akp - s * akq;
          a(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; k++) {
          double apk = a(p, k), aqk = a(q, k);
          a(p, k) = c * apk - s * aqk;
          a(q, k) = s * apk + c * aqk;
        }
      }
  }
  Vec ev(n);
  for (int i = 0; i < n; i++) ev[i] = a(i, i);
  std::sort(ev.begin(), ev.end());
  return ev;
}

// Gauss quadrature points of P^(alpha,beta)_{n+1} (Golub-Welsch), refined by Newton.
Vec jacobi_gq(double alpha, double beta, int n) {
  if (n == 0) return Vec{-(alpha - beta) / (alpha + beta + 2)};
  Mat j(n + 1, n + 1);
  for (int i = 0; i <= n; i++) {
    double h1 = 2 * i + alpha + beta;
    j(i, i) = -0.5 * (alpha * alpha - beta * beta) / (h1 + 2) / h1;
    if (alpha + beta < 1e-15 && i == 0) j(i, i) = 0.0;
    if (i < n) {
      int k = i + 1;
      double off = 2 / (h1 + 2) *
                   std::sqrt(k * (k + alpha + beta) * (k + alpha) * (k + beta) / (h1 + 1) / (h1 + 3));
      j(i, i + 1) = off;
      j(i + 1, i) = off;
    }
  }
  Vec x = sym_eigenvalues(j);
  // Newton polish on P_{n+1}(x) = 0 so the nodes do not carry the eigen-solver's error.
  for (int it = 0; it < 4; it++) {
    Vec p = jacobi_p(x, alpha, beta, n + 1), dp = grad_jacobi_p(x, alpha, beta, n + 1);
    for (size_t i = 0; i < x.size(); i++) x[i] -= p[i] / dp[i];
  }
  return x;
}

Vec jacobi_gl(int n) {
  if (n == 1) return Vec{-1.0, 1.0};
  Vec in = jacobi_gq(1.0, 1.0, n - 2);
  Vec x{-1.0};
  x.insert(x.end(), in.begin(), in.end());
  x.push_back(1.0);
  return x;
}

Mat vandermonde_1d(int n, const Vec &r) {
  Mat v((int)r.size(), n + 1);
  for (int j = 0; j <= n; j++) {
    Vec p = jacobi_p(r, 0, 0, j);
    for (size_t i = 0; i < r.size(); i++) v((int)i, j) = p[i];
  }
  return v;
}

Vec warpfactor(int n, const Vec &rout) {
  Vec lgl = jacobi_gl(n), req(n + 1);
  for (int i = 0; i <= n; i++) req[i] = -1.0 + 2.0 * i / n;
  Mat veq = vandermonde_1d(n, req);
  const int nr = (int)rout.size();
  Mat pmat(n + 1, nr);
  for (int i = 0; i <= n; i++) {
    Vec p = jacobi_p(rout, 0, 0, i);
    for (int k = 0; k < nr; k++) pmat(i, k) = p[k];
  }
  Mat lmat = mul(inverse(transpose(veq)), pmat);  // solve veq^T L = P
  Vec warp(nr, 0.0);
  for (int k = 0; k < nr; k++) {
    for (int i = 0; i <= n; i++) warp[k] += lmat(i, k) * (lgl[i] - req[i]);
    double zerof = std::fabs(rout[k]) < 1.0 - 1.0e-10 ? 1.0 : 0.0;
    double sf = 1.0 - (zerof * rout[k]) * (zerof * rout[k]);
    warp[k] = warp[k] / sf + warp[k] * (zerof - 1.0);
  }
  return warp;
}

const double kAlphaOpt[15] = {0.0000, 0.0000, 1.4152, 0.1001, 0.2751, 0.9800, 1.0999, 1.2832,
                              1.3648, 1.4773, 1.4959, 1.5743, 1.5770, 1.6223, 1.6258};

void nodes_2d(int n, Vec &x, Vec &y) {
  const double alpha = n < 16 ? kAlphaOpt[n - 1] : 5.0 / 3.0;
  const int np = (n + 1) * (n + 2) / 2;
  Vec l1(np), l2(np), l3(np);
  int sk = 0;
  for (int i = 1; i <= n + 1; i++)
    for (int j = 1; j <= n + 2 - i; j++) {
      l1[sk] = (i - 1) / (double)n;
      l3[sk] = (j - 1) / (double)n;
      sk++;
    }
  x.assign(np, 0.0);
  y.assign(np, 0.0);
  Vec d1(np), d2(np), d3(np);
  for (int i = 0; i < np; i++) {
    l2[i] = 1.0 - l1[i] - l3[i];
    x[i] = -l2[i] + l3[i];
    y[i] = (-l2[i] - l3[i] + 2 * l1[i]) / std::sqrt(3.0);
    d1[i] = l3[i] - l2[i];
    d2[i] = l1[i] - l3[i];
    d3[i] = l2[i] - l1[i];
  }
  Vec w1 = warpfactor(n, d1), w2 = warpfactor(n, d2), w3 = warpfactor(n, d3);
  for (int i = 0; i < np; i++) {
    double warp1 = 4 * l2[i] * l3[i] * w1[i] * (1 + (alpha * l1[i]) * (alpha * l1[i]));
    double warp2 = 4 * l1[i] * l3[i] * w2[i] * (1 + (alpha * l2[i]) * (alpha * l2[i]));
    double warp3 = 4 * l1[i] * l2[i] * w3[i] * (1 + (alpha * l3[i]) * (alpha * l3[i]));
    x[i] = x[i] + 1 * warp1 + std::cos(2 * M_PI / 3) * warp2 + std::cos(4 * M_PI / 3) * warp3;
    y[i] = y[i] + 0 * warp1 + std::sin(2 * M_PI / 3) * warp2 + std::sin(4 * M_PI / 3) * warp3;
  }
}

void simplex_2dp_grad(const Vec &a, const Vec &b, int i, int j, Vec &p, Vec &dr, Vec &ds) {
  const size_t m = a.size();
  Vec fa = jacobi_p(a, 0, 0, i), dfa = grad_jacobi_p(a, 0, 0, i);
  Vec gb = jacobi_p(b, 2 * i + 1, 0, j), dgb = grad_jacobi_p(b, 2 * i + 1, 0, j);
  p.assign(m, 0.0);
  dr.assign(m, 0.0);
  ds.assign(m, 0.0);
  for (size_t k = 0; k < m; k++) {
    double ob = 1 - b[k];
    p[k] = std::sqrt(2.0) * fa[k] * gb[k] * std::pow(ob, i);
    double half = 0.5 * ob;
    double drv = dfa[k] * gb[k];
    if (i > 0) drv *= std::pow(half, i - 1);
    double dsv = dfa[k] * (gb[k] * (0.5 * (1 + a[k])));
    if (i > 0) dsv *= std::pow(half, i - 1);
    double tmp = dgb[k] * std::pow(half, i);
    if (i > 0) tmp -= 0.5 * i * gb[k] * std::pow(half, i - 1);
    dsv += fa[k] * tmp;
    dr[k] = std::pow(2.0, i + 0.5) * drv;
    ds[k] = std::pow(2.0, i + 0.5) * dsv;
  }
}

}  // namespace

int build_operators(int n, Operators &o) {
  if (n < 1 || n > 6) return -1;
  o.N = n;
  o.Np = (n + 1) * (n + 2) / 2;
  o.Nfp = n + 1;
  const int np = o.Np, nfp = o.Nfp;
  Vec x, y;
  nodes_2d(n, x, y);
  o.r.assign(np, 0.0);
  o.s.assign(np, 0.0);
  for (int i = 0; i < np; i++) {
    double l1 = (std::sqrt(3.0) * y[i] + 1.0) / 3.0;
    double l2 = (-3.0 * x[i] - std::sqrt(3.0) * y[i] + 2.0) / 6.0;
    double l3 = (3.0 * x[i] - std::sqrt(3.0) * y[i] + 2.0) / 6.0;
    o.r[i] = -l2 + l3 - l1;
    o.s[i] = -l2 - l3 + l1;
  }
  Vec a(np), b(np);
  for (int i = 0; i < np; i++) {
    a[i] = (o.s[i] != 1.0) ? 2 * (1 + o.r[i]) / (1 - o.s[i]) - 1 : -1.0;
    b[i] = o.s[i];
  }
  Mat v(np, np), vr(np, np), vs(np, np);
  int col = 0;
  for (int i = 0; i <= n; i++)
    for (int j = 0; j <= n - i; j++) {
      Vec p, dr, ds;
      simplex_2dp_grad(a, b, i, j, p, dr, ds);
      for (int k = 0; k < np; k++) {
        v(k, col) = p[k];
        vr(k, col) = dr[k];
        vs(k, col) = ds[k];
      }
      col++;
    }
  Mat vinv = inverse(v);
  Mat dr = mul(vr, vinv), ds = mul(vs, vinv);
  Mat vt = transpose(v);
  Mat vvt_inv = inverse(mul(v, vt));
  Mat drw = mul(mul(v, transpose(vr)), vvt_inv);
  Mat dsw = mul(mul(v, transpose(vs)), vvt_inv);
  const double tol = 1e-12;
  std::vector<int> f0, f1, f2;
  for (int i = 0; i < np; i++) {
    if (std::fabs(o.s[i] + 1) < tol) f0.push_back(i);
    if (std::fabs(o.r[i] + o.s[i]) < tol) f1.push_back(i);
    if (std::fabs(o.r[i] + 1) < tol) f2.push_back(i);
  }
  std::reverse(f2.begin(), f2.end());
  if ((int)f0.size() != nfp || (int)f1.size() != nfp || (int)f2.size() != nfp) return -2;
  o.FMASK.clear();
  o.FMASK.insert(o.FMASK.end(), f0.begin(), f0.end());
  o.FMASK.insert(o.FMASK.end(), f1.begin(), f1.end());
  o.FMASK.insert(o.FMASK.end(), f2.begin(), f2.end());
  Mat e(np, 3 * nfp);
  const std::vector<int> *faces[3] = {&f0, &f1, &f2};
  for (int f = 0; f < 3; f++) {
    Vec coord(nfp);
    for (int k = 0; k < nfp; k++) coord[k] = (f == 2) ? o.s[(*faces[f])[k]] : o.r[(*faces[f])[k]];
    Mat v1 = vandermonde_1d(n, coord);
    Mat mass = inverse(mul(v1, transpose(v1)));
    for (int i = 0; i < nfp; i++)
      for (int k = 0; k < nfp; k++) e((*faces[f])[i], f * nfp + k) = mass(i, k);
  }
  Mat lift = mul(v, mul(vt, e));
  o.Dr = dr.a;
  o.Ds = ds.a;
  o.Drw = drw.a;
  o.Dsw = dsw.a;
  o.LIFT = lift.a;
  return 0;
}

}  // namespace dg
