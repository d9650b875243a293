// Nodal DG operators of the reference triangle (see dg_ops.cpp).
#pragma once
#include <vector>

namespace dg {

struct Operators {
  int N = 0, Np = 0, Nfp = 0;
  std::vector<double> r, s;        // Np
  std::vector<double> Dr, Ds;      // Np x Np, row-major
  std::vector<double> Drw, Dsw;    // Np x Np
  std::vector<double> LIFT;        // Np x 3Nfp
  std::vector<int> FMASK;          // 3Nfp
};

// 0 on success; N must be 1..6.
int build_operators(int N, Operators &out);

}  // namespace dg
