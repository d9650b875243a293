// A C++ application of the OP2 drop-in (include/op2_gb300.h): the airfoil app's declarations
// and loop sequence (src/airfoil.cpp:135-334) written against the OP2 API, with op_arg passed
// by value exactly as a translated driver (src/airfoil_op.cpp) passes it: what a user who links
// libdg_gb300.so in place of an OP2 backend runs.  Reads a mesh, operator tables and freestream
// constants from a binary file (dropin_app.py writes it), runs `iters` SSPRK3 steps, writes q
// and the dt of each step, and prints its wall-clock times: from the first declaration (host
// arrays in) to op_fetch_data (q out), and of the step loop alone.
//
//   dropin_airfoil <input> <output>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "op2_gb300.h"

namespace {

template <class T>
void read_into(FILE *f, std::vector<T> &v, size_t n) {
  v.resize(n);
  if (n && std::fread(v.data(), sizeof(T), n, f) != n) {
    std::fprintf(stderr, "short input\n");
    std::exit(2);
  }
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s input output\n", argv[0]);
    return 2;
  }
  FILE *in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  std::vector<int> hdr;
  read_into(in, hdr, 6);
  const int nn = hdr[0], nc = hdr[1], ne = hdr[2], nb = hdr[3], N = hdr[4], iters = hdr[5];
  const int Np = (N + 1) * (N + 2) / 2, Nfp = N + 1;
  std::vector<double> coords, phys, r, s, Dr, Ds, Drw, Dsw, LIFT;
  std::vector<int> cell2nodes, edge2cells, edgeNum, bedge2cell, bedgeNum, bedge_type, FMASK;
  read_into(in, coords, 2 * (size_t)nn);
  read_into(in, cell2nodes, 3 * (size_t)nc);
  read_into(in, edge2cells, 2 * (size_t)ne);
  read_into(in, edgeNum, 2 * (size_t)ne);
  read_into(in, bedge2cell, nb);
  read_into(in, bedgeNum, nb);
  read_into(in, bedge_type, nb);
  read_into(in, phys, 8);  // gam, bc_mach, bc_alpha, bc_p, bc_r, bc_u, bc_v, bc_e
  read_into(in, r, Np);
  read_into(in, s, Np);
  read_into(in, Dr, (size_t)Np * Np);
  read_into(in, Ds, (size_t)Np * Np);
  read_into(in, Drw, (size_t)Np * Np);
  read_into(in, Dsw, (size_t)Np * Np);
  read_into(in, LIFT, (size_t)Np * 3 * Nfp);
  read_into(in, FMASK, 3 * (size_t)Nfp);
  std::fclose(in);

  using clk = std::chrono::steady_clock;
  const auto t_begin = clk::now();
  op_init(argc, argv, 2);
  op_set nodes = op_decl_set(nn, "nodes");
  op_set cells = op_decl_set(nc, "cells");
  op_set edges = op_decl_set(ne, "edges");
  op_set bedges = op_decl_set(nb, "bedges");
  op_map cell2nodes_m = op_decl_map(cells, nodes, 3, cell2nodes.data(), "cell2nodes");
  op_map edge2cells_m = op_decl_map(edges, cells, 2, edge2cells.data(), "edge2cells");
  op_map bedge2cells_m = op_decl_map(bedges, cells, 1, bedge2cell.data(), "bedge2cells");
  op_dat node_coords = op_decl_dat(nodes, 2, "double", coords.data(), "node_coords");
  auto cell_dat = [&](int dim, const char *name) {
    std::vector<double> zero((size_t)nc * dim, 0.0);
    return op_decl_dat(cells, dim, "double", zero.data(), name);  // copied to the device
  };
  op_dat nodeX = cell_dat(3, "nodeX"), nodeY = cell_dat(3, "nodeY");
  op_dat x = cell_dat(Np, "x"), y = cell_dat(Np, "y");
  op_dat xr = cell_dat(Np, "xr"), yr = cell_dat(Np, "yr"), xs = cell_dat(Np, "xs"), ys = cell_dat(Np, "ys");
  op_dat rx = cell_dat(Np, "rx"), ry = cell_dat(Np, "ry"), sx = cell_dat(Np, "sx"), sy = cell_dat(Np, "sy");
  op_dat nx = cell_dat(3 * Nfp, "nx"), ny = cell_dat(3 * Nfp, "ny"), fscale = cell_dat(3 * Nfp, "fscale");
  op_dat q = cell_dat(4 * Np, "q"), workingQ = cell_dat(4 * Np, "workingQ");
  op_dat rk[3] = {cell_dat(4 * Np, "rk1"), cell_dat(4 * Np, "rk2"), cell_dat(4 * Np, "rk3")};
  op_dat exteriorQ = cell_dat(12 * Nfp, "exteriorQ");
  op_dat bedge_type_d = op_decl_dat(bedges, 1, "int", bedge_type.data(), "bedge_type");
  op_dat edgeNum_d = op_decl_dat(edges, 2, "int", edgeNum.data(), "edgeNum");
  op_dat bedgeNum_d = op_decl_dat(bedges, 1, "int", bedgeNum.data(), "bedgeNum");

  const char *pnames[8] = {"gam", "bc_mach", "bc_alpha", "bc_p", "bc_r", "bc_u", "bc_v", "bc_e"};
  for (int k = 0; k < 8; k++) op_decl_const2(pnames[k], 1, "double", &phys[k]);
  std::vector<double> ones(Np, 1.0);
  op_decl_const2("ones", Np, "double", ones.data());
  op_decl_const2("r", Np, "double", r.data());
  op_decl_const2("s", Np, "double", s.data());
  op_decl_const2("Dr", Np * Np, "double", Dr.data());
  op_decl_const2("Ds", Np * Np, "double", Ds.data());
  op_decl_const2("Drw", Np * Np, "double", Drw.data());
  op_decl_const2("Dsw", Np * Np, "double", Dsw.data());
  op_decl_const2("LIFT", Np * 3 * Nfp, "double", LIFT.data());
  op_decl_const2("FMASK", 3 * Nfp, "int", FMASK.data());

  const int d4 = 4 * Np, f12 = 12 * Nfp, f3 = 3 * Nfp;
  op_par_loop_init_grid("init_grid", cells,
                        op_arg_dat(node_coords, 0, cell2nodes_m, 2, "double", OP_READ),
                        op_arg_dat(node_coords, 1, cell2nodes_m, 2, "double", OP_READ),
                        op_arg_dat(node_coords, 2, cell2nodes_m, 2, "double", OP_READ),
                        op_arg_dat(nodeX, -1, OP_ID, 3, "double", OP_WRITE),
                        op_arg_dat(nodeY, -1, OP_ID, 3, "double", OP_WRITE),
                        op_arg_dat(x, -1, OP_ID, Np, "double", OP_WRITE), op_arg_dat(y, -1, OP_ID, Np, "double", OP_WRITE),
                        op_arg_dat(xr, -1, OP_ID, Np, "double", OP_WRITE), op_arg_dat(yr, -1, OP_ID, Np, "double", OP_WRITE),
                        op_arg_dat(xs, -1, OP_ID, Np, "double", OP_WRITE), op_arg_dat(ys, -1, OP_ID, Np, "double", OP_WRITE),
                        op_arg_dat(rx, -1, OP_ID, Np, "double", OP_WRITE), op_arg_dat(ry, -1, OP_ID, Np, "double", OP_WRITE),
                        op_arg_dat(sx, -1, OP_ID, Np, "double", OP_WRITE), op_arg_dat(sy, -1, OP_ID, Np, "double", OP_WRITE),
                        op_arg_dat(nx, -1, OP_ID, f3, "double", OP_WRITE), op_arg_dat(ny, -1, OP_ID, f3, "double", OP_WRITE),
                        op_arg_dat(fscale, -1, OP_ID, f3, "double", OP_WRITE));
  op_par_loop_set_ic("set_ic", cells, op_arg_dat(q, -1, OP_ID, d4, "double", OP_WRITE),
                     op_arg_dat(workingQ, -1, OP_ID, d4, "double", OP_WRITE));
  op_par_loop_neighbour_zero("neighbour_zero", cells, op_arg_dat(exteriorQ, -1, OP_ID, f12, "double", OP_WRITE));
  auto calc_dt = [&]() {
    double dt1 = 0.0;
    op_par_loop_calc_dt("calc_dt", cells, op_arg_dat(q, -1, OP_ID, d4, "double", OP_READ),
                        op_arg_dat(fscale, -1, OP_ID, f3, "double", OP_READ), op_arg_gbl(&dt1, 1, "double", OP_MAX));
    return 1.0 / dt1;
  };
  double dt = calc_dt();
  std::vector<double> dts;
  const auto t_steps = clk::now();  // calc_dt's OP_MAX returned: the set-up loops are done
  for (int it = 0; it < iters; it++) {
    dts.push_back(dt);
    for (int j = 0; j < 3; j++) {
      op_par_loop_get_neighbour_q("get_neighbour_q", edges, op_arg_dat(edgeNum_d, -1, OP_ID, 2, "int", OP_READ),
                                  op_arg_dat(nodeX, 0, edge2cells_m, 3, "double", OP_READ),
                                  op_arg_dat(nodeY, 0, edge2cells_m, 3, "double", OP_READ),
                                  op_arg_dat(nodeX, 1, edge2cells_m, 3, "double", OP_READ),
                                  op_arg_dat(nodeY, 1, edge2cells_m, 3, "double", OP_READ),
                                  op_arg_dat(workingQ, 0, edge2cells_m, d4, "double", OP_READ),
                                  op_arg_dat(workingQ, 1, edge2cells_m, d4, "double", OP_READ),
                                  op_arg_dat(exteriorQ, 0, edge2cells_m, f12, "double", OP_INC),
                                  op_arg_dat(exteriorQ, 1, edge2cells_m, f12, "double", OP_INC));
      op_par_loop_get_bedge_q("get_bedge_q", bedges, op_arg_dat(bedge_type_d, -1, OP_ID, 1, "int", OP_READ),
                              op_arg_dat(bedgeNum_d, -1, OP_ID, 1, "int", OP_READ),
                              op_arg_dat(nx, 0, bedge2cells_m, f3, "double", OP_READ),
                              op_arg_dat(ny, 0, bedge2cells_m, f3, "double", OP_READ),
                              op_arg_dat(workingQ, 0, bedge2cells_m, d4, "double", OP_READ),
                              op_arg_dat(exteriorQ, 0, bedge2cells_m, f12, "double", OP_INC));
      op_par_loop_euler_rhs("euler_rhs", cells, op_arg_dat(workingQ, -1, OP_ID, d4, "double", OP_READ),
                            op_arg_dat(exteriorQ, -1, OP_ID, f12, "double", OP_RW),
                            op_arg_dat(rx, -1, OP_ID, Np, "double", OP_READ), op_arg_dat(ry, -1, OP_ID, Np, "double", OP_READ),
                            op_arg_dat(sx, -1, OP_ID, Np, "double", OP_READ), op_arg_dat(sy, -1, OP_ID, Np, "double", OP_READ),
                            op_arg_dat(fscale, -1, OP_ID, f3, "double", OP_READ),
                            op_arg_dat(nx, -1, OP_ID, f3, "double", OP_READ), op_arg_dat(ny, -1, OP_ID, f3, "double", OP_READ),
                            op_arg_dat(rk[j], -1, OP_ID, d4, "double", OP_WRITE));
      if (j != 2)
        op_par_loop_set_workingQ("set_workingQ", cells, op_arg_gbl(&dt, 1, "double", OP_READ),
                                 op_arg_gbl(&j, 1, "int", OP_READ), op_arg_dat(q, -1, OP_ID, d4, "double", OP_READ),
                                 op_arg_dat(rk[0], -1, OP_ID, d4, "double", OP_READ),
                                 op_arg_dat(rk[1], -1, OP_ID, d4, "double", OP_READ),
                                 op_arg_dat(workingQ, -1, OP_ID, d4, "double", OP_WRITE));
    }
    op_par_loop_update_Q("update_Q", cells, op_arg_gbl(&dt, 1, "double", OP_READ),
                         op_arg_dat(q, -1, OP_ID, d4, "double", OP_RW), op_arg_dat(rk[0], -1, OP_ID, d4, "double", OP_READ),
                         op_arg_dat(rk[1], -1, OP_ID, d4, "double", OP_READ),
                         op_arg_dat(rk[2], -1, OP_ID, d4, "double", OP_READ),
                         op_arg_dat(workingQ, -1, OP_ID, d4, "double", OP_WRITE));
    dt = calc_dt();
  }
  const auto t_loop_end = clk::now();  // the last calc_dt's OP_MAX returned: every step is done
  std::vector<double> qh((size_t)nc * d4);
  op_fetch_data(q, qh.data());
  const auto t_end = clk::now();
  op_timing_output();
  std::printf("dropin_timing total_s=%.9f steps_s=%.9f iters=%d\n",
              std::chrono::duration<double>(t_end - t_begin).count(),
              std::chrono::duration<double>(t_loop_end - t_steps).count(), iters);
  op_exit();
  FILE *out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  const bool ok = std::fwrite(qh.data(), 8, qh.size(), out) == qh.size() &&
                  std::fwrite(dts.data(), 8, dts.size(), out) == dts.size();
  std::fclose(out);
  return ok ? 0 : 3;
}
