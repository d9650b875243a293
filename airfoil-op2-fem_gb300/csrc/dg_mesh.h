// Unstructured triangle meshes in the connectivity the hot path consumes.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace dg {

struct Mesh {
  std::vector<double> coords;      // 2 * n_nodes {x, y}
  std::vector<int> cell2nodes;     // 3 * n_cells, counter-clockwise
  std::vector<int> edge2nodes;     // 2 * n_edges
  std::vector<int> edge2cells;     // 2 * n_edges
  std::vector<int> edgeNum;        // 2 * n_edges: local face index in each cell
  std::vector<int> bedge2nodes;    // 2 * n_bedges
  std::vector<int> bedge2cell;     // n_bedges
  std::vector<int> bedgeNum;       // n_bedges
  std::vector<int> bedge_type;     // n_bedges: 0 inflow, 1 outflow, 2 wall, 3 farfield
  int n_nodes() const { return (int)coords.size() / 2; }
  int n_cells() const { return (int)cell2nodes.size() / 3; }
  int n_edges() const { return (int)edge2cells.size() / 2; }
  int n_bedges() const { return (int)bedge2cell.size(); }
};

// Reads a Gmsh legacy-ASCII VTK unstructured grid: the 3-point cells, with vertex ids 1<->2
// swapped as tools/vtk2CGNS.cpp:75-78 does.  Returns 0 or a negative error code.
int read_vtk(const std::string &path, std::vector<double> &coords, std::vector<int> &cells,
             std::string &err);

// Edge tables of tools/vtk2CGNS.cpp:112-199 and src/load_mesh.cpp:96-146: fixes clockwise
// cells by swapping vertices 0 and 2; face j of a cell joins vertices j and j+1 (mod 3);
// edges are ordered by their sorted vertex pair; the first cell (in cell order) to claim an
// edge is side 0.  Interior edges and boundary edges are split in that order.
int build_tables(Mesh &m, std::string &err);

// The same tables built on the GPU (dg_mesh_device.cu); bit-identical to build_tables.
// device_ms (optional) receives the device time of the build, copies excluded.
int build_tables_device(Mesh &m, float *device_ms, std::string &err);

// Boundary typing of src/load_mesh.cpp:147-171 for the reference's rectangular Gmsh box.
int classify_box(Mesh &m, std::string &err);

// O-grid around NACA 0012 (n_theta around, n_r layers); farfield: 0 = inflow/outflow by face
// midpoint x < 0, 1 = characteristic farfield (type 3).  The inner ring is a wall.
int naca_ogrid(int n_theta, int n_r, double stretch, double radius, int farfield, Mesh &m,
               std::string &err);

// [lo,hi]^2 in n x n squares, each cut along a diagonal drawn from std::mt19937_64(seed).
int vortex_square(int n, double lo, double hi, uint64_t seed, Mesh &m, std::string &err);

// The batched sweep: n instances, alpha ~ U[-4, 8] deg and Mach ~ U[0.3, 0.6] drawn from
// std::mt19937_64(seed) (53-bit uniforms, alpha then Mach per instance), O-grids running
// linearly from 128 x 32 to 384 x 96, order 3 for even and 4 for odd instances.
void sweep_config(int n, uint64_t seed, int *n_theta, int *n_r, int *order, double *alpha_deg, double *mach);

// Legacy-VTK (ASCII) unstructured grid with per-vertex scalars rho, p and vector velocity: the
// fields src/save_solution.cpp:48-98 writes to CGNS.
int write_vtk(const std::string &path, const Mesh &m, const double *rho, const double *u, const double *v,
              const double *p, std::string &err);
// The same grid with one per-vertex scalar (the advection app's q, advec/src/save_solution.cpp).
int write_vtk_scalar(const std::string &path, const Mesh &m, const char *name, const double *values,
                     std::string &err);

// Checks ranges and that every (cell, face) slot is covered by exactly one edge or boundary
// edge.  The hot path depends on this single-writer property.
int validate(const Mesh &m, std::string &err);

}  // namespace dg
