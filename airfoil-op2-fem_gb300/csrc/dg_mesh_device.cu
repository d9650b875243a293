// Edge tables built on the GPU (tools/vtk2CGNS.cpp:112-199, src/load_mesh.cpp:96-146): the same
// tables, bit for bit, as the host build_tables in dg_mesh.cpp, in a few sort and scan passes.
//
//   1. orient   one thread per cell: the clockwise test of vtk2CGNS.cpp:118-127 with the host's
//               rounding (no contraction), vertices 0 and 2 swapped when clockwise; the three
//               half-edges (face j joins vertices j and j+1) as key a * n_nodes + b (a < b) with
//               the value 3 * cell + face;
//   2. sort     a stable LSD radix sort of the keys (CUB): equal keys keep cell order, so the
//               first cell to claim an edge is its side 0, as the reference's map insert;
//   3. runs     one thread per sorted half-edge: a run of one key is a boundary edge, of two an
//               interior edge, longer runs are an error; heads are flagged (interior count in
//               the high 32 bits, boundary count in the low 32 bits of one 64-bit flag);
//   4. scan     one exclusive sum of the flags gives every edge its slot in both tables;
//   5. scatter  the heads write edge2nodes, edge2cells, edgeNum or the boundary tables.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <string>
#include <vector>

#include "dg_mesh.h"

namespace dg {
namespace {

typedef unsigned long long u64;

enum : unsigned { kErrRange = 1, kErrDegenerate = 2, kErrShared = 4, kErrSameCell = 8 };

__global__ void orient_kernel(int nc, int nn, const double *x, int *cells, u64 *keys, int *vals, unsigned *err) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nc) return;
  int p[3] = {cells[3 * c], cells[3 * c + 1], cells[3 * c + 2]};
  bool ok = true;
  for (int k = 0; k < 3; k++) ok = ok && p[k] >= 0 && p[k] < nn;
  if (!ok) {
    atomicOr(err, kErrRange);
    for (int j = 0; j < 3; j++) {
      keys[3 * (size_t)c + j] = 0;
      vals[3 * (size_t)c + j] = 3 * c + j;
    }
    return;
  }
  const double val = __dsub_rn(__dmul_rn(__dsub_rn(x[2 * p[1]], x[2 * p[0]]), __dsub_rn(x[2 * p[2] + 1], x[2 * p[1] + 1])),
                               __dmul_rn(__dsub_rn(x[2 * p[1] + 1], x[2 * p[0] + 1]), __dsub_rn(x[2 * p[2]], x[2 * p[1]])));
  if (val < 0) {
    const int t = p[0];
    p[0] = p[2];
    p[2] = t;
    cells[3 * c] = p[0];
    cells[3 * c + 2] = p[2];
  }
  for (int j = 0; j < 3; j++) {
    const int u = p[j], w = p[(j + 1) % 3];
    const int a = min(u, w), b = max(u, w);
    if (a == b) atomicOr(err, kErrDegenerate);
    keys[3 * (size_t)c + j] = (u64)a * (u64)nn + (u64)b;
    vals[3 * (size_t)c + j] = 3 * c + j;
  }
}

__global__ void runs_kernel(long long nh, const u64 *k, const int *v, u64 *flags, unsigned *err) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nh) return;
  if (p > 0 && k[p] == k[p - 1]) {
    flags[p] = 0;
    return;
  }
  if (p + 1 < nh && k[p + 1] == k[p]) {
    if (p + 2 < nh && k[p + 2] == k[p]) atomicOr(err, kErrShared);
    if (v[p] / 3 == v[p + 1] / 3) atomicOr(err, kErrSameCell);
    flags[p] = 1ull << 32;
  } else {
    flags[p] = 1ull;
  }
}

__global__ void scatter_kernel(long long nh, int nn, const u64 *k, const int *v, const u64 *flags, const u64 *pos,
                               int *e2n, int *e2c, int *enm, int *b2n, int *b2c, int *bnm) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nh || flags[p] == 0) return;
  const int a = (int)(k[p] / (u64)nn), b = (int)(k[p] % (u64)nn);
  if (flags[p] >> 32) {
    const long long i = (long long)(pos[p] >> 32);
    e2n[2 * i] = a;
    e2n[2 * i + 1] = b;
    e2c[2 * i] = v[p] / 3;
    e2c[2 * i + 1] = v[p + 1] / 3;
    enm[2 * i] = v[p] % 3;
    enm[2 * i + 1] = v[p + 1] % 3;
  } else {
    const long long i = (long long)(pos[p] & 0xffffffffull);
    b2n[2 * i] = a;
    b2n[2 * i + 1] = b;
    b2c[i] = v[p] / 3;
    bnm[i] = v[p] % 3;
  }
}

struct DeviceBuffers {
  std::vector<void *> ptrs;
  cudaStream_t s;
  explicit DeviceBuffers(cudaStream_t st) : s(st) {}
  ~DeviceBuffers() {
    for (void *p : ptrs) cudaFreeAsync(p, s);
    cudaStreamSynchronize(s);
  }
  template <class T>
  T *get(size_t n, cudaError_t &ce) {
    void *p = nullptr;
    if (ce == cudaSuccess) ce = cudaMallocAsync(&p, n ? n * sizeof(T) : 16, s);
    if (p) ptrs.push_back(p);
    return (T *)p;
  }
};

int bit_width(u64 v) {
  int b = 0;
  while (v) {
    b++;
    v >>= 1;
  }
  return b;
}

}  // namespace

int build_tables_device(Mesh &m, float *device_ms, std::string &err) {
  const int nc = m.n_cells(), nn = m.n_nodes();
  const long long nh = 3ll * nc;
  if (nc <= 0 || nn <= 0) { err = "empty mesh"; return -1; }
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) { err = "stream creation failed"; return -100; }
  cudaError_t ce = cudaSuccess;
  int rc = 0;
  {
    DeviceBuffers buf(s);
    double *x = buf.get<double>(2 * (size_t)nn, ce);
    int *cells = buf.get<int>(3 * (size_t)nc, ce);
    u64 *k0 = buf.get<u64>(nh, ce), *k1 = buf.get<u64>(nh, ce), *flags = buf.get<u64>(nh, ce), *pos = buf.get<u64>(nh, ce);
    int *v0 = buf.get<int>(nh, ce), *v1 = buf.get<int>(nh, ce);
    int *e2n = buf.get<int>(nh, ce), *e2c = buf.get<int>(nh, ce), *enm = buf.get<int>(nh, ce);
    int *b2n = buf.get<int>(2 * nh, ce), *b2c = buf.get<int>(nh, ce), *bnm = buf.get<int>(nh, ce);
    unsigned *derr = buf.get<unsigned>(1, ce);
    size_t sort_bytes = 0, scan_bytes = 0;
    const int end_bit = bit_width((u64)nn * (u64)nn);
    if (ce == cudaSuccess)
      ce = cub::DeviceRadixSort::SortPairs(nullptr, sort_bytes, k0, k1, v0, v1, (int)nh, 0, end_bit, s);
    if (ce == cudaSuccess) ce = cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, flags, pos, (int)nh, s);
    void *tmp = buf.get<char>(std::max(sort_bytes, scan_bytes), ce);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(x, m.coords.data(), 16 * (size_t)nn, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(cells, m.cell2nodes.data(), 12 * (size_t)nc, cudaMemcpyHostToDevice, s);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(derr, 0, 4, s);
    if (ce == cudaSuccess) ce = cudaEventRecord(e0, s);
    if (ce == cudaSuccess) {
      const unsigned gh = (unsigned)((nh + 255) / 256);
      orient_kernel<<<(nc + 255) / 256, 256, 0, s>>>(nc, nn, x, cells, k0, v0, derr);
      ce = cub::DeviceRadixSort::SortPairs(tmp, sort_bytes, k0, k1, v0, v1, (int)nh, 0, end_bit, s);
      if (ce == cudaSuccess) {
        runs_kernel<<<gh, 256, 0, s>>>(nh, k1, v1, flags, derr);
        ce = cub::DeviceScan::ExclusiveSum(tmp, scan_bytes, flags, pos, (int)nh, s);
      }
      if (ce == cudaSuccess) {
        scatter_kernel<<<gh, 256, 0, s>>>(nh, nn, k1, v1, flags, pos, e2n, e2c, enm, b2n, b2c, bnm);
        ce = cudaGetLastError();
      }
    }
    if (ce == cudaSuccess) ce = cudaEventRecord(e1, s);
    unsigned herr = 0;
    u64 last_pos = 0, last_flag = 0;
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&last_pos, pos + nh - 1, 8, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(&last_flag, flags + nh - 1, 8, cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce == cudaSuccess && device_ms) ce = cudaEventElapsedTime(device_ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (ce == cudaSuccess && herr) {
      err = (herr & kErrRange) ? "cell vertex out of range"
            : (herr & kErrDegenerate) ? "degenerate edge"
            : (herr & kErrShared) ? "edge shared by more than two cells"
                                  : "edge with identical cells";
      rc = -2;
    }
    if (ce == cudaSuccess && !rc) {
      const u64 tot = last_pos + last_flag;
      const int ne = (int)(tot >> 32), nb = (int)(tot & 0xffffffffull);
      m.edge2nodes.resize(2 * (size_t)ne);
      m.edge2cells.resize(2 * (size_t)ne);
      m.edgeNum.resize(2 * (size_t)ne);
      m.bedge2nodes.resize(2 * (size_t)nb);
      m.bedge2cell.resize(nb);
      m.bedgeNum.resize(nb);
      ce = cudaMemcpyAsync(m.cell2nodes.data(), cells, 12 * (size_t)nc, cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess && ne) ce = cudaMemcpyAsync(m.edge2nodes.data(), e2n, 8 * (size_t)ne, cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess && ne) ce = cudaMemcpyAsync(m.edge2cells.data(), e2c, 8 * (size_t)ne, cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess && ne) ce = cudaMemcpyAsync(m.edgeNum.data(), enm, 8 * (size_t)ne, cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess && nb) ce = cudaMemcpyAsync(m.bedge2nodes.data(), b2n, 8 * (size_t)nb, cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess && nb) ce = cudaMemcpyAsync(m.bedge2cell.data(), b2c, 4 * (size_t)nb, cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess && nb) ce = cudaMemcpyAsync(m.bedgeNum.data(), bnm, 4 * (size_t)nb, cudaMemcpyDeviceToHost, s);
      if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
      m.bedge_type.assign(nb, 2);
    }
  }
  cudaStreamDestroy(s);
  if (ce != cudaSuccess) {
    err = std::string("device edge build: ") + cudaGetErrorString(ce);
    return -100;
  }
  return rc;
}

}  // namespace dg
