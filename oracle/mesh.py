"""Oracle-side mesh construction — TEST INFRASTRUCTURE ONLY.

Independent restatement (numpy / pure Python) of how the reference builds the
connectivity its hot path consumes, used to check the product's C++ mesh
builder and to feed the CPU oracle:

* ``read_vtk``       Gmsh legacy-ASCII VTK reader; keeps the 3-point cells and
                     swaps vertex ids 1<->2 as tools/vtk2CGNS.cpp:75-78 does.
* ``build_tables``   tools/vtk2CGNS.cpp:112-199 — counter-clockwise fix
                     (:114-129), edge map keyed by the sorted vertex pair with
                     face j = (v_j, v_{j+1 mod 3}) (:130-177), split into interior
                     edges {p1,p2,c1,c2,num1,num2} and boundary edges
                     {p1,p2,c,num} in key order (:179-199), 0-based as
                     src/load_mesh.cpp:112-146 stores them.
* ``classify_box``   src/load_mesh.cpp:147-171 (0 inflow, 1 outflow, 2 wall).
* ``naca_ogrid`` / ``vortex_square``  the synthetic meshes of the airfoil and
                     vortex benchmark cases (no reference counterpart; their
                     definition is written out in the docstrings).
"""
from __future__ import annotations

import math

import numpy as np

MASK64 = (1 << 64) - 1


class MT19937_64:
    """64-bit Mersenne Twister (Nishimura & Matsumoto 2004), the engine the C++
    standard specifies as std::mt19937_64."""

    def __init__(self, seed: int):
        self.mt = [0] * 312
        self.mt[0] = seed & MASK64
        for i in range(1, 312):
            prev = self.mt[i - 1]
            self.mt[i] = (6364136223846793005 * (prev ^ (prev >> 62)) + i) & MASK64
        self.idx = 312

    def _twist(self):
        mt = self.mt
        for i in range(312):
            x = (mt[i] & 0xFFFFFFFF80000000) | (mt[(i + 1) % 312] & 0x7FFFFFFF)
            xa = x >> 1
            if x & 1:
                xa ^= 0xB5026F5AA96619E9
            mt[i] = mt[(i + 156) % 312] ^ xa
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= 312:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= (y >> 29) & 0x5555555555555555
        y ^= (y << 17) & 0x71D67FFFEDA60000
        y ^= (y << 37) & 0xFFF7EEE000000000
        y ^= y >> 43
        return y & MASK64


def read_vtk(path):
    """Gmsh legacy VTK (ASCII, UNSTRUCTURED_GRID) -> (coords[n,2], cells[k,3]) with the
    1<->2 vertex swap of tools/vtk2CGNS.cpp:75-78."""
    with open(path) as f:
        tok = f.read().split()
    i = tok.index("POINTS")
    npts = int(tok[i + 1])
    pts = np.array(tok[i + 3:i + 3 + 3 * npts], dtype=np.float64).reshape(npts, 3)
    j = tok.index("CELLS", i)
    ncells = int(tok[j + 1])
    p = j + 3
    cells = []
    used = set()
    for _ in range(ncells):
        k = int(tok[p])
        ids = [int(t) for t in tok[p + 1:p + 1 + k]]
        p += 1 + k
        if k == 3:
            cells.append([ids[0], ids[2], ids[1]])
            used.update(ids)
    if len(used) != npts:
        raise ValueError("VTK file has points not used by any triangle; ids would shift")
    return pts[:, :2].copy(), np.array(cells, dtype=np.int32)


def build_tables(coords, cells):
    """tools/vtk2CGNS.cpp:112-199 + src/load_mesh.cpp:96-146 -> dict of int32 arrays."""
    x = coords[:, 0]
    y = coords[:, 1]
    cells = np.array(cells, dtype=np.int32).copy()
    for i in range(cells.shape[0]):
        p1, p2, p3 = cells[i]
        val = (x[p2] - x[p1]) * (y[p3] - y[p2]) - (y[p2] - y[p1]) * (x[p3] - x[p2])
        if val < 0:
            cells[i, 0], cells[i, 2] = p3, p1
    emap = {}
    for i in range(cells.shape[0]):
        for j in range(3):
            p1 = int(cells[i, j])
            p2 = int(cells[i, (j + 1) % 3])
            key = (p1, p2) if p1 < p2 else (p2, p1)
            e = emap.get(key)
            if e is None:
                emap[key] = [i, -1, j, -1]
            else:
                if e[1] != -1:
                    raise ValueError("edge %s shared by more than two cells" % (key,))
                e[1] = i
                e[3] = j
    edges, bedges = [], []
    for key in sorted(emap):
        c0, c1, n0, n1 = emap[key]
        if c1 == -1:
            bedges.append((key[0], key[1], c0, n0))
        else:
            edges.append((key[0], key[1], c0, c1, n0, n1))
    edges = np.array(edges, dtype=np.int32).reshape(-1, 6)
    bedges = np.array(bedges, dtype=np.int32).reshape(-1, 4)
    return {
        "coords": np.ascontiguousarray(coords, dtype=np.float64),
        "cell2nodes": cells,
        "edge2nodes": np.ascontiguousarray(edges[:, 0:2]),
        "edge2cells": np.ascontiguousarray(edges[:, 2:4]),
        "edgeNum": np.ascontiguousarray(edges[:, 4:6]),
        "bedge2nodes": np.ascontiguousarray(bedges[:, 0:2]),
        "bedge2cell": np.ascontiguousarray(bedges[:, 2]),
        "bedgeNum": np.ascontiguousarray(bedges[:, 3]),
    }


def classify_box(mesh):
    """src/load_mesh.cpp:147-171 boundary types for the shipped Gmsh box mesh."""
    c = mesh["coords"]
    out = np.full(mesh["bedge2cell"].shape[0], -1, dtype=np.int32)
    for i, (a, b) in enumerate(mesh["bedge2nodes"]):
        x1, y1 = c[a]
        x2, y2 = c[b]
        if -1.0 < x1 < 2.0 and -1.0 < y1 < 1.0 and -1.0 < x2 < 2.0 and -1.0 < y2 < 1.0:
            out[i] = 2
        elif y1 == y2:
            out[i] = 2
        elif x1 == x2:
            out[i] = 0 if x1 < 0.0 else 1
        else:
            raise ValueError("unclassified boundary edge %d" % i)
    return out


def naca_thickness(x):
    """Closed-trailing-edge NACA 0012 half thickness, the polynomial of naca0012.geo:14."""
    return 0.594689181 * (0.298222773 * math.sqrt(x) - 0.127125232 * x - 0.357907906 * (x * x) +
                          0.291984971 * (x * x * x) - 0.105174696 * (x * x * x * x))


def naca_ogrid(n_theta=256, n_r=64, stretch=1.1, radius=20.0, farfield="reference"):
    """O-grid around NACA 0012.

    Node (k, j), k = 0..n_theta-1 around (periodic), j = 0..n_r outward, id = j*n_theta + k.
    Surface (j=0): phi = 2*pi*k/n_theta, x = (1 + cos phi)/2, y = +-max(t(x), 0) (+ for
    phi <= pi).  Far ring (j=n_r): (0.5, 0) + radius*(cos phi, sin phi).  Ring j lies at the
    fraction d_j = (stretch^j - 1)/(stretch^n_r - 1) of the straight line from the surface
    point to the far point.  Quad (k, j) gives the triangles
    [(k,j), (k,j+1), (k+1,j)] and [(k+1,j), (k,j+1), (k+1,j+1)], in (j, k) row-major order.
    Boundary types: inner ring 2 (wall); outer ring 0/1 by face-midpoint x < 0 ("reference",
    after src/load_mesh.cpp:159-165) or 3 (characteristic farfield).
    """
    nodes = np.zeros(((n_r + 1) * n_theta, 2))
    denom = stretch ** n_r - 1.0
    for k in range(n_theta):
        phi = 2.0 * math.pi * k / n_theta
        xs = 0.5 * (1.0 + math.cos(phi))
        yt = max(naca_thickness(xs), 0.0)
        ys = yt if k <= n_theta // 2 else -yt
        xf = 0.5 + radius * math.cos(phi)
        yf = radius * math.sin(phi)
        for j in range(n_r + 1):
            d = (stretch ** j - 1.0) / denom
            nodes[j * n_theta + k] = (xs + (xf - xs) * d, ys + (yf - ys) * d)
    cells = []
    for j in range(n_r):
        for k in range(n_theta):
            k1 = (k + 1) % n_theta
            a, b = j * n_theta + k, j * n_theta + k1
            c, d = (j + 1) * n_theta + k, (j + 1) * n_theta + k1
            cells.append((a, c, b))
            cells.append((b, c, d))
    mesh = build_tables(nodes, np.array(cells, dtype=np.int32))
    btype = np.zeros(mesh["bedge2cell"].shape[0], dtype=np.int32)
    for i, (p, q) in enumerate(mesh["bedge2nodes"]):
        if p < n_theta and q < n_theta:
            btype[i] = 2
        else:
            xm = 0.5 * (nodes[p, 0] + nodes[q, 0])
            btype[i] = 3 if farfield == "characteristic" else (0 if xm < 0.0 else 1)
    mesh["bedge_type"] = btype
    return mesh


def vortex_square(n=32, lo=-5.0, hi=5.0, seed=20261203):
    """Square [lo,hi]^2 in n x n squares, each cut along a diagonal drawn from
    std::mt19937_64(seed): node (i, j) at (lo + (hi-lo)*i/n, lo + (hi-lo)*j/n), id j*(n+1)+i;
    squares in row-major (j, i) order draw b = rng() >> 63; b == 0 cuts (i,j)-(i+1,j+1) into
    [(i,j),(i+1,j),(i+1,j+1)], [(i,j),(i+1,j+1),(i,j+1)]; b == 1 cuts (i+1,j)-(i,j+1) into
    [(i,j),(i+1,j),(i,j+1)], [(i+1,j),(i+1,j+1),(i,j+1)].  All boundary edges take the
    analytic vortex state (type 0 placeholder)."""
    rng = MT19937_64(seed)
    m = n + 1
    nodes = np.zeros((m * m, 2))
    for j in range(m):
        for i in range(m):
            nodes[j * m + i] = (lo + (hi - lo) * i / n, lo + (hi - lo) * j / n)
    cells = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * m + i, j * m + i + 1, (j + 1) * m + i, (j + 1) * m + i + 1
            if (rng() >> 63) == 0:
                cells += [(a, b, d), (a, d, c)]
            else:
                cells += [(a, b, c), (b, d, c)]
    mesh = build_tables(nodes, np.array(cells, dtype=np.int32))
    mesh["bedge_type"] = np.zeros(mesh["bedge2cell"].shape[0], dtype=np.int32)
    return mesh
