"""Oracle-side nodal DG operators on the reference triangle (test infrastructure only).

This module is part of the CPU oracle: only tests, the smoke check and the CPU
baseline leg of the benchmark may import it.  It restates, in numpy, the
published construction of Hesthaven & Warburton, *Nodal Discontinuous Galerkin
Methods* (Springer 2008), ch. 6 and appendix A (JacobiP, JacobiGL, Warpfactor,
Nodes2D, xytors, Simplex2DP, GradSimplex2DP, Vandermonde2D, Dmatrices2D, Lift2D),
which is how the reference's N=4 tables were produced:

* node coordinates   -> src/constants/constant_r.h, constant_s.h
* Dr, Ds             -> src/constants/constant_Dr.h, constant_Ds.h
* Drw, Dsw (weak)    -> src/constants/constant_Drw.h, constant_Dsw.h
                        Drw = (V Vr^T)(V V^T)^-1, Dsw = (V Vs^T)(V V^T)^-1
* LIFT               -> src/constants/constant_LIFT.h  (Np x 3Nfp)
* FMASK              -> src/constants/constant_util.h:15
  face 0: s=-1 with r increasing; face 1: r+s=0 from vertex 1 to vertex 2;
  face 2: r=-1 from vertex 2 back to vertex 0 (reversed w.r.t. node order).

It is deliberately independent of the product's C++ generator so that each
checks the other.
"""
from __future__ import annotations

import math
from functools import lru_cache

import numpy as np

# Warp & Blend optimised blending parameters, Hesthaven & Warburton table 6.1.
_ALPHA_OPT = [0.0000, 0.0000, 1.4152, 0.1001, 0.2751, 0.9800, 1.0999,
              1.2832, 1.3648, 1.4773, 1.4959, 1.5743, 1.5770, 1.6223, 1.6258]
NODETOL = 1e-12


def jacobi_p(x, alpha, beta, n):
    """Orthonormal Jacobi polynomial P_n^(alpha,beta)(x) (H&W appendix A, JacobiP)."""
    x = np.asarray(x, dtype=np.float64)
    pl = np.zeros((n + 1, x.size))
    gamma0 = 2 ** (alpha + beta + 1) / (alpha + beta + 1) * math.gamma(alpha + 1) * \
        math.gamma(beta + 1) / math.gamma(alpha + beta + 1)
    pl[0] = 1.0 / math.sqrt(gamma0)
    if n == 0:
        return pl[0]
    gamma1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * gamma0
    pl[1] = ((alpha + beta + 2) * x / 2 + (alpha - beta) / 2) / math.sqrt(gamma1)
    if n == 1:
        return pl[1]
    aold = 2 / (2 + alpha + beta) * math.sqrt((alpha + 1) * (beta + 1) / (alpha + beta + 3))
    for i in range(1, n):
        h1 = 2 * i + alpha + beta
        anew = 2 / (h1 + 2) * math.sqrt((i + 1) * (i + 1 + alpha + beta) * (i + 1 + alpha) *
                                        (i + 1 + beta) / (h1 + 1) / (h1 + 3))
        bnew = -(alpha ** 2 - beta ** 2) / h1 / (h1 + 2)
        pl[i + 1] = 1 / anew * (-aold * pl[i - 1] + (x - bnew) * pl[i])
        aold = anew
    return pl[n]


def grad_jacobi_p(x, alpha, beta, n):
    if n == 0:
        return np.zeros(np.asarray(x).size)
    return math.sqrt(n * (n + alpha + beta + 1)) * jacobi_p(x, alpha + 1, beta + 1, n - 1)


def jacobi_gq(alpha, beta, n):
    """Gauss quadrature nodes of P^(alpha,beta)_{n+1} (Golub-Welsch)."""
    if n == 0:
        return np.array([-(alpha - beta) / (alpha + beta + 2)])
    h1 = 2 * np.arange(n + 1) + alpha + beta
    je = np.diag(-0.5 * (alpha ** 2 - beta ** 2) / (h1 + 2) / h1)
    k = np.arange(1, n + 1)
    off = 2 / (h1[:n] + 2) * np.sqrt(k * (k + alpha + beta) * (k + alpha) * (k + beta) /
                                      (h1[:n] + 1) / (h1[:n] + 3))
    je = je + np.diag(off, 1)
    if alpha + beta < 10 * np.finfo(float).eps:
        je[0, 0] = 0.0
    je = je + je.T
    return np.sort(np.linalg.eigvalsh(je))


def jacobi_gl(alpha, beta, n):
    """Gauss-Lobatto nodes (H&W JacobiGL)."""
    if n == 1:
        return np.array([-1.0, 1.0])
    inner = jacobi_gq(alpha + 1, beta + 1, n - 2)
    return np.concatenate([[-1.0], inner, [1.0]])


def vandermonde_1d(n, r):
    return np.stack([jacobi_p(r, 0, 0, j) for j in range(n + 1)], axis=1)


def warpfactor(n, rout):
    lgl = jacobi_gl(0, 0, n)
    req = np.linspace(-1, 1, n + 1)
    veq = vandermonde_1d(n, req)
    nr = rout.size
    pmat = np.stack([jacobi_p(rout, 0, 0, i) for i in range(n + 1)])
    lmat = np.linalg.solve(veq.T, pmat)
    warp = lmat.T @ (lgl - req)
    zerof = (np.abs(rout) < 1.0 - 1.0e-10)
    sf = 1.0 - (zerof * rout) ** 2
    return warp / sf + warp * (zerof - 1)


def nodes_2d(n):
    alpha = _ALPHA_OPT[n - 1] if n < 16 else 5.0 / 3.0
    np_ = (n + 1) * (n + 2) // 2
    l1 = np.zeros(np_)
    l3 = np.zeros(np_)
    sk = 0
    for i in range(1, n + 2):
        for j in range(1, n + 3 - i):
            l1[sk] = (i - 1) / n
            l3[sk] = (j - 1) / n
            sk += 1
    l2 = 1.0 - l1 - l3
    x = -l2 + l3
    y = (-l2 - l3 + 2 * l1) / math.sqrt(3.0)
    blend1 = 4 * l2 * l3
    blend2 = 4 * l1 * l3
    blend3 = 4 * l1 * l2
    warpf1 = warpfactor(n, l3 - l2)
    warpf2 = warpfactor(n, l1 - l3)
    warpf3 = warpfactor(n, l2 - l1)
    warp1 = blend1 * warpf1 * (1 + (alpha * l1) ** 2)
    warp2 = blend2 * warpf2 * (1 + (alpha * l2) ** 2)
    warp3 = blend3 * warpf3 * (1 + (alpha * l3) ** 2)
    x = x + warp1 + math.cos(2 * math.pi / 3) * warp2 + math.cos(4 * math.pi / 3) * warp3
    y = y + 0 * warp1 + math.sin(2 * math.pi / 3) * warp2 + math.sin(4 * math.pi / 3) * warp3
    return x, y


def xy_to_rs(x, y):
    l1 = (math.sqrt(3.0) * y + 1.0) / 3.0
    l2 = (-3.0 * x - math.sqrt(3.0) * y + 2.0) / 6.0
    l3 = (3.0 * x - math.sqrt(3.0) * y + 2.0) / 6.0
    return -l2 + l3 - l1, -l2 - l3 + l1


def rs_to_ab(r, s):
    a = np.where(s != 1.0, 2 * (1 + r) / np.where(s != 1.0, 1 - s, 1.0) - 1, -1.0)
    return a, s.copy()


def simplex_2dp(a, b, i, j):
    h1 = jacobi_p(a, 0, 0, i)
    h2 = jacobi_p(b, 2 * i + 1, 0, j)
    return math.sqrt(2.0) * h1 * h2 * (1 - b) ** i


def grad_simplex_2dp(a, b, i, j):
    fa = jacobi_p(a, 0, 0, i)
    dfa = grad_jacobi_p(a, 0, 0, i)
    gb = jacobi_p(b, 2 * i + 1, 0, j)
    dgb = grad_jacobi_p(b, 2 * i + 1, 0, j)
    dmodedr = dfa * gb
    if i > 0:
        dmodedr = dmodedr * ((0.5 * (1 - b)) ** (i - 1))
    dmodeds = dfa * (gb * (0.5 * (1 + a)))
    if i > 0:
        dmodeds = dmodeds * ((0.5 * (1 - b)) ** (i - 1))
    tmp = dgb * ((0.5 * (1 - b)) ** i)
    if i > 0:
        tmp = tmp - 0.5 * i * gb * ((0.5 * (1 - b)) ** (i - 1))
    dmodeds = dmodeds + fa * tmp
    dmodedr = 2 ** (i + 0.5) * dmodedr
    dmodeds = 2 ** (i + 0.5) * dmodeds
    return dmodedr, dmodeds


def vandermonde_2d(n, r, s):
    a, b = rs_to_ab(r, s)
    cols = []
    for i in range(n + 1):
        for j in range(n - i + 1):
            cols.append(simplex_2dp(a, b, i, j))
    return np.stack(cols, axis=1)


def grad_vandermonde_2d(n, r, s):
    a, b = rs_to_ab(r, s)
    vr, vs = [], []
    for i in range(n + 1):
        for j in range(n - i + 1):
            dr, ds = grad_simplex_2dp(a, b, i, j)
            vr.append(dr)
            vs.append(ds)
    return np.stack(vr, axis=1), np.stack(vs, axis=1)


@lru_cache(maxsize=None)
def operators(n: int):
    """All nodal operators of order n as a dict of float64 arrays (row-major)."""
    x, y = nodes_2d(n)
    r, s = xy_to_rs(x, y)
    npts = (n + 1) * (n + 2) // 2
    nfp = n + 1
    v = vandermonde_2d(n, r, s)
    vr, vs = grad_vandermonde_2d(n, r, s)
    vinv = np.linalg.inv(v)
    dr = vr @ vinv
    ds = vs @ vinv
    vvt_inv = np.linalg.inv(v @ v.T)
    drw = (v @ vr.T) @ vvt_inv
    dsw = (v @ vs.T) @ vvt_inv
    f0 = np.nonzero(np.abs(s + 1) < NODETOL)[0]
    f1 = np.nonzero(np.abs(r + s) < NODETOL)[0]
    f2 = np.nonzero(np.abs(r + 1) < NODETOL)[0][::-1]
    fmask = np.concatenate([f0, f1, f2]).astype(np.int32)
    emat = np.zeros((npts, 3 * nfp))
    for f, (idx, coord) in enumerate(((f0, r), (f1, r), (f2, s))):
        v1 = vandermonde_1d(n, coord[idx])
        emat[idx, f * nfp:(f + 1) * nfp] = np.linalg.inv(v1 @ v1.T)
    lift = v @ (v.T @ emat)
    return {
        "N": n, "Np": npts, "Nfp": nfp, "r": r, "s": s, "Dr": dr, "Ds": ds,
        "Drw": drw, "Dsw": dsw, "LIFT": lift, "FMASK": fmask,
    }
