"""CPU reference for the standalone pressure-equation solves (test infrastructure).

The operator is the one PressureSolver.h:318-495 relaxes, assembled as a sparse matrix over the interior P
unknowns (i = 1..im-2, j = 1..jm-2, k = 0..km-2) with the boundary planes of :718-746 folded into the rows
next to them (p0 = c43 p1 - c13 p2 in r and theta) and the periodic seam in phi. The weights follow the
solver's own geometry: num1 = 1/dr^2, num2 = 1/(rm^2 dtheta^2), num3 = 1/(rm^2 sin^2 dphi^2) with the
exact-zero sine guard 1e-5 (PressureSolver.h:156-162, 349-353), den = 2 (num1 + num2 + num3).
"""
from __future__ import annotations

import numpy as np

C43, C13 = 4.0 / 3.0, 1.0 / 3.0


def weights(g, P):
    R_km = P["metric_radius_km"]
    rm = g.rad_z + (R_km / P["L_atm"] - 1.0) if R_km > 0 else g.rad_z.copy()
    sp = np.sin(g.the_z)
    sp = np.maximum(sp, P["sinthe_min"])
    sp = np.where(sp == 0.0, 1.0e-5, sp)
    inv_dr2, inv_dthe2, inv_dphi2 = 1.0 / (g.dr * g.dr), 1.0 / (g.dthe * g.dthe), 1.0 / (g.dphi * g.dphi)
    inv_rm2 = 1.0 / (rm * rm)
    num1 = np.full((g.im, g.jm), inv_dr2)
    num2 = (inv_rm2 * inv_dthe2)[:, None] * np.ones((1, g.jm))
    num3 = (inv_rm2[:, None] / (sp * sp)[None, :]) * inv_dphi2
    den = 2.0 * num1 + 2.0 * num2 + 2.0 * num3
    return num1, num2, num3, den


def matrix(g, P):
    import scipy.sparse as sps
    im, jm, km = g.shape
    n = km - 1
    NI, NJ = im - 2, jm - 2
    num1, num2, num3, den = weights(g, P)
    N = NI * NJ * n

    def idx(i, j, k):
        return ((i - 1) * NJ + (j - 1)) * n + (k % n)

    rows, cols, vals = [], [], []

    def add(r, i, j, k, v):
        # a reference to p[i][j][k], folded onto the unknowns
        if i == 0:
            add(r, 1, j, k, C43 * v); add(r, 2, j, k, -C13 * v); return
        if i == im - 1:
            add(r, im - 2, j, k, C43 * v); add(r, im - 3, j, k, -C13 * v); return
        if j == 0:
            add(r, i, 1, k, C43 * v); add(r, i, 2, k, -C13 * v); return
        if j == jm - 1:
            add(r, i, jm - 2, k, C43 * v); add(r, i, jm - 3, k, -C13 * v); return
        rows.append(r); cols.append(idx(i, j, k)); vals.append(v)

    for i in range(1, im - 1):
        for j in range(1, jm - 1):
            for k in range(n):
                r = idx(i, j, k)
                add(r, i + 1, j, k, num1[i, j]); add(r, i - 1, j, k, num1[i, j])
                add(r, i, j + 1, k, num2[i, j]); add(r, i, j - 1, k, num2[i, j])
                add(r, i, j, k + 1, num3[i, j]); add(r, i, j, k - 1 + n, num3[i, j])
                add(r, i, j, k, -den[i, j])
    return sps.csr_matrix((vals, (rows, cols)), shape=(N, N)), idx


def to_vec(g, a):
    n = g.km - 1
    return a[1:-1, 1:-1, :n].reshape(-1).copy()


def from_vec(g, v):
    n = g.km - 1
    out = np.zeros(g.shape)
    out[1:-1, 1:-1, :n] = v.reshape(g.im - 2, g.jm - 2, n)
    return out


def left_null(A):
    """y with y^T A = 0, normalised to y[0] = 1 (the transposed equation of unknown 0 replaced)."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    At = A.T.tolil()
    At[0, :] = 0.0
    At[0, 0] = 1.0
    b = np.zeros(A.shape[0])
    b[0] = 1.0
    return spla.spsolve(At.tocsc(), b)


def project(g, A, src):
    """src without its component along the left null vector's span (per phi-mean, as the solver does)."""
    y = left_null(A)
    f = to_vec(g, src)
    alpha = float(y @ f) / float(y @ y)
    out = src.copy()
    v = f - alpha * y
    out[1:-1, 1:-1, : g.km - 1] = v.reshape(g.im - 2, g.jm - 2, g.km - 1)
    return out, y


def solve(g, A, src):
    """The zero-mean solution of A p = src (src compatible): one unknown pinned, then shifted."""
    import scipy.sparse.linalg as spla
    B = A.tolil()
    B[0, :] = 0.0
    B[0, 0] = 1.0
    f = to_vec(g, src)
    f[0] = 0.0
    x = spla.spsolve(B.tocsc(), f)
    x -= x.mean()
    return x


def rel_residual(g, A, p, src):
    f = to_vec(g, src)
    r = f - A @ to_vec(g, p)
    return float(np.linalg.norm(r) / np.linalg.norm(f))
