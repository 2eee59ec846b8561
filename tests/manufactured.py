"""Manufactured smooth fields with a closed-form divergence of stress, for the
truncation-error checks of the elastic operators.

The reference checks its operator kernels this way (tests/testil/testil.C:186-200
fills u, mu, lambda from closed-form functions, :348-366 compares the operator with
the analytic rho * (div sigma) point by point).  The functions here are our own: each
displacement component and each Lame parameter is a constant plus a product of three
sines, so every first and second partial derivative is a product of sines and cosines
evaluated in numpy.

div sigma for an isotropic medium, sigma_ij = lambda delta_ij div u + mu (d_i u_j + d_j u_i):

    (div sigma)_i = d_i lambda * D + lambda * d_i D
                    + sum_j d_j mu (d_i u_j + d_j u_i) + mu sum_j (d_i d_j u_j + d_j d_j u_i),

with D = sum_j d_j u_j.
"""
from __future__ import annotations

import numpy as np


class SineProduct:
    """c + a * sin(kx x + px) sin(ky y + py) sin(kz z + pz): value, gradient, Hessian."""

    def __init__(self, c, a, k, p):
        self.c, self.a = c, a
        self.k = np.asarray(k, dtype=np.float64)
        self.p = np.asarray(p, dtype=np.float64)

    def _factors(self, xyz):
        s = [np.sin(self.k[d] * xyz[d] + self.p[d]) for d in range(3)]
        c = [self.k[d] * np.cos(self.k[d] * xyz[d] + self.p[d]) for d in range(3)]
        s2 = [-self.k[d] ** 2 * s[d] for d in range(3)]
        return s, c, s2

    def value(self, xyz):
        s, _, _ = self._factors(xyz)
        return self.c + self.a * s[0] * s[1] * s[2]

    def grad(self, xyz):
        s, c, _ = self._factors(xyz)
        return [self.a * c[0] * s[1] * s[2], self.a * s[0] * c[1] * s[2], self.a * s[0] * s[1] * c[2]]

    def hess(self, xyz):
        s, c, s2 = self._factors(xyz)
        h = [[None] * 3 for _ in range(3)]
        for d in range(3):
            for e in range(3):
                f = []
                for q in range(3):
                    if q == d and q == e:
                        f.append(s2[q])
                    elif q == d or q == e:
                        f.append(c[q])
                    else:
                        f.append(s[q])
                h[d][e] = self.a * f[0] * f[1] * f[2]
        return h


DISPLACEMENT = (
    SineProduct(0.1, 1.0, (1.3, 0.9, 1.1), (0.4, 1.2, 0.2)),
    SineProduct(-0.2, 0.8, (0.7, 1.5, 1.2), (1.0, 0.3, 0.9)),
    SineProduct(0.05, 1.2, (1.1, 0.8, 1.6), (0.6, 0.5, 1.4)),
)
MU = SineProduct(1.5, 0.4, (0.9, 1.2, 0.7), (0.3, 0.8, 0.5))
LAMBDA = SineProduct(1.2, 0.3, (1.4, 0.6, 1.0), (0.9, 0.2, 0.7))


def fields(xyz):
    """(u[3], mu, lambda) at the points xyz = (x, y, z) arrays of one shape."""
    return [f.value(xyz) for f in DISPLACEMENT], MU.value(xyz), LAMBDA.value(xyz)


def div_stress(xyz):
    """The three components of div sigma at the points xyz."""
    g = [f.grad(xyz) for f in DISPLACEMENT]  # g[m][d] = d_d u_m
    hs = [f.hess(xyz) for f in DISPLACEMENT]  # hs[m][d][e] = d_d d_e u_m
    mu, la = MU.value(xyz), LAMBDA.value(xyz)
    gmu, gla = MU.grad(xyz), LAMBDA.grad(xyz)
    div = g[0][0] + g[1][1] + g[2][2]
    out = []
    for i in range(3):
        ddiv = hs[0][i][0] + hs[1][i][1] + hs[2][i][2]
        r = gla[i] * div + la * ddiv
        for j in range(3):
            r = r + gmu[j] * (g[j][i] + g[i][j]) + mu * (hs[j][i][j] + hs[i][j][j])
        out.append(r)
    return out


def cartesian_points(bounds, h):
    """x, y, z of the grid points of a Cartesian grid with 1-based inclusive bounds,
    shaped [k, j, i]: x = (i - 1) h and so on."""
    ib, ie, jb, je, kb, ke = bounds
    k, j, i = np.meshgrid(np.arange(kb, ke + 1), np.arange(jb, je + 1), np.arange(ib, ie + 1),
                          indexing="ij")
    return (i - 1) * h, (j - 1) * h, (k - 1) * h


def mapped_z(x, y, r):
    """A smooth curvilinear mapping: the depth coordinate r = (k - 1) h bent by a
    product of sines (z_r stays within 1 +- 0.05, so no cell folds)."""
    return r + 0.1 * np.sin(0.9 * x + 0.2) * np.cos(0.7 * y + 0.1) * np.cos(0.5 * r)


def case(n, curvilinear=False, length=2.0):
    """The fields of an n^3 grid (two ghost points per side) on [0, length]^3, SoA
    [c, k, j, i] flattened: bounds, h, u, mu, lambda, the exact div sigma, and z
    (None for the Cartesian grid)."""
    h = length / (n - 1)
    b = (-1, n + 2, -1, n + 2, -1, n + 2)
    x, y, r = cartesian_points(b, h)
    z = mapped_z(x, y, r) if curvilinear else r
    u, mu, la = fields((x, y, z))
    flat = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1))
    return dict(bounds=b, h=h, n=n, u=flat(np.stack(u)), mu=flat(mu), la=flat(la),
                exact=np.stack(div_stress((x, y, z))), z=flat(z) if curvilinear else None)


def row_errors(lu, c):
    """max |L u - div sigma| over the interior points: the rows k >= 7 from both z
    sides, the six rows next to k = 1 and the six rows next to k = n."""
    m = c["n"] + 4
    err = np.abs(lu.reshape(3, m, m, m) - c["exact"])[:, 2:-2, 2:-2, 2:-2]
    return err[:, 6:-6].max(), err[:, :6].max(), err[:, -6:].max()


def rates(errs):
    """log2 of the ratios of successive errors (one halving of h each)."""
    e = np.asarray(errs)
    return np.log2(e[:-1] / e[1:])
