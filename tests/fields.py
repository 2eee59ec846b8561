"""Seeded synthetic inputs shared by the parity tests.

Grids use the reference's conventions: inclusive 1-based bounds that carry two
ghost points per side, i fastest, component layout AoS (soa=0) or SoA (soa=1).
"""
from __future__ import annotations

import numpy as np


class Grid:
    """Bounds of one Cartesian grid with N=(nx,ny,nz) interior points and 2 ghosts."""

    def __init__(self, nx, ny, nz, h=0.01, ghosts=2):
        self.nx, self.ny, self.nz = nx, ny, nz
        self.h = h
        self.ib, self.ie = 1 - ghosts, nx + ghosts
        self.jb, self.je = 1 - ghosts, ny + ghosts
        self.kb, self.ke = 1 - ghosts, nz + ghosts
        self.ni = self.ie - self.ib + 1
        self.nj = self.je - self.jb + 1
        self.nk = self.ke - self.kb + 1
        self.npts = self.ni * self.nj * self.nk

    @property
    def bounds(self):
        return (self.ib, self.ie, self.jb, self.je, self.kb, self.ke)

    def field3(self, rng, scale=1.0):
        return np.ascontiguousarray(rng.standard_normal(3 * self.npts) * scale)

    def material(self, rng, rho0=2.0, mu0=1.5, la0=1.0, spread=0.3):
        """Positive, randomly perturbed (rho, mu, lambda)."""
        def pos(v):
            return np.ascontiguousarray(v * (1 + spread * rng.uniform(-1, 1, self.npts)))
        return pos(rho0), pos(mu0), pos(la0)

    def strip(self, rng, n, lo=0.5, hi=1.0):
        return np.ascontiguousarray(rng.uniform(lo, hi, n))

    def stretching(self, rng):
        return (self.strip(rng, self.ni), self.strip(rng, self.nj), self.strip(rng, self.nk))

    def as4(self, a, soa):
        """View a 3-component field as [c, k, j, i]."""
        if soa:
            return a.reshape(3, self.nk, self.nj, self.ni)
        return np.moveaxis(a.reshape(self.nk, self.nj, self.ni, 3), 3, 0)

    def interior_mask(self, margin=2):
        m = np.zeros((self.nk, self.nj, self.ni), dtype=bool)
        m[margin:-margin, margin:-margin, margin:-margin] = True
        return m


def rel_err(a, b, mask=None):
    """max|a-b| / max|b| over the (optionally masked) entries."""
    a = np.asarray(a)
    b = np.asarray(b)
    if mask is not None:
        a = a[mask]
        b = b[mask]
    den = np.max(np.abs(b))
    if den == 0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / den)
