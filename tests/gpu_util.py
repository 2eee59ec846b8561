"""Helpers for the GPU parity tests: device copies and the problem set-up shared by
the CUDA path and the oracle."""
from __future__ import annotations

import ctypes as C

import numpy as np

import sw4lite_gb300 as sg
from oracle import oracle as O


def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("these tests need a CUDA GPU")
    return torch


def dev(a):
    torch = torch_cuda()
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch_cuda().cuda.synchronize()
    return t.cpu().numpy()


def stream():
    return torch_cuda().cuda.current_stream().cuda_stream


def smooth_material(nx, ny, nz, seed, rho0=2.0, cs=1.0, cp=1.8, amp=0.15):
    """Smoothly varying positive (rho, mu, lambda) on the (nz+4, ny+4, nx+4) array."""
    rng = np.random.default_rng(seed)
    k, j, i = np.meshgrid(np.arange(nz + 4), np.arange(ny + 4), np.arange(nx + 4), indexing="ij")

    def field(base):
        ph = rng.uniform(0, 2 * np.pi, 3)
        f = rng.uniform(0.05, 0.2, 3)
        return base * (1 + amp * np.sin(f[0] * i + ph[0]) * np.cos(f[1] * j + ph[1]) *
                       np.sin(f[2] * k + ph[2] + 0.3))

    rho = field(rho0)
    mu = field(rho0 * cs * cs)
    la = field(rho0 * cp * cp) - 2 * mu
    la = np.maximum(la, 0.1 * mu)
    return [np.ascontiguousarray(a.ravel()) for a in (rho, mu, la)]


def smooth_fields(nx, ny, nz, seed, scale=1e-3):
    rng = np.random.default_rng(seed)
    k, j, i = np.meshgrid(np.arange(nz + 4), np.arange(ny + 4), np.arange(nx + 4), indexing="ij")
    out = []
    for _ in range(2):
        comps = []
        for c in range(3):
            f = rng.uniform(0.1, 0.4, 3)
            ph = rng.uniform(0, 2 * np.pi, 3)
            comps.append(np.sin(f[0] * i + ph[0]) * np.sin(f[1] * j + ph[1]) * np.cos(f[2] * k + ph[2]))
        out.append(scale * np.ascontiguousarray(np.stack(comps).ravel()))
    return out


def discretize(grid, src):
    """The library's host discretisation of one source (the product's set-up path)."""
    cap = 4096
    ijk = np.zeros(3 * cap, dtype=np.int32)
    amp = np.zeros(3 * cap)
    n = C.c_int()
    sg.check(sg.lib().sw4g_discretize_source(C.byref(grid), C.byref(src), cap,
                                             ijk.ctypes.data_as(sg._I), amp.ctypes.data_as(sg._D),
                                             C.byref(n)))
    n = n.value
    return ijk[:3 * n].copy(), amp[:3 * n].copy()


def oracle_source(src):
    """An sw4g_source descriptor as the oracle's PointSource."""
    if src.moment:
        return O.PointSource(src.x, src.y, src.z, moment=(src.mxx, src.mxy, src.mxz, src.myy,
                                                          src.myz, src.mzz),
                             freq=src.freq, t0=src.t0, kind=src.kind)
    return O.PointSource(src.x, src.y, src.z, force=(src.fx, src.fy, src.fz), freq=src.freq,
                         t0=src.t0, kind=src.kind)


def oracle_discretize(grid, src):
    """The oracle's discretisation of one source on a grid descriptor's grid."""
    p = oracle_source(src)
    return O.discretize_source(grid.nx, grid.ny, grid.nz, grid.h, grid.zmin, grid.bc[4] == 0,
                               grid.bc[5] == 0, p.x, p.y, p.z, force=p.force, moment=p.moment)


class OracleProblem(O.CartProblem):
    """The oracle's problem for a GPU grid descriptor: the same material, supergrid
    profiles and sources, with the sources discretised by the oracle itself."""

    def __init__(self, grid, rho, mu, la, dt, sources=()):
        super().__init__(grid.nx, grid.ny, grid.nz, grid.h, [grid.bc[s] for s in range(6)], rho, mu,
                         la, dt, [oracle_source(s) for s in sources], zmin=grid.zmin,
                         sg_gp=grid.sg_gp, sg_damping=grid.sg_damping, sg_order=grid.sg_order)
        self.g = grid


def solution_mask(grid):
    """Every array point: the GPU paths reproduce the reference's values on the
    whole array, ghost shell included."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    return np.ones(3 * (nz + 4) * (ny + 4) * (nx + 4), dtype=bool)


def describe_error(a, b, grid, mask=None):
    """Location and size of the largest |a-b| over a 3-component field on grid."""
    shape = (3, grid.nz + 4, grid.ny + 4, grid.nx + 4)
    d = np.abs(np.asarray(a) - np.asarray(b))
    if mask is not None:
        d = np.where(mask, d, 0.0)
    q = int(np.argmax(d))
    c, kk, jj, ii = np.unravel_index(q, shape)
    scale = np.max(np.abs(b))
    # per-plane maximum of the error, to tell boundary rows from the interior
    planes = d.reshape(shape).max(axis=(0, 2, 3))
    worst = np.argsort(planes)[::-1][:4]
    return (f"max |diff| {d.flat[q]:.3e} (rel {d.flat[q] / scale:.3e}) at c={c} "
            f"i={ii - 1} j={jj - 1} k={kk - 1}; worst planes k=" +
            ", ".join(f"{w - 1}:{planes[w] / scale:.1e}" for w in worst))
