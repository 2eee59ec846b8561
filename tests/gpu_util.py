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
    cap = 4096
    ijk = np.zeros(3 * cap, dtype=np.int32)
    amp = np.zeros(3 * cap)
    n = C.c_int()
    sg.check(sg.lib().sw4g_discretize_source(C.byref(grid), C.byref(src), cap,
                                             ijk.ctypes.data_as(sg._I), amp.ctypes.data_as(sg._D),
                                             C.byref(n)))
    n = n.value
    return ijk[:3 * n].copy(), amp[:3 * n].copy()


class OracleProblem:
    """The oracle's sw4o_problem for a grid, with the same material, profiles and
    grid-point sources as a GPU EW object."""

    def __init__(self, grid, rho, mu, la, dt, sources=()):
        self.g = grid
        nx, ny, nz = grid.nx, grid.ny, grid.nz
        self.bounds = (-1, nx + 2, -1, ny + 2, -1, nz + 2)
        self.keep = [rho, mu, la]
        bc = [grid.bc[s] for s in range(6)]
        used = 2 in bc
        prof = []
        for ax, n, b0, b1 in [(0, nx, bc[0], bc[1]), (1, ny, bc[2], bc[3]), (2, nz, bc[4], bc[5])]:
            if used:
                xmax = (grid.zmin if ax == 2 else 0.0) + (n - 1) * grid.h
                p = O.supergrid_profile(-1, n + 2, grid.h, grid.zmin if ax == 2 else 0.0, b0 == 2,
                                        b1 == 2, 0.0, xmax, grid.sg_gp * grid.h)
            else:
                p = (np.zeros(n + 4), np.ones(n + 4), np.ones(n + 4))
            prof.append(p)
        self.prof = prof
        self.keep += [a for p in prof for a in p]
        wind, _ = O.boundary_windows(self.bounds, (nx, ny, nz), bc)
        P = O.Problem()
        P.ib, P.ie, P.jb, P.je, P.kb, P.ke = self.bounds
        P.nx, P.ny, P.nz = nx, ny, nz
        P.h, P.dt = grid.h, dt
        for s in range(6):
            P.bccnd[s] = bc[s]
        P.onesided[4] = int(bc[4] == 0)
        P.onesided[5] = int(bc[5] == 0)
        for q in range(36):
            P.wind[q] = int(wind[q])
        P.sg_beta = grid.sg_damping if used else 0.0
        P.sg_order = grid.sg_order
        dp = O._dp
        P.rho, P.mu, P.la = dp(rho), dp(mu), dp(la)
        P.dcx, P.strx, P.cox = [dp(a) for a in prof[0]]
        P.dcy, P.stry, P.coy = [dp(a) for a in prof[1]]
        P.dcz, P.strz, P.coz = [dp(a) for a in prof[2]]
        self.P = P
        ijk, amp, freq, t0, kind = [], [], [], [], []
        for src in sources:
            a, b = discretize(grid, src)
            n = len(a) // 3
            ijk.append(a)
            amp.append(b)
            freq += [src.freq] * n
            t0 += [src.t0] * n
            kind += [src.kind] * n
        self.set_grid_point_sources(np.concatenate(ijk) if ijk else np.zeros(0),
                                    np.concatenate(amp) if amp else np.zeros(0), freq, t0, kind)
        self.npts = (nx + 4) * (ny + 4) * (nz + 4)

    def set_grid_point_sources(self, ijk, amp, freq, t0, kind):
        """Grid-point sources (flat ijk and amp, 3 per source) of this problem."""
        self.src = (np.ascontiguousarray(ijk, dtype=np.int32).reshape(-1),
                    np.ascontiguousarray(amp, dtype=np.float64).reshape(-1),
                    np.asarray(freq, dtype=np.float64), np.asarray(t0, dtype=np.float64),
                    np.asarray(kind, dtype=np.int32))
        self.keep += list(self.src)
        P = self.P
        P.nsrc = len(self.src[2])
        P.src_ijk = self.src[0].ctypes.data_as(O._I)
        P.src_amp = self.src[1].ctypes.data_as(O._D)
        P.src_freq = self.src[2].ctypes.data_as(O._D)
        P.src_t0 = self.src[3].ctypes.data_as(O._D)
        P.src_kind = self.src[4].ctypes.data_as(O._I)

    def run(self, u, um, t0, nsteps, which="oracle", receivers=None):
        """nsteps oracle steps from (u, um); with receivers [(ijk, mode), ...] also
        returns the record rows (initial data, then one row per step)."""
        n3 = 3 * self.npts
        u, um = u.copy(), um.copy()
        up, lu, f, uacc = (np.zeros(n3) for _ in range(4))
        t = t0
        g = self.g
        dims = (g.nx, g.ny, g.nz)

        def row(a, b, initial):
            return np.concatenate([O.record(m, ijk, a, b, self.P.dt, g.h, dims, initial)
                                   for ijk, m in receivers])

        rows = [row(u, um, True)] if receivers else []
        for _ in range(nsteps):
            O.step(self.P, 1, t, up, u, um, lu, f, uacc, which=which)
            if receivers:
                rows.append(row(up, um, False))
            um, u, up = u, up, um
            t += self.P.dt
        if receivers:
            return u, um, np.array(rows)
        return u, um


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
