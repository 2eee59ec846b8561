"""A topography workload for the tests: a curvilinear grid over a Gaussian hill on
top of a Cartesian grid, as the reference builds it (EW::defineDimensionsZ
src/EW.C:2018-2046, generate_grid :6164, setup_supergrid :4640-4668).

The Cartesian grid runs from z = zmax_topo down (its top side is the interface,
boundary kind 4); the curvilinear grid has nc points from the topography down to
zmax_topo, nc = 1 + round((zmax_topo - topo_avg)/h) with topo_avg the midpoint of
the topography's z range.  Material is a depth gradient below the surface
(vs = vs0 + grad*depth, vp = sqrt(3) vs, constant rho).
"""
import numpy as np

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.gpu_util import OracleProblem

INTERFACE = 4


class TopoCase:
    def __init__(self, nx, ny, ncart, h, zmax_topo, amp, xc, yc, lx, ly, vs0=1.0, grad=0.5,
                 rho=1.0, gp=6, damping=0.02, sources=(), bc_sides=(2, 2, 2, 2), bc_bottom=2):
        self.nx, self.ny, self.ncart, self.h = nx, ny, ncart, h
        self.zmax_topo = zmax_topo
        self.hill = dict(amp=amp, xc=xc, yc=yc, lx=lx, ly=ly)
        i = np.arange(-1, nx + 3)
        j = np.arange(-1, ny + 3)
        X, Y = np.meshgrid((i - 1) * h, (j - 1) * h, indexing="xy")
        zs = -amp * np.exp(-((X - xc) / lx) ** 2 - ((Y - yc) / ly) ** 2)
        topo_avg = 0.5 * (zs.min() + zs.max())
        self.nc = nc = 1 + int(round((zmax_topo - topo_avg) / h))
        self.zs = zs
        bc = tuple(bc_sides) + (INTERFACE, bc_bottom)
        self.bc = bc
        self.grid = sg.grid_desc(nx, ny, ncart, h, bc=bc, zmin=zmax_topo, sg_gp=gp,
                                 sg_damping=damping)
        self.cbounds = (-1, nx + 2, -1, ny + 2, -1, nc + 2)
        self.z = O.gaussian_hill_z(self.cbounds, nc, h, zmax_topo, amp, xc, yc, lx, ly)
        n = self.z.size
        self.met, self.jac = np.zeros(4 * n), np.zeros(n)
        assert O.metric(1, self.cbounds, h, self.z, self.met, self.jac) == 0

        def material(zz, zsurf):
            depth = np.maximum(zz - zsurf, 0.0)
            vs = vs0 + grad * depth
            vp = np.sqrt(3.0) * vs
            r = np.full_like(zz, rho)
            mu = r * vs * vs
            return r, mu, r * vp * vp - 2 * mu

        kk = np.arange(-1, ncart + 3)
        zc = zmax_topo + (kk - 1) * h
        Zc = np.broadcast_to(zc[:, None, None], (ncart + 4, ny + 4, nx + 4))
        self.cart_mat = [np.ascontiguousarray(a.reshape(-1))
                         for a in material(Zc, np.broadcast_to(zs, Zc.shape))]
        Zv = self.z.reshape(nc + 4, ny + 4, nx + 4)
        self.curv_mat = [np.ascontiguousarray(a.reshape(-1))
                         for a in material(Zv, np.broadcast_to(zs, Zv.shape))]
        self.sources = list(sources)

    def time_step(self, cfl):
        """min of the Cartesian and the curvilinear limits (EW::computeDT)."""
        rho, mu, la = self.cart_mat
        dt_c = cfl * self.h / np.sqrt(np.max((4 * mu + la) / rho))
        rho, mu, la = self.curv_mat
        dt_v = O.curv_dt(1, self.cbounds, rho, mu, la, self.met, self.jac, cfl)
        return min(dt_c, dt_v)

    def oracle(self, dt):
        return OracleTopo(self, dt)


class OracleTopo:
    """The oracle's two-grid problem for a TopoCase (sw4o_step_topo)."""

    def __init__(self, case: TopoCase, dt):
        self.case = case
        self.cart = OracleProblem(case.grid, *case.cart_mat, dt, case.sources)
        cp = self.cart.prof
        c = O.Curv()
        c.ib, c.ie, c.jb, c.je, c.kb, c.ke = case.cbounds
        c.nx, c.ny, c.nz = case.nx, case.ny, case.nc
        c.h = case.h
        cbc = tuple(case.bc[:4]) + (0, INTERFACE)
        for s in range(6):
            c.bccnd[s] = cbc[s]
        wind, _ = O.boundary_windows(case.cbounds, (case.nx, case.ny, case.nc), cbc)
        for q in range(36):
            c.wind[q] = int(wind[q])
        self.keep = list(case.curv_mat) + [case.met, case.jac] + [a for p in cp[:2] for a in p]
        c.rho, c.mu, c.la = [O._dp(a) for a in case.curv_mat]
        c.met, c.jac = O._dp(case.met), O._dp(case.jac)
        c.dcx, c.strx, c.cox = [O._dp(a) for a in cp[0]]
        c.dcy, c.stry, c.coy = [O._dp(a) for a in cp[1]]
        self.curv = c
        self.cnpts = case.z.size

    def run(self, u, um, cu, cum, t0, nsteps, which="oracle"):
        n3, c3 = 3 * self.cart.npts, 3 * self.cnpts
        u, um, cu, cum = u.copy(), um.copy(), cu.copy(), cum.copy()
        up, lu, f, uacc = (np.zeros(n3) for _ in range(4))
        cup, clu, cf, cuacc = (np.zeros(c3) for _ in range(4))
        t = t0
        for _ in range(nsteps):
            O.step_topo(self.cart.P, self.curv, t, (up, u, um, lu, f, uacc),
                        (cup, cu, cum, clu, cf, cuacc), which=which)
            um, u, up = u, up, um
            cum, cu, cup = cu, cup, cum
            t += self.cart.P.dt
        return u, um, cu, cum


def smooth_topo_fields(case: TopoCase, seed, scale=1e-3):
    """Smooth initial levels on both grids, continuous across the interface (a
    function of the physical x, y, z)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.5, 1.5, size=(2, 3, 3))
    h = case.h

    def field(Z, lvl):
        kk, jj, ii = np.meshgrid(np.arange(Z.shape[0]), np.arange(case.ny + 4),
                                 np.arange(case.nx + 4), indexing="ij")
        X, Y = (ii - 2) * h, (jj - 2) * h
        out = []
        for c in range(3):
            w = a[lvl, c]
            out.append((scale * np.sin(w[0] * X + 0.3 * c) * np.cos(w[1] * Y - 0.2 * c) *
                        np.sin(w[2] * Z + 0.1)).reshape(-1))
        return np.concatenate(out)

    kc = np.arange(-1, case.ncart + 3)
    Zc = np.broadcast_to((case.zmax_topo + (kc - 1) * h)[:, None, None],
                         (case.ncart + 4, case.ny + 4, case.nx + 4))
    Zv = case.z.reshape(case.nc + 4, case.ny + 4, case.nx + 4)
    return field(Zc, 0), field(Zc, 1), field(Zv, 0), field(Zv, 1)
