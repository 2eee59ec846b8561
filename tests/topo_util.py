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
                 rho=1.0, gp=6, damping=0.02, sources=(), bc_sides=(2, 2, 2, 2), bc_bottom=2,
                 sg_order=4, precision=0):
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
                                 sg_damping=damping, sg_order=sg_order, precision=precision)
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
        self.cart = OracleProblem(case.grid, *case.cart_mat, dt, ())
        # sources of both grids from the restated two-grid discretisation
        per = {0: ([], [], [], [], []), 1: ([], [], [], [], [])}
        for src in case.sources:
            for g, (ijk, amp) in enumerate(discretize_two_grid(case, src)):
                n = len(ijk)
                per[g][0].append(ijk.reshape(-1))
                per[g][1].append(amp.reshape(-1))
                per[g][2].extend([src.freq] * n)
                per[g][3].extend([src.t0] * n)
                per[g][4].extend([src.kind] * n)
        cat = lambda v, dt_: np.concatenate(v).astype(dt_) if v else np.zeros(0, dtype=dt_)
        a = per[0]
        self.cart.set_grid_point_sources(cat(a[0], np.int32), cat(a[1], np.float64), a[2], a[3], a[4])
        b = per[1]
        self.csrc = (np.ascontiguousarray(cat(b[0], np.int32)), np.ascontiguousarray(cat(b[1], np.float64)),
                     np.asarray(b[2], dtype=np.float64), np.asarray(b[3], dtype=np.float64),
                     np.asarray(b[4], dtype=np.int32))
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
        c.nsrc = len(self.csrc[2])
        c.src_ijk = self.csrc[0].ctypes.data_as(O._I)
        c.src_amp = self.csrc[1].ctypes.data_as(O._D)
        c.src_freq = self.csrc[2].ctypes.data_as(O._D)
        c.src_t0 = self.csrc[3].ctypes.data_as(O._D)
        c.src_kind = self.csrc[4].ctypes.data_as(O._I)
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


# ---------------------------------------------------------------------------
# Two-grid source discretisation restated in numpy (Source::set_grid_point_sources4
# with its curvilinear branches, src/Source.C:1074-1990; mapping inversion
# src/EW.C:5722-5782; metric at the source src/Source.C:2191-2330), independent of
# the library's C++ version it checks.

def _wgh(a):
    """6-point delta weights (src/Source.C:553-560)."""
    p5 = a**5 * (5.0 / 3 - 7.0 / 24 * a - 17 / 12.0 * a**2 + 1.125 * a**3 - 0.25 * a**4)
    return np.array([1.0 / 24 * (2 * a - a**2 - 2 * a**3 - 19 * a**4) + p5,
                     1.0 / 6 * (-4 * a + 4 * a**2 + a**3) + 4 * a**4 - 5 * p5,
                     1 - 1.25 * a**2 - 97.0 / 12 * a**4 + 10 * p5,
                     1.0 / 6 * (4 * a + 4 * a**2 - a**3 + 49 * a**4) - 10 * p5,
                     1.0 / 24 * (-2 * a - a**2 + 2 * a**3) - 4.125 * a**4 + 5 * p5,
                     5.0 / 6 * a**4 - p5])


def _dwgh(a):
    """6-point delta' weights (src/Source.C:587-594)."""
    p5 = a**4 * (-25.0 / 12 - 0.75 * a + 59.0 / 12 * a**2 - 4 * a**3 + a**4)
    return np.array([1.0 / 12 * (-1 + a + 3 * a**2 + 8 * a**3) + p5,
                     2.0 / 3 * (1 - 2 * a) - 0.5 * a**2 - 3.5 * a**3 - 5 * p5,
                     2.5 * a + 22.0 / 3 * a**3 + 10 * p5,
                     2.0 / 3 * (-1 - 2 * a) + 0.5 * a**2 - 23.0 / 3 * a**3 - 10 * p5,
                     (1 + a) / 12 - 0.25 * a**2 + 4 * a**3 + 5 * p5,
                     -5.0 / 6 * a**3 - p5])


def _wgh_low(a):
    return np.array([(2 * a - a**2 - 2 * a**3 + a**4) / 24, (-4 * a + 4 * a**2 + a**3 - a**4) / 6,
                     1 - 1.25 * a**2 + 0.25 * a**4, (4 * a + 4 * a**2 - a**3 - a**4) / 6,
                     (-2 * a - a**2 + 2 * a**3 + a**4) / 24, 0.0])


def _dwgh_low(a):
    return np.array([(-1 + a + 3 * a**2 - 2 * a**3) / 12, (2 - 4 * a - 1.5 * a**2 + 2 * a**3) / 3,
                     2.5 * a - a**3, (-2 - 4 * a + 1.5 * a**2 + 2 * a**3) / 3,
                     (1 + a - 3 * a**2 - 2 * a**3) / 12, 0.0])


def _metwgh(a):
    """8-point interpolation weights and their derivative (src/Source.C:682-720)."""
    pol = a**7 * (-251 + 135 * a + 25 * a**2 - 33 * a**3 + 6 * a**4) / 720
    w = np.array([-1.0 / 60 * a + 1.0 / 180 * a**2 + 1.0 / 48 * a**3 + 23.0 / 144 * a**4
                  - (17.0 * a + 223.0) * a**5 / 720 - pol,
                  3.0 / 20 * a - 3.0 / 40 * a**2 - 1.0 / 6 * a**3 - 13.0 / 12 * a**4 + 97.0 / 45 * a**5
                  + 1.0 / 6 * a**6 + 7 * pol,
                  -0.75 * a + 0.75 * a**2 + (13.0 + 155 * a) * a**3 / 48 - 103.0 / 16 * a**5
                  - 121.0 / 240 * a**6 - 21 * pol,
                  1 - 49.0 / 36 * a**2 - 49.0 / 9 * a**4 + 385.0 / 36 * a**5 + 61.0 / 72 * a**6 + 35 * pol,
                  0.75 * a + 0.75 * a**2 - 13.0 / 48 * a**3 + 89.0 / 16 * a**4 - 1537.0 / 144 * a**5
                  - 41.0 / 48 * a**6 - 35 * pol,
                  -3.0 / 20 * a - 3.0 / 40 * a**2 + 1.0 / 6 * a**3 - 41.0 / 12 * a**4 + 6.4 * a**5
                  + 31.0 / 60 * a**6 + 21 * pol,
                  1.0 / 60 * a + 1.0 / 180 * a**2 - 1.0 / 48 * a**3 + 167.0 / 144 * a**4
                  - 1537.0 / 720 * a**5 - 25.0 / 144 * a**6 - 7 * pol,
                  -1.0 / 6 * a**4 + 11.0 / 36 * a**5 + 1.0 / 40 * a**6 + pol])
    pol = a**6 * (-1757.0 / 720 + 1.5 * a + 0.3125 * a**2 - (1.375 * a**3 - 0.275 * a**4) / 3)
    d = np.array([-1.0 / 60 + 1.0 / 90 * a + a**2 / 16 + 23.0 / 36 * a**3 - 223.0 / 144 * a**4
                  - 17.0 / 120 * a**5 - pol,
                  3.0 / 20 - 3.0 / 20 * a - 0.5 * a**2 - 13.0 / 3 * a**3 + 97.0 / 9 * a**4 + a**5 + 7 * pol,
                  -0.75 + 1.5 * a + 13.0 / 16 * a**2 + 155.0 * a**3 / 12 - 103.0 * 5.0 / 16 * a**4
                  - 121.0 / 40 * a**5 - 21 * pol,
                  -49.0 / 18 * a - 4 * 49.0 / 9.0 * a**3 + 385.0 * 5.0 / 36 * a**4 + 61.0 / 12 * a**5
                  + 35 * pol,
                  0.75 + 1.5 * a - 13.0 / 16 * a**2 + 89.0 / 4 * a**3 - 1537.0 * 5 / 144.0 * a**4
                  - 41.0 / 8 * a**5 - 35 * pol,
                  -3.0 / 20 - 3.0 / 20 * a + 0.5 * a**2 - 41.0 / 3 * a**3 + 32 * a**4 + 3.1 * a**5
                  + 21 * pol,
                  1.0 / 60 + 1.0 / 90 * a - 1.0 / 16 * a**2 + 167.0 / 36 * a**3 - 1537.0 / 144 * a**4
                  - 25.0 / 24 * a**5 - 7 * pol,
                  -2.0 / 3 * a**3 + 55.0 / 36 * a**4 + 3.0 / 20 * a**5 + pol])
    return w, d


def _elev(case, x, y):
    hl = case.hill
    return hl["amp"] * np.exp(-((x - hl["xc"]) / hl["lx"]) ** 2 - ((y - hl["yc"]) / hl["ly"]) ** 2)


def curvilinear_s(case, q, r, z, zeta_break=0.95, order=4):
    """s of (q, r, z) on the curvilinear grid (Newton, src/EW.C:5722-5782)."""
    h, nz, zmax = case.h, case.nc, case.zmax_topo
    ztopo = -_elev(case, (q - 1) * h, (r - 1) * h)
    izb = 1.0 / zeta_break
    sun = 1 - (zmax - z) / ((nz - 1) * h)
    if sun < zeta_break:
        for _ in range(10):
            omsm = (1 - izb * sun) ** (order - 1)
            fp = h * (nz - 1) + izb * order * omsm * (zmax - (nz - 1) * h - ztopo)
            omsm *= 1 - izb * sun
            f = zmax - (nz - 1) * h * (1 - sun) - omsm * (zmax - (nz - 1) * h - ztopo) - z
            ds = f / fp
            sun -= ds
            if abs(ds) <= 1e-9:
                break
    return (nz - 1) * sun + 1


def discretize_two_grid(case, src, zeta_break=0.95, order=4):
    """((ijk, amp) of the Cartesian grid, (ijk, amp) of the curvilinear grid)."""
    h, g = case.h, case.grid
    Ni, Nj = case.nx, case.ny
    x, y, z = src.x, src.y, src.z
    in_curv = not (z > g.zmin)
    Nz = case.nc if in_curv else case.ncart
    q0, r0 = x / h + 1, y / h + 1
    s0 = curvilinear_s(case, q0, r0, z, zeta_break, order) if in_curv else (z - g.zmin) / h + 1
    ic, jc, kc = int(np.floor(q0)), int(np.floor(r0)), int(np.floor(s0))
    ic = 3 if ic <= 2 else (Ni - 3 if ic >= Ni - 2 else ic)
    jc = 3 if jc <= 2 else (Nj - 3 if jc >= Nj - 2 else jc)
    kc = Nz - 1 if kc >= Nz else max(kc, 1)
    upper, lower = 1 <= kc <= 3, Nz - 3 <= kc <= Nz - 1
    across = (upper and not in_curv) or (lower and in_curv)
    if not across:
        kc = 3 if kc <= 2 else (Nz - 3 if kc >= Nz - 2 else kc)
    ai, bi, ci = q0 - ic, r0 - jc, s0 - kc
    wi, wj, wk = _wgh(ai), _wgh(bi), _wgh(ci)
    dwi, dwj, dwk = _dwgh(ai), _dwgh(bi), _dwgh(ci)
    if not across and kc == 3 and ci <= 0:
        wk, dwk = _wgh_low(ci), _dwgh_low(ci)
    norm = [17 / 48, 59 / 48, 43 / 48, 49 / 48]
    top_os = True if in_curv else g.bc[4] == 0
    bot_os = False if in_curv else g.bc[5] == 0
    for k in range(6):
        if top_os and 1 <= k + kc - 2 <= 4:
            wk[k] /= norm[k + kc - 3]
            dwk[k] /= norm[k + kc - 3]
        if bot_os and Nz - 3 <= k + kc - 2 <= Nz:
            wk[k] /= norm[Nz - k - kc + 2]
            dwk[k] /= norm[Nz - k - kc + 2]
    sx0 = [0.0, 0.0, 1 / h]
    force = (src.fx, src.fy, src.fz)
    moments = (src.mxx, src.mxy, src.mxz, src.myy, src.myz, src.mzz)
    if in_curv and src.moment:
        zq, zr, zs = 0.0, 0.0, h
        zpar = (s0 - 1) / (zeta_break * (Nz - 1))
        if kc <= Nz - 3 and zpar < 1:
            ai8, dai8 = _metwgh(q0 - ic)
            bj8, dbj8 = _metwgh(r0 - jc)
            ii = np.arange(ic - 3, ic + 5)
            jj = np.arange(jc - 3, jc + 5)
            T = _elev(case, (ii[None, :] - 1) * h, (jj[:, None] - 1) * h)  # [j, i]
            tavg = bj8 @ T @ ai8
            tq = bj8 @ T @ dai8
            tr = dbj8 @ T @ ai8
            pp = (1 - zpar) ** (order - 1)
            powo, dpowo = (1 - zpar) * pp, -order * pp / zeta_break
            zq, zr = -tq * powo, -tr * powo
            kbreak = 1 + zeta_break * (Nz - 1)
            c1 = (g.zmin - (Nz - kbreak) * h) + tavg - h * (kbreak - 1)
            zs = h + c1 * (-dpowo) / (Nz - 1)
        sx0 = [-zq / (h * zs), -zr / (h * zs), 1 / zs]
    jac = case.jac.reshape(case.nc + 4, Nj + 4, Ni + 4)
    cart, curv = [], []
    for k in range(kc - 2, kc + 4):
        for j in range(jc - 2, jc + 4):
            for i in range(ic - 2, ic + 4):
                if not (1 <= i <= Ni and 1 <= j <= Nj):
                    continue
                jaci = 1 / jac[k + 1, j + 1, i + 1] if in_curv else 1 / h**3
                a, b, c = i - ic + 2, j - jc + 2, k - kc + 2
                if not src.moment:
                    wF = wi[a] * wj[b] * wk[c]
                    if wF == 0 or not any(force):
                        continue
                    amp = [wF * jaci * f for f in force]
                else:
                    wFx = dwi[a] * wj[b] * wk[c] / h + wi[a] * wj[b] * dwk[c] * sx0[0]
                    wFy = wi[a] * dwj[b] * wk[c] / h + wi[a] * wj[b] * dwk[c] * sx0[1]
                    wFz = wi[a] * wj[b] * dwk[c] * sx0[2]
                    m = moments
                    amp = [-(m[0] * wFx + m[1] * wFy + m[2] * wFz) * jaci,
                           -(m[1] * wFx + m[3] * wFy + m[4] * wFz) * jaci,
                           -(m[2] * wFx + m[4] * wFy + m[5] * wFz) * jaci]
                own = curv if in_curv else cart
                if 1 <= k <= Nz:
                    own.append(((i, j, k), amp))
                if across and not in_curv and k <= 1:
                    curv.append(((i, j, case.nc - 1 + k), amp))
                if across and in_curv and k >= Nz:
                    cart.append(((i, j, k - Nz + 1), amp))

    def pack(v):
        return (np.array([p for p, _ in v], dtype=np.int32).reshape(-1, 3),
                np.array([a for _, a in v], dtype=np.float64).reshape(-1, 3))
    return pack(cart), pack(curv)
