"""Receivers on the curvilinear grid (topography) on the GPU.

Records: every record mode on grid 1, beside receivers on grid 0, against the
reference's curvilinear formulas of EW::extractRecordData (src/EW.C:5882-6068)
restated in numpy on the fields read back after each step: centred differences
along q, r, s combined with the metric at the receiver (m1 d/dq + m2 d/ds for x,
m1 d/dr + m3 d/ds for y, m4 d/ds for z) and scaled by 0.5/sqrt(J).  The device
sums in another order (and contracts products into FMAs), so each record column is
held to 1e-12 of its largest magnitude.

Placement: sw4g_ew_nearest_grid_point against the grids themselves.  A point on a
curvilinear grid point maps to that point (the inverted mapping gives s = k); points
a third of the way to the next plane keep k; Cartesian points follow the Cartesian
rule; a point above the topography is refused.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from tests.gpu_util import dev, host
from tests.topo_util import TopoCase, smooth_topo_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()


def _case():
    return TopoCase(30, 28, 22, 0.1, zmax_topo=1.0, amp=0.2, xc=1.4, yc=1.3, lx=0.6, ly=0.5, gp=5)


def _ew(c, precision=sg.FP64):
    g = sg.grid_desc(c.nx, c.ny, c.ncart, c.h, bc=c.bc, zmin=c.zmax_topo, sg_gp=c.grid.sg_gp,
                     sg_damping=c.grid.sg_damping, precision=precision)
    ew = sg.EW(g, topo=sg.topo_desc(**c.hill))
    ew.set_material(*[dev(a) for a in c.cart_mat])
    ew.set_material_grid(1, *[dev(a) for a in c.curv_mat])
    ew.add_source(sg.source_desc(1.5, 1.4, 0.5, moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=6.0))
    return ew


# (ijk, mode, grid): every mode on the curvilinear grid (surface, interior, next to the
# interface), and two on the Cartesian grid
RECS = [((17, 15, 1), sg.REC_DISPLACEMENT, 1), ((17, 15, 1), sg.REC_VELOCITY, 1),
        ((12, 10, 4), sg.REC_DIV, 1), ((20, 8, 7), sg.REC_CURL, 1), ((9, 20, 2), sg.REC_STRAINS, 1),
        ((14, 14, 9), sg.REC_GRADIENT, 1), ((10, 12, 5), sg.REC_DISPLACEMENT, 0),
        ((20, 9, 11), sg.REC_STRAINS, 0)]


def _expected(u, um, dt, h, met, jac, ijk, mode, grid):
    """One receiver's values from level u (and u^{n-1} = um) as [c, k, j, i] arrays."""
    i, j, k = ijk
    at = lambda c, di, dj, dk: u[c, k + 1 + dk, j + 1 + dj, i + 1 + di]  # arrays start at index -1
    if mode == sg.REC_DISPLACEMENT:
        return [at(c, 0, 0, 0) for c in range(3)]
    if mode == sg.REC_VELOCITY:
        return [(at(c, 0, 0, 0) - um[c, k + 1, j + 1, i + 1]) / (2 * dt) for c in range(3)]
    dq = [at(c, 1, 0, 0) - at(c, -1, 0, 0) for c in range(3)]
    dr = [at(c, 0, 1, 0) - at(c, 0, -1, 0) for c in range(3)]
    ds = [at(c, 0, 0, 1) - at(c, 0, 0, -1) for c in range(3)]
    if grid == 0:
        f = 1.0 / (2 * h)
        g = [[dq[c] * f, dr[c] * f, ds[c] * f] for c in range(3)]
        if mode == sg.REC_DIV:
            return [(dq[0] + dr[1] + ds[2]) * f]
        if mode == sg.REC_CURL:
            return [g[2][1] - g[1][2], g[0][2] - g[2][0], g[1][0] - g[0][1]]
    else:
        m = [met[q, k + 1, j + 1, i + 1] for q in range(4)]
        f = 0.5 / np.sqrt(jac[k + 1, j + 1, i + 1])
        if mode == sg.REC_DIV:
            return [(m[0] * dq[0] + m[0] * dr[1] + m[1] * ds[0] + m[2] * ds[1] + m[3] * ds[2]) * f]
        d = [[m[0] * dq[c] + m[1] * ds[c], m[0] * dr[c] + m[2] * ds[c], m[3] * ds[c]] for c in range(3)]
        if mode == sg.REC_CURL:
            return [(d[2][1] - d[1][2]) * f, (d[0][2] - d[2][0]) * f, (d[1][0] - d[0][1]) * f]
        g = [[d[c][a] * f for a in range(3)] for c in range(3)]
    if mode == sg.REC_STRAINS:
        return [g[0][0], g[1][1], g[2][2], 0.5 * (g[1][0] + g[0][1]), 0.5 * (g[2][0] + g[0][2]),
                0.5 * (g[1][2] + g[2][1])]
    return [g[c][a] for c in range(3) for a in range(3)]


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
def test_curvilinear_receivers_match_formulas(precision):
    c = _case()
    nsteps = 6
    dt = c.time_step(1.3)
    ew = _ew(c, precision)
    ew.set_time_step(dt, 0.0)
    fields = smooth_topo_fields(c, seed=7)
    ew.set_fields(dev(fields[0]), dev(fields[1]))
    ew.set_fields_grid(1, dev(fields[2]), dev(fields[3]))
    ew.set_receivers([r[0] for r in RECS], [r[1] for r in RECS], nsteps + 1, grids=[r[2] for r in RECS])
    nc = ew.grid_dims(1)[2]
    shp = {0: (3, c.ncart + 4, c.ny + 4, c.nx + 4), 1: (3, nc + 4, c.ny + 4, c.nx + 4)}
    n1 = ew.grid_dims(1)[3]
    met, jac = dev(np.zeros(4 * n1)), dev(np.zeros(n1))
    ew.curvilinear_arrays(met=met, jac=jac)
    met = host(met).reshape(4, nc + 4, c.ny + 4, c.nx + 4)
    jac = host(jac).reshape(nc + 4, c.ny + 4, c.nx + 4)

    def levels():
        out = {}
        for gi in (0, 1):
            u, um = dev(np.zeros(int(np.prod(shp[gi])))), dev(np.zeros(int(np.prod(shp[gi]))))
            if gi == 0:
                ew.get_fields(u, um)
            else:
                ew.get_fields_grid(1, u, um)
            out[gi] = (host(u).reshape(shp[gi]), host(um).reshape(shp[gi]))
        return out

    want = []
    prev = levels()
    want.append([v for (ijk, mode, gi) in RECS
                 for v in (_expected(prev[gi][0], prev[gi][1], dt, c.h, met, jac, ijk, mode, gi)
                           if mode != sg.REC_VELOCITY else [0.0, 0.0, 0.0])])
    for _ in range(nsteps):
        ew.step(1, sg.MODE_FUSED)
        now = levels()
        row = []
        for ijk, mode, gi in RECS:
            # velocity: (u^{n+1} - u^{n-1}) / (2 dt), u^{n-1} the level before this step's um
            um = prev[gi][1] if mode == sg.REC_VELOCITY else now[gi][1]
            row += _expected(now[gi][0], um, dt, c.h, met, jac, ijk, mode, gi)
        want.append(row)
        prev = now
    got = ew.records()
    ew.close()
    want = np.asarray(want)
    assert got.shape == want.shape
    for col in range(want.shape[1]):
        scale = np.abs(want[:, col]).max()
        assert scale > 0
        assert np.abs(got[:, col] - want[:, col]).max() <= 1e-12 * scale, col


def test_curvilinear_receivers_refused_without_topography_or_out_of_range():
    g = sg.grid_desc(20, 20, 20, 0.1)
    ew = sg.EW(g)
    with pytest.raises(sg.Sw4gError):
        ew.set_receivers([(5, 5, 5)], [sg.REC_DISPLACEMENT], 4, grids=[1])
    ew.close()
    c = _case()
    ew = _ew(c)
    nc = ew.grid_dims(1)[2]
    with pytest.raises(sg.Sw4gError):  # a derivative mode needs the neighbours in the array
        ew.set_receivers([(10, 10, nc + 2)], [sg.REC_STRAINS], 4, grids=[1])
    with pytest.raises(sg.Sw4gError):
        ew.set_receivers([(10, 10, 3)], [sg.REC_DISPLACEMENT], 4, grids=[2])
    ew.set_receivers([(10, 10, nc + 2)], [sg.REC_DISPLACEMENT], 4, grids=[1])
    ew.close()


def test_nearest_grid_point_on_both_grids():
    c = _case()
    ew = _ew(c)
    nc = ew.grid_dims(1)[2]
    n1 = ew.grid_dims(1)[3]
    z = dev(np.zeros(n1))
    ew.curvilinear_arrays(z=z)
    z = host(z).reshape(nc + 4, c.ny + 4, c.nx + 4)
    h = c.h
    rng = np.random.default_rng(3)
    for _ in range(40):
        i, j = int(rng.integers(1, c.nx + 1)), int(rng.integers(1, c.ny + 1))
        k = int(rng.integers(1, nc))
        x, y = (i - 1) * h, (j - 1) * h
        zk, zk1 = z[k + 1, j + 1, i + 1], z[k + 2, j + 1, i + 1]
        for zz, want in ((zk, k), (zk + 0.3 * (zk1 - zk), k), (zk1 - 0.3 * (zk1 - zk), k + 1)):
            assert ew.nearest_grid_point(x, y, zz) == ((i, j, want), 1)
    # the surface, by depth 0 below it
    x, y = 1.37, 1.21
    (i, j, k), grid = ew.nearest_grid_point(x, y, ew.topography_z(x, y))
    assert (i, j, k, grid) == (int(round(x / h)) + 1, int(round(y / h)) + 1, 1, 1)
    hill = c.hill
    assert ew.topography_z(x, y) == pytest.approx(
        -hill["amp"] * np.exp(-((x - hill["xc"]) / hill["lx"]) ** 2 - ((y - hill["yc"]) / hill["ly"]) ** 2),
        rel=1e-15)
    # the Cartesian grid below the interface
    assert ew.nearest_grid_point(0.52, 0.48, c.zmax_topo + 3.26 * h) == ((6, 6, 4), 0)
    with pytest.raises(sg.Sw4gError):  # above the topography
        ew.nearest_grid_point(x, y, ew.topography_z(x, y) - 0.01)
    ew.close()
