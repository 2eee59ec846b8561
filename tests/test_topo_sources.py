"""Sources in the two-grid (topography) set-up, host side (no GPU).

The library's discretisation (sw4g_discretize_source_topo) against the numpy
restatement in tests/topo_util.py, for sources in the curvilinear grid (graded
part under the hill, its uniform part), across the interface from either side
and in the Cartesian grid, point forces and moment tensors: every grid-point
amplitude to 1e-12 relative to the largest.  Properties of the restatement: the
mapping inversion lands on z to 1e-9 (the Newton tolerance), and with a flat
topography the curvilinear weights are the Cartesian ones (J = h^3, z_s = h).
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.topo_util import TopoCase, curvilinear_s, discretize_two_grid


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _case(amp=0.2):
    return TopoCase(30, 28, 22, 0.1, zmax_topo=1.0, amp=amp, xc=1.4, yc=1.3, lx=0.6, ly=0.5, gp=5)


def _sources(c):
    x, y = 1.37, 1.21
    zs = -c.hill["amp"] * np.exp(-((x - c.hill["xc"]) / c.hill["lx"]) ** 2 -
                                 ((y - c.hill["yc"]) / c.hill["ly"]) ** 2)
    out = []
    for z in (zs + 0.13, zs + 0.47, 0.5 * (zs + 1.0), 0.91, 1.0, 1.04, 1.16, 1.6):
        out.append(sg.source_desc(x, y, z, force=(0.7, -0.3, 1.1), freq=5.0))
        out.append(sg.source_desc(x, y, z, moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=5.0))
    return out


def _lib_discretize(c, s):
    return sg.discretize_source_topo(c.grid, sg.topo_desc(**c.hill), c.nc, c.jac, s)


def _same(a, b):
    (ia, aa), (ib, ab) = a, b
    assert ia.shape == ib.shape
    if len(ia) == 0:
        return
    # compare as per-point sums (the two may list a point in different orders)
    def dense(ijk, amp):
        d = {}
        for p, v in zip(map(tuple, ijk), amp):
            d[p] = d.get(p, 0) + v
        return d
    da, db = dense(ia, aa), dense(ib, ab)
    assert da.keys() == db.keys()
    scale = max(np.max(np.abs(ab)), 1e-300)
    for p in da:
        assert np.max(np.abs(da[p] - db[p])) <= 1e-12 * scale, p


@pytest.mark.parametrize("amp", [0.2, 0.0])
def test_library_matches_restatement(amp):
    c = _case(amp)
    for s in _sources(c):
        lc, lv = _lib_discretize(c, s)
        pc, pv = discretize_two_grid(c, s)
        _same(lc, pc)
        _same(lv, pv)


def test_grid_choice_and_interface_split():
    c = _case()
    deep = sg.source_desc(1.37, 1.21, 1.6, force=(0, 0, 1.0))
    (cart, curv) = _lib_discretize(c, deep)
    assert len(cart[0]) > 0 and len(curv[0]) == 0
    # one plane below the interface: the stencil reaches into the curvilinear grid
    near = sg.source_desc(1.37, 1.21, 1.04, force=(0, 0, 1.0))
    (cart, curv) = _lib_discretize(c, near)
    assert len(cart[0]) > 0 and len(curv[0]) > 0
    assert set(curv[0][:, 2]) <= {c.nc - 2, c.nc - 1, c.nc}
    # just above the interface: in the curvilinear grid, split into the Cartesian one
    up = sg.source_desc(1.37, 1.21, 0.96, force=(0, 0, 1.0))
    (cart, curv) = _lib_discretize(c, up)
    assert len(curv[0]) > 0 and len(cart[0]) > 0
    assert set(cart[0][:, 2]) <= {1, 2, 3}
    above = sg.source_desc(1.4, 1.3, -0.5, force=(0, 0, 1.0))
    with pytest.raises(sg.Sw4gError):
        _lib_discretize(c, above)


def test_mapping_inversion_and_flat_topography():
    c = _case()
    z = c.z.reshape(c.nc + 4, c.ny + 4, c.nx + 4)
    # a grid point of the curvilinear grid maps back to its own s
    for (i, j, k) in ((14, 13, 2), (14, 13, 5), (5, 20, 9), (20, 6, 11)):
        s = curvilinear_s(c, i, j, z[k + 1, j + 1, i + 1])
        assert abs(s - k) <= 1e-8
    # flat topography: the curvilinear grid is uniform, its point force weights equal
    # the Cartesian weights of the same point in an equivalent Cartesian grid
    f = _case(0.0)
    s = sg.source_desc(1.37, 1.21, 0.55, force=(0.7, -0.3, 1.1), freq=5.0)
    _, (ijk, amp) = discretize_two_grid(f, s)
    g = sg.grid_desc(30, 28, f.nc, 0.1, bc=(2, 2, 2, 2, 0, 2), zmin=1.0 - (f.nc - 1) * 0.1, sg_gp=5)
    from tests.gpu_util import discretize
    cijk, camp = discretize(g, s)
    d = {tuple(p): a for p, a in zip(cijk.reshape(-1, 3), camp.reshape(-1, 3))}
    for p, a in zip(map(tuple, ijk), amp):
        assert np.allclose(a, d[p], rtol=1e-10, atol=1e-12 * np.max(np.abs(camp)))
