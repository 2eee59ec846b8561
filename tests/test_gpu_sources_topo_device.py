"""Two-grid (topography) source discretisation on the device against the host path
(the curvilinear branches of Source::set_grid_point_sources4, src/Source.C:1530-1990,
and the grid choice of src/EW.C:5149-5213).

The device kernel evaluates the same stencil code as the host (source_weights.h) on
the Jacobian in device memory.  The Cartesian weights are bit-identical; the
curvilinear ones call exp and pow (topography, grid mapping, metric at the source),
whose device results may differ from the host's in the last bit, so the lists agree
in their grid points and order exactly and in their amplitudes to 1e-13 of the
largest.  The sources cover the graded part of the curvilinear grid under the hill,
its uniform part, stencils across the interface from either side, the Cartesian grid,
the side clamps and overlapping stencils.  Checks: the lists per grid against the
host's (grouped by grid point, host order within a point), per-point sums against the
numpy restatement (tests/topo_util.py) to 1e-12, the fields after a run against a run
on the host lists to 1e-12, and the host path's refusals (a source above the
topography) on the device path too.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.gpu_util import dev, host
from tests.topo_util import TopoCase, discretize_two_grid, smooth_topo_fields

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _case():
    return TopoCase(30, 28, 22, 0.1, zmax_topo=1.0, amp=0.2, xc=1.4, yc=1.3, lx=0.6, ly=0.5, gp=5)


def _sources(c, seed=21, n=30):
    x, y = 1.37, 1.21
    zs = -c.hill["amp"] * np.exp(-((x - c.hill["xc"]) / c.hill["lx"]) ** 2 -
                                 ((y - c.hill["yc"]) / c.hill["ly"]) ** 2)
    out = []
    # graded part, uniform part, across the interface from above and below, Cartesian
    for q, z in enumerate((zs + 0.13, zs + 0.47, 0.5 * (zs + 1.0), 0.91, 1.0, 1.04, 1.16, 1.6)):
        out.append(sg.source_desc(x, y, z, force=(0.7, -0.3, 1.1), freq=5.0 + q, t0=0.05))
        out.append(sg.source_desc(x, y, z, moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=6.0,
                                  kind=sg.C6SMOOTHBUMP))
    rng = np.random.default_rng(seed)
    for q in range(n):
        sx, sy = rng.uniform(0.0, (c.nx - 1) * c.h), rng.uniform(0.0, (c.ny - 1) * c.h)
        top = -c.hill["amp"] * np.exp(-((sx - c.hill["xc"]) / c.hill["lx"]) ** 2 -
                                      ((sy - c.hill["yc"]) / c.hill["ly"]) ** 2)
        sz = rng.uniform(top + 0.02, 1.0 + (c.ncart - 1) * c.h)
        kind = int(rng.integers(0, 4))
        if q % 2:
            out.append(sg.source_desc(sx, sy, sz, moment=tuple(rng.standard_normal(6)), freq=6.0 + q,
                                      t0=0.01 * q, kind=kind))
        else:
            out.append(sg.source_desc(sx, sy, sz, force=tuple(rng.standard_normal(3)), freq=5.0 + q,
                                      t0=0.02 * q, kind=kind))
    # two sources one point apart next to the interface: overlapping split stencils
    out.append(sg.source_desc(1.5, 1.4, 0.98, force=(1.0, 2.0, 3.0), freq=7.0))
    out.append(sg.source_desc(1.6, 1.4, 1.03, moment=(1, 0, 0, 1, 0, 1), freq=7.0))
    return out


def _ew(c, on_device, srcs):
    ew = sg.EW(c.grid, topo=sg.topo_desc(**c.hill))
    ew.set_material(*[dev(a) for a in c.cart_mat])
    ew.set_material_grid(1, *[dev(a) for a in c.curv_mat])
    if on_device:
        ew.set_source_discretization(True)
    for s in srcs:
        ew.add_source(s)
    return ew


def _grouped(ijk, amp):
    """The host list in the forcing's order: stable by grid point (k, j, i)."""
    order = np.lexsort((ijk[:, 0], ijk[:, 1], ijk[:, 2]))
    return ijk[order], amp[order]


def _per_point(ijk, amp):
    d = {}
    for p, v in zip(map(tuple, ijk), amp):
        d[p] = d.get(p, np.zeros(3)) + v
    return d


def test_device_lists_match_host_lists():
    c = _case()
    srcs = _sources(c)
    a, b = _ew(c, False, srcs), _ew(c, True, srcs)
    for grid in (0, 1):
        ha, aa = _grouped(*a.grid_point_sources(grid))
        hb, ab = b.grid_point_sources(grid)
        assert len(ha) == len(hb) > 0
        assert np.array_equal(ha, hb)
        scale = np.abs(aa).max()
        assert np.abs(aa - ab).max() <= 1e-13 * scale
    a.close()
    b.close()


def test_device_lists_match_the_restatement():
    c = _case()
    srcs = _sources(c, seed=5, n=12)
    ew = _ew(c, True, srcs)
    got = [_per_point(*ew.grid_point_sources(grid)) for grid in (0, 1)]
    ew.close()
    want = [{}, {}]
    for s in srcs:
        for grid, (ijk, amp) in enumerate(discretize_two_grid(c, s)):
            for p, v in _per_point(ijk, amp).items():
                want[grid][p] = want[grid].get(p, np.zeros(3)) + v
    for g, w in zip(got, want):
        scale = max(np.abs(v).max() for v in w.values())
        big = lambda d: {k for k, v in d.items() if np.abs(v).max() > 1e-12 * scale}
        assert big(g) == big(w)
        err = max(np.abs(g.get(k, np.zeros(3)) - w.get(k, np.zeros(3))).max() for k in set(g) | set(w))
        assert err <= 1e-12 * scale


def test_run_with_device_lists_matches_host_lists():
    c = _case()
    srcs = _sources(c, seed=8, n=10)
    dt = c.time_step(1.3)
    fields = smooth_topo_fields(c, seed=3)
    out = []
    for on_device in (False, True):
        ew = _ew(c, on_device, srcs)
        ew.set_time_step(dt, 0.0)
        ew.set_fields(dev(fields[0]), dev(fields[1]))
        ew.set_fields_grid(1, dev(fields[2]), dev(fields[3]))
        ew.step(10, sg.MODE_FUSED)
        r = [dev(np.zeros_like(f)) for f in fields[::2]]
        ew.get_fields(r[0], None)
        ew.get_fields_grid(1, r[1], None)
        out.append([host(x) for x in r])
        ew.close()
    for x, y in zip(*out):
        assert np.max(np.abs(x - y)) <= 1e-12 * np.max(np.abs(y))


def test_switching_back_to_the_host_rebuilds_both_lists():
    c = _case()
    srcs = _sources(c, seed=2, n=6)
    a, b = _ew(c, False, srcs), _ew(c, True, srcs)
    b.set_source_discretization(False)
    for grid in (0, 1):
        ha, aa = a.grid_point_sources(grid)
        hb, ab = b.grid_point_sources(grid)
        assert np.array_equal(ha, hb) and np.array_equal(aa, ab)
    a.close()
    b.close()


def test_device_path_keeps_the_host_refusals():
    c = _case()
    ew = _ew(c, True, [])
    with pytest.raises(sg.Sw4gError):  # above the topography (the hill top is at z = -0.2)
        ew.add_source(sg.source_desc(1.4, 1.3, -0.5, force=(1.0, 0, 0)))
    ew.add_source(sg.source_desc(1.0, 1.0, 0.5, force=(1.0, 0, 0)))  # in the curvilinear grid
    assert len(ew.grid_point_sources(1)[0]) > 0 and len(ew.grid_point_sources(0)[0]) == 0
    ew.close()


def test_mixed_run_with_device_lists_matches_host_lists():
    """The FP32-mixed two-grid loop with the device lists against the host lists.  The
    lists differ at most in the last bits of exp/pow, but such a difference can flip
    an FP32 rounding in the stencil, so the runs agree to the mixed form's own
    scale: 1e-7 of the field maximum after 10 steps."""
    c = _case()
    srcs = _sources(c, seed=4, n=8)
    dt = c.time_step(1.3)
    fields = smooth_topo_fields(c, seed=5)
    g = sg.grid_desc(c.nx, c.ny, c.ncart, c.h, bc=c.bc, zmin=c.zmax_topo, sg_gp=c.grid.sg_gp,
                     sg_damping=c.grid.sg_damping, precision=sg.MIXED)
    out = []
    for on_device in (False, True):
        ew = sg.EW(g, topo=sg.topo_desc(**c.hill))
        ew.set_material(*[dev(a) for a in c.cart_mat])
        ew.set_material_grid(1, *[dev(a) for a in c.curv_mat])
        if on_device:
            ew.set_source_discretization(True)
        for s in srcs:
            ew.add_source(s)
        ew.set_time_step(dt, 0.0)
        ew.set_fields(dev(fields[0]), dev(fields[1]))
        ew.set_fields_grid(1, dev(fields[2]), dev(fields[3]))
        ew.step(10, sg.MODE_FUSED)
        r = [dev(np.zeros_like(f)) for f in fields[::2]]
        ew.get_fields(r[0], None)
        ew.get_fields_grid(1, r[1], None)
        out.append([host(x) for x in r])
        ew.close()
    for x, y in zip(*out):
        assert np.all(np.isfinite(x))
        assert np.max(np.abs(x - y)) <= 1e-7 * np.max(np.abs(y))
