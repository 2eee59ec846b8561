"""Restart files in the reference's checkpoint format (sw4g_ew_write_checkpoint /
sw4g_ew_read_checkpoint; src/CheckPoint.C:251-470, restart at src/EW.C:2403-2415).

* The library's file matches the reference's layout (tests/checkpoint_format.py):
  header, grid sizes, and the interior of both levels exactly.
* A run restarted from a file continues bit for bit (FP64, one grid and the two-grid
  topography set-up) at every point but the outer ghost plane above a free surface,
  which no boundary condition sets and no stencil reads (it holds whatever the
  pointwise update left there, a function of the run's history, not of the file);
  the FP32-mixed form writes its double-float levels as FP64 and splits them again, so
  it continues to within the form's rounding.
* A file written from the oracle's levels (the reference CPU time loop) restarts the
  GPU run, which then matches the oracle's own continuation to 1e-12.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests import checkpoint_format as CF
from tests.fields import rel_err
from tests.gpu_util import OracleProblem, dev, host, smooth_fields, smooth_material

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _case(precision=sg.FP64):
    nx, ny, nz, h = 30, 28, 26, 0.05
    g = sg.grid_desc(nx, ny, nz, h, bc=(2, 2, 2, 2, 0, 2), sg_gp=7, sg_damping=0.02, precision=precision)
    mat = smooth_material(nx, ny, nz, seed=3)
    fields = smooth_fields(nx, ny, nz, seed=5)
    srcs = [sg.source_desc(0.45 * nx * h, 0.5 * ny * h, 0.4 * nz * h, force=(1.0, -0.5, 0.25), freq=8.0,
                           t0=0.05, kind=sg.GAUSSIAN),
            sg.source_desc(0.6 * nx * h, 0.4 * ny * h, 0.55 * nz * h, moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6),
                           freq=6.0, kind=sg.C6SMOOTHBUMP)]
    dt = 0.3 * h / np.sqrt(np.max((4 * mat[1] + mat[2]) / mat[0]))
    return g, mat, fields, srcs, dt


def _ew(g, mat, srcs, dt):
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in mat])
    for s in srcs:
        ew.add_source(s)
    ew.set_time_step(dt, 0.0)
    return ew


def _defined(grid_shape, free_top=True):
    """Mask of the points a restart reproduces: all but the outer ghost plane above a
    free surface (array plane 0)."""
    nz, ny, nx = grid_shape
    m = np.ones((3, nz + 4, ny + 4, nx + 4), dtype=bool)
    if free_top:
        m[:, 0] = False
    return m.reshape(-1)


def _levels(ew):
    u = dev(np.zeros(3 * ew.npts))
    um = dev(np.zeros(3 * ew.npts))
    ew.get_fields(u, um)
    return host(u), host(um)


def test_file_matches_reference_layout(tmp_path):
    g, mat, fields, srcs, dt = _case()
    ew = _ew(g, mat, srcs, dt)
    ew.set_fields(dev(fields[0]), dev(fields[1]))
    ew.step(5, sg.MODE_FUSED)
    p = tmp_path / "restart.cycle=5.sw4checkpoint"
    ew.write_checkpoint(str(p), 5)
    u, um = _levels(ew)
    t = ew.time
    ew.close()
    r = CF.read(p)
    assert (r["prec"], r["cycle"], r["time"]) == (8, 5, t)
    assert r["sizes"] == [[1, g.nx, 1, g.ny, 1, g.nz]]
    bum, bu = r["blocks"][0]
    assert np.array_equal(bum, CF.interior_block(um, g.nx, g.ny, g.nz))
    assert np.array_equal(bu, CF.interior_block(u, g.nx, g.ny, g.nz))


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
def test_restart_continues_the_run(tmp_path, precision):
    g, mat, fields, srcs, dt = _case(precision)
    n1, n2 = 7, 9
    p = tmp_path / "restart.sw4checkpoint"
    a = _ew(g, mat, srcs, dt)
    a.set_fields(dev(fields[0]), dev(fields[1]))
    a.step(n1, sg.MODE_FUSED)
    a.write_checkpoint(str(p), n1)
    a.step(n2, sg.MODE_FUSED)
    ua, uma = _levels(a)
    ta = a.time
    a.close()
    b = _ew(g, mat, srcs, dt)
    assert b.read_checkpoint(str(p)) == n1
    assert b.time == n1 * dt or abs(b.time - n1 * dt) < 1e-15
    b.step(n2, sg.MODE_FUSED)
    ub, umb = _levels(b)
    tb = b.time
    b.close()
    assert ta == tb
    assert np.max(np.abs(ua)) > 0
    m = _defined((g.nz, g.ny, g.nx))
    if precision == sg.FP64:
        assert np.array_equal(ua[m], ub[m]) and np.array_equal(uma[m], umb[m])
    else:  # a (hi, lo) pair whose lo is half an ulp of hi may come back split differently
        assert rel_err(ub[m], ua[m]) <= 1e-12 and rel_err(umb[m], uma[m]) <= 1e-12


def test_restart_topography_bit_identical(tmp_path):
    from tests.test_gpu_topo import _long_case
    from tests.topo_util import smooth_topo_fields
    c = _long_case()
    dt = c.time_step(1.3)
    fields = smooth_topo_fields(c, seed=6)
    p = tmp_path / "topo.sw4checkpoint"

    def make():
        ew = sg.EW(c.grid, topo=sg.topo_desc(**c.hill))
        ew.set_material(*[dev(q) for q in c.cart_mat])
        ew.set_material_grid(1, *[dev(q) for q in c.curv_mat])
        for s in c.sources:
            ew.add_source(s)
        ew.set_time_step(dt, 0.0)
        return ew

    def levels(ew):
        res = [dev(np.zeros_like(f)) for f in fields]
        ew.get_fields(res[0], res[1])
        ew.get_fields_grid(1, res[2], res[3])
        return [host(r) for r in res]

    a = make()
    a.set_fields(dev(fields[0]), dev(fields[1]))
    a.set_fields_grid(1, dev(fields[2]), dev(fields[3]))
    a.step(11, sg.MODE_FUSED)
    a.write_checkpoint(str(p), 11)
    a.step(13, sg.MODE_FUSED)
    ra = levels(a)
    a.close()
    r = CF.read(p)
    assert len(r["sizes"]) == 2 and r["cycle"] == 11
    b = make()
    assert b.read_checkpoint(str(p)) == 11
    b.step(13, sg.MODE_FUSED)
    rb = levels(b)
    b.close()
    g = c.grid
    nzc = (len(fields[2]) // 3) // ((g.nx + 4) * (g.ny + 4)) - 4
    masks = [_defined((g.nz, g.ny, g.nx), free_top=False)] * 2 + [_defined((nzc, g.ny, g.nx))] * 2
    for x, y, m in zip(ra, rb, masks):
        assert np.array_equal(x[m], y[m])
    assert max(np.max(np.abs(x)) for x in ra) > 0


def test_restart_from_oracle_levels(tmp_path):
    g, mat, fields, srcs, dt = _case()
    n1, n2 = 6, 5
    prob = OracleProblem(g, *mat, dt, srcs)
    u1, um1 = prob.run(*fields, 0.0, n1)
    p = tmp_path / "oracle.sw4checkpoint"
    CF.write(p, n1 * dt, n1, [(g.nx, g.ny, g.nz, um1, u1)])
    ref_u, ref_um = prob.run(*fields, 0.0, n1 + n2)
    ew = _ew(g, mat, srcs, dt)
    assert ew.read_checkpoint(str(p)) == n1
    ew.step(n2, sg.MODE_FUSED)
    u, um = _levels(ew)
    ew.close()
    m = _defined((g.nz, g.ny, g.nx))
    assert rel_err(u[m], ref_u[m]) <= 1e-12
    assert rel_err(um[m], ref_um[m]) <= 1e-12


def test_bad_files_are_refused(tmp_path):
    g, mat, fields, srcs, dt = _case()
    ew = _ew(g, mat, srcs, dt)
    with pytest.raises(sg.Sw4gError):
        ew.read_checkpoint(str(tmp_path / "missing.sw4checkpoint"))
    p = tmp_path / "small.sw4checkpoint"
    CF.write(p, 0.0, 0, [(g.nx - 1, g.ny, g.nz, np.zeros(3 * (g.nx + 3) * (g.ny + 4) * (g.nz + 4)),
                          np.zeros(3 * (g.nx + 3) * (g.ny + 4) * (g.nz + 4)))])
    with pytest.raises(sg.Sw4gError):  # grid sizes differ
        ew.read_checkpoint(str(p))
    ew.close()
