"""Curvilinear-grid kernels on the GPU against the oracle (pinned to the
reference's kernels in tests/test_oracle_curv_pin.py).

Tolerances, relative to the output's largest magnitude: 1e-13 for the operator,
the free surface and the damping (rounding of the same formulas in another
order), 1e-14 for the metric and the grid, 1e-13 for the time step.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.gpu_util import dev, host
from tests.test_oracle_curv_pin import _fields, _from_aos, _to_aos

pytestmark = pytest.mark.gpu

H = 0.1


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _setup(nx, ny, nz, seed=3):
    b = (-1, nx + 2, -1, ny + 2, -1, nz + 2)
    hill = dict(zmax=(nz - 1) * H, amp=0.25, xc=0.45 * nx * H, yc=0.55 * ny * H, lx=0.3 * nx * H,
                ly=0.25 * ny * H)
    z = O.gaussian_hill_z(b, nz, H, **hill)
    n = z.size
    met, jac = np.zeros(4 * n), np.zeros(n)
    assert O.metric(1, b, H, z, met, jac) == 0
    return b, hill, z, met, jac


def test_gaussian_hill_grid_and_metric():
    nx, ny, nz = 20, 17, 15
    b, hill, z, met, jac = _setup(nx, ny, nz)
    zd = dev(np.zeros_like(z))
    sg.check(sg.lib().sw4g_gaussian_hill_grid(*b, nz, H, hill["zmax"], 0.95, 4, hill["amp"],
                                              hill["xc"], hill["yc"], hill["lx"], hill["ly"],
                                              zd.data_ptr(), None), "hill")
    assert _rel(host(zd), z) <= 1e-14
    for soa in (1, 0):
        md, jd = dev(np.zeros_like(met)), dev(np.zeros_like(jac))
        sg.check(sg.lib().sw4g_metric(soa, *b, H, dev(z).data_ptr(), md.data_ptr(), jd.data_ptr(),
                                      None), "metric")
        m = host(md) if soa else _from_aos(host(md), 4)
        assert _rel(m, met) <= 1e-14
        assert _rel(host(jd), jac) <= 1e-14


def test_metric_of_folded_grid_is_rejected():
    nx, ny, nz = 10, 10, 10
    b, _, z, met, jac = _setup(nx, ny, nz)
    z = z.copy()
    z.reshape(nz + 4, ny + 4, nx + 4)[5, 6, 6] -= 5.0
    zd, md, jd = dev(z), dev(np.zeros_like(met)), dev(np.zeros_like(jac))
    st = sg.lib().sw4g_metric(1, *b, H, zd.data_ptr(), md.data_ptr(), jd.data_ptr(), None)
    assert st == 1  # SW4G_BAD_ARGUMENT


@pytest.mark.parametrize("soa", [1, 0])
@pytest.mark.parametrize("top", [1, 0])
@pytest.mark.parametrize("shape", [(15, 13, 17), (40, 33, 12)])
def test_rhs4sgcurv_matches_oracle(soa, top, shape):
    nx, ny, nz = shape
    b, _, z, met, jac = _setup(nx, ny, nz)
    u, mu, la, _, sx, sy = _fields(nx, ny, nz, seed=3 + top)
    onesided = (0, 0, 0, 0, top, 0)
    ref = np.zeros_like(u)
    O.rhs4sgcurv(1, b, onesided, ref, u, mu, la, met, jac, sx, sy)
    uu, mm = (u, met) if soa else (_to_aos(u, 3), _to_aos(met, 4))
    keep = [dev(a) for a in (uu, mu, la, mm, jac, sx, sy)]
    lu = dev(np.zeros_like(u))
    os_arr = np.asarray(onesided, dtype=np.int32)
    sg.check(sg.lib().sw4g_rhs4sgcurv(soa, *b, os_arr.ctypes.data_as(sg._I), lu.data_ptr(),
                                      *[k.data_ptr() for k in keep], None), "rhs4sgcurv")
    got = host(lu) if soa else _from_aos(host(lu), 3)
    assert _rel(got, ref) <= 1e-13


@pytest.mark.parametrize("soa", [1, 0])
def test_freesurfcurvisg_matches_oracle(soa):
    nx, ny, nz = 18, 16, 12
    b, _, z, met, jac = _setup(nx, ny, nz)
    u, mu, la, _, sx, sy = _fields(nx, ny, nz, seed=11)
    _, _, _, sbop = O.stencil_coefficients()
    forcing = np.random.default_rng(2).standard_normal(3 * (nx + 4) * (ny + 4)) * 0.1
    ref = u.copy()
    O.freesurfcurvisg(1, b, nz, 5, ref, mu, la, met, sbop, forcing, sx, sy)
    uu, mm = (u.copy(), met) if soa else (_to_aos(u, 3), _to_aos(met, 4))
    ud = dev(uu)
    keep = [dev(a) for a in (mu, la, mm)]
    fd, sxd, syd = dev(forcing), dev(sx), dev(sy)
    sbop_c = np.ascontiguousarray(sbop)
    sg.check(sg.lib().sw4g_freesurfcurvisg(soa, *b, nz, 5, ud.data_ptr(),
                                           *[k.data_ptr() for k in keep],
                                           sbop_c.ctypes.data_as(sg._D), fd.data_ptr(),
                                           sxd.data_ptr(), syd.data_ptr(), None), "freesurf")
    got = host(ud) if soa else _from_aos(host(ud), 3)
    assert _rel(got, ref) <= 1e-13


@pytest.mark.parametrize("soa", [1, 0])
@pytest.mark.parametrize("order", [4, 6])
def test_addsgd4c_matches_oracle(soa, order):
    nx, ny, nz = 17, 14, 11
    b, _, z, met, jac = _setup(nx, ny, nz)
    u, mu, la, rho, sx, sy = _fields(nx, ny, nz, seed=5)
    um, up0 = np.roll(u, 7) * 0.9, np.roll(u, 3)
    rng = np.random.default_rng(9)
    dcx, dcy = rng.random(nx + 4) * 0.1, rng.random(ny + 4) * 0.1
    cox, coy = 0.5 + rng.random(nx + 4), 0.5 + rng.random(ny + 4)
    ref = up0.copy()
    O.addsgd4c(1, b, ref, u, um, rho, dcx, dcy, sx, sy, jac, cox, coy, 0.02, order=order)
    cv = (lambda a: a) if soa else (lambda a: _to_aos(a, 3))
    upd = dev(cv(up0))
    keep = [dev(a) for a in (cv(u), cv(um), rho, dcx, dcy, sx, sy, jac, cox, coy)]
    fn = sg.lib().sw4g_addsgd6cfort if order == 6 else sg.lib().sw4g_addsgd4cfort
    sg.check(fn(soa, *b, upd.data_ptr(), *[k.data_ptr() for k in keep], 0.02, None), "addsgd c")
    got = host(upd) if soa else _from_aos(host(upd), 3)
    assert _rel(got - up0, ref - up0) <= 1e-13


def test_curvilinear_time_step_matches_oracle():
    nx, ny, nz = 20, 18, 14
    b, _, z, met, jac = _setup(nx, ny, nz)
    _, mu, la, rho, _, _ = _fields(nx, ny, nz, seed=8)
    keep = [dev(a) for a in (rho, mu, la, met, jac)]
    import ctypes as C
    dt = C.c_double()
    sg.check(sg.lib().sw4g_curvilinear_time_step(1, *b, *[k.data_ptr() for k in keep], 1.3,
                                                 C.byref(dt), None), "curv dt")
    assert dt.value == pytest.approx(O.curv_dt(1, b, rho, mu, la, met, jac, 1.3), rel=1e-13)
