"""The oracle's curvilinear restatement pinned to the reference's own kernels.

The reference's curvilinear kernels (rhs4sgcurv.C, rhs4sgcurv_rev.C,
curvilinear-c.C, ew-cfromfort.C) are compiled in place into oracle/_ref by
`make -C oracle ref`; these tests run both on the same seeded inputs.  They are
skipped where the reference tree is absent.

Tolerances: the restatement evaluates the same formulas in a different order
(table-driven terms, products formed once), so results agree to rounding:
1e-13 relative to the output's largest magnitude for the operator, the free
surface and the damping, 1e-14 for the metric.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference kernels not built here")


def _bounds(nx, ny, nz):
    return (-1, nx + 2, -1, ny + 2, -1, nz + 2)


def _hill(nx, ny, nz, h=0.1, amp=0.25):
    b = _bounds(nx, ny, nz)
    z = O.gaussian_hill_z(b, nz, h, zmax=(nz - 1) * h, amp=amp, xc=0.45 * nx * h,
                          yc=0.55 * ny * h, lx=0.3 * nx * h, ly=0.25 * ny * h)
    return b, z


def _to_aos(a, nc):
    return np.ascontiguousarray(a.reshape(nc, -1).T.reshape(-1))


def _from_aos(a, nc):
    return np.ascontiguousarray(a.reshape(-1, nc).T.reshape(-1))


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _fields(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    n = (nx + 4) * (ny + 4) * (nz + 4)
    k, j, i = np.meshgrid(np.arange(nz + 4), np.arange(ny + 4), np.arange(nx + 4), indexing="ij")
    u = np.concatenate([(np.sin(0.3 * i + 0.2 * c) * np.cos(0.25 * j - 0.1 * c) *
                         np.sin(0.35 * k + 0.3 * c)).reshape(-1) + 0.05 * rng.standard_normal(n)
                        for c in range(3)])
    mu = 1.0 + 0.3 * rng.random(n)
    la = 1.5 + 0.4 * rng.random(n)
    rho = 1.0 + 0.2 * rng.random(n)
    sx = 1.0 + 0.2 * rng.random(nx + 4)
    sy = 1.0 + 0.2 * rng.random(ny + 4)
    return u, mu, la, rho, sx, sy


@pytest.mark.parametrize("soa", [1, 0])
def test_metric_matches_reference(soa):
    nx, ny, nz = 14, 12, 16
    b, z = _hill(nx, ny, nz)
    n = z.size
    out = []
    for which in ("oracle", "ref"):
        met, jac = np.zeros(4 * n), np.zeros(n)
        assert O.metric(soa, b, 0.1, z, met, jac, which=which) == 0
        out.append((met, jac))
    assert _rel(out[0][0], out[1][0]) <= 1e-14
    assert _rel(out[0][1], out[1][1]) <= 1e-14


def test_metric_rejects_folded_grid():
    nx, ny, nz = 10, 10, 10
    b, z = _hill(nx, ny, nz)
    z = z.copy()
    z.reshape(nz + 4, ny + 4, nx + 4)[5, 6, 6] = z.reshape(nz + 4, ny + 4, nx + 4)[3, 6, 6] - 1.0
    met, jac = np.zeros(4 * z.size), np.zeros(z.size)
    assert O.metric(1, b, 0.1, z, met, jac) == -1
    assert O.metric(1, b, 0.1, z, met, jac, which="ref") == -1


@pytest.mark.parametrize("soa", [1, 0])
@pytest.mark.parametrize("top", [1, 0])
def test_rhs4sgcurv_matches_reference(soa, top):
    nx, ny, nz = 15, 13, 17
    b, z = _hill(nx, ny, nz)
    n = z.size
    met, jac = np.zeros(4 * n), np.zeros(n)
    O.metric(1, b, 0.1, z, met, jac)
    u, mu, la, _, sx, sy = _fields(nx, ny, nz, seed=3 + top)
    onesided = (0, 0, 0, 0, top, 0)
    res = []
    for which in ("oracle", "ref"):
        lu = np.zeros(3 * n)
        if soa:
            O.rhs4sgcurv(1, b, onesided, lu, u, mu, la, met, jac, sx, sy, which=which)
        else:
            lua = np.zeros(3 * n)
            O.rhs4sgcurv(0, b, onesided, lua, _to_aos(u, 3), mu, la, _to_aos(met, 4), jac, sx, sy,
                         which=which)
            lu = _from_aos(lua, 3)
        res.append(lu)
    assert np.max(np.abs(res[1])) > 0
    assert _rel(res[0], res[1]) <= 1e-13


@pytest.mark.parametrize("soa", [1, 0])
def test_freesurfcurvisg_matches_reference(soa):
    nx, ny, nz = 14, 15, 12
    b, z = _hill(nx, ny, nz)
    n = z.size
    met, jac = np.zeros(4 * n), np.zeros(n)
    O.metric(1, b, 0.1, z, met, jac)
    u, mu, la, _, sx, sy = _fields(nx, ny, nz, seed=11)
    _, _, _, sbop = O.stencil_coefficients()
    forcing = np.random.default_rng(2).standard_normal(3 * (nx + 4) * (ny + 4)) * 0.1
    res = []
    for which in ("oracle", "ref"):
        if soa:
            w = u.copy()
            O.freesurfcurvisg(1, b, nz, 5, w, mu, la, met, sbop, forcing, sx, sy, which=which)
        else:
            w = _to_aos(u, 3)
            O.freesurfcurvisg(0, b, nz, 5, w, mu, la, _to_aos(met, 4), sbop, forcing, sx, sy,
                              which=which)
            w = _from_aos(w, 3)
        res.append(w)
    assert not np.array_equal(res[1], u)
    assert _rel(res[0], res[1]) <= 1e-13


@pytest.mark.parametrize("order", [4, 6])
@pytest.mark.parametrize("soa", [1, 0])
def test_addsgd4c_matches_reference(soa, order):
    nx, ny, nz = 13, 14, 11
    b, z = _hill(nx, ny, nz)
    n = z.size
    met, jac = np.zeros(4 * n), np.zeros(n)
    O.metric(1, b, 0.1, z, met, jac)
    u, mu, la, rho, sx, sy = _fields(nx, ny, nz, seed=5)
    um = np.roll(u, 7) * 0.9
    up0 = np.roll(u, 3)
    rng = np.random.default_rng(9)
    dcx, dcy = rng.random(nx + 4) * 0.1, rng.random(ny + 4) * 0.1
    cox, coy = 0.5 + rng.random(nx + 4), 0.5 + rng.random(ny + 4)
    res = []
    for which in ("oracle", "ref"):
        if soa:
            up = up0.copy()
            O.addsgd4c(1, b, up, u, um, rho, dcx, dcy, sx, sy, jac, cox, coy, 0.02, which=which,
                       order=order)
        else:
            up = _to_aos(up0, 3)
            O.addsgd4c(0, b, up, _to_aos(u, 3), _to_aos(um, 3), rho, dcx, dcy, sx, sy, jac, cox,
                       coy, 0.02, which=which, order=order)
            up = _from_aos(up, 3)
        res.append(up - up0)
    assert np.max(np.abs(res[1])) > 0
    assert _rel(res[0], res[1]) <= 1e-13


def test_symmetric_3x3_min_eigenvalue():
    rng = np.random.default_rng(4)
    for _ in range(200):
        m = rng.standard_normal((3, 3))
        a = -(m @ m.T + 0.01 * np.eye(3))
        six = [a[0, 0], a[0, 1], a[0, 2], a[1, 1], a[1, 2], a[2, 2]]
        ref = np.linalg.eigvalsh(a)[0]
        assert O.sym3_min_eig(six) == pytest.approx(ref, rel=1e-12, abs=1e-13)
    assert O.sym3_min_eig([-3, 0, 0, -1, 0, -2]) == -3


def test_curvilinear_time_step_matches_eigen_definition():
    nx, ny, nz = 10, 9, 12
    b, z = _hill(nx, ny, nz)
    n = z.size
    met, jac = np.zeros(4 * n), np.zeros(n)
    O.metric(1, b, 0.1, z, met, jac)
    _, mu, la, rho, _, _ = _fields(nx, ny, nz, seed=8)
    m = met.reshape(4, -1)
    eigmax = -1.0
    for p in range(n):
        m1, m2, m3, m4 = m[:, p]
        l2m, mm, ll, ji = la[p] + 2 * mu[p], mu[p], la[p], 1 / jac[p]
        A = -4 * ji * np.array([
            [m1 * m1 * (l2m + mm) + m2 * m2 * l2m + (m3 * m3 + m4 * m4) * mm, m2 * m3 * (mm + ll), m2 * m4 * (mm + ll)],
            [m2 * m3 * (mm + ll), m1 * m1 * (mm + l2m) + m2 * m2 * mm + m3 * m3 * l2m + m4 * m4 * mm, m3 * m4 * (mm + ll)],
            [m2 * m4 * (mm + ll), m3 * m4 * (mm + ll), m1 * m1 * 2 * mm + (m2 * m2 + m3 * m3) * mm + m4 * m4 * l2m]])
        eigmax = max(eigmax, -np.linalg.eigvalsh(A)[0] / (4 * rho[p]))
    assert O.curv_dt(1, b, rho, mu, la, met, jac, 1.3) == pytest.approx(1.3 / np.sqrt(eigmax),
                                                                      rel=1e-12)
