"""Pin the CPU oracle (oracle/sw4_oracle.c) to the reference's own kernels.

The reference kernels are compiled from the reference sources into
oracle/_ref/libsw4ref.so (``make -C oracle ref``) where that tree exists; these
tests skip elsewhere.  Tolerances: FP64 results agree to 1e-13 relative to the
largest output magnitude (summation order differs); table lookups and copies
agree bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.fields import Grid, rel_err

@pytest.fixture(scope="module", autouse=True)
def _ref_lib():
    if not O.ref_available():
        if O.reference_src() is None:
            pytest.skip("reference sources not present; oracle pinned by tests/golden instead")
        O.build(ref=True)
    O.lib()
    assert O.ref() is not None


def test_stencil_table_matches_reference_exactly():
    mine = O.stencil_coefficients("oracle")
    ref = O.stencil_coefficients("ref")
    for a, b in zip(mine, ref):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("soa", [1, 0])
@pytest.mark.parametrize("onesided", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("shape", [(13, 11, 17), (9, 16, 14)])
def test_rhs4sg_matches_reference(soa, onesided, shape):
    g = Grid(*shape, h=0.37)
    rng = np.random.default_rng(1234 + 7 * soa + 3 * onesided[0] + onesided[1])
    u = g.field3(rng)
    rho, mu, la = g.material(rng)
    sx, sy, sz = g.stretching(rng)
    os6 = [0, 0, 0, 0, onesided[0], onesided[1]]
    lu_ref = np.zeros_like(u)
    lu_me = np.zeros_like(u)
    O.rhs4sg(soa, g.bounds, g.nz, os6, lu_ref, u, mu, la, g.h, sx, sy, sz, which="ref")
    O.rhs4sg(soa, g.bounds, g.nz, os6, lu_me, u, mu, la, g.h, sx, sy, sz)
    assert rel_err(lu_me, lu_ref) <= 1e-13
    # both leave the ghost shell untouched (zero on entry)
    m = g.interior_mask()
    assert np.all(g.as4(lu_me, soa)[:, ~m] == 0)


@pytest.mark.parametrize("soa", [1, 0])
def test_pointwise_updates_match_reference(soa):
    g = Grid(7, 6, 5)
    rng = np.random.default_rng(9 + soa)
    up0, u, um, lu, fo = (g.field3(rng) for _ in range(5))
    rho, _, _ = g.material(rng)
    dt = 0.013
    a, b = up0.copy(), up0.copy()
    O.predfort(soa, g.bounds, a, u, um, lu, fo, rho, dt * dt, which="ref")
    O.predfort(soa, g.bounds, b, u, um, lu, fo, rho, dt * dt)
    np.testing.assert_array_equal(a, b)
    O.corrfort(soa, g.bounds, a, lu, fo, rho, dt ** 4, which="ref")
    O.corrfort(soa, g.bounds, b, lu, fo, rho, dt ** 4)
    np.testing.assert_array_equal(a, b)
    c, d = np.zeros_like(u), np.zeros_like(u)
    O.dpdmtfort(g.bounds, up0, u, um, c, 1 / dt ** 2, which="ref")
    O.dpdmtfort(g.bounds, up0, u, um, d, 1 / dt ** 2)
    np.testing.assert_array_equal(c, d)


@pytest.mark.parametrize("order", [4, 6])
@pytest.mark.parametrize("soa", [1, 0])
def test_addsgd_matches_reference(order, soa):
    g = Grid(12, 10, 11)
    rng = np.random.default_rng(77 + order + soa)
    up0, u, um = g.field3(rng), g.field3(rng), g.field3(rng)
    rho, _, _ = g.material(rng)
    dc = (g.strip(rng, g.ni, 0, 1), g.strip(rng, g.nj, 0, 1), g.strip(rng, g.nk, 0, 1))
    st = g.stretching(rng)
    co = (g.strip(rng, g.ni, 0.3, 1), g.strip(rng, g.nj, 0.3, 1), g.strip(rng, g.nk, 0.3, 1))
    a, b = up0.copy(), up0.copy()
    O.addsgd(order, soa, g.bounds, a, u, um, rho, dc, st, co, 0.02, which="ref")
    O.addsgd(order, soa, g.bounds, b, u, um, rho, dc, st, co, 0.02)
    # compare the damping increments, relative to their own size
    assert rel_err(b - up0, a - up0) <= 1e-13


@pytest.mark.parametrize("soa", [1, 0])
@pytest.mark.parametrize("bccnd", [(2, 2, 2, 2, 0, 2), (1, 1, 1, 1, 1, 1), (3, 3, 3, 3, 0, 0),
                                   (2, 2, 2, 2, 2, 0)])
def test_bcfortsg_matches_reference(soa, bccnd):
    g = Grid(10, 9, 8, h=0.5)
    rng = np.random.default_rng(5 + soa)
    u0 = g.field3(rng)
    _, mu, la = g.material(rng)
    sx, sy, _ = g.stretching(rng)
    wind, npts = O.boundary_windows(g.bounds, (g.nx, g.ny, g.nz), bccnd)
    bforce = [g.field3(rng)[: 3 * max(1, n)].copy() if bccnd[s] in (0, 1) else None
              for s, n in enumerate(npts)]
    _, _, _, sbop = O.stencil_coefficients()
    a, b = u0.copy(), u0.copy()
    O.bcfortsg(soa, g.bounds, wind, (g.nx, g.ny, g.nz), a, g.h, bccnd, sbop, mu, la, bforce, sx,
               sy, which="ref")
    O.bcfortsg(soa, g.bounds, wind, (g.nx, g.ny, g.nz), b, g.h, bccnd, sbop, mu, la, bforce, sx,
               sy)
    assert rel_err(b, a) <= 1e-14


def test_supergrid_profiles_match_reference():
    import ctypes as C
    for (n, h, gp, left, right) in [(101, 0.01, 20, 1, 1), (64, 50.0, 30, 0, 1), (80, 1.0, 12, 1, 0)]:
        first, last = -1, n + 2
        width = gp * h
        mine = O.supergrid_profile(first, last, h, 0.0, left, right, 0.0, (n - 1) * h, width)
        m = last - first + 1
        ref = [np.zeros(m) for _ in range(3)]
        O.ref().sw4ref_supergrid_profile(C.c_int(first), C.c_int(last), C.c_double(h),
                                         C.c_double(0.0), C.c_int(left), C.c_int(right),
                                         C.c_double(0.0), C.c_double((n - 1) * h),
                                         C.c_double(width), *[O._dp(r) for r in ref])
        for a, b in zip(mine, ref):
            np.testing.assert_allclose(a, b, rtol=1e-14, atol=1e-15)


def test_time_functions_match_reference():
    import ctypes as C
    O.ref().sw4ref_timefunc.restype = C.c_double
    for kind, freq in [(0, 20.0), (0, 5.0), (1, 1.0), (1, 3.5)]:
        for t in np.linspace(-0.4, 1.4, 97):
            for tt in (0, 1):
                r = O.ref().sw4ref_timefunc(C.c_int(kind), C.c_double(freq), C.c_double(t),
                                            C.c_int(tt))
                m = O.timefunc(kind, freq, t, tt=bool(tt))
                assert abs(m - r) <= 1e-13 * max(1.0, abs(r)), (kind, freq, t, tt, m, r)
