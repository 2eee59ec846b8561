"""The C-ABI library: loads, exports every symbol include/sw4g.h declares, and its
host-side set-up helpers (no device work) agree with the oracle / reference."""
import ctypes as C

import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O


@pytest.fixture(scope="module")
def lib():
    sg.build()
    return sg.lib()


def test_library_exports_every_declared_symbol(lib):
    names = sg.header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert lib.sw4g_version().decode().startswith("sw4g")


def test_status_strings(lib):
    assert lib.sw4g_status_string(0).decode() == "ok"
    assert "argument" in lib.sw4g_status_string(1).decode()


def test_stencil_table_matches_oracle_and_reference(lib):
    mine = sg.stencil_coefficients()
    orc = O.stencil_coefficients("oracle")
    for a, b in zip(mine, orc):
        np.testing.assert_array_equal(a, b)
    if O.ref_available():
        for a, b in zip(mine, O.stencil_coefficients("ref")):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("bc", [(2, 2, 2, 2, 0, 2), (2, 2, 2, 2, 2, 2), (1, 2, 3, 3, 0, 0),
                                (0 + 2, 1, 2, 1, 2, 1)])
def test_supergrid_profiles_match_oracle(lib, bc):
    g = sg.grid_desc(41, 37, 33, 0.025, bc=bc, sg_gp=12)
    for ax, n, b0, b1 in [(0, 41, bc[0], bc[1]), (1, 37, bc[2], bc[3]), (2, 33, bc[4], bc[5])]:
        m = n + 4
        dc, st, co = np.zeros(m), np.zeros(m), np.zeros(m)
        sg.check(lib.sw4g_supergrid_profile(C.byref(g), ax, *[a.ctypes.data_as(sg._D) for a in (dc, st, co)]))
        used = 2 in bc
        if used:
            odc, ost, oco = O.supergrid_profile(-1, n + 2, g.h, 0.0, b0 == 2, b1 == 2, 0.0, (n - 1) * g.h,
                                                g.sg_gp * g.h)
        else:
            odc, ost, oco = np.zeros(m), np.ones(m), np.ones(m)
        np.testing.assert_allclose(dc, odc, rtol=1e-15, atol=0)
        np.testing.assert_allclose(st, ost, rtol=1e-15, atol=0)
        np.testing.assert_allclose(co, oco, rtol=1e-15, atol=0)


@pytest.mark.parametrize("bc", [(2, 2, 2, 2, 0, 2), (1, 1, 1, 1, 1, 1), (3, 3, 3, 3, 0, 0)])
def test_boundary_windows_match_oracle(lib, bc):
    g = sg.grid_desc(20, 18, 16, 0.1, bc=bc)
    w = np.zeros(36, dtype=np.int32)
    n = np.zeros(6, dtype=np.int32)
    sg.check(lib.sw4g_boundary_windows(C.byref(g), w.ctypes.data_as(sg._I), n.ctypes.data_as(sg._I)))
    ow, on = O.boundary_windows((-1, 22, -1, 20, -1, 18), (20, 18, 16), bc)
    np.testing.assert_array_equal(w, ow)
    np.testing.assert_array_equal(n, on)


def test_point_force_discretization_is_moment_exact(lib):
    """Discrete delta: weights reproduce the force and its first moments exactly."""
    g = sg.grid_desc(40, 40, 40, 0.1, bc=(2,) * 6)
    s = sg.source_desc(2.03, 1.977, 1.911, force=(1.0, -2.0, 0.5), freq=5.0)
    cap = 512
    ijk = np.zeros(3 * cap, dtype=np.int32)
    amp = np.zeros(3 * cap)
    n = C.c_int()
    sg.check(lib.sw4g_discretize_source(C.byref(g), C.byref(s), cap, ijk.ctypes.data_as(sg._I),
                                        amp.ctypes.data_as(sg._D), C.byref(n)))
    n = n.value
    assert 0 < n <= 216
    ijk = ijk[:3 * n].reshape(n, 3)
    amp = amp[:3 * n].reshape(n, 3)
    h3 = g.h ** 3
    np.testing.assert_allclose(amp.sum(0) * h3, [1.0, -2.0, 0.5], rtol=1e-12)
    x = (ijk - 1) * g.h
    for ax, x0 in enumerate((s.x, s.y, s.z)):
        np.testing.assert_allclose((amp[:, 0] * x[:, ax]).sum() * h3, 1.0 * x0, rtol=1e-12)


def test_moment_discretization_is_moment_exact(lib):
    """Discrete -M grad(delta): zeroth moment vanishes, first moments give -(-M) = M."""
    g = sg.grid_desc(40, 40, 40, 0.1, bc=(2,) * 4 + (0, 2))
    M = (1.0, 0.3, -0.2, 2.0, 0.7, -1.5)
    s = sg.source_desc(2.01, 1.96, 1.87, moment=M, freq=1.0, kind=sg.C6SMOOTHBUMP)
    cap = 512
    ijk = np.zeros(3 * cap, dtype=np.int32)
    amp = np.zeros(3 * cap)
    n = C.c_int()
    sg.check(lib.sw4g_discretize_source(C.byref(g), C.byref(s), cap, ijk.ctypes.data_as(sg._I),
                                        amp.ctypes.data_as(sg._D), C.byref(n)))
    n = n.value
    ijk = ijk[:3 * n].reshape(n, 3)
    amp = amp[:3 * n].reshape(n, 3)
    h3 = g.h ** 3
    np.testing.assert_allclose(amp.sum(0) * h3, 0.0, atol=1e-10)
    Mfull = np.array([[M[0], M[1], M[2]], [M[1], M[3], M[4]], [M[2], M[4], M[5]]])
    x = (ijk - 1) * g.h
    first = np.einsum("pc,pa->ca", amp, x) * h3  # int F_c x_a = M_ca
    np.testing.assert_allclose(first, Mfull, rtol=1e-10, atol=1e-10)


def test_bad_arguments_are_rejected_without_device_work(lib):
    g = sg.grid_desc(4, 4, 4, 0.1)  # too small for the time loop
    h = sg._VP()
    assert lib.sw4g_ew_create(C.byref(g), None, C.byref(h)) == 1
    g = sg.grid_desc(20, 20, 20, 0.1, bc=(0, 2, 2, 2, 2, 2))  # free surface on a lateral side
    assert lib.sw4g_ew_create(C.byref(g), None, C.byref(h)) == 4
    assert lib.sw4g_rhs4sg(1, 1, 0, 1, 0, 1, 0, 1, (C.c_int * 6)(), None, None, None, None, 1.0,
                           None, None, None, None) == 1


def test_nearest_grid_point_matches_reference_rule(lib):
    """sw4g_nearest_grid_point against the oracle's restatement of
    EW::computeNearestGridPoint, including points exactly half-way between two."""
    g = sg.grid_desc(40, 30, 20, 0.25, zmin=1.5)
    rng = np.random.default_rng(5)
    pts = list(rng.uniform([0, 0, 1.5], [9.75, 7.25, 6.25], size=(200, 3)))
    pts += [(0.125, 0.375, 1.625), (2.5, 2.5, 1.5), (9.75, 7.25, 6.25)]
    for x, y, z in pts:
        assert sg.nearest_grid_point(g, x, y, z) == O.nearest_grid_point(0.25, 1.5, x, y, z)
    with pytest.raises(sg.Sw4gError):
        sg.nearest_grid_point(g, 20.0, 1.0, 2.0)
    with pytest.raises(sg.Sw4gError):
        sg.nearest_grid_point(g, 1.0, 1.0, 0.0)
