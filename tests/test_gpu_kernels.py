"""Kernel-level parity on the GPU: each C-ABI kernel entry point against the CPU
oracle (oracle/sw4_oracle.c) on seeded random fields.

Tolerances (FP64): the operator and damping kernels agree with the oracle to
1e-13 relative to the largest output magnitude (different summation order and
FMA contraction); pointwise updates and ghost copies to 1e-14.
"""
import ctypes as C

import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.fields import Grid, rel_err
from tests.gpu_util import dev, host, stream

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _onesided(t, b):
    a = (C.c_int * 6)()
    a[4], a[5] = t, b
    return a


@pytest.mark.parametrize("soa", [1, 0])
@pytest.mark.parametrize("onesided", [(0, 0), (1, 0), (0, 1), (1, 1)])
@pytest.mark.parametrize("shape", [(13, 11, 17), (40, 9, 21), (33, 29, 27)])
def test_rhs4sg(soa, onesided, shape):
    g = Grid(*shape, h=0.37)
    rng = np.random.default_rng(11 + soa + 3 * onesided[0] + 5 * onesided[1])
    u = g.field3(rng)
    rho, mu, la = g.material(rng)
    sx, sy, sz = g.stretching(rng)
    os6 = [0, 0, 0, 0, onesided[0], onesided[1]]
    ref = np.zeros_like(u)
    O.rhs4sg(soa, g.bounds, g.nz, os6, ref, u, mu, la, g.h, sx, sy, sz)
    du, dmu, dla, dsx, dsy, dsz = (dev(a) for a in (u, mu, la, sx, sy, sz))
    dlu = dev(np.zeros_like(u))
    st = sg.lib().sw4g_rhs4sg(soa, *g.bounds, g.nz, _onesided(*onesided), dlu.data_ptr(),
                              du.data_ptr(), dmu.data_ptr(), dla.data_ptr(), g.h, dsx.data_ptr(),
                              dsy.data_ptr(), dsz.data_ptr(), stream())
    sg.check(st, "sw4g_rhs4sg")
    got = host(dlu)
    assert rel_err(got, ref) <= 1e-13
    # ghost shell untouched
    m = g.interior_mask()
    assert np.all(g.as4(got, soa)[:, ~m] == 0)


@pytest.mark.parametrize("soa", [1, 0])
def test_pointwise_updates(soa):
    g = Grid(17, 12, 10)
    rng = np.random.default_rng(3 + soa)
    up0, u, um, lu, fo = (g.field3(rng) for _ in range(5))
    rho, _, _ = g.material(rng)
    dt = 0.0123
    L = sg.lib()
    d = {k: dev(v) for k, v in dict(up=up0, u=u, um=um, lu=lu, fo=fo, rho=rho).items()}
    # predictor
    ref = up0.copy()
    O.predfort(soa, g.bounds, ref, u, um, lu, fo, rho, dt * dt)
    sg.check(L.sw4g_predfort(soa, *g.bounds, d["up"].data_ptr(), d["u"].data_ptr(),
                             d["um"].data_ptr(), d["lu"].data_ptr(), d["fo"].data_ptr(),
                             d["rho"].data_ptr(), dt * dt, stream()))
    np.testing.assert_allclose(host(d["up"]), ref, rtol=1e-14, atol=1e-15)
    # corrector on top of it
    O.corrfort(soa, g.bounds, ref, lu, fo, rho, dt ** 4)
    sg.check(L.sw4g_corrfort(soa, *g.bounds, d["up"].data_ptr(), d["lu"].data_ptr(),
                             d["fo"].data_ptr(), d["rho"].data_ptr(), dt ** 4, stream()))
    np.testing.assert_allclose(host(d["up"]), ref, rtol=1e-14, atol=1e-15)
    # dpdm
    ref2 = np.zeros_like(u)
    O.dpdmtfort(g.bounds, up0, u, um, ref2, 1 / dt ** 2)
    out = dev(np.zeros_like(u))
    dup0 = dev(up0)
    sg.check(L.sw4g_dpdmtfort(*g.bounds, dup0.data_ptr(), d["u"].data_ptr(),
                              d["um"].data_ptr(), out.data_ptr(), 1 / dt ** 2, stream()))
    np.testing.assert_allclose(host(out), ref2, rtol=1e-14, atol=1e-12)


@pytest.mark.parametrize("order", [4, 6])
@pytest.mark.parametrize("soa", [1, 0])
def test_addsgd(order, soa):
    g = Grid(19, 14, 16)
    rng = np.random.default_rng(21 + order + soa)
    up0, u, um = g.field3(rng), g.field3(rng), g.field3(rng)
    rho, _, _ = g.material(rng)
    dc = (g.strip(rng, g.ni, 0, 1), g.strip(rng, g.nj, 0, 1), g.strip(rng, g.nk, 0, 1))
    st = g.stretching(rng)
    co = (g.strip(rng, g.ni, 0.3, 1), g.strip(rng, g.nj, 0.3, 1), g.strip(rng, g.nk, 0.3, 1))
    ref = up0.copy()
    O.addsgd(order, soa, g.bounds, ref, u, um, rho, dc, st, co, 0.02)
    # every device buffer stays referenced until the kernel has run
    dup, du, dum, drho = dev(up0), dev(u), dev(um), dev(rho)
    prof = [dev(a) for a in (*dc, *st, *co)]
    fn = sg.lib().sw4g_addsgd6fort if order == 6 else sg.lib().sw4g_addsgd4fort
    sg.check(fn(soa, *g.bounds, dup.data_ptr(), du.data_ptr(), dum.data_ptr(),
                drho.data_ptr(), *[p.data_ptr() for p in prof], 0.02, stream()))
    got = host(dup)
    assert rel_err(got - up0, ref - up0) <= 1e-13


@pytest.mark.parametrize("soa", [1, 0])
@pytest.mark.parametrize("bccnd", [(2, 2, 2, 2, 0, 2), (1, 1, 1, 1, 1, 1), (3, 3, 3, 3, 0, 0),
                                   (2, 2, 2, 2, 2, 0)])
def test_bcfortsg(soa, bccnd):
    g = Grid(15, 13, 12, h=0.5)
    rng = np.random.default_rng(31 + soa)
    u0 = g.field3(rng)
    _, mu, la = g.material(rng)
    sx, sy, _ = g.stretching(rng)
    wind, npts = O.boundary_windows(g.bounds, (g.nx, g.ny, g.nz), bccnd)
    bforce = [g.field3(rng)[: 3 * max(1, n)].copy() if bccnd[s] in (0, 1) else None
              for s, n in enumerate(npts)]
    _, _, _, sbop = O.stencil_coefficients()
    ref = u0.copy()
    O.bcfortsg(soa, g.bounds, wind, (g.nx, g.ny, g.nz), ref, g.h, bccnd, sbop, mu, la, bforce, sx, sy)
    du = dev(u0)
    dbf = [dev(b) if b is not None else None for b in bforce]
    ptrs = (C.c_void_p * 6)(*[b.data_ptr() if b is not None else None for b in dbf])
    w = (C.c_int * 36)(*[int(x) for x in wind])
    bc = (C.c_int * 6)(*bccnd)
    sb = (C.c_double * 6)(*sbop)
    dmu, dla, dsx, dsy = dev(mu), dev(la), dev(sx), dev(sy)
    sg.check(sg.lib().sw4g_bcfortsg(soa, *g.bounds, w, g.nx, g.ny, g.nz, du.data_ptr(), g.h, bc,
                                    C.cast(sb, sg._D), dmu.data_ptr(), dla.data_ptr(), ptrs,
                                    dsx.data_ptr(), dsy.data_ptr(), stream()))
    assert rel_err(host(du), ref) <= 1e-14
