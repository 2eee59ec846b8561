"""Phase-level one-sided-row entry points (sw4g_pred_rows, sw4g_corr_rows) against
the oracle's reference phase sequence on the same rows.

Tolerance: the stage increment agrees to 1e-13 relative to its largest magnitude
(FP64, different summation order)."""
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


def _rows_mask(g, side):
    m = np.zeros((g.nk, g.nj, g.ni), dtype=bool)
    ks = range(1, 7) if side == 0 else range(g.nz - 5, g.nz + 1)
    for k in ks:
        m[k - g.kb, 2:-2, 2:-2] = True
    return np.broadcast_to(m, (3,) + m.shape).ravel()


def _problem(seed):
    g = Grid(21, 18, 24, h=0.3)
    rng = np.random.default_rng(seed)
    u, um, up = g.field3(rng), g.field3(rng), g.field3(rng)
    rho, mu, la = g.material(rng)
    st = g.stretching(rng)
    dc = (g.strip(rng, g.ni, 0, 1), g.strip(rng, g.nj, 0, 1), g.strip(rng, g.nk, 0, 1))
    co = (g.strip(rng, g.ni, 0.3, 1), g.strip(rng, g.nj, 0.3, 1), g.strip(rng, g.nk, 0.3, 1))
    return g, u, um, up, rho, mu, la, st, dc, co


@pytest.mark.parametrize("side", [0, 1])
def test_pred_rows(side):
    g, u, um, _, rho, mu, la, st, _, _ = _problem(40 + side)
    dt = 0.011
    lu = np.zeros_like(u)
    O.rhs4sg(1, g.bounds, g.nz, [0, 0, 0, 0, 1, 1], lu, u, mu, la, g.h, *st)
    ref = np.zeros_like(u)
    O.predfort(1, g.bounds, ref, u, um, lu, np.zeros_like(u), rho, dt * dt)
    d = [dev(a) for a in (u, um, mu, la, rho, *st)]
    out = dev(np.zeros_like(u))
    sg.check(sg.lib().sw4g_pred_rows(*g.bounds, g.nz, side, out.data_ptr(),
                                     *[t.data_ptr() for t in d], g.h, dt, stream()), "pred_rows")
    got = host(out)
    m = _rows_mask(g, side)
    inc_ref = (ref - (2 * u - um))[m]
    inc = (got - (2 * u - um))[m]
    assert rel_err(inc, inc_ref) <= 1e-13
    assert np.all(got[~m] == 0)  # nothing outside the rows is written


@pytest.mark.parametrize("side", [0, 1])
def test_corr_rows(side):
    g, u, um, up, rho, mu, la, st, dc, co = _problem(50 + side)
    dt, beta = 0.011, 0.02
    uacc = np.zeros_like(u)
    O.dpdmtfort(g.bounds, up, u, um, uacc, 1 / dt ** 2)
    lu = np.zeros_like(u)
    O.rhs4sg(1, g.bounds, g.nz, [0, 0, 0, 0, 1, 1], lu, uacc, mu, la, g.h, *st)
    ref = up.copy()
    O.corrfort(1, g.bounds, ref, lu, np.zeros_like(u), rho, dt ** 4)
    O.addsgd(4, 1, g.bounds, ref, u, um, rho, dc, st, co, beta)
    n = sg.lib().sw4g_corr_rows_scratch_len(g.ib, g.ie, g.jb, g.je)
    assert n == 3 * 10 * g.ni * g.nj
    scratch = dev(np.full(n, np.nan))
    d = [dev(a) for a in (up, u, um, mu, la, rho, *st, *dc, *co)]
    out = dev(np.zeros_like(u))
    sg.check(sg.lib().sw4g_corr_rows(*g.bounds, g.nz, side, out.data_ptr(),
                                     *[t.data_ptr() for t in d], g.h, dt, beta,
                                     scratch.data_ptr(), n, stream()), "corr_rows")
    got = host(out)
    m = _rows_mask(g, side)
    assert rel_err((got - up)[m], (ref - up)[m]) <= 1e-13
    # too small a scratch buffer is rejected
    assert sg.lib().sw4g_corr_rows(*g.bounds, g.nz, side, out.data_ptr(),
                                   *[t.data_ptr() for t in d], g.h, dt, beta,
                                   scratch.data_ptr(), n - 1, stream()) == 1
