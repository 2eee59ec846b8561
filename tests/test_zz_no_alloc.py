"""The allocation-free corrector-rows entry point (sw4g_corr_rows_noalloc).

It serves callers that may not call cudaMalloc: instead of a caller-provided
scratch slab it uses a fixed 64 MiB device array owned by the library.  This file
runs last so that, if it fails, a run that stops at the first failure has
already run every other test; it also passes on its own in a fresh process.

Check: two calls in a row (different inputs) through the C ABI give the same
output as the existing entry point sw4g_corr_rows with its own scratch buffer,
within the tolerance the row tests use (1e-13 relative); and a plane above the
documented limit is rejected without device work.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from tests.fields import Grid, rel_err
from tests.gpu_util import dev, host, stream

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()


def _inputs(seed):
    g = Grid(23, 19, 22, h=0.3)
    rng = np.random.default_rng(seed)
    up, u, um = g.field3(rng), g.field3(rng), g.field3(rng)
    rho, mu, la = g.material(rng)
    st = g.stretching(rng)
    dc = (g.strip(rng, g.ni, 0, 1), g.strip(rng, g.nj, 0, 1), g.strip(rng, g.nk, 0, 1))
    co = (g.strip(rng, g.ni, 0.3, 1), g.strip(rng, g.nj, 0.3, 1), g.strip(rng, g.nk, 0.3, 1))
    return g, [dev(a) for a in (up, u, um, mu, la, rho, *st, *dc, *co)]


@pytest.mark.parametrize("side", [0, 1])
def test_noalloc_matches_scratch_entry_point_on_two_calls(side):
    L = sg.lib()
    dt, beta = 0.0123, 0.02
    for call, seed in enumerate((61 + side, 71 + side)):
        g, d = _inputs(seed)
        ptrs = [t.data_ptr() for t in d]
        n = L.sw4g_corr_rows_scratch_len(g.ib, g.ie, g.jb, g.je)
        scratch = dev(np.zeros(n))
        want = dev(np.zeros(3 * g.npts))
        got = dev(np.zeros(3 * g.npts))
        sg.check(L.sw4g_corr_rows(*g.bounds, g.nz, side, want.data_ptr(), *ptrs, g.h, dt, beta,
                                  scratch.data_ptr(), n, stream()), "sw4g_corr_rows")
        sg.check(L.sw4g_corr_rows_noalloc(*g.bounds, g.nz, side, got.data_ptr(), *ptrs, g.h, dt,
                                          beta, stream()), "sw4g_corr_rows_noalloc")
        a, b = host(got), host(want)
        assert np.any(b != 0), "reference call wrote nothing"
        assert rel_err(a, b) <= 1e-13, f"call {call}"


def test_noalloc_rejects_planes_above_the_limit():
    L = sg.lib()
    # 600 x 600 points per plane is above the 279,620-point limit; no device work
    # happens, so null field pointers are never touched
    assert L.sw4g_corr_rows_noalloc(-1, 598, -1, 598, -1, 20, 18, 0, *([None] * 16), 1.0, 0.01,
                                    0.02, None) == 1
