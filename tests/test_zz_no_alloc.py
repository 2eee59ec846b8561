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


def _inputs(seed, shape=(23, 19, 22)):
    g = Grid(*shape, h=0.3)
    rng = np.random.default_rng(seed)
    up, u, um = g.field3(rng), g.field3(rng), g.field3(rng)
    rho, mu, la = g.material(rng)
    st = g.stretching(rng)
    dc = (g.strip(rng, g.ni, 0, 1), g.strip(rng, g.nj, 0, 1), g.strip(rng, g.nk, 0, 1))
    co = (g.strip(rng, g.ni, 0.3, 1), g.strip(rng, g.nj, 0.3, 1), g.strip(rng, g.nk, 0.3, 1))
    return g, [dev(a) for a in (up, u, um, mu, la, rho, *st, *dc, *co)]


def _both(g, d, side, dt=0.0123, beta=0.02):
    """Run the scratch entry point and the allocation-free one on the same inputs."""
    L = sg.lib()
    ptrs = [t.data_ptr() for t in d]
    n = L.sw4g_corr_rows_scratch_len(g.ib, g.ie, g.jb, g.je)
    scratch = dev(np.zeros(n))
    want = dev(np.zeros(3 * g.npts))
    got = dev(np.zeros(3 * g.npts))
    sg.check(L.sw4g_corr_rows(*g.bounds, g.nz, side, want.data_ptr(), *ptrs, g.h, dt, beta,
                              scratch.data_ptr(), n, stream()), "sw4g_corr_rows")
    sg.check(L.sw4g_corr_rows_noalloc(*g.bounds, g.nz, side, got.data_ptr(), *ptrs, g.h, dt,
                                      beta, stream()), "sw4g_corr_rows_noalloc")
    return host(got), host(want)


@pytest.mark.parametrize("side", [0, 1])
def test_noalloc_matches_scratch_entry_point_on_two_calls(side):
    # the second call has a larger plane than the first, so its slab layout in the
    # shared array differs from the one the first call left behind
    for call, (seed, shape) in enumerate(((61 + side, (23, 19, 22)), (71 + side, (37, 29, 12)))):
        g, d = _inputs(seed, shape)
        a, b = _both(g, d, side)
        assert np.any(b != 0), "reference call wrote nothing"
        assert rel_err(a, b) <= 1e-13, f"call {call}"


def test_noalloc_accepts_the_largest_plane():
    # 528 x 528 points per plane (524^2 interior) is the largest square plane
    # within the 279,620-point limit
    g, d = _inputs(81, (524, 524, 8))
    assert g.ni * g.nj == 528 * 528
    a, b = _both(g, d, 0)
    assert np.any(b != 0)
    assert rel_err(a, b) <= 1e-13


def test_noalloc_rejects_planes_above_the_limit():
    L = sg.lib()
    # 529 x 529 = 279,841 points per plane is just above the 279,620-point limit,
    # 600 x 600 far above it; no device work happens, so null field pointers are
    # never touched
    for last in (527, 598):
        assert L.sw4g_corr_rows_noalloc(-1, last, -1, last, -1, 20, 18, 0, *([None] * 16), 1.0,
                                        0.01, 0.02, None) == 1
