"""The FP32-mixed stage kernels fed by tensor copies against the synchronous kernels.

Both kernels evaluate the same FP32 expressions in the same order on the same
double-float levels; only the data movement differs (bulk tensor copies into
shared memory versus plain loads), so after several steps the levels agree to the
last bits of the FP32 stencil (tolerance 1e-7 relative to the field maximum; the
compiler may contract a product into an FMA differently in the two kernels).  The
shapes cover partial 32 x 8 tiles in x and y, free-surface, supergrid, Dirichlet
and periodic sides, and an array whose i extent is not a multiple of 4, where the
launcher keeps the synchronous kernel (the two runs are then identical).
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from tests.fields import rel_err
from tests.gpu_util import dev, host, smooth_fields, smooth_material

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    yield
    sg.set_mixed_tma(True)


def _run(shape, bc, tma, nsteps=4, gp=6):
    nx, ny, nz = shape
    h = 0.05
    rho, mu, la = smooth_material(nx, ny, nz, seed=31)
    u, um = smooth_fields(nx, ny, nz, seed=37)
    dt = 0.3 * h / float(np.sqrt(np.max((4 * mu + la) / rho)))
    g = sg.grid_desc(nx, ny, nz, h, bc=bc, sg_gp=gp, precision=sg.MIXED)
    sg.set_mixed_tma(tma)
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in (rho, mu, la)])
    ew.add_source(sg.source_desc(0.4 * nx * h, 0.55 * ny * h, 0.5 * nz * h,
                                 moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=6.0,
                                 kind=sg.C6SMOOTHBUMP))
    ew.set_time_step(dt, 0.0)
    ew.set_fields(dev(u), dev(um))
    ew.step(nsteps, sg.MODE_FUSED)
    assert ew.status() == sg.OK
    a = dev(np.zeros_like(u))
    b = dev(np.zeros_like(u))
    ew.get_fields(a, b)
    out = host(a), host(b)
    ew.close()
    sg.set_mixed_tma(True)
    return out


CASES = [
    ((36, 34, 40), (2, 2, 2, 2, 0, 2)),   # i extent 40: one full and one partial tile
    ((60, 21, 30), (2,) * 6),             # partial tiles in x (60 = 32 + 28) and y
    ((124, 20, 26), (1, 1, 2, 2, 0, 0)),  # Dirichlet x, free surface top and bottom
    ((28, 30, 24), (3, 3, 3, 3, 0, 2)),   # periodic x, y; a single x tile
]


@pytest.mark.parametrize("shape,bc", CASES)
def test_tma_stages_match_synchronous_stages(shape, bc):
    assert (shape[0] + 4) % 4 == 0  # the tensor-copy path applies
    got_u, got_um = _run(shape, bc, True)
    want_u, want_um = _run(shape, bc, False)
    assert np.all(np.isfinite(got_u))
    assert rel_err(got_u, want_u) <= 1e-7
    assert rel_err(got_um, want_um) <= 1e-7


def test_unaligned_extent_keeps_the_synchronous_kernel():
    shape, bc = (35, 22, 26), (2, 2, 2, 2, 0, 2)  # i extent 39
    got_u, _ = _run(shape, bc, True)
    want_u, _ = _run(shape, bc, False)
    assert np.array_equal(got_u, want_u)
