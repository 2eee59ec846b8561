"""The oracle's two-grid (topography) step pinned to the same step composed of
the reference's own kernels (oracle/_ref, sw4ref_step_topo), in the reference's
phase order with the curvilinear free surface and the interface copy.

Tolerance: 1e-12 relative to each field's largest magnitude after 4 steps
(rounding-level differences of each kernel carried through a few steps).
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.topo_util import TopoCase, smooth_topo_fields

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference kernels not built here")


def _case(sg_order=4):
    nx, ny, ncart, h = 26, 24, 20, 0.1
    src = [sg.source_desc(0.5 * nx * h, 0.45 * ny * h, 1.0 + 0.6 * ncart * h * 0.5,
                          force=(1.0, -0.5, 0.3), freq=8.0, t0=0.1, kind=sg.GAUSSIAN)]
    return TopoCase(nx, ny, ncart, h, zmax_topo=1.0, amp=0.2, xc=1.3, yc=1.2, lx=0.6, ly=0.5,
                    gp=5, sources=src, sg_order=sg_order)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_topo_case_dimensions():
    c = _case()
    assert c.nc == 1 + round((1.0 - 0.5 * (c.zs.min() + c.zs.max())) / 0.1)
    z = c.z.reshape(c.nc + 4, c.ny + 4, c.nx + 4)
    assert np.allclose(z[c.nc + 1], 1.0)            # bottom interior plane at zmax_topo
    assert np.allclose(z[2], c.zs)                  # top plane on the topography


@pytest.mark.parametrize("sg_order", [4, 6])
def test_topo_step_matches_reference_kernels(sg_order):
    c = _case(sg_order)
    dt = c.time_step(1.3)
    assert 0 < dt < 0.1
    fields = smooth_topo_fields(c, seed=4)
    res = [c.oracle(dt).run(*fields, 0.0, 4, which=w) for w in ("oracle", "ref")]
    for a, b in zip(*res):
        assert _rel(a, b) <= 1e-12
    # the interface copy held: Cartesian k=-1,0 equal curvilinear k=nc-2,nc-1
    u, _, cu, _ = res[0]
    U = u.reshape(3, c.ncart + 4, c.ny + 4, c.nx + 4)
    V = cu.reshape(3, c.nc + 4, c.ny + 4, c.nx + 4)
    assert np.array_equal(U[:, 0:2], V[:, c.nc - 1:c.nc + 1])
    assert np.array_equal(V[:, c.nc + 1:c.nc + 4], U[:, 2:5])
