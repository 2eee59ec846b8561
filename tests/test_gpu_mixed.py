"""The FP32-mixed form against the FP64 form on the GPU.

The mixed form keeps the solution levels as double-float pairs (48-bit) and runs
the interior stencil in FP32, so it differs from FP64 by the FP32 rounding of the
operator.  Tolerances:
  * level storage round trip (FP64 -> double-float -> FP64): 1e-14 relative;
  * one step from smooth data: 1e-6 relative to the field maximum;
  * 120 steps with sources, free surface and supergrid: relative L2 error
    <= 1e-5 against the FP64 form (the mixed form's stated accuracy bar).
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


def _run(g, mat, fields, srcs, dt, nsteps):
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in mat])
    for s in srcs:
        ew.add_source(s)
    ew.set_time_step(dt, 0.0)
    ew.set_fields(dev(fields[0]), dev(fields[1]))
    ew.step(nsteps, sg.MODE_FUSED)
    u = dev(np.zeros_like(fields[0]))
    um = dev(np.zeros_like(fields[0]))
    ew.get_fields(u, um)
    out = host(u), host(um)
    ew.close()
    return out


def _case(bc, shape=(36, 34, 40), gp=8, sg_order=4, damping=0.02):
    nx, ny, nz = shape
    h = 0.05
    rho, mu, la = smooth_material(nx, ny, nz, seed=17)
    fields = smooth_fields(nx, ny, nz, seed=19)
    srcs = [sg.source_desc(0.45 * nx * h, 0.5 * ny * h, 0.5 * nz * h,
                           moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=6.0,
                           kind=sg.C6SMOOTHBUMP),
            sg.source_desc(0.6 * nx * h, 0.4 * ny * h, 0.6 * nz * h, force=(1.0, -0.5, 0.25),
                           freq=8.0, t0=0.05)]
    dt = 0.3 * h / float(np.sqrt(np.max((4 * mu + la) / rho)))
    mk = lambda prec: sg.grid_desc(nx, ny, nz, h, bc=bc, sg_gp=gp, sg_order=sg_order,
                                   sg_damping=damping, precision=prec)
    return mk, (rho, mu, la), fields, srcs, dt


def test_level_storage_round_trip():
    mk, mat, fields, _, _ = _case((2, 2, 2, 2, 0, 2))
    ew = sg.EW(mk(sg.MIXED))
    ew.set_material(*[dev(a) for a in mat])
    ew.set_fields(dev(fields[0]), dev(fields[1]))
    u = dev(np.zeros_like(fields[0]))
    um = dev(np.zeros_like(fields[0]))
    ew.get_fields(u, um)
    assert rel_err(host(u), fields[0]) <= 1e-14
    assert rel_err(host(um), fields[1]) <= 1e-14
    # host-side buffers go through the library's staging buffer
    hu = np.zeros_like(fields[0])
    ew.get_fields(hu, None)
    assert rel_err(hu, fields[0]) <= 1e-14
    ew.close()


@pytest.mark.parametrize("bc", [(2, 2, 2, 2, 0, 2), (2,) * 6, (2, 2, 2, 2, 0, 0)])
def test_one_step_close_to_fp64(bc):
    mk, mat, fields, srcs, dt = _case(bc)
    a, _ = _run(mk(sg.FP64), mat, fields, srcs, dt, 1)
    b, _ = _run(mk(sg.MIXED), mat, fields, srcs, dt, 1)
    assert rel_err(b, a) <= 1e-6


@pytest.mark.parametrize("bc", [(2, 2, 2, 2, 0, 2), (3, 3, 1, 1, 0, 1)])
def test_many_steps_l2_error(bc):
    mk, mat, fields, srcs, dt = _case(bc)
    a, _ = _run(mk(sg.FP64), mat, fields, srcs, dt, 120)
    b, _ = _run(mk(sg.MIXED), mat, fields, srcs, dt, 120)
    l2 = float(np.linalg.norm(b - a) / np.linalg.norm(a))
    assert l2 <= 1e-5, l2


@pytest.mark.parametrize("nsteps,tol", [(1, 1e-6), (120, 1e-5)])
def test_sixth_order_damping_close_to_fp64(nsteps, tol):
    # the 6th-order damping runs as its own pass on the double-float levels (FP32
    # arithmetic, as the 4th-order damping in the mixed stage kernel)
    # 16-point layers and the reference's 6th-order default coefficient 0.005
    # (src/EW.C:1307-1310)
    mk, mat, fields, srcs, dt = _case((2, 2, 2, 2, 0, 2), shape=(68, 60, 52), gp=16, sg_order=6,
                                      damping=0.005)
    a, _ = _run(mk(sg.FP64), mat, fields, srcs, dt, nsteps)
    b, _ = _run(mk(sg.MIXED), mat, fields, srcs, dt, nsteps)
    if nsteps == 1:
        assert rel_err(b, a) <= tol
    else:
        l2 = float(np.linalg.norm(b - a) / np.linalg.norm(a))
        assert l2 <= tol, l2


def test_mixed_rejects_phase_mode():
    mk, mat, fields, _, dt = _case((2, 2, 2, 2, 0, 2))
    ew = sg.EW(mk(sg.MIXED))
    ew.set_material(*[dev(x) for x in mat])
    ew.set_time_step(dt)
    with pytest.raises(sg.Sw4gError):
        ew.step(1, sg.MODE_PHASES)
    ew.close()
