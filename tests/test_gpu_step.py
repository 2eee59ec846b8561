"""Full time steps on the GPU (both the reference phase order and the fused stage
kernels) against the oracle's restatement of the reference CPU time loop.

Tolerance: after a few steps the FP64 fields agree with the oracle to 1e-12
relative to the largest magnitude of the field (rounding-level differences of
each stage, ~1e-15, carried through a few steps of a linear, stable scheme).
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.fields import rel_err
from tests.gpu_util import (OracleProblem, describe_error, dev, host, smooth_fields, smooth_material,
                            solution_mask)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


CASES = {
    "halfspace": dict(shape=(36, 30, 40), bc=(2, 2, 2, 2, 0, 2), gp=8),
    "all_supergrid": dict(shape=(33, 34, 31), bc=(2,) * 6, gp=7),
    "layer_free_both": dict(shape=(30, 29, 32), bc=(2, 2, 2, 2, 0, 0), gp=6),
    "periodic_dirichlet": dict(shape=(28, 30, 26), bc=(3, 3, 1, 1, 0, 1), gp=6),
}


def _setup(name, order=4):
    c = CASES[name]
    nx, ny, nz = c["shape"]
    h = 0.05
    g = sg.grid_desc(nx, ny, nz, h, bc=c["bc"], sg_gp=c["gp"], sg_damping=0.02, sg_order=order)
    rho, mu, la = smooth_material(nx, ny, nz, seed=sum(map(ord, name)))
    u, um = smooth_fields(nx, ny, nz, seed=7)
    srcs = [sg.source_desc(0.43 * nx * h, 0.51 * ny * h, 0.47 * nz * h, force=(1.0, -0.5, 0.25),
                           freq=8.0, t0=0.05, kind=sg.GAUSSIAN),
            sg.source_desc(0.6 * nx * h, 0.4 * ny * h, 0.55 * nz * h,
                           moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=6.0, t0=0.0,
                           kind=sg.C6SMOOTHBUMP)]
    return g, (rho, mu, la), (u, um), srcs


def _gpu_run(g, mat, fields, srcs, dt, nsteps, mode):
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in mat])
    for s in srcs:
        ew.add_source(s)
    ew.set_time_step(dt, 0.0)
    ew.set_fields(dev(fields[0]), dev(fields[1]))
    ew.step(nsteps, mode)
    u = dev(np.zeros_like(fields[0]))
    um = dev(np.zeros_like(fields[0]))
    ew.get_fields(u, um)
    out = host(u), host(um)
    assert abs(ew.time - nsteps * dt) < 1e-12
    ew.close()
    return out


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("mode", [sg.MODE_PHASES, sg.MODE_FUSED])
def test_steps_match_oracle(name, mode):
    g, mat, fields, srcs = _setup(name)
    dt = 0.3 * g.h / np.sqrt(np.max((4 * mat[1] + mat[2]) / mat[0]))
    nsteps = 6
    ref_u, ref_um = OracleProblem(g, *mat, dt, srcs).run(*fields, 0.0, nsteps)
    u, um = _gpu_run(g, mat, fields, srcs, dt, nsteps, mode)
    m = solution_mask(g)
    assert rel_err(u[m], ref_u[m]) <= 1e-12, describe_error(u, ref_u, g, m)
    assert rel_err(um[m], ref_um[m]) <= 1e-12, describe_error(um, ref_um, g, m)


def test_sixth_order_damping_step():
    g, mat, fields, srcs = _setup("all_supergrid", order=6)
    dt = 0.3 * g.h / np.sqrt(np.max((4 * mat[1] + mat[2]) / mat[0]))
    ref_u, _ = OracleProblem(g, *mat, dt, srcs).run(*fields, 0.0, 4)
    for mode in (sg.MODE_PHASES, sg.MODE_FUSED):
        u, _ = _gpu_run(g, mat, fields, srcs, dt, 4, mode)
        assert rel_err(u, ref_u) <= 1e-12


def test_fused_and_phase_paths_agree_over_many_steps():
    g, mat, fields, srcs = _setup("halfspace")
    dt = 0.3 * g.h / np.sqrt(np.max((4 * mat[1] + mat[2]) / mat[0]))
    a, _ = _gpu_run(g, mat, fields, srcs, dt, 40, sg.MODE_PHASES)
    b, _ = _gpu_run(g, mat, fields, srcs, dt, 40, sg.MODE_FUSED)
    m = solution_mask(g)
    assert rel_err(b[m], a[m]) <= 1e-11


def test_compute_time_step_matches_reference_formula():
    g, mat, _, _ = _setup("halfspace")
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in mat])
    dt, n = ew.compute_time_step(1.3, 0.6)
    d0 = 1.3 * g.h / np.sqrt(np.max((4 * mat[1] + mat[2]) / mat[0]))
    n0 = max(1, int(0.6 / d0 + 0.5))
    assert n == n0
    assert abs(dt - 0.6 / n0) <= 1e-15
    ew.close()
