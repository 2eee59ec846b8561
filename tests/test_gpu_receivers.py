"""Receiver records on the GPU against the oracle.

The oracle steps the same problem and samples each receiver with its restatement
of EW::extractRecordData (src/EW.C:5854-6072) before rotating the levels, as the
reference's time loop does (src/EW.C:2797-2835).  Tolerance: the fields agree to
1e-12 relative (test_gpu_step.py); a recorded value is a field value or a
centred difference of two, so each record column is held to 1e-10 relative to
its largest magnitude.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.gpu_util import OracleProblem, dev, host, smooth_fields, smooth_material

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _case(precision=sg.FP64):
    nx, ny, nz = 34, 30, 36
    h = 0.05
    g = sg.grid_desc(nx, ny, nz, h, bc=(2, 2, 2, 2, 0, 2), sg_gp=8, precision=precision)
    mat = smooth_material(nx, ny, nz, seed=23)
    fields = smooth_fields(nx, ny, nz, seed=29)
    srcs = [sg.source_desc(0.45 * nx * h, 0.5 * ny * h, 0.4 * nz * h,
                           moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=6.0,
                           kind=sg.C6SMOOTHBUMP)]
    dt = 0.3 * h / float(np.sqrt(np.max((4 * mat[1] + mat[2]) / mat[0])))
    # every mode once, on the free surface, in the interior and inside the supergrid layer
    recs = [((17, 15, 1), sg.REC_DISPLACEMENT), ((17, 15, 1), sg.REC_VELOCITY),
            ((10, 12, 9), sg.REC_DIV), ((20, 8, 14), sg.REC_CURL), ((5, 25, 20), sg.REC_STRAINS),
            ((30, 3, 33), sg.REC_GRADIENT), ((2, 2, 34), sg.REC_VELOCITY)]
    return g, mat, fields, srcs, dt, recs


def _gpu_records(g, mat, fields, srcs, dt, recs, nsteps, mode, capacity=None):
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in mat])
    for s in srcs:
        ew.add_source(s)
    ew.set_time_step(dt, 0.0)
    ew.set_fields(dev(fields[0]), dev(fields[1]))
    ew.set_receivers([r[0] for r in recs], [r[1] for r in recs], capacity or nsteps + 1)
    ew.step(nsteps, mode)
    out = ew.records()
    dv = dev(np.zeros_like(out))
    ew.records(dv)
    assert np.array_equal(host(dv), out)
    ew.close()
    return out


def _col_rel_err(a, b):
    scale = np.maximum(np.abs(b).max(axis=0), 1e-300)
    return float((np.abs(a - b).max(axis=0) / scale).max())


@pytest.mark.parametrize("mode", [sg.MODE_PHASES, sg.MODE_FUSED])
def test_records_match_oracle(mode):
    g, mat, fields, srcs, dt, recs = _case()
    nsteps = 8
    _, _, ref = OracleProblem(g, *mat, dt, srcs).run(*fields, 0.0, nsteps, receivers=recs)
    got = _gpu_records(g, mat, fields, srcs, dt, recs, nsteps, mode)
    assert got.shape == ref.shape == (nsteps + 1, sum(O.REC_VALUES[m] for _, m in recs))
    assert _col_rel_err(got, ref) <= 1e-10


def test_mixed_records_close_to_fp64():
    g, mat, fields, srcs, dt, recs = _case()
    gm = _case(sg.MIXED)[0]
    a = _gpu_records(g, mat, fields, srcs, dt, recs, 40, sg.MODE_FUSED)
    b = _gpu_records(gm, mat, fields, srcs, dt, recs, 40, sg.MODE_FUSED)
    assert float(np.linalg.norm(b - a) / np.linalg.norm(a)) <= 1e-6


def test_record_capacity_and_bad_receivers_rejected():
    g, mat, fields, srcs, dt, recs = _case()
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in mat])
    ew.set_time_step(dt, 0.0)
    ew.set_receivers([(5, 5, 5)], [sg.REC_DISPLACEMENT], 5)
    with pytest.raises(sg.Sw4gError):
        ew.step(5)  # initial row + 5 steps > 5 rows: refused before any work
    assert ew.record_shape() == (0, 3)
    ew.step(4)
    assert ew.record_shape() == (5, 3)
    with pytest.raises(sg.Sw4gError):
        ew.step(1)
    for ijk, m in [((5, 5, 5), 9), ((-2, 5, 5), sg.REC_DISPLACEMENT), ((-1, 5, 5), sg.REC_DIV)]:
        with pytest.raises(sg.Sw4gError):
            ew.set_receivers([ijk], [m], 10)
    ew.set_receivers([], [], 0)
    ew.step(3)  # no receivers: no capacity limit
    assert ew.launches_per_step() > 0
    ew.close()
