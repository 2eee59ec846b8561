"""CUDA-graph replay of the time loop (sw4g_ew_set_graphs) against direct launches.

The graphed loop keeps the forcing time and the record row in device memory and
replays captured chunks of steps; the gradient replays its recompute and adjoint
segments.  Every result must be bit-identical to the direct launches: fields,
receiver records, misfit and gradients, FP64 and FP32-mixed.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.adjoint_util import AdjointCase, oracle_forward
from tests.gpu_util import dev, host, smooth_material

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _stream():
    import torch
    return torch.cuda.Stream()


def _forward(precision, graphs, nsteps=71):
    nx, ny, nz, h = 30, 28, 32, 0.05
    g = sg.grid_desc(nx, ny, nz, h, sg_gp=8, precision=precision)
    ew = sg.EW(g, stream=_stream())
    ew.set_material(*smooth_material(nx, ny, nz, seed=4))
    ew.add_source(sg.source_desc(0.5 * nx * h, 0.4 * ny * h, 0.5 * nz * h,
                                 moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=6.0,
                                 kind=sg.C6SMOOTHBUMP))
    ew.add_source(sg.source_desc(0.3 * nx * h, 0.6 * ny * h, 0.4 * nz * h, force=(1.0, -0.5, 0.2),
                                 freq=9.0, t0=0.1))
    rec = [(5, 7, 1), (15, 12, 9), (22, 20, 17)]
    ew.set_receivers(rec, [sg.REC_DISPLACEMENT, sg.REC_VELOCITY, sg.REC_STRAINS], nsteps + 1)
    ew.set_time_step(0.004)
    if graphs:
        ew.set_graphs(True)
    ew.step(nsteps, sg.MODE_FUSED)
    u = np.zeros(3 * ew.npts)
    um = np.zeros(3 * ew.npts)
    ew.get_fields(u, um)
    r = ew.records()
    t = ew.time
    ew.close()
    return u, um, r, t


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
def test_graphed_steps_bit_identical(precision):
    a = _forward(precision, False)
    b = _forward(precision, True)
    assert a[3] == b[3]
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)
    assert np.max(np.abs(a[2])) > 0


def test_graphed_topography_steps_bit_identical():
    from tests.test_gpu_topo import _long_case
    from tests.topo_util import smooth_topo_fields
    c = _long_case()
    dt = c.time_step(1.3)
    fields = smooth_topo_fields(c, seed=6)
    out = []
    for graphs in (False, True):
        ew = sg.EW(c.grid, stream=_stream(), topo=sg.topo_desc(**c.hill))
        ew.set_material(*[dev(q) for q in c.cart_mat])
        ew.set_material_grid(1, *[dev(q) for q in c.curv_mat])
        for s in c.sources:
            ew.add_source(s)
        ew.set_time_step(dt, 0.0)
        ew.set_fields(dev(fields[0]), dev(fields[1]))
        ew.set_fields_grid(1, dev(fields[2]), dev(fields[3]))
        if graphs:
            ew.set_graphs(True)
        ew.step(65, sg.MODE_FUSED)
        res = [dev(np.zeros_like(f)) for f in fields]
        ew.get_fields(res[0], res[1])
        ew.get_fields_grid(1, res[2], res[3])
        out.append([host(r) for r in res])
        ew.close()
    for x, y in zip(*out):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("precision,memory", [(sg.FP64, 0), (sg.FP64, -1), (sg.MIXED, 0)])
def test_graphed_gradient_bit_identical(precision, memory):
    c = AdjointCase(nsteps=47)
    obs_case = AdjointCase(seed=11, nsteps=47)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    res = []
    for graphs in (False, True):
        g = sg.grid_desc(c.nx, c.ny, c.nz, c.h, bc=[c.grid.bc[s] for s in range(6)],
                         sg_gp=c.grid.sg_gp, sg_damping=c.grid.sg_damping, precision=precision)
        ew = sg.EW(g, stream=_stream())
        ew.set_material(*c.mat)
        for s in c.sources:
            ew.add_source(s)
        ew.set_time_step(c.dt, 0.0)
        ew.set_receivers(c.rec, [sg.REC_DISPLACEMENT] * len(c.rec), c.nsteps + 1)
        ew.set_gradient_memory(memory)  # 0: segments recomputed (graphed), -1: kept
        if graphs:
            ew.set_graphs(True)
        gr = [np.zeros(c.npts) for _ in range(3)]
        J = ew.gradient(c.nsteps, 9, obs, *gr)  # 5 full segments of 9 steps and one of 2
        res.append((J, gr))
        ew.close()
    assert res[0][0] == res[1][0]
    for x, y in zip(res[0][1], res[1][1]):
        assert np.array_equal(x, y)
    assert max(np.max(np.abs(x)) for x in res[0][1]) > 0


def test_graphs_need_an_explicit_stream():
    import torch
    g = sg.grid_desc(16, 16, 16, 0.1)
    ew = sg.EW(g, stream=torch.cuda.default_stream())
    with pytest.raises(sg.Sw4gError):
        ew.set_graphs(True)
    ew.close()
