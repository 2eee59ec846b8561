"""Stream order between torch and the library for device tensors.

An EW object runs on its own CUDA stream.  Device tensors that torch produced on
its current stream must be complete before the library reads them, and tensors
the library fills must be complete before torch reads them.  Each test keeps one
stream busy with a timed spin (torch.cuda._sleep) so that a missing dependency
would read stale values deterministically.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from tests.gpu_util import smooth_fields

pytestmark = pytest.mark.gpu

SPIN = 200_000_000  # GPU cycles, about 0.1 s at 2 GHz


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()


def test_inputs_wait_for_torch_stream():
    import torch
    g = sg.grid_desc(16, 16, 16, 0.1)
    s = torch.cuda.Stream()
    ew = sg.EW(g, stream=s)
    n = ew.npts
    rho, mu, la = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3))
    torch.cuda._sleep(SPIN)  # on torch's current stream, before the values exist
    rho.fill_(2.0)
    mu.fill_(3.0)
    la.fill_(1.0)
    ew.set_material(rho, mu, la)
    dt, nsteps = ew.compute_time_step(1.0, 1.0)
    ew.close()
    ref = sg.EW(g)
    ref.set_material(*(np.full(n, v) for v in (2.0, 3.0, 1.0)))
    assert (dt, nsteps) == ref.compute_time_step(1.0, 1.0)
    ref.close()


def test_outputs_complete_before_torch_reads():
    import torch
    g = sg.grid_desc(16, 16, 16, 0.1)
    s = torch.cuda.Stream()
    ew = sg.EW(g, stream=s)
    u, um = smooth_fields(16, 16, 16, seed=5)
    ew.set_fields(u, um)  # host arrays: synchronous
    out = torch.zeros(3 * ew.npts, dtype=torch.float64, device="cuda")
    with torch.cuda.stream(s):
        torch.cuda._sleep(SPIN)  # the library's stream is busy when the copy is queued
    ew.get_fields(out, None)
    got = out.cpu().numpy()  # on torch's current stream
    ew.close()
    assert np.array_equal(got, u)


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
@pytest.mark.parametrize("graphs", [False, True])
def test_rows_beside_the_stage_match_rows_after_it(precision, graphs):
    """The one-sided rows next to a free surface run on a second stream beside each
    stage kernel (sw4g_dev_set_rows_overlap, default on): the levels after a run are
    bit-identical to running them after the stage on the object's stream, with and
    without CUDA graphs."""
    import torch
    from tests.gpu_util import dev, host, smooth_material
    nx, ny, nz, h = 40, 36, 30, 0.05
    rho, mu, la = smooth_material(nx, ny, nz, seed=3)
    u, um = smooth_fields(nx, ny, nz, seed=4)
    dt = 0.3 * h / float(np.sqrt(np.max((4 * mu + la) / rho)))
    out = []
    for on in (True, False):
        sg.set_rows_overlap(on)
        s = torch.cuda.Stream()
        g = sg.grid_desc(nx, ny, nz, h, bc=(2, 2, 2, 2, 0, 2), sg_gp=6, precision=precision)
        ew = sg.EW(g, stream=s)
        ew.set_material(*[dev(a) for a in (rho, mu, la)])
        ew.add_source(sg.source_desc(0.5 * nx * h, 0.5 * ny * h, 2 * h, force=(1.0, 0.5, -0.3), freq=6.0))
        ew.set_time_step(dt, 0.0)
        ew.set_fields(dev(u), dev(um))
        if graphs:
            ew.set_graphs(True)
        ew.step(7, sg.MODE_FUSED)
        a = dev(np.zeros_like(u))
        ew.get_fields(a, None)
        torch.cuda.synchronize()
        out.append(host(a))
        ew.close()
    sg.set_rows_overlap(True)
    assert np.array_equal(out[0], out[1])
    assert np.max(np.abs(out[0])) > 0


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
@pytest.mark.parametrize("graphs", [False, True])
def test_curvilinear_rows_beside_the_stages_match(precision, graphs):
    """With topography the curvilinear grid's top rows run on a second stream beside
    both grids' stage kernels: the levels of both grids after a run are bit-identical
    to running every piece in order on the object's stream."""
    import torch
    from tests.gpu_util import dev, host
    from tests.topo_util import TopoCase, smooth_topo_fields
    c = TopoCase(30, 28, 22, 0.1, zmax_topo=1.0, amp=0.2, xc=1.4, yc=1.3, lx=0.6, ly=0.5, gp=5,
                 sources=[sg.source_desc(1.5, 1.4, 0.6, force=(1.0, -0.5, 0.3), freq=8.0, t0=0.1)],
                 precision=precision)
    dt = c.time_step(1.3)
    fields = smooth_topo_fields(c, seed=7)
    out = []
    for on in (True, False):
        sg.set_rows_overlap(on)
        s = torch.cuda.Stream()
        ew = sg.EW(c.grid, stream=s, topo=sg.topo_desc(**c.hill))
        ew.set_material(*[dev(a) for a in c.cart_mat])
        ew.set_material_grid(1, *[dev(a) for a in c.curv_mat])
        for src in c.sources:
            ew.add_source(src)
        ew.set_time_step(dt, 0.0)
        ew.set_fields(dev(fields[0]), dev(fields[1]))
        ew.set_fields_grid(1, dev(fields[2]), dev(fields[3]))
        if graphs:
            ew.set_graphs(True)
        ew.step(6, sg.MODE_FUSED)
        r = [dev(np.zeros_like(f)) for f in fields[::2]]
        ew.get_fields(r[0], None)
        ew.get_fields_grid(1, r[1], None)
        torch.cuda.synchronize()
        out.append([host(x) for x in r])
        ew.close()
    sg.set_rows_overlap(True)
    for x, y in zip(*out):
        assert np.array_equal(x, y)
        assert np.max(np.abs(x)) > 0
