"""Size-independent properties at the workloads' full sizes (GPU).

The other GPU tests compare with the oracle at sizes the oracle finishes in
seconds; these run the full configurations:
  * the kernel-level operator at 512^3 (the layer-over-halfspace workload's grid)
    against the oracle's rhs4sg (OpenMP on the host), to 1e-13 relative;
  * linearity of the fused FP64 step at 512^3 (no sources: the step is linear in
    the levels), to 1e-11 relative;
  * the FP32-mixed step against FP64 at 512^3 (3 steps) and on the topography
    workload's 384 x 384 x 128 two-grid set-up (20 steps), relative L2 <= 1e-6;
  * CUDA-graph replay bit-identical to direct launches at 512^3 with sources and
    receivers;
  * the adjoint gradient at 256^3 (the adjoint workload's grid, 5 % log-normal
    medium) against a central finite difference of the misfit, to 1e-6.
"""
import ctypes

import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _axes(n, dev="cuda"):
    return torch.arange(n + 4, dtype=torch.float64, device=dev)


def _sep(n, seed, scale=1.0):
    """A smooth separable field sin(a i + p) sin(b j + q) cos(c k + r) on the
    (n+4)^3 array, 3 components, on the device."""
    rng = np.random.default_rng(seed)
    x = _axes(n)
    out = []
    for _ in range(3):
        f = rng.uniform(0.02, 0.2, 3)
        p = rng.uniform(0, 2 * np.pi, 3)
        out.append((torch.cos(f[2] * x + p[2])[:, None, None] * torch.sin(f[1] * x + p[1])[None, :, None] *
                    torch.sin(f[0] * x + p[0])[None, None, :]).reshape(-1))
    return scale * torch.cat(out)


def _material(n, seed, rho0=2.0, cs=1.0, cp=1.8, amp=0.15):
    rng = np.random.default_rng(seed)
    x = _axes(n)

    def field(base):
        f = rng.uniform(0.01, 0.05, 3)
        p = rng.uniform(0, 2 * np.pi, 3)
        return base * (1 + amp * torch.sin(f[2] * x + p[2])[:, None, None] *
                       torch.cos(f[1] * x + p[1])[None, :, None] * torch.sin(f[0] * x + p[0])[None, None, :])
    rho = field(rho0)
    mu = field(rho0 * cs * cs)
    la = torch.clamp(field(rho0 * cp * cp) - 2 * mu, min=0.0) + 0.1 * mu
    return [a.reshape(-1).contiguous() for a in (rho, mu, la)]


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def test_rhs4sg_full_size_matches_oracle():
    n = 512
    h = 50.0
    u = _sep(n, 1)
    rho, mu, la = _material(n, 2)
    rng = np.random.default_rng(3)
    st = [torch.tensor(1 + 0.2 * rng.random(n + 4), device="cuda") for _ in range(3)]
    bounds = (-1, n + 2, -1, n + 2, -1, n + 2)
    lu = torch.zeros_like(u)
    onesided = (0, 0, 0, 0, 1, 0)
    arr = (ctypes.c_int * 6)(*onesided)
    stream = torch.cuda.current_stream().cuda_stream or None
    sg.check(sg.lib().sw4g_rhs4sg(1, *bounds, n, arr, lu.data_ptr(), u.data_ptr(), mu.data_ptr(),
                                  la.data_ptr(), h, st[0].data_ptr(), st[1].data_ptr(),
                                  st[2].data_ptr(), stream), "sw4g_rhs4sg")
    torch.cuda.synchronize()
    got = lu.cpu().numpy()
    ref = np.zeros_like(got)
    O.rhs4sg(1, bounds, n, list(onesided), ref, u.cpu().numpy(), mu.cpu().numpy(), la.cpu().numpy(), h,
             *[s.cpu().numpy() for s in st])
    assert float(np.max(np.abs(got - ref)) / np.max(np.abs(ref))) <= 1e-13


def _c2_ew(n, precision=sg.FP64, stream=None):
    g = sg.grid_desc(n, n, n, 50.0, sg_gp=30, precision=precision)
    ew = sg.EW(g, stream=stream)
    ew.set_material(*_material(n, 5, rho0=2600.0, cs=2000.0, cp=4000.0))
    ew.set_time_step(0.008)
    return ew


def _run(ew, u, um, nsteps):
    ew.set_fields(u, um)
    ew.step(nsteps, sg.MODE_FUSED)
    out = torch.zeros_like(u)
    ew.get_fields(out, None)
    torch.cuda.synchronize()
    return out


def test_step_linearity_full_size():
    n = 512
    ew = _c2_ew(n)
    s1 = (_sep(n, 11, 1e-3), _sep(n, 12, 1e-3))
    s2 = (_sep(n, 13, 1e-3), _sep(n, 14, 1e-3))
    a = _run(ew, *s1, 3)
    b = _run(ew, *s2, 3)
    c = _run(ew, s1[0] + 0.5 * s2[0], s1[1] + 0.5 * s2[1], 3)
    ew.close()
    assert _rel(c, a + 0.5 * b) <= 1e-11


def test_mixed_close_to_fp64_full_size():
    n = 512
    u, um = _sep(n, 21, 1e-3), _sep(n, 22, 1e-3)
    ew = _c2_ew(n)
    a = _run(ew, u, um, 3)
    ew.close()
    ew = _c2_ew(n, sg.MIXED)
    b = _run(ew, u, um, 3)
    ew.close()
    assert float((b - a).norm() / a.norm()) <= 1e-6


def test_graphed_steps_full_size_bit_identical():
    n = 512
    res = []
    for graphs in (False, True):
        ew = _c2_ew(n, stream=torch.cuda.Stream())
        ew.add_source(sg.source_desc(12800.0, 12800.0, 2000.0, moment=(0, 1e18, 0, 0, 0, 0), freq=20.0,
                                     t0=0.3))
        ew.set_receivers([(100, 120, 1), (300, 200, 1)], [sg.REC_DISPLACEMENT, sg.REC_VELOCITY], 32)
        if graphs:
            ew.set_graphs(True)
        zero = torch.zeros(3 * ew.npts, dtype=torch.float64, device="cuda")
        u = _run(ew, zero, zero, 31)
        res.append((u, ew.records()))
        ew.close()
    assert torch.equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])
    assert float(res[0][0].abs().max()) > 0


def test_topography_mixed_close_to_fp64_full_size():
    import bench
    cfg = bench.c3_config(384, 384, 128)
    out = []
    stream = torch.cuda.Stream()
    for prec in (sg.FP64, sg.MIXED):
        ew, nc, ncart, dt = bench._make_topo_ew(sg, cfg, stream, prec)
        with torch.cuda.stream(stream):
            ew.step(20, sg.MODE_FUSED)
        n0, n1 = 3 * ew.grid_dims(0)[3], 3 * ew.grid_dims(1)[3]
        f = [torch.zeros(n, dtype=torch.float64, device="cuda") for n in (n0, n1)]
        ew.get_fields(f[0], None)
        ew.get_fields_grid(1, f[1], None)
        torch.cuda.synchronize()
        out.append(torch.cat(f))
        ew.close()
    a, b = out
    assert float(a.abs().max()) > 0
    assert float((b - a).norm() / a.norm()) <= 1e-6


def test_gradient_matches_finite_difference_full_size():
    import bench
    cfg = bench.c4_config(256)
    N, C = 20, 10
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        ew, dt = bench._make_c4(sg, torch, cfg, stream, N)
        ew.close()
        ew0, _ = bench._make_c4(sg, torch, cfg, stream, N, homogeneous=True, dt=dt)
        ew0.step(N, sg.MODE_FUSED)
        obs = torch.zeros(ew0.record_shape(), dtype=torch.float64, device="cuda")
        ew0.records(obs)
        ew0.close()
        ew, _ = bench._make_c4(sg, torch, cfg, stream, N, dt=dt)
        g = [torch.zeros(ew.npts, dtype=torch.float64, device="cuda") for _ in range(3)]
        J = ew.gradient(N, C, obs, *g)
        ew.close()
        # the medium itself, for the direction (same seeds as the workload)
        n = cfg["n"]
        shape = (n + 4, n + 4, n + 4)
        pr, ps, pv = (bench._lognormal(torch, shape, cfg["std"], cfg["corr"], cfg["seed"] + q)
                      for q in range(3))
        rho = cfg["rho"] * pr
        mu = rho * (cfg["vs"] * ps) ** 2
        la = rho * (cfg["vp"] * pv) ** 2 - 2 * mu
        mat = [a.reshape(-1) for a in (rho, mu, la)]
        d = [(bench._lognormal(torch, shape, 0.3, 5.0, 900 + q).reshape(-1) - 1.0) * m
             for q, m in enumerate(mat)]
        pred = float(sum((gq * dq).sum() for gq, dq in zip(g, d)))
        eps = 1e-5

        def misfit(m):
            e, _ = bench._make_c4(sg, torch, cfg, stream, N, dt=dt)
            e.set_material(*m)
            e.step(N, sg.MODE_FUSED)
            r = torch.zeros(e.record_shape(), dtype=torch.float64, device="cuda")
            e.records(r)
            e.close()
            return 0.5 * float(((r - obs) ** 2).sum())
        Jp = misfit([m + eps * dq for m, dq in zip(mat, d)])
        Jm = misfit([m - eps * dq for m, dq in zip(mat, d)])
    fd = (Jp - Jm) / (2 * eps)
    assert J > 0 and abs(pred) > 0
    assert abs(fd - pred) <= 1e-6 * abs(pred), (fd, pred)
