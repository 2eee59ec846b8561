"""The discrete adjoint on the GPU (sw4g_ew_gradient).

* Against the oracle's adjoint (tests/test_oracle_adjoint.py checks it by dot
  products and finite differences): misfit to 1e-12, gradients to 1e-9 relative
  to each gradient's largest magnitude, for several checkpoint spacings.
* Against central finite differences of GPU forward runs on a 48^3 copy of the
  adjoint workload (smooth 5% log-normal heterogeneity, one point force, 16
  receivers): the directional derivative along a smooth random direction in
  (rho, mu, lambda) to 1e-6 relative.
* Segments kept from the forward run (sw4g_ew_set_gradient_memory) instead of
  recomputed give bit-identical results.
* Free-surface z sides (one-sided SBP rows, ghost plane from the traction
  condition) with receivers on the free surface: the same bars against the
  oracle's free-surface adjoint (top, bottom, both) and against finite differences
  at 48^3; the FP32-mixed form against the FP64 gradient.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.adjoint_util import AdjointCase, oracle_forward, oracle_gradient, smooth_random
from tests.gpu_util import dev, host

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy")


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _ew(case, mat=None, precision=sg.FP64):
    mat = case.mat if mat is None else mat
    g = case.grid
    if precision != sg.FP64:
        g = sg.grid_desc(case.nx, case.ny, case.nz, case.h, bc=[g.bc[s] for s in range(6)],
                         sg_gp=g.sg_gp, sg_damping=g.sg_damping, sg_order=g.sg_order,
                         precision=precision)
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in mat])
    for s in case.sources:
        ew.add_source(s)
    ew.set_time_step(case.dt, 0.0)
    ew.set_receivers(case.rec, [sg.REC_DISPLACEMENT] * len(case.rec), case.nsteps + 1)
    return ew


def _gpu_gradient(case, obs, ckpt, precision=sg.FP64, memory=None):
    ew = _ew(case, precision=precision)
    if memory is not None:
        ew.set_gradient_memory(memory)
    g = [dev(np.zeros(case.npts)) for _ in range(3)]
    J = ew.gradient(case.nsteps, ckpt, dev(obs), *g)
    # the object ends after the forward run
    assert ew.time == pytest.approx(case.nsteps * case.dt, rel=1e-14)
    u = dev(np.zeros(3 * case.npts))
    ew.get_fields(u, None)
    ew.close()
    return J, [host(x) for x in g], host(u)


def _gpu_misfit(case, obs, mat):
    ew = _ew(case, mat)
    ew.step(case.nsteps, sg.MODE_FUSED)
    rec = ew.records()
    ew.close()
    return 0.5 * float(np.sum((rec - obs) ** 2))


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


# memory 0: every segment but the last recomputed from its checkpoint; None: the
# default budget, which keeps every segment of these small cases
@pytest.mark.parametrize("ckpt,memory", [(30, None), (7, 0), (7, None), (1, 0)])
def test_gradient_matches_oracle_adjoint(ckpt, memory):
    c = AdjointCase()
    obs_case = AdjointCase(seed=11)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J0, gr, gm, gl = oracle_gradient(c, obs)
    J, (r, m, l), ufin = _gpu_gradient(c, obs, ckpt, memory=memory)
    assert J == pytest.approx(J0, rel=1e-12)
    assert _rel(r, gr) <= 1e-9
    assert _rel(m, gm) <= 1e-9
    assert _rel(l, gl) <= 1e-9
    levels = oracle_forward(c)[0]
    assert _rel(ufin, levels[-1]) <= 1e-12


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
def test_gradient_receivers_sharing_a_point(precision):
    # three receivers on one grid point and two on another: their adjoint sources add
    # up at the point (a race between receivers of one point would drop some)
    c = AdjointCase()
    c.rec = c.rec + [c.rec[0], c.rec[0], c.rec[2]]
    obs_case = AdjointCase(seed=11)
    obs_case.rec = c.rec
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J0, gr, gm, gl = oracle_gradient(c, obs)
    J, g, _ = _gpu_gradient(c, obs, 10, precision=precision)
    tol = 1e-9 if precision == sg.FP64 else 1e-5
    assert J == pytest.approx(J0, rel=1e-12 if precision == sg.FP64 else 1e-6)
    for a, b in zip(g, (gr, gm, gl)):
        assert _rel(a, b) <= tol


def test_gradient_matches_finite_differences_48():
    # the finite-difference copy of the adjoint workload: 48^3, 5% log-normal
    # heterogeneity with correlation length 10h (here 10 points), 16 receivers
    c = AdjointCase(shape=(48, 48, 48), h=0.05, gp=10, seed=21, nsteps=160, nrec=16,
                    vp=1.732, vs=1.0, rho=1.0)
    from scipy.ndimage import gaussian_filter  # noqa: F401  (smooth_random needs scipy)
    obs_case = AdjointCase(shape=(48, 48, 48), h=0.05, gp=10, seed=22, nsteps=160, nrec=16,
                           vp=1.732, vs=1.0, rho=1.0)
    obs_case.rec = c.rec
    ew = _ew(obs_case)
    ew.step(obs_case.nsteps, sg.MODE_FUSED)
    obs = ew.records()
    ew.close()
    J, (gr, gm, gl), _ = _gpu_gradient(c, obs, 40)
    shape = (c.nz + 4, c.ny + 4, c.nx + 4)
    dirs = [smooth_random(shape, 60 + q, corr=5.0, amp=0.3).reshape(-1) - 1.0 for q in range(3)]
    dm = [dirs[q] * c.mat[q] for q in range(3)]
    pred = float(gr @ dm[0] + gm @ dm[1] + gl @ dm[2])
    eps = 1e-5
    Jp = _gpu_misfit(c, obs, [c.mat[q] + eps * dm[q] for q in range(3)])
    Jm = _gpu_misfit(c, obs, [c.mat[q] - eps * dm[q] for q in range(3)])
    fd = (Jp - Jm) / (2 * eps)
    assert J > 0 and abs(pred) > 0
    assert abs(fd - pred) <= 1e-6 * abs(pred), (fd, pred)


def test_gradient_rejects_unsupported_set_ups():
    c = AdjointCase(shape=(16, 16, 16), nsteps=4)
    obs = np.zeros((5, 3 * len(c.rec)))
    g = [np.zeros(c.npts) for _ in range(3)]
    # a free surface whose one-sided rows meet the other side's rows (nz < 22), and
    # one whose z supergrid layer reaches the ten planes next to it
    thin = sg.grid_desc(16, 16, 16, c.h, bc=(2, 2, 2, 2, 0, 2), sg_gp=5)
    layered = sg.grid_desc(40, 40, 24, c.h, bc=(2, 2, 2, 2, 0, 2), sg_gp=16)
    for grid in (thin, layered):
        npts = (grid.nx + 4) * (grid.ny + 4) * (grid.nz + 4)
        ew = sg.EW(grid)
        ew.set_material(*[dev(np.full(npts, v)) for v in (1.0, 1.0, 1.0)])
        ew.set_time_step(c.dt)
        ew.set_receivers(c.rec, [sg.REC_DISPLACEMENT] * len(c.rec), 5)
        with pytest.raises(sg.Sw4gError):
            ew.gradient(4, 2, obs, *g)
        ew.close()
    ew = _ew(c)
    ew.set_receivers(c.rec, [sg.REC_VELOCITY] * len(c.rec), 5)
    with pytest.raises(sg.Sw4gError):
        ew.gradient(4, 2, obs, *g)
    ew.set_receivers(c.rec, [sg.REC_DISPLACEMENT] * len(c.rec), 3)
    with pytest.raises(sg.Sw4gError):  # record capacity below nsteps + 1
        ew.gradient(4, 2, obs, *g)
    ew.close()


def test_torch_autograd_wrapper_matches_finite_differences():
    import torch
    from sw4lite_gb300 import autograd as sa
    c = AdjointCase(shape=(24, 22, 26), nsteps=40)
    obs_case = AdjointCase(shape=(24, 22, 26), nsteps=40, seed=11)
    obs = torch.tensor(obs_case.records(oracle_forward(obs_case)[0][1:]), device="cuda")
    shot = sa.Shot(grid=c.grid, dt=c.dt, nsteps=c.nsteps, checkpoint_every=10, receivers=c.rec,
                   observed=obs, sources=c.sources)
    rho, mu, la = [torch.tensor(a, device="cuda", requires_grad=True) for a in c.mat]
    J = sa.misfit(rho, mu, la, shot)
    J.backward()
    shape = (c.nz + 4, c.ny + 4, c.nx + 4)
    d = [torch.tensor(smooth_random(shape, 80 + q, corr=3.0, amp=0.3).reshape(-1) - 1.0,
                      device="cuda") * x.detach() for q, x in enumerate((rho, mu, la))]
    pred = float(sum((x.grad * dx).sum() for x, dx in zip((rho, mu, la), d)))
    eps = 1e-5
    base = [x.detach() for x in (rho, mu, la)]
    Jp = sa.forward_misfit(*[b + eps * dx for b, dx in zip(base, d)], shot)
    Jm = sa.forward_misfit(*[b - eps * dx for b, dx in zip(base, d)], shot)
    fd = (Jp - Jm) / (2 * eps)
    assert abs(fd - pred) <= 1e-6 * abs(pred), (fd, pred)
    # and the FP64 reference gradient of the oracle
    _, gr, gm, gl = oracle_gradient(c, obs.cpu().numpy())
    for x, ref in zip((rho, mu, la), (gr, gm, gl)):
        assert _rel(x.grad.cpu().numpy(), ref) <= 1e-9


@pytest.mark.parametrize("ckpt", [10, 3])
def test_mixed_gradient_close_to_fp64(ckpt):
    # FP32-mixed adjoint (double-float levels, FP32 stencils and gradient terms, FP64
    # accumulation) against the FP64 gradient of the same run: misfit to 1e-6,
    # gradients to 1e-5 relative to each gradient's largest magnitude (measured 7e-7)
    c = AdjointCase(nsteps=40)
    obs_case = AdjointCase(seed=11, nsteps=40)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J0, g0, _ = _gpu_gradient(c, obs, ckpt)
    J1, g1, _ = _gpu_gradient(c, obs, ckpt, precision=sg.MIXED)
    assert J1 == pytest.approx(J0, rel=1e-6)
    for a, b in zip(g1, g0):
        assert _rel(a, b) <= 1e-5, _rel(a, b)


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
def test_kept_segments_bit_identical(precision):
    """No extra segments kept, two kept, and all kept: identical misfit and gradients."""
    c = AdjointCase(nsteps=47)
    obs_case = AdjointCase(seed=11, nsteps=47)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    ckpt = 9  # 5 full segments of 9 steps and one of 2
    seg_bytes = (2 * ckpt + 2) * 3 * c.npts * 8
    res = [_gpu_gradient(c, obs, ckpt, precision=precision, memory=m)
           for m in (0, 2 * seg_bytes + seg_bytes // 2, -1)]
    for J, g, u in res[1:]:
        assert J == res[0][0]
        for x, y in zip(g, res[0][1]):
            assert np.array_equal(x, y)
        assert np.array_equal(u, res[0][2])
    assert max(np.max(np.abs(x)) for x in res[0][1]) > 0


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
def test_repeated_gradients_reuse_buffers(precision):
    """A second gradient of the same shape on the same object (its buffers kept from
    the first) and one of another shape (buffers made again) equal fresh objects'."""
    c = AdjointCase(nsteps=31)
    obs_case = AdjointCase(seed=12, nsteps=31)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    seg_bytes = (2 * 8 + 2) * 3 * c.npts * 8
    fresh = {k: _gpu_gradient(c, obs, k, precision=precision, memory=seg_bytes) for k in (8, 6)}
    ew = _ew(c, precision=precision)
    ew.set_gradient_memory(seg_bytes)
    zero = dev(np.zeros(3 * c.npts))
    for k in (8, 8, 6):
        ew.set_fields(zero, zero)
        ew.set_time_step(c.dt, 0.0)
        g = [dev(np.zeros(c.npts)) for _ in range(3)]
        J = ew.gradient(c.nsteps, k, dev(obs), *g)
        assert J == fresh[k][0]
        for x, y in zip(g, fresh[k][1]):
            assert np.array_equal(host(x), y)
    ew.close()


# ---- free-surface z sides ----

FS_CASES = [((2, 2, 2, 2, 0, 2), 1), ((2, 2, 2, 2, 2, 0), 24), ((2, 2, 2, 2, 0, 0), 1)]


@pytest.mark.parametrize("bc,rec_k", FS_CASES)
@pytest.mark.parametrize("ckpt,memory", [(30, None), (7, 0)])
def test_fs_gradient_matches_oracle_adjoint(bc, rec_k, ckpt, memory):
    kw = dict(shape=(16, 15, 24), bc=bc, rec_k=rec_k)
    c = AdjointCase(**kw)
    obs_case = AdjointCase(seed=11, **kw)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J0, gr, gm, gl = oracle_gradient(c, obs)
    J, (r, m, l), ufin = _gpu_gradient(c, obs, ckpt, memory=memory)
    assert J == pytest.approx(J0, rel=1e-12)
    assert _rel(r, gr) <= 1e-9
    assert _rel(m, gm) <= 1e-9
    assert _rel(l, gl) <= 1e-9


def test_fs_gradient_matches_finite_differences_48():
    # the 48^3 copy of the adjoint workload with a free surface on top and the 16
    # receivers on it (supergrid on the other five sides)
    kw = dict(shape=(48, 48, 48), h=0.05, gp=10, nsteps=160, nrec=16, vp=1.732, vs=1.0, rho=1.0,
              bc=(2, 2, 2, 2, 0, 2), rec_k=1)
    c = AdjointCase(seed=21, **kw)
    obs_case = AdjointCase(seed=22, **kw)
    obs_case.rec = c.rec
    ew = _ew(obs_case)
    ew.step(obs_case.nsteps, sg.MODE_FUSED)
    obs = ew.records()
    ew.close()
    J, (gr, gm, gl), _ = _gpu_gradient(c, obs, 40)
    shape = (c.nz + 4, c.ny + 4, c.nx + 4)
    dirs = [smooth_random(shape, 70 + q, corr=5.0, amp=0.3).reshape(-1) - 1.0 for q in range(3)]
    dm = [dirs[q] * c.mat[q] for q in range(3)]
    pred = float(gr @ dm[0] + gm @ dm[1] + gl @ dm[2])
    eps = 1e-5
    Jp = _gpu_misfit(c, obs, [c.mat[q] + eps * dm[q] for q in range(3)])
    Jm = _gpu_misfit(c, obs, [c.mat[q] - eps * dm[q] for q in range(3)])
    fd = (Jp - Jm) / (2 * eps)
    assert J > 0 and abs(pred) > 0
    assert abs(fd - pred) <= 1e-6 * abs(pred), (fd, pred)


@pytest.mark.parametrize("bc,rec_k", FS_CASES[:2])
def test_fs_mixed_gradient_close_to_fp64(bc, rec_k):
    kw = dict(shape=(16, 15, 24), bc=bc, rec_k=rec_k, nsteps=40)
    c = AdjointCase(**kw)
    obs_case = AdjointCase(seed=11, **kw)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J0, g0, _ = _gpu_gradient(c, obs, 10)
    J1, g1, _ = _gpu_gradient(c, obs, 10, precision=sg.MIXED)
    assert J1 == pytest.approx(J0, rel=1e-6)
    for a, b in zip(g1, g0):
        assert _rel(a, b) <= 1e-5, _rel(a, b)


# ---- sixth-order supergrid damping ----
# 12 steps: with these 5-point layers the sixth-order scheme has a mode that grows
# without bound after a few tens of steps (the reference formulation too).

@pytest.mark.parametrize("bc,rec_k,shape", [((2,) * 6, None, (20, 18, 22)),
                                            ((2, 2, 2, 2, 0, 2), 1, (16, 15, 24))])
@pytest.mark.parametrize("ckpt,memory", [(12, None), (5, 0)])
def test_sg6_gradient_matches_oracle_adjoint(bc, rec_k, shape, ckpt, memory):
    kw = dict(shape=shape, bc=bc, rec_k=rec_k, sg_order=6, damping=0.005, nsteps=12)
    c = AdjointCase(**kw)
    obs_case = AdjointCase(seed=11, **kw)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J0, gr, gm, gl = oracle_gradient(c, obs)
    J, (r, m, l), _ = _gpu_gradient(c, obs, ckpt, memory=memory)
    assert J == pytest.approx(J0, rel=1e-12)
    assert _rel(r, gr) <= 1e-9
    assert _rel(m, gm) <= 1e-9
    assert _rel(l, gl) <= 1e-9


def test_sg6_mixed_gradient_close_to_fp64():
    kw = dict(sg_order=6, damping=0.005, nsteps=12)
    c = AdjointCase(**kw)
    obs_case = AdjointCase(seed=11, **kw)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J0, g0, _ = _gpu_gradient(c, obs, 4)
    J1, g1, _ = _gpu_gradient(c, obs, 4, precision=sg.MIXED)
    assert np.all(np.isfinite(g0[2])) and J0 < 10  # the physical solution, not the growing mode
    assert J1 == pytest.approx(J0, rel=1e-6)
    for a, b in zip(g1, g0):
        assert _rel(a, b) <= 1e-5, _rel(a, b)
