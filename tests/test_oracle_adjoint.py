"""The oracle's discrete adjoint (oracle/sw4_oracle_adj.c) on CPU.

No reference output exists for a material gradient (sw4lite has source gradients
only), so the adjoint is checked by its defining identities:
  * dot products: <L x, y> = <x, L^T y> and <SG x, R y> = <x, SG^T R y> on the
    interior, to 1e-13 relative;
  * the coefficient gradient of v . L(w): L is linear in (mu, lambda), so
    sum_p mu_p G_mu[p] + la_p G_la[p] = v . L(w) (Euler), and each entry equals
    v . L(w; indicator) at sampled points, to 1e-12;
  * the whole gradient against central finite differences of the misfit along a
    smooth random direction in (rho, mu, lambda), to 1e-6 relative (the bar the
    adjoint is held to on the GPU).
With free-surface z sides (one-sided SBP rows, ghost plane from the traction
condition) the same identities: L^T = D L D^-1 (D = H W, H the SBP norm weights)
by dot products to 1e-13, the coefficient gradient including the one-sided rows by
Euler's identity and single-entry perturbations, and the gradient against finite
differences with receivers on the free surface.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.adjoint_util import AdjointCase, misfit, oracle_forward, oracle_gradient, smooth_random
from tests.gpu_util import OracleProblem

pytest.importorskip("scipy")


def _bounds(c):
    return (-1, c.nx + 2, -1, c.ny + 2, -1, c.nz + 2)


def _interior_mask(c):
    m = np.zeros((c.nz + 4, c.ny + 4, c.nx + 4), dtype=bool)
    m[2:-2, 2:-2, 2:-2] = True
    return np.tile(m.reshape(-1), 3)


def _rand_interior(c, seed):
    x = np.random.default_rng(seed).standard_normal(3 * c.npts)
    x[~_interior_mask(c)] = 0
    return x


def _profiles(c):
    P = OracleProblem(c.grid, *c.mat, c.dt)
    return [p[0] for p in P.prof], [p[1] for p in P.prof], [p[2] for p in P.prof]


def test_lt_dot_product():
    c = AdjointCase()
    dc, st, co = _profiles(c)
    x, y = _rand_interior(c, 1), _rand_interior(c, 2)
    Lx = np.zeros_like(x)
    acof = O.stencil_coefficients()
    O.rhs4sg(1, _bounds(c), c.nz, (0,) * 6, Lx, x, c.mat[1], c.mat[2], c.h, *st)
    Lx[~_interior_mask(c)] = 0
    lhs = float(Lx @ y)
    rhs = float(x @ O.apply_lt(_bounds(c), c.nz, y, c.mat[1], c.mat[2], c.h, *st))
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)
    assert np.max(np.abs(np.array(st[0]) - 1)) > 0.1  # stretched layers are present


def test_sg_adjoint_dot_product():
    c = AdjointCase()
    dc, st, co = _profiles(c)
    rho = c.mat[0]
    x, y = _rand_interior(c, 3), _rand_interior(c, 4)
    up = np.zeros_like(x)
    # sw4o_addsgd4: up -= beta/rho SG(u - um)
    O.addsgd(4, 1, _bounds(c), up, x, np.zeros_like(x), rho, dc, st, co, 1.0)
    lhs = -float(up @ y)                 # <R SG x, y>
    rhs = float(x @ O.sg_adjoint(_bounds(c), y, rho, dc, st, co))  # <x, SG^T R y>
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)


def test_coef_gradient_identities():
    c = AdjointCase(shape=(14, 13, 15))
    _, st, _ = _profiles(c)
    v = _rand_interior(c, 5)
    w = _rand_interior(c, 6)
    mu, la = c.mat[1], c.mat[2]
    n = c.npts
    gm, gl = np.zeros(n), np.zeros(n)
    O.coef_gradient(_bounds(c), v, w, c.h, st, gm, gl)

    def vLw(m, l):
        out = np.zeros_like(w)
        O.rhs4sg(1, _bounds(c), c.nz, (0,) * 6, out, w, m, l, c.h, *st)
        out[~_interior_mask(c)] = 0
        return float(v @ out)

    full = vLw(mu, la)
    assert abs(float(mu @ gm + la @ gl) - full) <= 1e-12 * abs(full)
    rng = np.random.default_rng(7)
    for p in rng.integers(0, n, size=12):
        e = np.zeros(n)
        e[p] = 1.0
        assert gm[p] == pytest.approx(vLw(e, np.zeros(n)), rel=1e-11, abs=1e-12 * abs(full))
        assert gl[p] == pytest.approx(vLw(np.zeros(n), e), rel=1e-11, abs=1e-12 * abs(full))


def test_sg_rho_gradient_identity():
    c = AdjointCase(shape=(14, 13, 15))
    dc, st, co = _profiles(c)
    rho = c.mat[0]
    a1, d = _rand_interior(c, 8), _rand_interior(c, 9)
    g = np.zeros(c.npts)
    O.sg_rho_gradient(_bounds(c), a1, d, rho, dc, st, co, 0.02, g)
    up = np.zeros_like(d)
    O.addsgd(4, 1, _bounds(c), up, d, np.zeros_like(d), rho, dc, st, co, 0.02)
    # -beta (R a1).SG(d) is linear in rho through E = rho dc at fixed R
    assert float(rho @ g) == pytest.approx(float(a1 @ up), rel=1e-12)


@pytest.mark.parametrize("which", ["rho", "mu", "la", "all"])
def test_oracle_gradient_matches_finite_differences(which):
    c = AdjointCase()
    # observed data: the same shot in a slightly different medium
    obs_case = AdjointCase(seed=11)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J, gr, gm, gl = oracle_gradient(c, obs)
    shape = (c.nz + 4, c.ny + 4, c.nx + 4)
    # a smooth direction of order the material itself (values in about [-0.6, 1.5])
    dirs = [smooth_random(shape, 40 + q, corr=3.0, amp=0.3).reshape(-1) - 1.0 for q in range(3)]
    keep = {"rho": (0,), "mu": (1,), "la": (2,), "all": (0, 1, 2)}[which]
    dm = [dirs[q] * c.mat[q] if q in keep else np.zeros(c.npts) for q in range(3)]
    pred = float(gr @ dm[0] + gm @ dm[1] + gl @ dm[2])
    eps = 1e-5  # central difference: truncation ~eps^2, rounding ~1e-16/eps
    Jp = misfit(c, oracle_forward(c, [c.mat[q] + eps * dm[q] for q in range(3)])[0], obs)
    Jm = misfit(c, oracle_forward(c, [c.mat[q] - eps * dm[q] for q in range(3)])[0], obs)
    fd = (Jp - Jm) / (2 * eps)
    assert abs(pred) > 0
    assert abs(fd - pred) <= 1e-6 * abs(pred), (fd, pred)


# ---- free-surface z sides ----

def _fs_case(bc, shape=(14, 13, 24)):
    # the z stretching is 1 on the ten planes next to a free-surface side (no layer there)
    return AdjointCase(shape=shape, bc=bc)


def _lfs(c, x, mu, la, st):
    """L x with the free-surface ghost planes solved from x (interior of x only)."""
    bccnd = np.array([1, 1, 1, 1, 0 if c.onesided[4] else 1, 0 if c.onesided[5] else 1], dtype=np.int32)
    wind, _ = O.boundary_windows(_bounds(c), (c.nx, c.ny, c.nz), bccnd)
    _, _, _, sbop = O.stencil_coefficients()
    u = np.where(_interior_mask(c), x, 0.0)
    O.bcfortsg(1, _bounds(c), wind, (c.nx, c.ny, c.nz), u, c.h, bccnd, sbop, mu, la, [None] * 6, *st[:2])
    out = np.zeros_like(u)
    O.rhs4sg(1, _bounds(c), c.nz, c.onesided, out, u, mu, la, c.h, *st)
    out[~_interior_mask(c)] = 0
    return out, u


@pytest.mark.parametrize("bc", [(2, 2, 2, 2, 0, 2), (2, 2, 2, 2, 2, 0), (2, 2, 2, 2, 0, 0)])
def test_lt_fs_dot_product(bc):
    c = _fs_case(bc)
    _, st, _ = _profiles(c)
    x, y = _rand_interior(c, 21), _rand_interior(c, 22)
    lhs = float(_lfs(c, x, c.mat[1], c.mat[2], st)[0] @ y)
    rhs = float(x @ O.apply_lt_fs(_bounds(c), (c.nx, c.ny, c.nz), c.onesided, y, c.mat[1], c.mat[2], c.h,
                                  *st))
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)


@pytest.mark.parametrize("bc", [(2, 2, 2, 2, 0, 2), (2, 2, 2, 2, 2, 0)])
def test_coef_gradient_fs_identities(bc):
    c = _fs_case(bc)
    _, st, _ = _profiles(c)
    v, w = _rand_interior(c, 23), _rand_interior(c, 24)
    mu, la = c.mat[1], c.mat[2]
    n = c.npts
    full, wg = _lfs(c, w, mu, la, st)
    full = float(v @ full)
    gm, gl = np.zeros(n), np.zeros(n)
    O.coef_gradient_fs(_bounds(c), c.nz, c.onesided, v, wg, c.h, st, gm, gl)
    # v . L(w) is linear in (mu, lambda), the ghost plane included
    assert abs(float(mu @ gm + la @ gl) - full) <= 1e-12 * abs(full)
    # single entries, by linearity, on the planes next to the free surface and elsewhere
    nk, nj, ni = c.nz + 4, c.ny + 4, c.nx + 4
    side_k = [1, 2, 3, 4, 5, 6, 7, 8] if c.onesided[4] else [c.nz - q for q in range(8)]
    pts = [int(np.ravel_multi_index((k + 1, 6, 5), (nk, nj, ni))) for k in side_k]
    pts += np.random.default_rng(25).integers(0, n, size=8).tolist()
    for p in pts:
        for which in (0, 1):
            m2, l2 = mu.copy(), la.copy()
            (m2 if which == 0 else l2)[p] += 1.0
            d = float(v @ _lfs(c, w, m2, l2, st)[0]) - full
            g = (gm if which == 0 else gl)[p]
            assert abs(d - g) <= 1e-12 * abs(full), (p, which, d, g)


@pytest.mark.parametrize("which,bc,rec_k", [("mu", (2, 2, 2, 2, 0, 2), 1), ("la", (2, 2, 2, 2, 0, 2), 1),
                                            ("all", (2, 2, 2, 2, 0, 2), 1), ("all", (2, 2, 2, 2, 2, 0), 24)])
def test_oracle_gradient_fs_matches_finite_differences(which, bc, rec_k):
    c = AdjointCase(shape=(16, 15, 24), bc=bc, rec_k=rec_k)
    obs_case = AdjointCase(shape=(16, 15, 24), bc=bc, rec_k=rec_k, seed=11)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J, gr, gm, gl = oracle_gradient(c, obs)
    shape = (c.nz + 4, c.ny + 4, c.nx + 4)
    dirs = [smooth_random(shape, 50 + q, corr=3.0, amp=0.3).reshape(-1) - 1.0 for q in range(3)]
    keep = {"mu": (1,), "la": (2,), "all": (0, 1, 2)}[which]
    dm = [dirs[q] * c.mat[q] if q in keep else np.zeros(c.npts) for q in range(3)]
    pred = float(gr @ dm[0] + gm @ dm[1] + gl @ dm[2])
    eps = 1e-5
    Jp = misfit(c, oracle_forward(c, [c.mat[q] + eps * dm[q] for q in range(3)])[0], obs)
    Jm = misfit(c, oracle_forward(c, [c.mat[q] - eps * dm[q] for q in range(3)])[0], obs)
    fd = (Jp - Jm) / (2 * eps)
    assert abs(pred) > 0
    assert abs(fd - pred) <= 1e-6 * abs(pred), (fd, pred)


# ---- sixth-order damping ----
# The small cases' 5-point supergrid layers with sixth-order damping let a mode grow
# without bound after a few tens of steps (the reference formulation does the same);
# the runs below stop at 12 steps, while the solution is still the physical one.
SG6 = dict(sg_order=6, damping=0.005, nsteps=12)

def test_sg6_adjoint_dot_product():
    c = AdjointCase(**SG6)
    dc, st, co = _profiles(c)
    rho = c.mat[0]
    x, y = _rand_interior(c, 31), _rand_interior(c, 32)
    up = np.zeros_like(x)
    # sw4o_addsgd6: up += beta/(2 rho) (...) = -beta R SG6(u - um), on the points three
    # away from the array edges
    O.addsgd(6, 1, _bounds(c), up, x, np.zeros_like(x), rho, dc, st, co, 1.0)
    lhs = -float(up @ y)                                          # <R SG6 x, y>
    rhs = float(x @ O.sg6_adjoint(_bounds(c), y, rho, dc, st, co))  # <x, SG6^T R y>
    assert abs(lhs - rhs) <= 1e-13 * abs(lhs)
    assert np.max(np.abs(np.array(dc[0]))) > 0  # damping layers are present


def test_sg6_rho_gradient_identity():
    c = AdjointCase(shape=(14, 13, 15), **SG6)
    dc, st, co = _profiles(c)
    rho = c.mat[0]
    a1, d = _rand_interior(c, 33), _rand_interior(c, 34)
    g = np.zeros(c.npts)
    O.sg6_rho_gradient(_bounds(c), a1, d, rho, dc, st, co, 0.005, g)
    up = np.zeros_like(d)
    O.addsgd(6, 1, _bounds(c), up, d, np.zeros_like(d), rho, dc, st, co, 0.005)
    # -beta (R a1).SG6(d) is linear in rho through E = rho dc at fixed R
    assert float(rho @ g) == pytest.approx(float(a1 @ up), rel=1e-12)


@pytest.mark.parametrize("which", ["rho", "all"])
def test_oracle_gradient_sg6_matches_finite_differences(which):
    kw = dict(SG6)
    c = AdjointCase(**kw)
    obs_case = AdjointCase(seed=11, **kw)
    obs = obs_case.records(oracle_forward(obs_case)[0][1:])
    J, gr, gm, gl = oracle_gradient(c, obs)
    shape = (c.nz + 4, c.ny + 4, c.nx + 4)
    dirs = [smooth_random(shape, 90 + q, corr=3.0, amp=0.3).reshape(-1) - 1.0 for q in range(3)]
    keep = {"rho": (0,), "all": (0, 1, 2)}[which]
    dm = [dirs[q] * c.mat[q] if q in keep else np.zeros(c.npts) for q in range(3)]
    pred = float(gr @ dm[0] + gm @ dm[1] + gl @ dm[2])
    eps = 1e-5
    Jp = misfit(c, oracle_forward(c, [c.mat[q] + eps * dm[q] for q in range(3)])[0], obs)
    Jm = misfit(c, oracle_forward(c, [c.mat[q] - eps * dm[q] for q in range(3)])[0], obs)
    fd = (Jp - Jm) / (2 * eps)
    assert abs(pred) > 0
    assert abs(fd - pred) <= 1e-6 * abs(pred), (fd, pred)
