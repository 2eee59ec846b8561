"""Test support for the discrete adjoint: a small supergrid problem (optionally with
free-surface z sides) with a smooth heterogeneous medium, receivers at grid points,
the oracle's forward run (every level and predicted level kept) and the oracle's
adjoint sweep.

Misfit J = 1/2 sum over steps n = 0..N and receivers r of |u^n(x_r) - d^n_r|^2
(displacement at the receiver grid points).
"""
import numpy as np

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.gpu_util import OracleProblem


def smooth_random(shape, seed, corr=4.0, amp=0.05):
    """exp(amp * g) with g a unit-variance smooth random field (Gaussian filter of
    white noise, correlation length `corr` points)."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal(shape)
    from scipy.ndimage import gaussian_filter
    g = gaussian_filter(g, corr, mode="wrap")
    g /= g.std()
    return np.exp(amp * g)


class AdjointCase:
    def __init__(self, shape=(20, 18, 22), h=0.1, gp=5, seed=3, nsteps=30, nrec=6,
                 vp=1.8, vs=1.0, rho=1.5, bc=(2,) * 6, rec_k=None, sg_order=4, damping=0.02):
        self.nx, self.ny, self.nz = shape
        nx, ny, nz = shape
        self.h = h
        self.grid = sg.grid_desc(nx, ny, nz, h, bc=bc, sg_gp=gp, sg_damping=damping, sg_order=sg_order)
        arr = (nz + 4, ny + 4, nx + 4)
        r = rho * smooth_random(arr, seed)
        cs = vs * smooth_random(arr, seed + 1)
        cp = vp * smooth_random(arr, seed + 2)
        mu = r * cs * cs
        self.mat = [np.ascontiguousarray(a.reshape(-1)) for a in (r, mu, r * cp * cp - 2 * mu)]
        self.dt = 0.35 * h / float(np.sqrt(np.max((4 * self.mat[1] + self.mat[2]) / self.mat[0])))
        self.nsteps = nsteps
        self.sources = [sg.source_desc(0.45 * (nx - 1) * h, 0.5 * (ny - 1) * h,
                                       0.55 * (nz - 1) * h, force=(0.3, -0.2, 1.0), freq=12.0,
                                       t0=0.12, kind=sg.GAUSSIAN)]
        rng = np.random.default_rng(seed + 10)
        self.rec = [(int(rng.integers(gp + 2, nx - gp)), int(rng.integers(gp + 2, ny - gp)),
                     int(rng.integers(gp + 2, nz - gp))) for _ in range(nrec)]
        if rec_k is not None:  # receivers on a plane (e.g. the free surface, k = 1)
            self.rec = [(i, j, rec_k) for i, j, _ in self.rec]
        self.onesided = (0, 0, 0, 0, int(bc[4] == 0), int(bc[5] == 0))
        self.npts = (nx + 4) * (ny + 4) * (nz + 4)

    def rec_index(self):
        nx, ny = self.nx, self.ny
        return [(i + 1) + (nx + 4) * ((j + 1) + (ny + 4) * (k + 1)) for i, j, k in self.rec]

    def records(self, levels):
        idx = self.rec_index()
        n = self.npts
        return np.array([[lv[c * n + p] for p in idx for c in range(3)] for lv in levels])


def oracle_forward(case: AdjointCase, mat=None):
    """Levels u^{-1}, u^0..u^N and predicted levels up^0..up^{N-1} (zero start)."""
    mat = case.mat if mat is None else mat
    P = OracleProblem(case.grid, *mat, case.dt, case.sources)
    n3 = 3 * case.npts
    um, u = np.zeros(n3), np.zeros(n3)
    levels, preds = [um.copy(), u.copy()], []
    lu, f, uacc = np.zeros(n3), np.zeros(n3), np.zeros(n3)
    t = 0.0
    for _ in range(case.nsteps):
        up, pred = np.zeros(n3), np.zeros(n3)
        O.step_pred(P.P, t, up, u, um, lu, f, uacc, pred)
        preds.append(pred)
        levels.append(up)
        um, u = u, up
        t += case.dt
    return levels, preds, P


def misfit(case, levels, obs):
    d = case.records(levels[1:]) - obs
    return 0.5 * float(np.sum(d * d))


def oracle_gradient(case: AdjointCase, obs):
    """(J, g_rho, g_mu, g_lambda) by the oracle's discrete adjoint."""
    levels, preds, P = oracle_forward(case)
    rho, mu, la = case.mat
    n, n3 = case.npts, 3 * case.npts
    bounds = (-1, case.nx + 2, -1, case.ny + 2, -1, case.nz + 2)
    prof = P.prof
    dc, st, co = [p[0] for p in prof], [p[1] for p in prof], [p[2] for p in prof]
    beta = case.grid.sg_damping
    dt, N = case.dt, case.nsteps
    rec = case.records(levels[1:])
    idx = case.rec_index()
    J = 0.5 * float(np.sum((rec - obs) ** 2))

    def g_of(nlev):  # dJ/du^nlev (nlev = 0..N)
        g = np.zeros(n3)
        res = (rec[nlev] - obs[nlev]).reshape(-1, 3)
        for r, p in enumerate(idx):
            for c in range(3):
                g[c * n + p] += res[r, c]
        return g

    R3 = np.tile(1.0 / rho, 3)
    gr, gm, gl = np.zeros(n), np.zeros(n), np.zeros(n)
    a2 = np.zeros(n3)
    a1 = g_of(N)
    fs = any(case.onesided)
    dims = (case.nx, case.ny, case.nz)

    def lt(y):
        if fs:
            return O.apply_lt_fs(bounds, dims, case.onesided, y, mu, la, case.h, *st)
        return O.apply_lt(bounds, case.nz, y, mu, la, case.h, *st)

    def cg(v, w):
        if fs:
            O.coef_gradient_fs(bounds, case.nz, case.onesided, v, w, case.h, st, gm, gl)
        else:
            O.coef_gradient(bounds, v, w, case.h, st, gm, gl)

    for step in range(N - 1, -1, -1):
        u, um, up, unew = levels[step + 1], levels[step], preds[step], levels[step + 2]
        s = lt(a1 * R3)
        m = a1 + dt * dt / 12 * s
        t = lt(m * R3)
        w1 = up - 2 * u + um
        cg(a1 * R3 * (dt * dt / 12), w1)
        cg(m * R3 * (dt * dt), u)
        gr -= ((m * w1 + a1 * (unew - up)).reshape(3, -1).sum(0)) / rho
        six = case.grid.sg_order == 6
        (O.sg6_rho_gradient if six else O.sg_rho_gradient)(bounds, a1, u - um, rho, dc, st, co, beta, gr)
        an = g_of(step) + 2 * m + dt * dt * t - dt * dt / 6 * s - a2 - beta * (
            O.sg6_adjoint if six else O.sg_adjoint)(bounds, a1 - a2, rho, dc, st, co)
        a2, a1 = a1, an
    return J, gr, gm, gl
