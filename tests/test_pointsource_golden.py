"""Point-source tests against the analytic whole-space solution.

Golden vector: the reference's own point-source run
(pytest/reference/pointsource/pointsource.in; its output
pytest/reference/pointsource/pointsource-h0p04/PointSourceErr.txt:1 =
"0.6 0.569416364119 0.0245360919934 3.74390307494", i.e. t, Linf, L2 of the
error and max of the exact solution).  The deck: an 8 x 8 x 4 box with h = 0.04
(201 x 201 x 101 points), rho = 1, cp = 1.6, cs = 0.8, free surface on top and
30-point supergrid layers on the other sides, an isotropic moment source
Mxx = Myy = Mzz = 1 at (4, 4, 1.34) with a C6SmoothBump of frequency 1, run to
t = 0.6 at CFL 1.3.  The reference's pytest driver accepts 1e-5 relative
(pytest/test_sw4lite.py:214).  The file prints 12 significant digits, and the
oracle's time loop (CPU) and the GPU time loop both reproduce all three numbers
to that precision, so the bar here is 1e-9.

The second workload is a 101^3 unit cube with a Gaussian point force (1, 1, 1)
at the centre, frequency 20, t0 = 0.15, rho = mu = lambda = 1, supergrid on all
six sides (20 points, damping 0.02), CFL 1.3, t = 0.6.  It has no stored
reference output: the GPU errors must equal the oracle's (1e-8 relative).
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.gpu_util import OracleProblem, dev, host

GOLDEN = (0.6, 0.569416364119, 0.0245360919934, 3.74390307494)


def _time_step(cfl, h, rho, mu, la, tmax):
    """dt from the CFL number, adjusted to land on tmax (src/EW.C:5041-5146)."""
    dt = cfl * h / np.sqrt(np.max((4 * mu + la) / rho))
    n = max(1, int(tmax / dt + 0.5))
    return tmax / n, n


def _deck(name):
    if name == "pointsource":
        n = (201, 201, 101)
        h, rho, cp, cs, gp, bc = 0.04, 1.0, 1.6, 0.8, 30, (2, 2, 2, 2, 0, 2)
        src = dict(xyz=(4.0, 4.0, 1.34), moment=(1.0, 0.0, 0.0, 1.0, 0.0, 1.0), force=None,
                   kind=sg.C6SMOOTHBUMP, freq=1.0, t0=0.0)
    else:
        n = (101, 101, 101)
        h, rho, cp, cs, gp, bc = 0.01, 1.0, np.sqrt(3.0), 1.0, 20, (2,) * 6
        src = dict(xyz=(0.5, 0.5, 0.5), moment=None, force=(1.0, 1.0, 1.0), kind=sg.GAUSSIAN,
                   freq=20.0, t0=0.15)
    nx, ny, nz = n
    g = sg.grid_desc(nx, ny, nz, h, bc=bc, sg_gp=gp, sg_damping=0.02)
    npts = (nx + 4) * (ny + 4) * (nz + 4)
    mu_v, la_v = rho * cs * cs, rho * cp * cp - 2 * rho * cs * cs
    mat = (np.full(npts, rho), np.full(npts, mu_v), np.full(npts, la_v))
    dt, nsteps = _time_step(1.3, h, *mat, 0.6)
    s = sg.source_desc(*src["xyz"], moment=src["moment"], force=src["force"], freq=src["freq"],
                       t0=src["t0"], kind=src["kind"])
    return dict(g=g, mat=mat, dt=dt, nsteps=nsteps, src=src, sdesc=s, rho=rho, cp=cp, cs=cs,
                gp=gp, bc=bc, h=h, n=n)


def _errors(d, u, t):
    """(Linf, L2, max exact) as the reference's normOfDifference: interior points
    outside the supergrid layers and outside a 4h ball around the source
    (src/EW.C:4537-4600)."""
    nx, ny, nz = d["n"]
    bounds = (-1, nx + 2, -1, ny + 2, -1, nz + 2)
    src = d["src"]
    kw = dict(kind=src["kind"], freq=src["freq"], t0=src["t0"])
    if src["moment"] is not None:
        kw["moment"] = src["moment"]
    else:
        kw["force"] = src["force"]
    uex = O.exact_point_source(bounds, d["h"], 0.0, d["rho"], d["cp"], d["cs"], *src["xyz"], t, **kw)
    gp, bc = d["gp"], d["bc"]
    region = (gp + 1 if bc[0] == 2 else 1, nx - gp if bc[1] == 2 else nx,
              gp + 1 if bc[2] == 2 else 1, ny - gp if bc[3] == 2 else ny,
              gp + 1 if bc[4] == 2 else 1, nz - gp if bc[5] == 2 else nz)
    return O.solerr3(bounds, d["h"], 0.0, uex, u, *src["xyz"], 4 * d["h"], region)


def _oracle_run(d):
    z = np.zeros(3 * d["mat"][0].size)
    u, _ = OracleProblem(d["g"], *d["mat"], d["dt"], [d["sdesc"]]).run(z, z, 0.0, d["nsteps"])
    return u


def _gpu_run(d, mode, precision=sg.FP64):
    g = d["g"]
    g.precision = precision
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in d["mat"]])
    ew.add_source(d["sdesc"])
    dt, n = ew.compute_time_step(1.3, 0.6)
    assert n == d["nsteps"] and abs(dt - d["dt"]) <= 1e-15 * d["dt"]
    ew.step(n, mode)
    u = dev(np.zeros(3 * d["mat"][0].size))
    ew.get_fields(u, None)
    t = ew.time
    ew.close()
    g.precision = sg.FP64
    return host(u), t


def test_oracle_reproduces_reference_point_source_errors():
    d = _deck("pointsource")
    assert d["nsteps"] * d["dt"] == pytest.approx(GOLDEN[0], rel=1e-14)
    u = _oracle_run(d)
    li, l2, xli = _errors(d, u, d["nsteps"] * d["dt"])
    assert li == pytest.approx(GOLDEN[1], rel=1e-9)
    assert l2 == pytest.approx(GOLDEN[2], rel=1e-9)
    assert xli == pytest.approx(GOLDEN[3], rel=1e-9)


def test_exact_solution_solves_the_discrete_problem_to_truncation_order():
    """Sanity of the analytic field itself (independent of the golden vector): at a
    smooth instant, away from the source, its numerical time second derivative
    matches L(u)/rho of the oracle's operator to a few percent of |u_tt|."""
    d = _deck("pointsource")
    nx, ny, nz = d["n"]
    bounds = (-1, nx + 2, -1, ny + 2, -1, nz + 2)
    src = d["src"]
    t, dt = 0.45, 1e-3
    u = [O.exact_point_source(bounds, d["h"], 0.0, d["rho"], d["cp"], d["cs"], *src["xyz"], tt,
                              moment=src["moment"], kind=src["kind"], freq=src["freq"])
         for tt in (t - dt, t, t + dt)]
    utt = (u[2] - 2 * u[1] + u[0]) / dt ** 2
    lu = np.zeros_like(u[1])
    one = np.ones(nx + 4)
    O.rhs4sg(1, bounds, nz, (0, 0, 0, 0, 0, 0), lu, u[1], d["mat"][1], d["mat"][2], d["h"], one,
             np.ones(ny + 4), np.ones(nz + 4))
    shape = (3, nz + 4, ny + 4, nx + 4)
    a, b = lu.reshape(shape) / d["rho"], utt.reshape(shape)
    # a shell around the source between 8h and the wave front, away from every boundary
    k, j, i = np.meshgrid(np.arange(nz + 4), np.arange(ny + 4), np.arange(nx + 4), indexing="ij")
    x, y, z = (i - 2) * d["h"], (j - 2) * d["h"], (k - 2) * d["h"]
    r = np.sqrt((x - 4.0) ** 2 + (y - 4.0) ** 2 + (z - 1.34) ** 2)
    sel = (r > 0.32) & (r < 0.6) & (z > 0.3)
    err = np.abs(a[:, sel] - b[:, sel]).max() / np.abs(b[:, sel]).max()
    assert err < 0.05, err


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [sg.MODE_FUSED, sg.MODE_PHASES])
def test_gpu_reproduces_reference_point_source_errors(mode):
    sg.build()
    d = _deck("pointsource")
    u, t = _gpu_run(d, mode)
    assert t == pytest.approx(GOLDEN[0], rel=1e-14)
    li, l2, xli = _errors(d, u, t)
    assert li == pytest.approx(GOLDEN[1], rel=1e-9)
    assert l2 == pytest.approx(GOLDEN[2], rel=1e-9)
    assert xli == pytest.approx(GOLDEN[3], rel=1e-9)


@pytest.mark.gpu
def test_gpu_point_force_cube_errors_match_oracle():
    sg.build()
    d = _deck("cube")
    u_gpu, t = _gpu_run(d, sg.MODE_FUSED)
    u_ref = _oracle_run(d)
    e_gpu = _errors(d, u_gpu, t)
    e_ref = _errors(d, u_ref, d["nsteps"] * d["dt"])
    assert np.allclose(e_gpu, e_ref, rtol=1e-8, atol=0), (e_gpu, e_ref)
    # the discrete solution is close to the analytic one: Linf below 5% of max |u_exact|
    assert e_gpu[0] < 0.05 * e_gpu[2], e_gpu


@pytest.mark.gpu
def test_gpu_mixed_form_meets_reference_point_source_bar():
    """The FP32-mixed form on the golden deck, held to the reference driver's own
    1e-5 relative bar on the error norms."""
    sg.build()
    d = _deck("pointsource")
    u, t = _gpu_run(d, sg.MODE_FUSED, precision=sg.MIXED)
    li, l2, xli = _errors(d, u, t)
    assert li == pytest.approx(GOLDEN[1], rel=1e-5)
    assert l2 == pytest.approx(GOLDEN[2], rel=1e-5)
    assert xli == pytest.approx(GOLDEN[3], rel=1e-5)
