"""The reference's own topography run reproduced on the GPU: the deck
pytest/reference/topo/curvilinear.in against the receiver traces the reference stored
for it (pytest/reference/topo/curvilinear-output/sta01-03.txt, all 64 rows kept in
tests/golden/usgs_topo_sta0N.txt by tests/golden/make_usgs_fixtures.py).

The deck (curvilinear.in:6-24): a 1.28 x 1.28 x 5.0 domain at h = 0.02, a Gaussian
hill of amplitude 0.1 at (0.6, 0.4) with widths 0.15 x 0.10 over a curvilinear grid
down to z = 2.0 (mapping order 6), a homogeneous medium (vp 2, vs 1, rho 1.5), a
30-point supergrid on the sides and the bottom, a free surface on the topography, a
moment source mxy = 0.87 at depth 0.2 below the surface with a Gaussian time function
(freq 16.6667, t0 0.36), run to t = 0.5 (63 steps of 0.5/63), and three receivers
recording displacement: two on the surface (depth 0) and one at depth 0.3, all on
the curvilinear grid.  This pins the two-grid step as a whole (curvilinear operator,
metric, free surface, interface, supergrid, time step, source discretisation on the
curvilinear grid and the receivers' placement) against the reference's own output.

Tolerances, relative to each trace's largest magnitude: FP64 1e-13 (observed
2.5e-15 to 6.4e-15 on GB300: the stored files print 17 digits, so the run agrees
with the reference's to its last bits, the differences coming from summation order
and FMA contraction); FP32-mixed 3e-6 (observed 2.5e-7 to 6.9e-7, the mixed form's
own error against FP64).
"""
import json
from pathlib import Path

import numpy as np
import pytest

import sw4lite_gb300 as sg

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
H, LX, LY, LZ, ZMAX, T_END = 0.02, 1.28, 1.28, 5.0, 2.0, 0.5
HILL = dict(amp=0.1, xc=0.6, yc=0.4, lx=0.15, ly=0.10, order=6)
VP, VS, RHO = 2.0, 1.0, 1.5
SRC = dict(x=0.52, y=0.48, depth=0.2, mxy=0.87, freq=16.6667, t0=0.36)
STATIONS = [("topo_sta01", 0.7, 0.6, 0.0), ("topo_sta02", 0.5, 0.3, 0.0), ("topo_sta03", 0.6, 0.5, 0.3)]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()


def _stored(name):
    """The stored trace: rows x (ux, uy, uz) and the times."""
    rows = [l for l in (GOLDEN / f"usgs_{name}.txt").read_text().splitlines() if not l.startswith("#")]
    a = np.array([[float(v) for v in l.split()] for l in rows])
    return a[:, 0], a[:, 1:]


def _run(precision):
    import torch

    nx, ny = int(round(LX / H)) + 1, int(round(LY / H)) + 1
    ncart = int(round((LZ - ZMAX) / H)) + 1
    g = sg.grid_desc(nx, ny, ncart, H, bc=(2, 2, 2, 2, sg.INTERFACE, 2), zmin=ZMAX, sg_gp=30,
                     sg_damping=0.02, precision=precision)
    ew = sg.EW(g, topo=sg.topo_desc(HILL["amp"], HILL["xc"], HILL["yc"], HILL["lx"], HILL["ly"],
                                    order=HILL["order"]))
    mu, la = RHO * VS * VS, RHO * VP * VP - 2 * RHO * VS * VS
    for grid in (0, 1):
        n = ew.grid_dims(grid)[3]
        mat = [torch.full((n,), v, dtype=torch.float64, device="cuda") for v in (RHO, mu, la)]
        if grid == 0:
            ew.set_material(*mat)
        else:
            ew.set_material_grid(1, *mat)
    zsrc = ew.topography_z(SRC["x"], SRC["y"]) + SRC["depth"]
    ew.add_source(sg.source_desc(SRC["x"], SRC["y"], zsrc, moment=(0.0, SRC["mxy"], 0.0, 0.0, 0.0, 0.0),
                                 freq=SRC["freq"], t0=SRC["t0"], kind=sg.GAUSSIAN))
    dt, nsteps = ew.compute_time_step(1.3, T_END)
    ijk, grids = [], []
    for _, x, y, depth in STATIONS:
        p, gi = ew.nearest_grid_point(x, y, ew.topography_z(x, y) + depth)
        ijk.append(p)
        grids.append(gi)
    ew.set_time_step(dt, 0.0)
    ew.set_receivers(ijk, [sg.REC_DISPLACEMENT] * len(STATIONS), nsteps + 1, grids=grids)
    ew.step(nsteps, sg.MODE_FUSED)
    rec = ew.records()
    ew.close()
    return dt, nsteps, ijk, grids, rec


@pytest.mark.parametrize("precision,tol", [(sg.FP64, 1e-13), (sg.MIXED, 3e-6)])
def test_topography_deck_reproduces_reference_traces(precision, tol):
    dt, nsteps, ijk, grids, rec = _run(precision)
    times, _ = _stored(STATIONS[0][0])
    assert nsteps == len(times) - 1 == 63
    assert np.allclose(np.arange(nsteps + 1) * dt, times, rtol=0, atol=5e-7)  # printed to 7 digits
    assert grids == [1, 1, 1]
    meta = json.loads((GOLDEN / "usgs_meta.json").read_text())
    for s, (name, *_) in enumerate(STATIONS):
        assert meta[name]["rows"] == nsteps + 1 and meta[name]["start"] == 0
        _, want = _stored(name)
        got = rec[:, 3 * s:3 * s + 3]
        scale = np.abs(want).max()
        err = np.abs(got - want).max() / scale
        assert err <= tol, f"{name} at {ijk[s]}: max error {err:.3e} of the trace's largest value"
