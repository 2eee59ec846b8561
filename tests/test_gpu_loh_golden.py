"""The reference's LOH.1 and LOH.2 runs at h = 100 reproduced on the GPU: the decks
pytest/reference/loh1/LOH.1-h100.in and loh2/LOH.2-h100.in against the receiver traces
the reference stored for station 10 (pytest/reference/loh{1,2}/LOH{1,2}-h100/sta10.txt:
48-row windows around the peak at 17 digits, kept in tests/golden/usgs_loh{1,2}_h100_sta10.txt)
and against the whole traces of the same station from the reference's
tests/loh{1,2}/loh{1,2}-h100-sta10/sta10.txt (all 537 rows at 17 digits, kept in
tests/golden/sac_loh{1,2}_h100_sta10_records.npz).  tests/golden/make_usgs_fixtures.py
writes these fixtures and LOH.2's source list (tests/golden/loh2_h100_sources.npz).

The decks: a 30 x 30 x 17 km domain at h = 100 (301 x 301 x 171 points), a free
surface on top and a 30-point supergrid on the other sides (damping coefficient 0.02,
the default), material blocks applied in order as MaterialBlock::set_material_properties
does (src/MaterialBlock.C:108-200: a point is inside a block when each coordinate lies
within its bounds +- 1e-5; later blocks overwrite; ghost points take the nearest
interior value, src/EW.C:5444-5560), mu = rho vs vs and lambda = rho vp vp - 2 mu
(src/EW.C:5469-5490), run to t = 9 s (536 steps at CFL 1.3), station 10 at (21, 23, 0)
km recording displacement.
* LOH.1 (LOH.1-h100.in:21-43): a half-space (vp 6000, vs 3464, rho 2700), the layer
  z <= 1000 (vp 4000, vs 2000, rho 2600), at z = 1000 the interface values (vp 4630.76,
  vs 2437.56, rho 2650); a moment source mxy = 1e18 at (15, 15, 2) km, Gaussian time
  function (freq 16.6667, t0 0.36).
* LOH.2: the same half-space and layer without the interface block; a finite fault of
  3200 moment sources (mxy = 3.23981e14 each, Gaussian, freq 16.6667, rupture times
  t0 0.89-1.6 s) half-way between grid points in y and z, so every source spreads over
  a 6 x 6 x 6 stencil and the stencils overlap.
These are the C2 workload's set-up (layer over half-space, free surface, supergrid,
moment sources, surface receivers) at a size whose output the reference kept.

Tolerances, relative to the trace's largest value: FP64 1e-12 (observed on GB300:
LOH.1 1.4e-14 on the window and 7.7e-14 over the whole trace, LOH.2 3.0e-14 and
2.1e-13, i.e. the reference's runs to their last bits through 536 steps), FP32-mixed
3e-6 (observed 7.4e-7 and 2.5e-7).
"""
import json
from pathlib import Path

import numpy as np
import pytest

import sw4lite_gb300 as sg

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
H, LX, LY, LZ, T_END = 100.0, 30000.0, 30000.0, 17000.0, 9.0
# (vp, vs, rho, zmin, zmax) in each deck's order
HALFSPACE, LAYER = (6000.0, 3464.0, 2700.0, -1e38, 1e38), (4000.0, 2000.0, 2600.0, -1e38, 1000.0)
BLOCKS = {"loh1": [HALFSPACE, LAYER, (4630.76, 2437.56, 2650.0, 999.0, 1001.0)],
          "loh2": [HALFSPACE, LAYER]}
STATION = (21000.0, 23000.0, 0.0)


def sources(deck):
    if deck == "loh1":
        return [sg.source_desc(15000.0, 15000.0, 2000.0, moment=(0.0, 1e18, 0.0, 0.0, 0.0, 0.0),
                               freq=16.6667, t0=0.36, kind=sg.GAUSSIAN)]
    d = np.load(GOLDEN / "loh2_h100_sources.npz")
    return [sg.source_desc(x, y, z, moment=tuple(m0 * m), freq=f, t0=t0, kind=sg.GAUSSIAN)
            for x, y, z, t0, f, m0, m in zip(d["x"], d["y"], d["z"], d["t0"], d["freq"], d["m0"], d["moment"])]


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()


def material_profile(blocks, nz, h):
    """(rho, mu, lambda) of the planes k = -1 .. nz + 2 (the medium depends on z only,
    so the ghost points' nearest interior values are the plane's own)."""
    z = (np.arange(-1, nz + 3) - 1) * h
    vp, vs, rho = (np.full(z.shape, -1.0) for _ in range(3))
    for bvp, bvs, brho, z1, z2 in blocks:
        inside = (z1 - 1e-5 <= z) & (z <= z2 + 1e-5)
        vp[inside], vs[inside], rho[inside] = bvp, bvs, brho
    assert np.all(rho > 0)
    mu = rho * vs * vs
    return rho, mu, rho * vp * vp - 2 * mu


def _run(deck, precision):
    import torch

    nx, ny, nz = int(round(LX / H)) + 1, int(round(LY / H)) + 1, int(round(LZ / H)) + 1
    g = sg.grid_desc(nx, ny, nz, H, bc=(2, 2, 2, 2, 0, 2), sg_gp=30, sg_damping=0.02,
                     precision=precision)
    ew = sg.EW(g)
    prof = material_profile(BLOCKS[deck], nz, H)
    shape = (nz + 4, ny + 4, nx + 4)
    mat = [torch.from_numpy(p).to("cuda")[:, None, None].expand(shape).reshape(-1).contiguous()
           for p in prof]
    ew.set_material(*mat)
    for src in sources(deck):
        ew.add_source(src)
    dt, nsteps = ew.compute_time_step(1.3, T_END)
    ijk, grid = ew.nearest_grid_point(*STATION)
    ew.set_time_step(dt, 0.0)
    ew.set_receivers([ijk], [sg.REC_DISPLACEMENT], nsteps + 1)
    ew.step(nsteps, sg.MODE_FUSED)
    rec = ew.records()
    ew.close()
    return dt, nsteps, ijk, grid, rec


def _usgs_window(deck):
    meta = json.loads((GOLDEN / "usgs_meta.json").read_text())[f"{deck}_h100_sta10"]
    rows = [l for l in (GOLDEN / f"usgs_{deck}_h100_sta10.txt").read_text().splitlines()
            if not l.startswith("#")]
    a = np.array([[float(v) for v in l.split()] for l in rows])
    return meta, a


@pytest.mark.parametrize("deck", ["loh1", "loh2"])
@pytest.mark.parametrize("precision,tol_usgs,tol_sac", [(sg.FP64, 1e-12, 1e-12), (sg.MIXED, 3e-6, 3e-6)])
def test_loh_h100_reproduces_reference_trace(deck, precision, tol_usgs, tol_sac):
    dt, nsteps, ijk, grid, rec = _run(deck, precision)
    meta, win = _usgs_window(deck)
    assert nsteps + 1 == meta["rows"] == 537
    assert (ijk, grid) == ((211, 231, 1), 0)
    start = meta["start"]
    assert np.allclose(np.arange(start, start + len(win)) * dt, win[:, 0], rtol=0, atol=5e-6)
    got = rec[start:start + len(win)]
    scale = np.abs(win[:, 1:]).max()
    err = np.abs(got - win[:, 1:]).max() / scale
    assert err <= tol_usgs, f"USGS window: max error {err:.3e} of its largest value"
    whole = np.load(GOLDEN / f"sac_{deck}_h100_sta10_records.npz")["records"]
    assert whole.shape == rec.shape
    scale = np.abs(whole).max()
    err = np.abs(rec - whole).max() / scale
    assert err <= tol_sac, f"whole trace: max error {err:.3e} of its largest value"
