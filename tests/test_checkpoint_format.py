"""The restart-file layout helper against the reference's byte layout
(src/CheckPoint.C:251-370), on hand-built bytes."""
import struct

import numpy as np

from tests import checkpoint_format as CF


def _level(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(3 * (nx + 4) * (ny + 4) * (nz + 4))


def test_bytes_match_the_reference_layout(tmp_path):
    nx, ny, nz = 2, 1, 1
    um, u = _level(nx, ny, nz, 1), _level(nx, ny, nz, 2)
    p = tmp_path / "restart.cycle=07.sw4checkpoint"
    CF.write(p, 0.125, 7, [(nx, ny, nz, um, u)])
    # header: precision, grids, time, cycle, {1, nx, 1, ny, 1, nz}
    want = struct.pack("<iidi", 8, 1, 0.125, 7) + struct.pack("<6i", 1, nx, 1, ny, 1, nz)

    def point(lev, i, j, k):  # the library's layout: component-major over the ghosted box
        ni, nij, npts = nx + 4, (nx + 4) * (ny + 4), (nx + 4) * (ny + 4) * (nz + 4)
        p = (i + 1) + (j + 1) * ni + (k + 1) * nij
        return [lev[c * npts + p] for c in range(3)]
    for lev in (um, u):  # Um block, then U; component fastest, then i, j, k over 1..n
        for k in range(1, nz + 1):
            for j in range(1, ny + 1):
                for i in range(1, nx + 1):
                    want += struct.pack("<3d", *point(lev, i, j, k))
    got = p.read_bytes()
    assert len(got) == CF.header_bytes(1) + 2 * 3 * nx * ny * nz * 8
    assert got == want


def test_round_trip_two_grids(tmp_path):
    grids = [(5, 4, 3, _level(5, 4, 3, 3), _level(5, 4, 3, 4)), (5, 4, 6, _level(5, 4, 6, 5), _level(5, 4, 6, 6))]
    p = tmp_path / "two.sw4checkpoint"
    CF.write(p, 1.5, 40, grids)
    r = CF.read(p)
    assert (r["prec"], r["time"], r["cycle"]) == (8, 1.5, 40)
    assert r["sizes"] == [[1, 5, 1, 4, 1, 3], [1, 5, 1, 4, 1, 6]]
    for (nx, ny, nz, um, u), (bum, bu) in zip(grids, r["blocks"]):
        assert np.array_equal(bum, CF.interior_block(um, nx, ny, nz))
        assert np.array_equal(bu, CF.interior_block(u, nx, ny, nz))
