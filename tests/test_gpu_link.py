"""A C++ program linked with -lsw4g (tests/integration/sw4g_link.cpp) calls
sw4g_rhs4sg and sw4g_bcfortsg through the C ABI with no Python in between; its
results match the oracle: the operator to 1e-13 and the ghost closure to 1e-14
relative to the largest value, as the ctypes kernel tests hold them."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.fields import Grid, rel_err

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def _build(tmp):
    lib = sg.build()
    exe = tmp / "sw4g_link"
    from sw4lite_gb300 import builder
    nvcc = builder.nvcc()
    cmd = [nvcc, "-std=c++17", f"-I{ROOT / 'include'}", str(ROOT / "tests/integration/sw4g_link.cpp"),
           f"-L{lib.parent}", "-lsw4g", "-Xlinker", f"-rpath={lib.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("soa", [1, 0])
def test_linked_program_matches_the_oracle(tmp_path, soa):
    exe = _build(tmp_path)
    g = Grid(23, 19, 21, h=0.4)
    rng = np.random.default_rng(77 + soa)
    u = g.field3(rng)
    _, mu, la = g.material(rng)
    sx, sy, sz = g.stretching(rng)
    onesided = [0, 0, 0, 0, 1, 0]
    bccnd = [2, 2, 2, 2, 0, 2]
    wind, _ = O.boundary_windows(g.bounds, (g.nx, g.ny, g.nz), bccnd)
    _, _, _, sbop = O.stencil_coefficients()
    hdr = np.array([soa, g.nx, g.ny, g.nz, *onesided, *bccnd, *wind], dtype="<i4")
    body = np.concatenate([[g.h], sbop[:5], u, mu, la, sx, sy, sz]).astype("<f8")
    (tmp_path / "in.bin").write_bytes(hdr.tobytes() + body.tobytes())
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    out = np.frombuffer((tmp_path / "out.bin").read_bytes(), dtype="<f8")
    lu, ubc = out[:u.size], out[u.size:]
    ref = np.zeros_like(u)
    O.rhs4sg(soa, g.bounds, g.nz, onesided, ref, u, mu, la, g.h, sx, sy, sz)
    assert rel_err(lu, ref) <= 1e-13
    ref_bc = u.copy()
    O.bcfortsg(soa, g.bounds, wind, (g.nx, g.ny, g.nz), ref_bc, g.h, bccnd, sbop, mu, la,
               [None] * 6, sx, sy)
    assert rel_err(ubc, ref_bc) <= 1e-14
