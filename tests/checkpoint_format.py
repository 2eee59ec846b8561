"""The reference's restart-file layout, restated with numpy for the tests.

src/CheckPoint.C:251-370 (write_checkpoint) and :373-470 (read_checkpoint):
  int precision (8 for double), int number of grids, double time, int cycle,
  per grid int[6] = {1, nx, 1, ny, 1, nz} (the interior's global index ranges),
  per grid the Um block then the U block: the interior points without ghost points
  (Sarray::extract_subarray, src/Sarray.C:616-633: component fastest, then i, j, k),
  doubles in the machine's byte order (little-endian here).
The header is 3 ints + 1 double + 6 ints per grid long (the reference's data offset).
A level here is the library's flat array: 3 components, each over the (nz+4, ny+4,
nx+4) box whose interior is [2:n+2] along every axis.
"""
import numpy as np


def interior_block(level, nx, ny, nz):
    """(nz, ny, nx, 3) interior of a level, component fastest."""
    a = np.asarray(level).reshape(3, nz + 4, ny + 4, nx + 4)[:, 2:nz + 2, 2:ny + 2, 2:nx + 2]
    return np.ascontiguousarray(np.moveaxis(a, 0, -1))


def header_bytes(ng):
    return 3 * 4 + 8 + ng * 6 * 4


def write(path, time, cycle, grids):
    """grids: [(nx, ny, nz, um_level, u_level), ...]."""
    with open(path, "wb") as f:
        np.array([8, len(grids)], dtype="<i4").tofile(f)
        np.array([time], dtype="<f8").tofile(f)
        np.array([cycle], dtype="<i4").tofile(f)
        for nx, ny, nz, _, _ in grids:
            np.array([1, nx, 1, ny, 1, nz], dtype="<i4").tofile(f)
        for nx, ny, nz, um, u in grids:
            interior_block(um, nx, ny, nz).astype("<f8").tofile(f)
            interior_block(u, nx, ny, nz).astype("<f8").tofile(f)


def read(path):
    """{'prec', 'time', 'cycle', 'sizes': [[6 ints]...], 'blocks': [(Um, U) (nz, ny, nx, 3)]}."""
    raw = open(path, "rb").read()
    prec, ng = np.frombuffer(raw, "<i4", 2, 0)
    time = float(np.frombuffer(raw, "<f8", 1, 8)[0])
    cycle = int(np.frombuffer(raw, "<i4", 1, 16)[0])
    sizes = np.frombuffer(raw, "<i4", 6 * ng, 20).reshape(ng, 6)
    off = header_bytes(ng)
    blocks = []
    for s in sizes:
        nx, ny, nz = int(s[1]), int(s[3]), int(s[5])
        n = 3 * nx * ny * nz
        um = np.frombuffer(raw, "<f8", n, off).reshape(nz, ny, nx, 3)
        u = np.frombuffer(raw, "<f8", n, off + 8 * n).reshape(nz, ny, nx, 3)
        off += 16 * n
        blocks.append((um, u))
    assert off == len(raw), "trailing bytes"
    return dict(prec=int(prec), time=time, cycle=cycle, sizes=sizes.tolist(), blocks=blocks)
