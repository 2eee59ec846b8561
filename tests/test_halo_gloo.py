"""Host logic of the decomposed time loop over processes (sw4lite_gb300.halo), on CPU
with the gloo backend: world sizes 2 (2 x 1 blocks), 3 (1 x 3) and 4 (2 x 2).

Each rank holds its block of a seeded global 3-component field with two ghost
planes per side; the ghost planes at sides shared with a neighbour start as NaN.
One exchange (halo.exchange over torch.distributed point-to-point batches, the
transport step_distributed uses with NCCL on GPUs; numpy pack / unpack that follow
the library's plane and buffer conventions, tests/halo_numpy.py) must leave every
rank's array equal to the global field's values over its whole block, corners
included (x is exchanged before y, so y carries the x ghost columns).  Also: the
block ranges tile the grid and the neighbour tables are symmetric."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GNX, GNY, NK = 13, 11, 6


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _global(seed=5):
    return np.random.default_rng(seed).standard_normal((3, NK, GNY + 4, GNX + 4))


def _block(G, rng_):
    i0, i1, j0, j1 = rng_
    # global interior point i sits at array offset i + 1 (two ghosts, 1-based)
    return G[:, :, j0 - 1:j1 + 4, i0 - 1:i1 + 4].copy()


def _rank_main(rank, world, px, py, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from sw4lite_gb300 import halo
    from tests import halo_numpy as hn
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dec = halo.Decomposition(GNX, GNY, px, py)
    nb = dec.neighbors(rank)
    G = _global()
    want = _block(G, dec.ranges(rank))
    f = want.copy()
    ni, nj = f.shape[3], f.shape[2]
    for axis in (0, 1):
        for side in (0, 1):
            if nb[2 * axis + side] >= 0:
                p = hn.planes(ni if axis == 0 else nj, side, False)
                if axis == 0:
                    f[:, :, :, p] = np.nan
                else:
                    f[:, :, p, :] = np.nan

    def pack(axis, side):
        return torch.from_numpy(hn.pack(f, axis, side))

    def unpack(axis, side, buf):
        hn.unpack(f, axis, side, buf.numpy())

    halo.exchange(nb, pack, unpack, halo.torch_transfer())
    ok = bool(np.array_equal(f, want))
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as fh:
        fh.write(f"{int(ok)} {int(np.isnan(f).sum())}\n")
    dist.destroy_process_group()


@pytest.mark.parametrize("px,py", [(2, 1), (1, 3), (2, 2)])
def test_exchange_fills_every_ghost_plane(tmp_path, px, py):
    world = px * py
    mp.spawn(_rank_main, args=(world, px, py, _free_port(), str(tmp_path)), nprocs=world, join=True)
    for r in range(world):
        ok, nans = open(tmp_path / f"rank{r}.txt").read().split()
        assert ok == "1" and nans == "0", (r, ok, nans)


@pytest.mark.parametrize("gnx,gny,px,py", [(13, 11, 2, 2), (40, 9, 3, 1), (17, 30, 4, 5)])
def test_blocks_tile_the_grid_and_neighbours_agree(gnx, gny, px, py):
    sys.path.insert(0, ROOT)
    from sw4lite_gb300 import halo
    dec = halo.Decomposition(gnx, gny, px, py)
    cover = np.zeros((gny + 1, gnx + 1), dtype=int)
    for r in range(dec.size):
        i0, i1, j0, j1 = dec.ranges(r)
        cover[j0:j1 + 1, i0:i1 + 1] += 1
        nb = dec.neighbors(r)
        for q, t in enumerate(nb):
            if t >= 0:
                assert dec.neighbors(t)[q ^ 1] == r
                # neighbours share the full side
                ti0, ti1, tj0, tj1 = dec.ranges(t)
                if q < 2:
                    assert (tj0, tj1) == (j0, j1) and (ti1 + 1 == i0 if q == 0 else ti0 == i1 + 1)
                else:
                    assert (ti0, ti1) == (i0, i1) and (tj1 + 1 == j0 if q == 2 else tj0 == j1 + 1)
    assert np.all(cover[1:, 1:] == 1)
