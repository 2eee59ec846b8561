"""Domain decomposition of one Cartesian grid over processes: the host logic of the
reference's 2-D (i, j) decomposition and its halo exchange (src/EW.C:1921-1949 for the
blocks, EW::communicate_arrayCU_X/Y, src/EW_cuda.C:1699-1900, for the exchange).

One subdomain per process: each rank builds its EW object with
``EW(global_grid, subdomain=dec.ranges(rank))`` and steps it with ``step_distributed``,
which runs the three parts of a step (sw4g_ew_step_part) and, after parts 0 and 1,
exchanges the halos of the level just left: x sides, then y sides, each pair of
neighbours swapping the two interior planes next to their shared side through
torch.distributed point-to-point messages (NCCL between GPUs; the packed buffers
are device tensors, so nothing is staged through the host).  ``exchange`` holds the
pairing and ordering; it takes the pack / unpack / transport as callables, so the
same code drives the GPU objects and the CPU tests (gloo, numpy fields).

Within one process the library's own lockstep driver (sw4lite_gb300.step_group,
sw4g_ew_step_group) does the same with device-to-device copies.
"""
from __future__ import annotations


def split_1d(n: int, parts: int, c: int) -> tuple[int, int]:
    """The 1-based range of block c of n points cut into `parts` nearly equal blocks
    (the first n % parts blocks one point longer)."""
    base, extra = divmod(n, parts)
    start = c * base + min(c, extra) + 1
    return start, start + base + (1 if c < extra else 0) - 1


class Decomposition:
    """gnx x gny interior points cut into px x py blocks; rank = cx + px * cy."""

    def __init__(self, gnx: int, gny: int, px: int, py: int):
        if px < 1 or py < 1 or gnx < px or gny < py:
            raise ValueError("more blocks than points")
        self.gnx, self.gny, self.px, self.py = gnx, gny, px, py
        self.size = px * py

    def coords(self, rank: int) -> tuple[int, int]:
        return rank % self.px, rank // self.px

    def ranges(self, rank: int) -> tuple[int, int, int, int]:
        """(i0, i1, j0, j1): the rank's interior points, global and 1-based."""
        cx, cy = self.coords(rank)
        return (*split_1d(self.gnx, self.px, cx), *split_1d(self.gny, self.py, cy))

    def neighbors(self, rank: int) -> list[int]:
        """Ranks across the x-low, x-high, y-low and y-high sides, -1 at the grid's edge."""
        cx, cy = self.coords(rank)
        at = lambda x, y: x + self.px * y if 0 <= x < self.px and 0 <= y < self.py else -1
        return [at(cx - 1, cy), at(cx + 1, cy), at(cx, cy - 1), at(cx, cy + 1)]

    def all_neighbors(self) -> list[list[int]]:
        return [self.neighbors(r) for r in range(self.size)]


def exchange(neighbors, pack, unpack, transfer):
    """One halo exchange of a rank: for axis x then y, pack the two interior planes next
    to each side that has a neighbour, swap them with that neighbour, and unpack what
    arrives into the side's ghost planes.  pack(axis, side) returns a buffer;
    transfer(ops) carries out a list of ("send", buf, peer) / ("recv", buf, peer)
    operations together and returns when all are complete; unpack(axis, side, buf).
    Posting one axis's sends and receives as one batch keeps two neighbours that
    both send first from waiting on each other."""
    for axis in (0, 1):
        ops, recvs = [], []
        for side in (0, 1):
            peer = neighbors[2 * axis + side]
            if peer < 0:
                continue
            out = pack(axis, side)
            inb = out.clone() if hasattr(out, "clone") else out.copy()
            ops += [("send", out, peer), ("recv", inb, peer)]
            recvs.append((side, inb))
        if ops:
            transfer(ops)
        for side, inb in recvs:
            unpack(axis, side, inb)


def torch_transfer(group=None):
    """transfer() for exchange over torch.distributed (NCCL or gloo): one batch of
    point-to-point operations, then a wait on each."""
    import torch.distributed as dist

    def run(ops):
        p2p = [dist.P2POp(dist.isend if kind == "send" else dist.irecv, buf, peer, group)
               for kind, buf, peer in ops]
        for req in dist.batch_isend_irecv(p2p):
            req.wait()
    return run


def step_distributed(ew, neighbors, nsteps, group=None):
    """nsteps steps of this rank's subdomain object with torch.distributed halo
    exchanges (NCCL for device buffers)."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device())
    bufs = {(a, s): torch.empty(ew.halo_bytes(a), dtype=torch.uint8, device=dev)
            for a in (0, 1) for s in (0, 1)}

    def pack(axis, side):
        ew.halo_pack(axis, side, bufs[(axis, side)])
        return bufs[(axis, side)]

    transfer = torch_transfer(group)
    for _ in range(nsteps):
        for part in range(3):
            ew.step_part(part)
            if part < 2:
                exchange(neighbors, pack, ew.halo_unpack, transfer)
