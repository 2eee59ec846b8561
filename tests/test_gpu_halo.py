"""Domain decomposition on the GPU: halo pack / unpack kernels and subdomain runs.

* sw4g_halo_pack / sw4g_halo_unpack move exactly the planes of tests/halo_numpy.py, in
  its buffer order, for both component layouts, both axes and both sides (bit for bit).
* A grid cut into 2 x 1, 1 x 2, 2 x 2 and 3 x 2 subdomains, stepped in lockstep by
  sw4g_ew_step_group with halo exchanges after the predictor and the corrector, gives
  bit for bit the undivided run's levels on every subdomain's interior points: the
  same supergrid profiles (taken from the global grid), the same grid-point sources
  (a moment tensor and a force, one of them across a subdomain boundary), the free
  surface on top.  FP64 and the FP32-mixed form (tensor-copy stage kernels on both
  sides: every array's i extent is a multiple of 4).
* step_part misuse and stepping a subdomain with sw4g_ew_step are refused.
The subdomains share one GPU here; across GPUs the same driver copies halos into the
receiving GPU's memory (cudaMemcpyPeerAsync), which this single-GPU run cannot reach.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from tests import halo_numpy as hn
from tests.fields import Grid
from tests.gpu_util import dev, host, smooth_fields, smooth_material, stream

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()


@pytest.mark.parametrize("soa", [1, 0])
def test_pack_unpack_match_the_planes(soa):
    g = Grid(21, 17, 9)
    rng = np.random.default_rng(3 + soa)
    u = g.field3(rng)
    shape = (g.nk, g.nj, g.ni)
    L = sg.lib()
    for axis in (0, 1):
        n = L.sw4g_halo_len(*g.bounds, axis)
        for side in (0, 1):
            du = dev(u)
            buf = dev(np.zeros(n))
            sg.check(L.sw4g_halo_pack(soa, *g.bounds, axis, side, du.data_ptr(), buf.data_ptr(),
                                      stream()), "pack")
            want = hn.pack(hn.as_cpk(u, shape, soa), axis, side)
            assert np.array_equal(host(buf), want)
            # unpack a marked buffer into the ghost planes
            mark = np.arange(n, dtype=np.float64) + 0.5
            sg.check(L.sw4g_halo_unpack(soa, *g.bounds, axis, side, dev(mark).data_ptr(),
                                        du.data_ptr(), stream()), "unpack")
            ref = u.copy()
            hn.unpack(hn.as_cpk(ref, shape, soa), axis, side, mark)
            assert np.array_equal(host(du), ref)


def _problem(nx, ny, nz, precision):
    h = 0.05
    g = sg.grid_desc(nx, ny, nz, h, bc=(2, 2, 2, 2, 0, 2), sg_gp=6, precision=precision)
    rho, mu, la = smooth_material(nx, ny, nz, seed=21)
    u, um = smooth_fields(nx, ny, nz, seed=22)
    srcs = [sg.source_desc(0.5 * (nx - 1) * h + 0.3 * h, 0.45 * (ny - 1) * h, 0.4 * nz * h,
                           moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6), freq=8.0, kind=sg.C6SMOOTHBUMP),
            sg.source_desc(0.3 * (nx - 1) * h, 0.7 * (ny - 1) * h, 2.5 * h, force=(0.3, -1.0, 0.6),
                           freq=7.0, t0=0.02)]
    dt = 0.3 * h / float(np.sqrt(np.max((4 * mu + la) / rho)))
    return g, (rho, mu, la), (u, um), srcs, dt


def _local(a, nx, ny, nz, i0, i1, j0, j1, ncomp):
    f = a.reshape(ncomp, nz + 4, ny + 4, nx + 4)
    return np.ascontiguousarray(f[:, :, j0 - 1:j1 + 4, i0 - 1:i1 + 4]).ravel()


def _decomposed(px, py, nx, ny, nz, precision, nsteps):
    from sw4lite_gb300 import halo
    g, mat, fields, srcs, dt = _problem(nx, ny, nz, precision)
    # the undivided run
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in mat])
    for s in srcs:
        ew.add_source(s)
    ew.set_time_step(dt, 0.0)
    ew.set_fields(*[dev(a) for a in fields])
    ew.step(nsteps, sg.MODE_FUSED)
    whole = dev(np.zeros_like(fields[0]))
    ew.get_fields(whole, None)
    whole = host(whole).reshape(3, nz + 4, ny + 4, nx + 4)
    ew.close()
    # the subdomains
    dec = halo.Decomposition(nx, ny, px, py)
    subs = []
    for r in range(dec.size):
        i0, i1, j0, j1 = dec.ranges(r)
        e = sg.EW(g, subdomain=(i0, i1, j0, j1))
        e.set_material(*[dev(_local(a, nx, ny, nz, i0, i1, j0, j1, 1)) for a in mat])
        for s in srcs:
            e.add_source(s)
        e.set_time_step(dt, 0.0)
        e.set_fields(*[dev(_local(a, nx, ny, nz, i0, i1, j0, j1, 3)) for a in fields])
        subs.append(e)
    sg.step_group(subs, dec.all_neighbors(), nsteps)
    worst = 0
    for r, e in enumerate(subs):
        i0, i1, j0, j1 = dec.ranges(r)
        lu = dev(np.zeros(3 * e.npts))
        e.get_fields(lu, None)
        lu = host(lu).reshape(3, nz + 4, j1 - j0 + 5, i1 - i0 + 5)
        mine = lu[:, :, 2:-2, 2:-2]  # the subdomain's interior columns, all planes
        ref = whole[:, :, j0 + 1:j1 + 2, i0 + 1:i1 + 2]
        if not np.array_equal(mine, ref):
            worst = max(worst, float(np.abs(mine - ref).max() / np.abs(ref).max()))
        e.close()
    return worst


@pytest.mark.parametrize("px,py", [(2, 1), (1, 2), (2, 2), (3, 2)])
def test_subdomains_reproduce_the_undivided_run_fp64(px, py):
    assert _decomposed(px, py, 40, 36, 26, sg.FP64, 8) == 0


def test_subdomains_reproduce_the_undivided_run_mixed():
    # i extents 76 (whole) and 40 (each half): the tensor-copy kernels on both sides
    assert _decomposed(2, 2, 72, 40, 28, sg.MIXED, 6) == 0


def test_step_part_order_and_refusals():
    g, mat, fields, _, dt = _problem(40, 36, 26, sg.FP64)
    e = sg.EW(g, subdomain=(1, 20, 1, 36))
    e.set_material(*[dev(_local(a, 40, 36, 26, 1, 20, 1, 36, 1)) for a in mat])
    e.set_time_step(dt, 0.0)
    with pytest.raises(sg.Sw4gError):
        e.step_part(1)  # parts run in order
    with pytest.raises(sg.Sw4gError):
        e.step(1)       # a subdomain steps with halo exchanges
    with pytest.raises(sg.Sw4gError):
        e.halo_pack(0, 1, dev(np.zeros(8)))  # no level to exchange before part 0
    e.step_part(0)
    assert e.halo_bytes(0) == 8 * 3 * 2 * (36 + 4) * (26 + 4)
    e.close()
    with pytest.raises(sg.Sw4gError):  # a periodic axis cannot be cut
        sg.EW(sg.grid_desc(40, 36, 26, 0.05, bc=(3, 3, 2, 2, 0, 2)), subdomain=(1, 20, 1, 36))
