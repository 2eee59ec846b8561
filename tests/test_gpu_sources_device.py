"""Source discretisation on the device (sw4g_ew_set_source_discretization; the host
loop of Source::set_grid_point_sources4, src/Source.C:1074-1530) against the host
path: the same grid-point sources bit for bit (grouped by grid point, in the host's
order within a point) and the same fields after a run, for a batch of point forces
and moment tensors that reaches the free surface (five-point weights, SBP
normalisation), the side clamps and overlapping stencils; and the device list
against the oracle's own discretisation (oracle/sw4_oracle_src.c), summed per grid
point, to 1e-14 of the largest amplitude (1e-12 for stencils clamped next to a side,
where the double evaluation of the published polynomials loses about two digits)."""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from tests.gpu_util import dev, host, oracle_discretize, smooth_fields, smooth_material

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()


NX, NY, NZ, H = 34, 30, 28, 0.05


def _sources(seed=9, n=24):
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        x, y = rng.uniform(0.0, (NX - 1) * H), rng.uniform(0.0, (NY - 1) * H)
        z = rng.uniform(0.0, 6 * H) if q % 3 == 0 else rng.uniform(0.0, (NZ - 1) * H)
        kind = int(rng.integers(0, 4))
        if q % 2:
            out.append(sg.source_desc(x, y, z, moment=tuple(rng.standard_normal(6)), freq=6.0 + q,
                                      t0=0.01 * q, kind=kind))
        else:
            out.append(sg.source_desc(x, y, z, force=tuple(rng.standard_normal(3)), freq=5.0 + q,
                                      t0=0.02 * q, kind=kind))
    # two sources one point apart: overlapping stencils
    out.append(sg.source_desc(0.5 * NX * H, 0.5 * NY * H, 0.5 * NZ * H, force=(1.0, 2.0, 3.0), freq=7.0))
    out.append(sg.source_desc(0.5 * NX * H + H, 0.5 * NY * H, 0.5 * NZ * H, moment=(1, 0, 0, 1, 0, 1),
                              freq=7.0))
    return out


def _ew(on_device, srcs):
    g = sg.grid_desc(NX, NY, NZ, H, bc=(2, 2, 2, 2, 0, 2), sg_gp=6)
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in smooth_material(NX, NY, NZ, seed=2)])
    if on_device:
        ew.set_source_discretization(True)
    for s in srcs:
        ew.add_source(s)
    return ew


def _grouped(ijk, amp):
    """The host list in the forcing's order: stable by grid point (k, j, i)."""
    ijk = ijk.reshape(-1, 3)
    order = np.lexsort((ijk[:, 0], ijk[:, 1], ijk[:, 2]))  # stable: k, then j, then i
    return ijk[order], amp.reshape(-1, 3)[order]


def test_device_sources_match_host_bit_for_bit():
    srcs = _sources()
    a, b = _ew(False, srcs), _ew(True, srcs)
    ha, aa = a.grid_point_sources()
    hb, ab = b.grid_point_sources()
    ga, gaa = _grouped(ha, aa)
    assert len(ga) == len(hb.reshape(-1, 3)) > 0
    assert np.array_equal(ga, hb.reshape(-1, 3))
    assert np.array_equal(gaa, ab.reshape(-1, 3))
    assert a.num_grid_point_sources() == b.num_grid_point_sources()
    # the same run
    dt = 0.3 * H / 2.0
    u, um = smooth_fields(NX, NY, NZ, seed=4)
    out = []
    for ew in (a, b):
        ew.set_time_step(dt, 0.0)
        ew.set_fields(dev(u), dev(um))
        ew.step(9, sg.MODE_FUSED)
        r = dev(np.zeros_like(u))
        ew.get_fields(r, None)
        out.append(host(r))
        ew.close()
    assert np.array_equal(out[0], out[1])


def _per_point(ijk, amp):
    d = {}
    for q in range(len(ijk) // 3):
        key = tuple(int(v) for v in ijk[3 * q:3 * q + 3])
        d[key] = d.get(key, np.zeros(3)) + amp[3 * q:3 * q + 3]
    return d


def _clamped(s):
    cells = [int(np.floor(s.x / H + 1)), int(np.floor(s.y / H + 1)), int(np.floor(s.z / H + 1))]
    return any(c <= 2 or c >= n - 2 for c, n in zip(cells, (NX, NY, NZ)))


def _device_vs_oracle(srcs):
    ew = _ew(True, srcs)
    g = ew.grid
    got = _per_point(*[a.reshape(-1) for a in ew.grid_point_sources()])
    ew.close()
    want = {}
    for s in srcs:
        for key, v in _per_point(*oracle_discretize(g, s)).items():
            want[key] = want.get(key, np.zeros(3)) + v
    scale = max(np.abs(v).max() for v in want.values())
    err = max(np.abs(got.get(k, np.zeros(3)) - want.get(k, np.zeros(3))).max()
              for k in set(got) | set(want))
    big = lambda d: {k for k, v in d.items() if np.abs(v).max() > 1e-12 * scale}
    return err / scale, big(got) == big(want)


def test_device_sources_match_the_oracle():
    srcs = _sources()
    err, same = _device_vs_oracle(srcs)
    assert err <= (1e-12 if any(_clamped(s) for s in srcs) else 1e-14), err
    assert same
    # the sources whose stencils are not clamped next to a side meet the tight bound
    err, same = _device_vs_oracle([s for s in srcs if not _clamped(s)])
    assert err <= 1e-14, err
    assert same


def test_switching_back_to_the_host_rebuilds_its_list():
    srcs = _sources(seed=3, n=8)
    a = _ew(False, srcs)
    b = _ew(True, srcs)
    b.set_source_discretization(False)
    ha, aa = a.grid_point_sources()
    hb, ab = b.grid_point_sources()
    assert np.array_equal(ha, hb) and np.array_equal(aa, ab)
    a.close()
    b.close()


def test_device_path_refusals():
    ew = _ew(False, [])
    ew.add_grid_point_sources([3, 4, 5], [1.0, 0.0, 0.0], [5.0], [0.0], [sg.GAUSSIAN])
    with pytest.raises(sg.Sw4gError):  # raw grid-point sources stay on the host path
        ew.set_source_discretization(True)
    ew.close()
    ew = _ew(True, [])
    with pytest.raises(sg.Sw4gError):
        ew.add_grid_point_sources([3, 4, 5], [1.0, 0.0, 0.0], [5.0], [0.0], [sg.GAUSSIAN])
    ew.close()
