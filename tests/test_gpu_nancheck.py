"""The time loop's non-finite check (sw4g_ew_set_nan_check), the counterpart of the
reference's checkfornan option (src/EW.C:2544-2759, check_nan_dev in
src/device-routines.C:8279).

Faults are planted on the host: a NaN or an infinity written into an input level
before the step.  No device fault is involved.  Checks: a clean run with the check
on returns normally; a poisoned level makes step() raise NonFiniteError after the
first checked step, with the object's time at that step, the count of non-finite
entries of the new level, and the first offending entry in storage order, which
must be the first non-finite entry of the level the test reads back.
"""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from tests.gpu_util import dev, host, smooth_fields, smooth_material

pytestmark = pytest.mark.gpu

NX, NY, NZ, H = 36, 30, 32, 0.05


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()


def _ew(precision, poison=None, bad=np.nan):
    rho, mu, la = smooth_material(NX, NY, NZ, seed=5)
    u, um = smooth_fields(NX, NY, NZ, seed=6)
    if poison is not None:
        c, i, j, k = poison
        ni, nj = NX + 4, NY + 4
        p = (i + 1) + ni * (j + 1) + ni * nj * (k + 1)  # 1-based (i, j, k) with 2 ghosts
        u[c * u.size // 3 + p] = bad
    dt = 0.3 * H / float(np.sqrt(np.max((4 * mu + la) / rho)))
    g = sg.grid_desc(NX, NY, NZ, H, bc=(2, 2, 2, 2, 0, 2), sg_gp=6, precision=precision)
    ew = sg.EW(g)
    ew.set_material(*[dev(a) for a in (rho, mu, la)])
    ew.set_time_step(dt, 0.0)
    ew.set_fields(dev(u), dev(um))
    return ew, dt, u.size


def _first_bad(ew, n3):
    u = dev(np.zeros(n3))
    ew.get_fields(u, None)
    a = host(u)
    bad = np.flatnonzero(~np.isfinite(a))
    np_ = n3 // 3
    off = int(bad[0])
    c, p = divmod(off, np_)
    ni, nj = NX + 4, NY + 4
    return len(bad), (c, p % ni - 1, (p // ni) % nj - 1, p // (ni * nj) - 1)


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
def test_clean_run_passes(precision):
    ew, dt, _ = _ew(precision)
    ew.set_nan_check(1)
    ew.step(5, sg.MODE_FUSED)
    assert ew.nan_report()["grid"] == -1
    ew.close()


@pytest.mark.parametrize("precision", [sg.FP64, sg.MIXED])
@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_poisoned_level_is_reported_after_the_first_checked_step(precision, bad):
    ew, dt, n3 = _ew(precision, poison=(1, 17, 14, 16), bad=bad)
    ew.set_nan_check(3)
    with pytest.raises(sg.NonFiniteError) as ei:
        ew.step(10, sg.MODE_FUSED)
    r = ei.value.report
    assert r["grid"] == 0
    assert abs(r["t"] - 3 * dt) <= 1e-12 * dt  # the object stopped at the first checked step
    assert abs(ew.time - 3 * dt) <= 1e-12 * dt
    count, (c, i, j, k) = _first_bad(ew, n3)
    # the mixed form's count covers the hi and lo halves of each value
    if precision == sg.MIXED:
        assert count <= r["count"] <= 2 * count
    else:
        assert r["count"] == count
    assert (r["c"], *r["ijk"]) == (c, i, j, k)
    # the poisoned point itself is still non-finite (the one-sided free-surface rows
    # read 8 planes deep, so the poison reaches the top ghost plane within 3 steps)
    assert k >= -1 and count > 1
    ew.close()


def test_check_off_runs_through():
    ew, dt, n3 = _ew(sg.FP64, poison=(0, 10, 10, 10))
    ew.step(2, sg.MODE_FUSED)  # no check: no error, the NaNs stay in the level
    count, _ = _first_bad(ew, n3)
    assert count > 0
    ew.close()
