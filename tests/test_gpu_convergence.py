"""Truncation error of the device operators on manufactured smooth fields, through the
C ABI (sw4g_rhs4sg; sw4g_metric then sw4g_rhs4sgcurv on a smoothly bent grid): the
same rates as the oracle's (tests/test_oracle_convergence.py), fourth order in the
interior and second order in the one-sided SBP rows, and errors within 1e-9 of the
oracle's own, so the device operators approximate div sigma as the reference's do
(tests/testil/testil.C:348-366 makes the same comparison on the host)."""
import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests import manufactured as M
from tests.gpu_util import dev, host, stream
from tests.test_oracle_convergence import SIZES, _cartesian, _curvilinear, check_rates

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    O.lib()


def _os(flags):
    return np.asarray(flags, dtype=np.int32)


def _device_cartesian(n, onesided):
    c = M.case(n)
    s = dev(np.ones(n + 4))
    d = [dev(c[k]) for k in ("u", "mu", "la")]
    lu = dev(np.zeros_like(c["u"]))
    flags = _os([0, 0, 0, 0, onesided, onesided])
    sg.check(sg.lib().sw4g_rhs4sg(1, *c["bounds"], n, flags.ctypes.data_as(sg._I), lu.data_ptr(),
                                  *[a.data_ptr() for a in d], c["h"], s.data_ptr(), s.data_ptr(),
                                  s.data_ptr(), stream()), "sw4g_rhs4sg")
    return M.row_errors(host(lu), c)


def _device_curvilinear(n, top):
    c = M.case(n, curvilinear=True)
    zd = dev(c["z"])
    met, jac = dev(np.zeros(4 * c["z"].size)), dev(np.zeros(c["z"].size))
    sg.check(sg.lib().sw4g_metric(1, *c["bounds"], c["h"], zd.data_ptr(), met.data_ptr(),
                                  jac.data_ptr(), None), "sw4g_metric")
    s = dev(np.ones(n + 4))
    keep = [dev(c[k]) for k in ("u", "mu", "la")] + [met, jac, s, s]
    lu = dev(np.zeros_like(c["u"]))
    flags = _os([0, 0, 0, 0, top, 0])
    sg.check(sg.lib().sw4g_rhs4sgcurv(1, *c["bounds"], flags.ctypes.data_as(sg._I), lu.data_ptr(),
                                      *[a.data_ptr() for a in keep], None), "sw4g_rhs4sgcurv")
    return M.row_errors(host(lu), c)


@pytest.mark.parametrize("onesided", [0, 1])
def test_device_cartesian_operator_converges(onesided):
    got = [_device_cartesian(n, onesided) for n in SIZES]
    check_rates(got, onesided, onesided)
    want = [_cartesian(n, onesided) for n in SIZES]
    assert np.abs(np.asarray(got) - np.asarray(want)).max() <= 1e-9


@pytest.mark.parametrize("top", [0, 1])
def test_device_curvilinear_operator_converges(top):
    got = [_device_curvilinear(n, top) for n in SIZES]
    check_rates(got, top, False)
    want = [_curvilinear(n, top) for n in SIZES]
    assert np.abs(np.asarray(got) - np.asarray(want)).max() <= 1e-9
