"""Truncation error of the oracle's elastic operators on manufactured smooth fields:
the fourth-order interior stencil and the second-order SBP boundary rows.

The reference makes this check with its own closed-form fields
(tests/testil/testil.C:186-200, :348-366): the operator applied to exact data against
the analytic rho * (div sigma).  Here the fields and their divergence of stress come
from tests/manufactured.py.  On n = 17, 33, 65 points per side (h halved twice), the
error in the interior rows falls with rate >= 3.6 then >= 3.85 (fourth order), and in
the six one-sided rows next to a free surface with rate >= 1.9 (the SBP closure's
second-order truncation); without the one-sided closure the rows next to the z sides
use the centred stencil on exact ghost values and fall at fourth order too.  The same
holds for the curvilinear operator on a smoothly bent grid with the numerical metric.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests import manufactured as M

SIZES = (17, 33, 65)


def _cartesian(n, onesided):
    c = M.case(n)
    lu = np.zeros_like(c["u"])
    s = np.ones(n + 4)
    O.rhs4sg(1, c["bounds"], n, [0, 0, 0, 0, onesided, onesided], lu, c["u"], c["mu"], c["la"],
             c["h"], s, s, s)
    return M.row_errors(lu, c)


def _curvilinear(n, top):
    c = M.case(n, curvilinear=True)
    met, jac = np.zeros(4 * c["z"].size), np.zeros(c["z"].size)
    assert O.metric(1, c["bounds"], c["h"], c["z"], met, jac) == 0
    lu = np.zeros_like(c["u"])
    s = np.ones(n + 4)
    O.rhs4sgcurv(1, c["bounds"], (0, 0, 0, 0, top, 0), lu, c["u"], c["mu"], c["la"], met, jac,
                 s, s)
    return M.row_errors(lu, c)


def check_rates(errs, top_sbp, bottom_sbp):
    """errs: per size (interior, top rows, bottom rows)."""
    e = np.asarray(errs)
    fourth = lambda r: r[0] >= 3.6 and r[1] >= 3.85
    assert fourth(M.rates(e[:, 0])), e
    for col, sbp in ((1, top_sbp), (2, bottom_sbp)):
        r = M.rates(e[:, col])
        assert (np.all(r >= 1.9) and np.all(r <= 2.3)) if sbp else fourth(r), (col, r, e)


def test_manufactured_divergence_matches_finite_differences():
    p = np.array([0.37, 0.81, 0.55])
    eps = 1e-4

    def sigma(q):
        xyz = [np.array(v) for v in q]
        g = [f.grad(xyz) for f in M.DISPLACEMENT]
        mu, la = M.MU.value(xyz), M.LAMBDA.value(xyz)
        d = g[0][0] + g[1][1] + g[2][2]
        return np.array([[la * d * (i == j) + mu * (g[i][j] + g[j][i]) for j in range(3)]
                         for i in range(3)])

    fd = sum((sigma(p + eps * np.eye(3)[j])[:, j] - sigma(p - eps * np.eye(3)[j])[:, j]) / (2 * eps)
             for j in range(3))
    exact = np.array([float(v) for v in M.div_stress([np.array(v) for v in p])])
    assert np.abs(fd - exact).max() <= 1e-6 * np.abs(exact).max()


@pytest.mark.parametrize("onesided", [0, 1])
def test_cartesian_operator_converges(onesided):
    check_rates([_cartesian(n, onesided) for n in SIZES], onesided, onesided)


@pytest.mark.parametrize("top", [0, 1])
def test_curvilinear_operator_converges(top):
    check_rates([_curvilinear(n, top) for n in SIZES], top, False)
