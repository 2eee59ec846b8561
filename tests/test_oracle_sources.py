"""The oracle's own source discretisation (oracle/sw4_oracle_src.c), and the library's
host discretisation (sw4g_discretize_source, the set-up path of every EW object)
against it.

The oracle restates the Cartesian branch of Source::set_grid_point_sources4
(src/Source.C:1074-1930) with the weight polynomials evaluated in monomial (Horner)
form, not the grouped form the reference and the library use.  Checks:
  * the weight tables satisfy the defining moment conditions of the published
    weights: sum_k w_k (x_k - a)^m = delta_{m0} (delta) and -delta_{m1} (delta'),
    m = 0..4, for the 6-point weights and the five-point free-surface variants;
  * for point forces and moment tensors at every depth k = 1..5 under a free
    surface, next to the supergrid sides and the bottom, on grids with and without
    one-sided top and bottom closures: the summed grid-point amplitude at every grid
    point agrees to 1e-14 of the largest amplitude (1e-12 where the stencil centre is
    clamped next to a side, see _clamped) and the points carrying more than 1e-12 of
    it are the same.  (Where a weight is zero in exact arithmetic, the two
    evaluation orders can give 0 or ~1e-16, so the reference's rule "emit where the
    weight is nonzero" can emit a different set of negligible entries.)
"""
from collections import defaultdict

import numpy as np
import pytest

import sw4lite_gb300 as sg
from oracle import oracle as O
from tests.gpu_util import discretize, oracle_discretize


@pytest.fixture(scope="module", autouse=True)
def _libs():
    O.lib()
    sg.build()


@pytest.mark.parametrize("which,first_moment", [(0, 0), (1, -1), (2, 0), (3, -1)])
def test_weight_tables_satisfy_their_moment_conditions(which, first_moment):
    for a in np.linspace(-1.0, 1.0, 41):
        w = O.source_weights(which, a)
        x = np.arange(-2, 4) - a
        moments = [float(np.sum(w * x ** m)) for m in range(5)]
        want = [1.0, 0, 0, 0, 0] if which in (0, 2) else [0, first_moment, 0, 0, 0]
        assert np.allclose(moments, want, atol=1e-12), (which, a, moments)
        if which in (2, 3):
            assert w[5] == 0  # the five-point variants leave the sixth point out


def _dense(ijk, amp):
    d = defaultdict(lambda: np.zeros(3))
    for q in range(len(ijk) // 3):
        d[tuple(ijk[3 * q:3 * q + 3])] += amp[3 * q:3 * q + 3]
    return d


def _compare(g, src):
    a = _dense(*discretize(g, src))
    b = _dense(*oracle_discretize(g, src))
    scale = max(np.abs(v).max() for v in b.values())
    keys = set(a) | set(b)
    err = max(np.abs(a.get(k, np.zeros(3)) - b.get(k, np.zeros(3))).max() for k in keys)
    big_a = {k for k, v in a.items() if np.abs(v).max() > 1e-12 * scale}
    big_b = {k for k, v in b.items() if np.abs(v).max() > 1e-12 * scale}
    return err / scale, big_a, big_b


NX, NY, NZ, H = 30, 28, 26, 0.1
GRIDS = {
    "free top": (2, 2, 2, 2, 0, 2),
    "free top and bottom": (2, 2, 1, 1, 0, 0),
    "supergrid everywhere": (2,) * 6,
}


def _sources():
    rng = np.random.default_rng(2024)
    out = []
    # depths k = 1..5 below the surface, on and between grid planes
    for k in range(1, 6):
        for frac in (0.0, 0.35, -0.4):
            z = max(0.0, (k - 1 + frac) * H)
            out.append(((11.3 * H, 9.6 * H, z), "depth"))
    # next to the x and y sides (clamped stencil centres) and the bottom
    out += [((0.4 * H, 14.2 * H, 9.1 * H), "x side"), ((28.7 * H, 3.5 * H, 12.4 * H), "x side"),
            ((16.6 * H, 0.9 * H, 6.2 * H), "y side"), ((15.2 * H, 13.1 * H, 24.6 * H), "bottom"),
            ((12.0 * H, 12.0 * H, 12.0 * H), "on a grid point")]
    for _ in range(6):
        out.append((tuple(rng.uniform(0.5, [28.5 * H, 26.5 * H, 24.5 * H])), "random"))
    return out


@pytest.mark.parametrize("bc", list(GRIDS.values()), ids=list(GRIDS))
@pytest.mark.parametrize("kind", ["force", "moment"])
def test_library_discretisation_matches_the_oracle(bc, kind):
    g = sg.grid_desc(NX, NY, NZ, H, bc=bc, sg_gp=6)
    for (x, y, z), where in _sources():
        if kind == "force":
            src = sg.source_desc(x, y, z, force=(1.0, -0.4, 0.7))
        else:
            src = sg.source_desc(x, y, z, moment=(1.0, 0.3, -0.2, 0.8, 0.1, -0.6))
        err, big_a, big_b = _compare(g, src)
        assert err <= (1e-12 if _clamped(x, y, z) else 1e-14), (where, (x, y, z), err)
        assert big_a == big_b, (where, (x, y, z))


def _clamped(x, y, z):
    """Whether the stencil centre is moved off the source's cell next to a side: the
    weights are then evaluated at |a| up to 2, where the grouped double evaluation of
    the published polynomials (reference and library alike) loses about two digits
    and the oracle's exact-coefficient evaluation does not."""
    cells = [int(np.floor(x / H + 1)), int(np.floor(y / H + 1)), int(np.floor(z / H + 1))]
    return any(c <= 2 or c >= n - 2 for c, n in zip(cells, (NX, NY, NZ)))


def test_near_surface_source_uses_the_five_point_stencil():
    # a source 1.7 h below a free surface: the stencil centre is clamped to plane 3
    # (ci = -0.3), the five-point weights keep it off the ghost plane k = 0, and the
    # z weights of planes 1..4 are divided by the SBP quadrature weights
    ijk, amp = O.discretize_source(NX, NY, NZ, H, 0.0, True, False, 11.3 * H, 9.6 * H, 1.7 * H,
                                   force=(0.0, 0.0, 1.0))
    ks = set(int(k) for k in ijk[2::3])
    assert min(ks) == 1 and max(ks) == 5  # plane 6 has weight zero and is not emitted
    wk = O.source_weights(2, -0.3)
    norm = [17 / 48, 59 / 48, 43 / 48, 49 / 48]
    col = defaultdict(float)
    for q in range(len(ijk) // 3):
        col[int(ijk[3 * q + 2])] += amp[3 * q + 2]
    # the (i, j) weights sum to 1, so each plane's sum is its z weight over h^3
    for t in range(5):
        k = 1 + t
        want = wk[t] / norm[k - 1] if k <= 4 else wk[t]
        assert abs(col[k] * H ** 3 - want) <= 1e-13, (k, col[k] * H ** 3, want)
