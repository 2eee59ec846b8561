"""The stage kernels' launch shape (host arithmetic, no device work): the k-chunk
choice of stage_kchunk (stage_fused.cu) that the Cartesian, mixed and curvilinear
stage kernels share.  A launch of cols CTA columns x chunks runs in waves of
resident x 152 CTAs on GB300; the choice minimises waves x (planes per chunk + 2)
over the chunk counts giving at least 3.5 waves, chunks of at least 12 planes."""
import math

import pytest

import sw4lite_gb300 as sg

SMS = 152


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    sg.lib()


def _cost(cols, nk, resident, per):
    chunks = math.ceil(nk / per)
    return math.ceil(cols * chunks / (resident * SMS)) * (per + 2), cols * chunks / (resident * SMS)


def _expected(cols, nk, resident, min_planes):
    """Python restatement of the rule, for the check."""
    most = max(1, nk // max(1, min_planes))
    best, choice = None, most
    for c in range(1, most + 1):
        per = math.ceil(nk / c)
        cost, waves = _cost(cols, nk, resident, per)
        if 2 * cols * math.ceil(nk / per) < 7 * resident * SMS:
            continue
        if best is None or cost < best * 0.999:
            best, choice = cost, c
    return math.ceil(nk / choice)


@pytest.mark.parametrize("cols,nk,resident", [
    (8 * 32, 256, 2),      # C4 256^3 FP64 stage (32 x 8 CTAs, 2 per SM)
    (16 * 64, 508, 2),     # C2 512^3 FP64 stage
    (16 * 64, 508, 3),     # C2 mixed stage (3 per SM)
    (12 * 48, 72, 2),      # C3 Cartesian part
    (12 * 48, 45, 2),      # C3 curvilinear interior
    (4, 20, 1), (1, 5, 1), (3000, 7, 2)])
def test_stage_kchunk_rule(cols, nk, resident):
    per = sg.stage_kchunk(cols, nk, resident, 12)
    assert per == _expected(cols, nk, resident, 12)
    assert 1 <= per <= nk


def test_stage_kchunk_known_shapes():
    # 256^3 at 2 CTAs per SM: 7 chunks of 37 planes, 1792 CTAs = 5.9 waves
    assert sg.stage_kchunk(256, 256, 2) == 37
    # a grid with enough columns for 3.5 waves keeps one chunk
    assert sg.stage_kchunk(2000, 100, 2) == 100


def test_stage_kchunk_rejects_bad_arguments():
    for args in [(0, 10, 1, 12), (10, 0, 1, 12), (10, 10, 0, 12), (10, 10, 1, 0)]:
        with pytest.raises(sg.Sw4gError):
            sg.stage_kchunk(*args)
