"""Host logic of bench.py that needs no GPU.

* A secondary workload that fails on one GPU is reported in its place on the line, and
  the headline figures still print; with several ranks the failure propagates, so no
  rank waits at a barrier another rank has left.
* The FP64-pipe instruction counts per point that bench.py divides by the launch time
  are the ones of the current table of the committed ncu summary, so the line's
  roofline fraction can be recomputed from that summary and the line's kernel times.
"""
import os
import re

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _boom():
    raise RuntimeError("planted failure")


def test_failed_workload_is_reported_on_one_gpu():
    out = bench._guarded(1, "adjoint", _boom)
    assert out == {"failed": "adjoint: RuntimeError: planted failure"}
    assert bench._guarded(1, "adjoint", lambda x: {"ok": x}, 3) == {"ok": 3}


def test_failed_workload_propagates_with_several_ranks():
    with pytest.raises(RuntimeError):
        bench._guarded(2, "adjoint", _boom)


def test_fp64_pipe_counts_match_the_committed_summary():
    text = open(os.path.join(ROOT, "profiles", "fp64_pipe_c2_512.md")).read()
    # the first table of the summary holds the current kernels' counts
    rows = {}
    for kind, count in re.findall(r"\| `fused_stage_kernel<(\d)>`[^|]*\|[^|]*\| ([\d,]+) \|", text):
        rows.setdefault(int(kind), int(count.replace(",", "")))
    assert set(rows) == {0, 1}
    n3 = 512 ** 3
    assert bench.FP64_WARP_INST_PER_PT["pred"] == rows[0] / n3
    assert bench.FP64_WARP_INST_PER_PT["corr"] == rows[1] / n3
