#!/usr/bin/env python
"""Writes the receiver-file fixtures of tests/test_usgs_format.py from the
reference's own stored outputs (USGS text files written by
TimeSeries::write_usgs_format, src/TimeSeries.C:924) and the decks that made them.

Each fixture keeps a file's header and either all its record rows (the 64-row
topography files) or a 48-row window around the largest value; usgs_meta.json
records the total row count, the window's first row and, from the deck, the grid
spacing, extent, run time and the receiver's requested location.  The LOH.2 deck's
3200 point sources (its finite fault) go into loh2_h100_sources.npz.

    python tests/golden/make_usgs_fixtures.py [REFERENCE_ROOT]
"""
import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# (fixture name, stored output, deck) under the reference's pytest/reference
FILES = [
    ("topo_sta01", "topo/curvilinear-output/sta01.txt", "topo/curvilinear.in"),
    ("topo_sta02", "topo/curvilinear-output/sta02.txt", "topo/curvilinear.in"),
    ("topo_sta03", "topo/curvilinear-output/sta03.txt", "topo/curvilinear.in"),
    ("many_blocks_sta01", "topo/many-blocks-out/sta01.txt", "topo/many-blocks.in"),
    ("loh1_h50_sta10", "loh1/LOH1-h50/sta10.txt", "loh1/LOH.1-h50.in"),
    ("loh1_h100_sta10", "loh1/LOH1-h100/sta10.txt", "loh1/LOH.1-h100.in"),
    ("loh2_h50_sta10", "loh2/LOH2-h50/sta10.txt", "loh2/LOH.2-h50.in"),
    ("loh2_h100_sta10", "loh2/LOH2-h100/sta10.txt", "loh2/LOH.2-h100.in"),
]
WINDOW = 48


def _tokens(line):
    return dict(t.split("=", 1) for t in line.split()[1:] if "=" in t)


def deck_params(text, station):
    out = {}
    for line in text.splitlines():
        line = line.strip()
        if line.startswith("grid "):
            g = _tokens(line)
            out.update(h=float(g["h"]), x_extent=float(g["x"]), y_extent=float(g["y"]),
                       z_extent=float(g["z"]))
        elif line.startswith("time "):
            out["t"] = float(_tokens(line)["t"])
        elif line.startswith("rec "):
            r = _tokens(line)
            if r.get("file") == station:
                out.update(x=float(r["x"]), y=float(r["y"]),
                           z=float(r.get("z", r.get("depth", "0"))))
    return out


def main(root):
    base = Path(root) / "pytest" / "reference"
    meta = {}
    for name, out, deck in FILES:
        lines = (base / out).read_text().splitlines(keepends=True)
        head = [l for l in lines if l.startswith("#")]
        data = lines[len(head):]
        station = re.search(r"# Station: (\S+)", "".join(head)).group(1)
        if len(data) <= 2 * WINDOW:
            start, keep = 0, data
        else:
            peak = max(range(len(data)), key=lambda i: max(abs(float(v)) for v in data[i].split()[1:]))
            start = max(0, min(len(data) - WINDOW, peak - WINDOW // 2))
            keep = data[start:start + WINDOW]
        (HERE / f"usgs_{name}.txt").write_text("".join(head + keep))
        p = deck_params((base / deck).read_text(), station)
        p.update(rows=len(data), start=start, source=f"pytest/reference/{out}",
                 deck=f"pytest/reference/{deck}")
        meta[name] = p
    (HERE / "usgs_meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    sac_fixtures(Path(root) / "tests")
    source_list(base / "loh2" / "LOH.2-h100.in", HERE / "loh2_h100_sources.npz")


def source_list(deck, out):
    """The point sources of a deck (one `source` line each) as arrays: x, y, z, t0,
    freq, m0 and the six moment components (mxx, mxy, mxz, myy, myz, mzz; a component
    the line does not name is 0).  LOH.2's finite fault is 3200 such lines."""
    import numpy as np
    comps = ("Mxx", "Mxy", "Mxz", "Myy", "Myz", "Mzz")
    rows = []
    for line in deck.read_text().splitlines():
        if not line.strip().startswith("source "):
            continue
        t = _tokens(line.strip())
        assert t.get("type") == "Gaussian", line
        rows.append([float(t["x"]), float(t["y"]), float(t["z"]), float(t["t0"]), float(t["freq"]),
                     float(t.get("m0", "1"))] + [float(t.get(c, "0")) for c in comps])
    a = np.array(rows)
    np.savez_compressed(out, x=a[:, 0], y=a[:, 1], z=a[:, 2], t0=a[:, 3], freq=a[:, 4], m0=a[:, 5],
                        moment=a[:, 6:])


# SAC traces stored beside the USGS file of the same run under the reference's
# tests/ (binary, written by TimeSeries::write_sac_format, src/TimeSeries.C:826):
# the traces are kept whole, the run's record values (the USGS file's columns) as
# compressed FP64, and the deck's grid, time, receiver and first source.  The stored
# headers name the event either as the source (EVLA, EVLO, EVDP, O) or as zeros
# (the reference source zeroes it before writing, src/TimeSeries.C:430); "event"
# says which.
SAC = [("loh1_h100_sta10", "loh1/loh1-h100-sta10", "loh1/LOH.1-h100.in"),
       ("loh2_h100_sta10", "loh2/loh2-h100-sta10", "loh2/LOH.2-h100.in")]


def sac_fixtures(tests):
    import numpy as np
    meta = {}
    for name, run, deck in SAC:
        text = (tests / run / "sta10.txt").read_text()
        lines = text.splitlines()
        head = [l for l in lines if l.startswith("#")]
        vals = np.array([[float(v) for v in l.split()[1:]] for l in lines[len(head):]])
        np.savez_compressed(HERE / f"sac_{name}_records.npz", records=vals)
        for c in "xyz":
            (HERE / f"sac_{name}.{c}").write_bytes((tests / run / f"sta10.{c}").read_bytes())
        d = (tests / deck).read_text()
        p = deck_params(d, "sta10")
        src = _tokens([l for l in d.splitlines() if l.strip().startswith("source ")][0])
        evla = np.frombuffer((tests / run / "sta10.x").read_bytes()[35 * 4:36 * 4], dtype="<f4")[0]
        p.update(date=[l for l in head if l.startswith("# Date:")][0], rows=len(vals),
                 source_xyz=[float(src["x"]), float(src["y"]), float(src["z"])], source_t0=float(src["t0"]),
                 event="source" if evla != 0 else "zero", run=f"tests/{run}", deck=f"tests/{deck}")
        meta[name] = p
    (HERE / "sac_meta.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        sys.path.insert(0, str(HERE.parent.parent))
        from oracle import oracle as O
        src = O.reference_src()
        if src is None:
            sys.exit("reference tree not found: pass its root or set SW4_REFERENCE_SRC")
        main(str(Path(src).parent))
