"""Receiver files in the USGS text format (sw4g_write_usgs) and the geographic
mapping (sw4g_geographic_coord), on the host.

Golden files: the reference's own stored receiver outputs, written by
TimeSeries::write_usgs_format (src/TimeSeries.C:924) for the decks
pytest/reference/topo/curvilinear.in, topo/many-blocks.in, loh1/LOH.1-h{50,100}.in and
loh2/LOH.2-h{50,100}.in.  tests/golden/make_usgs_fixtures.py keeps each file's header
and all its rows or a 48-row window around its peak.  Given the stored values, the
deck's receiver location and its nearest grid point (sw4g_nearest_grid_point), the
writer must reproduce header and rows byte for byte.  The stored files were made with
longitude origin +118 (their "Target location" longitudes are 118.0000-118.2594),
while the reference source's default is -118 (src/EW.C:193); the test passes +118.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

import sw4lite_gb300 as sg

GOLDEN = Path(__file__).resolve().parent / "golden"
META = json.loads((GOLDEN / "usgs_meta.json").read_text())


@pytest.fixture(scope="module", autouse=True)
def _lib():
    sg.build()
    sg.lib()


def _parse(text):
    lines = text.splitlines(keepends=True)
    head = [l for l in lines if l.startswith("#")]
    return head, lines[len(head):]


def _utc(head):
    # "# Date: UTC  MM/DD/YYYY:H:M:SS.mmm"
    d = [l for l in head if l.startswith("# Date:")][0].split("UTC")[1].strip()
    mdy, h, m, sms = d.split(":")
    mo, day, yr = (int(x) for x in mdy.split("/"))
    s, ms = sms.split(".")
    return (yr, mo, day, int(h), int(m), int(s), int(ms))


@pytest.mark.parametrize("name", sorted(META))
def test_writer_reproduces_reference_receiver_file(name, tmp_path):
    m = META[name]
    head, rows = _parse((GOLDEN / f"usgs_{name}.txt").read_text())
    station = [l for l in head if l.startswith("# Station:")][0].split(":", 1)[1].strip()
    h = m["h"]
    g = sg.grid_desc(int(round(m["x_extent"] / h)) + 1, int(round(m["y_extent"] / h)) + 1,
                     int(round(m["z_extent"] / h)) + 1, h)
    i, j, _ = sg.nearest_grid_point(g, m["x"], m["y"], m["z"])
    vals = np.zeros((m["rows"], 3))
    for r, line in enumerate(rows):
        vals[m["start"] + r] = [float(v) for v in line.split()[1:]]
    dt = m["t"] / (m["rows"] - 1)
    out = tmp_path / "rec.txt"
    rc = sg.write_usgs(out, vals, station=station, x=m["x"], y=m["y"], gp_x=(i - 1) * h,
                       gp_y=(j - 1) * h, dt=dt, utc=_utc(head), geo=sg.geo_desc(lon_origin=118.0))
    assert rc == sg.OK
    mine_head, mine_rows = _parse(out.read_text())
    assert mine_head == head
    assert len(mine_rows) == m["rows"]
    assert mine_rows[m["start"]:m["start"] + len(rows)] == rows


def _geo_np(geo, x, y):
    """numpy restatement of EW::computeGeographicCoord (src/EW.C:5794-5816)."""
    d = math.pi / 180.0
    phi = geo.az * d
    lat = geo.lat_origin + (x * math.cos(phi) - y * math.sin(phi)) / geo.meters_per_degree
    a = x * math.sin(phi) + y * math.cos(phi)
    if geo.const_meters_per_longitude:
        return geo.lon_origin + a / geo.meters_per_longitude, lat
    return geo.lon_origin + a / (geo.meters_per_degree * math.cos(lat * d)), lat


@pytest.mark.parametrize("az,const", [(0.0, 0), (33.0, 0), (-140.0, 1)])
def test_geographic_coord(az, const):
    geo = sg.geo_desc(az=az, const_meters_per_longitude=const)
    assert (geo.lon_origin, geo.lat_origin, geo.meters_per_degree) == (-118.0, 37.0, 111319.5)
    for x, y in [(0.0, 0.0), (21000.0, 23000.0), (-5000.0, 123456.7)]:
        assert sg.geographic_coord(geo, x, y) == _geo_np(geo, x, y)


@pytest.mark.parametrize("mode", [sg.REC_DISPLACEMENT, sg.REC_VELOCITY])
def test_geographic_components(mode, tmp_path):
    """xyz = 0: east-west, north-south, up-down (src/TimeSeries.C:226-246, 1036-1046)."""
    geo = sg.geo_desc(az=27.5)
    x, y = 14000.0, 9000.0
    rng = np.random.default_rng(7)
    v = rng.standard_normal((11, 3))
    out = tmp_path / "geo.txt"
    assert sg.write_usgs(out, v, station="g1", x=x, y=y, gp_x=x, gp_y=y, dt=0.01, mode=mode, xyz=False,
                         geo=geo) == sg.OK
    head, rows = _parse(out.read_text())
    want = ({sg.REC_DISPLACEMENT: ["East-west displacement (m)", "North-sourth displacement (m)",
                                   "Up-down displacement (m)"],
             sg.REC_VELOCITY: ["East-west velocity (m/s)", "Nort-south velocity (m/s)",
                               "Up-down velocity (m/s)"]}[mode])
    assert head[-3:] == [f"# Column {c + 2}: {w}\n" for c, w in enumerate(want)]
    _, lat = _geo_np(geo, x, y)
    ca, sa = math.cos(math.pi * geo.az / 180.0), math.sin(math.pi * geo.az / 180.0)
    d = (x * sa + y * ca) / math.cos(math.pi * lat / 180.0) / geo.meters_per_degree * (math.pi / 180.0) \
        * math.sin(math.pi * lat / 180.0)
    tx, ty = sa + d * ca, ca - d * sa
    n = math.sqrt(tx * tx + ty * ty)
    tx, ty = tx / n, ty / n
    for r, line in enumerate(rows):
        f = line.split()
        assert f[0] == "%e" % (r * 0.01)
        ew = sa * v[r, 0] + ca * v[r, 1]
        ns = ty * v[r, 0] - tx * v[r, 1]
        assert [float(s) for s in f[1:]] == [ew, ns, -v[r, 2]]


@pytest.mark.parametrize("mode,ncol", [(sg.REC_DIV, 1), (sg.REC_CURL, 3), (sg.REC_STRAINS, 6),
                                       (sg.REC_GRADIENT, 9)])
@pytest.mark.parametrize("xyz", [True, False])
def test_other_modes(mode, ncol, xyz, tmp_path):
    """Every mode's columns; divergence is written in either component system, curl,
    strains and gradient only in grid components (the reference writes the header
    alone otherwise)."""
    v = np.arange(4 * 10, dtype=np.float64).reshape(4, 10) * 0.25 - 3.0  # row stride 10
    out = tmp_path / "m.txt"
    rc = sg.write_usgs(out, v[:, :ncol], station="s", x=1.0, y=2.0, gp_x=1.0, gp_y=2.0, dt=0.5, mode=mode,
                       xyz=xyz)
    head, rows = _parse(out.read_text())
    assert f"# nColumns: {ncol + 1}\n" in head
    assert len([l for l in head if l.startswith("# Column")]) == ncol + 1
    if mode == sg.REC_GRADIENT:
        assert head[-1] == "# Column 10: duz/dz component ()\n"
        assert head[-9] == "# Column 2 : dux/dx component ()\n"
    if xyz or mode == sg.REC_DIV:
        assert rc == sg.OK
        assert len(rows) == 4
        for r, line in enumerate(rows):
            assert line == "%e" % (r * 0.5) + "".join(" %24.17e" % x for x in v[r, :ncol]) + "\n"
    else:
        assert rc == sg.NOT_SUPPORTED
        assert rows == []


def test_errors(tmp_path):
    st = dict(station="s", x=0.0, y=0.0, gp_x=0.0, gp_y=0.0, dt=0.1)
    with pytest.raises(sg.Sw4gError, match="status 6"):  # a directory is not writable as a file
        sg.write_usgs(tmp_path, np.zeros((2, 3)), **st)
    with pytest.raises(sg.Sw4gError, match="status 1"):  # unknown mode
        sg.write_usgs(tmp_path / "x.txt", np.zeros((2, 3)), mode=9, **st)
    with pytest.raises(sg.Sw4gError, match="status 1"):  # rows closer than the mode's values
        sg.write_usgs(tmp_path / "x.txt", np.zeros((2, 2)), **st)


# ---------------------------------------------------------------------------
# Binary SAC traces (sw4g_write_sac) against the reference's stored traces
# tests/loh1/loh1-h100-sta10/sta10.[xyz] and tests/loh2/loh2-h100-sta10/sta10.[xyz]
# (TimeSeries::write_sac_format, src/TimeSeries.C:826, with the SAC header library
# src/sacsubc.C), given the same run's record values (its USGS file's columns).
SAC_META = json.loads((GOLDEN / "sac_meta.json").read_text())
# The two stored runs come from different builds: the LOH.1 traces hold signed zeros
# where the records round to FP32 subnormals (a flush-to-zero build; 13-15 samples per
# trace), the LOH.2 traces hold the subnormals themselves (8-9 per trace).
SAC_FLUSH = {"loh1_h100_sta10": True, "loh2_h100_sta10": False}
# ... and different longitude origins: +118 for LOH.1, the source's default -118 for
# LOH.2 (the "Target location" of each run's own USGS file: 118.2594 and -117.7406).
SAC_LON0 = {"loh1_h100_sta10": 118.0, "loh2_h100_sta10": -118.0}


def _utc_of(date_line):
    return _utc([date_line])


@pytest.mark.parametrize("name", sorted(SAC_META))
def test_sac_writer_reproduces_reference_traces(name, tmp_path):
    m = SAC_META[name]
    rec = np.load(GOLDEN / f"sac_{name}_records.npz")["records"]
    assert rec.shape == (m["rows"], 3)
    geo = sg.geo_desc(lon_origin=SAC_LON0[name])
    if m["event"] == "source":
        sx, sy, sz = m["source_xyz"]
        lon, lat = sg.geographic_coord(geo, sx, sy)
        event = (lat, lon, sz, m["source_t0"])
    else:
        event = (0.0, 0.0, 0.0, 0.0)
    sg.write_sac(tmp_path / "sta10.", rec, station="sta10", x=m["x"], y=m["y"], dt=m["t"] / (m["rows"] - 1),
                 utc=_utc_of(m["date"]), event=event, geo=geo, flush_subnormals=SAC_FLUSH[name])
    for c in "xyz":
        mine = (tmp_path / f"sta10.{c}").read_bytes()
        ref = (GOLDEN / f"sac_{name}.{c}").read_bytes()
        assert len(mine) == len(ref) == 632 + 4 * m["rows"]
        assert mine == ref, c


def _sac(path):
    b = Path(path).read_bytes()
    return (np.frombuffer(b[:280], "<f4"), np.frombuffer(b[280:440], "<i4"),
            [b[440 + 8 * q:448 + 8 * q].decode() for q in range(24)], np.frombuffer(b[632:], "<f4"))


@pytest.mark.parametrize("mode,xyz,files", [
    (sg.REC_DISPLACEMENT, False, [("e", "EW", 90, 90), ("n", "NS", 90, 0), ("u", "UP", 0, 0)]),
    (sg.REC_VELOCITY, True, [("xv", "Vx", 90, 30), ("yv", "Vy", 90, 120), ("zv", "Vz", 180, 0)]),
    (sg.REC_VELOCITY, False, [("ev", "Vew", 90, 90), ("nv", "Vns", 90, 0), ("uv", "Vup", 0, 0)]),
    (sg.REC_DIV, True, [("div", "Div", 90, 30)]),
    (sg.REC_CURL, False, [("curlx", "Curlx", 90, 30), ("curly", "Curly", 90, 120), ("curlz", "Curlz", 180, 0)]),
    (sg.REC_STRAINS, True, [("xx", "Uxx", 90, 30), ("yy", "Uyy", 90, 120), ("zz", "Uzz", 180, 0),
                            ("xy", "Uxy", 90, 30), ("xz", "Uxz", 90, 30), ("yz", "Uyz", 90, 30)]),
    (sg.REC_GRADIENT, True, [("duxdx", "DUXDX", 90, 30), ("duxdy", "DUXDY", 90, 30), ("duxdz", "DUXDZ", 90, 30),
                             ("duydx", "DUYDX", 90, 30), ("duydy", "DUYDY", 90, 120), ("duydz", "DUYDZ", 90, 30),
                             ("duzdx", "DUZDX", 90, 30), ("duzdy", "DUZDY", 90, 30), ("duzdz", "DUZDZ", 180, 0)]),
])
def test_sac_modes(mode, xyz, files, tmp_path):
    """Every mode's files, names, inclinations and azimuths (src/TimeSeries.C:450-822),
    grid azimuth 30; geographic displacement, velocity and curl rotated from the FP32
    values (src/TimeSeries.C:704-713)."""
    geo = sg.geo_desc(az=30.0)
    n = len(files)
    rng = np.random.default_rng(11)
    v = rng.standard_normal((9, n))
    x, y = 3000.0, 4000.0
    sg.write_sac(tmp_path / "r.", v, station="station12345", x=x, y=y, dt=0.25, t_shift=-0.5, mode=mode,
                 xyz=xyz, utc=(2016, 12, 15, 17, 41, 34, 7), event=(1.0, 2.0, 3000.0, 0.5), geo=geo)
    f32 = v.astype(np.float32)
    if not xyz and mode in (sg.REC_DISPLACEMENT, sg.REC_VELOCITY, sg.REC_CURL):
        _, lat = sg.geographic_coord(geo, x, y)
        ca, sa = math.cos(math.pi * 30 / 180.0), math.sin(math.pi * 30 / 180.0)
        d = (x * sa + y * ca) / math.cos(math.pi * lat / 180.0) / geo.meters_per_degree * (math.pi / 180.0) \
            * math.sin(math.pi * lat / 180.0)
        tx, ty = sa + d * ca, ca - d * sa
        nrm = math.sqrt(tx * tx + ty * ty)
        tx, ty = tx / nrm, ty / nrm
        u0, u1, u2 = (f32[:, c].astype(np.float64) for c in range(3))
        f32 = np.stack([(sa * u0 + ca * u1), (ty * u0 - tx * u1), -u2], axis=1).astype(np.float32)
    for c, (suffix, name, inc, az) in enumerate(files):
        fh, ih, kh, data = _sac(tmp_path / f"r.{suffix}")
        assert np.array_equal(data, f32[:, c])
        assert kh[20] == f"{name:<8}"[:8] and kh[0] == "station1"
        assert (fh[58], fh[57]) == (np.float32(inc), np.float32(az))
        assert (fh[0], fh[5], fh[6], fh[7]) == (np.float32(0.25), np.float32(-0.5), np.float32(1.5), np.float32(0.5))
        assert (fh[1], fh[2]) == (f32[:, c].min(), f32[:, c].max())
        assert fh[56] == np.float32(f32[:, c].astype(np.float64).sum() / 9)
        assert (fh[35], fh[36], fh[38]) == (np.float32(1.0), np.float32(2.0), np.float32(3.0))
        assert list(ih[:10]) == [2016, 350, 17, 41, 34, 7, 6, 0, 0, 9]
        assert (ih[15], ih[35], ih[36], ih[37], ih[38], ih[39]) == (1, 1, 0, 1, 1, 0)
        assert kh[1] == "-12345  "


def test_sac_errors(tmp_path):
    kw = dict(station="s", x=0.0, y=0.0, dt=0.1)
    with pytest.raises(sg.Sw4gError, match="status 6"):  # no such directory
        sg.write_sac(tmp_path / "missing" / "r.", np.zeros((2, 3)), **kw)
    with pytest.raises(sg.Sw4gError, match="status 1"):  # unknown mode
        sg.write_sac(tmp_path / "r.", np.zeros((2, 3)), mode=7, **kw)
    with pytest.raises(sg.Sw4gError, match="status 1"):  # rows closer than the mode's values
        sg.write_sac(tmp_path / "r.", np.zeros((2, 2)), **kw)
    # no rows: header-only traces with NPTS 0 and the mean unset
    sg.write_sac(tmp_path / "e.", np.zeros((0, 1)), mode=sg.REC_DIV, **kw)
    fh, ih, _, data = _sac(tmp_path / "e.div")
    assert ih[9] == 0 and fh[56] == np.float32(-12345.0) and data.size == 0
