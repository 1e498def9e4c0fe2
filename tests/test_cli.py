"""The command-line driver (RasterJoin/main.cpp options and outputs), the
polygon text loader with its lat/lon transform, and the backend column-store
reader.  The dump mode needs no GPU; the joins run through librj.so."""
import os
import subprocess

import numpy as np
import pytest

import backend_format as bf
import oracle
from rasterjoin import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "raster-join_gb300", "lib", "rj_cli")
T0 = synth.T0
DAY = 86400


def fnv(data):
    h = 1469598103934665603
    for c in bytes(data):
        h = ((h ^ c) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def run_cli(args, check=True):
    r = subprocess.run([CLI] + [str(a) for a in args], capture_output=True, text=True, timeout=600)
    if check and r.returncode != 0:
        raise AssertionError("rj_cli failed (%d):\n%s\n%s" % (r.returncode, r.stdout, r.stderr))
    return r


@pytest.fixture(scope="module")
def fixture_dir(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("cli")
    pts = synth.points(60_000, seed=31, columns=True)
    cols = {0: (0, pts["xy"]), 1: (1, pts["t"]), 2: (3, pts["a"]), 3: (2, pts["f1"])}
    stem = str(d / "pts")
    chunks = bf.write_backend(stem, cols, loc_attrib=0, time_attrib=1, lx=7000.0, ly=5000.0, lz=10 * DAY,
                              flush_every=7000)
    verts, pidx = synth.voronoi_polygons(40, seed=8)
    polys = [verts[pidx[i]:pidx[i + 1]] for i in range(len(pidx) - 1)]
    bf.write_polygons(str(d / "neigh.txt"), polys)
    (d / "polys.txt").write_text("neigh,neigh.txt\n")
    return d, pts, chunks, verts, pidx


def expected_selection(fixture, t0, t1):
    d, pts, chunks, verts, pidx = fixture
    lo = (np.float32(verts[:, 0].min()), np.float32(verts[:, 1].min()), np.float32(t0))
    hi = (np.float32(verts[:, 0].max()), np.float32(verts[:, 1].max()), np.float32(t1))
    parts = bf.region_partitions(lo, hi, 7000.0, 5000.0, 10 * DAY)
    return bf.selected_rows(chunks, parts)


def base_args(d, t0, t1, join="raster"):
    return ["--joinType", join, "--backendIndexName", d / "pts", "--polygonList", d / "polys.txt",
            "--polygonDataset", "neigh", "--locAttrib", 0, "--startTime", t0, "--endTime", t1, "--world"]


def test_cli_requires_options(built):
    r = run_cli([], check=False)
    assert r.returncode == 1 and "help message" in r.stdout


@pytest.mark.parametrize("window", [(T0, T0 + 365 * DAY), (T0 + 50 * DAY, T0 + 80 * DAY)])
def test_dump_reads_backend_partitions(fixture_dir, window):
    d, pts, chunks, verts, pidx = fixture_dir
    out = run_cli(base_args(d, *window) + ["--avg", 2, "--dumpOnly"]).stdout.split("\n")
    head = out[0].split()
    assert int(head[1]) == len(pidx) - 1 and int(head[3]) == len(verts)
    bounds = [float(v) for v in head[5:9]]
    want_b = [np.float32(verts[:, 0].min()), np.float32(verts[:, 1].min()),
              np.float32(verts[:, 0].max()), np.float32(verts[:, 1].max())]
    np.testing.assert_array_equal(np.float32(bounds), want_b)
    rows = expected_selection(fixture_dir, *window)
    assert int(head[10]) == len(rows)
    attrs = {int(l.split()[1]): l.split() for l in out[1:] if l.startswith("attr")}
    assert set(attrs) == {0, 2}
    assert int(attrs[0][5], 16) == fnv(np.ascontiguousarray(pts["xy"][rows]).tobytes())
    assert int(attrs[2][5], 16) == fnv(np.ascontiguousarray(pts["a"][rows]).tobytes())


def test_polygon_loader_geo_transform(tmp_path, built):
    """lat/lon polygons: rings appended, repeated vertices and the closing
    vertex dropped, polygons leaving the US box skipped, float bounds."""
    rng = np.random.default_rng(4)
    polys, rings, keep = [], [], []
    for i in range(6):
        c = (rng.uniform(30, 45), rng.uniform(-120, -75))
        ang = np.sort(rng.uniform(0, 2 * np.pi, 9))
        p = np.c_[c[0] + 0.05 * np.cos(ang), c[1] + 0.05 * np.sin(ang)]
        p = np.r_[p, p[:1]]                    # closed ring
        p = np.r_[p[:3], p[2:3], p[3:]]        # a repeated vertex
        if i == 4:
            p[5] = (60.0, -100.0)              # outside the box: polygon dropped
        polys.append(p)
        rings.append([4] if i == 2 else None)  # polygon 2 written as two parts
        keep.append(i != 4)
    bf.write_polygons(str(tmp_path / "geo.txt"), polys, rings)
    (tmp_path / "list.txt").write_text("g,geo.txt\n")
    pts = synth.points(1000, seed=1, columns=True)
    bf.write_backend(str(tmp_path / "b"), {0: (0, pts["xy"]), 1: (1, pts["t"])}, 0, 1, 1e9, 1e9, 10 ** 9)
    r = run_cli(["--joinType", "raster", "--backendIndexName", tmp_path / "b", "--polygonList", tmp_path / "list.txt",
                 "--polygonDataset", "g", "--locAttrib", 0, "--startTime", 0, "--endTime", 1, "--dumpOnly"])
    head = r.stdout.split()
    world = []
    for p, k in zip(polys, keep):
        if not k:
            continue
        q = [p[0]]
        for v in p[1:]:
            if (v != q[-1]).any():
                q.append(v)
        if (q[0] == q[-1]).all():
            q.pop()
        world.append([bf.transform_point(a, b) for a, b in q])
    assert int(head[1]) == len(world)
    assert int(head[3]) == sum(len(w) for w in world)
    allv = np.array([v for w in world for v in w])
    want = [np.float32(allv[:, 0]).min(), np.float32(allv[:, 1]).min(), np.float32(allv[:, 0]).max(),
            np.float32(allv[:, 1]).max()]
    np.testing.assert_array_equal(np.float32([float(v) for v in head[5:9]]), want)


@pytest.mark.gpu
@pytest.mark.parametrize("join", ["raster", "index", "hybrid", "errorbounds"])
def test_cli_joins_match_oracle(fixture_dir, tmp_path, join):
    d, pts, chunks, verts, pidx = fixture_dir
    window = (T0 + 20 * DAY, T0 + 200 * DAY)
    outdir = tmp_path / "agg"
    outdir.mkdir()
    tfile = tmp_path / "times.txt"
    run_cli(base_args(d, *window, join=join) + ["--cellSize", 25.0, "--indexRes", 256, "--opAggregation", outdir,
                                                 "--outputTime", tfile, "--nIter", 2])
    rows = expected_selection(fixture_dir, *window)
    xy = pts["xy"][rows]
    bbox = np.array([np.float32(verts[:, 0].min()), np.float32(verts[:, 1].min()),
                     np.float32(verts[:, 0].max()), np.float32(verts[:, 1].max())], np.float64)
    acc = 100 if join in ("raster", "errorbounds") else 0
    if join == "errorbounds":
        c, _, b = oracle.raster_join(xy, verts, pidx, 25.0, bbox=bbox, bounds=True)
        got = np.loadtxt(outdir / ("err_bound_%d_%d.csv" % (window[1], acc)), dtype=np.int64).reshape(-1, 5)
        P = len(pidx) - 1
        np.testing.assert_array_equal(got[:, 1], c.astype(np.int64) - b[3 * P:])
        np.testing.assert_array_equal(got[:, 2], c.astype(np.int64) + b[2 * P:3 * P])
    else:
        if join == "raster":
            want = oracle.raster_join(xy, verts, pidx, 25.0, bbox=bbox)[0]
        elif join == "index":
            want = oracle.index_join(xy, verts, pidx, 256, bbox=bbox)[0]
        else:
            want = oracle.hybrid_join(xy, verts, pidx, 256, bbox=bbox)[0]
        got = np.loadtxt(outdir / ("raster_%d_%d.csv" % (window[1], acc)), dtype=np.int64).reshape(-1, 2)
        np.testing.assert_array_equal(got[:, 1], want.astype(np.int64))
    lines = tfile.read_text().strip().split("\n")
    fields = lines[-1].split("\t")
    assert len(fields) == 16 and int(fields[0]) == len(rows)   # "%llu\t\t..." leaves one empty field
    assert int(fields[3]) == {"raster": 0, "index": 1, "hybrid": 2, "errorbounds": 5}[join]


@pytest.mark.gpu
def test_cli_avg_and_exact_time(fixture_dir, tmp_path):
    d, pts, chunks, verts, pidx = fixture_dir
    window = (T0 + 20 * DAY, T0 + 200 * DAY)
    outdir = tmp_path / "agg"
    outdir.mkdir()
    run_cli(base_args(d, *window, join="index") + ["--avg", 2, "--exactTime", 1, "--opAggregation", outdir])
    rows = expected_selection(fixture_dir, *window)
    sel = rows[(pts["t"][rows] >= window[0]) & (pts["t"][rows] <= window[1])]
    cols = oracle.Columns({2: (oracle.Float, pts["a"][sel])})
    bbox = np.array([np.float32(verts[:, 0].min()), np.float32(verts[:, 1].min()),
                     np.float32(verts[:, 0].max()), np.float32(verts[:, 1].max())], np.float64)
    c, s = oracle.index_join(pts["xy"][sel], verts, pidx, 256, f=cols.filt(aggr_attrib=2), bbox=bbox)
    got = np.loadtxt(outdir / ("raster_%d_0.csv" % window[1])).reshape(-1, 2)
    # printResults decodes the lossy [count | sum/100 | decimal*10] layout in fp32
    want = np.where(c > 0, s / np.maximum(c, 1), 0.0)
    np.testing.assert_allclose(got[:, 1], want, rtol=2e-3, atol=0.06)
