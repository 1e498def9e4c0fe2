"""Generate the committed golden fixtures (inputs + expected outputs).

  python tests/golden/make_golden.py

Inputs are stored in the fixture itself, so the fixtures do not depend on the
generator's random streams.  Expected outputs come from the CPU oracle, whose
restatements are pinned separately against the reference's own known-answer
fixture (RasterJoin/test/baseline.hpp:139-217) in tests/test_oracle.py.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "raster-join_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from rasterjoin import synth  # noqa: E402


def cases():
    pts = synth.points(10_007, seed=11, columns=True)
    vor = synth.voronoi_polygons(24, seed=11, verts_per_poly=60)
    stars = synth.star_polygons(12, seed=11, vmin=5, vmax=80, rmin=800, rmax=8000)
    return pts, {"voronoi": vor, "stars": stars}


def outputs(pts, verts, pidx):
    cols = oracle.Columns({2: (oracle.Uint, pts["t"]), 3: (oracle.Float, pts["a"]), 4: (oracle.Int, pts["f1"]),
                           5: (oracle.Int, pts["f2"])})
    f = cols.filt([(4, oracle.GT, 2), (5, oracle.LT, 8), (3, oracle.LT, 50.0)], aggr_attrib=3,
                  time_range=(2, synth.T0, synth.T0 + synth.YEAR // 2))
    xy = pts["xy"]
    out = {}
    out["index64_count"], _ = oracle.index_join(xy, verts, pidx, 64)
    out["index64_clamp_count"], _ = oracle.index_join(xy, verts, pidx, 64, compat_clamp=True)
    out["hybrid64_count"], _ = oracle.hybrid_join(xy, verts, pidx, 64)
    out["cpujoin256_count"], _, _, _ = oracle.cpujoin(xy, verts, pidx, 256)
    out["index64_filt_count"], out["index64_filt_sum"] = oracle.index_join(xy, verts, pidx, 64, f=f)
    out["raster50_count"], _, out["raster50_bounds"] = oracle.raster_join(xy, verts, pidx, 50.0, bounds=True)
    out["raster50_filt_count"], out["raster50_filt_sum"], _ = oracle.raster_join(xy, verts, pidx, 50.0, f=f)
    out["raster20_tiles_count"], _, _ = oracle.raster_join(xy, verts, pidx, 20.0, max_res=700)
    return out


def main():
    pts, polys = cases()
    for name, (verts, pidx) in polys.items():
        d = {"xy": pts["xy"], "t": pts["t"], "a": pts["a"], "f1": pts["f1"], "f2": pts["f2"], "verts": verts,
             "pindex": pidx}
        d.update(outputs(pts, verts, pidx))
        np.savez_compressed(os.path.join(HERE, "golden_%s.npz" % name), **d)
        print(name, {k: (v.shape, v.dtype) for k, v in d.items()})


if __name__ == "__main__":
    main()
