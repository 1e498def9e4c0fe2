"""Fill rule against the reference's own triangulation.

The reference triangulates every polygon with clip2tri (clipper union,
coordinates snapped to 1/1000, poly2tri constrained Delaunay;
PolyHandler.cpp:82-115) and lets the GL rasteriser decide which pixel centres
each triangle covers.  The rasteriser is not available, so this test compiles
the reference's triangulation sources (oracle/ref_tri, into oracle/_ref) and
applies GL's triangle rule (edge functions on the same 1/256-pixel snapped
window coordinates; ties to left and top edges) to its triangles, then
compares, pixel centre by pixel centre, with the polygon crossing rule the
library implements (same snapping, same top-closed / left-closed ties).
Centres can only disagree where clip2tri's 1/1000 snapping moved an edge
across them; the test measures that no other disagreement exists."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from rasterjoin import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "oracle", "_ref", "libreftri.so")


def ref_lib():
    if not os.path.exists(LIB):
        import importlib.util
        spec = importlib.util.spec_from_file_location("reftri_build", os.path.join(ROOT, "oracle", "ref_tri", "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        if mod.build(optional=True) is None:
            pytest.skip("reference triangulation sources not available")
    L = C.CDLL(LIB)
    L.ref_triangulate.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double), C.c_int]
    L.ref_triangulate.restype = C.c_int
    return L


def triangulate(L, poly):
    xy = np.ascontiguousarray(poly, np.float64)
    cap = 4 * len(poly) + 16
    out = np.zeros(cap * 6, np.float64)
    nt = L.ref_triangulate(xy.ctypes.data_as(C.POINTER(C.c_double)), len(poly),
                           out.ctypes.data_as(C.POINTER(C.c_double)), cap)
    assert nt >= 0
    return out[:nt * 6].reshape(-1, 6)


def dist_to_edges(px, py, poly):
    a = poly
    b = np.roll(poly, -1, axis=0)
    d = b - a
    t = np.clip(((px - a[:, 0]) * d[:, 0] + (py - a[:, 1]) * d[:, 1]) / np.maximum((d ** 2).sum(1), 1e-30), 0, 1)
    qx, qy = a[:, 0] + t * d[:, 0], a[:, 1] + t * d[:, 1]
    return float(np.sqrt(((qx - px) ** 2 + (qy - py) ** 2).min()))


@pytest.mark.parametrize("kind,cell", [("voronoi", 40.0), ("stars", 25.0)])
def test_polygon_rule_matches_triangle_rule_on_reference_triangulation(kind, cell):
    L = ref_lib()
    if kind == "voronoi":
        verts, pidx = synth.voronoi_polygons(40, seed=21)
    else:
        verts, pidx = synth.star_polygons(12, seed=21, vmin=8, vmax=60, rmin=1500, rmax=5000)
    polys = [verts[pidx[i]:pidx[i + 1]].astype(np.float64) for i in range(len(pidx) - 1)]
    tris, tri_poly = [], []
    for i, p in enumerate(polys):
        t = triangulate(L, p)
        tris.append(t)
        tri_poly.extend([i] * len(t))
    tris = np.concatenate(tris)
    bbox = np.array([verts[:, 0].min(), verts[:, 1].min(), verts[:, 0].max(), verts[:, 1].max()], np.float64)
    a, b = oracle.cover_maps(verts, pidx, tris, np.array(tri_poly, np.int32), bbox, cell)
    if kind == "voronoi":
        assert (a != -2).all()           # a tessellation: every centre in at most one polygon
    covered = int((a >= 0).sum())
    assert covered > 10_000
    diff = np.argwhere(a != b)
    # every disagreement sits within clip2tri's 1/1000 snapping of an edge
    ry, rx = a.shape
    for j, i in diff:
        x = bbox[0] + (i + 0.5) * (bbox[2] - bbox[0]) / rx
        y = bbox[1] + (j + 0.5) * (bbox[3] - bbox[1]) / ry
        near = min(dist_to_edges(x, y, p) for p in polys)
        assert near < 0.01 * cell, (j, i, near)
    assert len(diff) <= max(3, covered // 10_000)
