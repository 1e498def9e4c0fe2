"""Seeded synthetic inputs with the shapes of the benchmark configurations.

The reference measured on NYC-taxi and Twitter extracts that are not shipped
with it; these generators stand in for them:

* points: float32 (x, y) metres in a 40 x 40 km box, 80 % from 8 Gaussians
  (sigma 2 km, centres uniform in the box, draws outside the box redrawn) and
  20 % uniform; optional columns t (uint32, uniform over one year), a (float32
  lognormal mu=2.5 sigma=0.8), f1 / f2 (int32 uniform 0..9).
* voronoi_polygons: a Voronoi tessellation of seeded sites clipped to the box
  (sites mirrored across the four sides), every inner edge subdivided and
  jittered perpendicular to itself; an edge shared by two cells is generated
  once, so neighbours share identical float32 vertices and the cells do not
  overlap.
* star_polygons: jittered radial stars around seeded centres (concave, may
  overlap each other).
"""
import numpy as np

BOX = 40000.0
T0 = 1230768000            # 2009-01-01, the reference's query start (main.cpp:358)
YEAR = 365 * 86400


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def points(n, seed=20261203, box=BOX, columns=False, chunk=1 << 24):
    """Return dict: xy float32 [n,2]; with columns also t, a, f1, f2."""
    rng = _rng(seed)
    centres = rng.uniform(0.0, box, size=(8, 2))
    xy = np.empty((n, 2), np.float32)
    done = 0
    while done < n:
        m = min(chunk, n - done)
        gauss = rng.random(m) < 0.8
        comp = rng.integers(0, 8, m)
        p = rng.uniform(0.0, box, size=(m, 2))
        g = centres[comp] + rng.normal(0.0, 2000.0, size=(m, 2))
        p[gauss] = g[gauss]
        p32 = p.astype(np.float32)
        ok = (p32[:, 0] >= 0) & (p32[:, 0] < np.float32(box)) & (p32[:, 1] >= 0) & (p32[:, 1] < np.float32(box))
        p32 = p32[ok]
        take = min(len(p32), n - done)
        xy[done:done + take] = p32[:take]
        done += take
    out = {"xy": xy}
    if columns:
        out["t"] = rng.integers(T0, T0 + YEAR, n, dtype=np.uint32)
        out["a"] = rng.lognormal(2.5, 0.8, n).astype(np.float32)
        out["f1"] = rng.integers(0, 10, n, dtype=np.int32)
        out["f2"] = rng.integers(0, 10, n, dtype=np.int32)
    return out


def _flatten(polys):
    pindex = np.zeros(len(polys) + 1, np.int32)
    pindex[1:] = np.cumsum([len(p) for p in polys])
    xy = np.concatenate(polys).astype(np.float32) if polys else np.zeros((0, 2), np.float32)
    return xy, pindex


def voronoi_polygons(nsites=260, seed=20261203, box=BOX, verts_per_poly=100, jitter=50.0):
    """Non-overlapping Voronoi cells covering the box; returns (xy [V,2] f32, pindex [P+1])."""
    from scipy.spatial import Voronoi

    rng = _rng(seed + 7)
    sites = rng.uniform(0.0, box, size=(nsites, 2))
    mirrored = [sites,
                np.c_[-sites[:, 0], sites[:, 1]], np.c_[2 * box - sites[:, 0], sites[:, 1]],
                np.c_[sites[:, 0], -sites[:, 1]], np.c_[sites[:, 0], 2 * box - sites[:, 1]]]
    vor = Voronoi(np.concatenate(mirrored))
    V = vor.vertices.copy()
    # vertices on the box boundary are computed with rounding error: snap them
    for d in range(2):
        V[np.abs(V[:, d]) < 1e-6 * box, d] = 0.0
        V[np.abs(V[:, d] - box) < 1e-6 * box, d] = box
    V = np.clip(V, 0.0, box)
    cells = []
    perim = 0.0
    for i in range(nsites):
        reg = vor.regions[vor.point_region[i]]
        assert -1 not in reg and len(reg) >= 3
        pts = V[reg]
        ang = np.arctan2(pts[:, 1] - sites[i, 1], pts[:, 0] - sites[i, 0])
        order = np.asarray(reg)[np.argsort(ang)]
        # drop repeated vertex indices / coincident vertices
        keep = [order[0]]
        for v in order[1:]:
            if np.any(V[v] != V[keep[-1]]):
                keep.append(v)
        if np.all(V[keep[-1]] == V[keep[0]]) and len(keep) > 1:
            keep.pop()
        cells.append(keep)
        for a, b in zip(keep, keep[1:] + keep[:1]):
            perim += np.hypot(*(V[b] - V[a]))
    target_seg = perim / max(1, nsites * verts_per_poly)
    edge_pts = {}

    def edge_points(a, b):
        key = (min(a, b), max(a, b))
        if key not in edge_pts:
            u, v = V[key[0]], V[key[1]]
            d = v - u
            L = float(np.hypot(*d))
            k = max(1, int(round(L / target_seg)))
            s = np.arange(1, k) / k
            on_box = (u[0] == v[0] and u[0] in (0.0, box)) or (u[1] == v[1] and u[1] in (0.0, box))
            if on_box or L == 0.0:
                off = np.zeros(k - 1)
            else:
                amp = min(jitter, 0.2 * L)
                off = rng.uniform(-1.0, 1.0, k - 1) * amp * np.sin(np.pi * s)
            nrm = np.array([-d[1], d[0]]) / (L if L > 0 else 1.0)
            inner = u[None, :] + s[:, None] * d[None, :] + off[:, None] * nrm[None, :]
            inner = np.clip(inner, 0.0, box)
            edge_pts[key] = inner.astype(np.float32)
        pts = edge_pts[key]
        return pts if a == key[0] else pts[::-1]

    V32 = V.astype(np.float32)
    polys = []
    for keep in cells:
        ring = []
        for a, b in zip(keep, keep[1:] + keep[:1]):
            ring.append(V32[a][None, :])
            ring.append(edge_points(a, b))
        poly = np.concatenate(ring)
        # remove consecutive duplicates (PolyHandler.cpp:155-163)
        dup = np.all(poly == np.roll(poly, 1, axis=0), axis=1)
        poly = poly[~dup] if len(poly) > 3 else poly
        polys.append(poly)
    return _flatten(polys)


def star_polygons(npolys, seed=20261203, box=BOX, vmin=20, vmax=500, rmin=200.0, rmax=2000.0, inner=0.35):
    """Jittered radial star polygons; vertex counts and radii log-uniform."""
    rng = _rng(seed + 11)
    polys = []
    for _ in range(npolys):
        n = int(round(np.exp(rng.uniform(np.log(vmin), np.log(vmax)))))
        n = max(n, 3)
        r = np.exp(rng.uniform(np.log(rmin), np.log(rmax)))
        c = rng.uniform(r, box - r, size=2) if box > 2 * r else rng.uniform(0, box, size=2)
        ang = 2 * np.pi * (np.arange(n) + rng.uniform(-0.3, 0.3, n)) / n
        ang = np.sort(ang)
        rad = r * rng.uniform(inner, 1.0, n)
        p = np.c_[c[0] + rad * np.cos(ang), c[1] + rad * np.sin(ang)]
        p = np.clip(p, 0.0, box).astype(np.float32)
        dup = np.all(p == np.roll(p, 1, axis=0), axis=1)
        polys.append(p[~dup])
    return _flatten(polys)


def kat_two_squares():
    """The 2-square / 5-point fixture of RasterJoin/test/baseline.hpp:139-217."""
    xy = np.array([[5.15, 5.15], [5.15, 5.15], [5.0, 5.0], [5.0, 5.0], [5.0, 5.0]], np.float32)
    sq0 = [(5.1, 5.1), (5.2, 5.1), (5.2, 5.2), (5.1, 5.2)]
    sq1 = [(4.9, 4.9), (5.1, 4.9), (5.1, 5.1), (4.9, 5.1)]
    polys = [np.array(sq0, np.float32), np.array(sq1, np.float32)]
    return xy, _flatten(polys), np.array([2, 3], np.uint64)
