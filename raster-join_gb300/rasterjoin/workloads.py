"""Seeded workloads of the batched and served benchmark configurations.

* device_table: the point table generated directly in GPU memory (torch),
  same distributions as synth.points (80 % of the points from 8 Gaussians
  with sigma 2 km, 20 % uniform, in a 40 x 40 km box; t uniform over one
  year; a lognormal(2.5, 0.8)), for tables too large to build on the host
  within a benchmark run (1B points).
* star_set: jittered radial star polygons, vectorised (the batched / served
  configurations draw hundreds of polygon sets).
* batched_queries: 512 raster queries, each with its own polygon set of
  1-5,000 stars (4-2,000 vertices, log-uniform), epsilon log-uniform in
  1-1,000 m, a time window selecting 10K-500M points, count or avg.
* served_requests: Poisson arrivals; each request 1-50 stars (8-300
  vertices, radii 200 m - 10 km), epsilon from a zoom level in
  {1, 10, 100, 1000} m and a time window of 1 hour to 30 days.
Epsilon is the pixel side (cell = epsilon), the convention the benchmark
configurations quote ("epsilon = 10 m, 4000^2 canvas" on a 40 km box).
"""
import numpy as np

from .synth import BOX, T0, YEAR

HOUR = 3600
DAY = 86400


def device_table(n, seed, device="cuda", chunk=1 << 26):
    """x, y (float32 [n,2]), t (int32 holding uint32 times), a (float32) as
    torch tensors on `device`."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    centres = torch.rand((8, 2), generator=g, device=device, dtype=torch.float64) * BOX
    xy = torch.empty((n, 2), dtype=torch.float32, device=device)
    t = torch.empty(n, dtype=torch.int32, device=device)
    a = torch.empty(n, dtype=torch.float32, device=device)
    box = torch.tensor(BOX, dtype=torch.float32, device=device)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        p = torch.empty((m, 2), dtype=torch.float32, device=device)
        todo = torch.arange(m, device=device)
        while todo.numel():
            k = todo.numel()
            gauss = torch.rand(k, generator=g, device=device) < 0.8
            comp = torch.randint(0, 8, (k,), generator=g, device=device)
            u = torch.rand((k, 2), generator=g, device=device, dtype=torch.float64) * BOX
            v = centres[comp] + torch.randn((k, 2), generator=g, device=device, dtype=torch.float64) * 2000.0
            q = torch.where(gauss[:, None], v, u).to(torch.float32)
            ok = (q[:, 0] >= 0) & (q[:, 0] < box) & (q[:, 1] >= 0) & (q[:, 1] < box)
            p[todo[ok]] = q[ok]
            todo = todo[~ok]
        xy[s:s + m] = p
        t[s:s + m] = torch.randint(T0, T0 + YEAR, (m,), generator=g, device=device, dtype=torch.int64).to(torch.int32)
        a[s:s + m] = torch.exp(torch.randn(m, generator=g, device=device) * 0.8 + 2.5)
    return {"xy": xy, "t": t, "a": a}


def star_set(rng, npolys, vmin, vmax, rmin, rmax, inner=0.35, box=BOX):
    """npolys stars: vertex counts and radii log-uniform; returns (xy float32
    [V,2], pindex int32 [P+1])."""
    nv = np.maximum(np.rint(np.exp(rng.uniform(np.log(vmin), np.log(vmax), npolys))).astype(np.int64), 3)
    r = np.exp(rng.uniform(np.log(rmin), np.log(rmax), npolys))
    lo = np.where(box > 2 * r, r, 0.0)
    hi = np.where(box > 2 * r, box - r, box)
    c = rng.uniform(lo[:, None], hi[:, None], (npolys, 2))
    off = np.zeros(npolys + 1, np.int64)
    off[1:] = np.cumsum(nv)
    pid = np.repeat(np.arange(npolys), nv)
    k = np.arange(off[-1]) - off[pid]
    # jitter below half a step keeps the angles increasing within a polygon
    ang = 2 * np.pi * (k + rng.uniform(-0.3, 0.3, off[-1])) / nv[pid]
    rad = r[pid] * rng.uniform(inner, 1.0, off[-1])
    p = np.c_[c[pid, 0] + rad * np.cos(ang), c[pid, 1] + rad * np.sin(ang)]
    p = np.clip(p, 0.0, box).astype(np.float32)
    prev = np.arange(off[-1]) - 1
    prev[off[:-1]] = off[1:] - 1
    keep = ~np.all(p == p[prev], axis=1)
    keep[off[:-1]] = True
    counts = np.bincount(pid[keep], minlength=npolys)
    pindex = np.zeros(npolys + 1, np.int32)
    pindex[1:] = np.cumsum(counts)
    return p[keep], pindex


def _window(rng, nrows, lo_rows, hi_rows):
    """Time window holding about [lo_rows, hi_rows] rows of a table of nrows
    rows uniform over one year (log-uniform in between)."""
    frac = np.exp(rng.uniform(np.log(lo_rows / nrows), np.log(min(1.0, hi_rows / nrows))))
    span = int(frac * YEAR)
    start = T0 + int(rng.uniform(0, max(1, YEAR - span)))
    return start, min(start + span, T0 + YEAR - 1)


def batched_queries(nq, nrows, seed=20261204, max_verts=600_000):
    """[(xy, pindex, cell, (t0, t1), avg)] for the batched configuration."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nq):
        npolys = int(np.exp(rng.uniform(0.0, np.log(5000.0))))
        vmax = min(2000.0, max(4.0, max_verts / npolys))
        rmax = 10000.0 if npolys <= 20 else max(300.0, 10000.0 / np.sqrt(npolys / 20.0))
        xy, pidx = star_set(rng, npolys, 4, vmax, 200.0, rmax)
        cell = float(np.exp(rng.uniform(0.0, np.log(1000.0))))
        out.append((xy, pidx, cell, _window(rng, nrows, 1e4, 5e8), bool(i % 2)))
    return out


def served_requests(nreq, rate_qps, seed=20261205):
    """[(arrival_s, xy, pindex, cell, (t0, t1))] with Poisson arrivals."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_qps, nreq))
    out = []
    for i in range(nreq):
        npolys = int(rng.integers(1, 51))
        xy, pidx = star_set(rng, npolys, 8, 300, 200.0, 10000.0)
        cell = float(rng.choice([1.0, 10.0, 100.0, 1000.0]))
        span = int(np.exp(rng.uniform(np.log(HOUR), np.log(30 * DAY))))
        start = T0 + int(rng.uniform(0, YEAR - span))
        out.append((float(arrivals[i]), xy, pidx, cell, (start, start + span)))
    return out
