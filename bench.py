#!/usr/bin/env python
"""Raster Join benchmark on GB300.

Headline (the metric "Gpoints/s joined at eps = 10 m", benchmark
configuration 3 at its eps = 10 m point): 2,000,000,000 points resident in
HBM (x, y float32: 16 GB), drawn from the configurations' generator (80 %
from 8 Gaussians with sigma 2 km, 20 % uniform, 40 x 40 km box); 260 Voronoi
neighbourhoods; the bounded raster join, count(), at eps = 10 m (the pixel
side, as the configurations quote it: a 4000 x 4000 canvas).  The reference's
own published point for this axis is the raster join at eps = 10 m over
335M taxi points (experiments/results-paper/scalability/taxi-in-memory.txt:1).

A step is one query answered from scratch: the polygon label map and its
block codes rebuilt (RJ_FLAG_NO_CACHE), one streaming pass over the points,
the per-polygon counts read back.  `value` is points joined per second with
the table resident; `e2e` adds, every step, the host->device copy of the
location column from pinned memory (rj_load_points) and the read-back.

In the same run:
  * the full 2B-point result is checked against an independent path of the
    library (the point canvas plus the polygon pass, RJ_FLAG_FORCE_CANVAS);
  * a 20M-point sample of the host generator is joined alone on the GPU and
    checked bit for bit against the oracle's raster join; the reference arm
    (--impl reference) times CPUJoin on the same sample;
  * extra keys: configuration 2 (hybrid / index joins with filters and avg,
    100M points), batched (configuration 4) and served (configuration 5).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--points N] [--no-config2] [--no-batched] [--no-served]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "raster-join_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

HEADLINE_POINTS = 2_000_000_000
HEADLINE_CELL = 10.0
HEADLINE_BYTES_PER_POINT = 8      # x, y float32: the only column a plain count reads
SAMPLE_POINTS = 20_000_000        # host-generated sample: oracle check and the CPU arms
POLY_SEED = 20261203
TABLE_SEED = 7
SAMPLE_SEED = 20261203
METRIC = "Gpoints/s joined at eps=10 m (raster count)"
WORKLOAD = ("config3 at eps 10 m: 2,000,000,000 points resident (x, y float32, 16 GB), 260 Voronoi "
            "neighbourhoods over a 40 x 40 km box, bounded raster join count(), cell 10 m (4000 x 4000 canvas)")

# configuration 2 (extra key)
C2_BYTES_PER_POINT = 24          # x, y, t, a, f1, f2: 4 bytes each, all read by the query
C2_WORKLOAD = ("config2: 100M pts (x,y,t,a,f1,f2), 260 Voronoi polys, 40x40 km, t in first 6 months & f1>2 & "
               "f2<8 & a<50, avg(a), grid 256")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--points", type=int, default=HEADLINE_POINTS, help="headline table size")
    ap.add_argument("--sample-points", type=int, default=SAMPLE_POINTS)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-config2", action="store_true")
    ap.add_argument("--c2-points", type=int, default=100_000_000)
    ap.add_argument("--c2-steps", type=int, default=50)
    ap.add_argument("--c2-shape", type=int, default=-1,
                    help="pin the lean pass's shape of the config-2 joins (rj_set_tuning; -1: autotuned)")
    ap.add_argument("--table-points", type=int, default=1_000_000_000,
                    help="resident table of the batched and served runs")
    ap.add_argument("--batch-queries", type=int, default=512)
    ap.add_argument("--served-requests", type=int, default=2000)
    ap.add_argument("--served-qps", type=float, default=500.0)
    ap.add_argument("--saturate-qps", type=float, default=5000.0,
                    help="offered rate of the saturation run of the served configuration (0: skip)")
    ap.add_argument("--saturate-requests", type=int, default=4000)
    ap.add_argument("--saturate-slots", type=int, default=2, help="serving slots of the saturation run")
    ap.add_argument("--saturate-clients", type=int, default=2,
                    help="client threads submitting the saturation run's requests (each uploads its polygons)")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--config3", action="store_true",
                    help="run all of configuration 3 instead (raster and error-bounds joins at eps 10 m and 1 m, "
                         "260 Voronoi cells and 2000 stars) and print its own line")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def headline_config(n, sample):
    """The workload both arms report (identical dicts, so their lines compare)."""
    return {"workload": WORKLOAD, "points": n, "polygons": 260, "cell_m": HEADLINE_CELL, "canvas": "4000x4000",
            "aggregation": "count", "sample_points": sample,
            "l2": "inputs (16 GB per step) larger than L2"}


def voronoi():
    from rasterjoin import synth
    return synth.voronoi_polygons(260, seed=POLY_SEED)


def host_sample(n):
    from rasterjoin import synth
    return synth.points(n, seed=SAMPLE_SEED)["xy"]


def make_workload(n, seed):
    from rasterjoin import synth
    pts = synth.points(n, seed=seed, columns=True)
    verts, pidx = synth.voronoi_polygons(260, seed=POLY_SEED)
    return pts, verts, pidx


def query_constraints():
    import rasterjoin as rj
    from rasterjoin import synth
    cons = [(4, rj.GT, 2), (5, rj.LT, 8), (3, rj.LT, 50.0)]
    trange = (2, synth.T0, synth.T0 + synth.YEAR // 2)
    return cons, trange


def fn_of(join):
    import rasterjoin as rj
    return {"hybrid": rj.HybridJoinFn, "index": rj.IndexJoinFn, "raster": rj.RasterJoinFn}[join]


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed loop runs."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu_id), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.time(), ln.strip()))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0=None, t1=None):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ts, ln in self.lines:
            if t0 is not None and (ts < t0 or ts > t1):
                continue
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(key, n):
    """DRAM bytes per launch of a point kernel from the committed ncu summary
    (bytes per point of a smaller capture), scaled to n points."""
    try:
        with open(os.path.join(ROOT, "profiles", "point_pass_traffic.json")) as fh:
            d = json.load(fh)
        return float(d[key]["dram_bytes_per_point"]) * n
    except Exception:
        return None


# ---------------------------------------------------------------------------
# CPU arms: the reference's own CPU join (CPUJoin, restated without Qt in the
# oracle: CPUJoin.cpp:62-122, GridIndexF.cpp:60-175,383-549), count, grid 1024
# as the reference's scripts run it (cpu-scalability.ps1:28).
def cpujoin_count(xy, verts, pidx, threads):
    """One CPUJoin run (grid built + join); returns (counts, wall s, join s, build s)."""
    import oracle
    t0 = time.perf_counter()
    c, _, tj, tb = oracle.cpujoin(xy, verts, pidx, 1024, nthreads=threads)
    return c, time.perf_counter() - t0, tj, tb


def cpu_baseline_headline(sample_xy, verts, pidx):
    threads = os.cpu_count() or 1
    _, wall, tj, tb = cpujoin_count(sample_xy, verts, pidx, threads)
    n1 = min(len(sample_xy), 2_000_000)
    _, wall1, tj1, tb1 = cpujoin_count(sample_xy[:n1], verts, pidx, 1)
    return {"value": len(sample_xy) / wall / 1e9, "unit": "Gpoints/s", "cores": threads, "kind": "port",
            "sample": "CPUJoin restatement (count, grid 1024 built %.2f s + join %.2f s) with %d threads over a "
                      "%d-point sample of the same generator (the sample the GPU also joins alone)"
                      % (tb, tj, threads, len(sample_xy)),
            "single_core": {"value": n1 / wall1 / 1e9, "unit": "Gpoints/s", "cores": 1,
                            "sample": "the first %d points of that sample, one thread (grid %.2f s + join %.2f s)"
                                      % (n1, tb1, tj1)}}


def metric_name(join=None):
    """The metric both arms report (same string, so their lines compare)."""
    return METRIC


def run_reference(args):
    """CPUJoin (the reference's CPU join, oracle restatement, all host threads)
    over the headline's sample; per step: grid build + join."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sample = min(args.sample_points, args.points)
    xy = host_sample(sample)
    verts, pidx = voronoi()
    threads = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        _, wall, _, _ = cpujoin_count(xy, verts, pidx, threads)
        if i >= args.warmup:
            times.append(wall)
    step = float(np.mean(times))
    value = sample / step / 1e9
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value, "unit": "Gpoints/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded; stands in for the NYC-taxi table)",
        "config": headline_config(args.points, sample),
        "parallelism": "cpu-threads",
        "cpu_baseline": {"value": value, "unit": "Gpoints/s", "cores": threads, "kind": "port",
                         "sample": "CPUJoin restatement (count, grid 1024 built each step + join) with %d threads "
                                   "over the %d-point sample of the headline's generator that the GPU arm also "
                                   "joins alone; a per-point rate of the same workload" % (threads, sample)},
        "e2e": {"value": value, "unit": "Gpoints/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# Batched and served configurations over one resident table generated on the
# device (1B points: x, y, t, a), reordered into time buckets.
def resident_table(rj, torch, n, seed, stream):
    from rasterjoin import workloads as W
    tab = W.device_table(n, seed)
    torch.cuda.synchronize()
    # rows per second of the year (exact row counts of any time window)
    secs = torch.bincount((tab["t"].to(torch.int64) - W.T0), minlength=W.YEAR)
    cum = torch.zeros(W.YEAR + 1, dtype=torch.int64, device="cuda")
    cum[1:] = torch.cumsum(secs, 0)
    cum = cum.cpu().numpy()
    del secs
    h = rj.GLHandler(stream=stream.cuda_stream)
    h.attachDevice([(1, rj.Location, tab["xy"].data_ptr()), (2, rj.Uint, tab["t"].data_ptr()),
                    (3, rj.Float, tab["a"].data_ptr())], n, 1)
    h.clusterPoints(2, 1024, 6)    # time buckets of 8.5 h, 625 m cells inside each (copies the table)
    del tab
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return h, cum


def window_rows(cum, t0, t1):
    from rasterjoin.synth import T0
    a = max(0, t0 - T0)
    b = min(len(cum) - 1, t1 - T0 + 1)
    return int(cum[b] - cum[a]) if b > a else 0


def make_raster_query(rj, cell, window, avg):
    q = rj.default_query()
    q.function_type = rj.RasterJoinFn
    q.cell_size = cell
    q.time_attrib, q.t_start, q.t_end = 2, int(window[0]), int(window[1])
    if avg:
        q.aggregation, q.aggr_attrib = rj.Avg, 3
    return q


def run_batched(rj, h, cum, n, nq):
    from rasterjoin import workloads as W
    work = W.batched_queries(nq, n)
    sets = [h.polyset(xy, p) for xy, p, _, _, _ in work]
    qs = [make_raster_query(rj, cell, win, avg) for _, _, cell, win, avg in work]
    pq = sum(window_rows(cum, *win) for _, _, _, win, _ in work)

    def timed(flags, reps):
        ms, out = [], None
        for _ in range(reps):
            t0 = time.perf_counter()
            out = h.execute_batch(qs, sets, flags=flags)
            ms.append((time.perf_counter() - t0) * 1e3)
        return float(np.median(ms)), out

    # warm-up: overlap checks of the new polygon sets, the lean passes' tuner
    # (on the lanes) and the fused pass's block-shape tuner
    h.execute_batch(qs, sets)
    h.execute_batch(qs, sets, flags=rj.BATCH_FUSE | rj.BATCH_AUTOTUNE)
    b_ms, (res, status, stats) = timed(0, 3)                      # the batch API's default route: lanes
    f_ms, (res_f, status_f, stats_f) = timed(rj.BATCH_FUSE, 2)    # fused pass for the small queries
    p_ms, (res_p, status_p, _) = timed(rj.BATCH_NO_FUSE, 2)       # plain: rj_execute in turn
    same = all(np.array_equal(a.count, b.count) and np.array_equal(a.sum, b.sum) and
               np.array_equal(a.count, c.count) and np.array_equal(a.sum, c.sum)
               for a, b, c in zip(res, res_f, res_p))
    for s in sets:
        s.close()
    return {
        "workload": "%d raster queries over a %d-point resident table; per query 1-5000 star polygons "
                    "(4-2000 vertices), eps log-uniform 1-1000 m, time window of 1e4-5e8 points, "
                    "count or avg" % (nq, n),
        "point_queries": pq, "batched_ms": b_ms, "plain_ms": p_ms, "speedup": p_ms / b_ms,
        "batched_gpoints_s": pq / b_ms / 1e6, "plain_gpoints_s": pq / p_ms / 1e6,
        "route": "every query on the lanes: rj_execute's device path on 8 streams with their own scratch, "
                 "queued without host waits, one wait per batch",
        "kernel_launches": stats["kernel_launches"],
        "fused_variant": {"ms": f_ms, "speedup": p_ms / f_ms, "fused_queries": stats_f["fused"],
                          "rows_read": stats_f["rows_read"], "segments": stats_f["segments"],
                          "point_pass_ms": stats_f["point_ms"], "polygon_side_ms": stats_f["poly_ms"],
                          "canvas_reduce_ms": stats_f["reduce_ms"], "kernel_launches": stats_f["kernel_launches"],
                          "shape": {"threads": stats_f["threads"], "rows_per_item": stats_f["rows_per_item"],
                                    "variant": "direct" if stats_f["direct"] else "staged"},
                          "route": "queries under 2^22 rows in one fused point pass per wave, the others on "
                                   "the lanes (RJ_BATCH_FUSE)"},
        "status_ok": bool((status == 0).all() and (status_f == 0).all() and (status_p == 0).all()),
        "same_result": bool(same),
        "plain": "each query through rj_execute in turn (one query per launch sequence, RJ_BATCH_NO_FUSE)",
    }


def run_served(rj, h, cum, n, nreq, qps, seed=20261205, slots=2, clients=1):
    from rasterjoin import workloads as W
    reqs = W.served_requests(nreq, qps, seed=seed)
    rows = [window_rows(cum, *r[4]) for r in reqs]
    qs = [make_raster_query(rj, cell, win, False) for _, _, _, cell, win in reqs]
    # ---- plain: one request at a time through rj_execute, FIFO
    service = []
    for (arr, xy, p, cell, win), q in zip(reqs, qs):
        t0 = time.perf_counter()
        ps = h.polyset(xy, p)
        h.usePolySet(ps)
        h.execute(rj.RasterJoinFn, query=q)
        service.append(time.perf_counter() - t0)
        h.usePolySet(None)
        ps.close()
    arrivals = np.array([r[0] for r in reqs])
    done = np.zeros(nreq)
    free_at = 0.0
    for i in range(nreq):
        start = max(arrivals[i], free_at)
        done[i] = start + service[i]
        free_at = done[i]
    plain_lat = (done - arrivals) * 1e3
    # ---- served: requests submitted at their arrival times
    srv = h.server(slots=slots, canvas_mb=16384, max_batch=64)
    tickets = [None] * nreq
    arrive_ms = np.zeros(nreq)
    live = []
    base = time.monotonic()

    def submitter(k):
        # client k submits requests k, k + clients, ... at their arrival times
        for i in range(k, nreq, clients):
            arr, xy, p, cell, win = reqs[i]
            now = time.monotonic() - base
            if arr > now:
                time.sleep(arr - now)
            arrive_ms[i] = time.monotonic() * 1e3
            ps = h.polyset(xy, p)            # the request's polygons go to the device on arrival
            live.append(ps)
            tickets[i] = srv.submit(qs[i], ps)

    ths = [threading.Thread(target=submitter, args=(k,)) for k in range(clients)]
    for th in ths:
        th.start()
    lat, sizes, last_done = [], [], 0.0
    for i in range(nreq):
        while tickets[i] is None:
            time.sleep(0.0002)
        r, info = srv.poll(tickets[i], -1)
        lat.append(info["done_ms"] - arrive_ms[i])
        sizes.append(info["batch_size"])
        last_done = max(last_done, info["done_ms"])
    for th in ths:
        th.join()
    srv.close()
    for ps in live:
        ps.close()
    span_s = (last_done - arrive_ms.min()) / 1e3
    lat = np.array(lat)
    pct = lambda a, q: float(np.percentile(a, q))
    return {
        "workload": "Poisson arrivals at %g qps, %d requests over a %d-point resident table; per request "
                    "1-50 star polygons (8-300 vertices, radius 200 m-10 km), eps in {1,10,100,1000} m, "
                    "time window 1 h-30 days, count" % (qps, nreq, n),
        "p50_ms": pct(lat, 50), "p95_ms": pct(lat, 95), "p99_ms": pct(lat, 99),
        "achieved_qps": nreq / span_s, "gpoints_s": sum(rows) / span_s / 1e9,
        "mean_batch": float(np.mean(sizes)),
        "plain": {"p50_ms": pct(plain_lat, 50), "p95_ms": pct(plain_lat, 95), "p99_ms": pct(plain_lat, 99),
                  "mean_service_ms": float(np.mean(service)) * 1e3,
                  "max_qps": 1.0 / float(np.mean(service)),
                  "method": "each request alone through rj_execute (polygons uploaded, join, results read); "
                            "latency from a FIFO queue over the same arrival times"},
        "latency": "arrival (before the polygon upload) to results in host memory",
        "slots": slots, "clients": clients,
    }


# ---------------------------------------------------------------------------
def clocks_around(sampler, t0, t1):
    timed = sampler.summary(t0, t1)
    c = dict(sampler.summary())
    c["samples_in_timed_region"] = timed["samples"]
    if timed["samples"]:
        c["sm_mhz_timed_region"] = timed["sm_mhz"]
    return c


def run_headline(args, rj, torch, local, world):
    """The headline line: eps = 10 m raster count over the resident 2B table."""
    from rasterjoin import workloads as W
    n = args.points
    verts, pidx = voronoi()
    P = len(pidx) - 1
    tab = W.device_table(n, TABLE_SEED + dist_env()[0])
    del tab["t"], tab["a"]
    xy_dev = tab["xy"]
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    stream = torch.cuda.Stream()
    h = rj.GLHandler(device=local, stream=stream.cuda_stream)
    h.attachDevice([(1, rj.Location, xy_dev.data_ptr())], n, 1)
    ps = h.polyset(verts, pidx)
    h.usePolySet(ps)
    q = rj.default_query()
    q.function_type = rj.RasterJoinFn
    q.cell_size = HEADLINE_CELL
    q.flags = rj.FLAG_NO_CACHE | rj.FLAG_PHASE_TIMING

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for _ in range(max(3, args.warmup)):          # the first also autotunes the count kernel
        h.execute(rj.RasterJoinFn, query=q)
    torch.cuda.synchronize()
    shape = (h.getTuning(rj.TUNE_COUNT_SHAPE), h.getTuning(rj.TUNE_COUNT_BLOCK_SHIFT))
    try:
        dev_uuid = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        dev_uuid = local
    sampler = ClockSampler(dev_uuid)
    sampler.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    pt_ms, launches = [], []
    barrier()
    torch.cuda.synchronize()
    t_wall0 = time.time()
    for i in range(args.steps):
        starts[i].record(stream)
        h.execute(rj.RasterJoinFn, query=q)
        ends[i].record(stream)
        t = h.timings()
        pt_ms.append(t["pt_render_ms"])
        launches.append(t["kernel_launches"])
    torch.cuda.synchronize()
    barrier()
    t_wall1 = time.time()
    total_ms = sum(s_.elapsed_time(e_) for s_, e_ in zip(starts, ends))
    if world > 1:
        tt = torch.tensor([total_ms], device="cuda")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(tt.item())
    probe_end = time.time() + max(0.0, 1.5 - (t_wall1 - t_wall0))
    while time.time() < probe_end:
        h.execute(rj.RasterJoinFn, query=q)
    torch.cuda.synchronize()
    sampler.stop()
    clocks = clocks_around(sampler, t_wall0, t_wall1)
    res = h.last
    ms_per_step = total_ms / args.steps
    value = world * n / (ms_per_step / 1e3) / 1e9

    # ---- the same step replayed as a prepared query (rj_prepare: one CUDA graph) ----
    plan = h.prepare(rj.RasterJoinFn, query=q)
    for _ in range(3):
        plan.execute()
    torch.cuda.synchronize()
    pe0, pe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nrep = max(5, args.steps // 4)
    pe0.record(stream)
    for _ in range(nrep):
        rp = plan.execute()
    pe1.record(stream)
    torch.cuda.synchronize()
    prep_ms = pe0.elapsed_time(pe1) / nrep
    prepared = {"ms_per_step": prep_ms, "gpoints_s": world * n / prep_ms / 1e6,
                "same_result": bool(np.array_equal(rp.count, res.count)),
                "method": "rj_prepare captures the step's device work (label map, block codes, count pass, "
                          "result copies) as a CUDA graph; rj_execute_prepared replays it"}
    plan.close()

    # ---- the full result against an independent path: point canvas + polygon pass ----
    qc = rj.default_query()
    qc.function_type = rj.RasterJoinFn
    qc.cell_size = HEADLINE_CELL
    qc.flags = rj.FLAG_FORCE_CANVAS
    canvas_equal = bool(np.array_equal(h.execute(rj.RasterJoinFn, query=qc).count, res.count))

    # ---- end to end: the location column from pinned host memory every step ----
    # Three ways through the public API, each with every byte of the table
    # crossing the host link inside the timed step:
    #   load:     rj_load_points (one copy of the column) + rj_execute;
    #   streamed: rj_attach_points_host once (host pointers, nothing copied),
    #             then every rj_execute streams the column in chunks through
    #             two device buffers, copying chunk k+1 while chunk k is joined
    #             (the reference's memory passes, GLFunction.cpp:330-337);
    #   mapped:   rj_attach_points_mapped once, then every rj_execute reads
    #             the pinned column in place over the link.
    pinned = torch.empty((n, 2), dtype=torch.float32, pin_memory=True)
    pinned.copy_(xy_dev)
    host_xy = pinned.numpy()
    del tab, xy_dev
    h.usePolySet(None)
    ps.close()
    h.close()
    torch.cuda.empty_cache()

    def e2e_run(he, step):
        times = []
        out = None
        for i in range(args.e2e_steps + 2):
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = step(he)
            torch.cuda.synchronize()
            if i >= 2:
                times.append(time.perf_counter() - t0)
        t = float(np.mean(times))
        if world > 1:
            tt = torch.tensor([t], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            t = float(tt.item())
        return t, out

    e2e = {}
    he = rj.GLHandler(device=local, stream=stream.cuda_stream)
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, host_xy)
    dh.setPolygons(verts, pidx)
    he.setDataHandler(dh)
    he.setCellSize(HEADLINE_CELL)
    he.flags = rj.FLAG_NO_CACHE

    def load_step(hh):
        hh.upload(force=True)                 # H2D of the location column (rj_load_points)
        return hh.execute(rj.RasterJoinFn)    # join + D2H of the counts

    t_load, r_load = e2e_run(he, load_step)
    e2e["load"] = {"gpoints_s": world * n / t_load / 1e9, "ms": t_load * 1e3,
                   "same_result": bool(np.array_equal(r_load.count, res.count))}
    he.close()
    hs2 = rj.GLHandler(device=local, stream=stream.cuda_stream)
    hs2.attachHost([(1, rj.Location, host_xy)], n, 1)
    qs = rj.default_query()
    qs.function_type = rj.RasterJoinFn
    qs.cell_size = HEADLINE_CELL
    qs.flags = rj.FLAG_NO_CACHE
    pset = hs2.polyset(verts, pidx)
    hs2.usePolySet(pset)
    t_str, r_str = e2e_run(hs2, lambda hh: hh.execute(rj.RasterJoinFn, query=qs))
    tm = hs2.timings()
    e2e["streamed"] = {"gpoints_s": world * n / t_str / 1e9, "ms": t_str * 1e3, "passes": tm["no_pt_passes"],
                       "copy_ms": tm["pt_mem_ms"], "same_result": bool(np.array_equal(r_str.count, res.count))}
    hs2.usePolySet(None)
    pset.close()
    hs2.close()
    # mapped: rj_attach_points_mapped once (the pinned column's device
    # address, nothing copied); every rj_execute's point pass reads the column
    # over the host link (NVLink-C2C) in place
    hs3 = rj.GLHandler(device=local, stream=stream.cuda_stream)
    hs3.attachMapped([(1, rj.Location, host_xy)], n, 1)
    pset = hs3.polyset(verts, pidx)
    hs3.usePolySet(pset)
    t_map, r_map = e2e_run(hs3, lambda hh: hh.execute(rj.RasterJoinFn, query=qs))
    e2e["mapped"] = {"gpoints_s": world * n / t_map / 1e9, "ms": t_map * 1e3,
                     "link_gbs": n * HEADLINE_BYTES_PER_POINT / t_map / 1e9,
                     "same_result": bool(np.array_equal(r_map.count, res.count))}
    hs3.usePolySet(None)
    pset.close()
    hs3.close()
    best = min(("load", t_load), ("streamed", t_str), ("mapped", t_map), key=lambda kv: kv[1])[0]
    e2e_s = min(t_str, t_load, t_map)
    e2e_same = e2e["load"]["same_result"] and e2e["streamed"]["same_result"] and e2e["mapped"]["same_result"]
    del pinned, host_xy, dh
    torch.cuda.empty_cache()

    # ---- the sample: joined alone on the GPU and checked against the oracle ----
    import oracle
    sample = min(args.sample_points, n)
    sxy = host_sample(sample)
    hs = rj.GLHandler(device=local, stream=stream.cuda_stream)
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, sxy)
    dh.setPolygons(verts, pidx)
    hs.setDataHandler(dh)
    hs.setCellSize(HEADLINE_CELL)
    hs.flags = rj.FLAG_NO_CACHE
    for _ in range(3):
        rs = hs.execute(rj.RasterJoinFn)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(10):
        rs = hs.execute(rj.RasterJoinFn)
    e1.record(stream)
    torch.cuda.synchronize()
    sample_ms = e0.elapsed_time(e1) / 10
    hs.close()
    want = oracle.raster_join(sxy, verts, pidx, HEADLINE_CELL)[0]
    oracle_equal = bool(np.array_equal(rs.count, want))

    peak, peak_kind = measured_peaks()
    mean_pt = float(np.mean(pt_ms))
    achieved = (n * HEADLINE_BYTES_PER_POINT / 1e9) / (mean_pt / 1e3) if mean_pt > 0 else None
    line = {
        "metric": METRIC,
        "value": value, "unit": "Gpoints/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded; stands in for the NYC-taxi table)",
        "config": headline_config(n, sample),
        "parallelism": "replicas" if world > 1 else "single-gpu",
        "e2e": {"value": world * n / e2e_s / 1e9, "unit": "Gpoints/s",
                "h2d_bytes_per_step": n * HEADLINE_BYTES_PER_POINT, "d2h_bytes_per_step": P * (8 + 8 + 12),
                "same_result": e2e_same, "method": best, "variants": e2e,
                "note": "the location column (16 GB) crosses the host link every step; 'load' = rj_load_points "
                        "+ rj_execute, 'streamed' = rj_attach_points_host then rj_execute copying chunk k+1 "
                        "while chunk k is joined, 'mapped' = rj_attach_points_mapped then rj_execute reading "
                        "the pinned column in place over the link; counts read back every step"},
        "gpu_launches": int(sum(launches)),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": profiled_traffic("raster_count", n),
                     "kernel": "k_label_count (shape %d, block codes 2^%d px)" % shape, "kernel_ms": mean_pt,
                     "algorithmic_bytes_per_launch": n * HEADLINE_BYTES_PER_POINT, "peak_kind": peak_kind},
        "clocks": clocks,
        "checks": {"full_table_vs_canvas_path": canvas_equal,
                   "sample_vs_oracle": oracle_equal,
                   "sample": "%d points of the host generator, joined alone on the GPU, against the oracle's "
                             "raster join (bit-exact counts)" % sample},
        "sample": {"points": sample, "gpu_gpoints_s": sample / sample_ms / 1e6, "gpu_ms": sample_ms},
        "prepared": prepared,
    }
    return line, (sxy, verts, pidx)


def run_config2(args, rj, torch, local, join, pts, verts, pidx):
    """Configuration 2 (hybrid or index join, filters, time range, avg(a)) on
    100M host-generated points; returns an extra-key dict and the result."""
    n = len(pts["xy"])
    stream = torch.cuda.Stream()
    h = rj.GLHandler(device=local, stream=stream.cuda_stream)
    dh = rj.DataHandler()
    dh.add_column(1, rj.Location, pts["xy"])
    dh.add_column(2, rj.Uint, pts["t"])
    dh.add_column(3, rj.Float, pts["a"])
    dh.add_column(4, rj.Int, pts["f1"])
    dh.add_column(5, rj.Int, pts["f2"])
    dh.setPolygons(verts, pidx)
    cons, trange = query_constraints()
    dh.setQueryConstraints(cons)
    dh.setTimeRange(*trange)
    dh.setAggregation(rj.Avg, 3)
    h.setDataHandler(dh)
    h.setAccuracyDistance(100.0)
    h.setPolyIndexResolution(256)
    h.flags = rj.FLAG_NO_CACHE | rj.FLAG_PHASE_TIMING
    fn = fn_of(join)
    h.upload()
    if args.c2_shape >= 0:
        h.setTuning(rj.TUNE_COUNT_SHAPE, args.c2_shape)
    q = h.make_query(fn)
    out = {}
    for _ in range(3):
        h.execute(fn, query=q)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pt = []
    e0.record(stream)
    for _ in range(args.c2_steps):
        h.execute(fn, query=q)
        pt.append(h.timings()["pt_render_ms"])
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.c2_steps
    res = h.last
    shape = h.getTuning(rj.TUNE_COUNT_SHAPE)              # the lean pass's autotuned shape (-1: generic pass)
    # one more (untimed) run counting the exact edge tests of the point pass
    qe = h.make_query(fn)
    qe.flags |= rj.FLAG_COUNT_EDGE_TESTS
    h.execute(fn, query=qe)
    edge_tests = int(h.timings()["edge_tests"])
    h.close()
    peak, _ = measured_peaks()
    mean_pt = float(np.mean(pt))
    achieved = (n * C2_BYTES_PER_POINT / 1e9) / (mean_pt / 1e3)
    out = {"workload": C2_WORKLOAD, "join": join, "gpoints_s": n / ms / 1e6, "ms_per_step": ms,
           "point_pass_ms": mean_pt, "lean_shape": shape,
           "edge_tests": {"count": edge_tests, "per_point": edge_tests / n,
                          "per_s": edge_tests / (mean_pt / 1e3),
                          "note": "exact crossing tests of the points near polygon edges (classified grid cells "
                                  "with candidate lists); counted in a separate run, rate over the timed point pass"},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "traffic": profiled_traffic(join, n)}}
    return out, res


def run_gb300(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    import __graft_entry__
    __graft_entry__.build()
    import rasterjoin as rj

    line, (sxy, verts, pidx) = run_headline(args, rj, torch, local, world)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_headline(sxy, verts, pidx)
    del sxy
    if rank == 0 and world == 1 and not args.no_config2:
        import oracle
        extra = {}
        pts, verts2, pidx2 = make_workload(args.c2_points, seed=20261203)
        results = {}
        for join in ("hybrid", "index"):
            extra[join], results[join] = run_config2(args, rj, torch, local, join, pts, verts2, pidx2)
        # the hybrid and index counts against CPUJoin's exact counts on the same 100M points
        cols = oracle.Columns({2: (oracle.Uint, pts["t"]), 3: (oracle.Float, pts["a"]),
                               4: (oracle.Int, pts["f1"]), 5: (oracle.Int, pts["f2"])})
        cons, trange = query_constraints()
        f = cols.filt(cons, aggr_attrib=3, time_range=trange)
        t0 = time.perf_counter()
        c, s_, _, _ = oracle.cpujoin(pts["xy"], verts2, pidx2, 256, f=f)
        rel = lambda r: float(np.max(np.abs(r.sum - s_) / np.maximum(np.abs(s_), 1e-30)))
        extra["check"] = {"hybrid_counts_vs_cpujoin": bool(np.array_equal(results["hybrid"].count, c)),
                          "index_counts_vs_cpujoin": bool(np.array_equal(results["index"].count, c)),
                          "hybrid_sums_max_rel_err": rel(results["hybrid"]),
                          "index_sums_max_rel_err": rel(results["index"]),
                          "cpujoin_s": time.perf_counter() - t0,
                          "oracle": "CPUJoin restatement (grid 256) with the config-2 filters and avg, fp64 sums"}
        line["config2"] = extra
        del pts
    if rank == 0 and world == 1 and not (args.no_batched and args.no_served):
        stream2 = torch.cuda.Stream()
        h2, cum = resident_table(rj, torch, args.table_points, 20261206, stream2)
        if not args.no_batched:
            line["batched"] = run_batched(rj, h2, cum, args.table_points, args.batch_queries)
        if not args.no_served:
            line["served"] = run_served(rj, h2, cum, args.table_points, args.served_requests, args.served_qps)
            if args.saturate_qps > 0:
                sat = run_served(rj, h2, cum, args.table_points, args.saturate_requests, args.saturate_qps,
                                 seed=20261207, slots=args.saturate_slots, clients=args.saturate_clients)
                line["served_saturated"] = {
                    "offered_qps": args.saturate_qps, "achieved_qps": sat["achieved_qps"],
                    "plain_max_qps": sat["plain"]["max_qps"],
                    "throughput_vs_plain": sat["achieved_qps"] / sat["plain"]["max_qps"],
                    "p50_ms": sat["p50_ms"], "p99_ms": sat["p99_ms"], "mean_batch": sat["mean_batch"],
                    "gpoints_s": sat["gpoints_s"],
                    "plain_p99_ms": sat["plain"]["p99_ms"], "slots": sat["slots"], "clients": sat["clients"],
                    "note": "requests offered faster than either path serves them; achieved_qps is the "
                            "served path's throughput with `clients` threads submitting (each uploads its "
                            "requests' polygons), plain_max_qps = 1 / mean single-request service time "
                            "(polygon upload included)"}
        h2.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_config3(args):
    """Configuration 3: 2B points resident (x, y generated on the device),
    two polygon sets, raster and error-bounds joins at eps 10 m and 1 m."""
    import torch
    import __graft_entry__
    __graft_entry__.build()
    import rasterjoin as rj
    from rasterjoin import synth, workloads as W
    n = args.points if args.points != 100_000_000 else 2_000_000_000
    tab = W.device_table(n, 7)
    torch.cuda.synchronize()
    h = rj.GLHandler()
    h.attachDevice([(1, rj.Location, tab["xy"].data_ptr())], n, 1)
    sets = {"voronoi260": synth.voronoi_polygons(260, seed=20261203),
            "stars2000": synth.star_polygons(2000, seed=20261203, vmin=20, vmax=500, rmin=200, rmax=2000)}
    out = []
    for name, (v, p) in sets.items():
        ps = h.polyset(v, p)
        h.usePolySet(ps)
        for eps in (10.0, 1.0):
            forms = [(rj.RasterJoinFn, 0), (rj.RasterJoinBoundFn, 0)]
            if eps == 1.0:
                # both canvas forms of the 40000 x 40000 canvas: flat (a label
                # map or count canvas per pixel) and tiered (16 x 16 blocks)
                forms += [(rj.RasterJoinFn, rj.FLAG_FLAT_CANVAS), (rj.RasterJoinFn, rj.FLAG_TIERED_CANVAS),
                          (rj.RasterJoinBoundFn, rj.FLAG_FLAT_CANVAS)]
            for fn, form in forms:
                q = rj.default_query()
                q.function_type = fn
                q.cell_size = eps
                q.flags |= rj.FLAG_PHASE_TIMING | form   # per-phase CUDA events (point pass, polygon side)
                h.execute(fn, query=q)                 # warm-up (builds the polygon structures once)
                ms = []
                for _ in range(max(1, args.steps)):
                    t0 = time.perf_counter()
                    r = h.execute(fn, query=q)
                    ms.append((time.perf_counter() - t0) * 1e3)
                P = len(p) - 1
                tm = h.timings()
                rec = {"polygons": name, "eps_m": eps, "join": "raster" if fn == rj.RasterJoinFn else "error-bounds",
                       "canvas": {0: "default", rj.FLAG_FLAT_CANVAS: "flat", rj.FLAG_TIERED_CANVAS: "tiered"}[form],
                       "ms": float(np.median(ms)), "gpoints_s": n / float(np.median(ms)) / 1e6,
                       "total_count": int(r.count.sum()),
                       "point_pass_ms": tm["pt_render_ms"], "polygon_side_ms": tm["poly_render_ms"],
                       "kernel_launches": tm["kernel_launches"]}
                if fn == rj.RasterJoinBoundFn:
                    b = r.bounds.astype(np.int64)
                    rec["mean_hard_range"] = float(np.mean(b[2 * P:3 * P] + b[3 * P:]))
                    if form == 0:
                        eb_default = b
                    else:                              # the flat canvas's bounds against the default form's
                        rec["bounds_equal_default"] = bool(np.array_equal(b, eb_default))
                out.append(rec)
        h.usePolySet(None)
        ps.close()
    h.close()
    print(json.dumps({"metric": "config 3: Gpoints/s joined over %d resident points" % n, "unit": "Gpoints/s",
                      "n_gpus": 1, "data": "synthetic, generated on the device", "results": out}), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config3:
        return run_config3(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
