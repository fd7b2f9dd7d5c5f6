"""GRG matmul benchmark (edge x K updates per second, and the HBM roofline of the sweep kernel).

Workload (default): the seeded window-tree GRG with N=200,000 haplotypes and M=1,000,000 variants
(seed 42, 100-variant windows), plain single-request matmul in both directions for
K in {1, 8, 32, 64} and dtypes int32 (0/1 genotype counts), float32 (compensated) and float64
(N(0,1) inputs).  One step = those 24 matmuls.  `value` = sum of E*K over the step's matmuls /
device time, inputs resident in HBM; `e2e` = the same through the host-buffer C-ABI path, with
every input copied in and every output copied back inside the timed region.

    python bench.py [--gpus 1] [--steps 5] [--warmup 3] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

DOWN, UP = 1, 2
METRIC = "GRG matmul edge*K updates/s"
UNIT = "edge*K/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="grgx", choices=["grgx", "reference"])
    ap.add_argument("--samples", type=int, default=200_000)
    ap.add_argument("--mutations", type=int, default=1_000_000)
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--ks", default="1,8,32,64")
    ap.add_argument("--dtypes", default="int32,float32,float64")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the full-size comparison with the oracle")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end pass")
    ap.add_argument("--e2e-streams", type=int, default=4,
                    help="CUDA streams the end-to-end pass spreads the step's calls over")
    ap.add_argument("--only", default=None,
                    help="restrict the step to dtype:K:dir entries, e.g. float32:64:UP,int32:1:DOWN")
    ap.add_argument("--breakdown", action="store_true",
                    help="print per-matmul device times (3 calls each, CUDA events) instead of the JSON line")
    ap.add_argument("--no-serve", action="store_true", help="skip the batched and served measurements")
    ap.add_argument("--batch-requests", type=int, default=256, help="requests in the batched measurement")
    ap.add_argument("--serve-rates", default="50,200,500,1000,2000", help="Poisson arrival rates (requests/s)")
    ap.add_argument("--narrow-rates", default="10,100,1000",
                    help="Poisson arrival rates (requests/s) of the narrow (K <= 8) served mix")
    ap.add_argument("--serve-seconds", type=float, default=4.0, help="longest arrival window of a served run")
    ap.add_argument("--serve-requests", type=int, default=96, help="most arrivals in a served run")
    ap.add_argument("--no-large", action="store_true", help="skip the large-graph measurement")
    ap.add_argument("--no-autotune", action="store_true", help="run the default launch shapes (no tuning pass)")
    ap.add_argument("--no-load", action="store_true", help="skip the .grg save / cold-load measurement")
    ap.add_argument("--large-samples", type=int, default=1_000_000)
    ap.add_argument("--large-mutations", type=int, default=300_000)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(args):
    if args.only:
        out = []
        for item in args.only.split(","):
            dt, K, d = item.split(":")
            out.append((np.dtype(dt), int(K), UP if d.upper() == "UP" else DOWN))
        return out
    ks = [int(k) for k in args.ks.split(",")]
    dts = [np.dtype(d) for d in args.dtypes.split(",")]
    return [(dt, K, d) for dt in dts for K in ks for d in (UP, DOWN)]


def workload_name(args, combos):
    return (f"plain matmul, window-tree GRG N={args.samples} M={args.mutations} seed={args.seed}, "
            + (f"K in {{{args.ks}}}, UP+DOWN, {args.dtypes}" if not args.only else args.only)
            + f"; {len(combos)} matmuls per step")


def make_inputs(rng, combos, N, M):
    out = []
    for dt, K, d in combos:
        cols = N if d == UP else M
        if dt.kind == "f":
            V = rng.standard_normal((K, cols)).astype(dt)
        else:
            V = rng.integers(0, 2, size=(K, cols)).astype(dt)
        out.append(V)
    return out


def graph_stats(g):
    info = g.info()
    return {"nodes": info["num_nodes"], "edges": info["num_edges"], "samples": info["num_samples"],
            "mutations": info["num_mutations"], "levels": info["num_levels"]}


def alg_bytes(stats, K, s, direction):
    """Algorithmic bytes of one traversal: edge ids once, node offsets, one operand row per edge,
    each node accumulator written once, plus the seed/gather I/O."""
    E, n, N, M = stats["edges"], stats["nodes"], stats["samples"], stats["mutations"]
    cols_in, cols_out = (N, M) if direction == UP else (M, N)
    return E * 4 + (n + 1) * 8 + E * K * s + n * K * s + K * (cols_in + cols_out) * s + 8 * M


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, device: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={device}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) >= 9 for i in range(4) if "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def workload_config(args, combos, stats):
    """The `config` object of both arms' lines: the workload and the graph it runs on."""
    return {"workload": workload_name(args, combos),
            "graph": {k: stats[k] for k in ("samples", "mutations", "nodes", "edges")},
            "l2": "inputs larger than L2 (the 8 GB edge CSR is streamed by every traversal)"}


class CpuSampler:
    """The reference CPU matmul (the oracle's restatement of GRG::matrixMultiplication,
    grg.h:1341-1517) run the way the reference runs on many cores: the graph cut into one
    window-aligned mutation range per core, each range's sub-graph (every sample and the nodes
    below the range, what saveGRGSubset keeps) multiplied on its own thread, DOWN partial outputs
    summed (test/endtoend/test_matmul.py:264-325).  Every product covers the whole graph."""

    def __init__(self, og, combos, inputs, threads):
        import oracle

        self.combos, self.inputs = combos, inputs
        self.threads = threads
        self.edges = og.num_edges
        t0 = time.perf_counter()
        self.sh = oracle.Shards(og, threads, build_threads=threads, align=100)
        self.build_s = time.perf_counter() - t0

    def run(self, idxs):
        """The combos `idxs` over the whole graph: (edge*K units, seconds, DOWN partial-sum seconds)."""
        units, secs, red = 0, 0.0, 0.0
        for i in idxs:
            (dt, K, d), V = self.combos[i], self.inputs[i]
            t0 = time.perf_counter()
            self.sh.matmul(V, d)
            secs += time.perf_counter() - t0
            red += self.sh.last_reduce_s
            units += self.edges * K
        return units, secs, red

    def one_core(self):
        """One thread on one range (the reference as shipped: a single-threaded call), for every
        combo with K in {1, 8}."""
        out = {}
        e0 = self.sh.edges(0, 1)
        for (dt, K, d), V in zip(self.combos, self.inputs):
            if K not in (1, 8):
                continue
            t0 = time.perf_counter()
            self.sh.matmul(V, d, first=0, count=1)
            out[f"{dt.name}:{K}:{'UP' if d == UP else 'DOWN'}"] = e0 * K / (time.perf_counter() - t0)
        return out


def step_plan(n_combos, steps):
    """Combo indices per timed step: every combo exactly once over the steps when steps <= n
    (consecutive groups), one combo per step, cycling, when steps > n."""
    if steps >= n_combos:
        return [[s % n_combos] for s in range(steps)]
    return [list(range(n_combos * s // steps, n_combos * (s + 1) // steps)) for s in range(steps)]


def cpu_baseline(args, combos, smp):
    """The CPU reference on the machine's cores over a bounded sample of the workload: the K in {1, 8}
    combos, each over the whole graph."""
    idxs = [i for i, (_, K, _) in enumerate(combos) if K in (1, 8)] or [0]
    units, secs, _ = smp.run(idxs)
    return {"value": units / secs, "unit": UNIT, "cores": smp.threads, "kind": "port",
            "sample": f"the {len(idxs)} K in {{1, 8}} combos of the workload, each over the whole benchmark graph "
                      f"(one window-aligned mutation range per core); {units:.3g} edge*K in {secs:.1f} s"}


def batched_vs_plain(gx, torch, g, E, rng, n_req, kmax, label, std_every=0, err_sample=0):
    """Plain one-request-per-call against matmul_batch on the same requests (device inputs,
    float32 compensated).  Every `std_every`-th request is a standardized product (plain path:
    matmul_standardized).  `err_sample` requests are also computed in float64 and the batched
    float32 results' error is stated against them, relative to the magnitude of the summed terms."""
    N, M = g.num_samples, g.num_mutations
    reqs = []
    for i in range(n_req):
        K = int(rng.integers(1, kmax + 1))
        d = UP if rng.random() < 0.5 else DOWN
        st = bool(std_every) and i % std_every == 0
        reqs.append((torch.from_numpy(rng.standard_normal((K, N if d == UP else M)).astype(np.float32)).cuda(), d, st))
    units = sum(E * V.shape[0] for V, _, _ in reqs)

    def plain(V, d, st):
        return gx.matmul_standardized(g, V, d) if st else gx.matmul(g, V, d)

    for _ in range(2):  # warm both paths (pool, plans, allele frequencies)
        plain(*reqs[0])
        gx.matmul_batch(g, reqs[:2])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in reqs:
        plain(*r)
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    # the batch is one call: the median of three runs (the plain side averages 256 calls)
    times = []
    outs = None
    for _ in range(3):
        outs = None  # the previous run's outputs go before the next run allocates its own
        t0 = time.perf_counter()
        outs = gx.matmul_batch(g, reqs)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    t_batch = sorted(times)[1]
    res = {"mix": label, "requests": n_req, "standardized_requests": sum(r[2] for r in reqs),
           "columns": int(sum(V.shape[0] for V, _, _ in reqs)), "plain_edgeK_per_s": units / t_plain,
           "batched_edgeK_per_s": units / t_batch, "speedup": t_plain / t_batch,
           "batched_runs_s": [round(t, 4) for t in times]}
    if err_sample:
        worst = {"plain": 0.0, "standardized": 0.0}
        picks = [i for i in range(n_req) if reqs[i][2]][:err_sample // 2] + \
                [i for i in range(n_req) if not reqs[i][2]][:err_sample - err_sample // 2]
        counts = None
        for i in picks:
            V, d, st = reqs[i]
            V64 = V.double()
            if st:
                if counts is None:
                    counts = gx.matmul(g, torch.ones((1, N), dtype=torch.int32, device="cuda"), UP)[0].double()
                ref = gx.matmul_standardized(g, V64, d)
                mu = counts / N
                var = mu * (1 - mu)
                inv = torch.where(var > 0, 1 / torch.sqrt(torch.where(var > 0, var, torch.ones_like(var))),
                                  torch.zeros_like(var))
                if d == UP:
                    scale = (gx.matmul(g, V64.abs(), UP) + V64.sum(dim=1, keepdim=True).abs() * mu[None, :]) * inv[None, :]
                else:
                    W = V64 * inv[None, :]
                    scale = gx.matmul(g, W.abs(), DOWN) + (W @ mu).abs()[:, None]
            else:
                ref = gx.matmul(g, V64, d)
                scale = gx.matmul(g, V64.abs(), d)
            e = ((outs[i].double() - ref).abs() / scale.clamp_min(1e-300)).max().item()
            key = "standardized" if st else "plain"
            worst[key] = max(worst[key], e)
        res["f32_max_err_vs_f64"] = {"requests_checked": len(picks), **worst,
                                     "relative_to": "sum of |terms| per output (|V| X, plus the mean "
                                                    "correction for standardized)"}
    return res


def served(gx, graphs, rate, seconds, max_requests, rng, kmax=256):
    """Poisson arrivals over resident graphs (K log-uniform in [1, kmax], UP/DOWN and int32/float32
    mixed), served by the continuous-batching server; against the same requests one per call.
    The arrival window is `seconds`, cut short after `max_requests` arrivals.  Each request's own
    time alone (one synchronous call, host buffers as in the served path) is measured too, so a
    rate below the server's capacity shows latency = service time, not queueing."""
    import threading

    sizes = [(g.num_samples, g.num_mutations, g.num_edges) for g in graphs]
    pools = {}
    for gi, (N, M, _) in enumerate(sizes):
        for d in (UP, DOWN):
            cols = N if d == UP else M
            pools[(gi, d, "int32")] = rng.integers(0, 2, size=(256, cols)).astype(np.int32)
            pools[(gi, d, "float32")] = rng.standard_normal((256, cols)).astype(np.float32)
    arrivals, t = [], 0.0
    while len(arrivals) < max_requests:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            break
        gi = 0 if (len(graphs) == 1 or rng.random() < 0.7) else 1
        K = int(np.exp(rng.uniform(0.0, np.log(float(kmax)))))
        d = UP if rng.random() < 0.5 else DOWN
        dt = "int32" if rng.random() < 0.5 else "float32"
        arrivals.append((t, gi, d, pools[(gi, d, dt)][:K]))
    if not arrivals:
        return {"arrival_rate_per_s": rate, "requests": 0}
    units = sum(sizes[gi][2] * V.shape[0] for _, gi, _, V in arrivals)
    lat = []
    with gx.Server(workers=3) as srv:
        ids = [srv.add_graph(g) for g in graphs]
        srv.result(srv.submit(ids[0], pools[(0, UP, "int32")][:1], UP), timeout=120)  # warm
        tickets = [None] * len(arrivals)

        def producer():
            t_start = time.perf_counter()
            for i, (ta, gi, d, V) in enumerate(arrivals):
                delay = ta - (time.perf_counter() - t_start)
                if delay > 0:
                    time.sleep(delay)
                tickets[i] = srv.submit(ids[gi], V, d)

        th = threading.Thread(target=producer)
        t0 = time.perf_counter()
        th.start()
        batches, kept = [], {}
        for i in range(len(arrivals)):
            while tickets[i] is None:
                time.sleep(0.0005)
            out, st = srv.result(tickets[i], timeout=600)
            if i % 4 == 0:
                kept[i] = out  # every fourth result is checked against the same request alone
            lat.append(st["latency_s"])
            batches.append(st["batch_requests"])
        th.join()
        t_served = time.perf_counter() - t0
    t0 = time.perf_counter()
    alone = {}
    alone_ms = []
    for i, (_, gi, d, V) in enumerate(arrivals):
        t1 = time.perf_counter()
        r = gx.matmul(graphs[gi], V, d)
        alone_ms.append(1e3 * (time.perf_counter() - t1))
        if i in kept:
            alone[i] = r
    t_plain = time.perf_counter() - t0
    # in the mix vs alone: integer results bit-exact; float32 sums may differ in their last bits
    # because a stacked call can run a different launch shape (another order of the additions)
    int_exact, f32_diff = True, 0.0
    for i, a in alone.items():
        b = kept[i]
        if a.dtype == np.int32:
            int_exact &= bool(np.array_equal(a, b))
        else:
            scale = max(float(np.max(np.abs(a))), 1e-30)
            f32_diff = max(f32_diff, float(np.max(np.abs(a.astype(np.float64) - b))) / scale)
    lat_ms = np.array(lat) * 1e3
    return {"arrival_rate_per_s": rate, "requests": len(arrivals), "k_max": kmax,
            "arrival_window_s": arrivals[-1][0] if arrivals else 0.0,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "alone_p50_ms": float(np.percentile(alone_ms, 50)),
            "p50_over_alone_p50": float(np.percentile(lat_ms, 50) / max(np.percentile(alone_ms, 50), 1e-9)),
            "served_edgeK_per_s": units / t_served, "plain_sequential_edgeK_per_s": units / t_plain,
            "mean_batch_requests": float(np.mean(batches)),
            "mix_vs_alone": {"checked": len(alone), "int32_bit_exact": int_exact,
                             "float32_max_diff_rel_to_max": f32_diff}}


def cold_start(gx, torch, g):
    """Serving cold start: the graph written as a .grg file, then read back (edge buckets kept
    encoded) and made resident (buckets decoded on the GPU, plan built on the GPU)."""
    fd, path = tempfile.mkstemp(suffix=".grg")
    os.close(fd)
    try:
        t0 = time.perf_counter()
        g.save(path)
        t_save = time.perf_counter() - t0
        size = os.path.getsize(path)
        t0 = time.perf_counter()
        g2 = gx.load_immutable_grg(path)
        t_load = time.perf_counter() - t0
        t0 = time.perf_counter()
        g2.upload()
        torch.cuda.synchronize()
        t_up = time.perf_counter() - t0
        resident = g2.info()["device_bytes"]
        del g2
        torch.cuda.empty_cache()
        return {"file_bytes": size, "edges": g.num_edges, "save_s": t_save, "read_s": t_load,
                "decode_and_plan_on_gpu_s": t_up, "load_to_resident_s": t_load + t_up, "device_bytes": resident}
    except (OSError, RuntimeError) as e:
        return {"unavailable": str(e)}
    finally:
        if os.path.exists(path):
            os.unlink(path)


def large_graph(gx, torch, args, l2_peak):
    """The large window-tree graph (N=1,000,000 haplotypes, a variant prefix sized to 2-4e9 edges):
    float32 compensated and float64 at K in {16, 64, 256}, both directions, device inputs.  Each
    entry: sweep device time (CUDA events), edge*K/s, gathered GB/s (edge ids + one row per edge)
    against the L2 read ceiling measured in this run, and the float32 result's max error against
    the float64 result, relative to the sum of |terms| per output (|V| X); the float64 result is
    checked against native FP64 accumulation at K=16.  Then float32 and float64 K=16 products in
    both directions against the oracle (all host cores) on this graph.""" 
    t0 = time.perf_counter()
    g = gx.window_tree_grg(args.large_samples, args.large_mutations, seed=args.seed)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    g.upload()
    torch.cuda.synchronize()
    t_up = time.perf_counter() - t0
    stats = graph_stats(g)
    stats["device_bytes"] = g.info()["device_bytes"]
    E = stats["edges"]
    t_tune = 0.0
    if not args.no_autotune:
        t0 = time.perf_counter()
        for K in (16, 64, 256):
            for dt in ("float64", "float32"):
                for d in (UP, DOWN):
                    gx.autotune(g, dt, K, d)
        t_tune = time.perf_counter() - t0
    rng = np.random.default_rng(5)
    rows = []
    gx.set_timing(True)
    for K in (16, 64, 256):
        for d in (UP, DOWN):
            cols = stats["samples"] if d == UP else stats["mutations"]
            V32 = torch.from_numpy(rng.standard_normal((K, cols)).astype(np.float32)).cuda()
            V64 = V32.double()
            for V in (V64, V32):
                res = None
                for _ in range(2):  # the second call is the timed one
                    res = gx.matmul(g, V, d)
                t = gx.last_timing()
                s = V.element_size()
                gath = E * (4 + K * s) / (t["sweep_ms"] / 1e3) / 1e9
                rows.append({"dtype": "float64" if s == 8 else "float32", "K": K, "dir": "UP" if d == UP else "DOWN",
                             "sweep_ms": t["sweep_ms"], "total_ms": t["total_ms"],
                             "edgeK_per_s": E * K / (t["sweep_ms"] / 1e3),
                             "gathered_GBps": gath, "l2_frac": gath / l2_peak})
                if s == 8:
                    y64 = res
                else:
                    y32 = res
            scale = gx.matmul(g, V32.abs(), d, f32_compensated=False).double().clamp_min(1e-30)
            rows[-1]["max_err_vs_f64"] = ((y32.double() - y64).abs() / scale).max().item()
            if K == 16:
                y64n = gx.matmul(g, V64, d, f64_native=True)
                rows[-2]["max_err_vs_native_f64"] = ((y64 - y64n).abs() / scale).max().item()
            del y32, y64, res, V32, V64
    gx.set_timing(False)
    units = sum(E * r["K"] for r in rows)
    secs = sum(r["sweep_ms"] for r in rows) / 1e3
    gbytes = sum(E * (4 + r["K"] * (8 if r["dtype"] == "float64" else 4)) for r in rows)
    # a batched mix on the same graph: 64 requests, K ~ U{1..128}, UP/DOWN 50/50, compensated
    # float32, stacked into shared traversals (wall clock around the whole batch)
    reqs = []
    for _ in range(64):
        K = int(rng.integers(1, 129))
        d = UP if rng.random() < 0.5 else DOWN
        cols = stats["samples"] if d == UP else stats["mutations"]
        reqs.append((torch.from_numpy(rng.standard_normal((K, cols)).astype(np.float32)).cuda(), d))
    gx.matmul_batch(g, reqs[:2])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gx.matmul_batch(g, reqs)
    torch.cuda.synchronize()
    t_b = time.perf_counter() - t0
    b_units = sum(E * V.shape[0] for V, _ in reqs)
    b_bytes = sum(E * (4 + 4 * V.shape[0]) for V, _ in reqs)
    batched = {"requests": len(reqs), "columns": int(sum(V.shape[0] for V, _ in reqs)), "seconds": t_b,
               "edgeK_per_s": b_units / t_b, "gathered_GBps": b_bytes / t_b / 1e9,
               "l2_frac": b_bytes / t_b / 1e9 / l2_peak,
               "mix": "K~U{1..128}, UP/DOWN 50/50, float32 compensated, device inputs"}
    del reqs
    # and served: Poisson arrivals at 1000 req/s, the serving mix, on this graph alone
    serve = served(gx, [g], 1000.0, 1.0, 48, rng)
    parity = None
    if not args.no_parity:
        og = oracle_graph(g)
        parity = parity_vs_oracle(gx, torch, g, og, [(np.float32, 16, UP), (np.float32, 16, DOWN),
                                                     (np.float64, 16, UP), (np.float64, 16, DOWN)], seed=17)
        parity["graph"] = "this graph (UP runs in split form above 2^31 edges)"
        del og
    del g
    torch.cuda.empty_cache()
    return {"graph": dict(stats, note=f"variant prefix M'={args.large_mutations} of the 10,000,000-variant "
                                      "generator run, sized to the 2-4e9-edge budget"),
            "edgeK_per_s": units / secs, "gathered_GBps": gbytes / secs / 1e9, "l2_frac": gbytes / secs / 1e9 / l2_peak,
            "matmuls": rows, "batched": batched, "served": serve, "parity_vs_oracle": parity,
            "setup_s": {"generate": t_gen, "plan_upload": t_up, "autotune": t_tune}}


def native_libraries():
    """Shared libraries of this repository mapped into the process (Linux /proc/self/maps)."""
    try:
        maps = Path("/proc/self/maps").read_text().splitlines()
    except OSError:
        return None
    root = str(ROOT)
    return sorted({ln.split()[-1][len(root) + 1:] for ln in maps
                   if ln.split()[-1].startswith(root) and ".so" in ln.split()[-1]})


def run_reference(args):
    """The reference arm: the reference's CPU matmul (the oracle's restatement, compiled on this
    host) on all the host cores, the reference's range-split pattern, on the same graph, inputs,
    combos and config as the GPU arm.  The timed steps cover every combo of the workload once,
    each over the whole graph (step_plan).  The process loads only the oracle library: the graph
    comes from the oracle's own generator (window_tree.c, the same graph bit for bit)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle

    oracle.build()
    combos = workload(args)
    threads = oracle.host_threads()
    t0 = time.perf_counter()
    og = oracle.window_tree(args.samples, args.mutations, seed=args.seed, threads=threads)
    t_gen = time.perf_counter() - t0
    stats = {"samples": og.num_samples, "mutations": og.num_mutations, "nodes": og.num_nodes, "edges": og.num_edges}
    inputs = make_inputs(np.random.default_rng(7), combos, og.num_samples, og.num_mutations)
    smp = CpuSampler(og, combos, inputs, threads)
    del og  # the shards hold their own sub-graphs
    k1 = [i for i, (_, K, _) in enumerate(combos) if K == 1] or [0]
    for s in range(args.warmup):  # warm-up steps: the single-vector combos
        smp.run([k1[s % len(k1)]])
    plan = step_plan(len(combos), args.steps)
    units, secs, red, per_step = 0, 0.0, 0.0, []
    for idxs in plan:
        u, t, r = smp.run(idxs)
        units += u
        secs += t
        red += r
        per_step.append(t)
    v = units / secs
    one = smp.one_core()
    passes = sum(len(x) for x in plan) / len(combos)
    cb = {"value": v, "unit": UNIT, "cores": smp.threads, "kind": "port",
          "sample": f"the whole workload: each of the {len(combos)} combos over the whole graph "
                    f"({passes:.2f} passes over the combos in the {args.steps} timed steps; {units:.3g} edge*K in "
                    f"{secs:.1f} s)"}
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int32,float32,float64",
            "data": "synthetic (seeded window-tree GRG)", "impl": "reference",
            "config": workload_config(args, combos, stats),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "reference_cpu": {
                "what": "the reference CPU GRG::matrixMultiplication (grg.h:1341-1517) as restated by the oracle "
                        "(grg_oracle.c, gcc -O3, loop for loop), run with the reference's own multi-core pattern",
                "timed_passes_over_combos": passes,
                "all_cores": {"cores": smp.threads, "edgeK_per_s": v,
                              "timed_steps_ms": [round(1e3 * t, 1) for t in per_step],
                              "combos_per_step": [len(x) for x in plan]},
                "one_core": {"edgeK_per_s": one, "mean_edgeK_per_s": statistics.fmean(one.values()) if one else None,
                             "what": "one thread, one call over one range (1/cores of the graph): the reference "
                                     "as shipped"},
                "split_overhead": {"range_build_s": smp.build_s,
                                   "down_partial_sum_s_per_step": red / args.steps,
                                   "down_partial_sum_share": red / secs,
                                   "what": "building the mutation ranges' sub-graphs (once) and summing DOWN partial "
                                           "outputs (inside the timed steps)"},
                "setup_s": {"generate": t_gen},
                "native_libraries": native_libraries(),
            }}
    print(json.dumps(line), flush=True)


def parity_vs_oracle(gx, torch, g, og, checks, seed, shards=None):
    """GPU products of `g` against the oracle (the reference algorithm, all host cores, sharded)
    on the same seeded inputs: integers bit-exact; floats against the oracle's float64 product,
    per output, relative to the sum of |terms| (the tolerance's scale) and to |output|."""
    import oracle

    sh = shards or oracle.Shards(og, oracle.host_threads(), align=100)
    rng = np.random.default_rng(seed)
    N, M = g.num_samples, g.num_mutations
    rows = []
    t_all = time.perf_counter()
    for dt, K, d in checks:
        dt = np.dtype(dt)
        cols = N if d == UP else M
        if dt.kind == "f":
            V = rng.standard_normal((K, cols)).astype(dt)
        else:
            V = rng.integers(0, 2, size=(K, cols)).astype(dt)  # 0/1 genotype rows; the first is all ones
            V[0] = 1
        got = gx.matmul(g, torch.from_numpy(V).cuda(), d)
        torch.cuda.synchronize()
        got = got.cpu().numpy()
        rec = {"dtype": dt.name, "K": K, "dir": "UP" if d == UP else "DOWN", "outputs": int(got.size)}
        if dt.kind != "f":
            ref = sh.matmul(V, d)
            mism = int(np.count_nonzero(got != ref))
            rec.update({"bit_exact": mism == 0, "mismatches": mism})
        else:
            V64 = V.astype(np.float64)
            ref = sh.matmul(V64, d)
            scale = sh.matmul(np.abs(V64), d)
            err = np.abs(got.astype(np.float64) - ref)
            tol = 1e-6 if dt == np.float32 else 1e-12
            nz = np.abs(ref) > 0
            rec.update({"max_err_rel_sum_abs_terms": float(np.max(err / np.maximum(scale, 1e-300))),
                        "max_err_rel_output": float(np.max(err[nz] / np.abs(ref[nz]))) if nz.any() else 0.0,
                        "median_err_rel_output": float(np.median(err[nz] / np.abs(ref[nz]))) if nz.any() else 0.0,
                        "tolerance_rel_sum_abs_terms": tol,
                        "within_tolerance": bool(np.all(err <= tol * scale + 1e-300)),
                        "reference": "oracle float64 on the same inputs"})
        rows.append(rec)
    return {"checks": rows, "oracle_threads": sh.nshards, "seconds": time.perf_counter() - t_all,
            "all_pass": all(r.get("bit_exact", r.get("within_tolerance")) for r in rows)}


def oracle_graph(g):
    import oracle

    a = g.export_arrays()
    return oracle.OracleGraph(num_samples=g.num_samples, ploidy=g.ploidy, down_off=a["down_off"],
                              down_adj=a["down_adj"], mut_node=a["mut_node"])


def load_peaks():
    pk = ROOT / "MEASURED_PEAKS.json"
    return json.loads(pk.read_text()) if pk.exists() else {}


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    import grgl_gb300 as gx

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    combos = workload(args)
    t0 = time.perf_counter()
    full = gx.window_tree_grg(args.samples, args.mutations, seed=args.seed)
    t_gen = time.perf_counter() - t0
    stats = graph_stats(full)
    # N > 1: range shards of the one graph (the reference's split pattern, serialize.h:147-166):
    # rank r keeps mutation range r (whole windows), DOWN partial outputs are all-reduced and UP
    # column blocks all-gathered over NCCL
    my_range = range(0, stats["mutations"])
    ranges = [my_range]
    g = full
    if world > 1:
        from grgl_gb300 import shard

        ranges = shard.mutation_ranges(full, world, align=100)
        assert len(ranges) == world, "fewer window-aligned ranges than ranks"
        my_range = ranges[rank]
        g = full.subset_mutations(np.arange(my_range.start, my_range.stop, dtype=np.uint32))
    t0 = time.perf_counter()
    g.upload()
    torch.cuda.synchronize()
    t_up = time.perf_counter() - t0
    shard_stats = graph_stats(g)
    levels = g.info()["num_levels"]
    device_bytes = g.info()["device_bytes"]
    rng = np.random.default_rng(7)
    host_inputs = make_inputs(rng, combos, stats["samples"], stats["mutations"])
    dev_inputs = [torch.from_numpy(V).cuda() for V in host_inputs]
    if world > 1:  # DOWN reads only this rank's mutation columns
        dev_inputs = [V if d == UP else V[:, my_range.start:my_range.stop].contiguous()
                      for (_, _, d), V in zip(combos, dev_inputs)]
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def combine(out, d):
        if world == 1:
            return out
        from grgl_gb300 import shard

        return shard.combine_rank_output(out, d, ranges)

    def step(inputs, record):
        for (dt, K, d), V in zip(combos, inputs):
            combine(gx.matmul(g, V, d), d)
            if record is not None:
                record.append((dt, K, d, gx.last_timing()))

    if args.breakdown:
        gx.set_timing(True)
        E = shard_stats["edges"]
        print(json.dumps({"graph": shard_stats}), flush=True)
        for (dt, K, d), V in zip(combos, dev_inputs):
            for _ in range(3):
                gx.matmul(g, V, d)
            t = gx.last_timing()
            rec = {"dtype": str(dt), "K": K, "dir": "UP" if d == UP else "DOWN", "total_ms": t["total_ms"],
                   "sweep_ms": t["sweep_ms"], "edgeK_per_s": E * K / (t["sweep_ms"] / 1e3),
                   "gathered_GBps": E * (4 + K * dt.itemsize) / (t["sweep_ms"] / 1e3) / 1e9,
                   "launches": t["launches"]}
            print(json.dumps(rec), flush=True)
        return

    # launch-shape autotuning: each level of every (dtype, K, direction) of the step
    tune = None
    if not args.no_autotune:
        gx.autotune_clear()
        t0 = time.perf_counter()
        levels_tuned, up_form = 0, {}
        for dt, K, d in dict.fromkeys(combos):
            rep = gx.autotune(g, dt, K, d)
            levels_tuned += sum(1 for ln in rep.splitlines() if " rows " in ln)
            for ln in rep.splitlines():
                if ln.startswith("UP runs"):
                    up_form[f"{np.dtype(dt).name}:{K}"] = "split" if "split form" in ln else "unsplit"
        torch.cuda.synchronize()
        table = gx.autotune_table()
        tune = {"seconds": time.perf_counter() - t0, "levels_tuned": levels_tuned,
                "table_entries": len(table.strip().splitlines()), "up_form": up_form}
        print("autotune table (kind stride rows_log2 degree_log2 g tiles variant):\n" + table, file=sys.stderr)

    # warm-up
    for _ in range(args.warmup):
        step(dev_inputs, None)
    barrier()
    # deferred per-call timing: CUDA events on each call's stream, read back after the region,
    # so the host never waits between calls
    gx.set_timing("deferred")
    clocks = Clocks(local)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    start.record()
    for _ in range(args.steps):
        step(dev_inputs, None)
    end.record()
    barrier()
    clk = clocks.stop()
    gx.set_timing(False)
    records = [(dt, K, d, t) for (dt, K, d), t in zip(combos * args.steps, gx.collect_timings())]
    ms = start.elapsed_time(end)
    ms_t = torch.tensor([ms], device="cuda")
    if world > 1:
        torch.distributed.all_reduce(ms_t, op=torch.distributed.ReduceOp.MAX)
    ms = float(ms_t.item())
    # the whole job's work: every edge of the one graph, K updates each, per matmul
    units_per_step = sum(stats["edges"] * K for _, K, _ in combos)
    value = units_per_step * args.steps / (ms / 1000.0)

    if tune is not None:
        # the same step on the default shapes, for the tuner's gain (untimed for `value`)
        saved = gx.autotune_table()
        gx.autotune_clear()
        gx.set_timing(True)
        step(dev_inputs, None)
        recs = []
        step(dev_inputs, recs)
        gx.set_timing(False)
        gx.autotune_load(saved)
        tune["sweep_ms_per_step_default_shapes"] = sum(t["sweep_ms"] for *_, t in recs)
        tune["sweep_ms_per_step_tuned"] = sum(t["sweep_ms"] for *_, t in records) / args.steps

    # ---- ceilings of the sweep kernel over the timed region -----------------------------------
    # The gathers are served by L2 (the node rows a level gathers are reused across its warps),
    # so the bound is L2 read bandwidth: edge ids + one gathered row per edge, per launch, against
    # the L2 -> SM read bandwidth measured in this run.  Beside it, the DRAM bytes ncu counts
    # (a capture of the same step on a quarter-size graph, scaled by edges) against the HBM peak.
    E = shard_stats["edges"]
    sweep_ms = sum(t["sweep_ms"] for *_, t in records)
    sweep_s_step = sweep_ms / args.steps / 1e3
    launches = sum(t["launches"] for *_, t in records)
    gathered = sum(E * (4 + K * dt.itemsize) for dt, K, d, _ in records) / args.steps
    abytes = sum(alg_bytes(shard_stats, K, dt.itemsize, d) for dt, K, d, _ in records) / args.steps
    compulsory = sum(E * 4 + (shard_stats["nodes"] + 1) * 8 + 2 * shard_stats["nodes"] * K * dt.itemsize
                     for dt, K, d, _ in records) / args.steps
    l2_peak = gx.measure_l2_bandwidth()
    peaks = load_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback 6800 GB/s (of fallback)"
    traffic = traffic_src = None
    tfile = ROOT / "profiles" / "sweep_traffic.json"
    default_step = (world == 1 and not args.only and args.samples == 200_000 and args.mutations == 1_000_000
                    and args.ks == "1,8,32,64" and args.dtypes == "int32,float32,float64")
    if tfile.exists() and default_step:
        tf = json.loads(tfile.read_text())
        if tf.get("dram_bytes_per_step") and tf.get("graph", {}).get("edges"):
            traffic = tf["dram_bytes_per_step"] * E / tf["graph"]["edges"]
            traffic_src = (f"ncu dram__bytes_read.sum + dram__bytes_write.sum over every sweep launch of one step on "
                           f"the N={tf['graph']['samples']}, M={tf['graph']['mutations']} graph "
                           f"(E={tf['graph']['edges']}), scaled by edges x{E / tf['graph']['edges']:.2f} "
                           "(profiles/sweep_traffic.json)")
    k1 = [(dt, d, t["sweep_ms"]) for dt, K, d, t in records if K == 1]
    id_stream = None
    if k1:
        rates = [E * 4 / (ms_ / 1e3) / 1e9 for _, _, ms_ in k1]
        id_stream = {"achieved": statistics.fmean(rates), "peak": hbm_peak, "unit": "GB/s",
                     "frac": statistics.fmean(rates) / hbm_peak,
                     "what": "K=1 matmuls: the 4-byte edge-id stream (E x 4 bytes, read once from HBM) / sweep "
                             "time; the part of the step HBM itself bounds"}
    roofline = {
        "bound": "l2", "kernel": "grgx::sweep_kernel",
        "achieved": gathered / sweep_s_step / 1e9, "peak": l2_peak, "unit": "GB/s",
        "frac": gathered / sweep_s_step / 1e9 / l2_peak,
        "traffic": traffic, "traffic_source": traffic_src,
        "what": "edge ids + one gathered row per edge (E x (4 + K x s) bytes per matmul) over the step's sweep "
                "launches / their CUDA-event time, against the L2 -> SM read bandwidth measured in this run",
        "peak_source": "grgx_measure_l2_bandwidth in this run (an L2-resident buffer read by every SM); the "
                       "ncu cross-check is in profiles/l2_ceiling_small.md",
        "sweep_ms_per_step": sweep_s_step * 1e3,
        "hbm": {"achieved": None if traffic is None else traffic / sweep_s_step / 1e9, "peak": hbm_peak,
                "unit": "GB/s", "frac": None if traffic is None else traffic / sweep_s_step / 1e9 / hbm_peak,
                "peak_source": hbm_src, "what": "measured DRAM bytes (scaled ncu capture) / sweep time"},
        "edge_id_stream": id_stream,
        "gather_model_GBps": abytes / sweep_s_step / 1e9,
        "gather_model_note": "the survey's algorithmic bytes (ids, offsets, one row per edge, one row per node, "
                             "I/O) / sweep time: exceeds the HBM peak because L2 serves the row gathers; not a "
                             "fraction of any peak",
        "compulsory_GBps": compulsory / sweep_s_step / 1e9,
    }

    # end to end: host buffers through the C-ABI (copies inside the timed region)
    barrier()
    h2d = sum(V.nbytes for V in host_inputs)
    d2h = sum(K * (stats["mutations"] if d == UP else stats["samples"]) * dt.itemsize for dt, K, d in combos)
    e2e_value = e2e_mean = e2e_sync = None
    e2e_steps, e2e_times = 0, []
    if not args.no_e2e and world == 1:
        # inputs in pinned host memory (host_empty); every call copies its input in and its
        # result back inside the timed region
        pinned_inputs = []
        for V in host_inputs:
            P = gx.host_empty(V.shape, V.dtype)
            P[...] = V
            pinned_inputs.append(P)
        streams = [torch.cuda.Stream() for _ in range(max(1, args.e2e_streams))]

        def step_async(inputs):
            # the step's calls go round-robin over the streams, so one call's copies overlap the
            # other streams' products; every result is read back before the step ends
            pend = [gx.matmul_async(g, V, d, stream=streams[i % len(streams)])
                    for i, ((_, _, d), V) in enumerate(zip(combos, inputs))]
            for p in pend:
                p.result()

        def timed_steps(fn):
            fn(pinned_inputs)  # untimed: warms the pinned result pool
            barrier()
            times = []
            for _ in range(e2e_steps):
                t0 = time.perf_counter()
                fn(pinned_inputs)
                barrier()
                times.append(time.perf_counter() - t0)
            return times

        e2e_steps = max(1, min(args.steps, 3))
        e2e_times = timed_steps(step_async)
        sync_times = timed_steps(lambda inputs: step(inputs, None))
        # median step: one host-side stall (page reclaim, another process) does not set the figure
        e2e_value = units_per_step / statistics.median(e2e_times)
        e2e_mean = units_per_step * e2e_steps / sum(e2e_times)
        e2e_sync = {"value": units_per_step / statistics.median(sync_times),
                    "step_ms": [round(x * 1e3, 1) for x in sync_times],
                    "api": "grgl_gb300.matmul (one synchronous call at a time, as pygrgl.matmul)"}
        del pinned_inputs

    cold = None
    if rank == 0 and world == 1 and not args.no_load:
        cold = cold_start(gx, torch, g)

    batched = serve = large = None
    if rank == 0 and world == 1 and not args.no_serve:
        rng2 = np.random.default_rng(11)
        nb = args.batch_requests
        batched = [batched_vs_plain(gx, torch, g, E, rng2, nb, 128,
                                    "K~U{1..128}, UP/DOWN 50/50, float32 compensated, half N(0,1) and half "
                                    "standardized inputs", std_every=2, err_sample=8),
                   batched_vs_plain(gx, torch, g, E, rng2, nb, 8,
                                    "K~U{1..8}, UP/DOWN 50/50, float32 compensated, N(0,1) inputs"),
                   batched_vs_plain(gx, torch, g, E, rng2, nb, 1,
                                    "K=1 (single-vector requests, the dot_product pattern), UP/DOWN 50/50, float32 "
                                    "compensated, N(0,1) inputs")]
        g2 = gx.window_tree_grg(max(2, args.samples // 4), max(1, args.mutations * 3 // 10), seed=args.seed + 1)
        g2.upload()
        serve = {"graphs": [graph_stats(x) for x in (g, g2)],
                 "mix": "K log-uniform in [1, 256], UP/DOWN 50/50, int32 0/1 and float32 N(0,1) 50/50, "
                        "70% of requests on the first graph",
                 "plain": "the same requests one per call, sequentially",
                 "runs": [served(gx, [g, g2], float(r), args.serve_seconds, args.serve_requests, rng2)
                          for r in args.serve_rates.split(",")],
                 "narrow_mix": "K log-uniform in [1, 8], otherwise as above",
                 "narrow_runs": [served(gx, [g, g2], float(r), args.serve_seconds, args.serve_requests, rng2,
                                        kmax=8) for r in args.narrow_rates.split(",")]}
        del g2
    if rank == 0 and world == 1 and not args.no_large:
        large = large_graph(gx, torch, args, l2_peak)

    cpu = parity = None
    if rank == 0 and world == 1 and not (args.no_cpu_baseline and args.no_parity):
        import oracle

        og = oracle_graph(g)
        smp = CpuSampler(og, combos, host_inputs, oracle.host_threads())
        del og
        if not args.no_parity:
            parity = parity_vs_oracle(gx, torch, g, None, [(np.int32, 1, UP), (np.int32, 1, DOWN), (np.int32, 8, UP),
                                                           (np.int32, 8, DOWN), (np.float64, 8, UP),
                                                           (np.float64, 8, DOWN), (np.float32, 8, UP),
                                                           (np.float32, 8, DOWN)], seed=13, shards=smp.sh)
            parity["graph"] = "the benchmark graph itself"
        if not args.no_cpu_baseline:
            cpu = cpu_baseline(args, combos, smp)
        del smp

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak",
            "vs_baseline": None, "dtype": "int32,float32,float64",
            "float64_accumulation": "scaled float pairs (hi + lo float32 words, ~48-bit significand; error <= "
                                    "4.5e-13 x sum |terms| per run), native FP64 when a row's range needs it",
            "data": "synthetic (seeded window-tree GRG)",
            "config": workload_config(args, combos, stats),
            "parallelism": (f"{world} GPUs, one window-aligned mutation range each: DOWN all-reduce, UP all-gather "
                            "(NCCL)") if world > 1 else "single GPU",
            "graph_levels": levels, "device_bytes": device_bytes,
            "roofline": roofline,
            "clocks": clk,
            "gpu_launches": launches,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": None if e2e_value is None else e2e_steps, "statistic": "median step",
                    "mean_value": e2e_mean,
                    "step_ms": [round(x * 1e3, 1) for x in e2e_times] if e2e_times else None,
                    "api": "grgl_gb300.matmul_async on numpy inputs in pinned memory (C ABI grgx_matmul, host "
                           f"pointers, GRGX_FLAG_ASYNC), calls round-robin over {args.e2e_streams} CUDA streams",
                    "one_call_at_a_time": e2e_sync},
            "cpu_baseline": cpu,
            "parity_full_size": parity,
            "batched_vs_plain": batched,
            "served": serve,
            "large_graph": large,
            "cold_start": cold,
            "autotune": tune,
            "setup_s": {"generate": t_gen, "plan_upload": t_up},
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
