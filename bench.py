"""Benchmark of the GB300 alignment-scoring engine.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one step): a 300-residue protein query (blosum62, gap 10/1) against
1,000,000 synthetic protein records (log-normal lengths, median 350, 0.1%
planted homologs), scored once with striped-semi-global (ends FFTT) and once
with striped-local, threshold 0.8 -- the single-query protein configuration of
ish's benchmarks.  Metric: GCUPS = sum over passes of Q x total record length /
seconds / 1e9 (ish's own definition, benchmarking/ish_bench_aligner.mojo:740-750).

  value     device time of the scoring + hit-compaction kernels, records
            resident in HBM (CUDA events on the engine stream); the record
            stream (~419 MB) is larger than L2, so every pass reads HBM.
  e2e       the same step through the C ABI from pinned host buffers: upload
            records, score both passes, copy scores/ends/hits back.  Before
            each step (untimed) the batch is written into the pinned buffer,
            as a runner fills its batch buffer from a file: a pinned buffer
            left untouched by the CPU for 0.1-1 s was measured to upload at
            30-110 GB/s instead of 211 GB/s on some GB300 hosts.
  roofline  integer cell-update roofline: measured DPX add-max throughput x 2
            cells per instruction / DPX instructions per cell pair (4 for
            semi-global, 5 for local; 4.5 cell-weighted over the step).
  cpu_baseline / --impl reference: the CPU oracle (a restatement of ish's
            striped CPU matchers) on all host cores, on a bounded sample.
  parity    the timed step's scores, ends and hit flags compared with the
            oracle on the CPU sample's records (outside the timed region); the
            run exits non-zero on any mismatch.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# DPX add-max instructions per cell pair of the wavefront kernel (wave.cuh).
# Local: T = max(Hdiag + P, E), u = max(T - open, 0), E = max(E - ext, u),
# H = max(Fs - open, T), Fs = max(Fs - ext, T).  Semi-global holds its rows in
# frames rising by ext per row, which folds u into the E update: four.
INSTR_SG, INSTR_SW = 4, 5


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["protein", "line", "batched", "long", "serving"], default="protein",
                    help="protein: single-query protein search (the headline line); line: ascii line search; "
                         "batched: 64 nucleotide queries in one launch; long: 1 Mb-class nucleotide records; "
                         "serving: Poisson query stream against a resident 4 GB set")
    ap.add_argument("--records", type=int, default=None, help="records in the batch (default: the workload's size)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU time of the baseline sample")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-kernel comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-batched", action="store_true",
                    help="protein line: skip the batched leg (64 nucleotide queries x 2M reads, one launch)")
    ap.add_argument("--no-serving", action="store_true",
                    help="protein line: skip the serving leg (Poisson query stream against a resident set)")
    ap.add_argument("--serve-gb", type=float, default=None,
                    help="resident set of the serving legs in GB (default: 1 in the protein line, 4 alone)")
    ap.add_argument("--serve-queries", type=int, default=None,
                    help="queries per arrival rate in the serving legs (default: 100 in the protein line)")
    return ap.parse_args()


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines = []
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.p = None

    def _read(self):
        for line in self.p.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
        return rank, world, local, dist
    return rank, world, local, None


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def _oracle_passes():
    """How the CPU oracle runs the striped passes on this host: NEON vectors at
    the reference's lane counts (aarch64) or lane loops."""
    import oracle as O

    return "NEON vectors, 8 x int16 / 16 x uint8 / 8 x uint16" if O.vectors() else "lane loops"


def cpu_sample(wl, seconds):
    """(records, offsets, cells per pass, seconds per step) of a sample sized to ~`seconds`."""
    import oracle as O

    rng = np.random.default_rng(123)
    q = wl.queries[0]
    mx = int(__import__("ish_gb300").ScoringMatrix(wl.kind).values[q, q].sum())
    threads = os.cpu_count() or 1
    def timed(idx):
        sub = wl.subset(idx)
        t = time.perf_counter()
        for algo, ends in ((O.SEMI_GLOBAL, O.TS | O.TE), (O.LOCAL, 0)):
            m = O.Matcher(algo, wl.kind, q, mx, 0.8, gap_open=10, gap_extend=1, ends=ends)
            m.batch(sub.records, sub.offsets, threads=threads, forward=False, matches=True)
        return sub, time.perf_counter() - t
    probe = np.sort(rng.choice(wl.n, min(wl.n, 400), replace=False))
    sub, dt = timed(probe)
    k = int(min(wl.n, max(len(probe), len(probe) * seconds / max(dt, 1e-3))))
    idx = np.sort(rng.choice(wl.n, k, replace=False))
    return idx, threads


def parity_check(wl, idx, passes, threads, gap_open, gap_ext, thr):
    """Bit-exact comparison of GPU results with the oracle on records `idx`.

    `passes` is a list of (label, oracle algo, ends, encoded query, gpu result)
    where the gpu result holds full-length "score"/"qend"/"tend" arrays (or a
    subset of them) and "hit_idx" in original record order.  Runs outside every
    timed region.  Returns {"records", "passes", "mismatches", "fields", ...}."""
    import oracle as O
    from ish_gb300.scoring import ScoringMatrix

    sub = wl.subset(idx)
    m = ScoringMatrix(wl.kind)
    total = 0
    bad = 0
    first = None
    fields = set()
    hits = 0
    for label, algo, ends, q, g in passes:
        mx = int(m.values[q, q].astype(np.int64).sum())
        om = O.Matcher(algo, wl.kind, q, mx, thr, gap_open=gap_open, gap_extend=gap_ext, ends=ends)
        o = om.batch(sub.records, sub.offsets, threads=threads, forward=True, matches=True)
        ghit = np.zeros(wl.n, np.uint8)
        ghit[np.asarray(g["hit_idx"], np.int64)] = 1
        cmp = [("hit", ghit[idx], o["hit"])]
        for k in ("score", "qend", "tend"):
            if k in g:
                cmp.append((k, np.asarray(g[k])[idx], o[k]))
        for k, a, b in cmp:
            fields.add(k)
            d = np.nonzero(a != b)[0]
            bad += len(d)
            if len(d) and first is None:
                i = int(d[0])
                first = f"{label} {k} record {int(idx[i])}: gpu {int(a[i])} oracle {int(b[i])}"
        hits += int(o["hit"].sum())
        total += len(idx)
    out = {"records": int(len(idx)), "passes": len(passes), "record_passes": total, "mismatches": int(bad),
           "fields": sorted(fields), "oracle_hits": hits}
    if first:
        out["first_mismatch"] = first
    return out


def batched_leg(local):
    """The batched configuration at full size beside the headline line: 64
    nucleotide queries (U[50,1000], actgn, gap 3/1, semi-global FFTT,
    threshold 0.8) against 2,000,000 reads of U[100,300] in one batched launch
    per step, against the same queries one wavefront launch each and the
    plain one-thread-per-record kernel in the reference GPU kernel's launch
    shape; parity of the batched kernel with the oracle on a record sample."""
    from ish_gb300 import native, workloads
    from ish_gb300.scoring import ScoringMatrix

    wl = workloads.nucleotide_multi(seed=2, n=2_000_000)
    queries, gap_open, gap_ext, thr = _queries_of("batched", wl)
    cells = sum(len(q) for q, *_ in queries) * int(wl.offsets[-1])
    m = ScoringMatrix(wl.kind)
    out = {"workload": "64 queries of U[50,1000] nt vs 2,000,000 reads of U[100,300] nt, actgn, gap 3/1, "
                       "semi-global FFTT, threshold 0.8"}
    with native.Context(local) as ctx:
        qids = [ctx.set_query(q, wl.kind, m.values, native.ALGO_SEMI_GLOBAL, gap_open, gap_ext,
                              native.FREE_TARGET_START | native.FREE_TARGET_END, mx, thr) for q, _, _, mx in queries]
        sid = ctx.records_load(wl.records, wl.offsets)
        ctx.autotune(sid, qids)
        ctx.score_multi(qids, sid, want=("hit_idx",))  # warm-up (captures the graph)
        ms = []
        for _ in range(2):
            ctx.score_multi(qids, sid, want=("hit_idx",))
            ms.append(ctx.last_kernel_ms())
        batched = cells / (float(np.mean(ms)) * 1e-3) / 1e9
        per = 0.0
        for qid in qids:
            ctx.score_set(qid, sid, want=("hit_idx",))
            per += ctx.last_kernel_ms()
        per_query = cells / (per * 1e-3) / 1e9
        # plain kernel (int16 per-thread arrays, 15,000 threads x 32) on a sample
        sub = wl.subset(np.arange(200_000))
        sid2 = ctx.records_load(sub.records, sub.offsets)
        pq = qids[::8]
        pcells = sum(len(queries[qids.index(q)][0]) for q in pq) * int(sub.offsets[-1])
        ctx.set_option(native.OPT_KERNEL, native.KERNEL_PLAIN16)
        pms = 0.0
        for qid in pq:
            ctx.score_set(qid, sid2, want=("hit_idx",))
            pms += ctx.last_kernel_ms()
        ctx.set_option(native.OPT_KERNEL, native.KERNEL_AUTO)
        ctx.records_free(sid2)
        plain = pcells / (pms * 1e-3) / 1e9
        # the batched kernel on a record sample against the oracle
        rng = np.random.default_rng(31)
        idx = np.sort(rng.choice(wl.n, 3000, replace=False))
        sample = wl.subset(idx)
        sid3 = ctx.records_load(sample.records, sample.offsets)
        full = ctx.score_multi(qids, sid3, want=("score", "qend", "tend", "hit_idx"))
        ctx.records_free(sid3)
        ctx.records_free(sid)
    import oracle as O

    bad = 0
    for i, (q, algo, ends, mx) in enumerate(queries):
        o = O.Matcher(algo, wl.kind, q, mx, thr, gap_open=gap_open, gap_extend=gap_ext, ends=ends).batch(
            sample.records, sample.offsets, threads=os.cpu_count() or 1)
        hit = np.zeros(len(idx), np.uint8)
        hit[np.asarray(full["hit_idx"][i], np.int64)] = 1
        bad += int(np.count_nonzero(full["score"][i] != o["score"]) + np.count_nonzero(full["qend"][i] != o["qend"])
                   + np.count_nonzero(full["tend"][i] != o["tend"]) + np.count_nonzero(hit != o["hit"]))
    out.update({"batched_gcups": round(batched, 1), "ms_per_step": round(float(np.mean(ms)), 2),
                "per_query_launches_gcups": round(per_query, 1),
                "batched_over_per_query": round(batched / per_query, 3),
                "plain_int16_15000x32_gcups": round(plain, 2), "batched_over_plain": round(batched / plain, 1),
                "parity": {"records": int(len(idx)), "queries": len(queries), "mismatches": bad}})
    return out


def serving_leg(local, gb, count, rates=None):
    """Poisson query streams through the serving loop (ish_gpu_serve_*)
    against a resident blosum62 protein set: per arrival rate the served rate
    and p50/p99 latency of `count` queries (Q ~ U[20,2000], striped-local /
    semi-global FFTT mix, gap 10/1, threshold 0.8); the device rate against
    the same queries scored one launch each; and each query's result in the
    mix against the same query alone."""
    from ish_gb300 import native, workloads
    from ish_gb300.scoring import ScoringMatrix

    wl = workloads.serving_records(seed=4, total_bytes=int(gb * (1 << 30)))
    residues = int(wl.offsets[-1])
    m = ScoringMatrix(wl.kind)
    out = {"workload": f"{gb:g} GB resident blosum62 set ({wl.n} records, lognormal median 350), Poisson arrivals, "
                       f"{count} queries per rate, Q ~ U[20,2000], striped-local / semi-global FFTT mix, gap 10/1, "
                       "threshold 0.8; capacity = the same queries scored one launch each",
           "records": wl.n, "residues": residues}

    deadline = time.perf_counter() + 900.0  # the whole leg; a stuck query fails it instead of hanging the run

    def wait(ctx, t):
        r = None
        while r is None:
            if time.perf_counter() > deadline:
                raise TimeoutError("serving leg: a query did not complete within the leg's 900 s")
            r = ctx.poll(t, wait_ms=200)
        return r

    def make(ctx, qs):
        ids = []
        for _, algo, q in qs:
            a = native.ALGO_LOCAL if algo == "striped-local" else native.ALGO_SEMI_GLOBAL
            ids.append(ctx.set_query(q, wl.kind, m.values, a, 10, 1,
                                     native.FREE_TARGET_START | native.FREE_TARGET_END if a == 0 else 0,
                                     int(m.values[q, q].sum()), 0.8))
        return ids

    with native.Context(local) as ctx:
        sid = ctx.records_load(wl.records, wl.offsets)
        # the stream's queries (the same queries at every rate: the rate only
        # scales their arrival times), each scored alone first: the device
        # rate and capacity every rate below is offered against
        stream = workloads.serving_queries(seed=5, count=count, rate=1.0)
        pids = make(ctx, stream)
        alone_ms = 0.0
        alone = []
        for qid in pids:
            r = ctx.score_set(qid, sid, want=("hit_idx",))
            alone_ms += ctx.last_kernel_ms()
            alone.append(r["hit_idx"])
        pcells = sum(len(q) for _, _, q in stream) * residues
        single = pcells / (alone_ms * 1e-3) / 1e9
        capacity = len(stream) / (alone_ms * 1e-3)
        # the same queries through the serving loop, submitted at once: the
        # device rate at saturation, and every result against the query alone
        ctx.serve_start(sid, max_active=64, chunks=8)
        tickets = [ctx.submit(q) for q in pids]
        same = True
        for t, want in zip(tickets, alone):
            r = wait(ctx, t)
            same = same and np.array_equal(r["hit_idx"], want)
        st = ctx.serve_stats()
        ctx.serve_stop()
        sat = st["cells"] / st["device_ms"] / 1e6
        for qid in pids:
            ctx.free_query(qid)
        per_rate = []
        for frac in (rates or (0.5, 0.9, 2.0)):
            rate = capacity * frac
            qs = workloads.serving_queries(seed=5, count=count, rate=rate)
            ids = make(ctx, qs)
            ctx.serve_start(sid, max_active=64, chunks=8)
            start = time.perf_counter()
            tickets = []
            for (arrival, _, _), qid in zip(qs, ids):
                now = time.perf_counter() - start
                if arrival > now:
                    time.sleep(arrival - now)
                tickets.append(ctx.submit(qid))
            lat = [wait(ctx, t)["latency_ms"] for t in tickets]
            span = time.perf_counter() - start
            st = ctx.serve_stats()
            ctx.serve_stop()
            for qid in ids:
                ctx.free_query(qid)
            per_rate.append({"offered_per_s": round(rate, 3), "offered_over_capacity": frac,
                             "served_per_s": round(count / span, 3),
                             "p50_ms": round(float(np.percentile(lat, 50)), 1),
                             "p99_ms": round(float(np.percentile(lat, 99)), 1),
                             "device_gcups": round(st["cells"] / st["device_ms"] / 1e6, 1),
                             "max_active": st["max_active"], "queries": count})
        ctx.records_free(sid)
    out.update({"single_query_launches_gcups": round(single, 1), "capacity_per_s": round(capacity, 3),
                "saturated_device_gcups": round(sat, 1), "saturated_over_single": round(sat / single, 3),
                "results_equal_alone": bool(same), "results_compared": len(alone), "rates": per_rate})
    return out


def run_reference(args):
    """CPU oracle (restatement of ish's striped CPU matchers) on all host cores."""
    import oracle as O
    from ish_gb300 import workloads

    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = workloads.protein(n=args.records)
    idx, threads = cpu_sample(wl, args.cpu_seconds / max(1, args.steps + args.warmup) * 4)
    sub = wl.subset(idx)
    q = wl.queries[0]
    mx = int(__import__("ish_gb300").ScoringMatrix(wl.kind).values[q, q].sum())
    cells = 2 * len(q) * int(sub.offsets[-1])
    times = []
    for s in range(args.warmup + args.steps):
        t = time.perf_counter()
        for algo, ends in ((O.SEMI_GLOBAL, O.TS | O.TE), (O.LOCAL, 0)):
            m = O.Matcher(algo, wl.kind, q, mx, 0.8, gap_open=10, gap_extend=1, ends=ends)
            m.batch(sub.records, sub.offsets, threads=threads, forward=False, matches=True)
        if s >= args.warmup:
            times.append(time.perf_counter() - t)
    ms = 1e3 * float(np.mean(times))
    gcups = cells / (ms * 1e-3) / 1e9
    sample = f"{len(idx)} of {wl.n} records ({int(sub.offsets[-1])} residues), semi-global + local per step"
    print(json.dumps({
        "impl": "reference", "metric": "GCUPS", "value": round(gcups, 4), "unit": "GCUPS",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16",
        "data": "synthetic", "config": workload_config(args.records),
        "cpu_baseline": {"value": round(gcups, 4), "unit": "GCUPS", "cores": threads, "kind": "port", "passes": _oracle_passes(),
                         "sample": sample},
        "e2e": {"value": round(gcups, 4), "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def workload_config(n):
    return {"workload": f"protein single-query search: 300-aa query vs {n} records, blosum62, gap 10/1, "
                        "striped-semi-global FFTT + striped-local per step, threshold 0.8",
            "query_len": 300, "records": n, "record_lengths": "lognormal(median 350, sigma 0.6) clipped 30-5000",
            "l2": "record stream larger than L2 (129 MB): every pass reads HBM", "parallelism": "records"}


def run_ours(args):
    rank, world, local, dist = dist_setup(args.gpus)
    from ish_gb300 import native, workloads
    from ish_gb300.scoring import ScoringMatrix

    native.load(build_if_missing=True)
    wl = workloads.protein(seed=1 + rank, n=args.records)
    q = wl.queries[0]
    m = ScoringMatrix(wl.kind)
    mx = int(m.values[q, q].sum())
    cells_per_pass = len(q) * int(wl.offsets[-1])
    cells = 2 * cells_per_pass
    ctx = native.Context(local)
    q_sg = ctx.set_query(q, wl.kind, m.values, native.ALGO_SEMI_GLOBAL, 10, 1,
                         native.FREE_TARGET_START | native.FREE_TARGET_END, mx, 0.8)
    q_sw = ctx.set_query(q, wl.kind, m.values, native.ALGO_LOCAL, 10, 1, 0, mx, 0.8)
    sid = ctx.records_load(wl.records, wl.offsets)

    def step():
        r1 = ctx.score_set(q_sg, sid, want=("score", "qend", "tend", "hit_idx"))
        t1 = ctx.last_kernel_ms()
        r2 = ctx.score_set(q_sw, sid, want=("score", "qend", "tend", "hit_idx"))
        t2 = ctx.last_kernel_ms()
        return t1 + t2, (r1, r2)

    for _ in range(args.warmup):
        step()
    clocks = Clocks(local)
    clocks.start()
    barrier(dist)
    dev_ms = []
    launches0 = ctx.launch_count()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ms, res = step()
        dev_ms.append(ms)
    launches = ctx.launch_count() - launches0
    wall_ms = 1e3 * (time.perf_counter() - t0) / args.steps
    barrier(dist)
    clk = clocks.stop()
    step_ms = reduce_max(dist, float(np.mean(dev_ms)))
    value = world * cells / (step_ms * 1e-3) / 1e9
    hits = (len(res[0]["hit_idx"]), len(res[1]["hit_idx"]))

    # ---- end to end through the C ABI from pinned host memory ----
    try:
        import torch

        pin = torch.empty(len(wl.records), dtype=torch.uint8, pin_memory=True).numpy()
        pin_off = torch.empty(len(wl.offsets), dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    except Exception:
        pin = np.empty(len(wl.records), np.uint8)
        pin_off = np.empty(len(wl.offsets), np.uint64)
    pin[:] = wl.records
    pin_off[:] = wl.offsets
    e2e_ms = []
    outs_sg, outs_sw = _pinned_outputs(wl.n), _pinned_outputs(wl.n)
    for s in range(args.warmup + args.steps):
        pin[:] = wl.records  # the step's batch, written as a runner fills its buffer (untimed)
        barrier(dist)
        t = time.perf_counter()
        sid2 = ctx.records_load(pin, pin_off)
        ctx.score_set(q_sg, sid2, want=("score", "qend", "tend", "hit_idx"), out=outs_sg)
        ctx.score_set(q_sw, sid2, want=("score", "qend", "tend", "hit_idx"), out=outs_sw)
        ctx.records_free(sid2)
        if s >= args.warmup:
            e2e_ms.append(1e3 * (time.perf_counter() - t))
    e2e_step = reduce_max(dist, float(np.mean(e2e_ms)))
    e2e_value = world * cells / (e2e_step * 1e-3) / 1e9
    n = wl.n
    h2d = int(len(wl.records) + 8 * len(wl.offsets))
    d2h = int(2 * (12 * n + 4 * 8 + 4 * sum(hits)))

    # ---- streamed: the step's records as 4 batches; each batch's upload and
    # packing run on the load stream while the previous batch is scored
    # (ish_gpu_records_load_async), as a runner streams batches of a file ----
    streamed = None
    try:
        import torch

        nbat = 4
        cut = np.linspace(0, wl.n, nbat + 1).astype(np.int64)
        bats = []
        for b in range(nbat):
            lo, hi = int(cut[b]), int(cut[b + 1])
            o0, o1 = int(wl.offsets[lo]), int(wl.offsets[hi])
            br = torch.empty(max(1, o1 - o0), dtype=torch.uint8, pin_memory=True).numpy()[: o1 - o0]
            bo = torch.empty(hi - lo + 1, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
            bo[:] = wl.offsets[lo:hi + 1] - wl.offsets[lo]
            bats.append((br, bo, lo, hi, o0, o1))
        bout_sg, bout_sw = _pinned_outputs(int(max(c[3] - c[2] for c in bats))), _pinned_outputs(
            int(max(c[3] - c[2] for c in bats)))
        st_ms, st_seq_ms = [], []
        for mode in ("async", "sync"):
            for s in range(args.warmup + args.steps):
                for br, bo, lo, hi, o0, o1 in bats:
                    br[:] = wl.records[o0:o1]  # the batches, freshly written (untimed)
                barrier(dist)
                t = time.perf_counter()
                nh_st = 0
                if mode == "async":
                    sid_b = ctx.records_load_async(bats[0][0], bats[0][1])
                for b in range(nbat):
                    if mode == "async":
                        nxt = ctx.records_load_async(bats[b + 1][0], bats[b + 1][1]) if b + 1 < nbat else None
                    else:
                        sid_b = ctx.records_load(bats[b][0], bats[b][1])
                    r1 = ctx.score_set(q_sg, sid_b, want=("score", "qend", "tend", "hit_idx"), out=bout_sg)
                    r2 = ctx.score_set(q_sw, sid_b, want=("score", "qend", "tend", "hit_idx"), out=bout_sw)
                    nh_st += len(r1["hit_idx"]) + len(r2["hit_idx"])
                    ctx.records_free(sid_b)
                    if mode == "async":
                        sid_b = nxt
                if s >= args.warmup:
                    (st_ms if mode == "async" else st_seq_ms).append(1e3 * (time.perf_counter() - t))
        streamed = {"value": round(world * cells / (reduce_max(dist, float(np.mean(st_ms))) * 1e-3) / 1e9, 2),
                    "unit": "GCUPS", "batches": nbat,
                    "same_records_loaded_one_by_one_gcups": round(
                        world * cells / (reduce_max(dist, float(np.mean(st_seq_ms))) * 1e-3) / 1e9, 2),
                    "hits_equal": bool(nh_st == sum(hits))}
    except Exception as e:  # reported, not fatal
        streamed = {"error": f"{type(e).__name__}: {e}"}

    # ---- plain one-thread-per-record kernels (the in-GPU comparison), on a
    # random tenth of the records: int32 columns in global scratch, and int16
    # per-thread arrays in the reference GPU kernel's launch shape ----
    plain = None
    if not args.no_plain:
        sub_idx = np.sort(np.random.default_rng(7).choice(wl.n, max(1, wl.n // 10), replace=False))
        psub = wl.subset(sub_idx)
        psid = ctx.records_load(psub.records, psub.offsets)
        pcells = 2 * len(q) * int(psub.offsets[-1])
        plain = {}
        for name, kern in (("int32_global_columns", native.KERNEL_PLAIN),
                           ("int16_thread_arrays_15000x32", native.KERNEL_PLAIN16)):
            ctx.set_option(native.OPT_KERNEL, kern)
            pm = []
            for r in range(2):
                ctx.score_set(q_sg, psid, want=("hit_idx",))
                t_sg = ctx.last_kernel_ms()
                ctx.score_set(q_sw, psid, want=("hit_idx",))
                if r:
                    pm.append(t_sg + ctx.last_kernel_ms())
            plain[name] = round(pcells / (float(np.mean(pm)) * 1e-3) / 1e9, 2)
        ctx.set_option(native.OPT_KERNEL, native.KERNEL_AUTO)
        ctx.records_free(psid)
        plain["sample"] = f"{len(sub_idx)} of {wl.n} records, semi-global + local"

    # ---- integer roofline ----
    dpx = ctx.calibrate()
    # the lane-width choice: local-alignment rows in registers on 2 x 16-bit
    # DPX lanes against 4 x 8-bit saturating SIMD byte lanes
    lanes = {k: round(v / 1e9, 1) for k, v in ctx.calibrate_lanes().items()}
    lanes = {"s16x2_gcups": lanes["s16x2_cells_per_s"], "u8x4_gcups": lanes["u8x4_cells_per_s"],
             "what": "local-alignment rows, registers only, no memory traffic"}
    instr = (INSTR_SG + INSTR_SW) / 2  # equal cells in both passes of a step
    peak_gcups = dpx * 2 / instr / 1e9
    per_gpu = cells / (step_ms * 1e-3) / 1e9
    # DRAM bytes per wave launch from the committed ncu capture (a smaller
    # record set), scaled to this run's record stream.
    traffic = None
    prof = os.path.join(ROOT, "profiles", "wave_protein_traffic.json")
    if os.path.exists(prof):
        try:
            tj = json.load(open(prof))
            per = tj["dram_bytes_per_launch_captured"]
            traffic = int((per["semi_global"] + per["local"]) / 2 * int(wl.offsets[-1])
                          / tj["captured_case"]["residues"])
        except Exception:
            traffic = None

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        import oracle as O

        idx, threads = cpu_sample(wl, args.cpu_seconds)
        sub = wl.subset(idx)
        t = time.perf_counter()
        for algo, ends in ((O.SEMI_GLOBAL, O.TS | O.TE), (O.LOCAL, 0)):
            om = O.Matcher(algo, wl.kind, q, mx, 0.8, gap_open=10, gap_extend=1, ends=ends)
            om.batch(sub.records, sub.offsets, threads=threads, forward=False, matches=True)
        dt = time.perf_counter() - t
        cpu = {"value": round(2 * len(q) * int(sub.offsets[-1]) / dt / 1e9, 4), "unit": "GCUPS", "cores": threads,
               "kind": "port", "passes": _oracle_passes(),
               "sample": f"{len(idx)} of {n} records, semi-global + local, {dt:.1f} s on {threads} threads"}
        # the last timed step's own outputs against the oracle on the same
        # records (outside the timed region)
        parity = parity_check(wl, idx, [("semi-global", O.SEMI_GLOBAL, O.TS | O.TE, q, res[0]),
                                        ("local", O.LOCAL, 0, q, res[1])], threads, 10, 1, 0.8)

    legs = {}
    if rank == 0 and world == 1:
        ctx.close()
        ctx = None
        if not args.no_batched:
            try:
                legs["batched"] = batched_leg(local)
            except Exception as e:  # reported, not fatal: the headline line stands on its own
                legs["batched"] = {"error": f"{type(e).__name__}: {e}"}
        if not args.no_serving:
            try:
                legs["serving"] = serving_leg(local, args.serve_gb or 1.0, args.serve_queries or 100)
            except Exception as e:
                legs["serving"] = {"error": f"{type(e).__name__}: {e}"}

    if rank == 0:
        lat = np.array(e2e_ms)
        out = {
            "metric": "GCUPS", "value": round(value, 2), "unit": "GCUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(step_ms, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "s16x2",
            "data": "synthetic", "config": workload_config(n),
            "roofline": {"bound": "int", "achieved": round(per_gpu, 2), "peak": round(peak_gcups, 2),
                         "unit": "GCUPS", "frac": round(per_gpu / peak_gcups, 4), "traffic": traffic,
                         "peak_source": f"measured now: {dpx / 1e12:.2f} T DPX add-max instr/s x 2 cells / "
                                        f"{instr:g} instr per cell pair (semi-global {INSTR_SG}, local {INSTR_SW})",
                         "hbm": {"achieved_gbs": round(2 * int(wl.offsets[-1]) / (step_ms * 1e-3) / 1e9, 2),
                                 "peak_gbs": 6790.0, "peak_source": "MEASURED_PEAKS.json hbm_gbs"}},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e_value, 2), "unit": "GCUPS", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 3),
                                   "p99": round(float(np.percentile(lat, 99)), 3)}},
            "gpu_launches": launches,
            "clocks": clk,
            "plain_kernel_gcups": plain,
            "e2e_streamed": streamed,
            "lane_width": lanes,
            "wall_ms_per_step": round(wall_ms, 3),
            "hits": {"semi_global": hits[0], "local": hits[1]},
            "parity": parity,
            **legs,
        }
        print(json.dumps(out))
    if ctx is not None:
        ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    if parity is not None and parity["mismatches"]:
        print(f"bench: GPU results differ from the oracle: {parity.get('first_mismatch')}", file=sys.stderr)
        sys.exit(3)


# ---------------------------------------------------------------------------
# The other workloads of ish's benchmark configurations (one JSON line each).
# ---------------------------------------------------------------------------

def _base_line(args, world, value, ms, config, dtype="s16x2"):
    return {"metric": "GCUPS", "value": round(value, 2), "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": config}


def _queries_of(name, wl):
    """[(encoded query, oracle algo, ends, max_score)], gap_open, gap_ext, threshold."""
    import oracle as O
    from ish_gb300.scoring import ScoringMatrix

    m = ScoringMatrix(wl.kind)
    mx = lambda q: int(m.values[q, q].astype(np.int64).sum())
    if name == "line":
        q = wl.queries[0]
        return [(q, O.SEMI_GLOBAL, O.TS | O.TE, mx(q))], 3, 1, 0.8
    if name == "batched":
        return [(q, O.SEMI_GLOBAL, O.TS | O.TE, mx(q)) for q in wl.queries], 3, 1, 0.8
    if name == "long":
        q = wl.queries[0]
        return [(q, O.SEMI_GLOBAL, O.TS | O.TE, mx(q))], 3, 1, 0.8
    raise ValueError(name)


def _cpu_sample(wl, queries, gap_open, gap_ext, thr, seconds, max_queries=8):
    """The oracle (all host threads) on a bounded sample: every k-th query and
    a random subset of records sized to about `seconds`."""
    import oracle as O

    threads = os.cpu_count() or 1
    qsel = list(range(len(queries)))[:: max(1, len(queries) // max_queries)][:max_queries]
    qs = [queries[i] for i in qsel]
    rng = np.random.default_rng(123)

    def timed(idx):
        sub = wl.subset(idx)
        t = time.perf_counter()
        for q, algo, ends, mx in qs:
            om = O.Matcher(algo, wl.kind, q, mx, thr, gap_open=gap_open, gap_extend=gap_ext, ends=ends)
            om.batch(sub.records, sub.offsets, threads=threads, forward=False, matches=True)
        return sub, time.perf_counter() - t

    n0 = min(wl.n, 64 if wl.lengths.mean() > 20000 else 400)
    sub, dt = timed(np.sort(rng.choice(wl.n, n0, replace=False)))
    k = int(min(wl.n, max(n0, n0 * seconds / max(dt, 1e-3))))
    idx = np.sort(rng.choice(wl.n, k, replace=False))
    sub, dt = timed(idx)
    cells = sum(len(q) for q, *_ in qs) * int(sub.offsets[-1])
    _cpu_sample.last = (idx, qsel, threads)
    return {"value": round(cells / dt / 1e9, 4), "unit": "GCUPS", "cores": threads, "kind": "port", "passes": _oracle_passes(),
            "sample": f"{len(qs)} of {len(queries)} queries x {k} of {wl.n} records, {dt:.1f} s on {threads} threads"}


def _roofline(ctx, gcups, instr=INSTR_SG):
    """Integer roofline: measured DPX add-max rate x 2 cells / instructions per
    cell pair (cell-weighted over the workload's passes)."""
    dpx = ctx.calibrate()
    peak = dpx * 2 / instr / 1e9
    return {"bound": "int", "achieved": round(gcups, 2), "peak": round(peak, 2), "unit": "GCUPS",
            "frac": round(gcups / peak, 4), "traffic": None,
            "peak_source": f"measured now: {dpx / 1e12:.2f} T DPX add-max instr/s x 2 cells / "
                           f"{instr:.3g} instr per cell pair"}


def _h2d_rate(pin):
    """GB/s of a plain host-to-device copy of the e2e input buffer (torch,
    outside the library): tells a slow host buffer from a slow load path."""
    try:
        import torch

        src = torch.from_numpy(pin)
        dst = torch.empty(len(pin), dtype=torch.uint8, device="cuda")
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        t = time.perf_counter()
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t
        del dst
        torch.cuda.empty_cache()
        return round(len(pin) / dt / 1e9, 1)
    except Exception:
        return None


def _pinned(wl):
    try:
        import torch

        t_rec = torch.empty(len(wl.records), dtype=torch.uint8, pin_memory=True)
        t_off = torch.empty(len(wl.offsets), dtype=torch.int64, pin_memory=True)
        if not (t_rec.is_pinned() and t_off.is_pinned()):
            raise RuntimeError("torch returned unpinned host memory")
        pin = t_rec.numpy()
        pin_off = t_off.numpy().view(np.uint64)
        _pinned.ok = True
    except Exception as e:
        print(f"bench: pinned host buffers unavailable ({e}); end-to-end copies are pageable", file=sys.stderr)
        _pinned.ok = False
        pin = np.empty(len(wl.records), np.uint8)
        pin_off = np.empty(len(wl.offsets), np.uint64)
    pin[:] = wl.records
    pin_off[:] = wl.offsets
    return pin, pin_off


def _pinned_outputs(n):
    """Pinned host arrays for one pass's outputs (score, ends, hit list),
    reused by every end-to-end step: the caller's buffers, as a runner would
    keep them."""
    try:
        import torch

        mk = lambda dt: torch.empty(max(n, 1), dtype=dt, pin_memory=True).numpy()
        return {"score": mk(torch.int32), "qend": mk(torch.int32), "tend": mk(torch.int32),
                "hit_idx": mk(torch.int32).view(np.uint32)}
    except Exception:
        return None


def run_workload(args):
    from ish_gb300 import native, workloads
    from ish_gb300.scoring import ScoringMatrix

    name = args.workload
    rank, world, local, dist = (0, 1, 0, None) if args.impl == "reference" else dist_setup(args.gpus)
    if args.impl == "reference" and int(os.environ.get("RANK", "0")) != 0:
        return
    seed_shift = rank
    if name == "line":
        wl = workloads.line_ascii(seed=0 + seed_shift, n=args.records or 100_000)
        config = {"workload": f"ascii line search: 24-byte query vs {wl.n} printable lines of U[20,120] bytes, "
                              "match +2 / mismatch -2, gap 3/1, striped-semi-global FFTT, threshold 0.8",
                  "records": wl.n, "l2": "7 MB of lines: resident in L2 between steps", "parallelism": "records"}
    elif name == "batched":
        wl = workloads.nucleotide_multi(seed=2 + seed_shift, n=args.records or 2_000_000)
        config = {"workload": f"batched nucleotide search: 64 queries of U[50,1000] nt vs {wl.n} reads of "
                              "U[100,300] nt, actgn, gap 3/1, striped-semi-global FFTT, threshold 0.8, one batched "
                              "launch per step", "queries": len(wl.queries), "records": wl.n,
                  "l2": "reads (400 MB) larger than L2", "parallelism": "records"}
    elif name == "long":
        wl = workloads.long_targets(seed=3 + seed_shift, n=args.records or 10_000)
        config = {"workload": f"long-target search: 1000-nt query vs {wl.n} records of log-uniform 10 kb-1 Mb, "
                              "actgn0, gap 3/1, striped-semi-global FFTT, threshold 0.8",
                  "records": wl.n, "residues": int(wl.offsets[-1]), "l2": "2.1 GB of records: every pass reads HBM",
                  "parallelism": "records"}
    else:
        return run_serving(args, rank, world, local, dist)
    queries, gap_open, gap_ext, thr = _queries_of(name, wl)
    residues = int(wl.offsets[-1])
    cells = sum(len(q) for q, *_ in queries) * residues

    if args.impl == "reference":
        times = []
        cpu = None
        for s in range(args.warmup + args.steps):
            cpu = _cpu_sample(wl, queries, gap_open, gap_ext, thr, args.cpu_seconds / max(1, args.steps + args.warmup))
            if s >= args.warmup:
                times.append(cpu["value"])
        v = float(np.mean(times))
        line = _base_line(args, 1, v, cells / (v * 1e9) * 1e3, config, "int16")
        line.update({"impl": "reference", "cpu_baseline": dict(cpu, value=round(v, 4)),
                     "e2e": {"value": round(v, 4), "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}})
        print(json.dumps(line))
        return

    native.load(build_if_missing=True)
    m = ScoringMatrix(wl.kind)
    # pinned host copy of the batch for the end-to-end arm, allocated before
    # the library's context exists
    pin, pin_off = _pinned(wl)
    ctx = native.Context(local)
    qids = [ctx.set_query(q, wl.kind, m.values, native.ALGO_SEMI_GLOBAL, gap_open, gap_ext,
                          native.FREE_TARGET_START | native.FREE_TARGET_END, mx, thr) for q, _, _, mx in queries]
    sid = ctx.records_load(wl.records, wl.offsets)
    extra = {}
    t0 = time.perf_counter()
    g, k = ctx.autotune(sid, qids)
    extra["autotune"] = {"seconds": round(time.perf_counter() - t0, 3),
                         "shapes": sorted({(int(a), int(b)) for a, b in zip(g, k)})[:16]}

    if name == "batched":
        def step():
            r = ctx.score_multi(qids, sid, want=("hit_idx",))
            return ctx.last_kernel_ms(), r
        launches_per_step = None
    else:
        def step():
            r = ctx.score_set(qids[0], sid, want=("score", "qend", "tend", "hit_idx"))
            return ctx.last_kernel_ms(), r

    for _ in range(args.warmup):
        step()
    clocks = Clocks(local)
    clocks.start()
    barrier(dist)
    dev = []
    launches0 = ctx.launch_count()
    for _ in range(args.steps):
        ms, res = step()
        dev.append(ms)
    launches = ctx.launch_count() - launches0
    barrier(dist)
    clk = clocks.stop()
    step_ms = reduce_max(dist, float(np.mean(dev)))
    value = world * cells / (step_ms * 1e-3) / 1e9

    # comparisons: the same queries one launch each (wavefront kernel), and
    # the plain one-thread-per-record kernel on a sample
    if name == "batched":
        per = []
        for qid in qids:
            ctx.score_set(qid, sid, want=("hit_idx",))
            per.append(ctx.last_kernel_ms())
        extra["per_query_wave_launches_gcups"] = round(cells / (sum(per) * 1e-3) / 1e9, 2)
    # (one thread per record: on 10 kb-1 Mb records a few records already take seconds)
    n_plain = min(wl.n, 200_000 if name == "batched" else (wl.n if name == "line" else 24))
    sub = wl.subset(np.arange(n_plain))
    sid2 = ctx.records_load(sub.records, sub.offsets)
    pq = qids[:: max(1, len(qids) // 8)][:8]
    pcells = sum(len(queries[qids.index(q)][0]) for q in pq) * int(sub.offsets[-1])
    plains = {}
    # int32 columns in global scratch; int16 per-thread arrays in the
    # reference GPU kernel's launch shape (15,000 threads in blocks of 32)
    for pname, kern in (("int32_global_columns", native.KERNEL_PLAIN),
                        ("int16_thread_arrays_15000x32", native.KERNEL_PLAIN16)):
        ctx.set_option(native.OPT_KERNEL, kern)
        pms = 0.0
        for qid in pq:
            ctx.score_set(qid, sid2, want=("hit_idx",))
            pms += ctx.last_kernel_ms()
        plains[pname] = round(pcells / (pms * 1e-3) / 1e9, 2)
    ctx.set_option(native.OPT_KERNEL, native.KERNEL_AUTO)
    ctx.records_free(sid2)
    plain = max(v for v in plains.values())
    extra["plain_per_query_gcups"] = plains
    extra["plain_sample"] = f"{len(pq)} queries x {n_plain} records, one launch per query"
    extra["speedup_vs_plain"] = round(value / world / plain, 1)

    # end to end from pinned host memory: upload + pack + score + results
    h2d_gbs = _h2d_rate(pin)
    e2e = []
    phases = []
    nh = 0
    outs = _pinned_outputs(wl.n)
    for s in range(args.warmup + args.steps):
        # the step's batch is written into the pinned buffer first, as a
        # runner fills its batch buffer from a file (untimed)
        pin[:] = wl.records
        barrier(dist)
        t = time.perf_counter()
        if name == "line":
            # small batches: the one-shot call (upload, pack, score, results)
            r = ctx.score(qids[0], pin, pin_off, want=("score", "qend", "tend", "hit_idx"), out=outs)
            t2 = time.perf_counter()
            nh = len(r["hit_idx"])
            if s >= args.warmup:
                lp = ctx.last_load_ms()  # device phases of the call's load
                ld = lp["upload"] + lp["pack"]
                e2e.append(1e3 * (t2 - t))
                phases.append((ld, 1e3 * (t2 - t) - ld, ctx.last_kernel_ms(), 0.0, lp["upload"], lp["pack"]))
            continue
        sid3 = ctx.records_load(pin, pin_off)
        t1 = time.perf_counter()
        lp = ctx.last_load_ms()
        if name == "batched":
            r = ctx.score_multi(qids, sid3, want=("hit_idx",))
            nh = sum(len(h) for h in r["hit_idx"])
        else:
            r = ctx.score_set(qids[0], sid3, want=("score", "qend", "tend", "hit_idx"), out=outs)
            nh = len(r["hit_idx"])
        t2 = time.perf_counter()
        dev_ms = ctx.last_kernel_ms()
        ctx.records_free(sid3)
        if s >= args.warmup:
            e2e.append(1e3 * (time.perf_counter() - t))
            phases.append((1e3 * (t1 - t), 1e3 * (t2 - t1), dev_ms, 1e3 * (time.perf_counter() - t2), lp["upload"],
                           lp["pack"]))
    e2e_ms = reduce_max(dist, float(np.mean(e2e)))
    ph = np.mean(np.array(phases), axis=0)
    extra["e2e_phases_ms"] = {"load": round(float(ph[0]), 2), "load_upload_device": round(float(ph[4]), 2),
                              "load_pack_device": round(float(ph[5]), 2), "score": round(float(ph[1]), 2),
                              "score_device": round(float(ph[2]), 2), "free": round(float(ph[3]), 2),
                              "pinned": bool(getattr(_pinned, "ok", False)), "h2d_gbs_torch": h2d_gbs}
    d2h = 4 * nh + (0 if name == "batched" else 12 * wl.n) + 8 * (len(qids) + 1)
    if name == "line":
        # from raw text, as a line runner holds a file: upload, split into
        # lines, encode and pack on the device, score, results back
        from ish_gb300.scoring import ScoringMatrix as _SM

        dec = _SM(wl.kind).code_to_ascii
        text = b"\n".join(dec[wl.records[int(wl.offsets[i]):int(wl.offsets[i + 1])]].tobytes()
                           for i in range(wl.n)) + b"\n"
        text_pin = np.frombuffer(text, np.uint8)
        try:
            import torch

            text_pin = torch.empty(len(text), dtype=torch.uint8, pin_memory=True).numpy()
            text_pin[:] = np.frombuffer(text, np.uint8)
        except Exception:
            pass
        tl = []
        for s in range(args.warmup + args.steps):
            t = time.perf_counter()
            sid4, nl = ctx.records_load_lines(text_pin, wl.kind)
            r = ctx.score_set(qids[0], sid4, want=("score", "qend", "tend", "hit_idx"), out=outs)
            ctx.records_free(sid4)
            if s >= args.warmup:
                tl.append(1e3 * (time.perf_counter() - t))
        extra["e2e_from_text"] = {"value": round(cells / (float(np.mean(tl)) * 1e-3) / 1e9, 2), "unit": "GCUPS",
                                  "h2d_bytes_per_step": len(text), "lines": nl,
                                  "hits_equal": bool(len(r["hit_idx"]) == nh)}
    if name == "batched":
        # from FASTQ text, as the FASTX runner holds a file: upload, split
        # into records, encode and pack on the device, score, hits back
        from ish_gb300.scoring import ScoringMatrix as _SM

        dec = _SM(wl.kind).code_to_ascii
        rngq = np.random.default_rng(44)
        parts = []
        for i in range(wl.n):
            seq = dec[wl.records[int(wl.offsets[i]):int(wl.offsets[i + 1])]].tobytes()
            parts.append(b"@read%d\n%s\n+\n%s\n" % (i, seq, bytes(rngq.integers(33, 75, len(seq), dtype=np.uint8))))
        text = np.frombuffer(b"".join(parts), np.uint8)
        del parts
        try:
            import torch

            tp = torch.empty(len(text), dtype=torch.uint8, pin_memory=True).numpy()
            tp[:] = text
            text = tp
        except Exception:
            pass
        text_src = text.copy()
        tl, tload, tphase = [], [], []
        for s in range(args.warmup + args.steps):
            text[:] = text_src  # the file's bytes, freshly read (untimed)
            t = time.perf_counter()
            sid4, nr, _ = ctx.records_load_fastx(text, wl.kind, bounds=False)
            t1 = time.perf_counter()
            lp = ctx.last_load_ms()
            r = ctx.score_multi(qids, sid4, want=("hit_idx",))
            ctx.records_free(sid4)
            if s >= args.warmup:
                tl.append(1e3 * (time.perf_counter() - t))
                tload.append(1e3 * (t1 - t))
                tphase.append((lp["upload"], lp["pack"]))
        del text_src
        same = nr == wl.n and all(np.array_equal(a, b) for a, b in zip(r["hit_idx"], res["hit_idx"]))
        extra["e2e_from_fastq"] = {"value": round(cells / (float(np.mean(tl)) * 1e-3) / 1e9, 2), "unit": "GCUPS",
                                   "h2d_bytes_per_step": len(text), "records": int(nr),
                                   "load_ms": round(float(np.mean(tload)), 2),
                                   "load_upload_and_split_device_ms": round(float(np.mean([x[0] for x in tphase])), 2),
                                   "load_pack_device_ms": round(float(np.mean([x[1] for x in tphase])), 2),
                                   "hits_equal": bool(same)}
        del text
    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        cpu = _cpu_sample(wl, queries, gap_open, gap_ext, thr, args.cpu_seconds)
        pidx, qsel, threads = _cpu_sample.last
        if name == "batched":
            # the timed step fetched hit lists only; one more batched launch
            # (untimed) returns the scores and ends of the same queries
            full = ctx.score_multi(qids, sid, want=("score", "qend", "tend", "hit_idx"))
            gres = [{"score": full["score"][i], "qend": full["qend"][i], "tend": full["tend"][i],
                     "hit_idx": res["hit_idx"][i]} for i in qsel]
            for i in qsel:
                if not np.array_equal(full["hit_idx"][i], res["hit_idx"][i]):
                    raise SystemExit(f"bench: batched hit lists differ between two launches (query {i})")
        else:
            gres = [res]
        parity = parity_check(wl, pidx, [(f"query {i}", queries[i][1], queries[i][2], queries[i][0], g)
                                         for i, g in zip(qsel, gres)], threads, gap_open, gap_ext, thr)
    if rank == 0:
        line = _base_line(args, world, value, step_ms, config)
        line.update({
            "roofline": _roofline(ctx, value / world),
            "cpu_baseline": cpu,
            "e2e": {"value": round(world * cells / (e2e_ms * 1e-3) / 1e9, 2), "unit": "GCUPS",
                    "h2d_bytes_per_step": int(len(wl.records) + 8 * len(wl.offsets)), "d2h_bytes_per_step": int(d2h),
                    "latency_ms": {"p50": round(float(np.percentile(e2e, 50)), 3),
                                   "p99": round(float(np.percentile(e2e, 99)), 3)}},
            "gpu_launches": launches, "clocks": clk, "hits": int(nh), "parity": parity, **extra,
        })
        print(json.dumps(line))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    if parity is not None and parity["mismatches"]:
        print(f"bench: GPU results differ from the oracle: {parity.get('first_mismatch')}", file=sys.stderr)
        sys.exit(3)


def run_serving(args, rank, world, local, dist):
    """Poisson query streams against a resident protein set through the
    serving loop (ish_gpu_serve_*): one JSON line whose value is the device
    rate with the loop saturated, with p50/p99 latency per arrival rate."""
    from ish_gb300 import workloads

    gb = args.serve_gb or float(os.environ.get("ISH_SERVE_GB", "4"))
    count = args.serve_queries or max(args.steps, 20)
    if args.impl == "reference":
        from ish_gb300.scoring import ScoringMatrix
        import oracle as O

        wl = workloads.serving_records(seed=4, total_bytes=int(gb * (1 << 30)))
        m = ScoringMatrix(wl.kind)
        qs = workloads.serving_queries(count=4, rate=1.0)
        queries = [(q, O.LOCAL if a == "striped-local" else O.SEMI_GLOBAL,
                    0 if a == "striped-local" else O.TS | O.TE, int(m.values[q, q].sum())) for _, a, q in qs]
        cpu = _cpu_sample(wl, queries, 10, 1, 0.8, args.cpu_seconds)
        config = {"workload": f"serving: {gb:g} GB resident blosum62 protein set, Q ~ U[20,2000], striped-local / "
                              "semi-global FFTT mix, gap 10/1, threshold 0.8", "parallelism": "records"}
        line = _base_line(args, 1, cpu["value"], 0.0, config, "int16")
        line.update({"impl": "reference", "cpu_baseline": cpu,
                     "e2e": {"value": cpu["value"], "unit": "GCUPS", "h2d_bytes_per_step": 0,
                             "d2h_bytes_per_step": 0}})
        print(json.dumps(line))
        return
    clocks = Clocks(local)
    clocks.start()
    leg = serving_leg(local, gb, count)
    clk = clocks.stop()
    value = leg["saturated_device_gcups"]
    config = {"workload": "serving: " + leg["workload"], "records": leg["records"], "residues": leg["residues"],
              "parallelism": "records"}
    line = _base_line(args, world, value, 0.0, config)
    mean_q = 1010.0  # U[20,2000]
    sat = leg["rates"][-1]
    line.update({"roofline": _roofline_ctxless(local, value, (INSTR_SG + INSTR_SW) / 2), "cpu_baseline": None,
                 "e2e": {"value": round(sat["served_per_s"] * mean_q * leg["residues"] / 1e9, 1), "unit": "GCUPS",
                         "h2d_bytes_per_step": int(mean_q) + 8, "d2h_bytes_per_step": 0,
                         "latency_ms": {"p50": sat["p50_ms"], "p99": sat["p99_ms"]}},
                 "serving": leg, "clocks": clk})
    if rank == 0:
        print(json.dumps(line))


def _roofline_ctxless(local, gcups, instr):
    from ish_gb300 import native

    with native.Context(local) as ctx:
        return _roofline(ctx, gcups, instr)


def main():
    args = parse()
    if args.workload != "protein":
        run_workload(args)
    elif args.impl == "reference":
        args.records = args.records or 1_000_000
        run_reference(args)
    else:
        args.records = args.records or 1_000_000
        run_ours(args)


if __name__ == "__main__":
    main()
