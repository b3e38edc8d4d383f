"""Benchmark: stabilizer inner products/s on the c2 workload (t = 40, chi = 2^16, L = 4096).

One step = the backend work of one probability query: numerator and
denominator estimates (multiSampledProjector of libcirc/innerprod.c:23 on G'
and H') over L = 4096 random stabilizer states each, every state paired with
all 2^16 terms of the k = 16 code.  The inputs (projectors G', H' of a seeded
random Clifford+T circuit, n = 24, t = 40, 8 measured qubits) are the committed
protocol file tests/golden/workload_c2.txt.

  value  pairs per second of device time (CUDA events on the library's stream,
         states drawn on the GPU, inputs resident)
  e2e    pairs per second of wall time through the C ABI with host buffers and
         the reference's own rand() draws (host word generation, uploads and
         result reads inside the timed region)
  batch  batched vs plain queries/s on the light queries of the c3 workload
         (tests/golden/workload_c3.json.gz): the same queries and draws through
         csim_run_queries in shared launches and one at a time, results checked
         bit-identical
  serve  p50/p99 latency and queries/s of the continuous-batching server vs
         plain one-at-a-time service, Poisson arrivals of light c3 queries

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun one query's states are split over the ranks (strong scaling,
circuitsimulator_gb300/shard.py): each rank draws its block of the
counter-based stream, rank 0 gathers one double per state and reduces, so the
numerator and denominator equal one GPU's; rank 0 prints.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = os.path.join(ROOT, "tests", "golden", "workload_c2.txt")
METRIC = "stabilizer inner products/s (t=40)"
UNIT = "inner products/s"
L2_FLUSH_BYTES = 256 << 20


# ------------------------------------------------------------------ workload
def parse_protocol(text):
    from circuitsimulator_gb300 import backend

    return backend.parse_protocol(text)


def load_workload():
    cfg, projs = parse_protocol(open(WORKLOAD).read())
    from circuitsimulator_gb300 import backend

    exact, k, norm, L = backend.decompose(cfg["t"], cfg["fidbound"], cfg["rank"], cfg["fidelity"], cfg["forceL"],
                                          cfg["exact"], cfg["k"])
    return cfg, projs, exact, k, norm, L


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nme, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nme)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


# ------------------------------------------------------------------ roofline
# Mean packed 64-bit row operations per (theta, term) pair of the
# elementary-update algorithm on this workload (the roofline's work unit),
# measured by `python oracle/rowops.py 24 400` over 9600 pairs (each checked
# against the dense restatement): 2576 row-ops/pair, 33% orthogonal pairs.
ROWOPS_PER_PAIR_T40 = 2576.0
# Rows of J and constraint masks the direct-restriction path reads, copies or
# updates per c2 pair (the same 9600 pairs, CSIM_COUNT_ROWS hook of the host build).
DIRECT_ROWS_PER_PAIR_T40 = 151.1


# ncu dram__bytes_read.sum + dram__bytes_write.sum of pair-kernel launches over
# projected c2 states.  The block-prefix kernel: the light launch over 64 states
# (profiles/k_terms_tp_c2_small.md: 657 KB read, 600 KB written), the codeword
# table once and the rest in proportion to the states.  The direct kernel: its
# H' launch over 64 and over 256 states (profiles/k_terms_direct_c2_small.md:
# 1.52 MB and 2.62 MB), a line through the two; per state 1.08 KB is read (the
# pivot form) and 4.66 KB written (the partial sums, and the write-back of the
# states and pivot forms the launches before it left in L2).
MEASURED_TRAFFIC_64_STATES = 657e3 + 600e3
MEASURED_TRAFFIC_CODEWORDS = 8 * 2 ** 16
DIRECT_TRAFFIC = ((64, 677888 + 843264), (256, 884736 + 1737472))


def dram_bytes_per_launch(states, kernel="block prefix"):
    """DRAM bytes of one pair-kernel launch over `states` states, from the
    measured captures above."""
    if kernel == "direct":
        (s0, b0), (s1, b1) = DIRECT_TRAFFIC
        return b0 + (b1 - b0) / (s1 - s0) * (states - s0)
    per_state = (MEASURED_TRAFFIC_64_STATES - MEASURED_TRAFFIC_CODEWORDS) / 64
    return MEASURED_TRAFFIC_CODEWORDS + per_state * states


def alu_peak_gops(num_sms, mhz):
    """Integer lane-op issue peak: SMs x 4 schedulers x 32 lanes x clock."""
    return num_sms * 4 * 32 * mhz * 1e6 / 1e9


# ------------------------------------------------------------------ CPU baseline (oracle leg)
def cpu_baseline(cfg, projs, k, L, budget_s=15.0):
    """The oracle restatement of the reference algorithm (oracle/csim_oracle.c)
    on all host cores, on a bounded sample of the same workload: a few states
    drawn and projected onto G' exactly as the reference does, paired with a
    block of consecutive terms of the same code."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_ffi import ORACLE_SO, Oracle, make_projector

    if not os.path.exists(ORACLE_SO):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    O = Oracle()
    t = cfg["t"]
    ph, xs, zs, nq = projs[0]
    P = make_projector(ph, xs, zs, nq)
    r = O.rng(12345)
    thetas = []
    while len(thetas) < 4:
        s = O.random_state(t, r)
        if O.project(s, P) != 0:
            thetas.append(s[0])
    th = np.array(thetas)
    Lw = np.asarray(L, dtype=np.uint64)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    O.term_products(t, 0, Lw, k, th, 0, 64, threads=cores)
    cal = (time.perf_counter() - t0) / (4 * 64)
    nj = int(max(64, min(2 ** k, budget_s / max(cal, 1e-9) / 4)))
    t0 = time.perf_counter()
    O.term_products(t, 0, Lw, k, th, 0, nj, threads=cores)
    dt = time.perf_counter() - t0
    return {"value": 4 * nj / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "4 projected thetas x %d terms of the c2 code (t=40), oracle/csim_oracle.c on %d threads, %.1f s"
                      % (nj, cores, dt)}


# ------------------------------------------------------------------ arms
def run_ours(args, rank, world, local_rank):
    import torch

    from circuitsimulator_gb300 import backend, shard

    torch.cuda.set_device(local_rank)
    cfg, projs, exact, k, norm, L = load_workload()
    gpu = backend.Backend(local_rank)
    if args.no_tune:
        gpu.set_option(backend.OPT_AUTOTUNE, 0)
    if args.pair_kernel is not None:
        gpu.set_option(backend.OPT_PAIR_KERNEL, args.pair_kernel)
    if args.per_thread is not None:
        gpu.set_option(backend.OPT_PER_THREAD, args.per_thread)
    P = [backend.projector(ph, xs, zs, nq) for (ph, xs, zs, nq) in projs]
    samples, bins = (args.samples or cfg["samples"]), cfg["bins"]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    seed0 = 1000003
    result = {}

    def step(i, rng):
        """One query: numerator and denominator.  Philox: the states of each
        projector split over the ranks, values gathered and reduced on rank 0
        (on one GPU, singleProjectorSample + the native median of means, which
        is multiSampledProjector).  rand() draws (e2e): multiSampledProjector
        through the C ABI; with N ranks each draws its share of the states
        from its own stream (seed + rank)."""
        st = []
        for q in range(2):
            seed = (seed0 + 2 * i + q) & 0xFFFFFFFF
            if rng == backend.RNG_PHILOX:
                vals = shard.sharded_values(gpu, P[q], L, exact, samples * bins, seed, rank, world)
                if vals is not None:
                    result[q] = shard.median_of_means(vals, samples, bins)
            elif world == 1:
                gpu.multiSampledProjector(P[q], L, exact, norm, samples, bins, rng, seed)
            else:
                lo, hi = shard.shard_bounds(samples * bins, rank, world)
                gpu.singleProjectorSample(P[q], L, exact, hi - lo, rng, (seed + rank) & 0xFFFFFFFF)
            st.append(gpu.last_stats().as_dict())
        return st

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    # ---- device-resident arm (value)
    for i in range(args.warmup):
        step(i, backend.RNG_PHILOX)
        flush.zero_()
    barrier()
    if args.no_tune:  # the launch the fixed rules and the forcing options give
        forced = {2: 0, 3: 1, 4: 2, 5: 3}.get(args.pair_kernel, 0)
        tuned = (args.per_thread or 0, 0, 0.0, forced)
    else:  # done by the first warm-up step; this reads the choice
        tuned = gpu.autotune(cfg["t"], P[0], [int(x) for x in L])
    kname = {0: "k_terms_tp (heavy and light launches)", 1: "k_terms_runs",
             2: "k_terms_tp (one launch per occupancy class)",
             3: "k_terms_direct (each state restricted once in pivot form)"}[tuned[3]]
    clocks = ClockSampler(local_rank)
    clocks.start()
    launches0 = gpu.launches
    dev_ms, pair_ms, pairs, states, live = 0.0, 0.0, 0, 0, 0
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        for s in step(args.warmup + i, backend.RNG_PHILOX):
            dev_ms += s["device_ms"]
            pair_ms += s["pair_kernel_ms"]
            pairs += s["pairs"]
            states += s["states"]
            live += s["states_live"]
    barrier()
    launches = gpu.launches - launches0
    clk = clocks.stop()

    # ---- end-to-end arm (e2e): C ABI with host buffers, the reference's rand() draws
    for i in range(min(args.warmup, 1)):
        step(10_000 + i, backend.RNG_LIBC)
    barrier()
    e2e_pairs, h2d, d2h = 0, 0, 0
    t0 = time.perf_counter()
    for i in range(args.steps):
        for s in step(20_000 + i, backend.RNG_LIBC):
            e2e_pairs += s["pairs"]
            h2d += s["h2d_bytes"]
            d2h += s["d2h_bytes"]
    barrier()
    e2e_s = time.perf_counter() - t0

    # max over ranks of the times, sum of the work
    totals = np.array([dev_ms, e2e_s, pairs, e2e_pairs, pair_ms], dtype=np.float64)
    if world > 1:
        tt = torch.tensor(totals, device="cuda")
        mx = tt.clone()
        torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
        sm = tt.clone()
        torch.distributed.all_reduce(sm, op=torch.distributed.ReduceOp.SUM)
        dev_ms, e2e_s, pair_ms = float(mx[0]), float(mx[1]), float(mx[4])
        pairs, e2e_pairs = int(sm[2]), int(sm[3])
    if rank != 0:
        return None

    value = pairs / (dev_ms / 1e3)
    props = torch.cuda.get_device_properties(local_rank)
    mhz = clk.get("sm_mhz") or 2070.0
    per_pair = ROWOPS_PER_PAIR_T40
    kernel_rate = (pairs / world) / (pair_ms / 1e3)  # pairs/s of the pair kernel alone (rank 0 share)
    achieved = kernel_rate * per_pair / 1e9 if per_pair else None
    peak = alu_peak_gops(props.multi_processor_count, clk.get("sm_max_mhz") or 2070.0)
    roofline = {"bound": "alu", "kernel": kname + ": (theta, prepL term) pairs, one thread per pair",
                "achieved": achieved, "peak": peak, "unit": "G packed row-ops/s",
                "frac": (achieved / peak) if achieved else None,
                "traffic": dram_bytes_per_launch(samples * bins / world,
                                                 "direct" if tuned[3] == 3 else "block prefix"),
                "traffic_source": ("ncu dram bytes (read + write) of this kernel's launches over 64 and 256 states "
                                   "(profiles/k_terms_direct_c2_small.md), on the line through them"
                                   if tuned[3] == 3 else
                                   "ncu dram bytes (read + write) of a 64-state launch of this kernel "
                                   "(profiles/k_terms_tp_c2_small.md), scaled to this launch's states"),
                "work_unit": "packed row-op of the reference's algorithm (one 64-bit row test/XOR/update of its "
                             "elementary updates), whichever kernel runs",
                "rowops_per_pair": per_pair,
                "kernel_rows_per_pair": DIRECT_ROWS_PER_PAIR_T40 if tuned[3] == 3 else per_pair,
                "peak_source": "SMs x 4 x 32 lanes x sm_max_mhz (MEASURED_PEAKS.json holds no integer peak)",
                "pair_kernel_share": pair_ms / dev_ms}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "u64 GF(2) rows; Z8 / exact int128 Z[w] sums; f64 final |.|^2",
        "data": "synthetic: seeded random Clifford+T circuit (n=24, t=40, 8 measured qubits) -> G', H' "
                "(tests/golden/workload_c2.txt); random stabilizer states drawn per step",
        "config": {"workload": "c2: t=40, chi=2^16 (k=16 code), L=%d states x 2 projectors per step" % samples,
                   "t": cfg["t"], "k": k, "samples": samples, "bins": bins, "states_per_step": states // args.steps,
                   "live_states_per_step": live // args.steps, "pairs_per_step": pairs // args.steps,
                   "ranks": "the states of each projector split over %d rank(s), values gathered on rank 0" % world,
                   "last_query": {"numerator": result.get(0), "denominator": result.get(1)},
                   "l2": "flushed between steps (256 MiB write); hot data (codewords 512 KiB) is L2-resident",
                   "rng": "Philox on device (value); the C library's rand() sequence (e2e)",
                   "launch": {"kernel": kname, "terms_per_thread": tuned[0] or "fixed rule (32)",
                              "light_zero_bound": tuned[1] or "fixed rule (24)",
                              "chosen_by": "fixed rules (--no-tune)" if args.no_tune else
                              "csim_autotune on this query's G' and code"}},
        "e2e": {"value": e2e_pairs / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
                "d2h_bytes_per_step": d2h // args.steps, "ms_per_step": 1e3 * e2e_s / args.steps},
        "roofline": roofline,
        "clocks": clk,
        "gpu_launches": launches,
    }
    if world == 1 and not args.no_batch:
        out["batch"] = batch_compare(gpu)
        # the same comparison on every 32nd c3 query (t 15..53, three of them heavy), so the line
        # carries the mixed set next to the light one
        out["batch_c3_sample"] = batch_compare(gpu, reps=1, light=False, every=32)
        out["serve"] = serve_compare(100.0, 150)
    if world == 1 and not args.no_cpu_baseline:
        try:
            out["cpu_baseline"] = cpu_baseline(cfg, projs, k, L)
        except Exception as e:  # the baseline never decides the run
            out["cpu_baseline"] = {"value": None, "unit": UNIT, "error": str(e)}
    return out


C3_WORKLOAD = os.path.join(ROOT, "tests", "golden", "workload_c3.json.gz")
C3_LIGHT_PAIRS = 1 << 26


def c3_queries(light=True, every=1):
    """The batched-query workload (tests/golden/workload_c3.json.gz, 256 queries,
    t ~ U[8, 60], relative error 0.05).  light=True keeps the queries of at most
    2^26 inner products, the ones too small to fill the GPU on their own;
    every > 1 keeps every every-th query of the file (before that filter)."""
    import gzip

    from circuitsimulator_gb300 import backend

    with gzip.open(C3_WORKLOAD, "rt") as f:
        recs = json.load(f)
    out = []
    for q in recs[::every]:
        cfg, projs = backend.parse_protocol(q["input"])
        t, k, ex = cfg["t"], cfg["k"], cfg["exact"]
        chi = 2 ** ((t + 1) // 2) if ex else 2 ** k
        na = cfg["noapprox"] or (not cfg["forceSample"] and cfg["samples"] * cfg["bins"] * 2 > chi - 1)
        pairs = sum(chi * (chi + 1) // 2 if na else cfg["samples"] * cfg["bins"] * chi
                    for p in projs if len(p[0]) > 0)
        if light and pairs > C3_LIGHT_PAIRS:
            continue
        out.append({"cfg": cfg, "projs": projs, "seed": q["seed"], "rng": backend.RNG_PHILOX})
    return out, len(recs)


def pretune(gpu, qs):
    """Tunes the thread-per-pair launches (csim_autotune) for every t bucket
    the queries use, on the first query of each bucket (its G' and code), so
    that no timed arm pays for tuning."""
    from circuitsimulator_gb300 import backend

    seen = set()
    for q in qs:
        cfg, projs = q["cfg"], q["projs"]
        if cfg["exact"] or cfg["t"] // 4 in seen or not projs[0][0]:
            continue
        seen.add(cfg["t"] // 4)
        e, k, norm, L = backend.decompose(cfg["t"], cfg["fidbound"], cfg["rank"], cfg["fidelity"], cfg["forceL"],
                                          cfg["exact"], cfg["k"])
        if not e:
            gpu.autotune(cfg["t"], backend.projector(*projs[0]), [int(x) for x in L])


def batch_compare(gpu, reps=3, light=True, every=1):
    """Batched vs plain queries/s on the c3 queries (the light ones by default,
    all 256 with light=False, every every-th of them with every > 1): the
    same queries, the same draws, results checked identical.  Plain = one
    query after another through the single-query entry points; batched =
    csim_run_queries."""
    qs, total = c3_queries(light=light, every=every)
    gpu.run_queries(qs[:4], batched=True)
    gpu.run_queries(qs[:4], batched=False)
    pretune(gpu, qs)
    tp, tb = [], []
    same = True
    pairs = 0
    for _ in range(reps):
        t0 = time.perf_counter()
        rp = gpu.run_queries(qs, batched=False)
        t1 = time.perf_counter()
        rb = gpu.run_queries(qs, batched=True)
        t2 = time.perf_counter()
        tp.append(t1 - t0)
        tb.append(t2 - t1)
        same = same and all((a["numerator"], a["denominator"]) == (b["numerator"], b["denominator"])
                            for a, b in zip(rp, rb))
        pairs = sum(b["pairs"] for b in rb)
    p, b = float(np.median(tp)), float(np.median(tb))
    if light:
        what = "c3 light: the %d of %d c3 queries with <= 2^26 inner products (t 8..23" % (len(qs), total)
    elif every > 1:
        what = "c3 sample: 1 in %d of the %d c3 queries, %d queries (t %d..%d" % (
            every, total, len(qs), min(q["cfg"]["t"] for q in qs), max(q["cfg"]["t"] for q in qs))
    else:
        what = "c3: all %d queries (t 8..60, chi 2^4..2^18" % total
    return {"workload": what + ", relative error 0.05, Philox draws)",
            "metric": "queries/s", "plain": len(qs) / p, "batched": len(qs) / b, "speedup": p / b,
            "identical_results": bool(same), "pairs": pairs, "reps": reps,
            "timing": "wall clock around the ABI call, host work included, median of reps"}


C5_EPS = (0.1, 0.05, 0.02)


def c5_stream(count, seed=505, max_pairs=1 << 30):
    """Queries of the c5 serving configuration, drawn in order from a seeded
    stream: t ~ U[8, 64], n ~ U[8, 40], eps ~ {0.1, 0.05, 0.02}, 1..4 measured
    qubits with a random outcome, the random Clifford+T circuits of
    tests/golden/circuits.py through this package's front end (equal to the
    reference's, tests/test_frontend.py).  Exact decomposition for t <= 16,
    else a code of k = min(18, the fidelity-0.02 rule of probability.c:330)
    rows; L from eps and failure probability 0.05 by probability.py:150-167.
    Draws whose inner products exceed max_pairs are skipped (a c5 query at
    eps = 0.02 and t = 60 takes 2.6e10 pairs, about 10 s of GPU time), so
    the kept stream still spans t = 8..64 and every eps.  Returns (queries,
    draws, [(t, eps, pairs)])."""
    import math

    from circuitsimulator_gb300 import backend, sample

    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from circuits import compiled, random_circuit

    rs = np.random.RandomState(seed)
    out, meta, draws = [], [], 0
    while len(out) < count:
        draws += 1
        n, t, nm = int(rs.randint(8, 41)), int(rs.randint(8, 65)), int(rs.randint(1, 5))
        eps = float(C5_EPS[int(rs.randint(3))])
        config = {"exact": True} if t <= 16 else {
            "exact": False, "fidbound": 0.02,
            "k": min(18, int(math.ceil(1 - 2 * t * math.log2(math.cos(math.pi / 8)) - math.log2(0.02))))}
        config.update({"error": eps, "failprob": 0.05, "quiet": True, "seed": 7000 + draws})
        circ = compiled(random_circuit(n, t, rs)[0])
        qubits = sorted(rs.choice(n, size=nm, replace=False).tolist())
        outcome = rs.randint(2, size=nm).tolist()
        try:
            q = next(sample.probability_steps(circ, {a: b for a, b in zip(qubits, outcome)}, config,
                                              np.random.RandomState(draws)))
        except Exception:  # StopIteration (answered without a backend query) or a front-end refusal
            continue
        cfg = q["cfg"]
        if cfg["t"] < 1:
            continue
        chi = 2 ** ((cfg["t"] + 1) // 2) if cfg["exact"] else 2 ** cfg["k"]
        na = cfg["noapprox"] or (not cfg["forceSample"] and cfg["samples"] * cfg["bins"] * 2 > chi - 1)
        pairs = sum(chi * (chi + 1) // 2 if na else cfg["samples"] * cfg["bins"] * chi
                    for p in q["projs"] if len(p[0]) > 0)
        if pairs > max_pairs:
            continue
        q["rng"] = backend.RNG_PHILOX
        out.append(q)
        meta.append((cfg["t"], eps, pairs))
    return out, draws, meta


def serve_compare(rate, count, seed=5, c5=False):
    """Serving under Poisson arrivals at `rate` queries/s: the continuous-batching
    server (csim_submit as each query arrives) vs plain one-at-a-time service
    (first come first served through the single-query entry points).  Latency
    = result time - arrival time.  Queries: the light c3 queries, or with c5
    the first `count` queries of c5_stream."""
    from circuitsimulator_gb300 import backend

    rs = np.random.RandomState(seed)
    if c5:
        qs, draws, meta = c5_stream(count)
    else:
        light, _ = c3_queries(light=True)
        qs = [light[i] for i in rs.randint(len(light), size=count)]
    arrivals = np.cumsum(rs.exponential(1.0 / rate, size=count))

    def pct(v):
        v = np.sort(np.asarray(v))
        return {"p50_ms": 1e3 * float(np.percentile(v, 50)), "p99_ms": 1e3 * float(np.percentile(v, 99)),
                "max_ms": 1e3 * float(v[-1])}

    tuner = backend.Backend(0)
    pretune(tuner, qs)  # tuned launches for every t of the stream, shared by the process
    tuner.close()
    srv = backend.Server(0)
    for t in [srv.submit(q) for q in qs[:8]]:  # warm-up: decompositions resident, buffers sized
        srv.wait(t)
        srv.release(t)
    t0 = time.perf_counter()
    tickets = []
    for q, a in zip(qs, arrivals):
        d = t0 + a - time.perf_counter()
        if d > 0:
            time.sleep(d)
        tickets.append(srv.submit(q))
    res = [srv.wait(t) for t in tickets]
    t_end = time.perf_counter()
    st = srv.stats()
    srv.close()
    server = dict(pct([r["latency_s"] for r in res]), queries_per_s=count / (t_end - t0),
                  rounds=st["rounds"], failed=sum(1 for r in res if r["status"]))

    gpu = backend.Backend(0)
    gpu.run_queries(qs[:8], batched=False)
    lat = []
    t0 = time.perf_counter()
    for q, a in zip(qs, arrivals):
        d = t0 + a - time.perf_counter()
        if d > 0:
            time.sleep(d)
        gpu.run_queries([q], batched=False)
        lat.append(time.perf_counter() - t0 - a)
    t_end = time.perf_counter()
    plain = dict(pct(lat), queries_per_s=count / (t_end - t0))
    if c5:
        ts = [m[0] for m in meta]
        what = ("c5 subset: the first %d of %d draws of the seeded c5 stream with <= 2^30 inner products each "
                "(t %d..%d, eps %s: %d at 0.02; %.3g pairs), Poisson arrivals at %g queries/s"
                % (count, draws, min(ts), max(ts), "/".join(str(e) for e in C5_EPS),
                   sum(1 for m in meta if m[1] == 0.02), sum(m[2] for m in meta), rate))
    else:
        what = ("c5 (scaled): %d light c3 queries (t 8..23, relative error 0.05), Poisson arrivals at %g queries/s"
                % (count, rate))
    return {"workload": what,
            "rate": rate, "server": server, "plain": plain,
            "throughput_ratio": server["queries_per_s"] / plain["queries_per_s"]}


C4_WORKLOAD = os.path.join(ROOT, "tests", "golden", "workload_c4.json")


def chain_compare(shots, nbits, samples=None, groups=2):
    """sampleQubits chains on the c4 circuit (tests/golden/workload_c4.json:
    n=32, t=64, k=14 code, L=2048 states per conditional): `shots` chains of
    `nbits` sampled qubits, plain (one shot after another, one query at a
    time) vs batched (all shots in lockstep, one csim_run_queries call per
    step).  Same numpy seeds and backend seed; outputs checked equal."""
    from circuitsimulator_gb300 import backend, sample

    w = json.load(open(C4_WORKLOAD))
    cfg = dict(w["config"], seed=4242)
    if samples:
        cfg["samples"] = samples
    bits = w["sample"][:nbits]
    seeds = list(range(1000, 1000 + shots))
    gpu = backend.Backend(0)
    sample.sample_qubits_batch(w["circ"], {}, bits[:1], dict(cfg), seeds[:2], backend=gpu)  # warm-up
    t0 = time.perf_counter()
    plain = [sample.sampleQubits(w["circ"], {}, list(bits), dict(cfg), rng=np.random.RandomState(s), backend=gpu)
             for s in seeds]
    t1 = time.perf_counter()
    st = {}
    batched = sample.sample_qubits_batch(w["circ"], {}, list(bits), dict(cfg), seeds, backend=gpu, stats=st,
                                         groups=groups)
    t2 = time.perf_counter()
    queries = sum(st["queries_per_step"])
    return {"workload": "c4 chain: %d shots x %d sampled qubits, n=32, t=64, k=%d, L=%d per conditional"
                        % (shots, nbits, cfg["k"], cfg["samples"]),
            "metric": "queries/s", "queries": queries, "plain": queries / (t1 - t0), "batched": queries / (t2 - t1),
            "speedup": (t1 - t0) / (t2 - t1), "identical_outputs": plain == batched, "steps": st["steps"],
            "plain_s": t1 - t0, "batched_s": t2 - t1,
            "batched_split": {"gpu_calls_s": st["gpu_s"], "device_s": st["device_s"],
                              "pair_kernel_s": st["pair_kernel_s"], "front_ends_s": st["host_s"],
                              "groups": groups,
                              "note": "shot groups: one group's front ends run while another's queries are on "
                                      "the GPU"}}


def c3_rates(ts=(28, 41, 47, 57), count=2000):
    """Pair-kernel rates inside c3 queries: for the first c3 query at each t in
    `ts`, one projector (G') with the query's own code (decompose) against a
    random code and random projector rows of the same t, k and row count,
    `count` counter-based states each (CUDA-event pair-kernel time)."""
    from circuitsimulator_gb300 import backend

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import rand_word, random_projector_rows

    import gzip

    with gzip.open(C3_WORKLOAD, "rt") as f:
        recs = json.load(f)
    gpu = backend.Backend(0)
    out = []
    seen = set()
    for q in recs:
        t = q["t"]
        if t not in ts or t in seen:
            continue
        seen.add(t)
        cfg, projs = backend.parse_protocol(q["input"])
        e, k, norm, L = backend.decompose(cfg["t"], cfg["fidbound"], cfg["rank"], cfg["fidelity"], cfg["forceL"],
                                          cfg["exact"], cfg["k"])
        rs = np.random.RandomState(t)
        Lr = [rand_word(rs, t) for _ in range(k)]
        rows = random_projector_rows(rs, t, len(projs[0][0]))
        arms = {"c3 query": (backend.projector(*projs[0]), [int(x) for x in L]),
                "random code and rows": (backend.projector(rows[0], rows[1], rows[2], t), Lr)}
        rec = {"t": t, "k": k, "rows": len(projs[0][0]), "states": count}
        for name, (P, LL) in arms.items():
            best = None
            for _ in range(2):
                gpu.singleProjectorSample(P, LL, False, count, backend.RNG_PHILOX, 11)
                st = gpu.last_stats()
                rate = st.pairs / (st.pair_kernel_ms / 1e3)
                best = rate if best is None else max(best, rate)
            rec[name] = best
        out.append(rec)
    gpu.close()
    return {"workload": "pair-kernel rates inside c3 queries vs random codes of the same t and k", "metric":
            "inner products/s (pair kernel, CUDA events)", "rates": out}


def pair_rates(count_pairs=1 << 26):
    """Pair-kernel rate of each thread-per-pair kernel (CSIM_OPT_PAIR_KERNEL 2
    block prefix, 3 runs, 4 occupancy classes, 5 direct restriction) at 16 and
    32 terms per thread, and the autotuner's choice: the c2 query's G' and
    code, and random projector rows (0.7 t of them) and codes at t = 24, 48,
    57, 64.  Each rate is the best of two calls of about `count_pairs` pairs
    (counter-based states, CUDA-event pair-kernel time)."""
    from circuitsimulator_gb300 import backend

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from helpers import rand_word, random_projector_rows

    cfg, projs, exact, k, norm, L = load_workload()
    cases = [("c2", cfg["t"], k, backend.projector(*projs[0]), [int(x) for x in L])]
    for t, kk in ((24, 14), (48, 16), (57, 18), (64, 14)):
        rs = np.random.RandomState(t)
        rows = random_projector_rows(rs, t, int(0.7 * t))
        cases.append(("random", t, kk, backend.projector(rows[0], rows[1], rows[2], t),
                      [rand_word(rs, t) for _ in range(kk)]))
    gpu = backend.Backend(0)
    gpu.set_option(backend.OPT_AUTOTUNE, 0)
    names = {2: "block prefix", 3: "runs", 4: "occupancy classes", 5: "direct"}
    out = []
    for name, t, kk, P, LL in cases:
        count = max(64, count_pairs >> kk)
        rec = {"case": name, "t": t, "k": kk, "states": count}
        for kern, kname in names.items():
            if kern == 3 and (1 << kk) % (64 * 32):
                continue
            for pt in (16, 32):
                gpu.set_option(backend.OPT_PAIR_KERNEL, kern)
                gpu.set_option(backend.OPT_PER_THREAD, pt)
                best = 0.0
                for _ in range(2):
                    gpu.singleProjectorSample(P, LL, False, count, backend.RNG_PHILOX, 7)
                    st = gpu.last_stats()
                    best = max(best, st.pairs / (st.pair_kernel_ms / 1e3))
                rec["%s pt %d" % (kname, pt)] = best
        out.append(rec)
    gpu.set_option(backend.OPT_PAIR_KERNEL, 0)
    gpu.set_option(backend.OPT_PER_THREAD, 0)
    gpu.set_option(backend.OPT_AUTOTUNE, 1)
    tuned_names = {0: "block prefix", 1: "runs", 2: "occupancy classes", 3: "direct"}
    for rec, (name, t, kk, P, LL) in zip(out, cases):
        pt, lz, ms, kern = gpu.autotune(t, P, LL)
        rec["tuned"] = {"kernel": tuned_names[kern], "terms_per_thread": pt, "light_zero_bound": lz}
    gpu.close()
    return {"workload": "pair-kernel rates per kernel, c2 and random codes", "metric":
            "inner products/s (pair kernel, CUDA events)", "rates": out}


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores (the oracle port of
    libcirc/stabilizer.c + stateprep.c + innerprod.c: the reference's own C
    code is not available on the GPU machine), one bounded sample per step."""
    if rank != 0:
        return None
    cfg, projs = parse_protocol(open(WORKLOAD).read())
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_ffi import ORACLE_SO, Oracle, make_projector

    if not os.path.exists(ORACLE_SO):
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    O = Oracle()
    kind = "port"
    t = cfg["t"]
    r1 = O.rng(1)
    exact, k, norm, L = O.decompose(t, cfg["fidbound"], cfg["rank"], cfg["fidelity"], cfg["forceL"], cfg["exact"],
                                    cfg["k"], r1)
    ph, xs, zs, nq = projs[0]
    P = make_projector(ph, xs, zs, nq)
    r = O.rng(777)
    cores = os.cpu_count() or 1
    per_step_s = 6.0
    rates = []
    nj = None
    for i in range(args.warmup + args.steps):
        thetas = []
        while len(thetas) < 2:
            s = O.random_state(t, r)
            if O.project(s, P) != 0:
                thetas.append(s[0])
        th = np.array(thetas)
        if nj is None:
            t0 = time.perf_counter()
            O.term_products(t, 0, L, k, th, 0, 32, threads=cores)
            cal = (time.perf_counter() - t0) / 64
            nj = int(max(32, min(2 ** k, per_step_s / max(cal, 1e-9) / 2)))
        j0 = (i * nj) % (2 ** k - nj + 1)
        t0 = time.perf_counter()
        O.term_products(t, 0, L, k, th, j0, nj, threads=cores)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            rates.append((2 * nj, dt))
    pairs = sum(a for a, _ in rates)
    secs = sum(b for _, b in rates)
    value = pairs / secs
    sample = "per step: 2 projected states x %d terms of the c2 code (t=40) on %d threads" % (nj, cores)
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (host C)",
            "data": "synthetic: tests/golden/workload_c2.txt",
            "config": {"workload": "c2: t=40, chi=2^16 (k=16 code) -- bounded sample per step", "t": t, "k": k},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--samples", type=int, default=None,
                    help="states per projector per step (default: the workload's L = 4096); smaller values are "
                         "profiling cases, not bench lines")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU-baseline leg (profiling runs)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-vs-plain queries/s leg")
    ap.add_argument("--no-tune", action="store_true",
                    help="fixed launch rules instead of the autotuner (profiling runs: a fixed launch sequence; on "
                         "this workload the tuner picks the same launch)")
    ap.add_argument("--pair-rates", action="store_true",
                    help="only time each thread-per-pair kernel at t = 24..64 (c2 and random codes)")
    ap.add_argument("--pair-kernel", type=int, default=None,
                    help="force the pair kernel (CSIM_OPT_PAIR_KERNEL: 2 block prefix, 3 runs, 4 occupancy classes, "
                         "5 direct restriction); with --no-tune a fixed launch sequence of that kernel")
    ap.add_argument("--per-thread", type=int, default=None, help="force terms per thread (CSIM_OPT_PER_THREAD)")
    ap.add_argument("--chain", default=None, metavar="SHOTSxBITS",
                    help="only time sampleQubits chains on the c4 circuit, plain vs batched (e.g. 16x4)")
    ap.add_argument("--chain-samples", type=int, default=None, help="L per conditional for --chain")
    ap.add_argument("--chain-groups", type=int, default=2,
                    help="shot groups of the batched --chain arm (1: one csim_run_queries call per step)")
    ap.add_argument("--serve", default=None, metavar="RATES",
                    help="only time serving under Poisson arrivals at these rates (queries/s, comma separated)")
    ap.add_argument("--serve-count", type=int, default=300, help="queries per rate for --serve")
    ap.add_argument("--serve-c5", action="store_true", help="--serve on the c5 stream (all t, every eps)")
    ap.add_argument("--c3-full", action="store_true",
                    help="only time all 256 c3 queries, plain vs batched (about 10 minutes per arm)")
    ap.add_argument("--c3-every", type=int, default=None, metavar="N",
                    help="only time every N-th of the 256 c3 queries, plain vs batched")
    ap.add_argument("--c3-rates", action="store_true",
                    help="only time the pair kernel inside c3 queries against random codes of the same t and k")
    args = ap.parse_args()
    if args.pair_rates:
        print(json.dumps(pair_rates()))
        return
    if args.c3_rates:
        print(json.dumps(c3_rates()))
        return
    if args.c3_full or args.c3_every:
        from circuitsimulator_gb300 import backend

        print(json.dumps(batch_compare(backend.Backend(0), reps=1, light=False, every=args.c3_every or 1)))
        return
    if args.serve:
        rates = [float(r) for r in args.serve.split(",")]
        print(json.dumps([serve_compare(r, args.serve_count, c5=args.serve_c5) for r in rates]))
        return
    if args.chain:
        shots, nbits = (int(v) for v in args.chain.lower().split("x"))
        print(json.dumps(chain_compare(shots, nbits, args.chain_samples, args.chain_groups)))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    else:
        if world > 1:
            import torch

            torch.cuda.set_device(local_rank)
            torch.distributed.init_process_group("nccl")
        out = run_ours(args, rank, world, local_rank)
        if world > 1:
            import torch

            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
