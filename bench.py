"""Benchmark of the similarity hot path: exact top-10 search over a
1,000,000 x 768 FP64 store (1,024-centre Gaussian mixture, sigma 0.05, seed
3), query batches drawn from the same mixture.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision bf16|fp8|fp64] [--q Q] [--metric cosine|euclidean|dot]

One step = one batch of Q queries answered end to end by the library's
top-k search.  `value` is queries/s with queries and results resident in HBM
(svdb_search_topk_device, timed with CUDA events on the library's stream);
`e2e` is the same metric through svdb_search_topk with host buffers
(host->device query upload and device->host result read inside the timed
region).  The store (6.1 GB FP64 + shadows) is far larger than L2, so every
step streams it from HBM.

--impl reference times the CPU path on the host cores instead: the FP64
brute-force top-k restated from the reference's metric formulas
(oracle/svdb_oracle.c), all host threads, on a bounded query sample.

Under torchrun (N > 1) every rank holds a full replica of the store and
answers its own query batches (replicas only: no collective); value is the
queries of all ranks over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "simple-vector-db_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRICS = {"cosine": 0, "euclidean": 1, "dot": 2}
N_ROWS, DIM, K_TOP, SEED = 1_000_000, 768, 10, 3
N_ROWS_DEFAULT = N_ROWS
METRIC_NAME = "exact top-10 queries/s, 1Mx768: BF16+FP64-rerank vs plain FP64 GPU; p50/p99 ms"
# DRAM bytes (read + write) of one k_screen_bf16 launch per store row, from an
# ncu capture of the screen on a 200,000-row store of the same mixture with the
# same 4096 cosine queries (the shadow is read once per launch, so the bytes
# grow with the rows and a full launch is this times N).  None when no capture
# of the current kernel exists.
SCREEN_DRAM_BYTES_PER_ROW = (419.859712e6 + 19.900160e6) / 200_000


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        j = json.load(open(p))
        return j["hbm_gbs"], j["bf16_tflops"], "measured"
    return 6800.0, 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        out, _ = self.p.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workloads():
    """The seeded workload generators (svdb_gb300/workloads.py, numpy only),
    loaded from their file so that the CPU reference arm never imports the
    package, whose import loads the CUDA library."""
    import importlib.util
    name = "svdb_workloads_standalone"
    if name not in sys.modules:
        spec = importlib.util.spec_from_file_location(name, os.path.join(PKG, "svdb_gb300", "workloads.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules[name] = mod
    return sys.modules[name]


def headline_config(args, ws):
    """The workload both arms measure (identical dicts: the reference arm
    times a bounded sample of it, described in its cpu_baseline)."""
    return {"workload": f"1M x 768 FP64 Gaussian mixture (1024 centres, sigma 0.05, seed 3), exact top-{K_TOP} "
                        f"{args.metric}", "rows": N_ROWS, "dim": DIM, "k": K_TOP, "metric": args.metric,
            "query_batch": args.q, "parallelism": f"replicas{ws}",
            "l2": "store (6.1 GB FP64) larger than L2; no flush needed"}


def guard_sample(nq):
    """Queries checked against the oracle: one in every 128-query tile (its
    middle), plus the batch's first and last."""
    return np.union1d(np.arange(64, nq, 128), [0, nq - 1]) if nq > 1 else np.array([0])


def oracle_topk(X, Q, metric, k):
    import oracle as O
    O.build(ref=False)
    return O.Oracle().topk(metric, X, Q, k, threads=os.cpu_count() or 1)


def cpu_baseline(X, Q, metric, k, sample, threads):
    """Oracle FP64 brute force on `sample` queries, all given threads."""
    import oracle as O
    O.build(ref=False)
    o = O.Oracle()
    q = Q[:sample]
    t = time.perf_counter()
    o.topk(metric, X, q, k, threads=threads)
    dt = time.perf_counter() - t
    return sample / dt, dt


def run_reference(args, ws, rank):
    """The CPU path: the oracle's multi-threaded FP64 brute force (the
    reference's metric formulas over every stored row, heap top-k) on all
    host cores, each step a bounded sample of the headline batch.  Touches
    neither the GPU nor the CUDA library."""
    if rank != 0:
        return
    W = workloads()
    mix, X = W.config3(N_ROWS, DIM, SEED)
    metric = METRICS[args.metric]
    threads = os.cpu_count() or 1
    times = []
    sample = min(args.cpu_sample, args.q)
    Qs = mix.sample(sample * (args.steps + args.warmup), 1)
    for s in range(args.warmup + args.steps):
        _, dt = cpu_baseline(X, Qs[s * sample:], metric, K_TOP, sample, threads)
        if s >= args.warmup:
            times.append(dt)
    tot = sum(times)
    v = sample * args.steps / tot
    line = {"impl": "reference", "metric": METRIC_NAME, "value": v, "unit": "queries/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": headline_config(args, ws),
            "cpu_baseline": {"value": v, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} queries of the {args.q}-query batch per step over the full "
                                       f"1M x 768 store (FP64 brute force, {threads} threads)"},
            "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import torch
    import svdb_gb300 as S
    W = workloads()

    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    metric = METRICS[args.metric]
    prec = {"bf16": S.PREC_BF16, "fp8": S.PREC_FP8, "fp64": S.PREC_FP64}[args.precision]
    nq, k = args.q, K_TOP

    t0 = time.perf_counter()
    mix, X = W.config3(N_ROWS, DIM, SEED)
    nbatch = 4
    Qh = [mix.sample(nq, 1 + rank * nbatch + b) for b in range(nbatch)]
    log(f"[bench] data {time.perf_counter() - t0:.1f}s")
    t0 = time.perf_counter()
    db = S.VectorDatabase(N_ROWS, 3)
    db.reserve(N_ROWS, DIM)
    db.insert_batch(X)
    db.sync()
    db.set_fp8_screen(1)  # FP8 lines time the E4M3 screen at every batch size, as asked
    log(f"[bench] store load {time.perf_counter() - t0:.1f}s")

    stream = torch.cuda.ExternalStream(db.stream())
    Qd = [torch.from_numpy(q).cuda() for q in Qh]
    ids = torch.empty((nq, k), dtype=torch.int64, device="cuda")
    dists = torch.empty((nq, k), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = S.SearchStats()

    def step(b, stats=None, p=None):
        q = Qd[b % nbatch]
        db.search_device(q.data_ptr(), nq, DIM, k, metric, prec if p is None else p, ids.data_ptr(), dists.data_ptr(),
                         0, stats)

    # correctness guard (outside the timed region): the whole first batch is
    # searched as measured, and a sample of its queries spread over every
    # 128-query tile must equal the oracle's FP64 brute force (ids and values)
    guard = guard_sample(nq)
    want_guard = oracle_topk(X, Qh[0][guard], metric, k)

    def check_guard(p, what):
        gi, gv = db.search(Qh[0], k, metric, p)
        if not (np.array_equal(gi[guard], want_guard[0]) and np.array_equal(gv[guard], want_guard[1])):
            raise SystemExit(f"bench: {what} top-k differs from the oracle on the guard sample")

    check_guard(prec, args.precision)

    for w in range(args.warmup):
        step(w)
    step(0, st)  # the candidate funnel and launch count of one search (statistics cost a host round trip)
    launches_per_step = st.kernels
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    db.profile(True)
    db.profile_read(reset=True)
    clocks = Clocks(local)
    kernels = 0
    per_step = []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    for s in range(args.steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step(s)
        kernels += launches_per_step
        b.record(stream)
        per_step.append((a, b))
    ev1.record(stream)
    torch.cuda.synchronize()
    cl = clocks.stop()
    ncalls, stage_ms = db.profile_read(reset=True)
    db.profile(False)
    ms = ev0.elapsed_time(ev1)
    lat = sorted(a.elapsed_time(b) for a, b in per_step)
    if dist:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * nq * args.steps / (ms / 1e3)

    # the FP8 screen (BF16-seeded thresholds, E4M3 tensor-core screen, same
    # refinement and re-rank) on the same batches, for comparison
    fp8 = None
    if prec == S.PREC_BF16 and metric == S.COSINE and rank == 0:
        check_guard(S.PREC_FP8, "fp8")
        for w in range(args.warmup):
            step(w, p=S.PREC_FP8)
        st8 = S.SearchStats()
        step(0, st8, p=S.PREC_FP8)
        db.profile(True)
        db.profile_read(reset=True)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for s_ in range(args.steps):
            step(s_, p=S.PREC_FP8)
        e1.record(stream)
        torch.cuda.synchronize()
        n8, stage8 = db.profile_read(reset=True)
        db.profile(False)
        ms8 = e0.elapsed_time(e1)
        fp8 = {"value": nq * args.steps / (ms8 / 1e3), "unit": "queries/s", "ms_per_step": ms8 / args.steps,
               "stage_ms_per_step": {n: float(stage8[i] / max(n8, 1)) for i, n in
                                     enumerate(("prep", "screen", "select", "refine", "rerank"))},
               "funnel_per_query": {"screen_candidates": st8.candidates / nq, "survivors": st8.survivors / nq,
                                    "fp64_reranked": st8.reranked / nq, "widened_queries": st8.widened,
                                    "bound_failures": st8.bound_failures}}

    # the same searches replayed from captured CUDA graphs: one one-part plan
    # (svdb_ragged_*) per batch buffer, one graph launch per step (the kernels
    # of a search are launched back to back by the GPU instead of the host)
    graph = None
    if rank == 0 and nq <= 1024:
        ks = np.full(nq, k, np.int64)
        plans = [S.RaggedPlan([(db, Qd[b].data_ptr(), nq, DIM, ks, ids.data_ptr(), dists.data_ptr(), k)], metric,
                              prec, 0) for b in range(nbatch)]
        for w in range(max(args.warmup, 1)):
            plans[w % nbatch].run()
        for pl in plans:
            pl.wait()
        t = time.perf_counter()
        for s in range(args.steps):
            plans[s % nbatch].run()
            plans[s % nbatch].wait()
        gs = time.perf_counter() - t
        t = time.perf_counter()
        for s in range(args.steps):  # the direct search, timed the same way
            step(s)
            stream.synchronize()
        ds = time.perf_counter() - t
        graph = {"value": nq * args.steps / gs, "unit": "queries/s", "ms_per_step": 1e3 * gs / args.steps,
                 "direct_ms_per_step": 1e3 * ds / args.steps,
                 "how": "one graph launch per step (a one-part plan per batch buffer) against the direct search "
                        "(its kernels launched by the host), both timed by the host clock around the call and "
                        "the wait for it"}
        ids_g = ids.cpu().numpy()
        db.search_device(Qd[(args.steps - 1) % nbatch].data_ptr(), nq, DIM, k, metric, prec, ids.data_ptr(),
                         dists.data_ptr(), 0)
        torch.cuda.synchronize()
        if not np.array_equal(ids_g, ids.cpu().numpy()):
            raise SystemExit("bench: graph replay results differ from the direct search")
        for pl in plans:
            pl.close()

    # e2e: host buffers through svdb_search_topk (query upload + result read
    # inside), queries and results in page-locked host memory
    Qp = [torch.from_numpy(q).pin_memory().numpy() for q in Qh]
    ids_h = torch.empty((nq, k), dtype=torch.int64).pin_memory().numpy()
    dists_h = torch.empty((nq, k), dtype=torch.float64).pin_memory().numpy()
    for w in range(min(args.warmup, 2)):
        db.search(Qp[w % nbatch], k, metric, prec, out=(ids_h, dists_h))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t = time.perf_counter()
    for s in range(args.steps):
        db.search(Qp[s % nbatch], k, metric, prec, out=(ids_h, dists_h))
    e2e_s = time.perf_counter() - t
    if dist:
        tt = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    e2e = ws * nq * args.steps / e2e_s

    # other batch sizes and metrics on the same store, device-resident queries,
    # CUDA events on the library's stream (reported beside the headline)
    batches = None
    if rank == 0 and args.extra:
        batches = {}

        def timed(qn, m, p, steps):
            for w in range(3):
                db.search_device(Qd[w % nbatch].data_ptr(), qn, DIM, k, m, p, ids.data_ptr(), dists.data_ptr(), 0)
            a_ = torch.cuda.Event(enable_timing=True)
            b_ = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            a_.record(stream)
            for s_ in range(steps):
                db.search_device(Qd[s_ % nbatch].data_ptr(), qn, DIM, k, m, p, ids.data_ptr(), dists.data_ptr(), 0)
            b_.record(stream)
            torch.cuda.synchronize()
            ms_ = a_.elapsed_time(b_) / steps
            return {"queries_per_s": qn / (ms_ / 1e3), "ms_per_batch": ms_}

        for mname in ("cosine", "euclidean"):
            m = METRICS[mname]
            for qn in (1, 64, 1024):
                batches[f"{mname}_bf16_q{qn}"] = timed(qn, m, S.PREC_BF16, 20)
            batches[f"{mname}_bf16_q{nq}"] = timed(nq, m, S.PREC_BF16, 10)
            batches[f"{mname}_fp8_q{nq}"] = timed(nq, m, S.PREC_FP8, 10)
        gi, gv = db.search(Qh[0], k, S.EUCLIDEAN, S.PREC_FP8)  # the FP8 Euclidean path, guarded too
        want_e = oracle_topk(X, Qh[0][guard], S.EUCLIDEAN, k)
        if not (np.array_equal(gi[guard], want_e[0]) and np.array_equal(gv[guard], want_e[1])):
            raise SystemExit("bench: fp8 euclidean top-k differs from the oracle on the guard sample")

    # a short serving trace on a second, server-side store of the same size:
    # Poisson arrivals at --rate (70 % /nearest top-10, 10 % /compare, 15 %
    # insert, 3 % update, 2 % delete), batched as they arrive
    served = None
    if rank == 0 and args.extra and args.serve_seconds_headline > 0:
        from svdb_gb300 import serve
        m5 = W.Mixture(DIM, 5)
        nreq = int(args.rate * args.serve_seconds_headline)
        srv = serve.Server(DIM, N_ROWS + 2 * nreq + 4096)
        st_ = 1000
        while srv.size < N_ROWS:
            srv.insert_block(m5.sample(min(1 << 18, N_ROWS - srv.size), st_))
            st_ += 1
        serve.replay(srv, serve.make_trace(m5.sample, srv.size, max(1000, nreq // 4), args.rate, seed=50),
                     S.PREC_BF16)
        tr = serve.make_trace(m5.sample, srv.size, nreq, args.rate, seed=5)
        r_ = serve.replay(srv, tr, S.PREC_BF16)
        served = {"store_rows": N_ROWS, "offered_per_s": args.rate, "trace_s": args.serve_seconds_headline,
                  "requests": r_["requests"], "served_per_s": r_["served_per_s"], "p50_ms": r_["p50_ms"],
                  "p99_ms": r_["p99_ms"], "max_ms": r_["max_ms"], "mean_batch": r_["mean_batch"],
                  "widened": r_["widened"], "bound_failures": r_["bound_failures"], "mix": tr.counts(),
                  "how": "svdb_server_execute batches formed as requests arrive (host clock: completion - "
                         "arrival, queueing included); rows from pageable host memory"}
        srv.close()

    # plain FP64 GPU path on the same batches (the comparison the metric names)
    plain = None
    if prec != S.PREC_FP64 and args.plain_q:
        pq = min(args.plain_q, nq)
        db.search_device(Qd[0].data_ptr(), pq, DIM, k, metric, S.PREC_FP64, ids.data_ptr(), dists.data_ptr(), 0)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for s in range(2):
            db.search_device(Qd[s % nbatch].data_ptr(), pq, DIM, k, metric, S.PREC_FP64, ids.data_ptr(),
                             dists.data_ptr(), 0)
        b.record(stream)
        torch.cuda.synchronize()
        plain = 2 * pq / (a.elapsed_time(b) / 1e3)

    hbm, bf16, src = peaks()
    scr = stage_ms[S.STAGE_SCREEN] / max(ncalls, 1)  # ms per launch of the dominant stage
    if prec == S.PREC_BF16:
        flops = 2.0 * nq * N_ROWS * DIM
        ach = flops / (scr / 1e3) / 1e12
        traffic = SCREEN_DRAM_BYTES_PER_ROW * N_ROWS if SCREEN_DRAM_BYTES_PER_ROW else None
        roof = {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16,
                "traffic": traffic, "traffic_unit": "bytes per launch (ncu, scaled by rows)",
                "algorithmic_bytes": N_ROWS * DIM * 2 + nq * DIM * 2, "peak_source": src, "kernel_ms": scr,
                "algorithmic": f"2*Q*N*D = {flops:.3e} FLOP per launch"}
    elif prec == S.PREC_FP8:
        # dense FP8 runs at twice the BF16 rate on this part; the measured BF16 peak x 2 is the denominator
        flops = 2.0 * nq * N_ROWS * DIM
        ach = flops / (scr / 1e3) / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": 2 * bf16, "unit": "TFLOP/s", "frac": ach / (2 * bf16),
                "traffic": None, "algorithmic_bytes": N_ROWS * DIM + nq * DIM, "peak_source": src + " bf16 x 2",
                "kernel_ms": scr, "algorithmic": f"2*Q*N*D = {flops:.3e} FLOP per launch (E4M3)"}
    else:
        nbytes = N_ROWS * (DIM * 8 + 1)
        ach = nbytes / (scr / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm, "traffic": None,
                "peak_source": src, "kernel_ms": scr,
                "algorithmic": f"N*(D*8+1) = {nbytes:.3e} bytes per launch (one pass over the FP64 master)"}

    cpu = None
    if rank == 0 and ws == 1 and args.cpu_sample:
        v, dt = cpu_baseline(X, Qh[0], metric, k, args.cpu_sample, os.cpu_count() or 1)
        cpu = {"value": v, "unit": "queries/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"{args.cpu_sample} queries over the full 1M x 768 store ({dt:.1f} s)"}

    if rank == 0:
        line = {"metric": METRIC_NAME, "value": value, "unit": "queries/s", "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": {S.PREC_BF16: "bf16+f64", S.PREC_FP8: "e4m3+f32+f64"}.get(prec, "f64"),
                "data": "synthetic", "precision": args.precision, "config": headline_config(args, ws),
                "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
                "stage_ms_per_step": {n: float(stage_ms[i] / max(ncalls, 1)) for i, n in
                                      enumerate(["prep", "screen", "select", "refine", "rerank"])},
                "plain_fp64_qps": plain,
                "funnel_per_query": {"screen_candidates": st.candidates / nq, "survivors": st.survivors / nq,
                                     "fp64_reranked": st.reranked / nq, "widened_queries": st.widened,
                                     "bound_failures": st.bound_failures},
                "e2e": {"value": e2e, "unit": "queries/s", "h2d_bytes_per_step": nq * DIM * 8,
                        "d2h_bytes_per_step": nq * k * 16},
                "gpu_launches": kernels, "roofline": roof, "cpu_baseline": cpu, "clocks": cl}
        if fp8:
            line["fp8_screen"] = fp8
        if batches:
            line["batches"] = batches
        if served:
            line["serve_20k"] = served
        if graph:
            line["graph_replay"] = graph
        print(json.dumps(line), flush=True)
    db.close()
    if dist:
        dist.destroy_process_group()


def run_scan128(args, ws, rank, local):
    """Plain FP64 single-query scan at scale: 1M x 128 L2-normalised N(0,1)
    rows (seed 2), queries issued one at a time, top-1 and top-10 for each
    metric.  Reported against the FP64 pipe (the scan's bound on GB300) and as
    HBM bytes per second."""
    import torch
    import svdb_gb300 as S
    W = workloads()

    torch.cuda.set_device(local)
    n, d = args.rows if args.rows != N_ROWS_DEFAULT else 1_000_000, 128
    X, Q = W.config2(n, d, max(args.steps, 1) + args.warmup)
    db = S.VectorDatabase(n, 3)
    db.insert_batch(X)
    db.sync()
    Qd = torch.from_numpy(Q).cuda()
    stream = torch.cuda.ExternalStream(db.stream())
    results = {}
    for metric_name, metric in METRICS.items():
        for k in (1, 10):
            ids = torch.empty((1, k), dtype=torch.int64, device="cuda")
            dists = torch.empty((1, k), dtype=torch.float64, device="cuda")
            for w in range(args.warmup):
                db.search_device(Qd[w].data_ptr(), 1, d, k, metric, S.PREC_FP64, ids.data_ptr(), dists.data_ptr())
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for s_ in range(args.steps):
                q = Qd[args.warmup + s_]
                db.search_device(q.data_ptr(), 1, d, k, metric, S.PREC_FP64, ids.data_ptr(), dists.data_ptr())
            b.record(stream)
            torch.cuda.synchronize()
            ms = a.elapsed_time(b) / args.steps
            results[f"{metric_name}_top{k}"] = {"queries_per_s": 1e3 / ms, "ms_per_query": ms,
                                               "hbm_gbs": n * d * 8 / (ms / 1e3) / 1e9,
                                               "fp64_tflops": 2.0 * n * d / (ms / 1e3) / 1e12}
    hbm, _, src = peaks()
    best = max(results.values(), key=lambda r: r["queries_per_s"])
    line = {"metric": "plain FP64 single-query scan, 1M x 128, queries/s", "value": best["queries_per_s"],
            "unit": "queries/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": best["ms_per_query"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "1M x 128 L2-normalised N(0,1) FP64 (seed 2), one query per step, FP64 scan"},
            "per_case": results,
            "roofline": {"bound": "fp64 pipe (HBM figure for reference)", "achieved": best["hbm_gbs"], "peak": hbm,
                         "unit": "GB/s", "frac": best["hbm_gbs"] / hbm, "traffic": None, "peak_source": src}}
    print(json.dumps(line), flush=True)
    db.close()


def run_ragged(args, ws, rank, local):
    """Uneven batched multi-collection search: 5 collections (D, N) =
    (64, 2M), (128, 1M), (384, 500k), (768, 200k), (1536, 50k), uniform[-1,1]
    float64 (seed 4); a ragged batch of 8,192 queries split 40/25/15/12/8 %,
    k per query uniform in [1, 100], cosine.  The batch is one ragged plan
    (svdb_ragged_*): bound once, autotuned, captured as one CUDA graph; one
    step is one run of the plan (one graph launch) over all five collections,
    each query answered with its own k."""
    import torch
    import svdb_gb300 as S
    W = workloads()

    torch.cuda.set_device(local)
    prec = S.PREC_BF16 if args.precision == "bf16" else S.PREC_FP64
    cols = W.config4(8192)
    tune = {"auto": S.RAGGED_AUTOTUNE, "fused": S.RAGGED_FUSED, "per-store": 0}[args.ragged_plan]
    if args.ragged_part:  # one collection's queries of one k class, default choices (small ncu captures)
        c, kc = (int(x) for x in args.ragged_part.split(":"))
        X, Q, ks = cols[c]
        sel = [ks <= 16, (ks > 16) & (ks <= 32), ks > 32][kc]
        cols = [(X, Q[sel], ks[sel])]
        tune = 0
    dbs, bufs, parts = [], [], []
    for X, Q, ks in cols:
        db = S.VectorDatabase(X.shape[0], 3)
        db.insert_batch(X)
        db.sync()
        stride = int(ks.max())
        qd = torch.from_numpy(Q).cuda()
        ids = torch.empty((Q.shape[0], stride), dtype=torch.int64, device="cuda")
        dd = torch.empty((Q.shape[0], stride), dtype=torch.float64, device="cuda")
        dbs.append(db)
        bufs.append((qd, ids, dd))
        parts.append((db, qd.data_ptr(), Q.shape[0], Q.shape[1], ks, ids.data_ptr(), dd.data_ptr(), stride))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    plan = S.RaggedPlan(parts, S.COSINE, prec, tune)
    tune_s = time.perf_counter() - t0
    info = plan.info()

    # correctness guard: a few queries of every collection against the oracle
    plan.run()
    plan.wait()
    for (X, Q, ks), db, (_, ids, dd) in zip(cols, dbs, bufs):
        gi, gd = ids.cpu().numpy(), dd.cpu().numpy()
        for i in (0, Q.shape[0] // 2, Q.shape[0] - 1):
            k = int(ks[i])
            wi, wv = oracle_topk(X, Q[i:i + 1], S.COSINE, k)
            if not (np.array_equal(gi[i, :k], wi[0]) and np.array_equal(gd[i, :k], wv[0])):
                raise SystemExit("bench: ragged plan results differ from the oracle")

    # CPU baseline: the oracle's FP64 brute force on all host cores over a
    # sample of each collection's queries (each with its own k), weighted by
    # the collections' query shares
    cpu = None
    if args.cpu_sample > 0:
        threads = os.cpu_count() or 1
        per_q_s = 0.0
        nq_all = sum(Q.shape[0] for _, Q, _ in cols)
        for X, Q, ks in cols:
            m = min(max(1, args.cpu_sample // 16), Q.shape[0])
            t = time.perf_counter()
            for i in range(m):
                oracle_topk(X, Q[i:i + 1], S.COSINE, int(ks[i]))
            per_q_s += (time.perf_counter() - t) / m * (Q.shape[0] / nq_all)
        cpu = {"value": 1.0 / per_q_s, "unit": "queries/s", "cores": threads, "kind": "port",
               "sample": f"{min(max(1, args.cpu_sample // 16), 1 << 30)} queries per collection (their own k), "
                         f"the oracle's FP64 brute force, weighted by the collections' query shares"}
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.ExternalStream(plan.stream())
    for _ in range(args.warmup):
        plan.run()
    plan.wait()
    clk = Clocks(local)
    ev0.record(stream)
    for _ in range(args.steps):
        plan.run()
    ev1.record(stream)
    plan.wait()
    clocks = clk.stop()
    dt = ev0.elapsed_time(ev1) / 1e3
    nq = sum(b[0].shape[0] for b in bufs)
    line = {"metric": "exact top-k queries/s, ragged batch over 5 collections (k in [1,100])",
            "value": nq * args.steps / dt, "unit": "queries/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16+f64" if prec == S.PREC_BF16 else "f64",
            "data": "synthetic",
            "config": {"workload": "5 collections (D,N) = (64,2M) (128,1M) (384,500k) (768,200k) (1536,50k), "
                                   "uniform[-1,1] seed 4, 8192 queries split 40/25/15/12/8 %, k ~ U[1,100], cosine",
                       "precision": args.precision, "l2": "stores (5.4 GB FP64) larger than L2; no flush needed",
                       "part": args.ragged_part or "all", "plan": args.ragged_plan},
            "plan": {"grouping": info["grouping"], "concurrent": info["concurrent"], "graph": info["graph"],
                     "searches_per_run": info["searches"], "graph_launches_per_step": 1,
                     "fp8_screen_stores": [i for i in range(5) if info["fp8_stores"] >> i & 1],
                     "autotune_ms_per_run": {"(grouping 0, concurrent 1)": info["tuned_ms"][0],
                                             "(1, 1)": info["tuned_ms"][1], "(0, 0)": info["tuned_ms"][2],
                                             "(1, 0)": info["tuned_ms"][3]},
                     "autotune_ms_fused_screen": {"grouping 0": info["fused_ms"][0],
                                                  "grouping 1": info["fused_ms"][1]},
                     "fused_screen": info["fused"], "fused_launches_per_run": info["fused_launches"],
                     "fused_epilogue_weight": info["epi_weight"],
                     "autotune_ms_fused_epilogue_weight_1_4_8": info["weight_ms"],
                     "seeded_thresholds": info["seeded"], "autotune_ms_seeded": info["seed_ms"],
                     "autotune_ms_with_store_screen_swapped": info["swap_ms"][:5],
                     "autotune_s": tune_s, "captures": info["captures"]},
            "cpu_baseline": cpu, "clocks": clocks}
    print(json.dumps(line), flush=True)
    plan.close()
    for db in dbs:
        db.close()


def run_serve(args, ws, rank, local):
    """Serving loop: a server store (rows only in HBM) of the D=768 mixture
    (1,024 centres, sigma 0.05, seed 5) grown from 1M to 5M rows; at each
    size a seeded Poisson trace at --rate requests/s (70 % /nearest top-10
    Euclidean, 10 % /compare with a uniform metric, 15 % insert, 3 % update,
    2 % delete) is served open-loop in real time by svdb_server_execute
    batches (BF16 screen + FP64 re-rank), then a second trace at the same
    offered load through the plain FP64 path, cut off after --fp64-seconds.
    Latency = completion - arrival per request, queueing included; the rows
    of every request come from pageable host memory and every answer goes
    back to it."""
    import torch
    import svdb_gb300 as S
    from svdb_gb300 import serve
    W = workloads()

    torch.cuda.set_device(local)
    m = W.Mixture(DIM, 5)
    sizes = [int(x) for x in args.serve_sizes.split(",")]
    nreq = int(args.rate * args.serve_seconds)
    reserve = max(sizes) + 2 * nreq
    t = time.perf_counter()
    srv = serve.Server(DIM, reserve)  # admission: the whole capacity must fit in free HBM now
    log(f"[bench] server store reserved for {reserve} rows ({time.perf_counter() - t:.1f}s)")
    phases, chunk, stream = [], 1 << 18, 1000
    clocks = Clocks(local)
    for si, size in enumerate(sizes):
        t = time.perf_counter()
        while srv.size < size:
            srv.insert_block(m.sample(min(chunk, size - srv.size), stream))
            stream += 1
        log(f"[bench] store at {srv.size} rows ({time.perf_counter() - t:.1f}s)")
        warm = serve.make_trace(m.sample, srv.size, max(1000, nreq // 10), args.rate, seed=50 + si)
        serve.replay(srv, warm, S.PREC_BF16)
        tr = serve.make_trace(m.sample, srv.size, nreq, args.rate, seed=5 + si)
        n_at_start = srv.size
        res = serve.replay(srv, tr, S.PREC_BF16)
        log(f"[bench] bf16 served {res['requests']}/{res['offered']} p50 {res['p50_ms']:.2f} p99 "
            f"{res['p99_ms']:.2f} ms, mean batch {res['mean_batch']:.1f}")
        trf = serve.make_trace(m.sample, srv.size, nreq, args.rate, seed=500 + si)
        resf = serve.replay(srv, trf, S.PREC_FP64, max_batch=256, time_limit=args.fp64_seconds)
        log(f"[bench] fp64 served {resf['requests']}/{resf['offered']} in {resf['wall_s']:.1f}s, p99 "
            f"{resf['p99_ms']:.1f} ms")
        phases.append({
            "store_rows": n_at_start, "offered_per_s": args.rate, "requests": res["requests"],
            "served_per_s": res["served_per_s"], "p50_ms": res["p50_ms"], "p99_ms": res["p99_ms"],
            "max_ms": res["max_ms"], "mean_batch": res["mean_batch"], "widened": res["widened"],
            "bound_failures": res["bound_failures"], "statuses": res["statuses"], "mix": tr.counts(),
            "plain_fp64": {"requests": resf["requests"], "offered": resf["offered"],
                           "served_per_s": resf["served_per_s"], "p50_ms": resf["p50_ms"],
                           "p99_ms": resf["p99_ms"], "cut_off_s": args.fp64_seconds}})
    clk = clocks.stop()
    total = sum(p["requests"] for p in phases)
    wall = sum(p["requests"] / p["served_per_s"] for p in phases)
    line = {"metric": f"served requests/s at {args.rate:.0f} req/s offered (70% /nearest top-10, 10% /compare, "
                      "15% insert, 3% update, 2% delete), store 1M->5M x 768; p50/p99 ms",
            "value": total / wall, "unit": "requests/s", "n_gpus": 1, "steps": len(phases), "warmup": len(phases),
            "ms_per_step": 1e3 * wall / len(phases), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16+f64", "data": "synthetic",
            "config": {"workload": "serving loop: D=768 mixture (1024 centres, sigma 0.05, seed 5), Poisson "
                                   f"arrivals at {args.rate:.0f}/s, {args.serve_seconds:.1f}s of trace per store "
                                   "size", "store_sizes": sizes, "precision": "bf16",
                       "l2": "store larger than L2"},
            "latency_ms": {"p50": max(p["p50_ms"] for p in phases), "p99": max(p["p99_ms"] for p in phases)},
            "phases": phases, "clocks": clk}
    print(json.dumps(line), flush=True)
    srv.close()


def run_uuid(args, ws, rank, local):
    """GET /vector?uuid= and persistence on a server store of 1,000,000 x 128
    FP64 rows (N(0,1), seed 6) with unique 36-character uuids: batches of
    4,096 lookups (90 % present, 10 % absent) through svdb_server_find_uuid
    (host keys in, host positions out: copies inside the timed region), then
    the store saved to and loaded from the reference's file format through
    HBM.  CPU baseline: the reference's linear strncmp scan (oracle port) on
    all host cores over a bounded sample of keys."""
    import tempfile

    import torch
    import svdb_gb300 as S
    from svdb_gb300 import serve

    torch.cuda.set_device(local)
    n, d, nb = 1_000_000, 128, 4096
    rng = np.random.default_rng(6)
    X = rng.normal(size=(n, d))
    hexd = np.frombuffer(b"0123456789abcdef", np.uint8)
    h = hexd[rng.integers(0, 16, (n, 32))]
    U = np.zeros((n, 37), np.uint8)
    U[:, 0:8], U[:, 9:13], U[:, 14:18], U[:, 19:23], U[:, 24:36] = h[:, 0:8], h[:, 8:12], h[:, 12:16], h[:, 16:20], h[:, 20:32]
    U[:, [8, 13, 18, 23]] = ord("-")
    table = U.tobytes()
    srv = serve.Server(d, n)
    t0 = time.perf_counter()
    first = C.c_size_t(0)
    S._check(S.lib.svdb_server_insert_rows(srv.ptr, X.ctypes.data_as(S._dp), table, n, C.byref(first)),
             "svdb_server_insert_rows")
    log(f"[bench] store + uuids {time.perf_counter() - t0:.1f}s")
    batches = []
    for b in range(4):
        pick = rng.integers(0, n, nb)
        keys = U[pick].copy()
        absent = rng.random(nb) < 0.1
        keys[absent, 0] = ord("z")  # no stored uuid starts with z
        batches.append((keys.tobytes(), np.where(absent, -1, pick)))
    out = np.empty(nb, np.int64)

    def step(b):
        keys, _ = batches[b % len(batches)]
        S._check(S.lib.svdb_server_find_uuid(srv.ptr, keys, nb, out.ctypes.data_as(S._i64p)), "find_uuid")

    for b, (keys, want) in enumerate(batches):  # correctness guard: positions equal the generator's
        step(b)
        if not np.array_equal(out, want):
            raise SystemExit("bench: uuid lookups differ from the stored positions")
    for w in range(args.warmup):
        step(w)
    clk = Clocks(local)
    t = time.perf_counter()
    for s_ in range(args.steps):
        step(s_)
    dt = time.perf_counter() - t
    clocks = clk.stop()
    lookups_s = nb * args.steps / dt

    # persistence through HBM (file of 8 + n x (45 + 8 d) bytes)
    tmpdir = tempfile.mkdtemp(prefix="svdb_bench_")
    fpath = os.path.join(tmpdir, "store.db")
    t = time.perf_counter()
    srv.save(fpath)
    save_s = time.perf_counter() - t
    fbytes = os.path.getsize(fpath)
    t = time.perf_counter()
    srv2 = serve.Server.load(fpath, d)
    srv2.find_uuid([b"warm"])
    load_s = time.perf_counter() - t
    keys, want = batches[0]
    got = np.empty(nb, np.int64)
    S._check(S.lib.svdb_server_find_uuid(srv2.ptr, keys, nb, got.ctypes.data_as(S._i64p)), "find_uuid")
    if srv2.size != n or not np.array_equal(got, want) or not np.array_equal(srv2.read(n - 1), X[n - 1]):
        raise SystemExit("bench: the loaded store differs from the saved one")
    srv2.close()
    os.remove(fpath)
    os.rmdir(tmpdir)

    cpu = None
    if args.cpu_sample > 0:
        import oracle as O
        cores = os.cpu_count() or 1
        o = O.Oracle()
        m = max(cores, min(args.cpu_sample * 512, 32768))
        t = time.perf_counter()
        res = o.find_uuid(table, batches[0][0][: m * 37], cores)
        cpu_dt = time.perf_counter() - t
        if not np.array_equal(res, batches[0][1][:m]):
            raise SystemExit("bench: oracle uuid scan disagrees")
        cpu = {"value": m / cpu_dt, "unit": "lookups/s", "cores": cores, "kind": "port",
               "sample": f"{m} lookups, each a linear strncmp scan of the 1M-row uuid array ({cpu_dt:.1f} s)"}
    line = {"metric": "GET /vector?uuid= lookups/s, 1M rows (batches of 4096, host buffers)", "value": lookups_s,
            "unit": "lookups/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u8 keys, i64 positions", "data": "synthetic",
            "config": {"workload": "server store 1M x 128 FP64 N(0,1) seed 6, unique 36-char uuids; lookups 90 % "
                                   "present / 10 % absent; persistence in the reference's file format",
                       "l2": "uuid records (40 MB) and table (68 MB) fit in L2: lookups are latency-bound"},
            "e2e": {"value": lookups_s, "unit": "lookups/s", "h2d_bytes_per_step": nb * 40,
                    "d2h_bytes_per_step": nb * 8},
            "persistence": {"file_bytes": fbytes, "save_s": save_s, "save_gbs": fbytes / save_s / 1e9,
                            "load_s": load_s, "load_gbs": fbytes / load_s / 1e9},
            "cpu_baseline": cpu, "clocks": clocks}
    print(json.dumps(line), flush=True)
    srv.close()


def run_nearest(args, ws, rank, local):
    """The reference's own CPU-runnable case and /nearest at scale.

    Part 1 (N=10,000 x 128 U[-1,1] seed 0, KD dimension 3; 1,000 queries seed
    1): per query, POST /nearest (the reference's insertion-order KD tree,
    svdb_nearest_batch) plus GET /compare against 10 random stored ids with
    cosine, Euclidean and dot (svdb_compare_batch, 30 pairs); one step = all
    1,000 queries.  Part 2 (N=1,000,000 x 128 N(0,1) seed 2, KD dimension 3;
    10,000 queries): /nearest through the insertion-order tree, and through
    the opt-in median tree (device build time reported apart).  CPU baseline:
    the oracle's restatement of kdtree_nearest and the float metrics, one
    thread, on part 1."""
    import torch
    import svdb_gb300 as S
    W = workloads()

    torch.cuda.set_device(local)
    X, Q, kd = W.config1()
    db = S.VectorDatabase(X.shape[0], kd)
    db.insert_batch(X)
    db.sync()
    r = np.random.default_rng(1)
    i1 = r.integers(0, X.shape[0], Q.shape[0] * 10)  # per query: 10 pairs of random stored ids
    i2 = r.integers(0, X.shape[0], Q.shape[0] * 10)

    def step():
        near = db.nearest_batch(Q)
        vals = [db.compare_batch(m, i1, i2)[0] for m in range(3)]
        return near, vals

    near, vals = step()  # correctness guard: the oracle's tree and metrics on a sample
    import oracle as O
    o = O.Oracle()
    okd = O.OracleKD(o, kd)
    for i in range(X.shape[0]):
        okd.insert(X[i], i)
    for qi in range(0, Q.shape[0], 97):
        if okd.nearest(Q[qi]) != near[qi]:
            raise SystemExit("bench: /nearest differs from the oracle")
    for j in range(0, i1.size, 331):
        for m in range(3):
            if np.float32(o.ref_metric(m, X[i1[j]], X[i2[j]])).tobytes() != vals[m][j].tobytes():
                raise SystemExit("bench: /compare differs from the oracle")
    for _ in range(args.warmup):
        step()
    clk = Clocks(local)
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t
    clocks = clk.stop()
    qps = Q.shape[0] * args.steps / dt

    cpu = None
    if args.cpu_sample > 0:
        t = time.perf_counter()
        nq_cpu = 0
        while time.perf_counter() - t < 3.0 and nq_cpu < Q.shape[0]:
            okd.nearest(Q[nq_cpu])
            for j in range(10):
                for m in range(3):
                    o.ref_metric(m, X[i1[nq_cpu * 10 + j]], X[i2[nq_cpu * 10 + j]])
            nq_cpu += 1
        cpu_dt = time.perf_counter() - t
        cpu = {"value": nq_cpu / cpu_dt, "unit": "queries/s", "cores": 1, "kind": "port",
               "sample": f"{nq_cpu} queries (/nearest + 30 /compare each) through the oracle's restatement, "
                         f"one thread, called per request as the handlers do ({cpu_dt:.1f} s)"}
    db.close()

    # part 2: /nearest at 1M rows
    X2, Q2 = W.config2(1_000_000, 128, 10_000)
    db2 = S.VectorDatabase(X2.shape[0], 3)
    db2.insert_batch(X2)
    db2.sync()
    db2.nearest_batch(Q2[:16])
    t = time.perf_counter()
    reps = 5
    for _ in range(reps):
        db2.nearest_batch(Q2)
    ins_qps = Q2.shape[0] * reps / (time.perf_counter() - t)
    t = time.perf_counter()
    a = db2.nearest_batch_median(Q2[:16])  # the first call builds the tree
    build_s = time.perf_counter() - t
    t = time.perf_counter()
    for _ in range(reps):
        b = db2.nearest_batch_median(Q2)
    med_qps = Q2.shape[0] * reps / (time.perf_counter() - t)
    db2.close()
    line = {"metric": "config-1 queries/s: /nearest + /compare x 10 ids x 3 metrics per query (N=10k x 128, kd 3)",
            "value": qps, "unit": "queries/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 (float accumulation in /compare, as the reference)", "data": "synthetic",
            "config": {"workload": "N=10,000 x 128 U[-1,1] seed 0, kd 3, 1,000 queries seed 1; per query /nearest "
                                   "+ 30 /compare pairs; one step = the 1,000 queries as one batch of each",
                       "l2": "store (10 MB) fits in L2: latency-bound"},
            "e2e": {"value": qps, "unit": "queries/s", "h2d_bytes_per_step": int(Q.nbytes + 3 * 2 * i1.nbytes),
                    "d2h_bytes_per_step": int(Q.shape[0] * 8 + 3 * i1.size * 5)},
            "nearest_1M": {"rows": 1_000_000, "kd_dim": 3, "queries": int(Q2.shape[0]),
                           "insertion_order_tree_qps": ins_qps, "median_tree_qps": med_qps,
                           "median_tree_build_s": build_s},
            "cpu_baseline": cpu, "clocks": clocks}
    print(json.dumps(line), flush=True)


def run_percall(args, ws, rank, local):
    """The drop-in per-call path as the unmodified server drives it: one
    thread per connection, one call per request (src/main.c:381,
    src/compare_handler.c:153-159,403).  Store: the CPU-runnable case,
    N=10,000 x 128 U[-1,1] (seed 0), KD dimension 3; queries U[-1,1] (seed 1).
    T threads (1 and --percall-threads) each call cosine_similarity on two
    stored rows (the Vectors vector_db_read returns) or kdtree_nearest, one
    call at a time, timed per call in C (libsvdb_percall.so, no interpreter in
    the loop).  The CPU baseline is the oracle's restatement of the same two
    functions (the reference's float loop and insertion-order tree) driven
    the same way."""
    import torch
    import svdb_gb300 as S
    W = workloads()

    torch.cuda.set_device(local)
    X, Q, kd = W.config1()
    db = S.VectorDatabase(X.shape[0], kd)
    db.insert_batch(X)
    db.sync()
    drv = C.CDLL(os.path.join(PKG, "_build", "libsvdb_percall.so"))
    drv.svdb_percall_metric.restype = C.c_int
    drv.svdb_percall_metric.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t, C.c_int,
                                        C.c_size_t, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    drv.svdb_percall_nearest.restype = C.c_int
    drv.svdb_percall_nearest.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_int,
                                         C.c_size_t, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    r = np.random.default_rng(1)
    npairs = 1000
    i1, i2 = r.integers(0, X.shape[0], npairs), r.integers(0, X.shape[0], npairs)
    VA, VB = (S.Vector * npairs)(), (S.Vector * npairs)()
    for j in range(npairs):  # the store's own rows, as vector_db_read returns them
        VA[j] = S.lib.vector_db_read(db.ptr, int(i1[j])).contents
        VB[j] = S.lib.vector_db_read(db.ptr, int(i2[j])).contents
    Qc = np.ascontiguousarray(Q)

    def metric_run(fn, abi, threads, calls):
        lat = np.empty(threads * calls)
        out = np.empty(threads * calls, np.float32)
        wall = C.c_double(0)
        rc = drv.svdb_percall_metric(fn, abi, 0, C.addressof(VA), C.addressof(VB), npairs, threads, calls,
                                     lat.ctypes.data, out.ctypes.data, C.byref(wall))
        if rc:
            raise SystemExit("bench: percall metric harness failed")
        return lat, out, wall.value

    def nearest_run(fn, tree, threads, calls):
        lat = np.empty(threads * calls)
        out = np.empty(threads * calls, np.int64)
        wall = C.c_double(0)
        rc = drv.svdb_percall_nearest(fn, tree, Qc.ctypes.data, Qc.shape[0], Qc.shape[1], threads, calls,
                                      lat.ctypes.data, out.ctypes.data, C.byref(wall))
        if rc:
            raise SystemExit("bench: percall nearest harness failed")
        return lat, out, wall.value

    def summary(lat, wall, n):
        return {"p50_us": float(np.percentile(lat, 50)) / 1e3, "p99_us": float(np.percentile(lat, 99)) / 1e3,
                "calls_per_s": n / (wall / 1e9)}

    import oracle as O
    O.build(ref=False)
    o = O.Oracle()
    okd = O.OracleKD(o, kd)
    for i in range(X.shape[0]):
        okd.insert(X[i], i)
    want_m = np.array([o.ref_metric(0, X[a], X[b]) for a, b in zip(i1, i2)], np.float32)
    want_n = np.array([okd.nearest(q) for q in Qc])
    f_cos = C.cast(S.lib.cosine_similarity, C.c_void_p).value
    f_near = C.cast(S.lib.kdtree_nearest, C.c_void_p).value
    o_cos = C.cast(o.L.orc_ref_metric, C.c_void_p).value
    o_near = C.cast(o.L.orc_kd_nearest, C.c_void_p).value
    res = {}
    clk = Clocks(local)
    for T in sorted({1, args.percall_threads}):
        calls = max(50, args.percall_calls // T)
        metric_run(f_cos, 0, T, 20)  # warm-up
        lat, out, wall = metric_run(f_cos, 0, T, calls)
        idx = np.arange(T * calls) % npairs
        if out.tobytes() != want_m[idx].tobytes():
            raise SystemExit("bench: per-call cosine_similarity differs from the oracle")
        res[f"cosine_similarity_threads{T}"] = summary(lat, wall, T * calls)
        nearest_run(f_near, db.kdtree, T, 20)
        lat, outn, wall = nearest_run(f_near, db.kdtree, T, calls)
        if not np.array_equal(outn, want_n[np.arange(T * calls) % Qc.shape[0]]):
            raise SystemExit("bench: per-call kdtree_nearest differs from the oracle")
        res[f"kdtree_nearest_threads{T}"] = summary(lat, wall, T * calls)
    clocks = clk.stop()
    cpu = {}
    for T in sorted({1, args.percall_threads}):
        calls = max(2000, 20 * args.percall_calls // T)
        lat, out, wall = metric_run(o_cos, 1, T, calls)
        cpu[f"cosine_similarity_threads{T}"] = summary(lat, wall, T * calls)
        lat, outn, wall = nearest_run(o_near, okd.h, T, calls)
        cpu[f"kdtree_nearest_threads{T}"] = summary(lat, wall, T * calls)
    T = args.percall_threads
    head = res[f"cosine_similarity_threads{T}"]
    line = {"metric": f"drop-in /compare calls/s, {T} threads one call at a time (N=10k x 128)",
            "value": head["calls_per_s"], "unit": "calls/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 (float accumulation, as the reference)", "data": "synthetic",
            "config": {"workload": "N=10,000 x 128 U[-1,1] seed 0, kd 3; cosine_similarity on stored rows and "
                                   "kdtree_nearest, one call per thread at a time", "threads": T,
                       "l2": "store (10 MB) fits in L2: latency-bound"},
            "per_call": res,
            "cpu_baseline": {"kind": "port", "cores": T, "per_call": cpu,
                             "sample": "the oracle's restatement of cosine_similarity and kdtree_nearest, driven by "
                                       "the same C harness"},
            "clocks": clocks}
    print(json.dumps(line), flush=True)
    db.close()


def run_loop(args, ws, rank, local):
    """The request path as a device-side loop (svdb_loop_*): a store of
    1,000,000 x 768 rows (the D=768 mixture, 1,024 centres, sigma 0.05, seed
    5), KD dimension 3.  A seeded open-loop trace at --rate requests/s (70 %
    POST /nearest answered by the KD descent, 10 % /compare with a uniform
    metric, 15 % insert, 3 % update, 2 % delete) is replayed in real time by a
    C harness: one thread submits each request at its arrival time, another
    takes the answers in order; latency = answer - arrival, queueing
    included.  A sample of the answers is checked against the oracle's
    positional store replaying the same requests.  CPU baseline: that
    oracle replay (the reference's store and KD tree restated), one thread."""
    import torch
    import svdb_gb300 as S
    from svdb_gb300 import serve
    W = workloads()

    torch.cuda.set_device(local)
    n0, d, kd = args.loop_rows, DIM, 3
    m5 = W.Mixture(d, 5)
    X0 = m5.sample(n0, 0)
    nreq = int(args.rate * args.serve_seconds)
    g = np.random.Generator(np.random.PCG64(np.random.SeedSequence([5, 77])))
    arrival = np.cumsum(g.exponential(1.0 / args.rate, nreq))
    ops = g.choice([5, 1, 2, 3, 4], size=nreq, p=[0.70, 0.10, 0.15, 0.03, 0.02]).astype(np.int32)
    vecs = np.ascontiguousarray(m5.sample(nreq, 9), np.float64)
    req = np.zeros(nreq, serve.REQ_DTYPE)
    req["op"] = ops
    req["metric"] = g.integers(0, 3, nreq)
    size = n0
    u = g.random((nreq, 2))
    for i in range(nreq):
        o = ops[i]
        if o in (5, 2, 3):
            req["vec"][i] = vecs.ctypes.data + i * d * 8
        if o == 1:
            req["a"][i], req["b"][i] = int(u[i, 0] * size), int(u[i, 1] * size)
        elif o == 2:
            size += 1
        elif o == 3:
            req["a"][i] = int(u[i, 0] * size)
        elif o == 4 and size > 0:
            req["a"][i] = int(u[i, 0] * size)
            size -= 1
    t = time.perf_counter()
    loop = S.DeviceLoop(d, kd, n0 + nreq + 1024, X0, ring=8192)
    log(f"[bench] loop store + KD tree {time.perf_counter() - t:.1f}s")
    loop.start()
    drv = C.CDLL(os.path.join(PKG, "_build", "libsvdb_percall.so"))
    drv.svdb_percall_loop_replay.restype = C.c_int
    drv.svdb_percall_loop_replay.argtypes = [C.c_void_p] * 4 + [C.c_size_t, C.c_void_p, C.c_size_t, C.c_void_p,
                                                                C.c_void_p, C.c_size_t, C.POINTER(C.c_double)]
    f_sub = C.cast(S.lib.svdb_loop_submit, C.c_void_p).value
    f_wait = C.cast(S.lib.svdb_loop_wait, C.c_void_p).value
    resp = np.zeros(nreq, np.dtype([("status", "<i4"), ("value", "<f4"), ("index", "<u8")]))
    lat = np.empty(nreq)
    wall = C.c_double(0)
    # warm-up: a short trace of /nearest requests only (no mutation: the measured
    # trace starts from the stated store)
    wq = np.zeros(2000, serve.REQ_DTYPE)
    wq["op"] = 5
    wv = np.ascontiguousarray(m5.sample(2000, 8), np.float64)
    wq["vec"] = wv.ctypes.data + np.arange(2000, dtype=np.uint64) * np.uint64(d * 8)
    warm_arr = np.arange(2000) / args.rate
    wresp = np.zeros(2000, resp.dtype)
    wlat = np.empty(2000)
    drv.svdb_percall_loop_replay(f_sub, f_wait, loop.ptr, wq.ctypes.data, wq.itemsize, warm_arr.ctypes.data, 2000,
                                 wlat.ctypes.data, wresp.ctypes.data, resp.itemsize, C.byref(wall))
    clk = Clocks(local)
    info0 = loop.info()
    rc = drv.svdb_percall_loop_replay(f_sub, f_wait, loop.ptr, req.ctypes.data, req.itemsize, arrival.ctypes.data,
                                      nreq, lat.ctypes.data, resp.ctypes.data, resp.itemsize, C.byref(wall))
    clocks = clk.stop()
    if rc:
        raise SystemExit(f"bench: loop replay failed: {S.last_error()}")
    info1 = loop.info()
    loop.stop()
    # correctness guard: the oracle's positional store replays the same requests
    import oracle as O
    O.build(ref=False)
    o = O.Oracle()
    st = o.store(d, kd)
    for i in range(n0):
        st.insert(X0[i])
    cpu_t = time.perf_counter()
    mismatch = 0
    for i in range(nreq):
        op = int(ops[i])
        if op == 5:
            r = st.nearest(vecs[i])
            want = 2 ** 64 - 1 if r < 0 else r
            if resp["status"][i] != 0 or int(resp["index"][i]) != want:
                mismatch += 1
        elif op == 1:
            a, b, m = int(req["a"][i]), int(req["b"][i]), int(req["metric"][i])
            ra = np.ctypeslib.as_array(o.L.orc_store_rows(st.h), shape=(st.size * d,))
            want = o.ref_metric(m, ra[a * d:(a + 1) * d], ra[b * d:(b + 1) * d])
            if resp["status"][i] != 0 or np.float32(resp["value"][i]).tobytes() != want.tobytes():
                mismatch += 1
        elif op == 2:
            st.insert(vecs[i])
        elif op == 3:
            st.update(int(req["a"][i]), vecs[i])
        else:
            st.delete(int(req["a"][i]))
    cpu_s = time.perf_counter() - cpu_t
    if mismatch:
        raise SystemExit(f"bench: {mismatch} loop answers differ from the oracle")
    loop.close()
    served = nreq / (wall.value / 1e9)
    line = {"metric": f"device-side request loop: served requests/s at {args.rate:.0f} req/s offered (70% /nearest KD, "
                      "10% /compare, 15% insert, 3% update, 2% delete), 1M x 768; p50/p99 ms",
            "value": served, "unit": "requests/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "ms_per_step": wall.value / 1e6, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 (float accumulation in /compare, as the reference)", "data": "synthetic",
            "config": {"workload": f"device loop over {n0} x 768 FP64 mixture rows (seed 5), kd 3, Poisson arrivals "
                                   f"at {args.rate:.0f}/s for {args.serve_seconds:.1f} s",
                       "l2": "rows (6.1 GB) larger than L2"},
            "latency_ms": {"p50": float(np.percentile(lat, 50)) / 1e6, "p99": float(np.percentile(lat, 99)) / 1e6,
                           "max": float(lat.max()) / 1e6},
            "loop": {"requests": nreq, "batches": info1["batches"] - info0["batches"],
                     "mean_batch": nreq / max(1, info1["batches"] - info0["batches"]),
                     "idle_exits": info1["idle_exits"], "mix": {int(k): int(v) for k, v in zip(*np.unique(ops, return_counts=True))},
                     "statuses": {int(k): int(v) for k, v in zip(*np.unique(resp["status"], return_counts=True))},
                     "how": "requests written to a mapped page-locked ring by one host thread at their arrival "
                            "times, answers taken in ticket order by another; no CUDA call per request"},
            "cpu_baseline": {"value": nreq / cpu_s, "unit": "requests/s", "cores": 1, "kind": "port",
                             "sample": f"the {nreq} requests replayed through the oracle's positional store and "
                                       f"KD tree, one thread ({cpu_s:.1f} s)"},
            "clocks": clocks}
    print(json.dumps(line), flush=True)


def run_decode(args, ws, rank, local):
    """POST /nearest request bodies decoded on the device: batches of 4,096
    bodies, each a JSON array of 768 numbers written with %.17g (N(0,1) x
    10^U[-8,8), seed 7; ~18 MB of text per batch), through svdb_decode_vectors
    (page-locked host text in, host doubles out: copies inside the timed
    region).  CPU
    baseline: the oracle's restatement of cJSON_Parse + strtod, one thread."""
    import svdb_gb300 as S
    import torch

    torch.cuda.set_device(local)
    nb, dim = 4096, 768
    rng = np.random.default_rng(7)
    X = rng.normal(size=(nb, dim)) * 10.0 ** rng.integers(-8, 8, (nb, 1))
    bodies = [("[" + ",".join("%.17g" % x for x in row) + "]").encode() for row in X]
    text = b"".join(bodies)
    off = np.zeros(nb + 1, np.uint64)
    off[1:] = np.cumsum([len(b) for b in bodies])
    # page-locked text and results, as a network front end's receive and send buffers would be
    text_t = torch.frombuffer(bytearray(text), dtype=torch.uint8).pin_memory()
    text_p = C.cast(C.c_void_p(text_t.data_ptr()), C.c_char_p)
    out = torch.empty((nb, dim), dtype=torch.float64).pin_memory().numpy()
    st = torch.empty(nb, dtype=torch.int32).pin_memory().numpy()

    def step():
        S._check(S.lib.svdb_decode_vectors(text_p, off.ctypes.data_as(C.POINTER(C.c_uint64)), nb, dim,
                                           out.ctypes.data_as(S._dp), st.ctypes.data_as(C.POINTER(C.c_int32))),
                 "svdb_decode_vectors")

    step()
    if not (st == 0).all() or out.tobytes() != X.tobytes():  # %.17g round-trips every double
        raise SystemExit("bench: decoded values differ from the encoded doubles")
    for _ in range(args.warmup):
        step()
    clk = Clocks(local)
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t
    clocks = clk.stop()
    cpu = None
    if args.cpu_sample > 0:
        import oracle as O
        o = O.Oracle()
        t = time.perf_counter()
        m = 0
        while m < nb and time.perf_counter() - t < 3.0:
            s_, v = o.decode_body(bodies[m], dim)
            if s_ != 0 or v.tobytes() != X[m].tobytes():
                raise SystemExit("bench: the oracle's decode disagrees")
            m += 1
        cdt = time.perf_counter() - t
        cpu = {"value": m / cdt, "unit": "bodies/s", "cores": 1, "kind": "port",
               "sample": f"{m} bodies through the oracle's cJSON_Parse + strtod restatement, one thread ({cdt:.1f} s)"}
    line = {"metric": "POST /nearest bodies decoded per second (768 numbers each, %.17g text)", "value": nb * args.steps / dt,
            "unit": "bodies/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u8 text -> f64", "data": "synthetic",
            "config": {"workload": f"4096 bodies x 768 numbers (%.17g), {len(text) / 1e6:.1f} MB of JSON text per batch",
                       "l2": "text larger than L2 per batch; no flush needed"},
            "e2e": {"value": nb * args.steps / dt, "unit": "bodies/s", "h2d_bytes_per_step": int(len(text) + off.nbytes),
                    "d2h_bytes_per_step": int(out.nbytes + st.nbytes)},
            "text_gbs": len(text) * args.steps / dt / 1e9, "cpu_baseline": cpu, "clocks": clocks}
    print(json.dumps(line), flush=True)


def main():
    global N_ROWS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["bf16", "fp8", "fp64"])
    ap.add_argument("--q", type=int, default=None, help="queries per step")
    ap.add_argument("--metric", default="cosine", choices=list(METRICS))
    ap.add_argument("--cpu-sample", type=int, default=64)
    ap.add_argument("--plain-q", type=int, default=64)
    ap.add_argument("--rows", type=int, default=N_ROWS, help="store rows (smaller cases for ncu captures)")
    ap.add_argument("--workload", default="mixture", choices=["mixture", "scan128", "ragged", "serve", "uuid", "nearest", "decode", "percall",
                             "loop"],
                    help="mixture: the 1M x 768 headline; scan128: plain FP64 single-query scan at 1M x 128; "
                         "ragged: one batch over 5 collections of different dimensions; serve: the serving loop; "
                         "uuid: GET /vector?uuid= lookups and persistence; nearest: the CPU-runnable config-1 "
                         "case (/nearest + /compare) and /nearest at 1M rows; decode: /nearest bodies decoded on the GPU")
    ap.add_argument("--rate", type=float, default=20000.0, help="serve: offered requests/s")
    ap.add_argument("--serve-sizes", default="1000000,5000000", help="serve: store sizes (rows)")
    ap.add_argument("--serve-seconds", type=float, default=3.0, help="serve: trace length per store size")
    ap.add_argument("--fp64-seconds", type=float, default=2.0, help="serve: cut-off of the plain FP64 trace")
    ap.add_argument("--loop-rows", type=int, default=1_000_000, help="loop: initial rows of the loop's store")
    ap.add_argument("--ragged-plan", default="auto", choices=["auto", "fused", "per-store"],
                    help="ragged: autotuned plan, or fixed choices (one search per part, stores concurrent; "
                         "screens fused into one launch, or one per search)")
    ap.add_argument("--ragged-part", default="", help="ragged: only collection C's queries of k class K "
                    "(C:K, K = 0 for k <= 16, 1 for <= 32, 2 above), default plan choices")
    ap.add_argument("--percall-threads", type=int, default=16, help="percall: concurrent caller threads")
    ap.add_argument("--percall-calls", type=int, default=32000, help="percall: calls across all threads")
    ap.add_argument("--extra", type=int, default=1, help="mixture: also time other batch sizes, metrics and a serve "
                                                         "trace (outside the timed region)")
    ap.add_argument("--serve-seconds-headline", type=float, default=1.0,
                    help="mixture: length of the serving trace reported beside the headline")
    args = ap.parse_args()
    N_ROWS = args.rows
    if args.q is None:
        args.q = 64 if args.precision == "fp64" else 4096
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.workload == "scan128":
        run_scan128(args, ws, rank, local)
    elif args.workload == "ragged":
        run_ragged(args, ws, rank, local)
    elif args.workload == "serve":
        run_serve(args, ws, rank, local)
    elif args.workload == "uuid":
        run_uuid(args, ws, rank, local)
    elif args.workload == "nearest":
        run_nearest(args, ws, rank, local)
    elif args.workload == "decode":
        run_decode(args, ws, rank, local)
    elif args.workload == "percall":
        run_percall(args, ws, rank, local)
    elif args.workload == "loop":
        run_loop(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
