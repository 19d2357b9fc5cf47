"""Benchmark: distinct (a,c) Mpairs/s of the GB300 join-project path.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]
                    [--workload chung_lu_20m|zipf_1m]

Workload (default): self join-project of an undirected Chung-Lu power-law
graph, 2^21 vertices, degree exponent 2.1, 1e7 edge samples -> ~20M directed
uint32 edges, R = S (distinct 2-hop neighbours).  Synthetic, seeded.

A step is one join-project call over the resident relations.  `value` times
K device-resident steps (inputs and output buffer in HBM) with CUDA events on
the library's stream; `e2e` times K steps through the host-buffer C ABI
(dim3g_join_project_into): H2D of R and S from pinned memory, the join, and
D2H of every output pair into pinned memory.  The inputs (320 MB) and the
output (~87 GB) are far larger than L2, so no flush is needed between steps.

--impl reference times the reference's CPU algorithm (the oracle port of
DIM3_parallel, all host threads) on a bounded A-slice of the same workload.
Under torchrun (N>1) the join is A-partitioned: rank r joins the rows of R
whose A hashes to shard r (fmix32(a) mod N) with all of S.  The shards'
outputs are disjoint, so no data moves between GPUs; `value` is the pairs of
all ranks (one integer all-reduce after the timed region) over the slowest
rank's time (total work fixed: strong scaling).  Rank 0 prints the line.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "joinproject-dim3_gb300"))

import numpy as np  # noqa: E402

METRIC = "distinct (a,c) Mpairs/s at 20M-edge 2-hop"
UNIT = "Mpairs/s"
WORKLOADS = {
    "chung_lu_20m": "self join-project, Chung-Lu 2^21 vertices, beta 2.1, 1e7 samples (~20M directed edges)",
    "zipf_1m": "R,S 1M tuples, dom(A)=dom(C)=50k uniform, dom(B)=20k Zipf s=1.0",
    "count16m": "COUNT(*) GROUP BY (A,C), R,S 16M tuples, dom(A)=dom(C)=1M uniform, dom(B)=200k Zipf s=1.2; "
                "~9.9e11 groups, summarised per A-tile (no output can hold them); a step = one of 16 A-slices",
    "batch512": "512 independent join-projects in one CUDA-graph launch; |R|,|S| log-uniform [1e4, 4e6], "
                "B Zipf s U[0.5, 1.5], dom(A)=dom(C)=dom(B) log-uniform [1e3, 1e6]; draws with "
                "E[OUT_J] > 2^28 or E[|OUT|] > 2^26 redrawn",
    "serve64": "Poisson arrivals (200 req/s) of join-project (75%) / COUNT (25%) requests over 64 resident "
               "relations, |R| log-uniform [1e6, 1.6e7], B degree exponent U[1.8, 2.5] over 2^18 shared B "
               "values (per-relation rank order), dom(A) = |R|/4; HBM budget 120 GB",
}


# The tensor roofline's peak: the product kernel's own ceiling on this
# device, measured by dim3g_calibrate (the measured peaks file holds bf16
# cuBLAS only; the product runs fp8 e4m3 operands with f32 accumulators).
FP8_PEAK_KIND = "measured: k_dense_mma (tcgen05 kind::f8f6f4) on all-ones operands, K = 4096, 8 tiles per SM"


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.samples = []
        self.stop = threading.Event()
        self.t = None

    def _run(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.FIELDS,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([x.strip() for x in out.stdout.strip().split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max(float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 4 + i and s[4 + i] == "Active"})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def profiled_traffic(kernel, workload):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu
    summary (a line `traffic <kernel> <workload> <bytes>`), else None."""
    import glob
    import re
    for f in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md"))):
        for line in open(f):
            m = re.match(r"\s*traffic\s+(\S+)\s+(\S+)\s+(\d+)", line)
            if m and m.group(1) == kernel and m.group(2) == workload:
                return int(m.group(3))
    return None


def make_workload(name):
    import dim3gpu
    return dim3gpu.workload(name, 1.0)


def a_slice(R, parts, which):
    """Rows of R whose first value falls in hash bucket `which` of `parts`."""
    h = (R[:, 0].astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15)) >> np.uint64(40)
    return np.ascontiguousarray(R[(h % np.uint64(parts)) == which])


def host_threads():
    """Cores this process may run on (`nproc`): THREAD_NUM of the OpenMP arm."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_run(R, S, parts, which, threads):
    """One oracle run on an A-slice: DIM3_parallel with `threads` OpenMP
    threads, or DIM3 serial for threads = 1."""
    from oracle import oracle_py
    Rs = a_slice(R, parts, which)
    t = time.perf_counter()
    # Full S as the first argument keeps it the larger side (no swap of
    # roles); the pairs are (c, a), the same set transposed.
    _, n, _, st = oracle_py.join_project(S, Rs, threads=threads, hash_only=False)
    dt = time.perf_counter() - t
    return n, dt, st


def serial_arm(args, R, S):
    """The reference's single-threaded path (DIM3::doJoinProject, main.cpp:19),
    as the oracle port, on a 1/(cpu_parts * serial_div) A-slice."""
    import platform
    parts = args.cpu_parts * args.serial_div
    n, dt, _ = cpu_run(R, S, parts, 0, 1)
    return {"value": round(n / dt / 1e6, 3), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "1/%d A-slice of %s (full S): %d pairs in %.2f s; oracle port of DIM3 (serial), %s"
                      % (parts, args.workload, n, dt, platform.machine())}


def run_reference(args, rank, world):
    if rank != 0:
        return
    threads = host_threads()
    R, S = make_workload(args.workload)
    parts = args.cpu_parts
    for w in range(args.warmup):
        cpu_run(R, S, parts, w % parts, threads)
    tot_n, tot_t = 0, 0.0
    for k in range(args.steps):
        n, dt, st = cpu_run(R, S, parts, (args.warmup + k) % parts, threads)
        tot_n += n
        tot_t += dt
    value = tot_n / tot_t / 1e6
    sample = ("1/%d A-slice of %s per step (full S), oracle port of DIM3_parallel, THREAD_NUM = nproc = %d"
              % (parts, args.workload, threads))
    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(tot_t / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": args.workload, "desc": WORKLOADS[args.workload], "sample": sample},
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample, "thread_num": threads, "nproc": threads,
                             "single_thread": serial_arm(args, R, S) if args.serial_div > 0 else None},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(args):
    """The reference's OpenMP path (DIM3_parallel, THREAD_NUM = nproc) and its
    single-threaded path, both as the oracle port, each on a bounded A-slice
    of the same workload, timed on this host's cores."""
    threads = host_threads()
    R, S = make_workload(args.workload)
    parts = args.cpu_parts
    n, dt, st = cpu_run(R, S, parts, 0, threads)
    return {"value": round(n / dt / 1e6, 3), "unit": UNIT, "cores": threads, "kind": "port",
            "thread_num": threads, "nproc": threads,
            "sample": "1/%d A-slice of %s (full S): %d pairs in %.2f s; oracle port of DIM3_parallel, %d threads"
                      % (parts, args.workload, n, dt, threads),
            "single_thread": serial_arm(args, R, S) if args.serial_div > 0 else None}


def run_gpu(args, rank, world, local_rank):
    import torch
    import dim3gpu
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    R, S = make_workload(args.workload)
    if world > 1:
        R = dim3gpu.a_shard(R, rank, world)
    nR, nS = R.shape[0], S.shape[0]
    ctx = dim3gpu.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    # the device's own product rates and bandwidth for the dense block's
    # cost model; the fp8 rate is also the tensor roofline's peak
    cal = ctx.calibrate()
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    torch.cuda.synchronize()
    n_out = ctx.join_project_count_device(dR, nR, dS, nS)
    out = torch.empty((n_out, 2), dtype=torch.int32, device="cuda")
    for _ in range(args.warmup):
        ctx.join_project_device(dR, nR, dS, nS, out, n_out)
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    ms_write, ms_bitmap, ms_mma = [], [], []
    ms_phase = {"ms_map": 0.0, "ms_csr": 0.0, "ms_count": 0.0, "ms_write": 0.0}
    launches0 = ctx.stats()["launches"]
    with ClockSampler(local_rank) as clk:
        barrier()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            n = ctx.join_project_device(dR, nR, dS, nS, out, n_out)
            st = ctx.stats()
            ms_write.append(st["ms_write"])
            ms_bitmap.append(st["ms_write_cls"][0])
            ms_mma.append(st["ms_dense"][1])
            for k in ms_phase:
                ms_phase[k] += st[k]
        ev1.record(stream)
        barrier()
        ms = ev0.elapsed_time(ev1) / args.steps
    assert n == n_out
    launches = ctx.stats()["launches"] - launches0
    clocks = clk.summary()
    n_all = n_out
    if dist is not None:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        c = torch.tensor([n_out], dtype=torch.int64, device="cuda")
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
        n_all = int(c.item())
    value = n_all / (ms / 1e3) / 1e6

    # e2e through the host-buffer ABI: pinned R, S and output.
    e2e = None
    if args.e2e_steps > 0:
        hR = torch.from_numpy(R.view(np.int32)).pin_memory().numpy().view(np.uint32)
        hS = torch.from_numpy(S.view(np.int32)).pin_memory().numpy().view(np.uint32)
        del out
        torch.cuda.empty_cache()
        hout = torch.empty((n_out, 2), dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
        ctx.join_project_into(hR, hS, hout)  # warm the staging buffers
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            n2 = ctx.join_project_into(hR, hS, hout)
        barrier()
        e2e_s = (time.perf_counter() - t0) / args.e2e_steps
        assert n2 == n_out
        if dist is not None:
            t = torch.tensor([e2e_s], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            e2e_s = float(t.item())
        e2e = {"value": round(n_all / e2e_s / 1e6, 3), "unit": UNIT,
               "h2d_bytes_per_step": int((nR + nS) * 8), "d2h_bytes_per_step": int(n_out * 8),
               "ms_per_step": round(e2e_s * 1e3, 3)}
    st = ctx.stats()
    peak, peak_kind = load_peaks()
    ms_b = sum(ms_bitmap) / len(ms_bitmap)
    dense = st["rows_dense"] > 0
    if dense:
        # The heavy rows went through the dense block: its dominant kernel is
        # the emission (k_dense_emit), whose algorithmic bytes are the 8 B of
        # every pair it writes (the bitmap it reads is < 2 % of that).
        kernel = "k_dense_emit"
        alg_bytes = 8 * st["n_out_cls"][0]
    else:
        # Dominant kernel: k_single_bitmap (the heavy rows' single-pass
        # expansion), timed by the library's CUDA events on its stream inside
        # the timed region.  Algorithmic bytes per launch: 4 B per candidate z
        # id read + 8 B per distinct pair written, over that kernel's rows.
        kernel = "k_single_bitmap"
        alg_bytes = 4 * st["out_j_cls"][0] + 8 * st["n_out_cls"][0]
    achieved = alg_bytes / (ms_b / 1e3) / 1e9
    ms_w = sum(ms_write) / len(ms_write)
    alg_all = 4 * st["out_j"] + 8 * n_out
    traffic = args.traffic if args.traffic is not None else profiled_traffic(kernel, args.workload)
    tensor = None
    if dense:
        # the tensor-core product: 2 Mp Np Kp MMA flops per launch (padded
        # tiles are executed), fp8 e4m3 operands, f32 accumulators
        mp = (st["rows_dense"] + 127) // 128 * 128
        np_ = (st["nz"] + 255) // 256 * 256
        flops = 2 * mp * np_ * st["dense_kp"]
        ms_t = sum(ms_mma) / len(ms_mma)
        ach_t = flops / (ms_t / 1e3) / 1e12
        bf16 = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("bf16_tflops") \
            if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
        peak_t = cal["fp8_tflops"]
        tensor = {"bound": "tensor", "kernel": "k_dense_mma", "achieved": round(ach_t, 1), "peak": peak_t,
                  "peak_kind": FP8_PEAK_KIND, "unit": "TFLOP/s", "frac": round(ach_t / peak_t, 4),
                  "vs_measured_bf16_burst": round(ach_t / bf16, 4) if bf16 else None,
                  "flops_per_launch": int(flops), "ms_per_launch": round(ms_t, 3), "rows": st["rows_dense"],
                  "heavy_y": st["heavy_y"], "kp": st["dense_kp"]}
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": args.workload, "desc": WORKLOADS[args.workload], "nR": int(nR), "nS": int(nS),
                   "n_out": int(n_all), "out_j": int(st["out_j"]), "l2": "inputs 8(|R|+|S|) and output > L2; no flush",
                   "parallelism": ("a_shard%d (R by fmix32(a) mod N, S whole)" % world) if world > 1 else "single"},
        "phases_ms": {k: round(v / args.steps, 3) for k, v in ms_phase.items()},
        "e2e": e2e,
        "roofline": {"bound": "hbm", "kernel": kernel,
                     "achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "alg_bytes_per_launch": int(alg_bytes), "ms_per_launch": round(ms_b, 3),
                     "expansion_all_classes": {"alg_bytes": int(alg_all), "ms": round(ms_w, 3),
                                               "achieved": round(alg_all / (ms_w / 1e3) / 1e9, 1)}},
        "roofline_tensor": tensor,
        "calibration": cal,
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(args) if not args.no_cpu else None
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


def _upload(arrs):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda() for a in arrs]


def run_batch(args, rank, world, local_rank):
    """512 independent joins as one CUDA-graph launch per step, against the
    plain drop-in (one dim3g_join_project_device call per query)."""
    import torch
    import dim3gpu
    torch.cuda.set_device(local_rank)
    params = dim3gpu.batch_queries(nq=args.batch_queries)
    rels = dim3gpu.batch_relations(params)
    ctx = dim3gpu.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    dev = _upload([a for rs in rels for a in rs])
    pairs = [((dev[2 * i], R.shape[0]), (dev[2 * i + 1], S.shape[0])) for i, (R, S) in enumerate(rels)]
    torch.cuda.synchronize()
    sizer = dim3gpu.Batch(ctx, pairs, [{"op": 0, "capacity": 0} for _ in rels])
    sized = sizer.run(check=False)
    need = [r["n_out"] for r in sized]
    sizer.close()
    outs = [torch.empty((max(n, 1), 2), dtype=torch.int32, device="cuda") for n in need]
    b = dim3gpu.Batch(ctx, pairs, [{"op": 0, "capacity": n, "out": o} for n, o in zip(need, outs)])
    # tile shapes and class thresholds from the autotuner, timing the batch
    # graph itself; the plain drop-in below runs under the same settings
    tuning = b.autotune(max_trials=args.tune_trials)
    for _ in range(args.warmup):
        b.run()
    launches0 = ctx.stats()["launches"]
    dev_ms = []
    with ClockSampler(local_rank) as clk:
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(args.steps):
            res = b.run()
            dev_ms.append(b.info()["ms_last"])
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
    assert [r["n_out"] for r in res] == need
    launches = ctx.stats()["launches"] - launches0
    total = sum(need)
    outj = sum(r["out_j"] for r in res)
    # plain drop-in, same inputs, one call per query into one scratch buffer
    buf = torch.empty((max(max(need), 1), 2), dtype=torch.int32, device="cuda")
    plain_ms = []
    for k in range(2):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        got = [ctx.join_project_device(dev[2 * i], R.shape[0], dev[2 * i + 1], S.shape[0], buf, buf.shape[0])
               for i, (R, S) in enumerate(rels)]
        e1.record(stream)
        torch.cuda.synchronize()
        plain_ms.append(e0.elapsed_time(e1))
        assert got == need
    plain = min(plain_ms)
    peak, peak_kind = load_peaks()
    ntup = sum(R.shape[0] + S.shape[0] for R, S in rels)
    alg = 4 * outj + 8 * total + 24 * ntup
    line = {
        "metric": METRIC, "value": round(total / (ms / 1e3) / 1e6, 3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "batch512", "desc": WORKLOADS["batch512"], "queries": len(rels),
                   "tuples": int(ntup), "n_out": int(total), "out_j": int(outj),
                   "redraws": int(sum(p["redraws"] for p in params)),
                   "tuning": {k: tuning[k] for k in ["tile_bits_log2", "block_threads", "block_slots_log2",
                                                     "warp_slots_log2", "cta_walk", "trials"]},
                   "l2": "inputs and outputs > L2; no flush"},
        "graph_device_ms": round(sum(dev_ms) / len(dev_ms), 3),
        "plain_dropin": {"value": round(total / (plain / 1e3) / 1e6, 3), "ms_per_step": round(plain, 3),
                         "calls": len(rels)},
        "batch_over_plain": round(plain / ms, 3),
        "roofline": {"bound": "hbm", "kernel": "whole graph (index build + query pass)",
                     "achieved": round(alg / (ms / 1e3) / 1e9, 1), "peak": peak, "peak_kind": peak_kind,
                     "unit": "GB/s", "frac": round(alg / (ms / 1e3) / 1e9 / peak, 4), "traffic": None,
                     "alg_bytes_per_launch": int(alg)},
        "gpu_launches": launches, "launches_per_step": b.info()["launches_per_run"],
        "clocks": clk.summary(), "e2e": None, "cpu_baseline": None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    b.close()
    ctx.close()


def run_count16m(args, rank, world, local_rank):
    """The 16M x 16M Zipf-1.2 COUNT join-aggregate: per-A-tile summaries
    (groups, count sum, hash), one of 16 A-slices per step."""
    import torch
    import dim3gpu
    from oracle import oracle_py as O
    torch.cuda.set_device(local_rank)
    R, S = make_workload("zipf12_16m")
    ctx = dim3gpu.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    cal = ctx.calibrate()
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
    tiles = 16
    for k in range(args.warmup):
        ctx.join_count_summary(dR, R.shape[0], dS, S.shape[0], tiles, k % tiles, k % tiles + 1)
    launches0 = ctx.stats()["launches"]
    groups, outj, ms_dev, ms_mma, flops = 0, 0, 0.0, 0.0, 0
    with ClockSampler(local_rank) as clk:
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for k in range(args.steps):
            sm = ctx.join_count_summary(dR, R.shape[0], dS, S.shape[0], tiles, k % tiles, k % tiles + 1)
            groups += int(sm[:, 0].sum())
            outj += int(sm[:, 1].sum())
            st = ctx.stats()
            ms_dev += st["ms_write"]
            if st["rows_dense"]:
                ms_mma += st["ms_dense"][1]
                flops += 2 * ((st["rows_dense"] + 127) // 128 * 128) * ((st["nz"] + 255) // 256 * 256) * st["dense_kp"]
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / args.steps
    launches = ctx.stats()["launches"] - launches0
    peak, peak_kind = load_peaks()
    cpu = None
    if rank == 0 and not args.no_cpu:
        # the oracle on a 1/4096 A-slice (S stays the larger side)
        sel = (O.fmix32(R[:, 0]) & np.uint64(4095)).astype(np.int64) == 0
        Rs = np.ascontiguousarray(R[sel])
        t = time.perf_counter()
        _, _, ng, _, _ = O.join_count(S, Rs, threads=host_threads(), hash_only=True)
        dt = time.perf_counter() - t
        cpu = {"value": round(ng / dt / 1e6, 3), "unit": "Mgroups/s", "cores": host_threads(),
               "kind": "port", "sample": "1/4096 A-slice of count16m (full S): %d groups in %.2f s" % (ng, dt)}
    # expansion of the slices: 4 B per candidate read, nothing written
    alg = 4 * outj
    if flops:
        # the dense block ran: its product (fp8 MMA, exact counts) with the
        # group-hash epilogue is the dominant kernel
        ach = flops / (ms_mma / 1e3) / 1e12
        roof = {"bound": "tensor", "kernel": "k_dense_mma (COUNT summary epilogue)", "achieved": round(ach, 1),
                "peak": cal["fp8_tflops"], "peak_kind": FP8_PEAK_KIND,
                "unit": "TFLOP/s", "frac": round(ach / cal["fp8_tflops"], 4), "traffic": None,
                "flops_per_launch": int(flops / max(args.steps, 1)), "ms_per_launch": round(ms_mma / args.steps, 3),
                "kp": st["dense_kp"], "note": "the epilogue's two splitmix64 hashes per group bound the tile rate"}
    else:
        roof = {"bound": "hbm", "kernel": "k_agg_tile (summaries)",
                "achieved": round(alg / (ms_dev / 1e3) / 1e9, 1), "peak": peak, "peak_kind": peak_kind,
                "unit": "GB/s", "frac": round(alg / (ms_dev / 1e3) / 1e9 / peak, 4), "traffic": None,
                "alg_bytes_per_launch": int(alg / max(args.steps, 1))}
    line = {
        "metric": "distinct (a,c) groups Mgroups/s, COUNT(*) GROUP BY (A,C) 16M x 16M Zipf 1.2",
        "value": round(groups / (ms * args.steps / 1e3) / 1e6, 3), "unit": "Mgroups/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32/u64", "data": "synthetic",
        "config": {"workload": "count16m", "desc": WORKLOADS["count16m"], "groups": groups, "out_j": outj,
                   "slices": args.steps, "l2": "relations > L2; no flush"},
        "roofline": roof, "calibration": cal,
        "gpu_launches": launches, "clocks": clk.summary(), "cpu_baseline": cpu, "e2e": None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def _pct(v, q):
    return float(np.percentile(np.asarray(v, dtype=np.float64), q)) if len(v) else None


def run_serve(args, rank, world, local_rank):
    """Poisson request stream over a resident set: served (continuous
    batching) and, on the same trace, the plain drop-in one call at a time."""
    import queue
    import torch
    import dim3gpu
    torch.cuda.set_device(local_rank)
    params = dim3gpu.serve_params(scale=args.serve_scale)
    rels = [dim3gpu.serve_relation(p) for p in params]
    n = len(rels)
    dev = _upload(rels)
    ctx = dim3gpu.Context(local_rank)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    torch.cuda.synchronize()
    t = time.perf_counter()
    rs = dim3gpu.RelSet(ctx, [(d, a.shape[0]) for d, a in zip(dev, rels)])
    build_s = time.perf_counter() - t
    srv = dim3gpu.Server(rs, lanes=args.lanes, max_batch=64, budget_bytes=args.budget_gb << 30)
    rng = np.random.default_rng(11)
    nreq = int(args.rate * args.duration)
    arrivals = np.cumsum(rng.exponential(1.0 / args.rate, nreq))
    # a uniformly chosen pair of two different relations (a skewed
    # relation joined with itself has OUT_J ~ |R|^2 sum p^2, ~1e13)
    rr = rng.integers(0, n, nreq)
    ss = (rr + 1 + rng.integers(0, n - 1, nreq)) % n
    ops = (rng.random(nreq) < 0.25).astype(int)
    for k in range(min(8, nreq)):  # warm-up requests (not in the trace)
        tk = srv.submit(int(rr[k]), int(ss[k]), int(ops[k]))
        srv.wait(tk)
        srv.release(tk)
    tickets = queue.Queue()
    done = []

    def waiter():
        while True:
            tk = tickets.get()
            if tk is None:
                return
            res = srv.wait(tk)
            done.append(res)
            srv.release(tk)

    th = threading.Thread(target=waiter, daemon=True)
    th.start()
    launches0 = ctx.stats()["launches"]
    refused = []
    with ClockSampler(local_rank) as clk:
        t0 = time.perf_counter()
        try:
            for i in range(nreq):
                dt = t0 + arrivals[i] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
                try:
                    tickets.put(srv.submit(int(rr[i]), int(ss[i]), int(ops[i])))
                except dim3gpu.Dim3GError:
                    refused.append(i)  # reservation above the whole output budget
        finally:
            tickets.put(None)
        th.join(timeout=args.duration * 10 + 60)
        wall = time.perf_counter() - t0
    if th.is_alive():
        raise RuntimeError("served requests did not complete")
    launches = ctx.stats()["launches"] - launches0
    st = srv.stats()
    lat = [(r["t_done"] - r["t_submit"]) * 1e3 for r in done]
    pairs = sum(r["n_out"] for r in done)
    span = max(r["t_done"] for r in done) - min(r["t_submit"] for r in done)
    bad = sum(1 for r in done if r["status"] != 0)
    srv.close()
    # the plain drop-in on the same trace: one call at a time, in arrival order
    cap = int(max(r["n_out"] for r in done))  # the served results are exact
    out = torch.empty((max(cap, 1), 2), dtype=torch.int32, device="cuda")
    cnt = torch.empty((max(cap, 1),), dtype=torch.int64, device="cuda")
    plain_lat, plain_pairs = [], 0
    t0 = time.perf_counter()
    nplain = 0
    refused_set = set(refused)
    for i in range(nreq):
        if i in refused_set:
            continue
        now = time.perf_counter() - t0
        if now < arrivals[i]:
            time.sleep(arrivals[i] - now)
        a, b_ = int(rr[i]), int(ss[i])
        if ops[i]:
            k = ctx.join_count_device(dev[a], rels[a].shape[0], dev[b_], rels[b_].shape[0], out, cnt, cap)
        else:
            k = ctx.join_project_device(dev[a], rels[a].shape[0], dev[b_], rels[b_].shape[0], out, cap)
        plain_pairs += k
        plain_lat.append((time.perf_counter() - t0 - arrivals[i]) * 1e3)
        nplain += 1
        if time.perf_counter() - t0 > args.duration * 3:
            break
    plain_span = time.perf_counter() - t0
    line = {
        "metric": METRIC, "value": round(pairs / span / 1e6, 3), "unit": UNIT, "n_gpus": world,
        "steps": nreq, "warmup": 8, "ms_per_step": round(span / max(len(done), 1) * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": {"workload": "serve64", "desc": WORKLOADS["serve64"], "relations": n,
                   "tuples": int(sum(a.shape[0] for a in rels)), "rate_per_s": args.rate,
                   "duration_s": args.duration, "lanes": args.lanes, "budget_gb": args.budget_gb,
                   "l2": "relations and outputs > L2; no flush"},
        "latency_ms": {"p50": round(_pct(lat, 50), 3), "p99": round(_pct(lat, 99), 3),
                       "max": round(max(lat), 3)},
        "requests": len(done), "failed": bad, "refused": len(refused), "passes": st["passes"],
        "wall_s": round(wall, 3),
        "relset_build_s": round(build_s, 3),
        "plain_dropin": {"value": round(plain_pairs / plain_span / 1e6, 3), "requests": nplain,
                         "latency_ms": {"p50": round(_pct(plain_lat, 50), 3), "p99": round(_pct(plain_lat, 99), 3)}},
        "gpu_launches": launches, "clocks": clk.summary(), "e2e": None, "cpu_baseline": None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    rs.close()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="chung_lu_20m", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-parts", type=int, default=64)
    ap.add_argument("--serial-div", type=int, default=4,
                    help="the single-threaded arm takes a 1/(cpu-parts * serial-div) A-slice (0: skip it)")
    ap.add_argument("--traffic", type=float, default=None)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--batch-queries", type=int, default=512)
    ap.add_argument("--tune-trials", type=int, default=12)
    ap.add_argument("--serve-scale", type=float, default=1.0)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--duration", type=float, default=10.0)
    ap.add_argument("--lanes", type=int, default=2)
    ap.add_argument("--budget-gb", type=int, default=120)
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local_rank = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        run_reference(args, rank, world)
    elif args.workload in ("batch512", "count16m", "serve64"):
        # one-GPU forms: under torchrun rank 0 runs them alone (n_gpus 1)
        if rank == 0:
            {"batch512": run_batch, "count16m": run_count16m, "serve64": run_serve}[args.workload](
                args, 0, 1, local_rank)
    else:
        run_gpu(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
