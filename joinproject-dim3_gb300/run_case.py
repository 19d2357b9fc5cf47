"""Run one join on a named workload and print its device-phase timings.

    python run_case.py --workload chung_lu_20m --scale 1.0 --mode count|project|aggregate [--repeat N]
    python run_case.py --workload zipf12_16m --mode count_summary --tiles 16 --tile-hi 1
    python run_case.py --mode batch [--queries 512]          # the mixed batch, one CUDA graph
    python run_case.py --mode relset_pass [--scale 1.0]      # 64 requests over the served set
    python run_case.py --workload zipf_1m --mode autotune    # the autotuner's choice for a workload
    python run_case.py --mode project --a-tiles 64 --a-tile 0  # R's rows of one A-tile, all of S

Prints one JSON line.  Used for profiling single launches (`ncu ...
python run_case.py ...`): --mode count runs the mapping, CSR and count pass
only (no output buffer), so a capture of the full-size workload stays within
a few GB of device memory; --mode batch builds the batch once to size its
outputs, then runs it once (the second graph's launches are the measured
ones); --mode relset_pass builds the served relation set and runs one pass of
64 requests of distinct relation pairs (25% COUNT) with outputs sized by the
pair matrix.
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import dim3gpu  # noqa: E402


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).cuda()


def run_batch(args, ctx):
    import torch
    params = dim3gpu.batch_queries(nq=args.queries)
    rels = dim3gpu.batch_relations(params)
    pairs = [((_dev(R), R.shape[0]), (_dev(S), S.shape[0])) for R, S in rels]
    sizer = dim3gpu.Batch(ctx, pairs, [{"op": 0, "capacity": 0} for _ in rels])
    need = [r["n_out"] for r in sizer.run(check=False)]
    sizer.close()
    outs = [torch.empty((max(n, 1), 2), dtype=torch.int32, device="cuda") for n in need]
    b = dim3gpu.Batch(ctx, pairs, [{"op": 0, "capacity": n, "out": o} for n, o in zip(need, outs)])
    ms = []
    for _ in range(args.repeat):
        res = b.run()
        ms.append(b.info()["ms_last"])
    return {"queries": len(rels), "n_out": int(sum(r["n_out"] for r in res)),
            "out_j": int(sum(r["out_j"] for r in res)), "graph_ms_each": [round(x, 3) for x in ms],
            "launches_per_run": b.info()["launches_per_run"]}


def run_relset_pass(args, ctx):
    import torch
    params = dim3gpu.serve_params(scale=args.scale)
    rels = [dim3gpu.serve_relation(p) for p in params]
    rs = dim3gpu.RelSet(ctx, [(_dev(a), a.shape[0]) for a in rels])
    m = rs.pair_outj()
    n = len(rels)
    rng = np.random.default_rng(3)
    specs = []
    for _ in range(64):
        r = int(rng.integers(0, n))
        s = int((r + 1 + rng.integers(0, n - 1)) % n)
        op = int(rng.random() < 0.25)
        cap = int(m[r, s])
        spec = {"r": r, "s": s, "op": op, "capacity": cap,
                "out": torch.empty((max(cap, 1), 2), dtype=torch.int32, device="cuda")}
        if op:
            spec["cnt"] = torch.empty((max(cap, 1),), dtype=torch.int64, device="cuda")
        specs.append(spec)
    ms = []
    for _ in range(args.repeat):
        torch.cuda.synchronize()
        t = time.perf_counter()
        res = rs.join(specs)
        torch.cuda.synchronize()
        ms.append((time.perf_counter() - t) * 1e3)
    return {"requests": 64, "n_out": int(sum(x["n_out"] for x in res)), "out_j": int(sum(x["out_j"] for x in res)),
            "pass_ms_each": [round(x, 3) for x in ms]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="chung_lu_20m")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--mode", default="count",
                    choices=["count", "project", "aggregate", "count_summary", "batch", "relset_pass", "autotune"])
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--param", action="append", default=[], help="name=value tuning knob")
    ap.add_argument("--tiles", type=int, default=16)
    ap.add_argument("--tile-lo", type=int, default=0)
    ap.add_argument("--tile-hi", type=int, default=1)
    ap.add_argument("--queries", type=int, default=512)
    ap.add_argument("--a-tiles", type=int, default=1,
                    help="keep only R's rows in A-tile --a-tile of this many (fmix32(a) & (tiles-1)); S stays whole")
    ap.add_argument("--a-tile", type=int, default=0)
    args = ap.parse_args()
    import torch
    ctx = dim3gpu.Context(0)
    for p in args.param:
        k, v = p.split("=")
        ctx.set_param(k, int(v))
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    if args.mode == "batch":
        print(json.dumps({"mode": "batch", **run_batch(args, ctx)}))
        ctx.close()
        return
    if args.mode == "relset_pass":
        print(json.dumps({"mode": "relset_pass", "scale": args.scale, **run_relset_pass(args, ctx)}))
        ctx.close()
        return
    R, S = dim3gpu.workload(args.workload, args.scale)
    if args.a_tiles > 1:
        # an A-slice keeps the heavy rows' shape (same z domain, same S) at
        # 1/a_tiles of the output: a representative case small enough to
        # profile section by section
        sel = (dim3gpu.fmix32_np(R[:, 0]) & np.uint64(args.a_tiles - 1)) == np.uint64(args.a_tile)
        R = np.ascontiguousarray(R[sel])
    dR = _dev(R)
    dS = _dev(S)
    torch.cuda.synchronize()
    res = []
    if args.mode == "count":
        for _ in range(args.repeat):
            n = ctx.join_project_count_device(dR, R.shape[0], dS, S.shape[0])
            res.append(ctx.stats())
    elif args.mode == "project":
        n = ctx.join_project_count_device(dR, R.shape[0], dS, S.shape[0])
        out = torch.empty((n, 2), dtype=torch.int32, device="cuda")
        for _ in range(args.repeat):
            ctx.join_project_device(dR, R.shape[0], dS, S.shape[0], out, n)
            res.append(ctx.stats())
    elif args.mode == "autotune":
        t = ctx.autotune(dR, R.shape[0], dS, S.shape[0])
        print(json.dumps({"workload": args.workload, "mode": "autotune", "tuning": t}))
        ctx.close()
        return
    elif args.mode == "count_summary":
        for _ in range(args.repeat):
            sm = ctx.join_count_summary(dR, R.shape[0], dS, S.shape[0], args.tiles, args.tile_lo, args.tile_hi)
            res.append(ctx.stats())
        n = int(sm[:, 0].sum())
    else:
        n = ctx.join_project_count_device(dR, R.shape[0], dS, S.shape[0])
        oxz = torch.empty((n, 2), dtype=torch.int32, device="cuda")
        oc = torch.empty((n,), dtype=torch.int64, device="cuda")
        for _ in range(args.repeat):
            ctx.join_count_device(dR, R.shape[0], dS, S.shape[0], oxz, oc, n)
            res.append(ctx.stats())
    torch.cuda.synchronize()
    st = res[-1]
    print(json.dumps({"workload": args.workload, "scale": args.scale, "mode": args.mode, "n_out": int(n),
                      "stats": {k: (round(v, 3) if isinstance(v, float) else v) for k, v in st.items()},
                      "ms_total_each": [round(r["ms_total"], 3) for r in res]}))
    ctx.close()


if __name__ == "__main__":
    main()
