"""Run one join-project (or COUNT join-aggregate) on a named workload.

    python run_case.py --workload chung_lu_20m --scale 1.0 --mode count|project|aggregate [--repeat N]

Prints one JSON line with the call's device-phase timings.  Used for
profiling single launches (`ncu ... python run_case.py ...`): --mode count
runs the mapping, CSR and count pass only (no output buffer), so a capture
of the full-size workload stays within a few GB of device memory.
"""
import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import dim3gpu  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="chung_lu_20m")
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--mode", default="count", choices=["count", "project", "aggregate"])
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--param", action="append", default=[], help="name=value tuning knob")
    args = ap.parse_args()
    import torch
    R, S = dim3gpu.workload(args.workload, args.scale)
    ctx = dim3gpu.Context(0)
    for p in args.param:
        k, v = p.split("=")
        ctx.set_param(k, int(v))
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    dR = torch.from_numpy(R.view(np.int32)).cuda()
    dS = torch.from_numpy(S.view(np.int32)).cuda()
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
