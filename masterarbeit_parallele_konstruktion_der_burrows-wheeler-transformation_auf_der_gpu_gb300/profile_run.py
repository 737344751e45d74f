"""Runs the device-resident PFP BWT a fixed number of times on one of the
benchmark workloads; the command profilers (ncu) are pointed at.

  python -m <package>.profile_run --workload config2 --iters 1
  python -m <package>.profile_run --workload config2 --scale 0.125 --iters 2
  python -m <package>.profile_run --workload config4 --iters 3            # batched
  python -m <package>.profile_run --workload config4 --per-text --iters 1 # one text per call
  python -m <package>.profile_run --workload config4 --tuning '{"radix_rank": 2}'

Prints one JSON line with the pipeline counts and per-stage times of the
last iteration.  Exits non-zero if the BWT is not a permutation of the text.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import sys

PKG = os.path.basename(os.path.dirname(os.path.abspath(__file__)))


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="config2", choices=["config1", "config2", "config3", "config4"])
    ap.add_argument("--per-text", action="store_true", help="config4: one call per text instead of one batch")
    ap.add_argument("--scale", type=float, default=1.0, help="base length scale of the workload")
    ap.add_argument("--iters", type=int, default=1)
    ap.add_argument("--W", type=int, default=None)
    ap.add_argument("--P", type=int, default=None)
    ap.add_argument("--small", action="store_true")
    ap.add_argument("--tuning", default=None,
                    help='JSON knobs laid over the size class\'s tuning, e.g. \'{"radix_rank": 2}\'')
    args = ap.parse_args(argv)
    import numpy as np
    import torch

    pkg = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")
    if args.workload == "config4":
        return run_batched(args, pkg, wl)
    text = getattr(wl, args.workload + "_text")(args.scale)
    W = args.W or 5
    P = args.P or (23 if args.workload == "config3" else 16)
    n = len(text)
    dt = torch.from_numpy(text).cuda()
    do = torch.empty_like(dt)
    torch.cuda.synchronize()
    with pkg.Storage(n) as st:
        apply_tuning(pkg, st, n, args.tuning)
        for i in range(args.iters):
            st.pfp_bwt_device(dt.data_ptr(), do.data_ptr(), n, W, P, args.small, stage_times=(i == args.iters - 1))
        torch.cuda.synchronize()
        stats = st.stats()
    out = do.cpu().numpy()
    if not np.array_equal(np.bincount(out, minlength=256), np.bincount(text, minlength=256)):
        print("profile_run: output is not a permutation of the text", file=sys.stderr)
        return 1
    stats.update({"workload": args.workload, "scale": args.scale, "n": n, "W": W, "P": P, "small": args.small,
                  "tuning": args.tuning})
    print(json.dumps(stats))
    return 0


def apply_tuning(pkg, st, n: int, override: str | None) -> None:
    """Size-class knobs (tuning.json) with the JSON `override` laid over them."""
    if not override:
        return
    base = pkg.tuning_for(n, pkg.load_tuning()) or {}
    st.set_tuning({**base, **json.loads(override)})


def run_batched(args, pkg, wl) -> int:
    import numpy as np
    import torch

    concat, offsets = wl.config4_texts(args.scale)
    W, P = args.W or 5, args.P or 16
    n = len(concat)
    dt = torch.from_numpy(concat).cuda()
    do = torch.empty_like(dt)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    with pkg.Storage(n) as st:
        st.set_stream(stream.cuda_stream)
        apply_tuning(pkg, st, n, args.tuning)
        ms = []
        for i in range(args.iters):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            if args.per_text:
                for t in range(len(offsets) - 1):
                    a, b = int(offsets[t]), int(offsets[t + 1])
                    st.pfp_bwt_device(dt.data_ptr() + a, do.data_ptr() + a, b - a, W, P, args.small)
            else:
                st.pfp_bwt_batch_device(dt.data_ptr(), offsets, do.data_ptr(), W, P, args.small,
                                        stage_times=(i == args.iters - 1))
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        stats = st.stats()
    out = do.cpu().numpy()
    if not np.array_equal(np.bincount(out, minlength=256), np.bincount(concat, minlength=256)):
        print("profile_run: output is not a permutation of the texts", file=sys.stderr)
        return 1
    stats.update({"workload": "config4", "per_text": args.per_text, "scale": args.scale, "n": n,
                  "texts": len(offsets) - 1, "W": W, "P": P, "tuning": args.tuning, "ms": [round(x, 3) for x in ms],
                  "MBps_last": round(n / (ms[-1] / 1000) / 1e6, 1)})
    print(json.dumps(stats))
    return 0


if __name__ == "__main__":
    sys.exit(main())
