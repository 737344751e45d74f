"""Runs the device-resident PFP BWT a fixed number of times on one of the
benchmark workloads; the command profilers (ncu) are pointed at.

  python -m <package>.profile_run --workload config2 --iters 1
  python -m <package>.profile_run --workload config2 --scale 0.125 --iters 2

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
    ap.add_argument("--workload", default="config2", choices=["config1", "config2", "config3"])
    ap.add_argument("--scale", type=float, default=1.0, help="base length scale of the workload")
    ap.add_argument("--iters", type=int, default=1)
    ap.add_argument("--W", type=int, default=None)
    ap.add_argument("--P", type=int, default=None)
    ap.add_argument("--small", action="store_true")
    args = ap.parse_args(argv)
    import numpy as np
    import torch

    pkg = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")
    text = getattr(wl, args.workload + "_text")(args.scale)
    W = args.W or 5
    P = args.P or (23 if args.workload == "config3" else 16)
    n = len(text)
    dt = torch.from_numpy(text).cuda()
    do = torch.empty_like(dt)
    torch.cuda.synchronize()
    with pkg.Storage(n) as st:
        for i in range(args.iters):
            st.pfp_bwt_device(dt.data_ptr(), do.data_ptr(), n, W, P, args.small, stage_times=(i == args.iters - 1))
        torch.cuda.synchronize()
        stats = st.stats()
    out = do.cpu().numpy()
    if not np.array_equal(np.bincount(out, minlength=256), np.bincount(text, minlength=256)):
        print("profile_run: output is not a permutation of the text", file=sys.stderr)
        return 1
    stats.update({"workload": args.workload, "scale": args.scale, "n": n, "W": W, "P": P, "small": args.small})
    print(json.dumps(stats))
    return 0


if __name__ == "__main__":
    sys.exit(main())
