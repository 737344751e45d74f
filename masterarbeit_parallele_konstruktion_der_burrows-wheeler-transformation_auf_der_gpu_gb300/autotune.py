"""Autotuner for the library's scheduling knobs (gbwt_tuning in include/gbwt.h).

For every size class it times candidate values of each knob on this GPU with
the others fixed (coordinate descent, median of a few CUDA-event timed runs,
inputs resident in HBM) and writes the winners to ``tuning.json`` next to the
package, where ``Storage(tuning="auto")`` finds them.  The knobs change how
the work is scheduled (table size, sort segments, digit width, ruler
density), never a result; tests check that.

  python -m <package>.autotune                      # classes 16, 128, 512 MiB
  python -m <package>.autotune --classes 64 --repeats 5 --out /tmp/t.json

Each class is measured on one repetitive DNA text of that size (hash table,
first sort keys, inverse-BWT rulers) and on the batched workload's text mix
scaled to the class's total size (batch knobs).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import sys
import time

PKG = os.path.basename(os.path.dirname(os.path.abspath(__file__)))

# candidate values per knob; 0 in a result means the library default
CANDIDATES = {
    "hash_log2_max": (20, 22, 24),
    "dict_key_bits": (64, 48, 40, 32),
    "parse_key_phrases": (0, 1, 2),
    "mixed_radix_bits": (8, 10),
    "batch_seg_tiles": (4, 8, 16, 32),
    "batch_pad_eighths": (1, 2, 4),
    "batch_radix_bits": (8, 9),
    "batch_ballot": (1, 2, 3),
    "unbwt_rate_log2": (6, 7, 8),
}
TEXT_KNOBS = ("hash_log2_max", "dict_key_bits", "parse_key_phrases", "mixed_radix_bits")
BATCH_KNOBS = ("batch_seg_tiles", "batch_pad_eighths", "batch_radix_bits", "batch_ballot")
START = {"hash_log2_max": 22, "dict_key_bits": 64, "parse_key_phrases": 0, "mixed_radix_bits": 8, "batch_seg_tiles": 8,
         "batch_pad_eighths": 1, "batch_radix_bits": 0, "batch_ballot": 3, "unbwt_rate_log2": 7}


def coordinate_descent(measure, knobs, start: dict, candidates: dict = CANDIDATES, sweeps: int = 2):
    """Minimises measure(config) one knob at a time; returns (best config, its
    time, number of measurements).  A knob keeps its value unless another
    candidate is faster with the others fixed; stops when a sweep changes
    nothing."""
    cache = {}

    def timed(cfg):
        key = tuple(sorted(cfg.items()))
        if key not in cache:
            cache[key] = measure(dict(cfg))
        return cache[key]

    best = dict(start)
    best_t = timed(best)
    for _ in range(sweeps):
        changed = False
        for k in knobs:
            for v in candidates[k]:
                if v == best.get(k):
                    continue
                cfg = dict(best)
                cfg[k] = v
                t = timed(cfg)
                if t < best_t:
                    best, best_t, changed = cfg, t, True
        if not changed:
            break
    return best, best_t, len(cache)


def _median_ms(fn, repeats):
    import torch

    fn()                                        # warm-up (scratch growth)
    torch.cuda.synchronize()
    times = []
    for _ in range(repeats):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    return statistics.median(times)


def tune_class(pkg, wl, mib: int, repeats: int, log) -> dict:
    import torch

    # one repetitive DNA text of the class size: hash table and first keys
    text = wl.dna_copies(base_len=max(4096, (mib << 20) // 64), copies=64, seed=50 + mib, indel_rate=1e-4)
    d_text = torch.from_numpy(text).cuda()
    d_bwt = torch.empty_like(d_text)
    st = pkg.Storage(len(text), tuning=None)
    st.set_stream(torch.cuda.current_stream().cuda_stream)

    def measure_text(cfg):
        st.set_tuning(cfg)
        return _median_ms(lambda: st.pfp_bwt_device(d_text.data_ptr(), d_bwt.data_ptr(), len(text)), repeats)

    best, t_best, runs = coordinate_descent(measure_text, TEXT_KNOBS, START)
    log(f"  {mib} MiB text: {t_best:.2f} ms after {runs} configurations: {best}")
    # the batched workload's text mix scaled to the class size: batch knobs
    count = max(8, int(round(4096 * mib / 512.0)))
    concat, offsets = wl.batch_texts(count, scale=1.0, seed=40 + mib)
    dT = torch.from_numpy(concat).cuda()
    dL = torch.empty_like(dT)

    def measure_batch(cfg):
        st.set_tuning(cfg)
        return _median_ms(lambda: st.pfp_bwt_batch_device(dT.data_ptr(), offsets, dL.data_ptr()), repeats)

    best, t_best, runs = coordinate_descent(measure_batch, BATCH_KNOBS, best)
    log(f"  {mib} MiB batch ({count} texts): {t_best:.2f} ms after {runs} configurations: {best}")
    del dT, dL
    # inverse BWT rulers on the text
    d_back = torch.empty_like(d_text)
    st.set_tuning(best)
    st.pfp_bwt_device(d_text.data_ptr(), d_bwt.data_ptr(), len(text))
    torch.cuda.synchronize()
    primary = st.stats()["primary_index"]

    def measure_unbwt(cfg):
        st.set_tuning(cfg)
        return _median_ms(lambda: st.unbwt_device(d_bwt.data_ptr(), d_back.data_ptr(), len(text), primary), repeats)

    best, t_ub, runs_ub = coordinate_descent(measure_unbwt, ("unbwt_rate_log2",), best)
    if not torch.equal(d_back, d_text):
        raise SystemExit("autotune: inverse BWT does not give the text back")
    log(f"  {mib} MiB inverse BWT: {t_ub:.2f} ms, rate 2^{best['unbwt_rate_log2']}")
    st.close()
    return {k: int(v) for k, v in best.items()}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--classes", default="16,128,512", help="size classes in MiB")
    ap.add_argument("--repeats", type=int, default=3)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    import torch

    pkg = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")
    log = lambda *a: print(*a, file=sys.stderr, flush=True)
    out = {"device": torch.cuda.get_device_name(0), "created": time.strftime("%Y-%m-%d"),
           "method": "coordinate descent over gbwt_tuning knobs, median CUDA-event time, inputs in HBM",
           "classes": {}}
    for mib in (int(x) for x in args.classes.split(",")):
        log(f"class {mib} MiB")
        out["classes"][str(mib)] = tune_class(pkg, wl, mib, args.repeats, log)
    path = args.out or pkg.TUNING_FILE
    # per-window-length overrides of an existing table are kept
    old = pkg.load_tuning(pkg.TUNING_FILE) or {}
    for key in ("windows", "windows_note"):
        if key in old:
            out[key] = old[key]
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
