#!/usr/bin/env python
"""Benchmark of the GB300 PFP BWT on the 512 MiB repetitive-DNA workload.

One step = one BWT (W=5, P=16) of the whole 512 MiB text.

  value     input MB/s (1e6 bytes/s) with the text already resident in HBM
            and the BWT left in HBM (CUDA events on the launching stream);
  e2e       the same through the public C ABI with pinned HOST buffers: the
            host->device copy of the text and the device->host copy of the
            BWT are inside every timed step;
  roofline  the dominant kernel's algorithmic bytes per launch / its average
            launch time (events around each of its launches in the timed
            region) against the measured HBM copy bandwidth;
  cpu_baseline  the CPU port of the reference's PFP (the oracle) on a
            bounded prefix of the same text, on this host's cores.

``--impl reference`` times the reference's CPU implementation of the path:
the reference itself is CUDA-only, so this is the oracle port (the CPU
restatement of its PFP algorithm) on a bounded sample, rank 0 only.

Multi-GPU: the single-text path does not shard; ``--gpus N`` under torchrun
runs N independent replicas (weak scaling, no collective on the data path).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
PKG = "masterarbeit_parallele_konstruktion_der_burrows-wheeler-transformation_auf_der_gpu_gb300"

with open(os.path.join(ROOT, "BASELINE.json")) as _f:
    METRIC = json.load(_f)["metric"]
UNIT = "MB/s"
WORKLOAD = ("512 MiB repetitive DNA: 4 MiB uniform ACGT base (seed 2), 128 copies with 0.1% substitutions "
            "+ 0.01% indels (length 1-10); PFP W=5 P=16, one text per step")

# Kernel whose launches are timed for the roofline, and its algorithmic
# bytes per element: the radix-sort scatter reads and writes every key and
# value once (u64 key + u32 value = 24 B/element on the sort of the parse).
PROBE_KERNEL = 1   # see gbwt_set_kernel_probe in include/gbwt.h


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if d.get("hbm_gbs"):
            return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            os.makedirs(os.path.join(ROOT, "gpurun_out"), exist_ok=True)
            self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{self.gpu}.csv")
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_port_sample(text, sample_bytes):
    """Times the oracle (CPU port of the reference PFP) on a prefix."""
    import oracle
    oracle.build()
    s = text[:sample_bytes]
    t0 = time.perf_counter()
    oracle.pfp_bwt(s, 5, 16, False)
    dt = time.perf_counter() - t0
    return len(s) / dt / 1e6, dt, len(s), oracle.max_threads_used()


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    wl = importlib.import_module(PKG + ".workloads")
    text = wl.config2_text()
    sample = args.cpu_sample_mib << 20
    times = []
    threads = 1
    for i in range(args.warmup + args.steps):
        mbps, dt, nbytes, threads = cpu_port_sample(text, sample)
        if i >= args.warmup:
            times.append(dt)
    ms = 1000.0 * statistics.mean(times)
    value = sample / (ms / 1000.0) / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": f"first {args.cpu_sample_mib} MiB of the text per step",
                   "W": 5, "P": 16},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"first {args.cpu_sample_mib} MiB of the 512 MiB text (oracle PFP port; the "
                                   "reference has no CPU implementation of this path)"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")

    t0 = time.time()
    text = wl.config2_text()
    n = len(text)
    log(f"[rank {rank}] workload generated: n={n} ({time.time() - t0:.1f}s)")

    dev_text = torch.from_numpy(text).cuda()
    dev_out = torch.empty_like(dev_text)
    host_text = torch.from_numpy(text).pin_memory()
    host_out = torch.empty(n, dtype=torch.uint8).pin_memory()
    stream = torch.cuda.current_stream()
    st = pkg.Storage(n)
    st.set_stream(stream.cuda_stream)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()

    # ---- device-resident timing ----------------------------------------
    for _ in range(args.warmup):
        st.pfp_bwt_device(dev_text.data_ptr(), dev_out.data_ptr(), n, 5, 16)
    torch.cuda.synchronize()
    stats = st.stats()
    st.set_kernel_probe(PROBE_KERNEL)
    launches = 0
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            st.pfp_bwt_device(dev_text.data_ptr(), dev_out.data_ptr(), n, 5, 16)
            launches += st.stats()["kernel_launches"]
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    probe = st.stats()
    st.set_kernel_probe(-1)
    clocks = clk.summary()

    # ---- stage breakdown (one extra, untimed step) ------------------------
    st.pfp_bwt_device(dev_text.data_ptr(), dev_out.data_ptr(), n, 5, 16, stage_times=True)
    torch.cuda.synchronize()
    stage = st.stats()

    # ---- end to end through the C ABI with pinned host buffers -------------
    for _ in range(max(1, args.warmup // 2)):
        st.pfp_bwt_into(host_text.numpy(), host_out.numpy(), 5, 16)
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        st.pfp_bwt_into(host_text.numpy(), host_out.numpy(), 5, 16)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps

    # ---- correctness of what was timed (size-independent checks) ----------
    got = host_out.numpy()
    if not np.array_equal(np.bincount(got, minlength=256), np.bincount(text, minlength=256)):
        raise SystemExit("bench: BWT is not a permutation of the text")
    if not np.array_equal(dev_out.cpu().numpy(), got):
        raise SystemExit("bench: device and host paths differ")

    if ws > 1:
        t = torch.tensor([ms, e2e_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, e2e_ms = float(t[0]), float(t[1])
    if rank != 0:
        torch.distributed.destroy_process_group()
        return 0

    value = ws * n / (ms / 1000.0) / 1e6
    e2e_value = ws * n / (e2e_ms / 1000.0) / 1e6
    peak, peak_kind = measured_peak()
    roofline = None
    if probe.get("probe_launches", 0) > 0 and probe.get("probe_ms", 0) > 0:
        per_launch_bytes = probe["probe_bytes"] / probe["probe_launches"]
        avg_s = probe["probe_ms"] / probe["probe_launches"] / 1000.0
        achieved = per_launch_bytes / avg_s / 1e9
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "traffic": traffic_per_launch(per_launch_bytes),
                    "kernel": "k_rs_downsweep (radix scatter)", "peak_kind": f"of {peak_kind}",
                    "launches_timed": probe["probe_launches"], "algorithmic_bytes_per_launch": int(per_launch_bytes),
                    "share_of_step": round(probe["probe_ms"] / args.steps / ms, 4)}
    cpu_value, cpu_dt, cpu_n, cpu_threads = cpu_port_sample(text, args.cpu_sample_mib << 20)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": WORKLOAD, "n": n, "W": 5, "P": 16, "small_alphabet": False,
                   "l2": "inputs larger than L2 (512 MiB text vs 129 MB L2), no flush",
                   "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
        "e2e": {"value": round(e2e_value, 2), "unit": UNIT, "h2d_bytes_per_step": n, "d2h_bytes_per_step": n,
                "ms_per_step": round(e2e_ms, 3)},
        "roofline": roofline,
        "cpu_baseline": {"value": round(cpu_value, 3), "unit": UNIT, "cores": cpu_threads, "kind": "port",
                         "sample": f"first {cpu_n >> 20} MiB of the same text, oracle PFP port, one run "
                                   f"({cpu_dt:.1f} s)"},
        "clocks": clocks,
        "gpu_launches": launches,
        "pipeline": {k: stats[k] for k in ("z", "d", "dict_bytes", "s", "mixed_blocks", "mixed_elems",
                                             "dict_rounds", "parse_rounds", "hash_retries")},
        "stage_ms": stage["stage_ms"],
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def traffic_per_launch(per_launch_bytes):
    """DRAM bytes per launch from the committed ncu capture, scaled to this
    launch size (bytes per algorithmic byte), or None when absent."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    ratio = d.get("dram_bytes_per_algorithmic_byte")
    return None if ratio is None else int(ratio * per_launch_bytes)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbwt", choices=["gbwt", "reference"])
    ap.add_argument("--cpu-sample-mib", type=int, default=16)
    args = ap.parse_args(argv)
    if args.warmup < 3:
        log("bench: warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
