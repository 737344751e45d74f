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

Two more sections ride on the same line (rank 0):
  batched   4096 independent texts (~512 MiB, log-normal lengths) in one
            gbwt_pfp_bwt_batch call, device-resident and end to end, next to
            the same texts run one call per text;
  serving   Poisson arrivals of mixed-size jobs into the serving loop
            (gbwt_server_*): p50/p99 latency and sustained MB/s, next to the
            same jobs run one after another through gbwt_pfp_bwt (FIFO
            latencies for the same arrival times).

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

# Kernels whose launches are timed for the roofline (gbwt_set_kernel_probe in
# include/gbwt.h), with the library's algorithmic bytes per launch:
#   k_seg_sort (the dominant kernel, prefix-doubling rounds sorted inside CTAs):
#     24 B per active element (read x, group, key; write rank and next entry)
#   k_rs_downsweep (radix scatter): every key and value read and written once
PROBE_SEG_SORT = 6
PROBE_RADIX = 1


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
    st.set_kernel_probe(PROBE_SEG_SORT)
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

    # ---- the radix scatter's launches (one extra, untimed step) -------------
    st.set_kernel_probe(PROBE_RADIX)
    st.pfp_bwt_device(dev_text.data_ptr(), dev_out.data_ptr(), n, 5, 16)
    torch.cuda.synchronize()
    probe_radix = st.stats()
    st.set_kernel_probe(-1)

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

    # ---- inverse BWT on the GPU (round trip of the timed output) -----------
    primary = stage["primary_index"]
    dev_back = torch.empty_like(dev_text)
    st.unbwt_device(dev_out.data_ptr(), dev_back.data_ptr(), n, primary)
    torch.cuda.synchronize()
    u0, u1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    u0.record(stream)
    for _ in range(3):
        st.unbwt_device(dev_out.data_ptr(), dev_back.data_ptr(), n, primary)
    u1.record(stream)
    torch.cuda.synchronize()
    unbwt_ms = u0.elapsed_time(u1) / 3
    if not torch.equal(dev_back, dev_text):
        raise SystemExit("bench: inverse BWT does not give the text back")
    del dev_back

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
    roofline = roofline_of(probe, "k_seg_sort", "k_seg_sort<ParseRem/DictRem> (prefix-doubling rounds in CTAs)",
                           peak, peak_kind, args.steps, ms)
    roofline_radix = roofline_of(probe_radix, "k_rs_downsweep", "k_rs_downsweep (radix scatter)", peak, peak_kind,
                                 1, ms)
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
        "roofline_radix": roofline_radix,
        "cpu_baseline": {"value": round(cpu_value, 3), "unit": UNIT, "cores": cpu_threads, "kind": "port",
                         "sample": f"first {cpu_n >> 20} MiB of the same text, oracle PFP port, one run "
                                   f"({cpu_dt:.1f} s)"},
        "clocks": clocks,
        "gpu_launches": launches,
        "inverse_bwt": {"value": round(n / (unbwt_ms / 1000.0) / 1e6, 2), "unit": UNIT, "ms": round(unbwt_ms, 3),
                        "check": "gbwt_unbwt(BWT, primary index) == text"},
        "pipeline": {k: stats[k] for k in ("z", "d", "dict_bytes", "s", "mixed_blocks", "mixed_elems",
                                             "dict_rounds", "parse_rounds", "hash_retries")},
        "stage_ms": stage["stage_ms"],
    }
    if "batched" in args.sections:
        line["batched"] = measure_batched(args, pkg, wl, stream)
        log(f"[rank 0] batched: {line['batched']['value']} MB/s")
    if "serving" in args.sections:
        line["serving"] = measure_serving(args, pkg, wl)
        log(f"[rank 0] serving: {line['serving']['latency_ms']}")
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


BATCH_WORKLOAD = ("4096 independent DNA texts, log-normal lengths (median 64 KiB, sigma 1.2, clipped to "
                  "4 KiB-16 MiB, ~512 MiB total, seed 4), each 8-64 copies of its own uniform ACGT base with 0.1% "
                  "substitutions; PFP W=5 P=16")


def measure_batched(args, pkg, wl, stream):
    """Config-4 batch: one gbwt_pfp_bwt_batch call per step."""
    import numpy as np
    import torch

    concat, offsets = wl.config4_texts()
    n = len(concat)
    k = len(offsets) - 1
    dev_in = torch.from_numpy(concat).cuda()
    dev_out = torch.empty_like(dev_in)
    host_in = torch.from_numpy(concat).pin_memory()
    host_out = torch.empty(n, dtype=torch.uint8).pin_memory()
    st = pkg.Storage(n)
    st.set_stream(stream.cuda_stream)
    for _ in range(args.warmup):
        st.pfp_bwt_batch_device(dev_in.data_ptr(), offsets, dev_out.data_ptr())
    torch.cuda.synchronize()
    steps = max(1, args.batch_steps)
    launches = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        st.pfp_bwt_batch_device(dev_in.data_ptr(), offsets, dev_out.data_ptr())
        launches += st.stats()["kernel_launches"]
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    st.pfp_bwt_batch_device(dev_in.data_ptr(), offsets, dev_out.data_ptr(), stage_times=True)
    torch.cuda.synchronize()
    stage = st.stats()
    # end to end: pinned host texts in, host BWTs out
    st.pfp_bwt_batch_into(host_in.numpy(), offsets, host_out.numpy())
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        st.pfp_bwt_batch_into(host_in.numpy(), offsets, host_out.numpy())
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / steps
    got = host_out.numpy()
    if not np.array_equal(got, dev_out.cpu().numpy()):
        raise SystemExit("bench: batched device and host paths differ")
    # one call per text on the same device-resident texts (the same library)
    for t in range(min(k, 32)):
        a, b = int(offsets[t]), int(offsets[t + 1])
        st.pfp_bwt_device(dev_in.data_ptr() + a, dev_out.data_ptr() + a, b - a)
    torch.cuda.synchronize()
    e0.record(stream)
    for t in range(k):
        a, b = int(offsets[t]), int(offsets[t + 1])
        st.pfp_bwt_device(dev_in.data_ptr() + a, dev_out.data_ptr() + a, b - a)
    e1.record(stream)
    torch.cuda.synchronize()
    per_text_ms = e0.elapsed_time(e1)
    if not np.array_equal(dev_out.cpu().numpy(), got):
        raise SystemExit("bench: batched and one-call-per-text results differ")
    st.close()
    value = n / (ms / 1000.0) / 1e6
    per_text_value = n / (per_text_ms / 1000.0) / 1e6
    return {
        "workload": BATCH_WORKLOAD, "texts": k, "n": n, "steps": steps, "value": round(value, 2), "unit": UNIT,
        "ms_per_step": round(ms, 3), "gpu_launches_per_step": launches // steps,
        "e2e": {"value": round(n / (e2e_ms / 1000.0) / 1e6, 2), "unit": UNIT, "ms_per_step": round(e2e_ms, 3),
                "h2d_bytes_per_step": n + 8 * (k + 1), "d2h_bytes_per_step": n},
        "one_call_per_text": {"value": round(per_text_value, 2), "unit": UNIT, "ms": round(per_text_ms, 1),
                              "calls": k},
        "speedup_vs_one_call_per_text": round(value / per_text_value, 2),
        "stage_ms": stage["stage_ms"],
    }


def measure_serving(args, pkg, wl):
    """Config-5 serving: Poisson arrivals into the serving loop."""
    import numpy as np

    texts, arrivals = wl.serving_jobs(args.serve_jobs, args.serve_rate)
    total = int(sum(len(t) for t in texts))
    small_max = 16 << 20
    with pkg.Server(workers=2, small_max=small_max) as srv:
        # warm-up: one large job and a burst of small ones
        warm = [srv.submit(t) for t in texts[:64]]
        warm.append(srv.submit(max(texts, key=len)))
        srv.drain()
        outs = [np.empty(len(t), np.uint8) for t in texts]
        t0 = time.perf_counter()
        tickets = []
        for t, at, o in zip(texts, arrivals, outs):
            delay = at - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            tickets.append(srv.submit(t, out=o))
        srv.drain()
        infos = [srv.poll(k) for k in tickets]
    if any(i["status"] != 0 for i in infos):
        raise SystemExit("bench: a serving job failed")
    lat = [(i["end_us"] - i["submit_us"]) / 1000.0 for i in infos]
    span_s = (max(i["end_us"] for i in infos) - min(i["submit_us"] for i in infos)) / 1e6
    # the same jobs, one gbwt_pfp_bwt call after another (FIFO for the same arrivals)
    st = pkg.Storage(max(len(t) for t in texts))
    for t in texts[:16]:
        st.pfp_bwt(t)
    service = []
    for t, o in zip(texts, outs):
        a = time.perf_counter()
        L = st.pfp_bwt(t)
        service.append(time.perf_counter() - a)
        if not np.array_equal(L, o):
            raise SystemExit("bench: serving result differs from the job run alone")
    st.close()
    fifo, end = [], 0.0
    for at, sv in zip(arrivals, service):
        start = max(at, end)
        end = start + sv
        fifo.append((end - at) * 1000.0)
    small = [l for l, t in zip(lat, texts) if len(t) <= small_max]
    large = [l for l, t in zip(lat, texts) if len(t) > small_max]
    return {
        "workload": (f"{len(texts)} jobs, Poisson arrivals at {args.serve_rate:g}/s; ~1% 64-256 MiB repetitive DNA "
                     "(prefixes of one text built like the 512 MiB workload), the rest with the batched workload's "
                     "log-normal lengths; W=5 P=16; 2 workers, jobs <= 16 MiB batched"),
        "jobs": len(texts), "bytes": total, "large_jobs": len(large),
        "latency_ms": pkg.percentiles(lat), "latency_ms_small": pkg.percentiles(small),
        "latency_ms_large": pkg.percentiles(large),
        "sustained": {"value": round(total / span_s / 1e6, 2), "unit": UNIT},
        "max_batch_jobs": max(i["batch_jobs"] for i in infos),
        "sequential": {"value": round(total / sum(service) / 1e6, 2), "unit": UNIT,
                       "latency_ms": pkg.percentiles(fifo)},
    }


def traffic_per_launch(kernel, per_launch_bytes):
    """DRAM bytes per launch from the committed ncu capture of `kernel`
    (profiles/traffic.json: DRAM bytes per algorithmic byte), scaled to this
    launch size, or None when absent."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    ratio = d.get(kernel, {}).get("dram_bytes_per_algorithmic_byte")
    return None if ratio is None else int(ratio * per_launch_bytes)


def roofline_of(probe, key, label, peak, peak_kind, steps, step_ms):
    """Roofline object from the probe counters of one kernel family."""
    if probe.get("probe_launches", 0) <= 0 or probe.get("probe_ms", 0) <= 0:
        return None
    per_launch_bytes = probe["probe_bytes"] / probe["probe_launches"]
    avg_s = probe["probe_ms"] / probe["probe_launches"] / 1000.0
    achieved = per_launch_bytes / avg_s / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": traffic_per_launch(key, per_launch_bytes),
            "kernel": label, "peak_kind": f"of {peak_kind}", "launches_timed": probe["probe_launches"],
            "algorithmic_bytes_per_launch": int(per_launch_bytes),
            "share_of_step": round(probe["probe_ms"] / steps / step_ms, 4)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbwt", choices=["gbwt", "reference"])
    ap.add_argument("--cpu-sample-mib", type=int, default=16)
    ap.add_argument("--sections", default="plain,batched,serving",
                    help="comma list: the plain headline always runs; batched, serving are extra sections")
    ap.add_argument("--batch-steps", type=int, default=5)
    ap.add_argument("--serve-jobs", type=int, default=800)
    ap.add_argument("--serve-rate", type=float, default=1000.0)
    args = ap.parse_args(argv)
    if args.warmup < 3:
        log("bench: warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
