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
  roofline_pipeline  the whole pipeline's algorithmic bytes
            (4n + (24+W)z + 3 dict_bytes + 8d + 8s) over the step time;
  cpu_baseline  the suffix-array (SA-IS) BWT of the whole text on one host
            core, run in a spawned process after the GPU measurements.

More sections ride on the same line (rank 0):
  reference_cuda  the reference's own PFP program (compiled unmodified for
            sm_103a, oracle/reference.py) on the same text: device span
            Compute_D + Compute_S and host-to-host span, bit-exactness;
  libcubwt  the libcubwt 1.6.3 copy the reference ships, host to host;
  variants  the same text with W=5 P=16 small-alphabet and W=35 P=81
            small-alphabet, each with its reference program;
  batched   4096 independent texts (~512 MiB, log-normal lengths) in one
            gbwt_pfp_bwt_batch call, device-resident and end to end, next to
            the same texts run one call per text;
  serving   Poisson arrivals of mixed-size jobs into the serving loop
            (gbwt_server_*): p50/p99 latency and sustained MB/s at the offered
            load and saturated, next to the same jobs run one after another;
  config3   the 256 MiB versioned large-alphabet text with W=5 P=23, with its
            reference program and libcubwt.

``--impl reference`` is the reference arm: the reference's own CUDA PFP
program (W=5 P=16) on the whole 512 MiB text, one process run per step, on
rank 0; the reference has no CPU implementation of this path.

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

METRIC = "BWT input MB/s (bit-exact) plain vs batched on 1 GB300; serving p50/p99 latency"
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


def replica_timing(ms, e2e_ms, ws, n, device):
    """One text per rank (replicas, no exchange between ranks): the step time of
    the job is the slowest rank's (max over ranks), the throughput every rank's
    text over it.  Returns (ms, e2e_ms, MB/s, e2e MB/s)."""
    if ws > 1:
        import torch
        t = torch.tensor([ms, e2e_ms], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, e2e_ms = float(t[0]), float(t[1])
    return ms, e2e_ms, ws * n / (ms / 1000.0) / 1e6, ws * n / (e2e_ms / 1000.0) / 1e6


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
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix=f"gbwt_clocks_gpu{self.gpu}_", suffix=".csv")
            self.fh = os.fdopen(fd, "w")
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
        self.samples = self._read()
        if self.path and os.path.exists(self.path):
            os.remove(self.path)

    def _read(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return None
        with open(self.path) as f:
            return f.read().splitlines()

    def summary(self):
        lines = getattr(self, "samples", None)
        if lines is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in lines:
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


def host_cores():
    try:
        aff = len(os.sched_getaffinity(0))
    except AttributeError:
        aff = os.cpu_count() or 1
    return {"nproc": os.cpu_count() or 1, "affinity": aff}


def _sa_is_child(queue):
    """Spawned process: the suffix-array (SA-IS) BWT of the whole 512 MiB text on one host core."""
    import hashlib
    sys.path.insert(0, ROOT)
    import oracle
    wl = importlib.import_module(PKG + ".workloads")
    text = wl.config2_text()
    oracle.build()
    t0 = time.perf_counter()
    L = oracle.sa_bwt(text)
    dt = time.perf_counter() - t0
    queue.put({"seconds": dt, "n": len(text), "blake2b": hashlib.blake2b(L.tobytes(), digest_size=16).hexdigest()})


def reference_programs(variants):
    """Stage (where a reference checkout exists) and compile the reference programs; None or why not."""
    try:
        from oracle import reference
        reference.stage()
        res = reference.build(variants)
        bad = [k for k, v in res.items() if v is not None]
        if bad:
            return "reference build failed: " + ", ".join(os.path.basename(b) for b in bad)
        missing = [v for v in variants if not reference.available(v)]
        if missing:
            return "reference sources not staged in oracle/_ref/src (" + ", ".join(missing) + ")"
        return None
    except Exception as e:          # noqa: BLE001 -- reported on the JSON line
        return f"reference build: {e}"


def run_reference(args):
    """The reference arm: the reference's own PFP program (W=5, P=16) on the whole 512 MiB text per step.

    The reference has no CPU implementation of this path: it is a CUDA program
    (Prefix_Free_Parsing_W=5_P=16.cu).  It is compiled unmodified for sm_103a
    (oracle/reference.py) and run once per step on this GPU, after the host
    guard has checked that the text holds no phrase its device asserts reject.
    value = the device-resident span Compute_D + Compute_S (CUDA events, the
    span this library's `value` measures); e2e = the host-to-host span
    (allocation + H2D + both stages + D2H), the span of this library's e2e.
    Where the program cannot be built or the guard refuses, the oracle's CPU
    port on a 16 MiB prefix stands in, and the line says so.
    """
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    wl = importlib.import_module(PKG + ".workloads")
    text = wl.config2_text()
    n = len(text)
    why = reference_programs(["W5_P16"])
    sess = None
    if why is None:
        from oracle import reference
        try:
            sess = reference.PfpSession(text, 5, 16, False)
        except reference.ReferenceRefused as e:
            why = f"refused by the host guard: {e}"
    dev, host = [], []
    if sess is not None:
        try:
            for i in range(args.warmup + args.steps):
                _, info = sess.run(keep_output=False)
                if i >= args.warmup:
                    dev.append(info["device_ms"])
                    host.append(info["host_ms"])
        except (RuntimeError, subprocess.TimeoutExpired) as e:
            why = f"the reference program failed: {e}"
        finally:
            sess.close()
    if why is None:
        ms, e2e_ms = statistics.mean(dev), statistics.mean(host)
        value = n / (ms / 1000.0) / 1e6
        e2e = n / (e2e_ms / 1000.0) / 1e6
        line = {
            "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n": n, "W": 5, "P": 16, "small_alphabet": False,
                       "program": "Prefix_Free_Parsing_W=5_P=16.cu, unmodified, nvcc -O2 --use_fast_math "
                                  "--expt-relaxed-constexpr for sm_103a; one process run per step",
                       "span": "value: Compute_D + Compute_S (CUDA events); e2e: allocation + H2D + both + D2H"},
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": 1, "kind": "reference",
                             "sample": "the whole 512 MiB text per step; the reference's own CUDA program on this "
                                       "GB300 (it has no CPU implementation of this path), one host thread",
                             "device": "GPU"},
            "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": n, "d2h_bytes_per_step": n,
                    "ms_per_step": round(e2e_ms, 3)},
            "device_ms_all": [round(x, 2) for x in dev],
        }
        print(json.dumps(line), flush=True)
        return 0
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
                   "W": 5, "P": 16, "reference_program_unavailable": why},
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"first {args.cpu_sample_mib} MiB of the 512 MiB text (oracle PFP port; the "
                                   "reference's CUDA program was unavailable: " + str(why) + ")"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def measure_reference_cuda(text, ours, ours_value, ours_e2e, W, P, small, runs):
    """The reference's own PFP program of one variant on `text`: MB/s of both spans, bit-exactness vs `ours`."""
    why = reference_programs([f"W{W}_P{P}" + ("_small" if small else "")])
    if why is not None:
        return {"unavailable": why}
    import numpy as np
    from oracle import reference
    try:
        sess = reference.PfpSession(text, W, P, small)
    except reference.ReferenceRefused as e:
        return {"unavailable": f"refused by the host guard: {e}"}
    n = len(text)
    dev, host, same = [], [], None
    try:
        for i in range(runs):
            L, info = sess.run(keep_output=(i == 0))
            if L is not None:
                same = bool(np.array_equal(L, ours))
            dev.append(info["device_ms"])
            host.append(info["host_ms"])
    finally:
        sess.close()
    ms, hms = statistics.median(dev), statistics.median(host)
    value, e2e = n / (ms / 1000.0) / 1e6, n / (hms / 1000.0) / 1e6
    return {"program": reference.PFP_VARIANTS[sess.variant][0], "runs": runs, "z": info["z"],
            "value": round(value, 2), "ms": round(ms, 2), "e2e": round(e2e, 2), "host_ms": round(hms, 2),
            "unit": UNIT, "bitexact_vs_gbwt": same,
            "speedup_of_gbwt": round(ours_value / value, 2) if ours_value else None,
            "speedup_of_gbwt_e2e": round(ours_e2e / e2e, 2) if ours_e2e else None}


def measure_libcubwt(text, ours, ours_e2e, reps):
    """libcubwt 1.6.3 as shipped by the reference: host-to-host MB/s, bit-exactness vs `ours`."""
    why = reference_programs([])
    if why is None:
        from oracle import reference
        if not reference.available():
            why = "libcubwt source not staged in oracle/_ref/src"
    if why is not None:
        return {"unavailable": why}
    import numpy as np
    from oracle import reference
    L, info = reference.run_libcubwt(text, repetitions=reps)
    n = len(text)
    e2e = n / (info["host_ms"] / 1000.0) / 1e6
    return {"program": "libcubwt.cu 1.6.3 (libcubwt_bwt, storage allocated once, pinned host buffers)",
            "runs": reps, "host_ms": round(info["host_ms"], 2), "e2e": round(e2e, 2), "unit": UNIT,
            "span": "host to host (libcubwt_bwt copies in and out inside the call)",
            "bitexact_vs_gbwt": bool(np.array_equal(L, ours)),
            "speedup_of_gbwt_e2e": round(ours_e2e / e2e, 2) if ours_e2e else None}


def roofline_pipeline(stats, n, W, ms, peak, peak_kind):
    """Whole-pipeline algorithmic bytes (4n + (24+W)z + 3L_d + 8d + 8s) over the step time."""
    b = 4 * n + (24 + W) * stats["z"] + 3 * stats["dict_bytes"] + 8 * stats["d"] + 8 * stats["s"]
    achieved = b / (ms / 1000.0) / 1e9
    return {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "algorithmic_bytes": int(b),
            "formula": "4n + (24+W)z + 3 dict_bytes + 8d + 8s", "peak_kind": f"of {peak_kind}"}


def time_device(st, dev_text, dev_out, n, W, P, small, steps):
    """Mean CUDA-event ms of `steps` device-resident BWTs on the storage's stream."""
    import torch
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        st.pfp_bwt_device(dev_text.data_ptr(), dev_out.data_ptr(), n, W, P, small)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def measure_text(args, pkg, text, W, P, small, peak, peak_kind, label):
    """One more workload or variant: device-resident and end-to-end MB/s, stage times, pipeline roofline,
    and the reference's own program and libcubwt on the same text (bit-exactness checked)."""
    import numpy as np
    import torch

    n = len(text)
    stream = torch.cuda.current_stream()
    dev_text = torch.from_numpy(text).cuda()
    dev_out = torch.empty_like(dev_text)
    host_text = torch.from_numpy(text).pin_memory()
    host_out = torch.empty(n, dtype=torch.uint8).pin_memory()
    steps = max(3, min(args.steps, 10))
    with pkg.Storage(n) as st:
        st.set_stream(stream.cuda_stream)
        for _ in range(3):
            st.pfp_bwt_device(dev_text.data_ptr(), dev_out.data_ptr(), n, W, P, small)
        torch.cuda.synchronize()
        ms = time_device(st, dev_text, dev_out, n, W, P, small, steps)
        stats = st.stats()
        st.pfp_bwt_device(dev_text.data_ptr(), dev_out.data_ptr(), n, W, P, small, stage_times=True)
        torch.cuda.synchronize()
        stage = st.stats()["stage_ms"]
        st.pfp_bwt_into(host_text.numpy(), host_out.numpy(), W, P, small)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            st.pfp_bwt_into(host_text.numpy(), host_out.numpy(), W, P, small)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1) / steps
    ours = host_out.numpy().copy()
    if not np.array_equal(dev_out.cpu().numpy(), ours):
        raise SystemExit(f"bench: device and host paths differ ({label})")
    del dev_text, dev_out, host_text, host_out
    value = n / (ms / 1000.0) / 1e6
    e2e = n / (e2e_ms / 1000.0) / 1e6
    out = {"workload": label, "n": n, "W": W, "P": P, "small_alphabet": small, "steps": steps,
           "value": round(value, 2), "unit": UNIT, "ms_per_step": round(ms, 3),
           "e2e": {"value": round(e2e, 2), "unit": UNIT, "ms_per_step": round(e2e_ms, 3),
                   "h2d_bytes_per_step": n, "d2h_bytes_per_step": n},
           "stage_ms": stage,
           "pipeline": {k: stats[k] for k in ("z", "d", "dict_bytes", "s", "mixed_blocks", "mixed_elems",
                                              "dict_rounds", "parse_rounds")},
           "roofline_pipeline": roofline_pipeline(stats, n, W, ms, peak, peak_kind)}
    if "reference" in args.sections:
        out["reference_cuda"] = measure_reference_cuda(text, ours, value, e2e, W, P, small, args.ref_runs)
        if not small:
            out["libcubwt"] = measure_libcubwt(text, ours, e2e, args.libcubwt_reps)
    return out, ours


def run_gpu(args):
    import multiprocessing as mp

    import numpy as np

    ws, rank, local = dist_env()
    # Nothing runs beside the GPU measurements on the host: the 256 MiB Markov
    # text is generated right before its own section, and the SA-IS baseline
    # runs in a spawned process (never forked after CUDA is up) after every GPU
    # measurement.  Host-side work in parallel slowed the end-to-end copies and
    # the serving latencies.
    ctx = mp.get_context("spawn")
    sa_queue = sa_proc = None

    import torch
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
    got = host_out.numpy().copy()
    if not np.array_equal(np.bincount(got, minlength=256), np.bincount(text, minlength=256)):
        raise SystemExit("bench: BWT is not a permutation of the text")
    if not np.array_equal(dev_out.cpu().numpy(), got):
        raise SystemExit("bench: device and host paths differ")

    ms, e2e_ms, value, e2e_value = replica_timing(ms, e2e_ms, ws, n, "cuda")
    if rank != 0:
        torch.distributed.destroy_process_group()
        return 0

    peak, peak_kind = measured_peak()
    roofline = roofline_of(probe, "k_seg_sort", "k_seg_sort<ParseRem/DictRem> (prefix-doubling rounds in CTAs)",
                           peak, peak_kind, args.steps, ms)
    roofline_radix = roofline_of(probe_radix, "k_rs_downsweep", "k_rs_downsweep (radix scatter)", peak, peak_kind,
                                 1, ms)
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
        "roofline_pipeline": roofline_pipeline(stats, n, 5, ms, peak, peak_kind),
        "clocks": clocks,
        "gpu_launches": launches,
        "inverse_bwt": {"value": round(n / (unbwt_ms / 1000.0) / 1e6, 2), "unit": UNIT, "ms": round(unbwt_ms, 3),
                        "check": "gbwt_unbwt(BWT, primary index) == text"},
        "pipeline": {k: stats[k] for k in ("z", "d", "dict_bytes", "s", "mixed_blocks", "mixed_elems",
                                             "dict_rounds", "parse_rounds", "hash_retries")},
        "stage_ms": stage["stage_ms"],
    }
    del dev_text, dev_out, host_text, host_out
    st.close()
    torch.cuda.empty_cache()

    # latency first, before the long sections and while the host is quiet
    if "serving" in args.sections:
        line["serving"] = measure_serving(args, pkg, wl)
        log(f"[rank 0] serving: {line['serving']['latency_ms']}")
    if "reference" in args.sections:
        line["reference_cuda"] = measure_reference_cuda(text, got, value, e2e_value, 5, 16, False, args.ref_runs)
        log(f"[rank 0] reference program: {line['reference_cuda']}")
        line["libcubwt"] = measure_libcubwt(text, got, e2e_value, args.libcubwt_reps)
        log(f"[rank 0] libcubwt: {line['libcubwt']}")
    if "variants" in args.sections:
        line["variants"] = {}
        for (W, P, small) in ((5, 16, True), (35, 81, True)):
            res, other = measure_text(args, pkg, text, W, P, small, peak, peak_kind,
                                      "the same 512 MiB text, " + f"W={W} P={P}" + (" small alphabet" if small
                                                                                    else ""))
            res["bitexact_vs_w5p16"] = bool(np.array_equal(other, got))
            line["variants"][f"W{W}_P{P}" + ("_small" if small else "")] = res
            log(f"[rank 0] variant W={W} P={P} small={small}: {res['value']} MB/s")
    if "batched" in args.sections:
        line["batched"] = measure_batched(args, pkg, wl, stream)
        log(f"[rank 0] batched: {line['batched']['value']} MB/s")
    if "config3" in args.sections:
        t0 = time.time()
        t3 = wl.config3_text()
        log(f"[rank 0] config 3 text generated ({time.time() - t0:.1f}s)")
        res, _ = measure_text(args, pkg, t3, 5, 23, False, peak, peak_kind, CONFIG3_WORKLOAD)
        line["config3"] = res
        log(f"[rank 0] config 3: {res['value']} MB/s")
        del t3
    if "cpu" in args.sections:
        sa_queue = ctx.Queue()
        sa_proc = ctx.Process(target=_sa_is_child, args=(sa_queue,), daemon=True)
        sa_proc.start()
    line["cpu_baseline"] = cpu_baseline(sa_proc, sa_queue, got, args)
    print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


CONFIG3_WORKLOAD = ("256 MiB versioned text: 2 MiB order-3 Markov base over the 96 byte values 32..127 (rows "
                    "Dirichlet(0.1), seed 3), 128 successive versions with 1-64-byte block replacements at rate 1e-4 "
                    "per byte; PFP W=5 P=23")


def cpu_baseline(sa_proc, sa_queue, ours, args):
    """The suffix-array BWT (SA-IS, one host core) of the whole 512 MiB text, from the spawned helper."""
    import hashlib
    cores = host_cores()
    if sa_proc is None:
        text = importlib.import_module(PKG + ".workloads").config2_text()
        v, dt, nb, threads = cpu_port_sample(text, args.cpu_sample_mib << 20)
        return {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": "port", "host": cores,
                "sample": f"first {nb >> 20} MiB of the same text, oracle PFP port, one run ({dt:.1f} s)"}
    try:
        res = sa_queue.get(timeout=args.cpu_timeout)
    except Exception:                      # noqa: BLE001 -- the helper did not finish in time
        sa_proc.terminate()
        return {"unavailable": f"SA-IS of the whole text did not finish within {args.cpu_timeout} s", "host": cores}
    sa_proc.join(timeout=30)
    same = res["blake2b"] == hashlib.blake2b(ours.tobytes(), digest_size=16).hexdigest()
    return {"value": round(res["n"] / res["seconds"] / 1e6, 3), "unit": UNIT, "cores": 1, "kind": "port",
            "method": "SA-IS suffix-array BWT (oracle/sa_bwt.c, Nong-Zhang-Chan induced sorting), one thread",
            "sample": f"the whole {res['n']}-byte text, one run ({res['seconds']:.1f} s), in a spawned process "
                      "after the GPU measurements", "host": cores, "bitexact_vs_gbwt": same}


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
    outs = [np.empty(len(t), np.uint8) for t in texts]

    def run(arrive):
        with pkg.Server(workers=2, small_max=small_max) as srv:
            # warm-up: one large job and a burst of small ones
            for t in texts[:64]:
                srv.submit(t)
            srv.submit(max(texts, key=len))
            srv.drain()
            t0 = time.perf_counter()
            tickets = []
            for t, at, o in zip(texts, arrive, outs):
                delay = at - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                tickets.append(srv.submit(t, out=o))
            srv.drain()
            return [srv.poll(k) for k in tickets]

    # saturated: every job arrives at once, so the loop runs at its capacity
    sat = run([0.0] * len(texts))
    if any(i["status"] != 0 for i in sat):
        raise SystemExit("bench: a serving job failed (saturated)")
    sat_lat = [(i["end_us"] - i["submit_us"]) / 1000.0 for i in sat]
    sat_span = (max(i["end_us"] for i in sat) - min(i["submit_us"] for i in sat)) / 1e6
    infos = run(arrivals)
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
        "saturated": {"value": round(total / sat_span / 1e6, 2), "unit": UNIT,
                      "arrivals": "all jobs submitted at once (arrival rate above capacity)",
                      "latency_ms": pkg.percentiles(sat_lat),
                      "max_batch_jobs": max(i["batch_jobs"] for i in sat)},
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
    ap.add_argument("--sections", default="plain,reference,variants,batched,serving,config3,cpu",
                    help="comma list: the plain headline always runs; reference (the reference's own PFP "
                         "program and libcubwt), variants (small-alphabet W=5 P=16 and W=35 P=81), batched, "
                         "serving, config3 (256 MiB versioned text, W=5 P=23) and cpu (SA-IS of the whole text) "
                         "are extra sections")
    ap.add_argument("--ref-runs", type=int, default=3, help="process runs of each reference PFP program")
    ap.add_argument("--libcubwt-reps", type=int, default=5, help="timed libcubwt_bwt calls")
    ap.add_argument("--cpu-timeout", type=float, default=900.0, help="seconds to wait for the SA-IS baseline")
    ap.add_argument("--batch-steps", type=int, default=5)
    ap.add_argument("--serve-jobs", type=int, default=800)
    ap.add_argument("--serve-rate", type=float, default=1000.0)
    args = ap.parse_args(argv)
    args.sections = set(args.sections.split(","))
    if args.warmup < 3:
        log("bench: warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
