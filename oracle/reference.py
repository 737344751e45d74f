"""The reference's own CUDA programs, built and run as a checker -- TEST INFRASTRUCTURE ONLY.

The reference ships its PFP BWT as stand-alone CUDA programs
(``Prefix_Free_Parsing_W=*_P=*[_small_alphabet].cu``, one per variant) and a
copy of libcubwt 1.6.3 (``libcubwt.cu``/``libcubwt.cuh``) that its
``compare_script.sh:7-10`` checks the PFP output against.  This module

* ``stage()``  -- copies those unmodified source files from a reference
  checkout into ``oracle/_ref/src/`` (git-ignored: the sources never enter
  this repository's history; the folder travels with the working tree so the
  GPU host can compile them);
* ``build()``  -- compiles ``oracle/ref_pfp_driver.cu`` once per variant and
  ``oracle/ref_libcubwt_driver.cu`` around them with the reference's own
  nvcc flags (Makefile:7-8) retargeted to sm_103a, into ``oracle/_ref/``;
* ``guard()``  -- decides on the host, before any launch, whether a text is
  one the reference program accepts: its device code asserts
  ``W < phrase length < 8192`` (K:584-585), and a failed device assert would
  take down the GPU context, so such texts are never handed to it;
* ``run_pfp()`` / ``run_libcubwt()`` -- run one program on a text and return
  its output bytes (the reference's output convention) and its times.

Only tests/, ``__graft_entry__`` (to build) and ``bench.py``'s baseline legs
use this module.  The product path never does.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
SRC_DIR = os.path.join(REF_DIR, "src")
DEFAULT_CHECKOUT = "/root/reference"

# variant -> (source file, W, P, small alphabet); the nine programs of Makefile:13-23
PFP_VARIANTS = {
    "W5_P11": ("Prefix_Free_Parsing_W=5_P=11.cu", 5, 11, False),
    "W5_P13": ("Prefix_Free_Parsing_W=5_P=13.cu", 5, 13, False),
    "W5_P14": ("Prefix_Free_Parsing_W=5_P=14.cu", 5, 14, False),
    "W5_P16": ("Prefix_Free_Parsing_W=5_P=16.cu", 5, 16, False),
    "W5_P23": ("Prefix_Free_Parsing_W=5_P=23.cu", 5, 23, False),
    "W5_P14_small": ("Prefix_Free_Parsing_W=5_P=14_small_alphabet.cu", 5, 14, True),
    "W5_P16_small": ("Prefix_Free_Parsing_W=5_P=16_small_alphabet.cu", 5, 16, True),
    "W5_P23_small": ("Prefix_Free_Parsing_W=5_P=23_small_alphabet.cu", 5, 23, True),
    "W35_P81_small": ("Prefix_Free_Parsing_W=35_P=81_small_alphabet.cu", 35, 81, True),
}
LIBCUBWT_SOURCES = ("libcubwt.cu", "libcubwt.cuh")
# the reference's Makefile:7-8 flags, sm_75 replaced by this GPU's architecture
NVCC_FLAGS = ["-O2", "--use_fast_math", "--expt-relaxed-constexpr", "-std=c++17",
              "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-O2"]

# Texts below this size are not handed to the reference programs: the thesis
# ran them on 45-558 MB files only, and their small-size paths are unexercised.
MIN_TEXT = 1 << 20
MAX_PHRASE = 8192          # K:584: assert(length_d < 8192)


def variant_name(W: int, P: int, small: bool) -> str:
    return f"W{W}_P{P}" + ("_small" if small else "")


def pfp_binary(variant: str) -> str:
    return os.path.join(REF_DIR, "ref_pfp_" + variant)


LIBCUBWT_BIN = os.path.join(REF_DIR, "ref_libcubwt")


def stage(checkout: str = DEFAULT_CHECKOUT) -> bool:
    """Copy the reference's unmodified sources into oracle/_ref/src; False without a checkout."""
    if not os.path.isdir(checkout):
        return False
    os.makedirs(SRC_DIR, exist_ok=True)
    names = [v[0] for v in PFP_VARIANTS.values()] + list(LIBCUBWT_SOURCES)
    for name in names:
        src = os.path.join(checkout, name)
        dst = os.path.join(SRC_DIR, name)
        if os.path.exists(src) and (not os.path.exists(dst) or os.path.getmtime(dst) < os.path.getmtime(src)):
            shutil.copyfile(src, dst)
    return True


def _nvcc() -> str | None:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand if os.path.exists(cand) else None


def _jobs(variants) -> list[tuple[str, list[str]]]:
    nvcc = _nvcc()
    jobs = []
    if nvcc is None:
        return jobs
    drv = os.path.join(HERE, "ref_pfp_driver.cu")
    for v in variants:
        src = os.path.join(SRC_DIR, PFP_VARIANTS[v][0])
        out = pfp_binary(v)
        if not os.path.exists(src):
            continue
        if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(src), os.path.getmtime(drv)):
            continue
        jobs.append((out, [nvcc, *NVCC_FLAGS, "-I" + SRC_DIR, f'-DREF_PFP_SOURCE="{PFP_VARIANTS[v][0]}"',
                           "-o", out, drv]))
    ldrv = os.path.join(HERE, "ref_libcubwt_driver.cu")
    lsrc = os.path.join(SRC_DIR, "libcubwt.cu")
    if os.path.exists(lsrc) and (not os.path.exists(LIBCUBWT_BIN) or os.path.getmtime(LIBCUBWT_BIN) <
                                 max(os.path.getmtime(lsrc), os.path.getmtime(ldrv))):
        jobs.append((LIBCUBWT_BIN, [nvcc, *NVCC_FLAGS, "-I" + SRC_DIR, "-o", LIBCUBWT_BIN, ldrv]))
    return jobs


def build(variants=None, stage_first: bool = True) -> dict:
    """Compile the staged reference programs (if stale) in parallel; returns {binary: error or None}."""
    if stage_first:
        stage()
    variants = list(PFP_VARIANTS) if variants is None else list(variants)
    jobs = _jobs(variants)
    result = {}

    def run(job):
        out, cmd = job
        r = subprocess.run(cmd, capture_output=True, text=True)
        return out, (None if r.returncode == 0 else (r.stdout + r.stderr)[-2000:])

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for out, err in ex.map(run, jobs):
                result[out] = err
    return result


def available(variant: str | None = None) -> bool:
    if variant is None:
        return os.path.exists(LIBCUBWT_BIN)
    return os.path.exists(pfp_binary(variant))


def guard(text, W: int, P: int, small: bool) -> str | None:
    """None when the reference PFP program accepts ``text``; otherwise why it must not run.

    Checked on the host with the oracle's trigger scan (the reference's own
    trigger rule, K:443-576): bytes in [2,254] (K:130-132; [2,15] for the
    small-alphabet digit packing, SA16:995-1002), the size range, and every
    phrase length L with W < L < 8192 (the device asserts of K:584-585).
    """
    from . import trigger_scan
    t = np.ascontiguousarray(text, dtype=np.uint8)
    n = len(t)
    if n < MIN_TEXT:
        return f"text of {n} bytes is below the {MIN_TEXT}-byte minimum handed to the reference programs"
    if n + W + 2 > 0x7fffffff:
        return "text too long for the reference's int sizes"
    lo, hi = int(t.min()), int(t.max())
    if lo < 2 or hi > 254:
        return f"byte values [{lo},{hi}] outside the reference's input range [2,254]"
    if small and hi > 15:
        return f"byte value {hi} above 15: the small-alphabet digit packing does not fit"
    D = trigger_scan(t, W, P)
    lens = np.empty(len(D), dtype=np.int64)
    lens[0] = D[0] + 1
    lens[1:] = np.diff(D) + W
    if int(lens.max()) >= MAX_PHRASE:
        return f"a phrase of {int(lens.max())} bytes: the reference asserts length < {MAX_PHRASE} on the GPU"
    if int(lens.min()) <= W:
        return f"a phrase of {int(lens.min())} bytes: the reference asserts length > W on the GPU"
    return None


class ReferenceRefused(RuntimeError):
    """The text is outside what the reference program accepts; nothing was launched."""


def _tmpdir() -> str:
    return tempfile.mkdtemp(prefix="gbwt_ref_")


def run_pfp(text, W: int, P: int, small: bool, timeout: float = 600.0, checked: str | None = "check"):
    """Run the reference PFP program of the variant on ``text``.

    Returns (bwt bytes, info dict with device_ms / host_ms / z).  The guard
    runs first unless the caller passes ``checked=None`` after running
    ``guard`` on the same text itself; a refused text raises
    ReferenceRefused without launching anything.
    """
    variant = variant_name(W, P, small)
    if variant not in PFP_VARIANTS:
        raise ValueError(f"the reference has no program for {variant}")
    if not available(variant):
        raise FileNotFoundError(pfp_binary(variant))
    if checked is not None:
        why = guard(text, W, P, small)
        if why is not None:
            raise ReferenceRefused(why)
    t = np.ascontiguousarray(text, dtype=np.uint8)
    d = _tmpdir()
    try:
        tin = os.path.join(d, "text.bin")
        t.tofile(tin)
        return _run_pfp_file(variant, tin, len(t), d, timeout, keep_output=True)
    finally:
        shutil.rmtree(d, ignore_errors=True)


def _run_pfp_file(variant: str, text_path: str, n: int, workdir: str, timeout: float, keep_output: bool):
    out = os.path.join(workdir, "bwt.bin")
    r = subprocess.run([pfp_binary(variant), text_path, out], capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference {variant} exited {r.returncode}: {r.stderr[-1000:]}")
    info = json.loads(r.stdout.strip().splitlines()[-1])
    L = np.fromfile(out, dtype=np.uint8) if keep_output else None
    os.remove(out)
    if keep_output and len(L) != n:
        raise RuntimeError(f"reference {variant} wrote {len(L)} bytes for a {n}-byte text")
    return L, info


class PfpSession:
    """Repeated runs of one reference PFP program on one text, written to a file once.

    The guard runs once in the constructor (ReferenceRefused without a
    launch); each ``run()`` is one process run of the program: one BWT,
    returned with its times when ``keep_output``.
    """

    def __init__(self, text, W: int, P: int, small: bool, timeout: float = 600.0):
        self.variant = variant_name(W, P, small)
        if self.variant not in PFP_VARIANTS:
            raise ValueError(f"the reference has no program for {self.variant}")
        if not available(self.variant):
            raise FileNotFoundError(pfp_binary(self.variant))
        why = guard(text, W, P, small)
        if why is not None:
            raise ReferenceRefused(why)
        t = np.ascontiguousarray(text, dtype=np.uint8)
        self.n = len(t)
        self.timeout = timeout
        self.dir = _tmpdir()
        self.path = os.path.join(self.dir, "text.bin")
        t.tofile(self.path)

    def run(self, keep_output: bool = False):
        return _run_pfp_file(self.variant, self.path, self.n, self.dir, self.timeout, keep_output)

    def close(self):
        shutil.rmtree(self.dir, ignore_errors=True)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def run_libcubwt(text, repetitions: int = 1, timeout: float = 600.0):
    """Run libcubwt_bwt (warm-up + ``repetitions`` timed calls); returns (bwt bytes, info dict)."""
    if not available():
        raise FileNotFoundError(LIBCUBWT_BIN)
    t = np.ascontiguousarray(text, dtype=np.uint8)
    if len(t) < 16:
        raise ReferenceRefused("libcubwt_bwt needs at least 16 bytes (libcubwt.cu:2418)")
    d = _tmpdir()
    try:
        tin, tout = os.path.join(d, "text.bin"), os.path.join(d, "bwt.bin")
        t.tofile(tin)
        r = subprocess.run([LIBCUBWT_BIN, tin, tout, str(int(repetitions))], capture_output=True, text=True,
                           timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"libcubwt exited {r.returncode}: {r.stderr[-1000:]}")
        info = json.loads(r.stdout.strip().splitlines()[-1])
        L = np.fromfile(tout, dtype=np.uint8)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    if len(L) != len(t):
        raise RuntimeError(f"libcubwt wrote {len(L)} bytes for a {len(t)}-byte text")
    return L, info


if __name__ == "__main__":
    import sys
    staged = stage()
    res = build()
    for out, err in sorted(res.items()):
        print(("ok    " if err is None else "FAILED ") + out + ("" if err is None else "\n" + err), file=sys.stderr)
    print(json.dumps({"staged": staged, "built": sorted(k for k, v in res.items() if v is None),
                      "failed": sorted(k for k, v in res.items() if v is not None)}))
