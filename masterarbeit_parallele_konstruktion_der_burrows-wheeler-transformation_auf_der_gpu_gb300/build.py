"""Build recipe for the in-tree CUDA library ``libgbwt.so`` and the CLI.

Every translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked into
``libgbwt.so`` next to this file.  The command-line drop-in ``gbwt_pfp``
(the reference's ``input.txt`` -> ``out.txt`` programs) links against it.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbwt.so")
CLI = os.path.join(HERE, "gbwt_pfp")

CU_SOURCES = ["pfp_scan.cu", "pfp_phrases.cu", "pfp_sort.cu", "pfp_assembly.cu", "pfp_batch.cu", "gbwt_api.cu",
              "gbwt_serve.cu", "pfp_unbwt.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build libgbwt")
    return cand


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> str:
    """Compile the CUDA sources (if stale) and return the path of libgbwt.so."""
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(HERE, "..", "include", "gbwt.h"))
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", *ARCH]
    if ptxas_info:
        flags += ["-Xptxas", "-v"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or ptxas_info or _stale(o, [s, *headers]):
            jobs.append([nvcc(), *flags, "-c", s, "-o", o])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for cmd, fut in zip(jobs, [ex.submit(_run, j) for j in jobs]):
                fut.result()
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc(), "-shared", *ARCH, "-o", LIB, *objs])
    cli_src = os.path.join(CSRC, "gbwt_cli.cpp")
    if force or _stale(CLI, [cli_src, LIB]):
        _run([nvcc(), "-O2", "-std=c++17", "-o", CLI, cli_src, "-L" + HERE, "-lgbwt",
              "-Xlinker", "-rpath=$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
