"""The oracle -- TEST INFRASTRUCTURE ONLY.

CPU restatement of the reference's prefix-free-parsing BWT (pfp_oracle.c) and
an independent suffix-array BWT (sa_bwt.c), loaded through ctypes.  Only
tests/, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` may use
this package; the product path never does.

Parity anchor: the reference ships no golden vectors; its only correctness
check compares the PFP output byte for byte with libcubwt's
(compare_script.sh:7-10).  This restatement is checked against the
suffix-array BWT in that output convention on every test input, and the
reference's own CUDA programs and its libcubwt copy, built and run by
``oracle.reference``, are compared with the GPU path on the benchmark texts.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
SOURCES = ["pfp_oracle.c", "sa_bwt.c"]


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc (OpenMP when available)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, "oracle.h")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return LIB
    base = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-o", LIB, *srcs]
    r = subprocess.run(base[:4] + ["-fopenmp"] + base[4:], capture_output=True, text=True)
    if r.returncode != 0:
        r = subprocess.run(base, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


class Stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in
                ("z", "d", "dict_bytes", "s", "mixed_blocks", "mixed_elems", "max_phrase_len")]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        i64p = ctypes.POINTER(ctypes.c_int64)
        L.gbo_trigger_scan.argtypes = [u8p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, i64p]
        L.gbo_trigger_scan.restype = ctypes.c_int64
        L.gbo_pfp_bwt_ex.argtypes = [u8p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int, u8p,
                                     ctypes.POINTER(Stats), i64p, i64p]
        L.gbo_pfp_bwt_ex.restype = ctypes.c_int
        L.gbo_sa_bwt.argtypes = [u8p, ctypes.c_int64, u8p]
        L.gbo_sa_bwt.restype = ctypes.c_int
        L.gbo_suffix_array.argtypes = [u8p, ctypes.c_int64, i64p]
        L.gbo_suffix_array.restype = ctypes.c_int
        L.gbo_validate.argtypes = [u8p, ctypes.c_int64, ctypes.c_int]
        L.gbo_validate.restype = ctypes.c_int
        L.gbo_max_threads.restype = ctypes.c_int
        L.gbo_threads_used.restype = ctypes.c_int
        L.gbo_primary_index.argtypes = [u8p, ctypes.c_int64]
        L.gbo_primary_index.restype = ctypes.c_int64
        L.gbo_unbwt.argtypes = [u8p, ctypes.c_int64, ctypes.c_int64, u8p]
        L.gbo_unbwt.restype = ctypes.c_int
        _lib = L
    return _lib


def _u8(a):
    a = np.ascontiguousarray(a, dtype=np.uint8)
    return a, a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def trigger_scan(text, W: int, P: int) -> np.ndarray:
    """Phrase end positions D (K:443-576)."""
    t, tp = _u8(text)
    D = np.zeros(len(t) + 2, dtype=np.int64)
    z = lib().gbo_trigger_scan(tp, len(t), W, P, D.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    return D[:z].copy()


class OracleError(RuntimeError):
    def __init__(self, code: int):
        super().__init__(f"oracle error {code}")
        self.code = code


def pfp_bwt(text, W: int = 5, P: int = 16, small_alphabet: bool = False, with_parse: bool = False):
    """PFP BWT restated on the CPU; returns (L, stats[, meta, parse_sa])."""
    t, tp = _u8(text)
    n = len(t)
    L = np.zeros(max(n, 1), dtype=np.uint8)
    st = Stats()
    i64p = ctypes.POINTER(ctypes.c_int64)
    meta = sa = None
    if with_parse:
        meta = np.zeros(n + 2, dtype=np.int64)
        sa = np.zeros(n + 2, dtype=np.int64)
    rc = lib().gbo_pfp_bwt_ex(tp, n, W, P, int(small_alphabet), L.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                              ctypes.byref(st), meta.ctypes.data_as(i64p) if with_parse else None,
                              sa.ctypes.data_as(i64p) if with_parse else None)
    if rc != 0:
        raise OracleError(rc)
    stats = {k: getattr(st, k) for k, _ in Stats._fields_}
    if with_parse:
        z = stats["z"]
        return L[:n], stats, meta[:z].copy(), sa[:z].copy()
    return L[:n], stats


def sa_bwt(text) -> np.ndarray:
    """Suffix-array BWT (SA-IS) in the PFP output convention."""
    t, tp = _u8(text)
    n = len(t)
    L = np.zeros(max(n, 1), dtype=np.uint8)
    rc = lib().gbo_sa_bwt(tp, n, L.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    if rc != 0:
        raise OracleError(rc)
    return L[:n]


def suffix_array(text) -> np.ndarray:
    t, tp = _u8(text)
    SA = np.zeros(max(len(t), 1), dtype=np.int64)
    rc = lib().gbo_suffix_array(tp, len(t), SA.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    if rc != 0:
        raise OracleError(rc)
    return SA[:len(t)]


def validate(text, small_alphabet: bool = False) -> int:
    t, tp = _u8(text)
    return lib().gbo_validate(tp, len(t), int(small_alphabet))


def primary_index(text) -> int:
    """Output row of the suffix starting at text[0]."""
    t, tp = _u8(text)
    return int(lib().gbo_primary_index(tp, len(t)))


def unbwt(L_bytes, pidx: int) -> np.ndarray:
    """Inverse of the PFP-convention BWT given the primary index."""
    b, bp = _u8(L_bytes)
    T = np.zeros(max(len(b), 1), dtype=np.uint8)
    rc = lib().gbo_unbwt(bp, len(b), int(pidx), T.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    if rc != 0:
        raise OracleError(rc)
    return T[:len(b)]


def max_threads() -> int:
    return lib().gbo_max_threads()


def max_threads_used() -> int:
    """Host threads the PFP port actually runs on."""
    return lib().gbo_threads_used()


def dense_ranks(meta: np.ndarray) -> np.ndarray:
    """The reference's meta-characters (index of the last equal occurrence in
    lexicographic order) mapped to dense ranks 0..d-1."""
    u = np.unique(meta)
    return np.searchsorted(u, meta).astype(np.int64)
