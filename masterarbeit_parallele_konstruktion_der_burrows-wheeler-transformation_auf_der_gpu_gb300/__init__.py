"""GB300-native prefix-free-parsing (PFP) BWT construction.

Python host interface over the C ABI of ``libgbwt.so`` (include/gbwt.h).  It
mirrors the reference programs' surface: a text of bytes in [2,254], the
trigger parameters W and P (plus the small-alphabet variants), and the BWT
byte array in the reference's convention (Prefix_Free_Parsing_W=5_P=16
_kommentiert.cu, "K": Scan_input K:111-150, Compute_D K:2415-2506,
Compute_S K:4330-4771, print_Output K:4776-4790).

There is no CPU fallback: without the built CUDA library every compute call
raises ``GbwtLibraryMissing``.
"""
from __future__ import annotations

import ctypes
import json
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgbwt.so")

# Error codes (include/gbwt.h).
NO_ERROR = 0
BAD_PARAMETER = -1
NOT_ENOUGH_MEMORY = -2
UNSUPPORTED_INPUT = -5
TIMEOUT = -6
GPU_ERROR = -7
GPU_NOT_SUPPORTED = -8
GPU_NOT_ENOUGH_MEMORY = -9
INTERNAL_ERROR = -10

FLAG_SMALL_ALPHABET = 1
FLAG_DEVICE_POINTERS = 2
FLAG_STAGE_TIMES = 4
SERVER_SIMULATE = 0x100
JOB_PENDING = 1
JOB_RUNNING = 2

# The reference's binaries (Makefile:11-23) and their (W, P, small) variants.
VARIANTS = {
    "Prefix_Free_Parsing_W=5_P=16": (5, 16, False),
    "Prefix_Free_Parsing_W=5_P=14": (5, 14, False),
    "Prefix_Free_Parsing_W=5_P=13": (5, 13, False),
    "Prefix_Free_Parsing_W=5_P=11": (5, 11, False),
    "Prefix_Free_Parsing_W=5_P=23": (5, 23, False),
    "Prefix_Free_Parsing_W=35_P=81_small_alphabet": (35, 81, True),
    "Prefix_Free_Parsing_W=5_P=16_small_alphabet": (5, 16, True),
    "Prefix_Free_Parsing_W=5_P=23_small_alphabet": (5, 23, True),
    "Prefix_Free_Parsing_W=5_P=14_small_alphabet": (5, 14, True),
}

STAGES = ("scan", "phrases", "dictionary", "parse_sa", "s_groups", "runs", "mixed", "total")


class GbwtError(RuntimeError):
    """A negative return code of the C ABI."""

    def __init__(self, code: int, where: str = ""):
        self.code = int(code)
        msg = _lib().gbwt_error_string(self.code).decode() if _LIB is not None else str(code)
        super().__init__(f"{where}: {msg} ({self.code})" if where else f"{msg} ({self.code})")


class GbwtLibraryMissing(ImportError):
    pass


class Stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in (
        "n", "z", "d", "dict_bytes", "s", "s_elems", "mixed_blocks", "mixed_elems",
        "dict_rounds", "parse_rounds", "hash_retries", "kernel_launches", "primary_index",
        "probe_launches", "probe_bytes")] + [("probe_ms", ctypes.c_double), ("stage_ms", ctypes.c_float * 8),
                                             ("device_bytes", ctypes.c_int64)]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "stage_ms"}
        d["stage_ms"] = {name: float(self.stage_ms[i]) for i, name in enumerate(STAGES)}
        return d


_LIB = None

# Every exported entry point of include/gbwt.h.
EXPORTS = (
    "gbwt_allocate_device_storage", "gbwt_free_device_storage", "gbwt_set_stream", "gbwt_pfp_bwt",
    "gbwt_pfp_trigger_scan", "gbwt_pfp_parse", "gbwt_get_stats", "gbwt_read_input_txt",
    "gbwt_write_out_txt", "gbwt_free_host", "gbwt_error_string", "gbwt_set_kernel_probe",
    "gbwt_libcubwt_bwt", "gbwt_pfp_trigger_scan_noalloc", "gbwt_pfp_bwt_batch", "gbwt_trim_device_storage",
    "gbwt_server_create", "gbwt_server_destroy", "gbwt_submit", "gbwt_poll", "gbwt_wait", "gbwt_server_drain",
    "gbwt_server_peak_admitted", "gbwt_unbwt", "gbwt_libcubwt_unbwt", "gbwt_set_tuning", "gbwt_check_tuning",
    "gbwt_libcubwt_bwt_aux",
)

TUNING_KNOBS = ("hash_log2_max", "batch_seg_tiles", "batch_pad_eighths", "batch_radix_bits", "unbwt_rate_log2",
                "dict_key_bits", "parse_key_phrases", "mixed_radix_bits", "batch_ballot")


class Tuning(ctypes.Structure):
    """gbwt_tuning (include/gbwt.h): scheduling knobs, 0 = default."""
    _fields_ = [(k, ctypes.c_int32) for k in TUNING_KNOBS] + [("reserved", ctypes.c_int32 * 3)]

    @classmethod
    def from_dict(cls, d: dict | None) -> "Tuning":
        t = cls()
        for k, v in (d or {}).items():
            if k not in TUNING_KNOBS:
                raise ValueError(f"unknown tuning knob {k}")
            setattr(t, k, int(v))
        return t


def check_tuning(d: dict) -> bool:
    """True when the C library accepts these knob values (no GPU needed)."""
    t = Tuning.from_dict(d)
    return _lib().gbwt_check_tuning(ctypes.byref(t)) == 0


TUNING_FILE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning.json")


def load_tuning(path: str | None = None) -> dict | None:
    """Size classes written by the autotuner ({"classes": {"<MiB>": {knob: value}}}), or None."""
    p = path or os.environ.get("GBWT_TUNING", TUNING_FILE)
    if not p or not os.path.exists(p):
        return None
    with open(p) as f:
        return json.load(f)


_MERGED: dict = {}


def tuning_for(n: int, table: dict | None, W: int | None = None) -> dict | None:
    """The knobs of the largest size class not above n bytes (the smallest class for smaller n),
    with the table's per-window-length overrides for W laid over them ({"windows": {"35": {...}}})."""
    if not table or not table.get("classes"):
        return None
    classes = sorted((int(k), v) for k, v in table["classes"].items())
    best = classes[0][1]
    for mib, knobs in classes:
        if (mib << 20) <= n:
            best = knobs
    over = (table.get("windows") or {}).get(str(W)) if W is not None else None
    if not over:
        return best
    key = (id(best), id(over))
    if key not in _MERGED:
        _MERGED[key] = {**best, **over}
    return _MERGED[key]


class JobInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int64), ("n", ctypes.c_int64), ("est_bytes", ctypes.c_int64),
                ("submit_us", ctypes.c_double), ("start_us", ctypes.c_double), ("end_us", ctypes.c_double),
                ("batch_jobs", ctypes.c_int32), ("worker", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}

PROBE_NONE = -1
PROBE_RADIX_SCATTER = 1
PROBE_TRIGGER_SCAN = 2
PROBE_PHRASE_HASH = 3
PROBE_RUN_FILL = 4
PROBE_MIXED_SCATTER = 5
PROBE_SEG_SORT = 6


def _lib() -> ctypes.CDLL:
    """Loads libgbwt.so (built by build.py); raises if it is missing."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise GbwtLibraryMissing(
            f"{LIB_PATH} is not built; run __graft_entry__.build() (no CPU fallback exists)")
    L = ctypes.CDLL(LIB_PATH)
    vp, u8p, i64, i32, u32 = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_uint32
    L.gbwt_allocate_device_storage.argtypes = [ctypes.POINTER(vp), i64]
    L.gbwt_allocate_device_storage.restype = i64
    L.gbwt_free_device_storage.argtypes = [vp]
    L.gbwt_free_device_storage.restype = i64
    L.gbwt_set_stream.argtypes = [vp, vp]
    L.gbwt_set_stream.restype = i64
    L.gbwt_pfp_bwt.argtypes = [vp, u8p, u8p, i64, i32, i32, u32]
    L.gbwt_pfp_bwt.restype = i64
    L.gbwt_pfp_trigger_scan.argtypes = [vp, u8p, i64, i32, i32, u32, ctypes.c_void_p, i64]
    L.gbwt_pfp_trigger_scan.restype = i64
    L.gbwt_pfp_parse.argtypes = [vp, u8p, i64, i32, i32, u32, ctypes.c_void_p, ctypes.c_void_p, i64]
    L.gbwt_pfp_parse.restype = i64
    L.gbwt_get_stats.argtypes = [vp, ctypes.POINTER(Stats)]
    L.gbwt_get_stats.restype = i64
    L.gbwt_read_input_txt.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(i64)]
    L.gbwt_read_input_txt.restype = i64
    L.gbwt_write_out_txt.argtypes = [ctypes.c_char_p, u8p, i64]
    L.gbwt_write_out_txt.restype = i64
    L.gbwt_free_host.argtypes = [vp]
    L.gbwt_free_host.restype = None
    L.gbwt_error_string.argtypes = [i64]
    L.gbwt_error_string.restype = ctypes.c_char_p
    L.gbwt_set_kernel_probe.argtypes = [vp, i32]
    L.gbwt_set_kernel_probe.restype = i64
    L.gbwt_libcubwt_bwt.argtypes = [vp, u8p, u8p, i64]
    L.gbwt_libcubwt_bwt.restype = i64
    L.gbwt_pfp_bwt_batch.argtypes = [vp, u8p, ctypes.c_void_p, i32, u8p, i32, i32, u32]
    L.gbwt_pfp_bwt_batch.restype = i64
    L.gbwt_libcubwt_bwt_aux.argtypes = [vp, u8p, u8p, i64, i64, ctypes.c_void_p]
    L.gbwt_libcubwt_bwt_aux.restype = i64
    L.gbwt_set_tuning.argtypes = [vp, ctypes.c_void_p]
    L.gbwt_set_tuning.restype = i64
    L.gbwt_check_tuning.argtypes = [ctypes.c_void_p]
    L.gbwt_check_tuning.restype = i64
    L.gbwt_unbwt.argtypes = [vp, u8p, u8p, i64, i64, u32]
    L.gbwt_unbwt.restype = i64
    L.gbwt_libcubwt_unbwt.argtypes = [vp, u8p, u8p, i64, ctypes.c_void_p, i32]
    L.gbwt_libcubwt_unbwt.restype = i64
    L.gbwt_trim_device_storage.argtypes = [vp]
    L.gbwt_trim_device_storage.restype = i64
    L.gbwt_server_create.argtypes = [ctypes.POINTER(vp), i64, i32, i64, u32]
    L.gbwt_server_create.restype = i64
    L.gbwt_server_destroy.argtypes = [vp]
    L.gbwt_server_destroy.restype = i64
    L.gbwt_submit.argtypes = [vp, u8p, u8p, i64, i32, i32, u32, ctypes.POINTER(i64)]
    L.gbwt_submit.restype = i64
    L.gbwt_poll.argtypes = [vp, i64, ctypes.POINTER(JobInfo)]
    L.gbwt_poll.restype = i64
    L.gbwt_wait.argtypes = [vp, i64, ctypes.c_double, ctypes.POINTER(JobInfo)]
    L.gbwt_wait.restype = i64
    L.gbwt_server_drain.argtypes = [vp, ctypes.c_double]
    L.gbwt_server_drain.restype = i64
    L.gbwt_server_peak_admitted.argtypes = [vp]
    L.gbwt_server_peak_admitted.restype = i64
    _LIB = L
    return L


def _check(rc: int, where: str) -> int:
    if rc < 0:
        raise GbwtError(rc, where)
    return rc


def _host_u8(a) -> np.ndarray:
    if isinstance(a, (bytes, bytearray, memoryview)):
        a = np.frombuffer(bytes(a), dtype=np.uint8)
    return np.ascontiguousarray(a, dtype=np.uint8)


class Storage:
    """Device storage (stream + scratch pools), libcubwt_allocate_device_storage
    style (libcubwt.cuh:48-59).  Use one per thread; reuse across calls."""

    def __init__(self, max_length: int = 0, tuning="auto"):
        """tuning: "auto" applies the autotuner's size classes (tuning.json, if
        present) to every call; a dict of knobs fixes them; None = defaults."""
        self._p = ctypes.c_void_p()
        _check(_lib().gbwt_allocate_device_storage(ctypes.byref(self._p), int(max_length)),
               "gbwt_allocate_device_storage")
        self._table = load_tuning() if tuning == "auto" else None
        self._applied = None
        if isinstance(tuning, dict):
            self._set_raw(tuning)

    def _set_raw(self, knobs: dict | None) -> None:
        t = Tuning.from_dict(knobs) if knobs else None
        _check(_lib().gbwt_set_tuning(self.handle, ctypes.byref(t) if t is not None else None), "gbwt_set_tuning")

    def set_tuning(self, knobs: dict | None) -> None:
        """Fixes the tuning knobs (None = defaults); size classes no longer apply."""
        self._table = None
        self._set_raw(knobs)

    def _auto(self, n: int, W: int | None = None) -> None:
        if self._table is None:
            return
        knobs = tuning_for(int(n), self._table, W)
        if knobs is not self._applied:
            self._set_raw(knobs)
            self._applied = knobs

    @property
    def handle(self) -> ctypes.c_void_p:
        if not self._p:
            raise ValueError("storage is closed")
        return self._p

    def close(self) -> None:
        if self._p:
            _lib().gbwt_free_device_storage(self._p)
            self._p = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None) -> None:
        _check(_lib().gbwt_set_stream(self.handle, ctypes.c_void_p(stream_handle or 0)), "gbwt_set_stream")

    def stats(self) -> dict:
        s = Stats()
        _check(_lib().gbwt_get_stats(self.handle, ctypes.byref(s)), "gbwt_get_stats")
        return s.as_dict()

    # -- compute ---------------------------------------------------------
    def pfp_bwt(self, text, W: int = 5, P: int = 16, small_alphabet: bool = False,
                stage_times: bool = False) -> np.ndarray:
        t = _host_u8(text)
        out = np.empty(max(len(t), 1), dtype=np.uint8)
        flags = (FLAG_SMALL_ALPHABET if small_alphabet else 0) | (FLAG_STAGE_TIMES if stage_times else 0)
        self._auto(len(t), W)
        _check(_lib().gbwt_pfp_bwt(self.handle, t.ctypes.data, out.ctypes.data, len(t), W, P, flags),
               "gbwt_pfp_bwt")
        return out[:len(t)]

    def pfp_bwt_into(self, text: np.ndarray, out: np.ndarray, W: int = 5, P: int = 16,
                     small_alphabet: bool = False) -> int:
        """Host buffers owned by the caller (e.g. pinned): text -> out."""
        if text.dtype != np.uint8 or out.dtype != np.uint8 or not text.flags.c_contiguous \
                or not out.flags.c_contiguous or len(out) < len(text):
            raise ValueError("text/out must be contiguous uint8 arrays, len(out) >= len(text)")
        flags = FLAG_SMALL_ALPHABET if small_alphabet else 0
        self._auto(len(text), W)
        return _check(_lib().gbwt_pfp_bwt(self.handle, text.ctypes.data, out.ctypes.data, len(text), W, P, flags),
                      "gbwt_pfp_bwt")

    def pfp_bwt_batch(self, texts, W: int = 5, P: int = 16, small_alphabet: bool = False,
                      stage_times: bool = False) -> list[np.ndarray]:
        """BWTs of many texts in one pipeline run; each equals pfp_bwt(text)."""
        parts = [_host_u8(t) for t in texts]
        offsets = np.zeros(len(parts) + 1, dtype=np.int64)
        np.cumsum([len(t) for t in parts], out=offsets[1:])
        concat = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint8)
        out = np.empty(max(len(concat), 1), dtype=np.uint8)
        self.pfp_bwt_batch_into(concat, offsets, out, W, P, small_alphabet, stage_times)
        return [out[offsets[i]:offsets[i + 1]] for i in range(len(parts))]

    def pfp_bwt_batch_into(self, concat: np.ndarray, offsets: np.ndarray, out: np.ndarray, W: int = 5,
                           P: int = 16, small_alphabet: bool = False, stage_times: bool = False) -> int:
        """Concatenated texts with int64 offsets[k+1] (host arrays) -> out at the same offsets."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        if concat.dtype != np.uint8 or out.dtype != np.uint8 or not concat.flags.c_contiguous \
                or not out.flags.c_contiguous or len(offsets) < 1 or len(out) < offsets[-1] \
                or len(concat) < offsets[-1]:
            raise ValueError("concat/out must be contiguous uint8 arrays covering offsets[-1] bytes")
        flags = (FLAG_SMALL_ALPHABET if small_alphabet else 0) | (FLAG_STAGE_TIMES if stage_times else 0)
        self._auto(int(offsets[-1]))
        return _check(_lib().gbwt_pfp_bwt_batch(self.handle, concat.ctypes.data, offsets.ctypes.data,
                                                len(offsets) - 1, out.ctypes.data, W, P, flags),
                      "gbwt_pfp_bwt_batch")

    def pfp_bwt_batch_device(self, text_ptr: int, offsets: np.ndarray, out_ptr: int, W: int = 5, P: int = 16,
                             small_alphabet: bool = False, stage_times: bool = False) -> int:
        """Device-pointer batch: text_ptr/out_ptr are CUDA addresses, offsets a host int64 array."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        flags = FLAG_DEVICE_POINTERS | (FLAG_SMALL_ALPHABET if small_alphabet else 0) | (
            FLAG_STAGE_TIMES if stage_times else 0)
        self._auto(int(offsets[-1]))
        return _check(_lib().gbwt_pfp_bwt_batch(self.handle, ctypes.c_void_p(text_ptr), offsets.ctypes.data,
                                                len(offsets) - 1, ctypes.c_void_p(out_ptr), W, P, flags),
                      "gbwt_pfp_bwt_batch")

    def libcubwt_bwt(self, text) -> tuple[np.ndarray, int]:
        """libcubwt_bwt semantics (any byte values, <= 253 distinct): returns
        (L, primary index) with L[0] = T[n-1] and the '$' entry removed."""
        t = _host_u8(text)
        out = np.empty(max(len(t), 1), dtype=np.uint8)
        idx = _check(_lib().gbwt_libcubwt_bwt(self.handle, t.ctypes.data, out.ctypes.data, len(t)),
                     "gbwt_libcubwt_bwt")
        return out[:len(t)], idx

    def unbwt(self, L, primary: int) -> np.ndarray:
        """Inverse BWT on the GPU of gbwt_pfp_bwt's output and its primary index."""
        b = _host_u8(L)
        T = np.empty(max(len(b), 1), dtype=np.uint8)
        self._auto(len(b))
        _check(_lib().gbwt_unbwt(self.handle, b.ctypes.data, T.ctypes.data, len(b), int(primary), 0), "gbwt_unbwt")
        return T[:len(b)]

    def unbwt_device(self, L_ptr: int, T_ptr: int, n: int, primary: int) -> int:
        self._auto(n)
        return _check(_lib().gbwt_unbwt(self.handle, ctypes.c_void_p(L_ptr), ctypes.c_void_p(T_ptr), n, int(primary),
                                        FLAG_DEVICE_POINTERS), "gbwt_unbwt")

    def libcubwt_unbwt(self, L, primary: int) -> np.ndarray:
        """libcubwt_unbwt semantics: libcubwt's BWT and primary index -> text."""
        b = _host_u8(L)
        U = np.empty(max(len(b), 1), dtype=np.uint8)
        _check(_lib().gbwt_libcubwt_unbwt(self.handle, b.ctypes.data, U.ctypes.data, len(b), None, int(primary)),
               "gbwt_libcubwt_unbwt")
        return U[:len(b)]

    def libcubwt_bwt_aux(self, text, r: int) -> tuple[np.ndarray, np.ndarray]:
        """libcubwt_bwt_aux semantics: (L, I) with I[k] = libcubwt row of the suffix at k*r."""
        t = _host_u8(text)
        out = np.empty(max(len(t), 1), dtype=np.uint8)
        I = np.empty(max((len(t) - 1) // max(int(r), 1) + 1, 1), dtype=np.uint32)
        self._auto(len(t))
        _check(_lib().gbwt_libcubwt_bwt_aux(self.handle, t.ctypes.data, out.ctypes.data, len(t), int(r),
                                            I.ctypes.data), "gbwt_libcubwt_bwt_aux")
        return out[:len(t)], I

    def set_kernel_probe(self, kernel: int) -> None:
        """Time every launch of one kernel family (PROBE_*) from now on."""
        _check(_lib().gbwt_set_kernel_probe(self.handle, int(kernel)), "gbwt_set_kernel_probe")

    def pfp_bwt_device(self, text_ptr: int, out_ptr: int, n: int, W: int = 5, P: int = 16,
                       small_alphabet: bool = False, stage_times: bool = False) -> int:
        """Device-pointer variant: ``text_ptr``/``out_ptr`` are CUDA device addresses."""
        flags = FLAG_DEVICE_POINTERS | (FLAG_SMALL_ALPHABET if small_alphabet else 0) | (
            FLAG_STAGE_TIMES if stage_times else 0)
        self._auto(n, W)
        return _check(_lib().gbwt_pfp_bwt(self.handle, ctypes.c_void_p(text_ptr), ctypes.c_void_p(out_ptr), n, W, P,
                                          flags), "gbwt_pfp_bwt")

    def trigger_scan(self, text, W: int = 5, P: int = 16, small_alphabet: bool = False) -> np.ndarray:
        t = _host_u8(text)
        if len(t) == 0:
            return np.zeros(0, dtype=np.int64)
        D = np.empty(len(t) + 2, dtype=np.int64)
        z = _check(_lib().gbwt_pfp_trigger_scan(self.handle, t.ctypes.data, len(t), W, P,
                                                FLAG_SMALL_ALPHABET if small_alphabet else 0, D.ctypes.data, len(D)),
                   "gbwt_pfp_trigger_scan")
        return D[:z].copy()

    def parse(self, text, W: int = 5, P: int = 16, small_alphabet: bool = False):
        """(dense lexicographic phrase rank per occurrence, suffix array of the parse)."""
        t = _host_u8(text)
        if len(t) == 0:
            return np.zeros(0, dtype=np.int32), np.zeros(0, dtype=np.int32)
        cap = len(t) + 2
        ranks = np.empty(cap, dtype=np.int32)
        psa = np.empty(cap, dtype=np.int32)
        z = _check(_lib().gbwt_pfp_parse(self.handle, t.ctypes.data, len(t), W, P,
                                         FLAG_SMALL_ALPHABET if small_alphabet else 0, ranks.ctypes.data,
                                         psa.ctypes.data, cap), "gbwt_pfp_parse")
        return ranks[:z].copy(), psa[:z].copy()


class Server:
    """Serving loop (gbwt_server_* in include/gbwt.h): jobs are admitted
    under a device-memory budget, small ones run together as batched
    pipeline calls, several workers overlap on the device.  ``simulate``
    runs the same scheduler without a GPU (a job copies its text)."""

    def __init__(self, hbm_budget: int = 0, workers: int = 2, small_max: int = 0, simulate: bool = False):
        self._h = ctypes.c_void_p()
        _check(_lib().gbwt_server_create(ctypes.byref(self._h), int(hbm_budget), int(workers), int(small_max),
                                         SERVER_SIMULATE if simulate else 0), "gbwt_server_create")
        self._bufs = {}

    def submit(self, text, W: int = 5, P: int = 16, small_alphabet: bool = False, out=None) -> int:
        t = np.ascontiguousarray(text, dtype=np.uint8)
        L = np.empty(max(len(t), 1), dtype=np.uint8) if out is None else out
        if L.dtype != np.uint8 or not L.flags.c_contiguous or len(L) < len(t):
            raise GbwtError(BAD_PARAMETER, "submit: out must be a contiguous uint8 array of len(text) bytes")
        ticket = ctypes.c_int64()
        _check(_lib().gbwt_submit(self._h, t.ctypes.data, L.ctypes.data, len(t), W, P,
                                  FLAG_SMALL_ALPHABET if small_alphabet else 0, ctypes.byref(ticket)), "gbwt_submit")
        self._bufs[ticket.value] = (t, L)            # alive until the job is done
        return ticket.value

    def poll(self, ticket: int) -> dict:
        if ticket not in self._bufs:
            raise GbwtError(BAD_PARAMETER, "poll: unknown ticket")
        info = JobInfo()
        _lib().gbwt_poll(self._h, ticket, ctypes.byref(info))
        return info.as_dict()

    def wait(self, ticket: int, timeout: float | None = None) -> dict:
        info = JobInfo()
        _lib().gbwt_wait(self._h, ticket, -1.0 if timeout is None else float(timeout), ctypes.byref(info))
        return info.as_dict()

    def result(self, ticket: int) -> np.ndarray:
        """The job's BWT (waits for it); raises GbwtError if the job failed."""
        info = self.wait(ticket)
        _check(info["status"], "server job")
        t, L = self._bufs[ticket]
        return L[:len(t)]

    def release(self, ticket: int) -> None:
        """Drops the wrapper's references to a finished job's buffers."""
        self._bufs.pop(ticket, None)

    def drain(self, timeout: float | None = None) -> None:
        _check(_lib().gbwt_server_drain(self._h, -1.0 if timeout is None else float(timeout)), "gbwt_server_drain")

    def peak_admitted(self) -> int:
        return _lib().gbwt_server_peak_admitted(self._h)

    def close(self) -> None:
        if self._h:
            _lib().gbwt_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def percentiles(values, qs=(50, 99)) -> dict:
    """Nearest-rank percentiles of a list of latencies."""
    v = np.sort(np.asarray(values, dtype=np.float64))
    if len(v) == 0:
        return {f"p{q}": None for q in qs}
    return {f"p{q}": float(v[min(len(v) - 1, int(np.ceil(q / 100 * len(v))) - 1)]) for q in qs}


_DEFAULT: Storage | None = None


def default_storage() -> Storage:
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = Storage(0)
    return _DEFAULT


def pfp_bwt(text, W: int = 5, P: int = 16, small_alphabet: bool = False) -> np.ndarray:
    """BWT of ``text`` (bytes in [2,254]) in the reference's output convention."""
    return default_storage().pfp_bwt(text, W, P, small_alphabet)


# The reference's Lyndon-grammar program writes the same BWT (its output is
# compared with libcubwt's, compare_script_lyndon.sh); here the PFP pipeline
# builds it with these parameters.
LYNDON_PROGRAM = "Lyndon_Grammar_BWT"
LYNDON_VARIANT = (5, 16, False)


def variant(name: str) -> tuple[int, int, bool]:
    """(W, P, small_alphabet) of a reference binary name (with or without _Linux)."""
    base = os.path.basename(name)
    if base.endswith("_Linux"):
        base = base[: -len("_Linux")]
    if base.endswith(".cu"):
        base = base[:-3]
    if base == LYNDON_PROGRAM:
        return LYNDON_VARIANT
    return VARIANTS[base]


# -- reference file formats --------------------------------------------------
def scan_input(path: str) -> np.ndarray:
    """Reads the reference's input.txt (K:111-150)."""
    L = _lib()
    p = ctypes.c_void_p()
    n = ctypes.c_int64()
    rc = L.gbwt_read_input_txt(path.encode(), ctypes.byref(p), ctypes.byref(n))
    _check(rc, "gbwt_read_input_txt")
    try:
        return np.ctypeslib.as_array((ctypes.c_uint8 * max(n.value, 1)).from_address(p.value))[: n.value].copy() \
            if n.value else np.zeros(0, dtype=np.uint8)
    finally:
        L.gbwt_free_host(p)


def print_output(path: str, L_bytes) -> None:
    """Writes the reference's out.txt (K:4776-4790)."""
    a = _host_u8(L_bytes)
    _check(_lib().gbwt_write_out_txt(path.encode(), a.ctypes.data, len(a)), "gbwt_write_out_txt")


@dataclass
class Variant:
    W: int
    P: int
    small_alphabet: bool = False
