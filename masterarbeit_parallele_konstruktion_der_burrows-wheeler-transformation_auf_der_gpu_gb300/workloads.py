"""Seeded synthetic texts with the shapes of the PFP BWT benchmark workloads.

The thesis measured the Pizza&Chili repetitive corpus, which is not
available here; these generators stand in for it with the same kind of
content (multi-copy mutated DNA; versioned large-alphabet text).  DNA is
coded A,C,G,T -> 2,3,4,5 so one buffer is valid for the plain and the
small-alphabet variants (bytes in [2,15]).  No explicit sentinel byte is
written: the PFP sentinel is implicit (W copies of byte 1).

  dna_copies(...)       8 MiB: 256 KiB base (seed 1), 32 copies, 0.1 % substitutions
  dna_copies_indels(...) 512 MiB: 4 MiB base (seed 2), 128 copies, 0.1 % subs + 0.01 % indels
  versioned_markov(...) 256 MiB: 2 MiB order-3 Markov base over bytes 32..127
                        (rows Dirichlet(0.1), seed 3), 128 versions with
                        1..64-byte block replacements at rate 1e-4 per byte
"""
from __future__ import annotations

import numpy as np

MiB = 1 << 20
DNA = np.array([2, 3, 4, 5], dtype=np.uint8)


def _substitute(rng: np.random.Generator, seq: np.ndarray, rate: float) -> np.ndarray:
    out = seq.copy()
    hit = np.flatnonzero(rng.random(len(seq)) < rate)
    if len(hit):
        shift = rng.integers(1, 4, size=len(hit)).astype(np.uint8)      # new base != old
        out[hit] = (((out[hit] - 2) + shift) % 4 + 2).astype(np.uint8)
    return out


def _indels(rng: np.random.Generator, seq: np.ndarray, rate: float) -> np.ndarray:
    k = rng.binomial(len(seq), rate)
    if k == 0:
        return seq
    pos = np.sort(rng.integers(0, len(seq), size=k))
    kind = rng.integers(0, 2, size=k)            # 0 = insertion, 1 = deletion
    lens = rng.integers(1, 11, size=k)
    parts = []
    cur = 0
    for p, t, ln in zip(pos.tolist(), kind.tolist(), lens.tolist()):
        if p < cur:
            continue
        parts.append(seq[cur:p])
        if t == 0:
            parts.append(DNA[rng.integers(0, 4, size=ln)])
            cur = p
        else:
            cur = min(len(seq), p + ln)
    parts.append(seq[cur:])
    return np.concatenate(parts)


def dna_copies(base_len: int = 256 * 1024, copies: int = 32, sub_rate: float = 1e-3, seed: int = 1,
               indel_rate: float = 0.0) -> np.ndarray:
    """`copies` mutated copies of a uniform ACGT base, concatenated."""
    rng = np.random.default_rng(seed)
    base = DNA[rng.integers(0, 4, size=base_len)]
    out = []
    for _ in range(copies):
        c = _substitute(rng, base, sub_rate)
        if indel_rate:
            c = _indels(rng, c, indel_rate)
        out.append(c)
    return np.concatenate(out)


def config1_text(scale: float = 1.0) -> np.ndarray:
    """8 MiB: 256 KiB base, 32 copies, 0.1 % substitutions (seed 1)."""
    return dna_copies(int(256 * 1024 * scale), 32, 1e-3, seed=1)


def config2_text(scale: float = 1.0) -> np.ndarray:
    """512 MiB: 4 MiB base, 128 copies, 0.1 % substitutions + 0.01 % indels (seed 2)."""
    return dna_copies(int(4 * MiB * scale), 128, 1e-3, seed=2, indel_rate=1e-4)


def _markov(rng: np.random.Generator, length: int, rows: dict, ctx: tuple, alphabet: int = 96) -> tuple:
    out = np.empty(length, dtype=np.uint8)
    a, b, c = ctx
    u = rng.random(length)
    for i in range(length):
        key = (a << 14) | (b << 7) | c
        cdf = rows.get(key)
        if cdf is None:
            cdf = np.cumsum(rng.dirichlet(np.full(alphabet, 0.1)))
            rows[key] = cdf
        s = int(np.searchsorted(cdf, u[i], side="right"))
        if s >= alphabet:
            s = alphabet - 1
        out[i] = 32 + s
        a, b, c = b, c, s
    return out, (a, b, c)


def versioned_markov(base_len: int = 2 * MiB, versions: int = 128, rate: float = 1e-4, seed: int = 3) -> np.ndarray:
    """Order-3 Markov base over bytes 32..127 and successive edited versions."""
    rng = np.random.default_rng(seed)
    rows: dict = {}
    base, ctx = _markov(rng, base_len, rows, (0, 0, 0))
    out = [base]
    cur = base
    for _ in range(versions - 1):
        cur = cur.copy()
        k = rng.binomial(len(cur), rate)
        for p, ln in zip(rng.integers(0, len(cur), size=k).tolist(), rng.integers(1, 65, size=k).tolist()):
            ln = min(ln, len(cur) - p)
            fresh, ctx = _markov(rng, ln, rows, ctx)
            cur[p:p + ln] = fresh
        out.append(cur)
    return np.concatenate(out)


def config3_text(scale: float = 1.0) -> np.ndarray:
    """256 MiB: 2 MiB Markov base, 128 versions (seed 3)."""
    return versioned_markov(int(2 * MiB * scale), 128, 1e-4, seed=3)


def random_text(n: int, alphabet: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return rng.integers(2, 2 + alphabet, size=n).astype(np.uint8)


def batch_lengths(count: int = 4096, median: float = 64 * 1024, sigma: float = 1.2, lo: int = 4 * 1024,
                  hi: int = 16 * MiB, seed: int = 4) -> np.ndarray:
    """Log-normal text lengths (median, sigma), clipped to [lo, hi]."""
    rng = np.random.default_rng(seed)
    return np.clip(np.rint(rng.lognormal(np.log(median), sigma, size=count)), lo, hi).astype(np.int64)


def batch_texts(count: int = 4096, scale: float = 1.0, seed: int = 4, sub_rate: float = 1e-3):
    """Batched workload: `count` independent texts with log-normal lengths
    (median 64 KiB * scale, sigma 1.2, clipped to [4 KiB, 16 MiB] * scale),
    each 8..64 mutated copies of its own uniform ACGT base.  Returns
    (concatenated bytes, int64 offsets[count + 1])."""
    lens = batch_lengths(count, 64 * 1024 * scale, 1.2, max(1, int(4 * 1024 * scale)), max(1, int(16 * MiB * scale)),
                         seed)
    rng = np.random.default_rng(seed + 1)
    parts = []
    for ln in lens.tolist():
        copies = int(rng.integers(8, 65))
        base = DNA[rng.integers(0, 4, size=max(1, ln // copies))]
        t = np.tile(base, copies)[:ln]
        if len(t) < ln:
            t = np.concatenate([t, DNA[rng.integers(0, 4, size=ln - len(t))]])
        parts.append(_substitute(rng, t, sub_rate))
    offsets = np.zeros(count + 1, dtype=np.int64)
    np.cumsum(lens, out=offsets[1:])
    return np.concatenate(parts), offsets


def config4_texts(scale: float = 1.0):
    """4096 texts, about 512 MiB in total (seed 4)."""
    return batch_texts(4096, scale, seed=4)


def serving_jobs(count: int = 800, rate: float = 1000.0, seed: int = 5, large_frac: float = 0.01,
                 large_lo: int = 64 * MiB, large_hi: int = 256 * MiB):
    """Serving workload: `count` jobs with Poisson arrivals (`rate` per
    second).  A fraction `large_frac` are large repetitive-DNA texts of
    large_lo..large_hi bytes, cut from one text built like the 512 MiB
    workload (4 MiB base, mutated copies with substitutions and indels);
    the others have the batched workload's log-normal lengths, each text
    8..64 mutated copies of its own base.  Returns (texts, arrival times in
    seconds from the first arrival)."""
    rng = np.random.default_rng(seed)
    is_large = rng.random(count) < large_frac
    if count and not is_large.any():
        is_large[count // 2] = True
    lens = batch_lengths(count, seed=seed + 1)
    big = None
    if is_large.any():
        big_len = int(large_hi)
        copies = max(1, big_len // (4 * MiB) + 1)
        big = dna_copies(4 * MiB, copies, 1e-3, seed=seed + 2, indel_rate=1e-4)[:big_len]
    texts = []
    for i in range(count):
        if is_large[i]:
            ln = int(rng.integers(large_lo, large_hi + 1))
            texts.append(big[:ln])
        else:
            ln = int(lens[i])
            copies = int(rng.integers(8, 65))
            base = DNA[rng.integers(0, 4, size=max(1, ln // copies))]
            t = np.tile(base, copies + 1)[:ln]
            texts.append(_substitute(rng, t, 1e-3))
    gaps = rng.exponential(1.0 / rate, size=count)
    gaps[0] = 0.0
    return texts, np.cumsum(gaps)
