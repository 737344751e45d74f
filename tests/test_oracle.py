"""The oracle (CPU) against the definition of the BWT and hand-checked cases.

The reference ships no golden vectors; its acceptance test is equality of
the PFP output with libcubwt's suffix-array BWT (compare_script.sh:7-10).
These tests pin the PFP restatement to that criterion: a naive sort of all
suffixes, an independent SA-IS BWT, and hand-derived trigger positions.
"""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

VARIANTS = [(5, 16, False), (5, 14, False), (5, 13, False), (5, 11, False), (5, 23, False),
            (35, 81, True), (5, 16, True), (5, 23, True), (5, 14, True)]


def naive_bwt(t):
    n = len(t)
    tl = t.tolist()
    order = sorted(range(n), key=lambda j: tl[j:])
    return np.array([tl[j - 1] if j else tl[n - 1] for j in order], dtype=np.uint8)


def naive_triggers(t, W, P):
    n = len(t)
    D = []
    for s in range(1, n - W + 1):
        h = 0
        for k in range(W):
            h = (h + int(t[s + W - 1 - k]) * (pow(2, k, P))) % P
        if h == 0 or list(t[s:s + W]) == list(t[:W]):
            D.append(s + W - 1)
    D.append(n + W - 1)
    return np.array(D, dtype=np.int64)


@pytest.mark.parametrize("W,P,small", VARIANTS)
def test_pfp_restatement_equals_naive_bwt(orc, W, P, small):
    rng = np.random.default_rng(W * 100 + P)
    for i in range(150):
        n = int(rng.integers(1, 160))
        alpha = int(rng.choice([1, 2, 4, 14] if small else [1, 2, 4, 30, 253]))
        t = rng.integers(2, 2 + alpha, size=n).astype(np.uint8)
        if i % 10 == 0:
            t[:] = t[0]
        L, _ = orc.pfp_bwt(t, W, P, small)
        assert np.array_equal(L, naive_bwt(t)), (W, P, small, t.tolist())


def test_sa_bwt_equals_naive(orc):
    rng = np.random.default_rng(3)
    for _ in range(300):
        n = int(rng.integers(1, 300))
        t = rng.integers(2, 2 + int(rng.choice([1, 2, 5, 250])), size=n).astype(np.uint8)
        assert np.array_equal(orc.sa_bwt(t), naive_bwt(t))


@pytest.mark.parametrize("W,P", [(5, 16), (5, 11), (5, 23), (35, 81), (3, 2), (1, 5)])
def test_trigger_scan_matches_definition(orc, W, P):
    rng = np.random.default_rng(P)
    for _ in range(60):
        n = int(rng.integers(1, 120))
        t = rng.integers(2, 2 + int(rng.choice([1, 3, 40])), size=n).astype(np.uint8)
        assert np.array_equal(orc.trigger_scan(t, W, P), naive_triggers(t, W, P))


def test_trigger_hand_checked(orc):
    # W=5, P=16: weights (2^k mod 16) = 1,2,4,8,0 -> the oldest byte has weight 0.
    # window "2 2 2 2 2": h = 2*(1+2+4+8) = 30 = 14 mod 16 -> no hash trigger, but
    # every window equal to T[0..4] triggers except the one at 0.
    t = np.array([2] * 8, np.uint8)
    assert orc.trigger_scan(t, 5, 16).tolist() == [5, 6, 7, 12]
    # h(T[s..s+4]) = 8*T[s+1] + 4*T[s+2] + 2*T[s+3] + T[s+4] mod 16
    t = np.array([5, 3, 2, 2, 2, 4, 9, 9, 9, 9], np.uint8)
    # window 1 (3,2,2,2,4): 16+8+4+4 = 32 -> 0 mod 16 -> trigger at end 5
    assert orc.trigger_scan(t, 5, 16).tolist()[0] == 5
    # no windows at all when n < W: only the forced final trigger n+W-1
    assert orc.trigger_scan(np.array([7, 7, 7], np.uint8), 5, 16).tolist() == [7]


def test_unbwt_round_trip(orc):
    rng = np.random.default_rng(8)
    for _ in range(200):
        n = int(rng.integers(1, 500))
        t = rng.integers(2, 2 + int(rng.choice([1, 2, 4, 100])), size=n).astype(np.uint8)
        L = orc.sa_bwt(t)
        assert np.array_equal(orc.unbwt(L, orc.primary_index(t)), t)


def test_validation_priority(orc):
    t = np.array([3, 20, 4], np.uint8)
    assert orc.validate(t, True) == -5          # outside the small-alphabet range
    assert orc.validate(t, False) == 0
    t = np.array([3, 20, 0], np.uint8)
    assert orc.validate(t, True) == -1          # a byte outside [2,254] wins
    assert orc.validate(np.array([255], np.uint8), False) == -1


def test_intermediates_consistent(orc, wl):
    t = wl.dna_copies(base_len=8192, copies=6, seed=2)
    L, st, meta, sa = orc.pfp_bwt(t, 5, 16, False, with_parse=True)
    assert st["z"] == len(orc.trigger_scan(t, 5, 16))
    # sum over S of block lengths is n (K:2571-2592)
    assert len(L) == len(t)
    assert sorted(sa.tolist()) == list(range(st["z"]))
    assert len(np.unique(meta)) == st["d"]
    # every variant gives the same BWT: it is a property of the text
    for W, P, small in VARIANTS:
        assert np.array_equal(orc.pfp_bwt(t, W, P, small)[0], L)


def test_golden_fixtures(orc):
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        cases = json.load(f)
    assert len(cases) >= 10
    for c in cases:
        t = np.array(c["text"], np.uint8)
        assert orc.trigger_scan(t, c["W"], c["P"]).tolist() == c["D"], c["name"]
        L, st = orc.pfp_bwt(t, c["W"], c["P"], c["small"])
        assert L.tolist() == c["bwt"], c["name"]
        assert orc.primary_index(t) == c["primary_index"], c["name"]
