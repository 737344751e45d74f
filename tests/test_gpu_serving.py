"""Serving loop on the GPU: jobs of mixed sizes arriving over time are
admitted, batched and overlapped, and every result equals the one-text
entry point's result for that job alone (bit-exact)."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
MiB = 1 << 20


def _mix(wl, seed):
    concat, offsets = wl.batch_texts(96, scale=1 / 16, seed=seed)
    texts = [concat[offsets[i]:offsets[i + 1]].copy() for i in range(len(offsets) - 1)]
    big = wl.dna_copies(base_len=256 * 1024, copies=80, seed=seed)        # 20 MiB: runs alone
    texts.insert(10, big)
    texts.insert(50, wl.dna_copies(base_len=512 * 1024, copies=40, seed=seed + 1))
    return texts


def test_results_identical_alone_and_in_the_mix(pkg, storage, wl):
    texts = _mix(wl, 21)
    rng = np.random.default_rng(21)
    with pkg.Server(workers=2, small_max=16 * MiB) as srv:
        tickets = []
        for t in texts:
            tickets.append(srv.submit(t))
            time.sleep(float(rng.exponential(0.0005)))         # Poisson arrivals
        srv.drain(timeout=300)
        infos = [srv.poll(k) for k in tickets]
        results = [srv.result(k).copy() for k in tickets]
    assert all(i["status"] == 0 for i in infos)
    assert max(i["batch_jobs"] for i in infos) > 1              # small jobs were batched
    assert {i["batch_jobs"] for i in infos if i["n"] > 16 * MiB} == {1}
    for t, L in zip(texts, results):
        assert np.array_equal(L, storage.pfp_bwt(t))


def test_invalid_job_fails_alone(pkg, storage, wl):
    texts = _mix(wl, 22)[:30]
    bad = texts[5].copy()
    bad[len(bad) // 2] = 1                                     # byte outside [2, 254]
    texts[5] = bad
    with pkg.Server(workers=1, small_max=16 * MiB) as srv:
        tickets = [srv.submit(t) for t in texts]
        srv.drain(timeout=300)
        infos = [srv.poll(k) for k in tickets]
        results = [srv.result(k).copy() if i["status"] == 0 else None for k, i in zip(tickets, infos)]
    assert infos[5]["status"] == pkg.BAD_PARAMETER
    for i, (t, L) in enumerate(zip(texts, results)):
        if i != 5:
            assert infos[i]["status"] == 0
            assert np.array_equal(L, storage.pfp_bwt(t))


def test_small_alphabet_and_other_variants_in_one_server(pkg, storage, wl, orc):
    rng = np.random.default_rng(23)
    jobs = []
    for i in range(40):
        t = wl.dna_copies(base_len=int(rng.integers(200, 4000)), copies=int(rng.integers(2, 20)), seed=100 + i)
        W, P, small = [(5, 16, False), (35, 81, True), (5, 23, False)][i % 3]
        jobs.append((t, W, P, small))
    with pkg.Server(workers=2) as srv:
        tickets = [srv.submit(t, W=W, P=P, small_alphabet=s) for t, W, P, s in jobs]
        srv.drain(timeout=300)
        for (t, W, P, s), k in zip(jobs, tickets):
            assert np.array_equal(srv.result(k), orc.sa_bwt(t))
