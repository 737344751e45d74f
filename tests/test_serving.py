"""The serving loop's scheduler without a GPU (GBWT_SERVER_SIMULATE: a job
"runs" for n / 1 GB/s and copies its text): every job completes, small
jobs that wait together are batched, a large job and small batches
overlap, the memory budget serialises jobs that do not fit together, and
bad submissions are refused."""
import time

import numpy as np
import pytest

MiB = 1 << 20


def _est_single(n):        # the scheduler's estimate for a job run alone
    return 20 * n + 64 * MiB


def test_all_jobs_complete_with_their_results(pkg):
    rng = np.random.default_rng(1)
    with pkg.Server(workers=2, simulate=True) as srv:
        texts = [rng.integers(2, 6, size=int(rng.integers(0, 5000))).astype(np.uint8) for _ in range(200)]
        tickets = [srv.submit(t) for t in texts]
        srv.drain(timeout=30)
        for t, k in zip(texts, tickets):
            info = srv.poll(k)
            assert info["status"] == 0
            assert info["end_us"] >= info["start_us"] >= info["submit_us"]
            assert np.array_equal(srv.result(k), t)      # simulated "BWT" = copy


def test_small_jobs_are_batched_while_a_large_job_runs(pkg):
    big = np.full(64 * MiB, 3, np.uint8)
    small = [np.full(64 * 1024, 4, np.uint8) for _ in range(60)]
    with pkg.Server(workers=2, small_max=16 * MiB, simulate=True) as srv:
        kb = srv.submit(big)
        time.sleep(0.005)                                 # the large job is running
        ks = [srv.submit(t) for t in small]
        srv.drain(timeout=30)
        ib = srv.poll(kb)
        infos = [srv.poll(k) for k in ks]
    assert ib["batch_jobs"] == 1
    assert max(i["batch_jobs"] for i in infos) > 1        # continuous batching
    assert all(i["worker"] != ib["worker"] for i in infos)
    # the small jobs ran on the other worker while the large one was running
    assert max(i["end_us"] for i in infos) < ib["end_us"]


def test_budget_serialises_jobs_that_do_not_fit_together(pkg):
    n = 32 * MiB
    budget = _est_single(n) + _est_single(n) // 2          # one large job at a time
    texts = [np.full(n, 2 + i, np.uint8) for i in range(3)]
    with pkg.Server(hbm_budget=budget, workers=3, small_max=MiB, simulate=True) as srv:
        ks = [srv.submit(t) for t in texts]
        srv.drain(timeout=30)
        infos = sorted((srv.poll(k) for k in ks), key=lambda i: i["start_us"])
        peak = srv.peak_admitted()
    for a, b in zip(infos, infos[1:]):
        assert b["start_us"] >= a["end_us"]               # no overlap
    assert peak <= budget


def test_job_larger_than_budget_runs_alone(pkg):
    t = np.full(8 * MiB, 5, np.uint8)
    with pkg.Server(hbm_budget=MiB, workers=2, small_max=MiB, simulate=True) as srv:
        k = srv.submit(t)
        info = srv.wait(k, timeout=30)
    assert info["status"] == 0 and info["batch_jobs"] == 1


def test_small_jobs_pass_a_large_job_that_waits_for_memory(pkg):
    n = 32 * MiB
    budget = _est_single(n) + _est_single(1000) + MiB     # room for k1 and k3, not k2
    with pkg.Server(hbm_budget=budget, workers=2, small_max=MiB, simulate=True) as srv:
        k1 = srv.submit(np.full(n, 2, np.uint8))
        time.sleep(0.003)
        k2 = srv.submit(np.full(n, 3, np.uint8))           # must wait for k1's memory
        k3 = srv.submit(np.full(1000, 4, np.uint8))        # fits next to k1
        srv.drain(timeout=30)
        i1, i2, i3 = srv.poll(k1), srv.poll(k2), srv.poll(k3)
    assert i2["start_us"] >= i1["end_us"]
    assert i3["end_us"] < i2["start_us"]


def test_bad_submissions_are_refused(pkg):
    with pkg.Server(workers=1, simulate=True) as srv:
        for W, P in [(0, 16), (65, 16), (5, 0)]:
            with pytest.raises(pkg.GbwtError):
                srv.submit(np.full(10, 3, np.uint8), W=W, P=P)
        with pytest.raises(pkg.GbwtError):
            srv.poll(12345)
        with pytest.raises(pkg.GbwtError):
            srv.submit(np.full(10, 3, np.uint8), out=np.empty(5, np.uint8))


def test_percentiles():
    import importlib
    pkg = importlib.import_module("masterarbeit_parallele_konstruktion_der_burrows-wheeler-transformation_auf_der_gpu_gb300")
    p = pkg.percentiles(list(range(1, 101)))
    assert p == {"p50": 50.0, "p99": 99.0}
    assert pkg.percentiles([])["p50"] is None
