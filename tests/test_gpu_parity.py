"""GPU parity: the CUDA path through the C ABI against the oracle.

Every comparison is bit-exact (integer/byte work).  The oracle's PFP
restatement is itself checked against the suffix-array BWT in
tests/test_oracle.py.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ALL_VARIANTS = [(5, 16, False), (5, 14, False), (5, 13, False), (5, 11, False), (5, 23, False),
                (35, 81, True), (5, 16, True), (5, 23, True), (5, 14, True)]


def _cases(seed, count, max_n=400):
    rng = np.random.default_rng(seed)
    for i in range(count):
        n = int(rng.integers(1, max_n))
        alpha = int(rng.choice([1, 2, 3, 4, 8, 14, 60, 253]))
        t = rng.integers(2, 2 + alpha, size=n).astype(np.uint8)
        if i % 9 == 0:
            t[:] = t[0]
        if i % 13 == 0 and n > 8:
            period = int(rng.integers(1, 6))
            t = np.resize(t[:period], n)
        yield t


@pytest.mark.parametrize("W,P,small", ALL_VARIANTS)
def test_random_small_all_variants(storage, orc, W, P, small):
    for t in _cases(seed=W * 1000 + P + (7 if small else 0), count=120):
        if small and t.max() > 15:
            t = (t % 14 + 2).astype(np.uint8)
        got = storage.pfp_bwt(t, W, P, small)
        want, _ = orc.pfp_bwt(t, W, P, small)
        assert np.array_equal(got, want), (len(t), W, P, small, t[:40].tolist())


@pytest.mark.parametrize("W,P", [(5, 16), (35, 81), (5, 23), (3, 7), (1, 2), (8, 5), (2, 1), (64, 97)])
def test_trigger_scan_matches_oracle(storage, orc, W, P):
    rng = np.random.default_rng(W * 31 + P)
    for n in [1, 2, W - 1, W, W + 1, 100, 4095, 4096, 4097, 4096 + W, 20000, 100003]:
        if n < 1:
            continue
        t = rng.integers(2, 6, size=n).astype(np.uint8)
        got = storage.trigger_scan(t, W, P)
        want = orc.trigger_scan(t, W, P)
        assert np.array_equal(got, want), (W, P, n)


def test_trigger_scan_unaligned_device_views(storage, orc):
    # host-pointer path copies into an aligned buffer; exercise odd lengths
    rng = np.random.default_rng(5)
    for n in range(4080, 4120):
        t = rng.integers(2, 10, size=n).astype(np.uint8)
        assert np.array_equal(storage.trigger_scan(t, 5, 16), orc.trigger_scan(t, 5, 16))


@pytest.mark.parametrize("W,P", [(5, 16), (35, 81), (5, 11)])
def test_parse_ranks_and_parse_sa(storage, orc, W, P):
    for t in _cases(seed=P, count=60, max_n=3000):
        ranks, psa = storage.parse(t, W, P)
        _, st, meta, sa = orc.pfp_bwt(t, W, P, False, with_parse=True)
        assert np.array_equal(ranks, orc.dense_ranks(meta)), (W, P, len(t))
        assert np.array_equal(psa, sa), (W, P, len(t))


def test_edge_cases(storage, orc):
    cases = [
        np.array([2], np.uint8), np.array([7, 3], np.uint8), np.array([254] * 3, np.uint8),
        np.full(10000, 9, np.uint8),                        # every window equals the first word
        np.resize(np.array([2, 3], np.uint8), 5001),         # period 2
        np.resize(np.array([2, 3, 4, 5, 6, 7, 8], np.uint8), 7777),
        np.arange(2, 255, dtype=np.uint8),                   # all byte values
    ]
    for t in cases:
        for W, P in [(5, 16), (35, 81), (5, 23)]:
            got = storage.pfp_bwt(t, W, P)
            assert np.array_equal(got, orc.sa_bwt(t)), (len(t), W, P)


def test_phrases_longer_than_reference_limit(storage, orc):
    # the reference asserts phrase length < 8192 (K:584-585); here they work
    rng = np.random.default_rng(11)
    t = np.concatenate([np.array([3], np.uint8), np.full(30000, 2, np.uint8),
                        rng.integers(2, 6, size=5000).astype(np.uint8), np.full(20000, 4, np.uint8)])
    for W, P in [(5, 16), (5, 23), (35, 81)]:
        got = storage.pfp_bwt(t, W, P)
        assert np.array_equal(got, orc.sa_bwt(t)), (W, P)
    assert storage.stats()["z"] >= 1


def test_invalid_bytes_are_errors(storage, pkg):
    for bad in (0, 1, 255):
        t = np.full(100, 3, np.uint8)
        t[57] = bad
        with pytest.raises(pkg.GbwtError) as e:
            storage.pfp_bwt(t, 5, 16)
        assert e.value.code == pkg.BAD_PARAMETER
    t = np.full(100, 3, np.uint8)
    t[10] = 16
    with pytest.raises(pkg.GbwtError) as e:
        storage.pfp_bwt(t, 5, 16, small_alphabet=True)
    assert e.value.code == pkg.UNSUPPORTED_INPUT
    # the storage stays usable after an error
    assert np.array_equal(storage.pfp_bwt(t, 5, 16), storage.pfp_bwt(t, 5, 16))


def test_bad_parameters(storage, pkg):
    t = np.full(10, 3, np.uint8)
    for W, P in [(0, 16), (65, 16), (5, 0), (5, 70000)]:
        with pytest.raises(pkg.GbwtError) as e:
            storage.pfp_bwt(t, W, P)
        assert e.value.code == pkg.BAD_PARAMETER


def test_empty_text(storage):
    assert len(storage.pfp_bwt(np.zeros(0, np.uint8), 5, 16)) == 0


def test_primary_index(storage, orc):
    for t in _cases(seed=99, count=80, max_n=2000):
        L = storage.pfp_bwt(t, 5, 16)
        p = storage.stats()["primary_index"]
        assert p == orc.primary_index(t)
        assert np.array_equal(orc.unbwt(L, p), t)


def test_mixed_text_medium(storage, orc, wl):
    t = wl.dna_copies(base_len=64 * 1024, copies=16, sub_rate=1e-3, seed=3, indel_rate=1e-4)
    ref = orc.sa_bwt(t)
    for W, P, small in [(5, 16, False), (5, 16, True), (35, 81, True), (5, 23, False)]:
        assert np.array_equal(storage.pfp_bwt(t, W, P, small), ref), (W, P, small)


def test_large_alphabet_versioned(storage, orc, wl):
    t = wl.versioned_markov(base_len=64 * 1024, versions=8, rate=1e-3, seed=3)
    want, _ = orc.pfp_bwt(t, 5, 23)
    assert np.array_equal(storage.pfp_bwt(t, 5, 23), want)


def test_config1_8mib_against_oracle(storage, orc, wl):
    t = wl.config1_text()
    got = storage.pfp_bwt(t, 5, 16)
    want, st = orc.pfp_bwt(t, 5, 16)
    assert np.array_equal(got, want)
    s = storage.stats()
    assert s["z"] == st["z"] and s["d"] == st["d"] and s["s"] == st["s"]
    assert s["mixed_blocks"] == st["mixed_blocks"] and s["mixed_elems"] == st["mixed_elems"]


def test_repeat_calls_deterministic(storage, wl):
    t = wl.dna_copies(base_len=32 * 1024, copies=8, seed=4)
    a = storage.pfp_bwt(t, 5, 16)
    b = storage.pfp_bwt(t, 5, 16)
    assert np.array_equal(a, b)


def test_device_pointer_path(pkg, orc, wl):
    torch = pytest.importorskip("torch")
    t = wl.dna_copies(base_len=32 * 1024, copies=8, seed=6)
    dt = torch.from_numpy(t).cuda()
    dout = torch.empty_like(dt)
    torch.cuda.synchronize()
    with pkg.Storage(len(t)) as st:
        st.pfp_bwt_device(dt.data_ptr(), dout.data_ptr(), len(t), 5, 16)
        torch.cuda.synchronize()
        assert np.array_equal(dout.cpu().numpy(), orc.sa_bwt(t))


def test_pinned_host_buffers(storage, orc, wl):
    # pinned host buffers (asynchronous copies) give the same bytes as
    # pageable ones, also for texts without mixed blocks
    torch = pytest.importorskip("torch")
    cases = list(_cases(seed=77, count=40, max_n=3000))
    cases.append(wl.dna_copies(base_len=64 * 1024, copies=16, seed=21))
    cases.append(np.full(5000, 7, dtype=np.uint8))
    for t in cases:
        ht = torch.from_numpy(t.copy()).pin_memory()
        ho = torch.full((len(t),), 1, dtype=torch.uint8).pin_memory()
        storage.pfp_bwt_into(ht.numpy(), ho.numpy(), 5, 16)
        want, _ = orc.pfp_bwt(t, 5, 16)
        assert np.array_equal(ho.numpy(), want), (len(t), t[:20].tolist())
        assert np.array_equal(storage.pfp_bwt(t, 5, 16), want)


def test_stage_times_add_up(storage, wl):
    # every stage gets its own time and the parts add up to the total
    t = wl.dna_copies(base_len=128 * 1024, copies=32, seed=22)
    storage.pfp_bwt(t, 5, 16, stage_times=True)
    ms = storage.stats()["stage_ms"]
    parts = [ms[k] for k in ("scan", "phrases", "dictionary", "parse_sa", "s_groups", "runs", "mixed")]
    assert all(v > 0 for v in parts), ms
    assert abs(sum(parts) - ms["total"]) <= 0.02 * ms["total"] + 0.01, ms
