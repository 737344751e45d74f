"""Inverse BWT on the GPU (gbwt_unbwt, gbwt_libcubwt_unbwt): round trips
against the forward transform on random, degenerate and repetitive texts;
the oracle's inverse is the independent check of the forward side."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _texts(seed):
    rng = np.random.default_rng(seed)
    yield np.array([7], np.uint8)
    yield np.array([3, 3], np.uint8)
    yield np.full(5000, 9, np.uint8)
    yield np.resize(np.array([2, 3, 4], np.uint8), 10007)
    for _ in range(40):
        n = int(rng.integers(1, 30000))
        alpha = int(rng.choice([1, 2, 4, 20, 253]))
        yield rng.integers(2, 2 + alpha, size=n).astype(np.uint8)


def test_round_trip_pfp_convention(storage, orc):
    for t in _texts(1):
        L = storage.pfp_bwt(t)
        p = storage.stats()["primary_index"]
        assert p == orc.primary_index(t)
        assert np.array_equal(storage.unbwt(L, p), t), len(t)


def test_round_trip_libcubwt_convention(storage):
    rng = np.random.default_rng(2)
    for n in [1, 2, 3, 100, 4095, 4096, 4097, 65536 + 13]:
        for lo, alpha in [(0, 256), (0, 2), (250, 6), (0, 1)]:
            t = (rng.integers(0, alpha, size=n) + lo).astype(np.uint8)
            if len(np.unique(t)) > 253:
                t[t > 252] = 252
            L, idx = storage.libcubwt_bwt(t)
            assert np.array_equal(storage.libcubwt_unbwt(L, idx), t), (n, lo, alpha)


def test_round_trip_repetitive_dna(storage, wl):
    t = wl.dna_copies(base_len=128 * 1024, copies=40, seed=5, indel_rate=1e-4)
    L = storage.pfp_bwt(t)
    p = storage.stats()["primary_index"]
    assert np.array_equal(storage.unbwt(L, p), t)


def test_device_pointers(storage, wl):
    torch = pytest.importorskip("torch")
    t = wl.dna_copies(base_len=64 * 1024, copies=16, seed=6)
    L = storage.pfp_bwt(t)
    p = storage.stats()["primary_index"]
    dL = torch.from_numpy(L).cuda()
    dT = torch.empty_like(dL)
    torch.cuda.synchronize()
    storage.unbwt_device(dL.data_ptr(), dT.data_ptr(), len(t), p)
    assert np.array_equal(dT.cpu().numpy(), t)


def test_bad_primary_index(storage, pkg):
    t = np.array([2, 3, 4, 2, 3], np.uint8)
    L = storage.pfp_bwt(t)
    for p in (-1, len(t)):
        with pytest.raises(pkg.GbwtError) as e:
            storage.unbwt(L, p)
        assert e.value.code == pkg.BAD_PARAMETER
    assert len(storage.unbwt(np.zeros(0, np.uint8), 0)) == 0
