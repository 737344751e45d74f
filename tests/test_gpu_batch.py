"""Batched PFP BWT on the GPU: many texts in one pipeline run, each result
bit-exact against the oracle for that text alone (and against the one-text
entry point)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mixed_texts(seed, count, max_n=3000):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        kind = i % 7
        n = int(rng.integers(0, max_n))
        if kind == 0:
            n = int(rng.integers(0, 9))            # empty and shorter than a window
        alpha = int(rng.choice([1, 2, 4, 14, 60, 253]))
        t = rng.integers(2, 2 + alpha, size=n).astype(np.uint8)
        if kind == 3 and n > 20:
            t = np.resize(t[: max(1, n // 8)], n)   # repeats
        if kind == 5 and out:
            t = out[int(rng.integers(0, len(out)))].copy()   # an identical text
        out.append(t)
    return out


@pytest.mark.parametrize("W,P,small", [(5, 16, False), (5, 23, False), (35, 81, True), (5, 16, True),
                                       (7, 19, False), (1, 2, False)])
def test_batch_matches_oracle_per_text(storage, orc, W, P, small):
    texts = _mixed_texts(W * 100 + P, 60)
    if small:
        texts = [(t % 14 + 2).astype(np.uint8) for t in texts]
    got = storage.pfp_bwt_batch(texts, W, P, small)
    assert len(got) == len(texts)
    for i, (t, L) in enumerate(zip(texts, got)):
        want, _ = orc.pfp_bwt(t, W, P, small) if len(t) else (np.zeros(0, np.uint8), None)
        assert np.array_equal(L, want), (i, len(t), W, P, small)


def test_batch_equals_single_text_runs(storage, wl):
    concat, offsets = wl.batch_texts(48, scale=1 / 8, seed=11)
    texts = [concat[offsets[i]:offsets[i + 1]] for i in range(len(offsets) - 1)]
    got = storage.pfp_bwt_batch(texts)
    for i, t in enumerate(texts):
        assert np.array_equal(got[i], storage.pfp_bwt(t)), i


def test_batch_one_text_equals_pfp_bwt(storage, wl):
    t = wl.dna_copies(base_len=32 * 1024, copies=12, seed=3)
    assert np.array_equal(storage.pfp_bwt_batch([t])[0], storage.pfp_bwt(t))


def test_batch_texts_with_shared_content(storage, orc, wl):
    # texts cut from one repetitive text: phrases and whole suffixes repeat across texts
    base = wl.dna_copies(base_len=4096, copies=16, seed=8)
    rng = np.random.default_rng(8)
    texts = []
    for _ in range(40):
        a = int(rng.integers(0, len(base) - 10))
        b = int(rng.integers(a + 1, min(len(base), a + 9000)))
        texts.append(base[a:b].copy())
    texts += [texts[3].copy(), texts[3].copy(), base[:5].copy(), base[:6].copy()]
    got = storage.pfp_bwt_batch(texts)
    for i, t in enumerate(texts):
        want, _ = orc.pfp_bwt(t, 5, 16, False)
        assert np.array_equal(got[i], want), i


def test_batch_all_empty_and_no_texts(storage):
    assert storage.pfp_bwt_batch([]) == []
    got = storage.pfp_bwt_batch([np.zeros(0, np.uint8)] * 3)
    assert [len(g) for g in got] == [0, 0, 0]


def test_batch_rejects_bad_bytes(storage, pkg):
    ok = np.full(100, 3, np.uint8)
    bad = ok.copy()
    bad[50] = 1
    with pytest.raises(pkg.GbwtError) as e:
        storage.pfp_bwt_batch([ok, bad, ok])
    assert e.value.code == pkg.BAD_PARAMETER
    big = ok.copy()
    big[7] = 40
    with pytest.raises(pkg.GbwtError) as e:
        storage.pfp_bwt_batch([ok, big], small_alphabet=True)
    assert e.value.code == pkg.UNSUPPORTED_INPUT
    # the storage stays usable
    assert len(storage.pfp_bwt_batch([ok, ok])[1]) == 100


def test_batch_device_pointers(storage, wl):
    torch = pytest.importorskip("torch")
    concat, offsets = wl.batch_texts(16, scale=1 / 16, seed=12)
    dT = torch.from_numpy(concat).cuda()
    dL = torch.empty_like(dT)
    torch.cuda.synchronize()
    storage.pfp_bwt_batch_device(dT.data_ptr(), offsets, dL.data_ptr())
    L = dL.cpu().numpy()
    for i in range(len(offsets) - 1):
        t = concat[offsets[i]:offsets[i + 1]]
        assert np.array_equal(L[offsets[i]:offsets[i + 1]], storage.pfp_bwt(t)), i


def test_batch_scaled_mix_round_trip(storage, orc, wl):
    # many texts of the batched workload's shape; every BWT inverts to its text
    concat, offsets = wl.batch_texts(256, scale=1 / 16, seed=13)
    out = np.empty_like(concat)
    storage.pfp_bwt_batch_into(concat, offsets, out)
    for i in range(0, len(offsets) - 1, 5):
        t = concat[offsets[i]:offsets[i + 1]]
        L = out[offsets[i]:offsets[i + 1]]
        assert np.array_equal(L, orc.sa_bwt(t)), i


def test_batch_one_text_per_segment(storage, orc, wl):
    # lengths that are whole radix tiles: no padding, so every text gets its own sort segment
    rng = np.random.default_rng(14)
    texts = [wl.dna_copies(base_len=512 * int(rng.integers(1, 5)), copies=8, seed=200 + i)[:4096 * int(rng.integers(1, 4))]
             for i in range(12)]
    got = storage.pfp_bwt_batch(texts)
    for i, t in enumerate(texts):
        assert np.array_equal(got[i], orc.sa_bwt(t)), i


@pytest.mark.parametrize("shift", [1, 2, 3])
def test_batch_device_pointers_unaligned(storage, wl, shift):
    """Texts at an odd device address: the padded copy takes its byte path
    for every unit and must give the same BWTs."""
    torch = pytest.importorskip("torch")
    concat, offsets = wl.batch_texts(12, scale=1 / 32, seed=13 + shift)
    buf = torch.zeros(len(concat) + 8, dtype=torch.uint8, device="cuda")
    buf[shift:shift + len(concat)] = torch.from_numpy(concat).cuda()
    dL = torch.empty(len(concat) + 8, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    storage.pfp_bwt_batch_device(buf.data_ptr() + shift, offsets, dL.data_ptr() + shift)
    L = dL.cpu().numpy()[shift:shift + len(concat)]
    want = storage.pfp_bwt_batch([concat[offsets[i]:offsets[i + 1]] for i in range(len(offsets) - 1)])
    assert np.array_equal(L, np.concatenate(want))
