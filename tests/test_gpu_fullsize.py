"""Full-size checks on the benchmark workloads, through size-independent
properties (the oracle would need minutes at these sizes):

* the BWT is a property of the text, so every (W, P, small) variant of the
  reference must produce the same bytes;
* the output is a permutation of the text;
* inverting the BWT with the primary index gives the text back exactly.
"""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def dna512(wl):
    return wl.config2_text()


def test_512mib_dna_variants_agree_and_invert(pkg, orc, dna512):
    t = dna512
    with pkg.Storage(len(t)) as st:
        a = st.pfp_bwt(t, 5, 16)
        pidx = st.stats()["primary_index"]
        b = st.pfp_bwt(t, 5, 16, small_alphabet=True)
        c = st.pfp_bwt(t, 35, 81, small_alphabet=True)
        assert st.stats()["primary_index"] == pidx
    assert np.array_equal(a, b)
    assert np.array_equal(a, c)
    assert np.array_equal(np.bincount(a, minlength=256), np.bincount(t, minlength=256))
    assert np.array_equal(orc.unbwt(a, pidx), t)
    with pkg.Storage(len(t)) as st:
        assert np.array_equal(st.unbwt(a, pidx), t)          # the GPU inverse, same round trip


def test_versioned_markov_inverts(pkg, orc, wl):
    t = wl.versioned_markov(base_len=256 * 1024, versions=128, rate=1e-4, seed=3)   # 32 MiB
    with pkg.Storage(len(t)) as st:
        a = st.pfp_bwt(t, 5, 23)
        pidx = st.stats()["primary_index"]
        b = st.pfp_bwt(t, 5, 16)
    assert np.array_equal(a, b)
    assert np.array_equal(orc.unbwt(a, pidx), t)


def test_random_text_many_distinct_phrases(pkg, orc, wl):
    # non-repetitive input: d close to z, large dictionary, full-size hash table
    t = wl.random_text(16 << 20, 4, seed=12)
    with pkg.Storage(len(t)) as st:
        a = st.pfp_bwt(t, 5, 16)
        s = st.stats()
    assert s["d"] > s["z"] // 2
    assert np.array_equal(a, orc.sa_bwt(t))
