"""Parity against the reference's own programs, run on the same GPU.

The reference's correctness check is `cmp` of its PFP output against
libcubwt's (compare_script.sh:7-10).  Here both of them -- the reference's
PFP programs, compiled unmodified for sm_103a, and the libcubwt 1.6.3 copy it
ships -- run on the same synthetic texts as this library, and all three
outputs must be equal byte for byte:

* 8 MiB multi-copy DNA (256 KiB base, 32 copies, 0.1 % substitutions), all
  nine reference programs;
* 512 MiB multi-copy DNA with indels, W=5 P=16, its small-alphabet program
  and W=35 P=81 small-alphabet;
* 256 MiB versioned order-3 Markov text over 96 byte values, W=5 P=23.

Before any reference program runs, the oracle's trigger scan checks on the
host that the text holds no phrase the reference's device asserts reject
(oracle.reference.guard); a refused text is reported as a skip, never run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref():
    import oracle
    from oracle import reference
    oracle.build()
    reference.stage()
    res = reference.build()
    failed = {k: v for k, v in res.items() if v is not None}
    assert not failed, f"reference build failed: {failed}"
    if not reference.available() or not reference.available("W5_P16"):
        pytest.skip("reference sources are not staged in oracle/_ref/src (run `python -m oracle.reference` "
                    "where the reference checkout exists)")
    return reference


def _ref_pfp(ref, t, W, P, small):
    why = ref.guard(t, W, P, small)
    if why is not None:
        pytest.skip(f"reference W={W} P={P} small={small} not run: {why}")
    L, info = ref.run_pfp(t, W, P, small, checked=None)
    return L, info


@pytest.fixture(scope="module")
def cfg1(wl):
    return wl.config1_text()


@pytest.mark.parametrize("variant", ["W5_P16", "W5_P11", "W5_P13", "W5_P14", "W5_P23", "W5_P14_small",
                                     "W5_P16_small", "W5_P23_small", "W35_P81_small"])
def test_8mib_dna_equals_reference_pfp(pkg, ref, cfg1, variant):
    _, W, P, small = ref.PFP_VARIANTS[variant]
    want, info = _ref_pfp(ref, cfg1, W, P, small)
    with pkg.Storage(len(cfg1)) as st:
        got = st.pfp_bwt(cfg1, W, P, small)
        z = st.stats()["z"]
    assert info["z"] == z                       # same phrase count as the reference's size_D
    assert np.array_equal(got, want)


def test_8mib_dna_equals_libcubwt(pkg, ref, cfg1):
    want, info = ref.run_libcubwt(cfg1)
    with pkg.Storage(len(cfg1)) as st:
        got = st.pfp_bwt(cfg1, 5, 16)
        L2, pidx = st.libcubwt_bwt(cfg1)       # this library's libcubwt-compatible entry
    assert np.array_equal(got, want)
    assert pidx == info["primary_index"]        # libcubwt_bwt's return value
    # libcubwt's raw layout re-assembled as its harness does (libcubwt.cu:2989-3020)
    assert np.array_equal(np.concatenate([L2[1:pidx], L2[:1], L2[pidx:]]), want)


@pytest.mark.slow
def test_512mib_dna_equals_reference_and_libcubwt(pkg, ref, wl):
    t = wl.config2_text()
    with pkg.Storage(len(t)) as st:
        got = st.pfp_bwt(t, 5, 16)
        got_small = st.pfp_bwt(t, 5, 16, small_alphabet=True)
        got_81 = st.pfp_bwt(t, 35, 81, small_alphabet=True)
    assert np.array_equal(got, got_small)
    assert np.array_equal(got, got_81)
    want, _ = ref.run_libcubwt(t)
    assert np.array_equal(got, want)
    del want
    for (W, P, small) in ((5, 16, False), (5, 16, True), (35, 81, True)):
        want, _ = _ref_pfp(ref, t, W, P, small)
        assert np.array_equal(got, want), (W, P, small)


@pytest.mark.slow
def test_256mib_versioned_equals_reference_and_libcubwt(pkg, ref, orc, wl):
    t = wl.config3_text()
    with pkg.Storage(len(t)) as st:
        got = st.pfp_bwt(t, 5, 23)
        pidx = st.stats()["primary_index"]
    want, _ = ref.run_libcubwt(t)
    assert np.array_equal(got, want)
    del want
    assert np.array_equal(orc.unbwt(got, pidx), t)
    want, _ = _ref_pfp(ref, t, 5, 23, False)
    assert np.array_equal(got, want)
