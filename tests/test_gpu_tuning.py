"""Tuning knobs change scheduling, never results: the same inputs under
different gbwt_tuning values give identical BWTs and inverses."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIGS = [None, {"hash_log2_max": 16}, {"hash_log2_max": 24, "batch_radix_bits": 8},
           {"batch_seg_tiles": 1, "batch_pad_eighths": 64, "batch_radix_bits": 9},
           {"batch_seg_tiles": 64, "batch_pad_eighths": 0}, {"unbwt_rate_log2": 2}, {"unbwt_rate_log2": 12},
           {"dict_key_bits": 8, "parse_key_phrases": 1}, {"dict_key_bits": 33}]


def test_batch_and_single_results_do_not_depend_on_tuning(pkg, wl):
    concat, offsets = wl.batch_texts(64, scale=1 / 8, seed=31)
    texts = [concat[offsets[i]:offsets[i + 1]] for i in range(len(offsets) - 1)]
    single = wl.dna_copies(base_len=64 * 1024, copies=20, seed=32)
    ref_batch = ref_single = None
    with pkg.Storage(len(concat), tuning=None) as st:
        for cfg in CONFIGS:
            st.set_tuning(cfg)
            got = np.concatenate(st.pfp_bwt_batch(texts))
            L = st.pfp_bwt(single)
            p = st.stats()["primary_index"]
            assert np.array_equal(st.unbwt(L, p), single), cfg
            if ref_batch is None:
                ref_batch, ref_single = got, L
            assert np.array_equal(got, ref_batch), cfg
            assert np.array_equal(L, ref_single), cfg
