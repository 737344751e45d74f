"""Autotuner logic without a GPU: the coordinate-descent search, size-class
selection, and the C library's validation of tuning knobs."""
import importlib

import pytest

PKG = "masterarbeit_parallele_konstruktion_der_burrows-wheeler-transformation_auf_der_gpu_gb300"


def test_coordinate_descent_finds_separable_minimum():
    at = importlib.import_module(PKG + ".autotune")
    cands = {"a": (1, 2, 3, 4), "b": (10, 20, 30)}
    calls = []

    def f(cfg):
        calls.append(cfg)
        return (cfg["a"] - 3) ** 2 + abs(cfg["b"] - 20) / 10

    best, t, runs = at.coordinate_descent(f, ("a", "b"), {"a": 1, "b": 10}, cands)
    assert best == {"a": 3, "b": 20} and t == 0
    assert runs == len({tuple(sorted(c.items())) for c in calls})      # each configuration timed once


def test_coordinate_descent_keeps_start_when_nothing_is_faster():
    at = importlib.import_module(PKG + ".autotune")
    best, t, runs = at.coordinate_descent(lambda c: 1.0, ("a",), {"a": 2}, {"a": (1, 2, 3)})
    assert best == {"a": 2} and t == 1.0 and runs == 3


def test_tuning_for_size_classes(pkg):
    table = {"classes": {"16": {"hash_log2_max": 20}, "128": {"hash_log2_max": 22}, "512": {"hash_log2_max": 24}}}
    MiB = 1 << 20
    assert pkg.tuning_for(1000, table) == {"hash_log2_max": 20}           # below the smallest class
    assert pkg.tuning_for(100 * MiB, table) == {"hash_log2_max": 20}
    assert pkg.tuning_for(128 * MiB, table) == {"hash_log2_max": 22}
    assert pkg.tuning_for(2000 * MiB, table) == {"hash_log2_max": 24}
    assert pkg.tuning_for(5, None) is None


def test_library_validates_knobs(pkg):
    assert pkg.check_tuning({})
    assert pkg.check_tuning({"hash_log2_max": 24, "batch_radix_bits": 9, "unbwt_rate_log2": 6})
    for bad in ({"hash_log2_max": 8}, {"batch_radix_bits": 10}, {"unbwt_rate_log2": 20}, {"batch_seg_tiles": -1},
                {"dict_key_bits": 4}, {"parse_key_phrases": 3}):
        assert not pkg.check_tuning(bad), bad
    with pytest.raises(ValueError):
        pkg.Tuning.from_dict({"no_such_knob": 1})


def test_committed_tuning_file_is_valid(pkg):
    table = pkg.load_tuning()
    if table is None:
        pytest.skip("no tuning.json next to the package")
    for knobs in table["classes"].values():
        assert pkg.check_tuning(knobs), knobs
