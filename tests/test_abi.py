"""The C ABI library without a GPU: it builds, loads, exports every entry
point declared in include/gbwt.h, and its host-only parts (the reference's
file formats, error strings) behave.  No compute call is made here."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(gbwt_[a-z_0-9]+)\s*\(", src, re.M))
    return names


def test_library_exports_every_declared_symbol(pkg):
    lib = ctypes.CDLL(pkg.LIB_PATH)
    names = declared_symbols()
    assert len(names) >= 11
    for name in names:
        assert hasattr(lib, name), name
    assert set(pkg.EXPORTS) <= names


def test_input_output_file_formats(pkg, tmp_path):
    t = np.array([2, 254, 17, 3, 3, 100], np.uint8)
    p = tmp_path / "input.txt"
    p.write_text(f"{len(t)}\n" + " ".join(str(v) for v in t) + "\n")
    got = pkg.scan_input(str(p))
    assert got.tolist() == t.tolist()
    q = tmp_path / "out.txt"
    pkg.print_output(str(q), t)
    # print_Output (K:4776-4790): "%d\n" then "%d " per byte
    assert q.read_text() == "6\n2 254 17 3 3 100 "


@pytest.mark.parametrize("body", ["3\n2 3 1\n", "2\n2 255\n", "3\n2 3\n", "x\n"])
def test_input_validation(pkg, tmp_path, body):
    p = tmp_path / "input.txt"
    p.write_text(body)
    with pytest.raises(pkg.GbwtError) as e:
        pkg.scan_input(str(p))
    assert e.value.code == pkg.BAD_PARAMETER


def test_error_strings(pkg):
    lib = pkg._lib()
    for code in (0, -1, -2, -5, -6, -7, -8, -9, -10):
        assert lib.gbwt_error_string(code)


def test_no_gpu_fails_loudly(pkg):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(pkg.GbwtError):
        pkg.Storage(16)


def test_variant_names(pkg):
    assert pkg.variant("Prefix_Free_Parsing_W=35_P=81_small_alphabet_Linux") == (35, 81, True)
    assert pkg.variant("./Prefix_Free_Parsing_W=5_P=13_Linux") == (5, 13, False)
    assert pkg.variant("Lyndon_Grammar_BWT_Linux") == (5, 16, False)     # same BWT, built by PFP
    assert len(pkg.VARIANTS) == 9


def test_cli_built(pkg):
    cli = os.path.join(os.path.dirname(pkg.LIB_PATH), "gbwt_pfp")
    assert os.access(cli, os.X_OK)


def test_batch_workload_shape(wl):
    lens = wl.batch_lengths(4096)
    assert lens.min() >= 4 * 1024 and lens.max() <= 16 * 1024 * 1024
    assert 400 * 2**20 < lens.sum() < 640 * 2**20          # about 512 MiB
    assert abs(np.median(lens) - 64 * 1024) < 8 * 1024
    c, o = wl.batch_texts(8, scale=1 / 64, seed=5)
    c2, o2 = wl.batch_texts(8, scale=1 / 64, seed=5)
    assert np.array_equal(c, c2) and np.array_equal(o, o2)
    assert o[0] == 0 and o[-1] == len(c) and c.min() >= 2 and c.max() <= 5


def test_batch_wrapper_validates_before_calling(pkg):
    st = object.__new__(pkg.Storage)      # no device storage: validation must fail first
    with pytest.raises(ValueError):
        pkg.Storage.pfp_bwt_batch_into(st, np.zeros(4, np.uint8), np.array([0, 8]), np.zeros(8, np.uint8))
