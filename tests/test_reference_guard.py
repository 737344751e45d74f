"""The host-side guard in front of the reference's own CUDA programs (CPU only).

The reference's PFP programs assert W < phrase length < 8192 on the GPU
(K:584-585); a failed device assert would take down the GPU context, so
oracle.reference.guard must refuse every such text before anything runs.
These tests need no GPU and launch nothing.
"""
import numpy as np
import pytest

from oracle import reference


def test_guard_accepts_8mib_dna(orc, wl):
    t = wl.config1_text()
    for name, (_, W, P, small) in reference.PFP_VARIANTS.items():
        assert reference.guard(t, W, P, small) is None, name


def test_guard_refuses_long_phrase(orc):
    # first window 2,2,2,2,2; then only 3s: hash 3*(1+2+4+8) = 45 = 13 (mod 16), never the first
    # window -> no trigger at all, one phrase of n+W bytes
    t = np.full(reference.MIN_TEXT + 100, 3, dtype=np.uint8)
    t[:5] = 2
    why = reference.guard(t, 5, 16, False)
    assert why is not None and "8192" in why
    assert len(orc.trigger_scan(t, 5, 16)) == 1          # only the forced final trigger


def test_guard_refuses_bytes_and_sizes(orc, wl):
    t = wl.config1_text()[: reference.MIN_TEXT].copy()
    assert reference.guard(t, 5, 16, False) is None
    for bad in (0, 1, 255):
        u = t.copy()
        u[1000] = bad
        assert "range" in reference.guard(u, 5, 16, False)
    u = t.copy()
    u[7] = 40
    assert reference.guard(u, 5, 16, False) is None
    assert "small-alphabet" in reference.guard(u, 5, 16, True)
    assert "minimum" in reference.guard(t[:1000], 5, 16, False)


def test_run_refuses_without_launch(orc, monkeypatch):
    # a refused text never reaches the binary, even when one exists
    monkeypatch.setattr(reference, "available", lambda variant=None: True)
    t = np.full(reference.MIN_TEXT + 100, 3, dtype=np.uint8)
    t[:5] = 2
    with pytest.raises(reference.ReferenceRefused):
        reference.run_pfp(t, 5, 16, False)


def test_variant_table_matches_makefile():
    # the nine PFP programs of Makefile:13-23, one per (W, P, small) pair
    assert len(reference.PFP_VARIANTS) == 9
    for name, (src, W, P, small) in reference.PFP_VARIANTS.items():
        assert name == reference.variant_name(W, P, small)
        assert src == f"Prefix_Free_Parsing_W={W}_P={P}" + ("_small_alphabet" if small else "") + ".cu"
