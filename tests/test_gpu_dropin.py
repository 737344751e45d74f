"""Drop-in surfaces on the GPU: the CLI run like the reference's programs
(input.txt -> out.txt, program from its name: the PFP variants,
Lyndon_Grammar_BWT and libcubwt), the raw-byte fast path, and the
libcubwt-compatible entry point."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cli(pkg):
    return os.path.join(os.path.dirname(pkg.LIB_PATH), "gbwt_pfp")


@pytest.mark.parametrize("variant", ["Prefix_Free_Parsing_W=5_P=16", "Prefix_Free_Parsing_W=35_P=81_small_alphabet",
                                     "Prefix_Free_Parsing_W=5_P=23", "Lyndon_Grammar_BWT"])
def test_cli_as_reference_program(pkg, orc, wl, tmp_path, variant):
    t = wl.dna_copies(base_len=8 * 1024, copies=6, seed=9)
    (tmp_path / "input.txt").write_text(f"{len(t)}\n" + " ".join(map(str, t.tolist())) + "\n")
    exe = tmp_path / f"{variant}_Linux"
    os.symlink(_cli(pkg), exe)
    r = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lines = (tmp_path / "out.txt").read_text().split("\n", 1)
    assert int(lines[0]) == len(t)
    got = np.array(list(map(int, lines[1].split())), dtype=np.uint8)
    assert np.array_equal(got, orc.sa_bwt(t))


def _write_input(path, t):
    path.write_text(f"{len(t)}\n" + " ".join(map(str, t.tolist())) + "\n")


def _libcubwt_harness_output(L, idx):
    # LC:2989-3020: raw layout for index 0, else L[0] moved to the index
    # (and dropped when the index is n)
    if idx == 0:
        return L
    return np.array([v for i in range(1, len(L)) for v in ((L[0], L[i]) if i == idx else (L[i],))], dtype=np.uint8)


@pytest.mark.parametrize("case", ["any_bytes", "dna", "index_n"])
def test_cli_as_libcubwt_program(pkg, orc, wl, tmp_path, case):
    rng = np.random.default_rng(7)
    if case == "any_bytes":
        # 0, 1 and 255 included; at most 253 distinct values (gbwt_libcubwt_bwt's contract)
        vals = np.array([v for v in range(256) if v not in (100, 101, 102)], dtype=np.uint8)
        t = vals[rng.integers(0, len(vals), size=5000)]
        t[:3] = (0, 1, 255)
    elif case == "dna":
        t = wl.dna_copies(base_len=8 * 1024, copies=6, seed=11)
    else:
        t = np.array([9, 3, 3, 4, 3, 3], dtype=np.uint8)    # the whole text sorts last: index n
    _write_input(tmp_path / "input.txt", t)
    exe = tmp_path / "libcubwt_Linux"
    os.symlink(_cli(pkg), exe)
    r = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    head, body = (tmp_path / "out.txt").read_text().split("\n", 1)
    assert int(head) == len(t)
    got = np.array(list(map(int, body.split())), dtype=np.uint8)
    L, idx = _libcubwt_expected(orc, t)
    if case == "index_n":
        assert idx == len(t)
    assert np.array_equal(got, _libcubwt_harness_output(L, idx))
    if case == "dna":
        assert np.array_equal(got, orc.sa_bwt(t))     # valid PFP input: the same bytes as the PFP programs


def test_cli_binary_fast_path(pkg, orc, wl, tmp_path):
    t = wl.dna_copies(base_len=16 * 1024, copies=8, seed=10)
    (tmp_path / "t.bin").write_bytes(t.tobytes())
    r = subprocess.run([_cli(pkg), "--W", "5", "--P", "16", "--binary-in", "t.bin", "--binary-out", "L.bin"],
                       cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = np.frombuffer((tmp_path / "L.bin").read_bytes(), dtype=np.uint8)
    assert np.array_equal(got, orc.sa_bwt(t))


def test_cli_rejects_invalid_input(pkg, tmp_path):
    (tmp_path / "input.txt").write_text("4\n3 4 255 5\n")
    r = subprocess.run([_cli(pkg)], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0


def _libcubwt_expected(orc, t):
    n = len(t)
    O = orc.sa_bwt(t)
    p = orc.primary_index(t)
    return np.concatenate([t[-1:], O[:p], O[p + 1:]]), p + 1


@pytest.mark.parametrize("alpha,lo", [(4, 0), (253, 0), (30, 200), (2, 254)])
def test_libcubwt_compatible(storage, orc, alpha, lo):
    rng = np.random.default_rng(alpha + lo)
    for n in (1, 2, 17, 1000, 50000):
        t = (rng.integers(0, alpha, size=n) + lo).astype(np.uint8)
        L, idx = storage.libcubwt_bwt(t)
        want, widx = _libcubwt_expected(orc, t)
        assert idx == widx and np.array_equal(L, want), (alpha, lo, n)


def test_libcubwt_too_many_symbols(storage, pkg):
    t = np.arange(256, dtype=np.uint8).repeat(3)
    with pytest.raises(pkg.GbwtError) as e:
        storage.libcubwt_bwt(t)
    assert e.value.code == pkg.UNSUPPORTED_INPUT


@pytest.mark.parametrize("r", [2, 4, 32])
def test_libcubwt_aux_indexes(storage, orc, wl, r):
    rng = np.random.default_rng(r)
    cases = [rng.integers(0, 256, size=5000).astype(np.uint8), np.array([7], np.uint8),
             rng.integers(10, 13, size=333).astype(np.uint8), wl.dna_copies(base_len=8192, copies=12, seed=r)]
    for t in cases:
        t = t.copy()
        if len(np.unique(t)) > 253:
            t[t > 252] = 252
        L, I = storage.libcubwt_bwt_aux(t, r)
        L0, idx = storage.libcubwt_bwt(t)
        assert np.array_equal(L, L0)
        sa = orc.suffix_array(t)
        isa = np.empty(len(t), np.int64)
        isa[sa] = np.arange(len(t))
        want = isa[::r] + 1
        assert np.array_equal(I.astype(np.int64), want), (len(t), r)
        assert I[0] == idx
