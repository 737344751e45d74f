"""Generates tests/golden/golden.json.

The reference ships no golden vectors (its only check is `cmp` against
libcubwt, compare_script.sh:7-10), so these fixtures are computed here from
the definitions alone, in plain Python, independent of the C oracle and of
the CUDA path:
  * D: trigger windows by the rule of Compute_D1/D2/D3
    (Prefix_Free_Parsing_W=5_P=16_kommentiert.cu:443-576);
  * bwt: a naive sort of all suffixes, output in the reference's convention
    (row byte = T[j-1], T[n-1] for j = 0);
  * primary_index: the row of the suffix starting at T[0].

Run:  python tests/golden/make_golden.py
"""
import json
import os
import random


def triggers(t, W, P):
    n = len(t)
    D = []
    for s in range(1, n - W + 1):
        h = 0
        for k in range(W):
            h = (h + t[s + W - 1 - k] * pow(2, k, P)) % P
        if h == 0 or t[s:s + W] == t[:W]:
            D.append(s + W - 1)
    D.append(n + W - 1)
    return D


def bwt(t):
    n = len(t)
    order = sorted(range(n), key=lambda j: t[j:])
    return [t[j - 1] if j else t[n - 1] for j in order], order.index(0)


def main():
    rnd = random.Random(20261203)
    dna = lambda n: [rnd.choice([2, 3, 4, 5]) for _ in range(n)]
    cases = [
        ("single", [2], 5, 16, False),
        ("two", [9, 3], 5, 16, False),
        ("shorter_than_W", [7, 7, 7], 5, 16, False),
        ("all_equal", [2] * 40, 5, 16, False),
        ("period2", [2, 3] * 30, 5, 16, False),
        ("banana_like", [3, 2, 15, 2, 15, 2], 5, 16, True),
        ("hash_zero_window", [5, 3, 2, 2, 2, 4, 9, 9, 9, 9], 5, 16, False),
        ("dna_w5p11", dna(120), 5, 11, False),
        ("dna_w5p13", dna(120), 5, 13, False),
        ("dna_w5p14", dna(120), 5, 14, False),
        ("dna_w5p14_small", dna(120), 5, 14, True),
        ("dna_w5p23", dna(150), 5, 23, False),
        ("dna_w5p23_small", dna(150), 5, 23, True),
        ("dna_w35p81_small", dna(300), 35, 81, True),
        ("ascii_w5p16", [rnd.randint(32, 127) for _ in range(200)], 5, 16, False),
        ("repeats_w5p16", (dna(30) * 5)[:140], 5, 16, False),
        ("all_values", list(range(2, 255)), 5, 23, False),
    ]
    out = []
    for name, t, W, P, small in cases:
        L, pidx = bwt(t)
        out.append({"name": name, "text": t, "W": W, "P": P, "small": small, "D": triggers(t, W, P),
                    "bwt": L, "primary_index": pidx})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(path, "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print(path, len(out))


if __name__ == "__main__":
    main()
