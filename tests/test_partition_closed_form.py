"""The GPU builder replaces the reference's sequential in-place partition
(src/math/bvh.ts:126-140) with a closed-form permutation computed from prefix
counts. This CPU test checks the closed form against the sequential loop on
random flag patterns (the same rule the CUDA kernel implements in
partition_dest, lucent_gb300/csrc/bvh_build.cu)."""
import numpy as np


def sequential(flags):
    a = list(range(len(flags)))
    i, j = 0, len(a) - 1
    while i <= j:
        if flags[a[i]]:
            i += 1
        else:
            a[i], a[j] = a[j], a[i]
            j -= 1
    return a, i


def closed_form(flags):
    n = len(flags)
    L = int(sum(flags))
    P = [r for r in range(L) if not flags[r]]  # front right-goers, ascending
    Qasc = [r for r in range(L, n) if flags[r]]  # back left-goers, ascending
    m = len(P)
    assert m == len(Qasc)
    out = [None] * n
    fr = bl = 0
    for r in range(n):
        left = flags[r]
        if r < L:
            if left:
                d = r
            else:
                d = n - 1 if fr == 0 else Qasc[m - fr] - 1
                fr += 1
        elif left:
            d = P[m - 1 - bl]
            bl += 1
        elif bl > 0:
            d = r - 1
        elif r == L:
            d = Qasc[0] - 1 if m > 0 else n - 1
        else:
            d = r - 1
        out[d] = r
    return out, L


def test_closed_form_matches_sequential_partition():
    rng = np.random.default_rng(1)
    for _ in range(20000):
        n = int(rng.integers(2, 48))
        flags = list(rng.random(n) < rng.random())
        if not any(flags):
            continue
        assert closed_form(flags) == sequential(flags)
