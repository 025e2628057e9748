"""The device's hash-list reduction (pn_internal.cuh: hash_mod, spatial_hash), restated with
Python integers and checked on the CPU: Julia's mod(h, list_size) of the wrapped Int64 hash,
computed as |h| - floor(|h| magic / 2^64) size with magic = floor((2^64 - 1) / size) and at
most two corrections, equals Python's h % list_size for every list size up to 2^31 - 2,
including h = typemin(Int64) and the sizes next to powers of two."""
import numpy as np

M64 = (1 << 64) - 1


def hash_mod(h, size):
    magic = M64 // size
    neg = h < 0
    ax = (-h) & M64 if neg else h
    r = ax - ((ax * magic) >> 64) * size
    corrections = 0
    while r >= size:  # the device applies at most two
        r -= size
        corrections += 1
    assert corrections <= 2
    return size - r if neg and r != 0 else r


def test_barrett_equals_mod():
    rng = np.random.default_rng(3)
    sizes = [1, 2, 3, 7, 1000, 2**31 - 2]
    for k in range(1, 31):
        sizes += [2**k - 1, 2**k, 2**k + 1]
    sizes += [int(s) for s in rng.integers(1, 2**31 - 1, 200)]
    hs = [0, 1, -1, 2**63 - 1, -2**63, -2**63 + 1]
    hs += [int(v) for v in rng.integers(-2**63, 2**63 - 1, 400, dtype=np.int64)]
    for size in sizes:
        for h in hs:
            assert hash_mod(h, size) == h % size, (h, size)
