"""The pair cache's hit-mask recording of the Float32 3D density sweep (WithMask::group and
WithMask::flush in csrc/pn_traverse.cuh), restated with 64-bit unsigned words on the CPU.

The sweep takes a clipped row's run [b0, e0) in groups of GROUP = 4 candidates; each
group's 4 hit bits enter the top of a 128-bit shift register (hi, lo) and the row's flush
shifts the register down by sh = 128 - 4 ceil((e0 - b0) / 4).  The stored mask must equal
the positional one that record() builds candidate by candidate (bit t for slot b0 + t), for
every run length the cache holds (0 to 128 slots) and every hit pattern; a tail group's
slots past the run are never hits.
"""
import numpy as np

GROUP = 4
M64 = (1 << 64) - 1


def positional(hits):
    lo = hi = 0
    for t, h in enumerate(hits):
        if h:
            if t < 64:
                lo |= 1 << t
            else:
                hi |= 1 << (t - 64)
    return lo, hi


def shift_register(hits):
    n = len(hits)
    lo = hi = 0
    for e in range(0, n, GROUP):  # WithMask::group, once per group of the run
        g = 0
        for u in range(GROUP):
            if e + u < n and hits[e + u]:
                g |= 1 << u
        lo = ((lo >> GROUP) | (hi << (64 - GROUP))) & M64
        hi = ((hi >> GROUP) | (g << (64 - GROUP))) & M64
    sh = 128 - GROUP * ((max(n, 0) + GROUP - 1) // GROUP)  # row_begin
    if sh >= 64:  # flush
        lo = 0 if sh >= 128 else hi >> (sh - 64)
        hi = 0
    elif sh > 0:
        lo = ((lo >> sh) | (hi << (64 - sh))) & M64
        hi >>= sh
    return lo, hi


def test_every_run_length_and_pattern_density():
    rng = np.random.default_rng(7)
    for n in range(0, 129):
        for p in (0.0, 0.27, 0.5, 1.0):
            for _ in range(4):
                hits = list(rng.random(n) < p)
                assert shift_register(hits) == positional(hits), (n, p)


def test_single_bits_at_every_position():
    for n in range(1, 129):
        for t in (0, n // 2, n - 1):
            hits = [False] * n
            hits[t] = True
            assert shift_register(hits) == positional(hits), (n, t)
