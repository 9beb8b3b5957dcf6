"""Host-side parts of the serving engine that need no GPU: the range allocator
the server carves request regions from, and request validation."""
import numpy as np
import pytest

import dgtd_gb300 as dg


def test_arena_first_fit_and_merge():
    a = dg.Arena(1 << 20, 256)
    offs = [a.alloc(1000) for _ in range(4)]
    assert offs == [0, 1024, 2048, 3072]            # rounded up to the 256-byte alignment
    assert a.usage()["in_use"] == 4096
    a.release(offs[1])
    a.release(offs[2])                                 # neighbours merge into one 2 KiB hole
    u = a.usage()
    assert u["in_use"] == 2048 and u["n_free_ranges"] == 2
    assert a.alloc(2048) == 1024                       # first fit reuses the merged hole
    a.release(offs[0]); a.release(1024); a.release(offs[3])
    u = a.usage()
    assert u["in_use"] == 0 and u["n_free_ranges"] == 1 and u["largest_free"] == 1 << 20


def test_arena_exhaustion_and_bad_release():
    a = dg.Arena(4096, 256)
    assert a.alloc(4096) == 0
    assert a.alloc(1) == -1
    with pytest.raises(dg.DgtdError):
        a.release(17)
    a.release(0)
    assert a.alloc(0) == -1
    assert a.alloc(5000) == -1


def test_arena_random_churn_keeps_invariants():
    rng = np.random.default_rng(3)
    cap = 1 << 16
    a = dg.Arena(cap, 64)
    live = {}
    for _ in range(2000):
        if live and rng.random() < 0.45:
            off = list(live)[rng.integers(len(live))]
            a.release(off)
            del live[off]
        else:
            n = int(rng.integers(1, 3000))
            off = a.alloc(n)
            if off >= 0:
                size = (n + 63) // 64 * 64
                assert off % 64 == 0 and off + size <= cap
                for o, s in live.items():               # no overlap with any live range
                    assert off + size <= o or o + s <= off
                live[off] = size
        assert a.usage()["in_use"] == sum(live.values())
    for off in list(live):
        a.release(off)
    assert a.usage()["largest_free"] == cap


def test_arena_rejects_bad_alignment():
    with pytest.raises(dg.DgtdError):
        dg.Arena(1024, 3)
