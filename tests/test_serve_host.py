"""Host logic of the serving loop (no GPU): the pool allocator that admits
requests by device memory."""
import numpy as np

from thejoker_gb300.serve import PoolAllocator


def test_first_fit_and_merge():
    p = PoolAllocator(1 << 16, align=1024)
    a = p.alloc(1000)
    b = p.alloc(5000)
    c = p.alloc(1024)
    assert a == (0, 1024) and b == (1024, 5120) and c == (6144, 1024)
    p.release(*b)
    assert p.alloc(70000) is None
    d = p.alloc(2048)                      # first fit: inside b's hole
    assert d == (1024, 2048)
    p.release(*a)
    p.release(*c)
    p.release(*d)
    assert p.free == [(0, 1 << 16)]
    assert p.available == p.size


def test_random_alloc_release_never_overlaps():
    rng = np.random.default_rng(0)
    p = PoolAllocator(1 << 20, align=4096)
    live = []
    for _ in range(2000):
        if live and rng.random() < 0.45:
            p.release(*live.pop(rng.integers(len(live))))
        else:
            r = p.alloc(int(rng.integers(1, 1 << 17)))
            if r is not None:
                live.append(r)
        spans = sorted(live)
        for (o1, n1), (o2, _) in zip(spans, spans[1:]):
            assert o1 + n1 <= o2
        assert sum(n for _, n in live) + p.available == p.size
    for r in live:
        p.release(*r)
    assert p.free == [(0, 1 << 20)]
