"""Multi-rank logic on CPU with gloo, world size 2 (no GPU): the sharding plans,
the order-preserving key all-reduce, and the sharded acceptance protocol
(ranks own row ranges of one star's samples, exchange the maximum, test their
own samples against the star's uniform stream at their offset, and gather).
The ln L values come from the CPU oracle."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from thejoker_gb300 import parallel


def test_shard_rows_cover_and_balance():
    for n, w in [(10, 3), (7, 7), (2 ** 28, 8), (5, 8)]:
        parts = [parallel.shard_rows(n, w, r) for r in range(w)]
        assert parts[0][0] == 0
        for (a0, c0), (a1, _) in zip(parts, parts[1:]):
            assert a0 + c0 == a1
        assert sum(c for _, c in parts) == n
        assert max(c for _, c in parts) - min(c for _, c in parts) <= 1


def test_shard_stars_lpt():
    rng = np.random.default_rng(0)
    ep = rng.integers(3, 257, 4096)
    parts = parallel.shard_stars(ep, 8)
    assert sorted(sum(parts, [])) == list(range(4096))
    loads = [ep[p].sum() for p in parts]
    assert max(loads) - min(loads) <= ep.max()


def test_keys_order_and_roundtrip():
    x = np.array([-np.inf, -1e300, -3.5, -0.0, 0.0, 2e-300, 7.0, 1e308, np.inf])
    k = parallel.key_of(x)
    assert np.all(np.diff(k.astype(object)) >= 0)
    np.testing.assert_array_equal(parallel.value_of(k), x)
    assert parallel.key_of(np.nan) == np.uint64(0xFFFFFFFFFFFFFFFF)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, ret):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle
        from thejoker_gb300.linear import rv_unit_columns
        rng = np.random.default_rng(5)
        N, S = 9, 6000
        t = np.sort(rng.uniform(0, 800, N)) + 56000
        err = rng.uniform(0.1, 0.4, N)
        rv = 4 * rv_unit_columns(t, t.min(), [33.0], [0.2], [1.0], [2.0])[0] + rng.normal(0, err)
        chunk = np.stack([np.exp(rng.uniform(np.log(2), np.log(1024), S)),
                          rng.beta(0.867, 3.03, S), rng.uniform(0, 6.28, S),
                          rng.uniform(0, 6.28, S), np.zeros(S)], 1)
        row0, n = parallel.shard_rows(S, world, rank)
        lls = oracle.batch_marginal_ln_likelihood(
            t, rv, 1 / err ** 2, t.min(), np.ones((N, 1)), [0, 0], [0, 1e4],
            chunk[row0:row0 + n], True, 30., 365.25, 500.)
        # exchange the maximum as order-preserving keys
        keys = torch.from_numpy(np.array([parallel.key_of(lls.max())]).view(np.int64).copy())
        parallel.allreduce_max_keys(keys)
        gmax = float(parallel.value_of(keys.numpy().view(np.uint64))[0])
        # this rank's uniforms: the star's stream from position row0
        gen = np.random.default_rng(77)
        gen.bit_generator.advance(row0)
        uu = gen.uniform(size=n)
        local = np.where(np.exp(lls - gmax) > uu)[0] + row0
        ret[rank] = (gmax, parallel.gather_indices(local))
    finally:
        dist.destroy_process_group()


def test_sharded_accept_equals_single_process():
    world = 2
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    ret = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, ret)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    # single-process reference
    from oracle import oracle
    from thejoker_gb300.linear import rv_unit_columns
    rng = np.random.default_rng(5)
    N, S = 9, 6000
    t = np.sort(rng.uniform(0, 800, N)) + 56000
    err = rng.uniform(0.1, 0.4, N)
    rv = 4 * rv_unit_columns(t, t.min(), [33.0], [0.2], [1.0], [2.0])[0] + rng.normal(0, err)
    chunk = np.stack([np.exp(rng.uniform(np.log(2), np.log(1024), S)), rng.beta(0.867, 3.03, S),
                      rng.uniform(0, 6.28, S), rng.uniform(0, 6.28, S), np.zeros(S)], 1)
    lls = oracle.batch_marginal_ln_likelihood(t, rv, 1 / err ** 2, t.min(), np.ones((N, 1)),
                                              [0, 0], [0, 1e4], chunk, True, 30., 365.25, 500.)
    uu = np.random.default_rng(77).uniform(size=S)
    good = np.where(np.exp(lls - lls.max()) > uu)[0]
    for r in range(world):
        gmax, idx = ret[r]
        assert gmax == lls.max()
        np.testing.assert_array_equal(idx, good)
