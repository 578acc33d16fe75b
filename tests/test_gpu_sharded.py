"""The multi-rank engines, executed (GB300 only): two gloo ranks in separate
processes, both on cuda:0.  No kernel of one rank waits on the other's: the
only exchange is the host-side all-reduce of the maxima (row sharding) or the
gather of results (star sharding).

* ShardedRejection (one star's prior samples split by rows): each rank holds
  its half of the rows in its own cache, evaluates, exchanges the maxima
  and accepts its rows against the star's uniform stream at its offset.  The
  gathered indices and the global count must equal a single-process
  BatchRejection over all rows, for the FP64 and the mixed path.
* StarShardedRejection (many stars split by epoch load): every rank holds the
  whole cache and its stars; the gathered counts and indices must equal a
  single-process BatchRejection over all stars.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

S_ROWS = 1 << 20
N_STARS = 24


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _row_star():
    from gpu_util import synth_star
    rng = np.random.default_rng(8)
    return synth_star(rng, 30, base=2000.0, sig=(0.1, 0.5), K=12.0)


def _row_chunk():
    from gpu_util import synth_chunk
    return synth_chunk(np.random.default_rng(9), S_ROWS, jitter=True)


def _survey():
    from thejoker_gb300.synthetic import survey_stars
    return survey_stars(N_STARS, seed=5, n_max=128)


def _worker(rank, world, port, ret):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from thejoker_gb300 import build, device as dev
        from thejoker_gb300.parallel import (ShardedRejection, StarShardedRejection,
                                             gather_indices, shard_rows)
        from thejoker_gb300.synthetic import fill_prior_cache
        build.build()
        out = {}
        # one star's rows across the ranks
        star, chunk = _row_star(), _row_chunk()
        row0, n = shard_rows(S_ROWS, world, rank)
        table = dev.StarTable([star], jitter="applied")
        cache = dev.PriorCache.from_samples(chunk[row0:row0 + n])
        gen = np.random.default_rng(1234)
        pcg = dev.pcg64_state(gen)
        for prec in ("fp64", "mixed"):
            sr = ShardedRejection(table, cache, row0=row0, precision=prec, max_out=n)
            idx, total = sr.run(pcg)
            out[("rows", prec)] = (gather_indices(idx), total)
        # many stars across the ranks
        stars = _survey()
        S = 1 << 18
        scache = dev.PriorCache.from_samples(fill_prior_cache(np.empty((S, 5)), 0))
        for prec in ("fp64", "mixed"):
            ss = StarShardedRejection(stars, scache, precision=prec, max_out=300,
                                      seeds=np.arange(N_STARS) + 50, chunk=1024)
            ss.run()
            out[("stars", prec)] = ss.gather()
        ret[rank] = out
    finally:
        dist.destroy_process_group()


def test_sharded_engines_equal_single_process(cuda):
    from thejoker_gb300 import device as dev
    from thejoker_gb300.batch import BatchRejection
    from thejoker_gb300.synthetic import fill_prior_cache
    world = 2
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    ret = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, ret)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(600)
        assert p.exitcode == 0
    # single process: one star over all rows
    table = dev.StarTable([_row_star()], jitter="applied")
    cache = dev.PriorCache.from_samples(_row_chunk())
    for prec in ("fp64", "mixed"):
        b = BatchRejection(table, cache, precision=prec, max_out=S_ROWS, seeds=[1234])
        b.run()
        counts, idx, _ = b.results()
        assert counts[0] > 0
        for r in range(world):
            g_idx, total = ret[r][("rows", prec)]
            assert total == counts[0]
            np.testing.assert_array_equal(g_idx, idx[0])
    # single process: all stars
    stars = _survey()
    S = 1 << 18
    scache = dev.PriorCache.from_samples(fill_prior_cache(np.empty((S, 5)), 0))
    for prec in ("fp64", "mixed"):
        b = BatchRejection(stars, scache, precision=prec, max_out=300,
                           seeds=np.arange(N_STARS) + 50, chunk=1024)
        b.run()
        counts, idx, ll = b.results()
        for r in range(world):
            c2, i2, l2 = ret[r][("stars", prec)]
            np.testing.assert_array_equal(c2, counts)
            for k in range(N_STARS):
                np.testing.assert_array_equal(i2[k], idx[k])
                np.testing.assert_allclose(l2[k], ll[k], rtol=0,
                                           atol=0 if prec == "fp64" else 2e-4)
