"""Multi-process path: two gloo ranks each run a contiguous shard of the
realizations and merge moments with tl_merge_moments; the result must equal
one process running every realization, because streams are keyed by the
realization id.  On CPU the FP64 oracle stands in for the per-rank engine;
where a GPU is present, a second test runs the engine itself in each rank
(both ranks on the one GPU: their launches are independent, nothing in one
waits on the other)."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from tau_leaping_gb300.shard import merge_moments, shard_range

T, R, SEED = 0.5, 301, 4


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _oracle_shard(off, cnt):
    from oracle import py as ora
    from tau_leaping_gb300 import Model
    m = Model.generate("dimer", x0_min=500, x0_max=500)
    o = ora.OracleModel.from_desc(m.desc())
    s = o.simulate(T, R, seed=SEED, intervals=2, tracked=[0, 1], r_begin=off, r_end=off + cnt, threads=2)
    x = s["samples"][0].astype(np.float64)
    return x.mean(0), x.std(0, ddof=1), s["samples"][0]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from tau_leaping_gb300.shard import simulate_sharded
    keep = {}

    def run(off, cnt):
        mean, sd, samp = _oracle_shard(off, cnt)
        keep["samp"] = samp
        return mean, sd

    n, mean, sd = simulate_sharded(run, R)
    out[rank] = (n, mean, sd, keep["samp"], shard_range(R, world, rank))
    dist.destroy_process_group()


def test_shard_ranges_partition():
    for total, world in ((10, 3), (7, 7), (5, 8), (100000, 8)):
        got = [shard_range(total, world, r) for r in range(world)]
        assert sum(c for _, c in got) == total
        assert got[0][0] == 0
        for (o1, c1), (o2, _) in zip(got, got[1:]):
            assert o1 + c1 == o2


def test_merge_moments_matches_pooled():
    rng = np.random.default_rng(0)
    parts = [rng.normal(5, 2, size=(n, 3)) for n in (1, 17, 200, 3)]
    n, m, s = merge_moments([len(p) for p in parts], [p.mean(0) for p in parts],
                            [p.std(0, ddof=1) if len(p) > 1 else np.zeros(3) for p in parts])
    allx = np.concatenate(parts)
    assert n == len(allx)
    assert np.allclose(m, allx.mean(0), rtol=1e-12)
    assert np.allclose(s, allx.std(0, ddof=1), rtol=1e-12)


def test_two_gloo_ranks_equal_one_process():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as man:
        out = man.dict()
        procs = [ctx.Process(target=_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    full_mean, full_sd, full_samp = _oracle_shard(0, R)
    for rank in range(world):
        n, mean, sd, samp, (off, cnt) = res[rank]
        assert n == R
        assert np.allclose(mean, full_mean, rtol=1e-12)
        assert np.allclose(sd, full_sd, rtol=1e-10)
        # realization streams do not depend on the partition
        assert np.array_equal(samp, full_samp[off:off + cnt])


def _engine_worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from tau_leaping_gb300 import Model
    from tau_leaping_gb300.shard import simulate_sharded
    m = Model.generate("toy", n_species=32, n_channels=64, seed=4, x0_max=3000)
    keep = {}

    def run(off, cnt):
        r = m.simulate(0.004, cnt, seed=SEED, intervals=2, tracked=[0, 1], keep_samples=True,
                       realization_offset=off)
        keep["samp"] = r.samples[0]
        return r.mean[0], r.stddev[0]

    n, mean, sd = simulate_sharded(run, 1001)
    out[rank] = (n, mean, sd, keep["samp"], shard_range(1001, world, rank))
    dist.destroy_process_group()


@pytest.mark.gpu
def test_two_gloo_ranks_running_the_engine_equal_one_call():
    from tau_leaping_gb300 import Model
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as man:
        out = man.dict()
        procs = [ctx.Process(target=_engine_worker, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
            assert p.exitcode == 0
        res = dict(out)
    m = Model.generate("toy", n_species=32, n_channels=64, seed=4, x0_max=3000)
    full = m.simulate(0.004, 1001, seed=SEED, intervals=2, tracked=[0, 1], keep_samples=True)
    for rank in range(world):
        n, mean, sd, samp, (off, cnt) = res[rank]
        assert n == 1001
        assert np.allclose(mean, full.mean[0], rtol=1e-12)
        assert np.allclose(sd, full.stddev[0], rtol=1e-9)
        assert np.array_equal(samp, full.samples[0, off:off + cnt])
