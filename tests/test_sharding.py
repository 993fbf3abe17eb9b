"""Multi-rank event sharding on CPU (gloo, world size 2): each rank owns a
contiguous block of solves, computes its partial misfit and gradient (here
with the FP64 oracle standing in for its GPU), and one all-reduce gives the
same result as the single-process batch."""
import os
import socket

import numpy as np
import pytest

from adtomo_gb300.shard import allreduce_sum_f64, shard_solves


def test_shard_solves_partition():
    for n in (0, 1, 7, 256, 2000):
        for world in (1, 2, 3, 8):
            blocks = [shard_solves(n, r, world) for r in range(world)]
            assert blocks[0][0] == 0 and blocks[-1][1] == n
            assert all(blocks[i][1] == blocks[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in blocks]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_solves(10, 2, 2)


def _problem():
    rng = np.random.default_rng(11)
    m, n, l, h = 9, 8, 7, 0.5
    f = 0.2 + 0.05 * rng.random((m, n, l))
    sta = np.column_stack([rng.uniform(0, m - 1, 5), rng.uniform(0, n - 1, 5), np.zeros(5)])
    src = np.column_stack([rng.uniform(1, m - 2, 5), rng.uniform(1, n - 2, 5), rng.uniform(1, l - 2, 5)])
    t_obs = rng.uniform(0.5, 2.0, 25)
    w = np.ones(25)
    return f, h, sta, src, t_obs, w


def _worker(rank, world, port, out_path):
    import torch.distributed as dist

    from oracle import oracle as O

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    f, h, sta, src, t_obs, w = _problem()
    a, b = shard_solves(len(src), rank, world)
    mis, _, (g,), _ = O.batch_misfit_grad([(f, h)], [sta], np.zeros(b - a, np.int32), src[a:b],
                                          t_obs[5 * a:5 * b], w[5 * a:5 * b])
    mis_t, g_t = allreduce_sum_f64([np.array([mis]), g])
    if rank == 0:
        np.savez(out_path, mis=mis_t, g=g_t)
    dist.destroy_process_group()


def test_two_rank_gloo_matches_single_process(tmp_path):
    import torch.multiprocessing as mp

    from oracle import oracle as O

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "r0.npz")
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    r = np.load(out)
    f, h, sta, src, t_obs, w = _problem()
    mis, _, (g,), _ = O.batch_misfit_grad([(f, h)], [sta], np.zeros(len(src), np.int32), src, t_obs,
                                          w)
    assert abs(r["mis"][0] - mis) <= 1e-12 * mis
    np.testing.assert_allclose(r["g"], g, rtol=0, atol=1e-12 * np.abs(g).max())
