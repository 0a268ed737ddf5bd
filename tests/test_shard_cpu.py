"""The multi-rank path on CPU: two gloo ranks each take a slab of one seeded
global batch (shard.slab + bilu.gen_stencil(first=...)), solve it with the
oracle, and gather the results; the gathered batch equals the single-process
solve of the whole batch bit for bit.  The step-time reduction takes the
slowest rank.  No GPU; the same partition runs one rank per GPU under
torchrun."""
import os
import socket

import numpy as np
import pytest

import bilu
import shard

FIELDS = ("x", "iters", "conv", "res", "true_res")


def test_slab_partition():
    for nsys in (0, 1, 7, 64, 1001):
        for world in (1, 2, 3, 8):
            got = [shard.slab(nsys, r, world) for r in range(world)]
            assert sum(c for _, c in got) == nsys
            assert got[0][0] == 0
            for (f0, c0), (f1, _) in zip(got, got[1:]):
                assert f1 == f0 + c0
            assert max(c for _, c in got) - min(c for _, c in got) <= 1
    with pytest.raises(ValueError):
        shard.slab(4, 2, 2)


def test_generator_range_matches_whole_batch(built):
    rp, ci, v, b = bilu.gen_stencil(5, 7, 7, 7, 10, seed=3)
    rp2, ci2, v2, b2 = bilu.gen_stencil(5, 7, 7, 7, 4, seed=3, first=6)
    np.testing.assert_array_equal(rp, rp2)
    np.testing.assert_array_equal(ci, ci2)
    np.testing.assert_array_equal(v[6:], v2)
    np.testing.assert_array_equal(b[6:], b2)


def _solve(rp, ci, v, b):
    import helpers as H
    o = H.oracle_pipeline(rp, ci, v, b, bilu.PRECOND_ILU0, tol_mode=1, tol=1e-10)
    return {k: o[k] for k in FIELDS}


def _rank(rank, world, port, nsys, out_dir):
    import torch.distributed as dist
    os.environ["OMP_NUM_THREADS"] = "2"
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        first, count = shard.slab(nsys, rank, world)
        rp, ci, v, b = bilu.gen_stencil(1, 8, 8, 1, count, seed=21, first=first)
        res = shard.gather(_solve(rp, ci, v, b))
        slowest = shard.max_over_ranks(10.0 + rank)
        if rank == 0:
            np.savez(os.path.join(out_dir, "gathered.npz"), slowest=slowest, **res)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_equal_single_process(built, tmp_path):
    import torch.multiprocessing as mp
    nsys, world = 13, 2
    mp.spawn(_rank, args=(world, _free_port(), nsys, str(tmp_path)), nprocs=world, join=True)
    got = np.load(os.path.join(str(tmp_path), "gathered.npz"))
    assert float(got["slowest"]) == 11.0
    rp, ci, v, b = bilu.gen_stencil(1, 8, 8, 1, nsys, seed=21)
    want = _solve(rp, ci, v, b)
    for k in FIELDS:
        assert got[k].shape == want[k].shape, k
        assert np.array_equal(got[k], want[k]), k
    assert np.all(want["conv"] == 1)
