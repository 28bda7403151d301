"""Sharding (fit, sequence) items across ranks: the partition covers every
sequence exactly once with balanced cost, and the gather reassembles the
shards into the unsharded layout -- over two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from cuda_mcmc_gb300 import shard


def _check_partition(nseqs, costs, world):
    parts = shard.partition(nseqs, costs, world)
    assert len(parts) == world
    seen = [np.zeros(n, int) for n in nseqs]
    for p in parts:
        for f, s0, s1 in p:
            assert 0 <= s0 < s1 <= nseqs[f]
            seen[f][s0:s1] += 1
    assert all(np.all(x == 1) for x in seen)
    loads = shard.rank_cost(parts, costs)
    total = sum(n * c for n, c in zip(nseqs, costs))
    assert max(loads) <= total / world + max(costs) + 1e-9
    return parts


@pytest.mark.parametrize("world", [1, 2, 3, 5, 8])
def test_partition_covers_every_sequence_once_and_balances(world):
    rng = np.random.default_rng(world)
    nseqs = rng.integers(1, 20, 13).tolist()
    costs = np.exp(rng.uniform(0, 5, 13)).tolist()
    _check_partition(nseqs, costs, world)


def test_partition_of_one_fit_is_contiguous_ranges():
    parts = _check_partition([64], [1.0], 4)
    assert parts == [[(0, 0, 16)], [(0, 16, 32)], [(0, 32, 48)], [(0, 48, 64)]]


def test_more_ranks_than_sequences_leaves_ranks_idle():
    parts = _check_partition([2], [1.0], 4)
    assert sum(len(p) for p in parts) == 2


def _full(nseqs, f):
    """A fit's 'unsharded' arrays: values encode (fit, position)."""
    n = nseqs[f]
    return {"pout": np.arange(3 * 4 * n * 5, dtype=np.float32).reshape(3, 4, n, 5) + 1000 * f,
            "tout": np.arange(4 * n * 5, dtype=np.int32).reshape(4, n, 5) + 100 * f,
            "chi2": np.arange(n * 5, dtype=np.float32).reshape(n, 5) - f}


def _slice(full, s0, s1):
    return {k: np.take(v, range(s0, s1), axis=shard.SEQ_AXIS[k]) for k, v in full.items()}


def _rank_main(rank, world, port, nseqs, costs, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        parts = shard.partition(nseqs, costs, world)[rank]
        local = [(f, s0, s1, _slice(_full(nseqs, f), s0, s1)) for f, s0, s1 in parts]
        got = shard.gather(local, len(nseqs))
        if rank == 0:
            ok = all(np.array_equal(got[f][k], _full(nseqs, f)[k])
                     for f in range(len(nseqs)) for k in ("pout", "tout", "chi2"))
            with open(out_path, "w") as fh:
                fh.write("ok" if ok else "mismatch")
        else:
            assert got is None
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_gather_over_two_gloo_ranks(tmp_path):
    nseqs, costs = [5, 1, 7], [2.0, 9.0, 1.0]
    out = tmp_path / "result.txt"
    mp.spawn(_rank_main, args=(2, _free_port(), nseqs, costs, str(out)), nprocs=2, join=True)
    assert out.read_text() == "ok"


def test_gather_without_a_process_group_assembles_local_shards():
    full = _full([4], 0)
    local = [(0, 2, 4, _slice(full, 2, 4)), (0, 0, 2, _slice(full, 0, 2))]
    got = shard.gather(local, 1)
    assert all(np.array_equal(got[0][k], full[k]) for k in full)
    with pytest.raises(ValueError, match="missing"):
        shard.gather(local[:1], 1)
