"""Batch sharding by scene across processes (CPU, gloo, world size 2): every
rank derives the same partition, the shards are disjoint and cover every
scene, particle loads are balanced within the largest scene, and the
host-side gather of per-rank reductions gives the whole batch's values."""
import os
import socket

import numpy as np
import pytest

from lustrine_gb300 import sharding


def _config3_counts():
    rng = np.random.default_rng(3)
    return np.round(np.exp(rng.uniform(np.log(1024), np.log(65536), 512))).astype(int)


def test_partition_is_disjoint_complete_and_balanced():
    counts = _config3_counts()
    for world in (1, 2, 3, 4, 8):
        shards = sharding.shard_scenes(counts, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(counts)))
        loads = [int(counts[s].sum()) for s in shards]
        assert max(loads) - min(loads) <= counts.max()
        assert sharding.shard_scenes(counts, world) == shards  # deterministic


def test_partition_edge_cases():
    assert sharding.shard_scenes([], 2) == [[], []]
    assert sharding.shard_scenes([5], 3) == [[0], [], []]
    with pytest.raises(ValueError):
        sharding.shard_scenes([1, 2], 0)


def _stats(x, v):
    m = float(len(x))
    return {"mass": m, "momentum": v.sum(0).tolist(), "kinetic": 0.5 * float((v * v).sum()),
            "com": (x.sum(0) / m).tolist(), "max_density_error": float(np.abs(x[:, 0]).max() % 1)}


def _scene_data(counts):
    rng = np.random.default_rng(11)
    return [(rng.normal(size=(c, 3)), rng.normal(size=(c, 3))) for c in counts]


def _worker(rank, world, port, counts, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = sharding.my_scenes(counts, world, rank)
        data = _scene_data(counts)
        # a rank's batch: its scenes concatenated (what one batched context holds)
        if mine:
            x = np.concatenate([data[i][0] for i in mine])
            v = np.concatenate([data[i][1] for i in mine])
            local = _stats(x, v)
        else:
            local = None
        # every rank derived the same partition
        parts = [None] * world
        dist.all_gather_object(parts, mine)
        total = sharding.gather_reductions(local, world)
        if rank == 0:
            np.save(out_path, np.array([parts, total], dtype=object), allow_pickle=True)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_ranks_gloo_gather_matches_single_process(tmp_path):
    import torch.multiprocessing as mp
    counts = [int(c) for c in _config3_counts()[:40] // 64]
    out = str(tmp_path / "r.npy")
    mp.start_processes(_worker, args=(2, _free_port(), counts, out), nprocs=2, start_method="spawn")
    parts, total = np.load(out, allow_pickle=True)
    assert sorted(parts[0] + parts[1]) == list(range(len(counts)))
    assert not set(parts[0]) & set(parts[1])
    data = _scene_data(counts)
    x = np.concatenate([d[0] for d in data])
    v = np.concatenate([d[1] for d in data])
    ref = _stats(x, v)
    assert total["mass"] == ref["mass"]
    np.testing.assert_allclose(total["momentum"], ref["momentum"], rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(total["kinetic"], ref["kinetic"], rtol=1e-12)
    np.testing.assert_allclose(total["com"], ref["com"], rtol=1e-12, atol=1e-12)
    assert total["max_density_error"] == ref["max_density_error"]
