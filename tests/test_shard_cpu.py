"""Scene sharding across ranks (batched workloads): the partition, and world_size-2 gloo runs on CPU
whose gathered results equal the unsharded run. The CPU FP64 oracle stands in for each rank's GPU
engine here (no GPU in these tests)."""
import os
import socket

import numpy as np
import pytest

from cardillocxx_gb300 import scenes
from cardillocxx_gb300.shard import gather_rows, gather_scene_values, partition_scenes, rank_shard, scene_body_counts


def test_partition_balances_sphere_counts():
    rng = np.random.default_rng(0)
    counts = np.round(np.exp(rng.uniform(np.log(16), np.log(512), 4096))).astype(int)
    for world in (1, 2, 3, 8):
        parts = partition_scenes(counts, world)
        allp = np.sort(np.concatenate(parts))
        assert np.array_equal(allp, np.arange(4096))
        loads = np.array([counts[p].sum() for p in parts])
        assert loads.max() - loads.min() <= counts.max()
        assert loads.max() <= counts.sum() / world + counts.max()
        assert all(np.all(np.diff(p) > 0) for p in parts)
    assert [list(p) for p in partition_scenes([5, 1, 4, 2], 2)] == [[0, 1], [2, 3]]


def test_shard_keeps_every_per_static_array():
    # cylinders and boxes carry per-static arrays beyond the halfspace's (half length, half extents):
    # a shard takes its scenes' rows of every one of them
    from cardillocxx_gb300.scenes import make_scene
    from cardillocxx_gb300.shard import shard_scene
    bodies = [{"pos": (0.0, 0.0, 0.5 + 0.2 * i), "radius": 0.05} for i in range(6)]
    statics = [{"kind": "halfspace", "pos": (0, 0, 0), "dir": (0, 0, 1)},
               {"kind": "cylinder", "pos": (0, 0, 0.2), "dir": (1, 0, 0), "radius": 0.1, "half_length": 0.3},
               {"kind": "box", "pos": (0, 0, 0.1), "half_extents": (0.3, 0.2, 0.1)},
               {"kind": "box", "pos": (0, 0, 0.1), "half_extents": (0.5, 0.6, 0.7)}]
    s = make_scene(bodies, statics, scene_ids=[0, 0, 1, 1, 2, 2], static_scene_ids=[0, 1, 1, 2])
    out, bsel = shard_scene(s, [1, 2])
    assert out["static_kind"].tolist() == [2, 3, 3]
    assert out["static_half_length"].tolist() == [0.3, 0.0, 0.0]
    assert out["static_half_extents"].tolist() == [[0.0, 0.0, 0.0], [0.3, 0.2, 0.1], [0.5, 0.6, 0.7]]
    assert out["static_scene"].tolist() == [0, 0, 1] and out["body_scene"].tolist() == [0, 0, 1, 1]
    for k, v in out.items():
        if k.startswith("static_") and isinstance(v, np.ndarray):
            assert v.shape[0] == 3, k


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O

    # batched piles: each rank steps its scenes, positions gathered in the original order
    s = scenes.generate("batch_4096", scale=6 / 4096)
    cfg = scenes.config_for("batch_4096")
    sub, keep, bsel = rank_shard(s, rank, world)
    o = O.Oracle(sub, cfg)
    o.step(15)
    pos = gather_rows(o.state()["pos"], bsel, s["pos"].shape[0], dist)
    # differentiation workload: per-scene COM loss and friction gradient, gathered by scene
    d = scenes.generate("diff_256x256", scale=4 / 256)
    dcfg = scenes.config_for("diff_256x256")
    dsub, dkeep, dsel = rank_shard(d, rank, world)
    A = O.AdjOracle(dsub, dcfg)
    mu = np.full(len(dkeep), 0.3)
    xT, _, _ = A.rollout(10, dsub["pos"], dsub["vel"], dsub["omega"], mu)
    sc, m = dsub["body_scene"], dsub["mass"]
    M = np.bincount(sc, weights=m, minlength=len(dkeep))
    com = np.stack([np.bincount(sc, weights=m * xT[:, k], minlength=len(dkeep)) for k in range(3)], 1) / M[:, None]
    target = np.array([0.5, 0.5, 0.2])
    loss = ((com - target) ** 2).sum(1)
    gx = 2 * (com - target)[sc] * (m / M[sc])[:, None]
    z = np.zeros_like(gx)
    gmu = A.gradient(10, dsub["pos"], dsub["vel"], dsub["omega"], mu, gx, z, z)[3]
    L = gather_scene_values(loss, dkeep, int(d["num_scenes"]), dist)
    G = gather_scene_values(gmu, dkeep, int(d["num_scenes"]), dist)
    if rank == 0:
        np.savez(os.path.join(out_dir, "sharded.npz"), pos=pos, loss=L, gmu=G)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_the_unsharded_run(oracle_mod, tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, start_method="spawn",
                       join=True)
    r = np.load(tmp_path / "sharded.npz")
    s = scenes.generate("batch_4096", scale=6 / 4096)
    o = oracle_mod.Oracle(s, scenes.config_for("batch_4096"))
    o.step(15)
    assert np.array_equal(r["pos"], o.state()["pos"])
    d = scenes.generate("diff_256x256", scale=4 / 256)
    A = oracle_mod.AdjOracle(d, scenes.config_for("diff_256x256"))
    nsc = int(d["num_scenes"])
    mu = np.full(nsc, 0.3)
    xT, _, _ = A.rollout(10, d["pos"], d["vel"], d["omega"], mu)
    sc, m = d["body_scene"], d["mass"]
    M = np.bincount(sc, weights=m, minlength=nsc)
    com = np.stack([np.bincount(sc, weights=m * xT[:, k], minlength=nsc) for k in range(3)], 1) / M[:, None]
    target = np.array([0.5, 0.5, 0.2])
    gx = 2 * (com - target)[sc] * (m / M[sc])[:, None]
    z = np.zeros_like(gx)
    gmu = A.gradient(10, d["pos"], d["vel"], d["omega"], mu, gx, z, z)[3]
    np.testing.assert_allclose(r["loss"], ((com - target) ** 2).sum(1), rtol=1e-12, atol=0)
    np.testing.assert_allclose(r["gmu"], gmu, rtol=1e-10, atol=1e-300)
