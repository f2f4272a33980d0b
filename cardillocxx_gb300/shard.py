"""Scene sharding for batched workloads across ranks (one process per GPU).

Independent scenes (thousands of small piles, the differentiation workload's 256 scenes) need no
exchange while they step: the scenes are partitioned across ranks, balanced by their sphere counts,
each rank steps its shard on its own GPU, and the results meet once at the end (positions gathered,
or for a loss the per-scene loss and gradient values gathered). A single pile does not shard here:
its ranks would need a halo exchange every sweep, so the pile workloads run as replicas.

The partition is greedy longest-processing-time: scenes in decreasing size, each to the rank with
the fewest spheres so far (ties to the lower rank), so the largest rank load is within one scene of
the optimum.
"""
from __future__ import annotations

import numpy as np

SCENE_KEYS_STATIC = ("static_kind", "static_pos", "static_quat", "static_vel", "static_omega", "static_dir",
                     "static_radius", "static_mu", "static_rest_n", "static_rest_t", "static_half_length",
                     "static_half_extents")


def partition_scenes(body_counts, world: int) -> list[np.ndarray]:
    """Scene indices per rank, balanced by sphere count (each list sorted ascending)."""
    counts = np.asarray(body_counts, np.int64)
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(counts)), key=lambda s: (-int(counts[s]), s))
    load = [0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for s in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(s)
        load[r] += int(counts[s])
    return [np.array(sorted(p), np.int64) for p in parts]


def scene_body_counts(scene: dict) -> np.ndarray:
    n = int(scene.get("num_scenes", 1))
    bs = scene.get("body_scene")
    if bs is None:
        return np.array([scene["pos"].shape[0]], np.int64)
    return np.bincount(np.asarray(bs), minlength=n).astype(np.int64)


def shard_scene(scene: dict, keep) -> tuple[dict, np.ndarray]:
    """The scenes `keep` of a batched scene dict, renumbered in the order given; also the mask of
    the bodies kept (in the original body order, which the shard preserves)."""
    keep = [int(k) for k in keep]
    N = scene["pos"].shape[0]
    bs = np.asarray(scene.get("body_scene", np.zeros(N, np.int32)))
    S = np.asarray(scene["static_kind"]).shape[0]
    ss = np.asarray(scene.get("static_scene", np.zeros(S, np.int32)))
    bsel = np.isin(bs, keep)
    ssel = np.isin(ss, keep)
    remap = np.full(int(scene.get("num_scenes", 1)), -1, np.int64)
    remap[keep] = np.arange(len(keep))
    out = {}
    for k, v in scene.items():
        if k in SCENE_KEYS_STATIC:
            out[k] = np.ascontiguousarray(v[ssel])
        elif isinstance(v, np.ndarray) and v.shape[:1] == (N,):
            out[k] = np.ascontiguousarray(v[bsel])
        else:
            out[k] = v
    out["body_scene"] = remap[bs[bsel]].astype(np.int32)
    out["static_scene"] = remap[ss[ssel]].astype(np.int32)
    out["num_scenes"] = len(keep)
    # bodies of a scene must stay contiguous and scenes in increasing order
    if np.any(np.diff(out["body_scene"]) < 0) or np.any(np.diff(out["static_scene"]) < 0):
        raise ValueError("the kept scenes must be given in increasing order of their bodies")
    return out, bsel


def rank_shard(scene: dict, rank: int, world: int) -> tuple[dict, np.ndarray, np.ndarray]:
    """This rank's shard: (scene dict, kept scene ids, mask of kept bodies)."""
    parts = partition_scenes(scene_body_counts(scene), world)
    keep = parts[rank]
    sub, bsel = shard_scene(scene, keep)
    return sub, keep, bsel


def gather_rows(local: np.ndarray, bsel: np.ndarray, n_total: int, dist=None) -> np.ndarray:
    """Reassemble per-body rows of every rank's shard in the original body order (all ranks get
    the full array). `dist` is torch.distributed (initialised) or None for a single rank."""
    out = np.zeros((n_total,) + local.shape[1:], local.dtype)
    if dist is None or dist.get_world_size() == 1:
        out[bsel] = local
        return out
    world = dist.get_world_size()
    pieces = [None] * world
    dist.all_gather_object(pieces, (np.nonzero(bsel)[0], local))
    for idx, rows in pieces:
        out[idx] = rows
    return out


def gather_scene_values(local: np.ndarray, keep: np.ndarray, n_scenes: int, dist=None) -> np.ndarray:
    """Per-scene values (loss terms, friction gradients) of every rank, in scene order."""
    out = np.zeros((n_scenes,) + local.shape[1:], local.dtype)
    if dist is None or dist.get_world_size() == 1:
        out[keep] = local
        return out
    world = dist.get_world_size()
    pieces = [None] * world
    dist.all_gather_object(pieces, (np.asarray(keep), local))
    for k, vals in pieces:
        out[k] = vals
    return out
