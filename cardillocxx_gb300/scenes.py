"""Seeded benchmark scenes (generated by the library's C++ generator) and their configurations.

Presets follow the five workloads the path is measured on:
  pile_1k       1,000 spheres r=0.05 in a 1x1x2 m box, mu 0.3, h 1e-3, 50 PJ sweeps, alpha 0.5
  pile_200k     200,000 spheres r~U[0.02,0.05] in a 4x4x8 m box, mu 0.4, h 5e-4, 100 sweeps or residual 1e-6
  batch_4096    4,096 scenes of log-uniform[16,512] spheres r~U[0.03,0.06], mu~U[0.1,0.8], 50 sweeps
  diff_256x256  256 scenes x 256 spheres r=0.04, v0~N(0,0.5^2), mu 0.3, 50 sweeps
  drum_1m       1,000,000 spheres r~U[0.01,0.015] in a drum R=3.36 m L=1 m at 2 rad/s, mu 0.5, h 2e-4, 80 sweeps
`scale` shrinks a preset for tests: body count (or scene count for the batched presets) times
scale, box edge times scale^(1/3) so the packing fraction is kept.
Seeds are 0xC0FFEE00 + preset number.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import CdxError, CdxGenParams, CdxScene

SEED_BASE = 0xC0FFEE00

PRESETS = {
    "pile_1k": dict(num=1, kind=0, num_scenes=1, num_bodies=1000, r=(0.05, 0.05), box=(1.0, 1.0, 2.0), mu=0.3,
                    cfg={"sim.dt": 1e-3, "pj.max_iterations": 50, "pj.alpha": 0.5, "pj.relaxation": 0.5,
                         "pj.tol_abs": 0.0, "pj.tol_rel": 0.0, "friction.default_mu": 0.3}, steps=500),
    "pile_200k": dict(num=2, kind=0, num_scenes=1, num_bodies=200000, r=(0.02, 0.05), box=(4.0, 4.0, 8.0), mu=0.4,
                      cfg={"sim.dt": 5e-4, "pj.max_iterations": 100, "pj.alpha": 0.5, "pj.tol_abs": 0.0,
                           "pj.tol_rel": 0.0, "gpu.residual_tol": 1e-6, "friction.default_mu": 0.4}, steps=2000),
    "batch_4096": dict(num=3, kind=0, num_scenes=4096, nb=(16, 512), r=(0.03, 0.06), box=(1.0, 1.0, 2.0),
                       mu_range=(0.1, 0.8), cfg={"sim.dt": 1e-3, "pj.max_iterations": 50, "pj.alpha": 0.5,
                                                 "pj.tol_abs": 0.0, "pj.tol_rel": 0.0}, steps=1000),
    "diff_256x256": dict(num=4, kind=0, num_scenes=256, num_bodies=256, r=(0.04, 0.04), box=(1.0, 1.0, 2.0),
                         mu=0.3, v_sigma=0.5, cfg={"sim.dt": 1e-3, "pj.max_iterations": 50, "pj.alpha": 0.5,
                                                   "pj.tol_abs": 0.0, "pj.tol_rel": 0.0}, steps=200),
    "drum_1m": dict(num=5, kind=1, num_bodies=1000000, r=(0.01, 0.015), drum=(3.36, 1.0, 2.0), mu=0.5,
                    cfg={"sim.dt": 2e-4, "pj.max_iterations": 80, "pj.alpha": 0.5, "pj.tol_abs": 0.0,
                         "pj.tol_rel": 0.0}, steps=5000),
}

COMMON_CFG = {"friction.enable": True, "friction.combine": "min", "restitution.default_normal": 0.0,
              "restitution.default_tangential": 0.0, "moreau.theta": 0.5, "pj.warmstart": True,
              "collision.security_margin": 0.0, "collision.match_max_dist": 0.02}


def config_for(preset: str, **overrides) -> dict:
    cfg = dict(COMMON_CFG)
    cfg.update(PRESETS[preset]["cfg"])
    cfg.update(overrides)
    return cfg


def generate(preset: str, scale: float = 1.0, seed: int | None = None, **kw) -> dict:
    """Generate a preset scene as a dict of numpy arrays (host memory, FP64)."""
    P = dict(PRESETS[preset])
    P.update(kw)
    g = CdxGenParams()
    g.kind = P["kind"]
    g.density = P.get("density", 1000.0)
    g.r_lo, g.r_hi = P["r"]
    g.seed = (SEED_BASE + P["num"]) if seed is None else seed
    g.max_attempts = P.get("max_attempts", 200000)
    g.v_sigma = P.get("v_sigma", 0.0)
    g.mu = P.get("mu", 0.0)
    if "mu_range" in P:
        g.mu_lo, g.mu_hi = P["mu_range"]
    if g.kind == 0:
        ns = P.get("num_scenes", 1)
        if ns > 1:
            g.num_scenes = max(1, int(round(ns * scale)))
            g.num_bodies = P.get("num_bodies", 0)
            edge = 1.0
        else:
            g.num_scenes = 1
            g.num_bodies = max(1, int(round(P["num_bodies"] * scale)))
            edge = scale ** (1.0 / 3.0)
        if "nb" in P:
            g.nb_lo, g.nb_hi = P["nb"]
        for k in range(3):
            g.box[k] = P["box"][k] * edge
    else:
        R, Ldrum, w = P["drum"]
        g.num_bodies = max(1, int(round(P["num_bodies"] * scale)))
        g.drum_radius = R * math.sqrt(scale)
        g.drum_length = Ldrum
        g.drum_omega = w
    L = _lib.lib()
    h = C.c_void_p()
    st = L.cdx_gen_create(C.byref(g), C.byref(h))
    if st:
        raise CdxError(st, f"scene generation failed for {preset} (scale {scale})")
    try:
        v = CdxScene()
        L.cdx_gen_view(h, C.byref(v))
        N, S = v.num_bodies, v.num_statics

        def arr(p, n, dt=np.float64):
            if n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True)

        out = {
            "pos": arr(v.pos, 3 * N).reshape(N, 3), "quat": arr(v.quat, 4 * N).reshape(N, 4),
            "vel": arr(v.vel, 3 * N).reshape(N, 3), "omega": arr(v.omega, 3 * N).reshape(N, 3),
            "radius": arr(v.radius, N), "mass": arr(v.mass, N), "inertia": arr(v.inertia, N), "mu": arr(v.mu, N),
            "rest_n": arr(v.rest_n, N), "rest_t": arr(v.rest_t, N), "body_scene": arr(v.body_scene, N, np.int32),
            "static_kind": arr(v.static_kind, S, np.int32), "static_pos": arr(v.static_pos, 3 * S).reshape(S, 3),
            "static_quat": arr(v.static_quat, 4 * S).reshape(S, 4),
            "static_vel": arr(v.static_vel, 3 * S).reshape(S, 3),
            "static_omega": arr(v.static_omega, 3 * S).reshape(S, 3),
            "static_dir": arr(v.static_dir, 3 * S).reshape(S, 3), "static_radius": arr(v.static_radius, S),
            "static_mu": arr(v.static_mu, S), "static_rest_n": arr(v.static_rest_n, S),
            "static_rest_t": arr(v.static_rest_t, S), "static_scene": arr(v.static_scene, S, np.int32),
            "num_scenes": int(v.num_scenes),
        }
    finally:
        L.cdx_gen_destroy(h)
    return out


def settled_pile(path: str) -> dict:
    """The settled pile stored by tests/golden/make_pile_200k_settled.py as a scene dict, at rest.

    Positions and radii are the stored FP32 values; velocities are zero and orientations the
    identity; mass and inertia follow from the radius and the stored density (solid spheres). NumPy
    only: building the scene loads no native code, so a CPU-only process can use it too.
    """
    d = np.load(path)
    pos = d["pos"].astype(np.float64)
    r = d["radius"].astype(np.float64)
    N = pos.shape[0]
    mass = float(d["density"]) * ((4.0 / 3.0) * math.pi * r * r * r)
    out = {"pos": pos, "quat": np.tile(np.array([0.0, 0.0, 0.0, 1.0]), (N, 1)), "vel": np.zeros((N, 3)),
           "omega": np.zeros((N, 3)), "radius": r, "mass": mass, "inertia": (2.0 / 5.0) * r * r * mass,
           "mu": np.full(N, float(d["mu"])), "rest_n": np.zeros(N), "rest_t": np.zeros(N),
           "body_scene": np.zeros(N, np.int32)}
    for k in ("static_kind", "static_pos", "static_quat", "static_vel", "static_omega", "static_dir",
              "static_radius", "static_mu", "static_rest_n", "static_rest_t"):
        out[k] = np.array(d[k])
    out["static_scene"] = np.zeros(out["static_kind"].shape[0], np.int32)
    out["num_scenes"] = 1
    return out


def scene_digest(scene: dict) -> str:
    """SHA-256 (first 16 hex digits) of a scene's arrays, to show two processes start alike."""
    import hashlib
    h = hashlib.sha256()
    for k in sorted(scene):
        v = scene[k]
        if isinstance(v, np.ndarray):
            h.update(k.encode())
            h.update(np.ascontiguousarray(v).tobytes())
    return h.hexdigest()[:16]


def state_digest(state: dict) -> str:
    """SHA-256 (first 16 hex digits) of a body state (positions, orientations, velocities)."""
    import hashlib
    h = hashlib.sha256()
    for k in ("pos", "quat", "vel", "omega"):
        h.update(np.ascontiguousarray(state[k], np.float64).tobytes())
    return h.hexdigest()[:16]


def make_scene(bodies: list[dict], statics: list[dict], scene_ids=None, static_scene_ids=None) -> dict:
    """Hand-built scene from per-body dicts (pos, radius, density|mass, vel, omega, quat, mu, rest_n)
    and statics (kind 'halfspace'|'drum'|'cylinder'|'box', pos, dir, radius, half_length, half_extents,
    quat, vel, omega, mu). A box's axes are the columns of its quaternion's rotation; it needs no dir."""
    N, S = len(bodies), len(statics)
    out = {k: np.zeros((N, d)) for k, d in (("pos", 3), ("quat", 4), ("vel", 3), ("omega", 3))}
    for k in ("radius", "mass", "inertia", "mu", "rest_n", "rest_t"):
        out[k] = np.zeros(N)
    for i, b in enumerate(bodies):
        r = float(b["radius"])
        out["pos"][i] = b["pos"]
        out["quat"][i] = b.get("quat", (0, 0, 0, 1))
        out["vel"][i] = b.get("vel", (0, 0, 0))
        out["omega"][i] = b.get("omega", (0, 0, 0))
        out["radius"][i] = r
        if "mass" in b:
            m = float(b["mass"])
        else:
            m = float(b.get("density", 1000.0)) * ((4.0 / 3.0) * math.pi * r * r * r)
        out["mass"][i] = m
        out["inertia"][i] = (2.0 / 5.0 * r * r) * m
        out["mu"][i] = b.get("mu", 0.3)
        out["rest_n"][i] = b.get("rest_n", 0.0)
        out["rest_t"][i] = b.get("rest_t", 0.0)
    out["body_scene"] = np.asarray(scene_ids if scene_ids is not None else np.zeros(N), np.int32)
    kinds = {"halfspace": 0, "drum": 1, "cylinder": 2, "box": 3}
    out["static_kind"] = np.array([kinds[s.get("kind", "halfspace")] for s in statics], np.int32)
    for k, d in (("static_pos", 3), ("static_vel", 3), ("static_omega", 3), ("static_dir", 3),
                 ("static_half_extents", 3)):
        out[k] = np.zeros((S, d))
    out["static_quat"] = np.tile(np.array([0.0, 0.0, 0.0, 1.0]), (S, 1)) if S else np.zeros((0, 4))
    for k in ("static_radius", "static_mu", "static_rest_n", "static_rest_t", "static_half_length"):
        out[k] = np.zeros(S)
    for i, s in enumerate(statics):
        out["static_pos"][i] = s["pos"]
        out["static_dir"][i] = s.get("dir", (0, 0, 1))
        out["static_vel"][i] = s.get("vel", (0, 0, 0))
        out["static_omega"][i] = s.get("omega", (0, 0, 0))
        if "quat" in s:
            out["static_quat"][i] = s["quat"]
        out["static_radius"][i] = s.get("radius", 0.0)
        out["static_half_length"][i] = s.get("half_length", 0.0)
        out["static_half_extents"][i] = s.get("half_extents", (0.0, 0.0, 0.0))
        out["static_mu"][i] = s.get("mu", 0.3)
        out["static_rest_n"][i] = s.get("rest_n", 0.0)
        out["static_rest_t"][i] = s.get("rest_t", 0.0)
    out["static_scene"] = np.asarray(static_scene_ids if static_scene_ids is not None else np.zeros(S), np.int32)
    out["num_scenes"] = int(max([0] + list(out["body_scene"]) + list(out["static_scene"]))) + 1
    return out
