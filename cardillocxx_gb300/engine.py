"""Host-side mirror of the reference's engine interface for the contact path.

`Config` keeps the reference's key=value keys (ConfigReader::fromFile, src/config/config.cpp:22-420);
parsing happens in C++ (cdx_config_set) so the semantics are the library's. `PhysicsEngine`
wraps one cdx context: load a scene, `step()` (MoreauIntegrator::step, moreau.cpp:6-13), read
the state back. `pj_solve_csr` is the solver-level drop-in (ProjectedJacobiSolver::solve,
projected_jacobi.cpp:451-500). Every call goes to the CUDA library; nothing here computes physics.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import CdxConfig, CdxError, CdxScene, CdxStats, dp, ip


class Config:
    """Reference-compatible configuration (pj.*, moreau.*, friction.*, collision.*, sim.*, gpu.*)."""

    def __init__(self, values: dict | None = None):
        self._c = CdxConfig()
        _lib.lib().cdx_config_default(C.byref(self._c))
        for k, v in (values or {}).items():
            self.set(k, v)

    @classmethod
    def from_file(cls, path: str) -> "Config":
        cfg = cls()
        st = _lib.lib().cdx_config_from_file(path.encode(), C.byref(cfg._c))
        if st:
            raise CdxError(st, f"config file {path}")
        return cfg

    def set(self, key: str, value) -> "Config":
        if isinstance(value, bool):
            value = "true" if value else "false"
        elif isinstance(value, (list, tuple)):
            value = " ".join(repr(float(v)) for v in value)
        elif isinstance(value, float):
            value = repr(value)
        st = _lib.lib().cdx_config_set(C.byref(self._c), str(key).encode(), str(value).encode())
        if st:
            raise CdxError(st, f"config key {key}={value}")
        return self

    @property
    def struct(self) -> CdxConfig:
        return self._c

    def get(self, field: str):
        v = getattr(self._c, field)
        return list(v) if field == "sim_gravity" else v

    def to_keys(self) -> dict:
        """Typed dict of the reference keys (used to configure the CPU oracle identically)."""
        c = self._c
        return {
            "sim.dt": c.sim_dt, "sim.gravity": tuple(c.sim_gravity), "moreau.theta": c.moreau_theta,
            "friction.enable": bool(c.friction_enable),
            "friction.combine": {0: "min", 1: "arith", 2: "geom"}[c.friction_combine],
            "pj.max_iterations": c.pj_max_iterations, "pj.warmstart": bool(c.pj_warmstart),
            "pj.tol_abs": c.pj_tol_abs, "pj.tol_rel": c.pj_tol_rel, "pj.alpha": c.pj_alpha,
            "collision.security_margin": c.collision_security_margin,
            "collision.match_max_dist": c.collision_match_max_dist, "gpu.residual_tol": c.gpu_residual_tol,
        }


def scene_struct(scene: dict) -> tuple[CdxScene, dict]:
    keep = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v) for k, v in scene.items()}
    s = CdxScene()
    s.num_bodies = int(keep["pos"].shape[0])
    for name in ("pos", "quat", "vel", "omega", "radius", "mass", "inertia", "mu", "rest_n", "rest_t"):
        arr = keep[name]
        assert arr.dtype == np.float64, name
        setattr(s, name, dp(arr))
    s.body_scene = ip(keep.get("body_scene"))
    s.num_statics = int(keep["static_kind"].shape[0])
    s.static_kind = ip(keep["static_kind"])
    for name in ("static_pos", "static_quat", "static_vel", "static_omega", "static_dir", "static_radius",
                 "static_mu", "static_rest_n", "static_rest_t"):
        setattr(s, name, dp(keep[name]))
    s.static_scene = ip(keep.get("static_scene"))
    s.num_scenes = int(keep.get("num_scenes", 1))
    if "static_half_length" in keep:
        s.static_half_length = dp(keep["static_half_length"])
    if "static_half_extents" in keep:
        s.static_half_extents = dp(keep["static_half_extents"])
    return s, keep


class PhysicsEngine:
    """One cdx context on the current CUDA device: the GPU Moreau midpoint step."""

    def __init__(self, cfg: Config | dict | None = None):
        if not isinstance(cfg, Config):
            cfg = Config(cfg or {})
        self.cfg = cfg
        self.L = _lib.lib()
        h = C.c_void_p()
        st = self.L.cdx_create(C.byref(cfg.struct), C.byref(h))
        self.h = h
        if st:
            msg = self.L.cdx_last_error(h).decode() if h else ""
            self.close()
            raise CdxError(st, msg)
        self.N = 0

    def _check(self, st: int):
        if st:
            raise CdxError(st, self.L.cdx_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.cdx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_config(self, cfg: "Config | dict"):
        """Replace the configuration from the next step on (gpu.precision stays as created)."""
        if not isinstance(cfg, Config):
            cfg = Config(cfg)
        self._check(self.L.cdx_set_config(self.h, C.byref(cfg.struct)))
        self.cfg = cfg
        return self

    def load_scene(self, scene: dict):
        s, keep = scene_struct(scene)
        self._check(self.L.cdx_load_scene(self.h, C.byref(s)))
        self.N = s.num_bodies
        self._nstatics = s.num_statics
        return self

    def step(self, n: int = 1):
        self._check(self.L.cdx_step(self.h, int(n)))

    def synchronize(self):
        self._check(self.L.cdx_synchronize(self.h))

    def set_timing(self, on: bool = True):
        self._check(self.L.cdx_set_timing(self.h, int(on)))

    def state(self) -> dict:
        N = self.N
        pos = np.empty((N, 3)); quat = np.empty((N, 4)); vel = np.empty((N, 3)); om = np.empty((N, 3))
        self._check(self.L.cdx_get_state(self.h, dp(pos), dp(quat), dp(vel), dp(om)))
        return {"pos": pos, "quat": quat, "vel": vel, "omega": om}

    def state_into(self, pos, quat, vel, omega):
        """Copy the state into caller-owned host arrays (e.g. pinned buffers); one D2H copy each."""
        for a in (pos, quat, vel, omega):
            assert a is None or (a.dtype == np.float64 and a.flags["C_CONTIGUOUS"])
        self._check(self.L.cdx_get_state(self.h, dp(pos), dp(quat), dp(vel), dp(omega)))

    def set_state(self, pos=None, quat=None, vel=None, omega=None):
        conv = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (pos, quat, vel, omega)]
        self._check(self.L.cdx_set_state(self.h, *[dp(a) for a in conv]))

    def stats(self) -> dict:
        st = CdxStats()
        self._check(self.L.cdx_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in CdxStats._fields_}

    def contacts(self) -> dict:
        n = C.c_int32(0)
        self._check(self.L.cdx_get_contacts(self.h, None, None, None, None, None, C.byref(n)))
        m = n.value
        ia = np.empty(m, np.int32); ib = np.empty(m, np.int32)
        pt = np.empty((m, 3)); lam = np.empty((m, 3)); nrm = np.empty((m, 3))
        self._check(self.L.cdx_get_contacts(self.h, ip(ia), ip(ib), dp(pt), dp(lam), dp(nrm), C.byref(n)))
        return {"id_a": ia, "id_b": ib, "point": pt, "lambda": lam, "normal": nrm}

    def set_contacts(self, contacts: dict):
        """Load the warm-start memory of the next step (id_a, id_b, point, lambda as contacts() gives)."""
        ia = np.ascontiguousarray(contacts["id_a"], np.int32)
        ib = np.ascontiguousarray(contacts["id_b"], np.int32)
        pt = np.ascontiguousarray(contacts["point"], np.float64).reshape(-1, 3)
        lam = np.ascontiguousarray(contacts["lambda"], np.float64).reshape(-1, 3)
        n = ia.shape[0]
        assert ib.shape[0] == n and pt.shape[0] == n and lam.shape[0] == n
        self._check(self.L.cdx_set_contacts(self.h, n, ip(ia), ip(ib), dp(pt), dp(lam)))
        return self

    def set_static_motion(self, statics, pos=None, quat=None, vel=None, omega=None):
        """Prescribed pose/twist of the listed statics for the next step (what Trajectory::update
        sets from a static's callbacks); None leaves that part as it is."""
        idx = np.ascontiguousarray(np.atleast_1d(statics), np.int32)
        n = idx.shape[0]

        def arr(a, w):
            if a is None:
                return None
            a = np.ascontiguousarray(a, np.float64).reshape(n, w)
            return a
        p, q, v, w = arr(pos, 3), arr(quat, 4), arr(vel, 3), arr(omega, 3)
        self._check(self.L.cdx_set_static_motion(self.h, n, ip(idx), *[None if a is None else dp(a) for a in (p, q, v, w)]))
        return self

    def static_state(self) -> dict:
        s = self._nstatics
        out = {"pos": np.empty((s, 3)), "quat": np.empty((s, 4)), "vel": np.empty((s, 3)), "omega": np.empty((s, 3))}
        self._check(self.L.cdx_get_static_state(self.h, dp(out["pos"]), dp(out["quat"]), dp(out["vel"]),
                                                dp(out["omega"])))
        return out

    def scene_solve(self, nscenes: int) -> dict:
        """Batched scenes (per-scene solve): each scene's alpha and its sweeps in its last solve."""
        a = np.empty(nscenes, np.float32)
        it = np.empty(nscenes, np.int32)
        self._check(self.L.cdx_get_scene_solve(self.h, a.ctypes.data_as(C.POINTER(C.c_float)), ip(it), nscenes))
        return {"alpha": a, "sweeps": it}

    def track(self, body: int, name: str):
        """Write sphere `body` to <output.folder>/<output.filename_prefix>_tracked.csv every step."""
        self._check(self.L.cdx_track(self.h, int(body), str(name).encode()))

    def flush_output(self):
        """Wait until the background writer has written every queued frame."""
        self._check(self.L.cdx_output_flush(self.h))

    def set_trace(self, on: bool = True):
        self._check(self.L.cdx_set_trace(self.h, int(on)))

    def trace(self, nrows: int):
        n = C.c_int64(0)
        self._check(self.L.cdx_get_trace(self.h, None, 0, C.byref(n)))
        out = np.empty(n.value)
        self._check(self.L.cdx_get_trace(self.h, dp(out), n.value, C.byref(n)))
        return out.reshape(-1, nrows) if nrows else out

    def time_sweeps(self, n: int = 20) -> dict:
        """Average per-launch time and algorithmic bytes of the sweep kernels (CUDA events)."""
        vals = [C.c_double(0) for _ in range(4)]
        self._check(self.L.cdx_time_sweeps(self.h, int(n), *[C.byref(v) for v in vals]))
        return {"ms_contact": vals[0].value, "ms_body": vals[1].value, "bytes_contact": vals[2].value,
                "bytes_body": vals[3].value}

    @staticmethod
    def split_variants() -> list:
        """Names of the split-form sweep launch shapes (index = gpu.sweep_variant)."""
        L = _lib.lib()
        return [L.cdx_split_variant_name(k).decode() for k in range(L.cdx_split_variant_count())]

    def selftest_nr64(self, x):
        """Device Newton-Raphson reciprocal / inverse square root of x (diagnostic)."""
        x = np.ascontiguousarray(x, np.float64)
        r = np.empty_like(x)
        q = np.empty_like(x)
        self._check(self.L.cdx_selftest_nr64(self.h, x.shape[0], dp(x), dp(r), dp(q)))
        return r, q

    def stream(self) -> int:
        return int(self.L.cdx_stream(self.h) or 0)

    def pj_solve_csr(self, row_ptr, col, val, contact_bias, mu, restitution, minv, mdiag, v, f_ext, f_gyro, dt,
                     alpha, max_iter, tol_abs, tol_rel, lam0, nfl=0):
        """Solver-level drop-in: ProjectedJacobiSolver::solve with S = diag(M) on host arrays."""
        row_ptr = np.ascontiguousarray(row_ptr, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        arrs = [np.ascontiguousarray(a, np.float64) for a in (val, contact_bias, mu, restitution, minv, mdiag, v,
                                                              f_ext, f_gyro)]
        nrows = row_ptr.shape[0] - 1
        nv = arrs[4].shape[0]
        lam = np.array(lam0, np.float64, copy=True)
        x = np.empty(nv)
        it = C.c_int32(0)
        self._check(self.L.cdx_pj_solve_csr(self.h, nrows, nv, int(nfl), ip(row_ptr), ip(col),
                                            *[dp(a) for a in arrs], float(dt), float(alpha), int(max_iter),
                                            float(tol_abs), float(tol_rel), dp(lam), dp(x), C.byref(it)))
        return x, lam, it.value

    def pj_solve_csr_cfg(self, cfg, row_ptr, col, val, contact_bias, mu, restitution, minv, mdiag, v, f_ext, f_gyro,
                         dt, lam0, nfl=0):
        """The solver-level drop-in under a configuration (loop, block preconditioner, stop rules)."""
        if not isinstance(cfg, Config):
            cfg = Config(cfg)
        row_ptr = np.ascontiguousarray(row_ptr, np.int32)
        col = np.ascontiguousarray(col, np.int32)
        arrs = [np.ascontiguousarray(a, np.float64) for a in (val, contact_bias, mu, restitution, minv, mdiag, v,
                                                              f_ext, f_gyro)]
        nrows = row_ptr.shape[0] - 1
        nv = arrs[4].shape[0]
        lam = np.array(lam0, np.float64, copy=True)
        x = np.empty(nv)
        it = C.c_int32(0)
        self._check(self.L.cdx_pj_solve_csr_cfg(self.h, C.byref(cfg.struct), nrows, nv, int(nfl), ip(row_ptr),
                                                ip(col), *[dp(a) for a in arrs], float(dt), dp(lam), dp(x),
                                                C.byref(it)))
        return x, lam, it.value
