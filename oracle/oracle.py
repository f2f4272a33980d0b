"""ctypes binding for the CPU oracle (test infrastructure only).

The oracle is a plain C++ FP64 restatement of CardilloCxx's Moreau midpoint step for sphere
scenes (see cdx_oracle.cpp for the file:line citations). Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline leg import this module; the product package never does.

Parity status: unpinned (the reference cannot be built here and ships no golden vectors).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no FMA contraction, OpenMP). Rebuilt unless the library carries
    a stamp equal to the digest of its sources, command and machine (file times are not trusted)."""
    import hashlib
    import platform
    srcs = [os.path.join(HERE, "cdx_oracle.cpp"), os.path.join(HERE, "cdx_adjoint.cpp")]
    hdr = os.path.join(HERE, "cdx_oracle.h")
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           "-fno-fast-math", *srcs, "-o", LIB]
    h = hashlib.sha256((" ".join(cmd) + platform.machine()).encode())
    for f in srcs + [hdr]:
        with open(f, "rb") as fh:
            h.update(fh.read())
    stamp = h.hexdigest()
    if not force and os.path.exists(LIB) and os.path.exists(LIB + ".stamp"):
        with open(LIB + ".stamp") as fh:
            if fh.read().strip() == stamp:
                return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".{os.getpid()}.tmp"
    subprocess.check_call([tmp if c == LIB else c for c in cmd])
    os.replace(tmp, LIB)
    with open(LIB + ".stamp", "w") as fh:
        fh.write(stamp + "\n")
    return LIB


class OrConfig(C.Structure):
    _fields_ = [
        ("sim_dt", C.c_double),
        ("sim_gravity", C.c_double * 3),
        ("moreau_theta", C.c_double),
        ("friction_enable", C.c_int32),
        ("friction_combine", C.c_int32),
        ("pj_max_iterations", C.c_int32),
        ("pj_warmstart", C.c_int32),
        ("pj_tol_abs", C.c_double),
        ("pj_tol_rel", C.c_double),
        ("pj_alpha", C.c_double),
        ("collision_security_margin", C.c_double),
        ("collision_match_max_dist", C.c_double),
        ("residual_tol", C.c_double),
        ("omp_mode", C.c_int32),
        ("num_threads", C.c_int32),
        ("pj_nesterov", C.c_int32),
        ("pj_nesterov_beta_threshold", C.c_double),
        ("pj_nesterov_restart_limit", C.c_int32),
        ("pj_chebyshev", C.c_int32),
        ("pj_anderson", C.c_int32),
        ("pj_anderson_m", C.c_int32),
        ("pj_rdiag_true_delassus", C.c_int32),
        ("moreau_implicit_gyroscopy", C.c_int32),
        ("solver_type", C.c_int32),
        ("condensed_sweep_mode", C.c_int32),
        ("pj_relaxation", C.c_double),
        ("pad0", C.c_int32),
        ("status", C.c_int32),
    ]


_P = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int32)


class OrScene(C.Structure):
    _fields_ = [
        ("num_bodies", C.c_int32),
        ("pos", _P), ("quat", _P), ("vel", _P), ("omega", _P),
        ("radius", _P), ("mass", _P), ("inertia", _P), ("mu", _P), ("rest_n", _P), ("rest_t", _P),
        ("body_scene", _PI),
        ("num_statics", C.c_int32),
        ("static_kind", _PI),
        ("static_pos", _P), ("static_quat", _P), ("static_vel", _P), ("static_omega", _P),
        ("static_dir", _P), ("static_radius", _P),
        ("static_mu", _P), ("static_rest_n", _P), ("static_rest_t", _P),
        ("static_scene", _PI),
        ("num_scenes", C.c_int32),
        ("static_half_length", _P),
        ("static_half_extents", _P),
    ]


class OrStats(C.Structure):
    _fields_ = [
        ("num_contacts", C.c_int32),
        ("num_rows", C.c_int32),
        ("iterations", C.c_int32),
        ("residual", C.c_double),
        ("residual_last", C.c_double),
    ]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(build())
            L.or_create.restype = C.c_void_p
            L.or_create.argtypes = [C.POINTER(OrConfig), C.POINTER(OrScene)]
            L.or_destroy.argtypes = [C.c_void_p]
            L.or_step.restype = C.c_int
            L.or_step.argtypes = [C.c_void_p, C.c_int32]
            L.or_get_state.argtypes = [C.c_void_p, _P, _P, _P, _P]
            L.or_get_stats.argtypes = [C.c_void_p, C.POINTER(OrStats)]
            L.or_get_contacts.restype = C.c_int32
            L.or_get_contacts.argtypes = [C.c_void_p, _PI, _PI, _P, _P, _P]
            L.or_set_trace.argtypes = [C.c_void_p, C.c_int32]
            L.or_set_contacts.argtypes = [C.c_void_p, C.c_int32, _PI, _PI, _P, _P]
            L.or_set_static_motion.argtypes = [C.c_void_p, C.c_int32, _PI, _P, _P, _P, _P]
            L.or_get_static_state.argtypes = [C.c_void_p, _P, _P, _P, _P]
            L.or_get_trace.restype = C.c_int32
            L.or_get_trace.argtypes = [C.c_void_p, _P, C.c_int64]
            L.or_pj_solve_csr.restype = C.c_int32
            L.or_pj_solve_csr.argtypes = [C.c_int32, C.c_int32, C.c_int32, _PI, _PI, _P, _P, _P, _P, _P, _P,
                                          _P, _P, _P, C.c_double, C.c_double, C.c_int32, C.c_double,
                                          C.c_double, _P, _P]
            L.or_pj_solve_csr_cfg.restype = C.c_int32
            L.or_pj_solve_csr_cfg.argtypes = [C.POINTER(OrConfig), C.c_int32, C.c_int32, C.c_int32, _PI, _PI, _P, _P,
                                              _P, _P, _P, _P, _P, _P, _P, C.c_double, _P, _P]
            L.or_block_inverse.restype = C.c_int32
            L.or_block_inverse.argtypes = [_P, C.c_int32, _P]
            _lib = L
    return _lib


def block_inverse(A):
    """(inverse, counts_as_diagonal) of a small SPD block as the pj.rdiag_true_delassus setup makes it."""
    A = np.ascontiguousarray(np.asarray(A, np.float64))
    n = A.shape[0]
    X = np.zeros((n, n))
    d = lib().or_block_inverse(_dp(A), n, _dp(X))
    if d < 0:
        raise ValueError("block size must be 1..3")
    return X, bool(d)


def _dp(a):
    return a.ctypes.data_as(_P) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(_PI) if a is not None else None


def config_from(cfg: dict, omp_mode: int = 0, num_threads: int = 0) -> OrConfig:
    """Build the oracle config from the same dict of reference keys the product uses."""
    c = OrConfig()
    c.sim_dt = float(cfg.get("sim.dt", 1e-3))
    g = cfg.get("sim.gravity", (0.0, 0.0, -9.81))
    for k in range(3):
        c.sim_gravity[k] = float(g[k])
    c.moreau_theta = float(cfg.get("moreau.theta", 1.0))
    c.friction_enable = int(bool(cfg.get("friction.enable", False)))
    c.friction_combine = {"min": 0, "arith": 1, "geom": 2}[cfg.get("friction.combine", "min")]
    c.pj_max_iterations = int(cfg.get("pj.max_iterations", 200000))
    c.pj_warmstart = int(bool(cfg.get("pj.warmstart", True)))
    c.pj_tol_abs = float(cfg.get("pj.tol_abs", 1e-5))
    c.pj_tol_rel = float(cfg.get("pj.tol_rel", 1e-5))
    c.pj_alpha = float(cfg.get("pj.alpha", 0.3))
    c.collision_security_margin = float(cfg.get("collision.security_margin", 0.0))
    c.collision_match_max_dist = float(cfg.get("collision.match_max_dist", 0.02))
    c.residual_tol = float(cfg.get("gpu.residual_tol", 0.0))
    c.pj_nesterov = int(bool(cfg.get("pj.nesterov", False)))
    c.pj_nesterov_beta_threshold = float(cfg.get("pj.nesterov_beta_threshold", 1.0))
    c.pj_nesterov_restart_limit = int(cfg.get("pj.nesterov_restart_limit", 10000))
    c.pj_chebyshev = int(bool(cfg.get("pj.chebyshev", False)))
    c.pj_anderson = int(bool(cfg.get("pj.anderson", False)))
    c.pj_anderson_m = int(cfg.get("pj.anderson_m", 2))
    c.pj_rdiag_true_delassus = int(bool(cfg.get("pj.rdiag_true_delassus", False)))
    c.moreau_implicit_gyroscopy = int(bool(cfg.get("moreau.implicit_gyroscopy", False)))
    c.solver_type = {"projected_jacobi": 0, "condensed": 1, "projected_gauss_seidel": 2, "pgs": 2}[
        str(cfg.get("solver.type", "projected_jacobi"))]
    c.condensed_sweep_mode = {"gauss_seidel": 0, "jacobi": 1, "colored": 2, "chaotic": 3}[
        str(cfg.get("condensed.sweep_mode", "gauss_seidel"))]
    c.pj_relaxation = float(cfg.get("pj.relaxation", 1.0))
    c.omp_mode = omp_mode
    c.num_threads = num_threads
    return c


class Oracle:
    """CPU FP64 engine over a scene dict (numpy arrays, see cardillocxx_gb300.scenes)."""

    def __init__(self, scene: dict, cfg: dict, omp_mode: int = 0, num_threads: int = 0):
        self.L = lib()
        self._keep = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v) for k, v in scene.items()}
        s = self._keep
        sc = OrScene()
        sc.num_bodies = int(s["pos"].shape[0])
        for name in ("pos", "quat", "vel", "omega", "radius", "mass", "inertia", "mu", "rest_n", "rest_t"):
            setattr(sc, name, _dp(s[name]))
        sc.body_scene = _ip(s.get("body_scene"))
        sc.num_statics = int(s["static_kind"].shape[0])
        sc.static_kind = _ip(s["static_kind"])
        for name in ("static_pos", "static_quat", "static_vel", "static_omega", "static_dir", "static_radius",
                     "static_mu", "static_rest_n", "static_rest_t"):
            setattr(sc, name, _dp(s[name]))
        sc.static_scene = _ip(s.get("static_scene"))
        sc.num_scenes = int(s.get("num_scenes", 1))
        if "static_half_length" in s:
            sc.static_half_length = _dp(s["static_half_length"])
        if "static_half_extents" in s:
            sc.static_half_extents = _dp(s["static_half_extents"])
        self.cfg = config_from(cfg, omp_mode, num_threads)
        self.h = self.L.or_create(C.byref(self.cfg), C.byref(sc))
        self.N = sc.num_bodies

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.L.or_destroy(h)
            self.h = None

    def step(self, n: int = 1):
        st = self.L.or_step(self.h, int(n))
        if st:
            raise RuntimeError(f"oracle step failed with status {st} (a solve diverged)")

    def state(self):
        N = self.N
        pos = np.empty((N, 3)); quat = np.empty((N, 4)); vel = np.empty((N, 3)); om = np.empty((N, 3))
        self.L.or_get_state(self.h, _dp(pos), _dp(quat), _dp(vel), _dp(om))
        return {"pos": pos, "quat": quat, "vel": vel, "omega": om}

    def stats(self) -> dict:
        st = OrStats()
        self.L.or_get_stats(self.h, C.byref(st))
        return {k: getattr(st, k) for k, _ in OrStats._fields_}

    def contacts(self):
        n = self.L.or_get_contacts(self.h, None, None, None, None, None)
        ia = np.empty(n, np.int32); ib = np.empty(n, np.int32)
        pt = np.empty((n, 3)); lam = np.empty((n, 3)); nrm = np.empty((n, 3))
        self.L.or_get_contacts(self.h, _ip(ia), _ip(ib), _dp(pt), _dp(lam), _dp(nrm))
        return {"id_a": ia, "id_b": ib, "point": pt, "lambda": lam, "normal": nrm}

    def set_contacts(self, contacts: dict):
        """Warm-start memory of the next step (id_a, id_b, point, lambda)."""
        ia = np.ascontiguousarray(contacts["id_a"], np.int32)
        ib = np.ascontiguousarray(contacts["id_b"], np.int32)
        pt = np.ascontiguousarray(contacts["point"], np.float64).reshape(-1, 3)
        lam = np.ascontiguousarray(contacts["lambda"], np.float64).reshape(-1, 3)
        self.L.or_set_contacts(self.h, int(ia.shape[0]), _ip(ia), _ip(ib), _dp(pt), _dp(lam))
        return self

    def set_static_motion(self, statics, pos=None, quat=None, vel=None, omega=None):
        """Prescribed pose/twist of the listed statics for the next step (Trajectory::update)."""
        idx = np.ascontiguousarray(np.atleast_1d(statics), np.int32)
        n = idx.shape[0]
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64).reshape(n, w)
                for a, w in ((pos, 3), (quat, 4), (vel, 3), (omega, 3))]
        self._motion = arrs
        self.L.or_set_static_motion(self.h, n, _ip(idx), *[None if a is None else _dp(a) for a in arrs])
        return self

    def static_state(self):
        S = int(self._keep["static_kind"].shape[0])
        out = {"pos": np.empty((S, 3)), "quat": np.empty((S, 4)), "vel": np.empty((S, 3)), "omega": np.empty((S, 3))}
        self.L.or_get_static_state(self.h, _dp(out["pos"]), _dp(out["quat"]), _dp(out["vel"]), _dp(out["omega"]))
        return out

    def set_trace(self, on: bool = True):
        self.L.or_set_trace(self.h, int(on))

    def trace(self, nrows: int):
        n = self.L.or_get_trace(self.h, None, 0)
        out = np.empty(n)
        self.L.or_get_trace(self.h, _dp(out), n)
        return out.reshape(-1, nrows) if nrows else out


def pj_solve_csr_cfg(cfg: dict, row_ptr, col, val, contact_bias, mu, restitution, minv, mdiag, v, f_ext, f_gyro, dt,
                     lam0, nfl=0):
    """Oracle for the solver-level drop-in with a configuration (the keys of the engine's config)."""
    L = lib()
    c = config_from(cfg)
    row_ptr = np.ascontiguousarray(row_ptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    arrs = [np.ascontiguousarray(a, np.float64) for a in (val, contact_bias, mu, restitution, minv, mdiag, v,
                                                          f_ext, f_gyro)]
    nrows = row_ptr.shape[0] - 1
    nv = arrs[4].shape[0]
    lam = np.array(lam0, np.float64, copy=True)
    x = np.empty(nv)
    it = L.or_pj_solve_csr_cfg(C.byref(c), nrows, nv, int(nfl), _ip(row_ptr), _ip(col), *[_dp(a) for a in arrs],
                               float(dt), _dp(lam), _dp(x))
    return x, lam, it


def pj_solve_csr(row_ptr, col, val, contact_bias, mu, restitution, minv, mdiag, v, f_ext, f_gyro, dt, alpha,
                 max_iter, tol_abs, tol_rel, lam0, nfl=0):
    """Oracle for the solver-level drop-in (ProjectedJacobiSolver::solve, S = diag(M))."""
    L = lib()
    row_ptr = np.ascontiguousarray(row_ptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    arrs = [np.ascontiguousarray(a, np.float64) for a in (val, contact_bias, mu, restitution, minv, mdiag, v,
                                                          f_ext, f_gyro)]
    nrows = row_ptr.shape[0] - 1
    nv = arrs[4].shape[0]
    lam = np.array(lam0, np.float64, copy=True)
    x = np.empty(nv)
    it = L.or_pj_solve_csr(nrows, nv, int(nfl), _ip(row_ptr), _ip(col), *[_dp(a) for a in arrs], float(dt),
                           float(alpha), int(max_iter), float(tol_abs), float(tol_rel), _dp(lam), _dp(x))
    return x, lam, it


# ---- FP64 CPU adjoint of the world-frame sphere step (cdx_adjoint.cpp)
class OrAdjProblem(C.Structure):
    _fields_ = [
        ("num_bodies", C.c_int32),
        ("radius", _P), ("mass", _P), ("inertia", _P),
        ("body_scene", _PI),
        ("num_scenes", C.c_int32),
        ("num_statics", C.c_int32),
        ("static_dir", _P), ("static_pos", _P),
        ("static_scene", _PI),
        ("dt", C.c_double),
        ("gravity", C.c_double * 3),
        ("theta", C.c_double),
        ("alpha", C.c_double),
        ("iterations", C.c_int32),
        ("margin", C.c_double),
    ]


def _adj_lib():
    L = lib()
    if not getattr(L, "_adj_ready", False):
        L.or_adj_create.restype = C.c_void_p
        L.or_adj_create.argtypes = [C.POINTER(OrAdjProblem)]
        L.or_adj_destroy.argtypes = [C.c_void_p]
        L.or_adj_rollout.restype = C.c_int32
        L.or_adj_rollout.argtypes = [C.c_void_p, C.c_int32, _P, _P, _P, _P, _P, _P, _P]
        L.or_adj_gradient.restype = C.c_int32
        L.or_adj_gradient.argtypes = [C.c_void_p, C.c_int32, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]
        L._adj_ready = True
    return L


class AdjOracle:
    """FP64 CPU rollout and adjoint of the world-frame sphere step (halfspaces only, lambda_0 = 0,
    fixed sweep count, per-scene friction coefficient)."""

    def __init__(self, scene: dict, cfg: dict):
        kinds = np.asarray(scene.get("static_kind", np.zeros(0, np.int32)))
        if kinds.size and np.any(kinds != 0):
            raise ValueError("the adjoint model covers halfspaces only")
        N = scene["pos"].shape[0]
        S = kinds.size
        self._keep = []

        def arr(a, dt=np.float64):
            a = np.ascontiguousarray(a, dt)
            self._keep.append(a)
            return a

        p = OrAdjProblem()
        p.num_bodies = N
        p.radius = _dp(arr(scene["radius"]))
        p.mass = _dp(arr(scene["mass"]))
        p.inertia = _dp(arr(scene["inertia"]))
        bs = scene.get("body_scene")
        p.body_scene = _ip(arr(bs, np.int32)) if bs is not None else None
        self.num_scenes = int(scene.get("num_scenes", 1))
        p.num_scenes = self.num_scenes
        p.num_statics = S
        p.static_dir = _dp(arr(scene["static_dir"])) if S else None
        p.static_pos = _dp(arr(scene["static_pos"])) if S else None
        ss = scene.get("static_scene")
        p.static_scene = _ip(arr(ss, np.int32)) if (S and ss is not None) else None
        p.dt = float(cfg.get("sim.dt", 1e-3))
        g = cfg.get("sim.gravity", (0.0, 0.0, -9.81))
        for k in range(3):
            p.gravity[k] = float(g[k])
        p.theta = float(cfg.get("moreau.theta", 1.0))
        p.alpha = float(cfg.get("pj.alpha", 0.3))
        p.iterations = int(cfg.get("pj.max_iterations", 50))
        p.margin = float(cfg.get("collision.security_margin", 0.0))
        self.N = N
        self._p = p
        self.L = _adj_lib()
        self.h = self.L.or_adj_create(C.byref(p))
        if not self.h:
            raise ValueError("or_adj_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            self.L.or_adj_destroy(self.h)
            self.h = None

    def rollout(self, nsteps, x0, v0, w0, mu):
        x0, v0, w0 = (np.ascontiguousarray(a, np.float64).reshape(self.N, 3) for a in (x0, v0, w0))
        mu = np.ascontiguousarray(np.broadcast_to(mu, (self.num_scenes,)), np.float64)
        out = [np.empty((self.N, 3)) for _ in range(3)]
        self.L.or_adj_rollout(self.h, int(nsteps), _dp(x0), _dp(v0), _dp(w0), _dp(mu), *[_dp(o) for o in out])
        return tuple(out)

    def gradient(self, nsteps, x0, v0, w0, mu, gxT, gvT, gwT):
        x0, v0, w0, gxT, gvT, gwT = (np.ascontiguousarray(a, np.float64).reshape(self.N, 3)
                                     for a in (x0, v0, w0, gxT, gvT, gwT))
        mu = np.ascontiguousarray(np.broadcast_to(mu, (self.num_scenes,)), np.float64)
        out = [np.empty((self.N, 3)) for _ in range(3)]
        gmu = np.empty(self.num_scenes)
        self.L.or_adj_gradient(self.h, int(nsteps), _dp(x0), _dp(v0), _dp(w0), _dp(mu), _dp(gxT), _dp(gvT),
                               _dp(gwT), *[_dp(o) for o in out], _dp(gmu))
        return out[0], out[1], out[2], gmu
