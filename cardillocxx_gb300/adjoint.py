"""Differentiable rollout of sphere scenes: the GPU step and its hand-written adjoint (cdx_adj_*).

The reference has no adjoint; the map differentiated here is its Moreau midpoint step for sphere
scenes (MoreauIntegrator::step, src/physics/integration/moreau.cpp:6-13) with projected Jacobi
unrolled over its fixed sweep count (projected_jacobi.cpp:371-377), written on world-frame angular
velocities. `Rollout` wraps one cdx_adj context; `rollout` is a torch.autograd.Function over it
for checking gradients with torch (the arithmetic is in the CUDA library either way).

States are (N, 3) float64 arrays: positions x, velocities v, world-frame angular velocities w;
`mu` holds one friction coefficient per scene.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import CdxError, dp
from .engine import Config, scene_struct


class Rollout:
    """A differentiable rollout context: forward keeps checkpoints, backward recomputes from them."""

    def __init__(self, scene: dict, cfg: Config | dict, checkpoint_every: int = 20):
        if not isinstance(cfg, Config):
            cfg = Config(cfg)
        self.cfg = cfg
        self.L = _lib.lib()
        s, self._keep = scene_struct(scene)
        self.N = s.num_bodies
        self.num_scenes = s.num_scenes
        h = C.c_void_p()
        st = self.L.cdx_adj_create(C.byref(cfg.struct), C.byref(s), int(checkpoint_every), C.byref(h))
        self.h = h
        if st:
            msg = self.L.cdx_adj_last_error(h).decode() if h else ""
            self.close()
            raise CdxError(st, msg or "cdx_adj_create")
        self._last = None

    def _check(self, st):
        if st:
            raise CdxError(st, self.L.cdx_adj_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.cdx_adj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _arr(self, a, shape):
        return np.ascontiguousarray(np.asarray(a, np.float64).reshape(shape))

    def forward(self, nsteps: int, x0, v0, w0, mu):
        x0, v0, w0 = (self._arr(a, (self.N, 3)) for a in (x0, v0, w0))
        mu = self._arr(np.broadcast_to(np.asarray(mu, np.float64), (self.num_scenes,)), (self.num_scenes,))
        out = [np.empty((self.N, 3)) for _ in range(3)]
        self._check(self.L.cdx_adj_forward(self.h, int(nsteps), dp(x0), dp(v0), dp(w0), dp(mu), *[dp(o) for o in out]))
        return tuple(out)

    def backward(self, gxT, gvT, gwT):
        gxT, gvT, gwT = (self._arr(a, (self.N, 3)) for a in (gxT, gvT, gwT))
        out = [np.empty((self.N, 3)) for _ in range(3)]
        gmu = np.empty(self.num_scenes)
        self._check(self.L.cdx_adj_backward(self.h, dp(gxT), dp(gvT), dp(gwT), *[dp(o) for o in out], dp(gmu)))
        return out[0], out[1], out[2], gmu

    def contact_counts(self):
        """Per scene, the contacts of the last forward summed over its steps (an event signature)."""
        out = np.zeros(self.num_scenes, np.int64)
        self._check(self.L.cdx_adj_contact_counts(self.h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def info(self) -> dict:
        a, b, c = C.c_int64(0), C.c_int64(0), C.c_int32(0)
        self._check(self.L.cdx_adj_info(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return {"contact_slots": a.value, "device_bytes": b.value, "checkpoints": c.value}


def _function():
    import torch

    class RolloutFn(torch.autograd.Function):
        """(x0, v0, w0, mu) -> (xT, vT, wT) through cdx_adj_forward / cdx_adj_backward."""

        @staticmethod
        def forward(ctx, roll, nsteps, x0, v0, w0, mu):
            dev = x0.device
            xT, vT, wT = roll.forward(nsteps, *(t.detach().cpu().double().numpy() for t in (x0, v0, w0, mu)))
            ctx.roll = roll
            return tuple(torch.from_numpy(a).to(dev) for a in (xT, vT, wT))

        @staticmethod
        def backward(ctx, gxT, gvT, gwT):
            dev = gxT.device
            g = ctx.roll.backward(*(t.detach().cpu().double().numpy() for t in (gxT, gvT, gwT)))
            gx0, gv0, gw0, gmu = (torch.from_numpy(a).to(dev) for a in g)
            return None, None, gx0, gv0, gw0, gmu

    return RolloutFn


def rollout(roll: Rollout, nsteps: int, x0, v0, w0, mu):
    """torch.autograd entry: tensors in, (xT, vT, wT) out, differentiable in x0, v0, w0 and mu.
    One backward per forward: the backward replays the checkpoints of the latest forward call."""
    return _function().apply(roll, nsteps, x0, v0, w0, mu)
