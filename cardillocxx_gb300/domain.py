"""Spatial decomposition of one pile across ranks: the host-side plan of a projected Jacobi solve
whose ranks exchange halo bodies once per sweep.

A single pile does not split into independent scenes: every sweep needs the velocities of the
bodies that a rank's contacts touch, and every body collects the impulses of all its contacts.
This module is the plan for running the projected Jacobi solve of `ProjectedJacobiSolver`
(projected_jacobi.cpp:121-144, 316-377; the solver-level problem of `cdx_pj_solve_csr`) on
`world` ranks, one per GPU, written as host code that runs on CPU ranks (gloo) here:

- **Bodies** are ordered along the pile's longest axis (by grid slab, then index) and cut into
  `world` slabs of equal body count (`slab_owner`).
- **Contacts** (a frictionless row, or the three rows of a frictional contact) belong to the rank
  that owns their higher-indexed body. A rank's *ghosts* are the other ranks' bodies that its
  contacts touch.
- **Per sweep** each rank: (1) computes its contacts' impulses from the velocities of its own and
  its ghost bodies; (2) sends every W^T dlambda term that lands on another rank's body to that
  rank, as (row, column) terms, not pre-summed; (3) adds all terms of its own bodies in global row
  order, exactly the order of the single-process gather, so the velocities are bit-identical to
  the unsplit solve; (4) sends its updated boundary velocities to the ranks that ghost them.
- **The stop test** (every 10th sweep) adds each rank's share of the scaled velocity increments,
  then the shares in rank order on every rank, so all ranks stop together. Its rounding differs
  from one sequential sum only when the residual lands within rounding of 1.

Exchanges are point-to-point (`isend`/`irecv` between neighbouring slabs) through
torch.distributed: gloo on CPU here, NCCL on GPUs. With one GPU per box this path is exercised on
CPU ranks only; the per-rank sweep on a GPU would be the engine's sweep kernels over the rank's
rows, with the halo terms packed and unpacked around them.
"""
from __future__ import annotations

import numpy as np


def slab_owner(pos: np.ndarray, world: int, cell: float | None = None) -> np.ndarray:
    """Rank owning each body: slabs of equal body count along the longest axis of the pile."""
    pos = np.asarray(pos, np.float64)
    n = pos.shape[0]
    if world < 1:
        raise ValueError("world must be >= 1")
    if n == 0:
        return np.zeros(0, np.int32)
    ext = pos.max(0) - pos.min(0)
    ax = int(np.argmax(ext))
    cell = float(cell) if cell else max(float(ext[ax]) / max(1, 4 * world), 1e-12)
    key = np.floor((pos[:, ax] - pos[:, ax].min()) / cell).astype(np.int64)
    order = np.lexsort((np.arange(n), key))
    owner = np.empty(n, np.int32)
    owner[order] = (np.arange(n) * world) // n
    return owner


def row_bodies(ptr: np.ndarray, col: np.ndarray) -> np.ndarray:
    """The higher-indexed body of every row (rows of one contact share their columns)."""
    return (np.asarray(col)[np.asarray(ptr)[1:] - 1] // 6).astype(np.int64)


class PileDomain:
    """One rank's share of a split projected Jacobi solve over CSR rows (W: rows x 6 N)."""

    def __init__(self, ptr, col, nfl: int, owner, rank: int, world: int):
        self.ptr = np.asarray(ptr, np.int64)
        self.col = np.asarray(col, np.int64)
        self.nfl = int(nfl)
        self.owner = np.asarray(owner, np.int32)
        self.rank, self.world = int(rank), int(world)
        nrows = len(self.ptr) - 1
        self.nrows = nrows
        row_owner = self.owner[row_bodies(self.ptr, self.col)] if nrows else np.zeros(0, np.int32)
        self.rows = np.nonzero(row_owner == self.rank)[0]
        self.owned = np.nonzero(self.owner == self.rank)[0]
        # every (row, entry) of the local rows, with its body and that body's owner
        starts, ends = self.ptr[self.rows], self.ptr[self.rows + 1]
        self.k = np.concatenate([np.arange(s, e) for s, e in zip(starts, ends)]) if len(self.rows) else \
            np.zeros(0, np.int64)
        self.k_row = np.repeat(self.rows, ends - starts)
        kb = self.col[self.k] // 6
        kown = self.owner[kb]
        bodies = np.unique(kb)
        self.ghosts = bodies[self.owner[bodies] != self.rank]
        # halo velocities: ghosts owned by r arrive from r; r's ghosts among my bodies go to r
        self.recv_x = {r: self.ghosts[self.owner[self.ghosts] == r] for r in range(world) if r != self.rank}
        # W^T terms: entries of my rows on r's bodies go to r (in row order)
        self.send_terms = {r: np.nonzero(kown == r)[0] for r in range(world) if r != self.rank}
        self.own_terms = np.nonzero(kown == self.rank)[0]
        self.plan_sizes = None  # exchanged in `connect`

    def connect(self, dist=None):
        """Exchange the plan's sizes and ids with the other ranks (once per contact set)."""
        import torch

        w, me = self.world, self.rank
        self.send_x = {}
        self.recv_terms = {}
        if dist is None or w == 1:
            return self
        reqs, bufs = [], {}
        for r in range(w):
            if r == me:
                continue
            n_out = torch.tensor([len(self.recv_x[r]), len(self.send_terms[r])], dtype=torch.int64)
            n_in = torch.zeros(2, dtype=torch.int64)
            reqs.append(dist.isend(n_out, r))
            reqs.append(dist.irecv(n_in, r))
            bufs[r] = n_in
        for q in reqs:
            q.wait()
        reqs, ids = [], {}
        for r in range(w):
            if r == me:
                continue
            nx, nt = (int(v) for v in bufs[r])
            # my requested ghost ids to r; r's requested ids from me
            reqs.append(dist.isend(torch.from_numpy(self.recv_x[r].astype(np.int64)), r, tag=1))
            want = torch.zeros(nx, dtype=torch.int64)
            reqs.append(dist.irecv(want, r, tag=1))
            # (row, column) of the terms I send to r; those r sends to me
            t = self.send_terms[r]
            reqs.append(dist.isend(torch.from_numpy(np.stack([self.k_row[t], self.col[self.k[t]]]).astype(np.int64)
                                                    .reshape(-1).copy()), r, tag=2))
            rt = torch.zeros(2 * nt, dtype=torch.int64)
            reqs.append(dist.irecv(rt, r, tag=2))
            ids[r] = (want, rt, nt)
        for q in reqs:
            q.wait()
        for r, (want, rt, nt) in ids.items():
            self.send_x[r] = want.numpy()
            rt = rt.numpy().reshape(2, nt)
            self.recv_terms[r] = (rt[0], rt[1])
        return self

    def _exchange(self, dist, out: dict, sizes: dict):
        import torch

        reqs, got = [], {}
        for r, arr in out.items():
            reqs.append(dist.isend(torch.from_numpy(np.ascontiguousarray(arr, np.float64)), r, tag=3))
        for r, n in sizes.items():
            got[r] = torch.zeros(n, dtype=torch.float64)
            reqs.append(dist.irecv(got[r], r, tag=3))
        for q in reqs:
            q.wait()
        return {r: t.numpy() for r, t in got.items()}

    def _gather_wt(self, y_rows: np.ndarray, val: np.ndarray, dist, init=None) -> np.ndarray:
        """init_j + sum_r W_rj y_r for my bodies' columns, added one term at a time in global row
        order (the order of the single-process gather)."""
        nv = 6 * len(self.owner)
        terms = val[self.k] * y_rows[self.k_row]
        rows = [self.k_row[self.own_terms]]
        cols = [self.col[self.k[self.own_terms]]]
        vals = [terms[self.own_terms]]
        if dist is not None and self.world > 1:
            got = self._exchange(dist, {r: terms[t] for r, t in self.send_terms.items()},
                                 {r: len(rc[0]) for r, rc in self.recv_terms.items()})
            for r in sorted(got):
                rows.append(self.recv_terms[r][0])
                cols.append(self.recv_terms[r][1])
                vals.append(got[r])
        rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
        order = np.argsort(rows, kind="stable")
        acc = np.zeros(nv) if init is None else np.array(init, np.float64)
        np.add.at(acc, cols[order], vals[order])  # unbuffered: sequential in row order per column
        return acc

    def _halo(self, x: np.ndarray, dist):
        """Refresh the ghost bodies' six velocity components from their owners."""
        if dist is None or self.world == 1:
            return
        out = {r: x[(6 * ids[:, None] + np.arange(6)).reshape(-1)] for r, ids in self.send_x.items()}
        got = self._exchange(dist, out, {r: 6 * len(ids) for r, ids in self.recv_x.items()})
        for r, vals in got.items():
            x[(6 * self.recv_x[r][:, None] + np.arange(6)).reshape(-1)] = vals

    def solve(self, val, contact_bias, mu, restitution, minv, mdiag, v, f_ext, f_gyro, dt, alpha, max_iter,
              tol_abs, tol_rel, lam0, dist=None):
        """The standard loop of ProjectedJacobiSolver over this rank's rows. Inputs are the global
        arrays (each rank reads its part); returns the velocities (valid on my bodies and ghosts),
        the impulses of my rows (global row numbering, others zero) and the sweep count."""
        val = np.asarray(val, np.float64)
        nv = 6 * len(self.owner)
        ptr, col, rows = self.ptr, self.col, self.rows
        mine = np.zeros(nv, bool)
        mine[(6 * self.owned[:, None] + np.arange(6)).reshape(-1)] = True
        # PjAssembler::rhs (pj_assembler.cpp:152-153)
        rhs = (mdiag * v + dt * f_ext) + dt * f_gyro
        # build_workspace + rdiag_sparse (projected_jacobi.cpp:316-369, 57-69) for my rows
        width = int((ptr[rows + 1] - ptr[rows]).max()) if len(rows) else 0
        K = np.full((len(rows), width), -1, np.int64)
        for j in range(width):
            kk = ptr[rows] + j
            K[:, j] = np.where(kk < ptr[rows + 1], kk, -1)
        valid = K >= 0
        Kc = np.where(valid, K, 0)
        W = np.where(valid, val[Kc], 0.0)
        C = np.where(valid, col[Kc], 0)

        def rowdot(coef, vec):
            t = np.zeros(len(rows))
            for j in range(width):
                t = np.where(valid[:, j], t + coef[:, j] * vec[C[:, j]], t)
            return t

        vp = rowdot(W, v) + contact_bias[rows]
        bias = contact_bias[rows] + restitution[rows] * vp
        D = np.zeros(len(rows))
        for j in range(width):
            D = np.where(valid[:, j], D + (W[:, j] * W[:, j]) * minv[C[:, j]], D)
        R = np.where(D > 0.0, alpha / np.where(D > 0.0, D, 1.0), 0.0)
        RW = R[:, None] * W
        biasR = R * bias
        lam = np.zeros(self.nrows)
        lam[rows] = lam0[rows]
        # warm start: x0 = S^-1 (rhs + W^T p)
        rhs = self._gather_wt(lam, val, dist, init=rhs)
        x = np.where(mine, rhs / mdiag, 0.0)
        self._halo(x, dist)
        fr = rows >= self.nfl
        blk = np.nonzero(fr)[0]
        heads = blk[(rows[blk] - self.nfl) % 3 == 0]
        maxit = max(1, int(max_iter))
        it = 0
        for it in range(maxit):
            xprev = x.copy()
            g = rowdot(RW, x) + biasR
            lold = lam[rows].copy()
            lnew = lold - g
            # project (projected_jacobi.cpp:100-119)
            lnew[~fr] = np.maximum(lnew[~fr], 0.0)
            n0 = lnew[heads]
            n0 = np.maximum(n0, 0.0)
            t1, t2 = lnew[heads + 1], lnew[heads + 2]
            tn2 = t1 * t1 + t2 * t2
            pos = tn2 > 0
            s = np.where(pos, np.minimum(1.0, (mu[rows[heads]] * n0) / np.sqrt(np.where(pos, tn2, 1.0))), 1.0)
            lnew[heads] = n0
            lnew[heads + 1] = np.where(pos, s * t1, t1)
            lnew[heads + 2] = np.where(pos, s * t2, t2)
            dlam = np.zeros(self.nrows)
            dlam[rows] = lnew - lold
            lam[rows] = lnew
            acc = self._gather_wt(dlam, val, dist)
            x = np.where(mine, x + acc / mdiag, x)
            self._halo(x, dist)
            if it % 10 == 0:
                q = np.maximum(np.abs(x), np.abs(xprev)) * tol_rel + tol_abs
                with np.errstate(divide="ignore", invalid="ignore"):
                    d = (x - xprev) / np.where(mine, q, 1.0)
                part = 0.0
                for j in np.nonzero(mine)[0]:
                    part = part + d[j] * d[j]
                total = part
                if dist is not None and self.world > 1:
                    import torch

                    parts = [torch.zeros(1, dtype=torch.float64) for _ in range(self.world)]
                    dist.all_gather(parts, torch.tensor([part], dtype=torch.float64))
                    total = 0.0
                    for p in parts:
                        total = total + float(p[0])
                if 1.0 / np.sqrt(nv) * np.sqrt(total) <= 1:
                    break
        return x, lam, it + 1
