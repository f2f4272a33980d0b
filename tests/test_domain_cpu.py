"""Spatial decomposition of one pile (host side): the slab partition, and the split projected
Jacobi solve on world_size-2 gloo ranks against the single-process solve of the oracle."""
import os
import socket

import numpy as np
import pytest

from cardillocxx_gb300.domain import PileDomain, slab_owner


def pile_problem(seed=3, nb=60):
    # a CSR contact problem with pile structure: bodies along x, contacts between neighbours
    # (frictional, three rows) and with the ground (one body), frictionless ones first
    rng = np.random.default_rng(seed)
    pos = np.column_stack([np.sort(rng.uniform(0, 6, nb)), rng.uniform(0, 1, nb), rng.uniform(0, 1, nb)])
    pairs = [(i, j) for i in range(nb) for j in range(i + 1, min(nb, i + 4)) if rng.uniform() < 0.6]
    ground = [(-1, i) for i in range(nb) if rng.uniform() < 0.3]
    fl = [(-1, i) for i in range(nb) if rng.uniform() < 0.15]
    contacts = [(c, False) for c in fl] + [(c, True) for c in ground + pairs]
    ptr, col, val = [0], [], []
    for (a, b), fr in contacts:
        for _ in range(3 if fr else 1):
            for body in (a, b):
                if body < 0:
                    continue
                for k in range(6):
                    col.append(6 * body + k)
                    val.append(rng.normal())
            ptr.append(len(col))
    nrows = len(ptr) - 1
    nv = 6 * nb
    m = rng.uniform(0.5, 2.0, nv)
    args = dict(row_ptr=np.array(ptr, np.int32), col=np.array(col, np.int32), val=np.array(val),
                contact_bias=rng.normal(size=nrows) * 0.1, mu=rng.uniform(0.1, 0.6, nrows),
                restitution=rng.uniform(0, 0.2, nrows), minv=1.0 / m, mdiag=1.0 / (1.0 / m),
                v=rng.normal(size=nv), f_ext=rng.normal(size=nv), f_gyro=rng.normal(size=nv) * 1e-3, dt=1e-3,
                alpha=0.3, max_iter=60, tol_abs=0.0, tol_rel=0.0,
                lam0=np.abs(rng.normal(size=nrows)) * 0.01, nfl=len(fl))
    return pos, args


def run_domain(args, owner, rank, world, dist=None):
    d = PileDomain(args["row_ptr"], args["col"], args["nfl"], owner, rank, world).connect(dist)
    keys = ("val", "contact_bias", "mu", "restitution", "minv", "mdiag", "v", "f_ext", "f_gyro", "dt", "alpha",
            "max_iter", "tol_abs", "tol_rel", "lam0")
    x, lam, it = d.solve(*[args[k] for k in keys], dist=dist)
    return d, x, lam, it


def test_slab_owner_balances_and_orders():
    rng = np.random.default_rng(0)
    pos = rng.uniform(0, 1, (1000, 3)) * [4, 1, 1]
    for world in (1, 2, 3, 8):
        own = slab_owner(pos, world)
        counts = np.bincount(own, minlength=world)
        assert counts.max() - counts.min() <= 1
        # slabs along x: every rank's bodies sit left of the next rank's, up to one slab cell
        for r in range(world - 1):
            assert pos[own == r, 0].min() <= pos[own == r + 1, 0].min()


def test_one_rank_equals_the_oracle(oracle_mod):
    pos, args = pile_problem()
    xo, lo, ito = oracle_mod.pj_solve_csr(**args)
    _, x, lam, it = run_domain(args, np.zeros(len(pos), np.int32), 0, 1)
    assert it == ito
    assert np.array_equal(x, xo) and np.array_equal(lam, lo)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir, tol):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pos, args = pile_problem()
    if tol:
        args.update(tol_abs=1e-7, tol_rel=1e-5, max_iter=2000)
    owner = slab_owner(pos, world)
    d, x, lam, it = run_domain(args, owner, rank, world, dist)
    np.savez(os.path.join(out_dir, f"rank{rank}.npz"), x=x, lam=lam, it=it, owned=d.owned, rows=d.rows,
             ghosts=d.ghosts)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("tol", [False, True])
def test_two_gloo_ranks_equal_the_single_process_solve(oracle_mod, tmp_path, tol):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.start_processes(_worker, args=(world, _free_port(), str(tmp_path), tol), nprocs=world, start_method="spawn",
                       join=True)
    pos, args = pile_problem()
    if tol:
        args.update(tol_abs=1e-7, tol_rel=1e-5, max_iter=2000)
    xo, lo, ito = oracle_mod.pj_solve_csr(**args)
    x = np.zeros_like(xo)
    lam = np.zeros_like(lo)
    its, nghost = [], 0
    for r in range(world):
        f = np.load(tmp_path / f"rank{r}.npz")
        dofs = (6 * f["owned"][:, None] + np.arange(6)).reshape(-1)
        x[dofs] = f["x"][dofs]
        lam[f["rows"]] = f["lam"][f["rows"]]
        its.append(int(f["it"]))
        nghost += len(f["ghosts"])
    assert nghost > 0  # contacts cross the slab boundary
    assert its[0] == its[1] == ito
    assert np.array_equal(x, xo)
    assert np.array_equal(lam, lo)
