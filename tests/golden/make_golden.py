"""Generate the frozen golden fixtures of the contact path (run on a CPU; needs no GPU).

Each fixture stores a seeded scene (inputs), the reference-key configuration, and the CPU
oracle's outputs after a number of Moreau midpoint steps: the body state, the contacts of the
last step (entity ids, points, impulses) and the solver statistics. The oracle is IEEE FP64 with
no FMA contraction and no transcendental functions on the step, so the fixtures reproduce
bit-for-bit on any IEEE-754 host; the tests check the oracle (CPU) and the plain FP64 GPU method
against them.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from cardillocxx_gb300 import scenes  # noqa: E402
from oracle import oracle  # noqa: E402

SCENE_KEYS = ("pos", "quat", "vel", "omega", "radius", "mass", "inertia", "mu", "rest_n", "rest_t", "body_scene",
              "static_kind", "static_pos", "static_quat", "static_vel", "static_omega", "static_dir",
              "static_radius", "static_mu", "static_rest_n", "static_rest_t", "static_scene")


def cases():
    out = []
    s = scenes.generate("pile_1k", scale=0.05)
    out.append(("pile50", s, scenes.config_for("pile_1k"), 120))
    d = scenes.generate("drum_1m", num_bodies=120, r=(0.02, 0.03), drum=(0.3, 0.3, 2.0))
    out.append(("drum120", d, scenes.config_for("drum_1m", **{"sim.dt": 1e-3}), 300))
    b = scenes.generate("batch_4096", scale=0.001)
    out.append(("batch4", b, scenes.config_for("batch_4096"), 60))
    m = scenes.generate("pile_1k", scale=0.05, seed=77)
    m["mu"][::3] = 0.0
    out.append(("mixed50", m, scenes.config_for("pile_1k", **{"friction.combine": "arith"}), 80))
    return out


def csr_case():
    rng = np.random.default_rng(11)
    nb, nfl, nfr = 12, 3, 10
    nv = 6 * nb
    cols, vals, ptr = [], [], [0]
    for r in range(nfl + 3 * nfr):
        a, b = sorted(rng.choice(nb, 2, replace=False))
        for body in (a, b):
            for k in range(6):
                cols.append(6 * body + k)
                vals.append(rng.normal())
        ptr.append(len(cols))
    nrows = nfl + 3 * nfr
    m = rng.uniform(0.5, 2.0, nv)
    return dict(row_ptr=np.array(ptr, np.int32), col=np.array(cols, np.int32), val=np.array(vals),
                contact_bias=rng.normal(size=nrows) * 0.1, mu=rng.uniform(0.1, 0.6, nrows),
                restitution=rng.uniform(0, 0.2, nrows), minv=1.0 / m, mdiag=1.0 / (1.0 / m), v=rng.normal(size=nv),
                f_ext=rng.normal(size=nv), f_gyro=rng.normal(size=nv) * 1e-3, lam0=np.abs(rng.normal(size=nrows)) * 0.01,
                nfl=np.int32(nfl))


def main():
    oracle.build()
    for name, scene, cfg, steps in cases():
        o = oracle.Oracle(scene, cfg)
        o.step(steps)
        st = o.state()
        c = o.contacts()
        stats = o.stats()
        arrs = {f"in_{k}": np.asarray(scene[k]) for k in SCENE_KEYS}
        arrs.update({f"out_{k}": v for k, v in st.items()})
        arrs.update({f"contact_{k}": v for k, v in c.items()})
        meta = {"cfg": cfg, "steps": steps, "num_scenes": int(scene["num_scenes"]), "stats": stats}
        arrs["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
        print(name, scene["pos"].shape[0], "bodies", stats)
    p = csr_case()
    args = {k: v for k, v in p.items() if k != "nfl"}
    x, lam, it = oracle.pj_solve_csr(**args, dt=1e-3, alpha=0.3, max_iter=40, tol_abs=0.0, tol_rel=0.0,
                                     nfl=int(p["nfl"]))
    np.savez_compressed(os.path.join(HERE, "csr.npz"), **p, out_x=x, out_lambda=lam, out_iters=np.int32(it))
    print("csr", it)


def load(name):
    d = np.load(os.path.join(HERE, f"{name}.npz"))
    meta = json.loads(bytes(d["meta"]).decode())
    scene = {k: d[f"in_{k}"] for k in SCENE_KEYS}
    scene["num_scenes"] = meta["num_scenes"]
    return scene, meta, d


NAMES = ("pile50", "drum120", "batch4", "mixed50")

if __name__ == "__main__":
    main()
