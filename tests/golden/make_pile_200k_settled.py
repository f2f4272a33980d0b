"""Make the settled 200,000-sphere pile that the step benchmark and the pile-size parity test start from.

The seeded pile_200k scene (200,000 spheres, r ~ U[0.02, 0.05] m, 4 x 4 x 8 m box, mu 0.4,
h 5e-4, 100 projected Jacobi sweeps a step, alpha 0.5) is stepped 6,000 times (3 s of simulated
time; the pile is at rest after about 2.5 s) with the plain FP64 GPU method, which is
bit-identical to the CPU oracle, so the file reproduces exactly on any GB300 and is also what the
oracle computes from the same seed. Stored: the centres rounded to FP32 and the radii rounded to
FP32 (scenes.settled_pile builds the scene from them, at rest: zero velocities, identity
orientations), and the box's static planes. Needs a CUDA GPU; about three minutes on a GB300.

    python tests/golden/make_pile_200k_settled.py [steps]
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

OUT = os.path.join(HERE, "pile_200k_settled.npz")
STATIC_KEYS = ("static_kind", "static_pos", "static_quat", "static_vel", "static_omega", "static_dir",
               "static_radius", "static_mu", "static_rest_n", "static_rest_t")


def main(steps: int = 6000) -> None:
    from cardillocxx_gb300 import PhysicsEngine, scenes
    scene = scenes.generate("pile_200k")
    cfg = scenes.config_for("pile_200k", **{"gpu.precision": "fp64"})
    e = PhysicsEngine(cfg).load_scene(scene)
    t0 = time.time()
    done = 0
    while done < steps:
        k = min(500, steps - done)
        e.step(k)
        done += k
        st = e.stats()
        v = np.linalg.norm(e.state()["vel"], axis=1)
        print(f"{done}/{steps}: contacts {st['num_contacts']} mean |v| {v.mean():.2e} ({time.time() - t0:.0f} s)",
              flush=True)
    state = e.state()
    out = {"pos": state["pos"].astype(np.float32), "radius": scene["radius"].astype(np.float32),
           "steps": np.int64(steps), "seed": np.int64(scenes.SEED_BASE + scenes.PRESETS["pile_200k"]["num"]),
           "density": np.float64(1000.0), "mu": np.float64(scenes.PRESETS["pile_200k"]["mu"])}
    for k in STATIC_KEYS:
        out[k] = scene[k]
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}", flush=True)


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 6000)
