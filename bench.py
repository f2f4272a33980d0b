#!/usr/bin/env python3
"""Benchmark of the GPU contact step on the 200,000-sphere pile (~1M contacts once settled).

One "step" is one Moreau midpoint step of the whole pile: grid broad phase, narrow phase, contact
setup, projected Jacobi (100 sweeps or complementarity residual 1e-6), velocity update and drift.

Workload: 200,000 spheres r~U[0.02,0.05] m in a 4x4x8 m box, mu 0.4, h 5e-4, seeded placement.
The input is synthesised by settling the seeded pile for --settle steps with the engine
(untimed); both arms then start from that settled state.

  value         ms/step of the split form (FP32 contacts/Delassus/projection, FP64 state and
                residual), device time from CUDA events on the engine's stream, L2 flushed
                between timed steps
  plain_fp64    the plain FP64 GPU method on the same state (beside the chosen form)
  cpu_baseline  the CPU oracle (FP64 restatement of the reference path, all host threads) on a
                bounded sample of the same state
  e2e           the same step through the C ABI with the state uploaded from pinned host
                buffers and read back every step
  roofline      the dominant kernel (FP32 contact sweep) timed per launch with CUDA events

--impl reference times the reference path's CPU implementation (the oracle port; the reference
itself cannot be built here) on the same workload and prints the same line with "impl".
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/step at residual 1e-6: batched FP32 vs plain FP64 GPU vs CPU; HBM GB/s"
FALLBACK_HBM_GBS = 6800.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="cdx", choices=["cdx", "reference"])
    p.add_argument("--precision", default="split", choices=["split", "fp64"])
    p.add_argument("--scene", default="pile_200k")
    p.add_argument("--scale", type=float, default=1.0)
    p.add_argument("--settle", type=int, default=2000)
    p.add_argument("--fp64-steps", type=int, default=3)
    p.add_argument("--cpu-seconds", type=float, default=20.0)
    p.add_argument("--cpu-steps", type=int, default=None, help="CPU baseline steps (default: about --cpu-seconds)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-graph", action="store_true", help="launch the sweep kernels one by one (profiling)")
    p.add_argument("--sweep-variant", default=None,
                   help="pin the split-form solver shape (index or name; default: autotuned)")
    p.add_argument("--save-state", default=None, help="write the settled state (npz) and continue")
    p.add_argument("--load-state", default=None, help="start from a settled state written by --save-state")
    p.add_argument("--adjoint", action="store_true",
                   help="time the differentiable rollout (forward with checkpoints, then the adjoint) of "
                        "--scene (default diff_256x256) over --rollout-steps steps instead of the step bench")
    p.add_argument("--rollout-steps", type=int, default=200)
    p.add_argument("--set", action="append", default=[], metavar="KEY=VALUE",
                   help="extra configuration key for the timed engine (repeatable), e.g. gpu.coop_blocks=8")
    return p.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region (SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def settled_state(scene, cfg, steps: int, log):
    """Input synthesis: settle the seeded pile (split form), return the host state."""
    from cardillocxx_gb300 import PhysicsEngine
    e = PhysicsEngine(dict(cfg, **{"gpu.precision": "split"})).load_scene(scene)
    t = time.time()
    chunk = 250
    done = 0
    while done < steps:
        k = min(chunk, steps - done)
        e.step(k)
        done += k
        st = e.stats()
        log(f"settle {done}/{steps}: contacts {st['num_contacts']} iters {st['iterations']} "
            f"residual {st['residual']:.2e} ({time.time() - t:.1f}s)")
    state = e.state()
    e.close()
    return state


def load_or_settle(a, scene, cfg, log):
    import numpy as np
    if a.load_state:
        d = np.load(a.load_state)
        state = {k: d[k] for k in ("pos", "quat", "vel", "omega")}
        assert state["pos"].shape == scene["pos"].shape
        log(f"loaded settled state from {a.load_state}")
        return state
    state = settled_state(scene, cfg, a.settle, log)
    if a.save_state:
        np.savez(a.save_state, **state)
    return state


def with_state(scene, state):
    s = dict(scene)
    for k in ("pos", "quat", "vel", "omega"):
        s[k] = state[k].copy()
    return s


def time_engine(scene, cfg, steps, warmup, log, flush=None):
    """Per-step device time (CUDA events on the engine's stream), L2 flushed between steps."""
    import torch
    from cardillocxx_gb300 import PhysicsEngine
    e = PhysicsEngine(cfg).load_scene(scene)
    for _ in range(warmup):
        e.step(1)
    ext = torch.cuda.ExternalStream(e.stream())
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    st0 = e.stats()
    iters, contacts, res = [], [], []
    torch.cuda.synchronize()
    for k in range(steps):
        if flush is not None:
            with torch.cuda.stream(ext):
                flush.fill_(k & 0xff)
        starts[k].record(ext)
        e.step(1)
        ends[k].record(ext)
        st = e.stats()
        iters.append(st["iterations"])
        contacts.append(st["num_contacts"])
        res.append(st["residual"])
    torch.cuda.synchronize()
    ms = [s.elapsed_time(t) for s, t in zip(starts, ends)]
    st1 = e.stats()
    return e, ms, iters, contacts, res, st1["kernel_launches"] - st0["kernel_launches"]


def run_cdx(a, log):
    import torch
    from cardillocxx_gb300 import scenes

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    hbm, peak_kind = peaks()
    scene = scenes.generate(a.scene, scale=a.scale)
    cfg = scenes.config_for(a.scene)
    N = scene["pos"].shape[0]
    state = load_or_settle(a, scene, cfg, log)
    sscene = with_state(scene, state)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    run_cfg = dict(cfg, **{"gpu.precision": a.precision, "gpu.graph": not a.no_graph})
    for kv in a.set:
        k, _, v = kv.partition("=")
        run_cfg[k.strip()] = v.strip()
    if a.sweep_variant is not None:
        from cardillocxx_gb300 import PhysicsEngine
        names = PhysicsEngine.split_variants()
        v = a.sweep_variant
        run_cfg["gpu.sweep_variant"] = names.index(v) if v in names else int(v)
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    eng, ms, iters, contacts, res, launches = time_engine(sscene, run_cfg, a.steps, a.warmup, log, flush)
    est = eng.stats()
    clk = clocks.stop()
    total_ms = sum(ms)
    if world > 1:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / a.steps
    cit = sum(c * i for c, i in zip(contacts, iters)) / (sum(ms) / 1e3)
    log(f"{a.precision}: {ms_step:.3f} ms/step, contacts {contacts[-1]}, iters {iters[-1]}, residual {res[-1]:.2e}")

    # dominant kernel: the contact sweep, timed per launch with CUDA events on the engine stream.
    # Algorithmic bytes of one projected Jacobi iteration: every datum of the iteration counted once,
    # 40 words + 8 B a contact (frame 9, lever arms 18, R + bias + mu 7, impulse read and write 6,
    # two body indices) and 20 words a body (velocities read, accumulated, written; inverse masses),
    # with 4-byte words in the split form and 8-byte words in the plain FP64 method.
    tsw = eng.time_sweeps(60)
    w = 4 if a.precision == "split" else 8
    alg_bytes = contacts[-1] * (40 * w + 8) + N * (20 * w)
    t_sweep_ms = tsw["ms_contact"] + tsw["ms_body"]
    achieved = alg_bytes / (t_sweep_ms * 1e-3) / 1e9 if t_sweep_ms > 0 else None
    moved = (tsw["bytes_contact"] + tsw["bytes_body"]) / (t_sweep_ms * 1e-3) / 1e9 if t_sweep_ms > 0 else None
    # the dominant kernel: the cooperative whole solve (timed per sweep inside one launch) or the
    # streaming sweep kernel (one launch per sweep), whichever shape the autotuner chose
    from cardillocxx_gb300 import PhysicsEngine
    names = PhysicsEngine.split_variants()
    cv = est.get("sweep_variant", -1)
    vname = names[cv] if a.precision == "split" and 0 <= cv < len(names) else None
    if a.precision != "split":
        kernel, per, units = "k_sweep_contact64", "contact", contacts[-1]
    elif vname and vname.startswith("coop"):
        kernel, per, units = "k_s_solve_coop", "body", N
    else:
        kernel, per, units = "k_s_sweep_t", "contact", contacts[-1]
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        if kernel in tj and tj[kernel].get("per") == per:
            traffic = tj[kernel]["dram_bytes_per_sweep_per_unit"] * units
    roofline = {"kernel": kernel, "variant": vname, "bound": "hbm", "launch": "one projected Jacobi sweep",
                "achieved": achieved, "peak": hbm, "peak_kind": f"{peak_kind} hbm_gbs", "unit": "GB/s",
                "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
                "bytes_per_launch": alg_bytes, "word_bytes": w, "ms_per_launch": t_sweep_ms,
                # what this kernel has to move per sweep (the cooperative solve keeps the contact
                # side on chip across sweeps; the streaming sweep rereads its records)
                "bytes_moved_per_launch": tsw["bytes_contact"] + tsw["bytes_body"], "achieved_moved": moved,
                "frac_moved": (moved / hbm) if moved else None,
                "body_kernel_ms": tsw["ms_body"]}

    # e2e through the C ABI: state uploaded from pinned host memory and read back every step
    e2e = None
    if not a.no_e2e:
        pins = {k: torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy()
                for k, v in state.items()}
        eng.state_into(pins["pos"], pins["quat"], pins["vel"], pins["omega"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            eng.set_state(pins["pos"], pins["quat"], pins["vel"], pins["omega"])
            eng.step(1)
            eng.state_into(pins["pos"], pins["quat"], pins["vel"], pins["omega"])
        torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) * 1e3 / a.steps
        if world > 1:
            t = torch.tensor([e2e_ms], device=dev, dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_ms = float(t.item())
        nbytes = 13 * 8 * N
        e2e = {"value": e2e_ms, "unit": "ms/step", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes}
    eng.close()

    # plain FP64 GPU method on the same state (beside the chosen form)
    plain = None
    if a.precision == "split" and a.fp64_steps > 0:
        e64, ms64, it64, c64, r64, _ = time_engine(sscene, dict(cfg, **{"gpu.precision": "fp64"}), a.fp64_steps,
                                                  1, log, flush)
        m64 = sum(ms64) / len(ms64)
        plain = {"ms_per_step": m64, "contact_iters_per_s": sum(c * i for c, i in zip(c64, it64)) / (sum(ms64) / 1e3),
                 "iterations": it64[-1], "residual": r64[-1], "contacts": c64[-1],
                 "speedup_of_split": m64 / ms_step}
        if c64[-1] > 0:  # the sweep timing replays the last step's contacts
            t64 = e64.time_sweeps(5)
            plain["contact_kernel_ms"] = t64["ms_contact"]
            plain["contact_kernel_gbs"] = t64["bytes_contact"] / (t64["ms_contact"] * 1e-3) / 1e9
        e64.close()
        log(f"fp64 plain: {m64:.3f} ms/step ({m64 / ms_step:.1f}x the split form)")

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cpu = cpu_baseline(sscene, cfg, a.cpu_seconds, log, steps=a.cpu_steps)

    out = {"metric": METRIC, "value": ms_step, "unit": "ms/step", "n_gpus": world, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32-contact/f64-state" if a.precision == "split" else "f64",
           "data": f"synthetic: seeded {a.scene} (seed 0xC0FFEE02) settled {a.settle} steps on the GPU",
           "config": {"workload": a.scene, "bodies": N, "contacts": contacts[-1], "iterations_per_step": iters[-1],
                      "residual": res[-1], "residual_tol": cfg.get("gpu.residual_tol"),
                      "max_iterations": cfg["pj.max_iterations"], "dt": cfg["sim.dt"], "precision": a.precision,
                      "l2": "flushed between timed steps (256 MiB write outside the timed events)",
                      "contact_variant": est.get("contact_variant"), "autotune_runs": est.get("autotune_runs"),
                      "parallelism": "replicas" if world > 1 else "single"},
           "contact_iters_per_s": cit * (world if world > 1 else 1), "roofline": roofline,
           "plain_fp64": plain, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def cpu_model() -> str:
    """The host CPU's model name (x86 /proc/cpuinfo, else lscpu on Arm)."""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    try:
        import subprocess
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def cpu_baseline(sscene, cfg, seconds, log, steps=None):
    """The CPU oracle on the same state, a bounded number of steps: all host threads (SpMV rows,
    body gathers and projection in OpenMP), and the reference's own threading (OpenMP on the
    projection only, projected_jacobi.cpp:109) on a shorter sample."""
    from oracle import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    of = oracle.Oracle(sscene, cfg, omp_mode=0, num_threads=threads)
    t0 = time.perf_counter()
    of.step(1)
    faithful_ms = (time.perf_counter() - t0) * 1e3
    o = oracle.Oracle(sscene, cfg, omp_mode=1, num_threads=threads)
    t0 = time.perf_counter()
    o.step(1)
    first = time.perf_counter() - t0
    n = steps if steps is not None else max(1, min(20, int(seconds / max(first, 1e-3))))
    t0 = time.perf_counter()
    if n > 1:
        o.step(n - 1)
    rest = time.perf_counter() - t0
    ms = (first + rest) * 1e3 / n
    st = o.stats()
    log(f"cpu oracle: {ms:.1f} ms/step over {n} steps ({threads} threads), contacts {st['num_contacts']}; "
        f"reference threading {faithful_ms:.1f} ms for one step")
    return {"value": ms, "unit": "ms/step", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
            "sample": f"{n} full steps from the same state (cold warm start), {st['num_contacts']} contacts at the end",
            "iterations": st["iterations"], "residual": st["residual"],
            "reference_threading": {"value": faithful_ms, "unit": "ms/step", "steps": 1,
                                    "threads": "OpenMP on the projection only, SpMV and gathers on one thread"}}


def run_reference(a, log):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from cardillocxx_gb300 import scenes
    scene = scenes.generate(a.scene, scale=a.scale)
    cfg = scenes.config_for(a.scene)
    state = load_or_settle(a, scene, cfg, log)
    sscene = with_state(scene, state)
    from oracle import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    o = oracle.Oracle(sscene, cfg, omp_mode=1, num_threads=threads)
    for _ in range(a.warmup):
        o.step(1)
    t0 = time.perf_counter()
    o.step(a.steps)
    ms = (time.perf_counter() - t0) * 1e3 / a.steps
    st = o.stats()
    out = {"metric": METRIC, "value": ms, "unit": "ms/step", "impl": "reference", "n_gpus": 1, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": f"synthetic: seeded {a.scene} settled {a.settle} steps",
           "config": {"workload": a.scene, "bodies": int(scene["pos"].shape[0]), "contacts": st["num_contacts"],
                      "iterations_per_step": st["iterations"], "residual": st["residual"],
                      "implementation": "CPU restatement of the reference path (the reference needs Eigen, EnTT "
                                        "and coal, absent here); OpenMP over all host threads"},
           "cpu_baseline": {"value": ms, "unit": "ms/step", "cores": threads, "kind": "port",
                            "cpu_model": cpu_model(),
                            "sample": f"{a.steps} full steps after {a.warmup} warm-up steps"},
           "e2e": {"value": ms, "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_adjoint(a, log):
    """The differentiation workload: 256 scenes of 256 spheres, a COM loss on the final state,
    gradients w.r.t. the initial state and the per-scene friction through the adjoint kernels
    (checkpoints every 20 steps). Prints one JSON line with the forward and adjoint wall times
    (both calls return after the device finished)."""
    import numpy as np
    from cardillocxx_gb300 import scenes
    from cardillocxx_gb300.adjoint import Rollout
    name = a.scene if a.scene != "pile_200k" else "diff_256x256"
    s = scenes.generate(name, scale=a.scale)
    cfg = scenes.config_for(name)
    nsc = int(s["num_scenes"])
    sc, m = s["body_scene"], s["mass"]
    M = np.bincount(sc, weights=m, minlength=nsc)
    target = np.random.default_rng(6).uniform((0.2, 0.2, 0.1), (0.8, 0.8, 0.5), size=(nsc, 3))
    R = Rollout(s, cfg, checkpoint_every=20)
    mu = np.full(nsc, 0.3)
    T = a.rollout_steps
    fwd, bwd = [], []
    for k in range(a.warmup + a.steps):
        t0 = time.perf_counter()
        xT, _, _ = R.forward(T, s["pos"], s["vel"], s["omega"], mu)
        t1 = time.perf_counter()
        com = np.stack([np.bincount(sc, weights=m * xT[:, q], minlength=nsc) for q in range(3)], 1) / M[:, None]
        gx = 2 * (com - target)[sc] * (m / M[sc])[:, None]
        t2 = time.perf_counter()
        R.backward(gx, np.zeros_like(gx), np.zeros_like(gx))
        t3 = time.perf_counter()
        if k >= a.warmup:
            fwd.append(1e3 * (t1 - t0))
            bwd.append(1e3 * (t3 - t2))
        log(f"rollout {k}: forward {1e3 * (t1 - t0):.1f} ms, adjoint {1e3 * (t3 - t2):.1f} ms")
    f, b = float(np.median(fwd)), float(np.median(bwd))
    print(json.dumps({"metric": "differentiable rollout ms (forward with checkpoints + adjoint)",
                      "value": f + b, "unit": "ms", "n_gpus": 1, "steps": a.steps, "warmup": a.warmup,
                      "higher_is_better": False, "dtype": "f64", "data": f"synthetic: seeded {name}",
                      "config": {"workload": name, "scenes": nsc, "bodies": int(s["pos"].shape[0]),
                                 "rollout_steps": T, "checkpoint_every": 20, "info": R.info()},
                      "forward_ms": f, "adjoint_ms": b}), flush=True)


def main():
    a = parse()
    if a.gpus > 1 and "LOCAL_RANK" in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]
    import __graft_entry__
    __graft_entry__.build()

    def log(msg):
        print(f"[bench] {msg}", file=sys.stderr, flush=True)

    if a.impl == "reference":
        run_reference(a, log)
    elif a.adjoint:
        run_adjoint(a, log)
    else:
        run_cdx(a, log)


if __name__ == "__main__":
    main()
