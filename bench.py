#!/usr/bin/env python3
"""Benchmark of the GPU contact step on the settled 200,000-sphere pile.

One "step" is one Moreau midpoint step of the whole pile: grid broad phase, narrow phase, contact
setup, projected Jacobi (100 sweeps or complementarity residual 1e-6, warm-started from the
previous step), velocity update and drift.

Input: the seeded pile_200k scene (200,000 spheres r ~ U[0.02, 0.05] m in a 4 x 4 x 8 m box,
mu 0.4, h 5e-4) settled for 6,000 steps by the plain FP64 method, stored in
tests/golden/pile_200k_settled.npz (FP32 centres and radii, at rest; made by
tests/golden/make_pile_200k_settled.py). Both arms build the same scene from that file with NumPy
and print its digest; neither synthesises its input with the other's code.

  value         ms/step of the split form (FP32 contacts/Delassus/projection, FP64 state and
                residual): --warmup untimed steps, then --steps timed steps, device time from CUDA
                events on the engine's stream, L2 flushed between timed steps
  plain_fp64    the plain FP64 GPU method over the same steps; its final state digest equals the
                reference arm's (the method is bit-identical to the CPU oracle)
  cpu_baseline  the CPU oracle (FP64 restatement of the reference path, all host threads) on a
                bounded sample of the same steps
  e2e           the same steps through the C ABI with the state uploaded from pinned host
                buffers and read back every step
  roofline      the dominant kernel (the split form's projected Jacobi solve) per sweep
  at_residual   every form solved to complementarity residual <= 1e-6 on the warm-started pile
                (the input stepped --warm-steps times by the plain FP64 method, bit-reproducible;
                state and contact memory loaded into each form): ms/step, sweeps, residual, and the
                speed-up of the
                split form over the plain FP64 method at equal residual
  split_error   the split form against the plain FP64 method on one step from the warm-started
                pile, both solved to residual 1e-6
  workloads     the batched scenes, the rotating drum and the differentiable rollout

--impl reference times the reference path's CPU implementation (the oracle port; the reference
itself cannot be built here) on the same input and steps, with all host threads, and prints the
same line with "impl". It loads no code of the GPU library.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms/step at residual 1e-6: batched FP32 vs plain FP64 GPU vs CPU; HBM GB/s"
FALLBACK_HBM_GBS = 6800.0
PILE_INPUT = os.path.join(ROOT, "tests", "golden", "pile_200k_settled.npz")


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="cdx", choices=["cdx", "reference"])
    p.add_argument("--precision", default="split", choices=["split", "fp64"])
    p.add_argument("--scene", default="pile_200k")
    p.add_argument("--scale", type=float, default=1.0)
    p.add_argument("--input", default=None,
                   help="settled input file (default: the committed pile_200k input for --scene pile_200k)")
    p.add_argument("--settle", type=int, default=None,
                   help="scenes without an input file: steps that settle the seeded scene first (untimed)")
    p.add_argument("--fp64-steps", type=int, default=None,
                   help="timed steps of the plain FP64 leg (default --steps, after the same warm-up)")
    p.add_argument("--cpu-seconds", type=float, default=20.0)
    p.add_argument("--cpu-steps", type=int, default=None, help="CPU baseline steps (default: about --cpu-seconds)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-graph", action="store_true", help="launch the sweep kernels one by one (profiling)")
    p.add_argument("--sweep-variant", default=None,
                   help="pin the split-form solver shape (index or name; default: autotuned)")
    p.add_argument("--warm-steps", type=int, default=3000,
                   help="at_residual leg: plain FP64 steps that rebuild the warm start on the input")
    p.add_argument("--residual-steps", type=int, default=10, help="at_residual leg: timed steps per GPU form")
    p.add_argument("--residual-warmup", type=int, default=3,
                   help="at_residual leg: untimed steps per GPU form (its first steps hold the shape autotuner's "
                        "trials and the graph capture)")
    p.add_argument("--residual-cap", type=int, default=20000, help="at_residual leg: sweep cap a step")
    p.add_argument("--no-residual-leg", action="store_true")
    p.add_argument("--residual-forms", default="split,fp64,split_nesterov,condensed",
                   help="at_residual leg: the forms to run (comma-separated)")
    p.add_argument("--no-workloads", action="store_true", help="skip the batched, drum and rollout workloads")
    p.add_argument("--adjoint", action="store_true",
                   help="time only the differentiable rollout (forward with checkpoints, then the adjoint) of "
                        "--scene (default diff_256x256) over --rollout-steps steps")
    p.add_argument("--rollout-steps", type=int, default=200)
    p.add_argument("--set", action="append", default=[], metavar="KEY=VALUE",
                   help="extra configuration key for the timed engine (repeatable), e.g. gpu.coop_blocks=8")
    return p.parse_args()


def log(msg):
    print(f"[bench] {msg}", file=sys.stderr, flush=True)


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


# ---------------------------------------------------------------------------------------- input
def workload_input(a):
    """The scene both arms start from, its configuration and a description (NumPy only for the
    committed pile input; other scenes are generated and, in the GPU arm, settled first)."""
    from cardillocxx_gb300 import scenes
    cfg = scenes.config_for(a.scene)
    path = a.input or (PILE_INPUT if a.scene == "pile_200k" and a.scale == 1.0 else None)
    if path:
        scene = scenes.settled_pile(path)
        desc = f"seeded {a.scene} settled by the plain FP64 method, committed as {os.path.relpath(path, ROOT)}"
        return scene, cfg, desc, os.path.basename(path)
    return None, cfg, None, None


def shared_config(a, scene, cfg, input_name) -> dict:
    """The workload definition both arms print (equal lines mean equal inputs and work)."""
    from cardillocxx_gb300 import scenes
    return {"workload": a.scene, "bodies": int(scene["pos"].shape[0]), "input": input_name,
            "input_digest": scenes.scene_digest(scene), "dt": cfg["sim.dt"], "theta": cfg["moreau.theta"],
            "max_iterations": cfg["pj.max_iterations"], "residual_tol": cfg.get("gpu.residual_tol", 0.0),
            "alpha": cfg["pj.alpha"], "warm_start": bool(cfg["pj.warmstart"]), "warmup_steps": a.warmup,
            "timed_steps": a.steps}


def with_state(scene, state):
    s = dict(scene)
    for k in ("pos", "quat", "vel", "omega"):
        s[k] = state[k].copy()
    return s


def settle_gpu(scene, cfg, steps: int, precision="split", extra=None):
    """Steps a generated scene with the GPU engine (input synthesis for scenes without a file)."""
    from cardillocxx_gb300 import PhysicsEngine
    e = PhysicsEngine(dict(cfg, **{"gpu.precision": precision}, **(extra or {}))).load_scene(scene)
    t = time.time()
    done = 0
    while done < steps:
        k = min(500, steps - done)
        e.step(k)
        done += k
        st = e.stats()
        log(f"settle {done}/{steps}: contacts {st['num_contacts']} iters {st['iterations']} "
            f"residual {st['residual']:.2e} ({time.time() - t:.1f}s)")
    state, mem = e.state(), e.contacts()
    e.close()
    return state, mem


# ---------------------------------------------------------------------------------------- timing
def time_engine(eng, steps, warmup, flush=None):
    """Per-step device time (CUDA events on the engine's stream), L2 flushed between steps."""
    import torch
    for _ in range(warmup):
        eng.step(1)
    ext = torch.cuda.ExternalStream(eng.stream())
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    st0 = eng.stats()
    iters, contacts, res = [], [], []
    torch.cuda.synchronize()
    for k in range(steps):
        if flush is not None:
            with torch.cuda.stream(ext):
                flush.fill_(k & 0xff)
        starts[k].record(ext)
        eng.step(1)
        ends[k].record(ext)
        st = eng.stats()
        iters.append(st["iterations"])
        contacts.append(st["num_contacts"])
        res.append(st["residual"])
    torch.cuda.synchronize()
    ms = [s.elapsed_time(t) for s, t in zip(starts, ends)]
    st1 = eng.stats()
    return ms, iters, contacts, res, st1["kernel_launches"] - st0["kernel_launches"]


def roofline_of(eng, precision, contacts, N, hbm, peak_kind):
    """The dominant kernel per projected Jacobi sweep: algorithmic bytes (every datum of one
    iteration counted once: 40 words + 8 B a contact, 20 words a body; 4-byte words in the split
    form, 8-byte in the plain method) over the CUDA-event time of one sweep."""
    from cardillocxx_gb300 import PhysicsEngine
    tsw = eng.time_sweeps(60)
    w = 4 if precision == "split" else 8
    alg = contacts * (40 * w + 8) + N * (20 * w)
    t_ms = tsw["ms_contact"] + tsw["ms_body"]
    achieved = alg / (t_ms * 1e-3) / 1e9 if t_ms > 0 else None
    moved_b = tsw["bytes_contact"] + tsw["bytes_body"]
    moved = moved_b / (t_ms * 1e-3) / 1e9 if t_ms > 0 else None
    names = PhysicsEngine.split_variants()
    cv = eng.stats().get("sweep_variant", -1)
    vname = names[cv] if precision == "split" and 0 <= cv < len(names) else None
    coop = bool(vname and vname.startswith("coop"))
    if precision != "split":
        kernel, per, units, bound = "k_sweep_contact64", "contact", contacts, "fp64 issue"
    elif coop:
        kernel, per, units, bound = "k_s_solve_coop", "body", N, "latency/L2"
    else:
        kernel, per, units, bound = "k_s_sweep_t", "contact", contacts, "latency/L2"
    traffic, l2frac = None, None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            tj = json.load(f)
        if kernel in tj and tj[kernel].get("per") == per:
            traffic = tj[kernel]["dram_bytes_per_sweep_per_unit"] * units
            l2frac = tj[kernel].get("lts_throughput_frac")
    return {"kernel": kernel, "variant": vname, "bound": bound, "launch": "one projected Jacobi sweep",
            "achieved": achieved, "peak": hbm, "peak_kind": f"{peak_kind} hbm_gbs", "unit": "GB/s",
            "frac": (achieved / hbm) if achieved else None, "traffic": traffic,
            "bytes_per_launch": alg, "word_bytes": w, "ms_per_launch": t_ms,
            # what the kernel has to move per sweep: the cooperative solve keeps the contact side in
            # shared memory for the whole solve, so only body velocities cross L2/HBM each sweep
            "bytes_moved_per_launch": moved_b, "achieved_moved": moved,
            "frac_moved": (moved / hbm) if moved else None, "l2_throughput_frac_ncu": l2frac,
            "note": ("frac counts the iteration's algorithmic bytes; the cooperative solve keeps them on chip, "
                     "so frac above 1 is not DRAM traffic (traffic is the ncu DRAM bytes per sweep)") if coop else None}


# ---------------------------------------------------------------------------------------- legs
def split_error(scene, mem, cfg):
    """The split form against the plain FP64 method (the oracle's arithmetic) on one step from the same
    warm-started state, both solved to complementarity residual <= 1e-6: impulses over the contacts
    both found, velocities, positions. Maxima and the 99.9th percentile and median are stated: a
    contact that FP32 detection admits or drops at the margin (a gap within its resolution) moves
    its two spheres differently, while everywhere else the forms differ by the residual tolerance."""
    import numpy as np
    from cardillocxx_gb300 import PhysicsEngine
    out = {}
    rule = {"gpu.residual_tol": 1e-6, "pj.max_iterations": 20000, "gpu.check_every": 1}
    for prec in ("fp64", "split"):
        e = PhysicsEngine(dict(cfg, **rule, **{"gpu.precision": prec})).load_scene(scene).set_contacts(mem)
        e.step(1)
        out[prec] = (e.state(), e.contacts(), e.stats())
        e.close()
    (s64, c64, t64), (s32, c32, t32) = out["fp64"], out["split"]
    k64 = c64["id_a"].astype(np.int64) << 32 | c64["id_b"].astype(np.int64)
    k32 = c32["id_a"].astype(np.int64) << 32 | c32["id_b"].astype(np.int64)
    common, i64, i32 = np.intersect1d(k64, k32, return_indices=True)
    lmax = float(np.abs(c64["lambda"]).max()) if k64.size else 1.0
    dl = np.abs(c64["lambda"][i64] - c32["lambda"][i32]).max(axis=1) / lmax
    vs = float(np.abs(s64["vel"]).max()) + 9.81 * cfg["sim.dt"]
    dv = np.abs(s64["vel"] - s32["vel"]).max(axis=1) / vs

    def q(x):
        return {"max": float(x.max()), "p99_9": float(np.percentile(x, 99.9)), "median": float(np.median(x))}
    return {"contacts_fp64": int(k64.size), "contacts_split": int(k32.size), "contacts_common": int(common.size),
            "dlambda_over_max_lambda": q(dl), "dv_over_v_scale": q(dv),
            "max_domega": float(np.abs(s64["omega"] - s32["omega"]).max()),
            "max_dx_m": float(np.abs(s64["pos"] - s32["pos"]).max()),
            "residual_fp64": t64["residual"], "residual_split": t32["residual"],
            "sample": "one step from the warm-started pile (the at_residual state), both solved to residual 1e-6"}


def at_residual_leg(a, scene, cfg, flush):
    """ms/step at complementarity residual <= 1e-6: the input stepped --warm-steps times by the plain
    FP64 method under the pile's own configuration (100 sweeps a step, or residual 1e-6 sooner),
    which rebuilds the warm start a settled pile carries; then that state and contact memory loaded
    into each form, which solves every step until the residual is at most 1e-6 (cap --residual-cap
    sweeps): --residual-warmup untimed steps, then --residual-steps timed ones.
    The FP64 method is bit-reproducible, so every run measures the same steps from the same state
    (the FP64 form's sweeps repeat exactly, the split form's up to its FP32 sums). Warm steps by the
    split form gave states whose sweeps to 1e-6 varied severalfold between runs; warm steps under
    the residual rule itself never reach 1e-6 on this pile (20,000 sweeps a step leave about 1e-5:
    projected Jacobi's convergence on 200,000 stacked spheres is that slow), so the rule applies to
    the measured steps only."""
    import numpy as np
    from cardillocxx_gb300 import PhysicsEngine, scenes
    tol = 1e-6
    t0 = time.time()
    state, mem = settle_gpu(scene, cfg, a.warm_steps, "fp64")
    warm_s = time.time() - t0
    s2 = with_state(scene, state)
    rule = {"gpu.residual_tol": tol, "pj.max_iterations": a.residual_cap}
    split_tol = 0.98 * tol
    out = {"residual_tol": tol, "sweep_cap": a.residual_cap, "warm_steps": a.warm_steps,
           "warm_form": "fp64, the pile's configuration (100 sweeps or residual 1e-6)",
           "warm_state_digest": scenes.state_digest(state),
           "form_warmup_steps": a.residual_warmup,
           "warm_seconds": warm_s, "contacts": int(mem["id_a"].shape[0]),
           "stop_test": "every 10 sweeps in every form (gpu.check_every = 10: the plain FP64 method's host polls "
                        "the residual every 10 sweeps, the split form's device tests it every 10 sweeps)"}
    # The split form stops on its FP32 in-sweep residual; the FP64 residual of its result is
    # evaluated afterwards on FP64 geometry and ran up to 0.1 % above it, so the split forms stop at
    # 0.98e-6 for their FP64 residual to stay within 1e-6. Nesterov runs with a velocity tolerance
    # too small to end the loop, so the residual ends it.
    forms = {"split": {"gpu.precision": "split", "gpu.check_every": 10, "gpu.residual_tol": split_tol},
             "fp64": {"gpu.precision": "fp64", "gpu.check_every": 10},
             "split_nesterov": {"gpu.precision": "split", "gpu.check_every": 10, "gpu.residual_tol": split_tol,
                                "pj.nesterov": True, "pj.tol_abs": 1e-100, "pj.tol_rel": 0.0}}
    out["split_stop_tol"] = split_tol
    chosen = set(a.residual_forms.split(","))
    forms = {k: v for k, v in forms.items() if k in chosen}
    for name, over in forms.items():
        e = PhysicsEngine(dict(cfg, **dict(rule, **over))).load_scene(s2).set_contacts(mem)
        n = a.residual_steps
        # a few untimed steps first (the shape autotuner's trials, the step graph's capture): every
        # form then times the same steps from the same state
        ms, it, con, res, _ = time_engine(e, n, a.residual_warmup, flush)
        e.close()
        tot_s = sum(ms) / 1e3
        out[name] = {"ms_per_step": sum(ms) / len(ms), "sweeps_per_step": sum(it) / len(it),
                     "max_sweeps": max(it), "residual_max": max(res), "residual_last": res[-1], "steps": n,
                     "contact_iters_per_s": sum(c * i for c, i in zip(con, it)) / tot_s}
        log(f"at residual 1e-6, {name}: {out[name]['ms_per_step']:.2f} ms/step, {out[name]['sweeps_per_step']:.0f} "
            f"sweeps, residual <= {out[name]['residual_max']:.2e}")
    # the condensed solver's colored Gauss-Seidel sweeps (plain FP64, solver.type=condensed) on the
    # same state, with its own stop rule (the velocity-increment residual, here at tolerances 1e-6)
    # and alpha = relaxation = 1; the memory's tangential impulses enter in its own sign convention
    if "condensed" in chosen:
        cmem = dict(mem)
        cmem["lambda"] = mem["lambda"] * np.array([1.0, -1.0, -1.0])
        ccfg = dict(cfg, **{"gpu.precision": "fp64", "solver.type": "condensed", "condensed.sweep_mode": "colored",
                            "pj.alpha": 1.0, "pj.relaxation": 1.0, "pj.tol_abs": 1e-6, "pj.tol_rel": 1e-6,
                            "pj.max_iterations": a.residual_cap, "gpu.check_every": 10})
        e = PhysicsEngine(ccfg).load_scene(s2).set_contacts(cmem)
        ms, it, con, res, _ = time_engine(e, min(a.residual_steps, 5), min(a.residual_warmup, 5), flush)
        e.close()
        out["condensed_colored_fp64"] = {"ms_per_step": sum(ms) / len(ms), "sweeps_per_step": sum(it) / len(it),
                                         "residual_max": max(res), "steps": len(ms),
                                         "stop": "velocity-increment residual <= 1 at pj.tol_abs = pj.tol_rel = 1e-6",
                                         "alpha": 1.0, "relaxation": 1.0}
        log(f"condensed colored (fp64): {out['condensed_colored_fp64']['ms_per_step']:.2f} ms/step, "
            f"{out['condensed_colored_fp64']['sweeps_per_step']:.0f} sweeps, residual <= {max(res):.2e}")
    if "split" not in out or "fp64" not in out:
        out["speedup_at_equal_residual"] = None
    elif out["split"]["residual_max"] <= tol and out["fp64"]["residual_max"] <= tol:
        out["speedup_at_equal_residual"] = out["fp64"]["ms_per_step"] / out["split"]["ms_per_step"]
    else:
        out["speedup_at_equal_residual"] = None
        out["note"] = "a form reached the sweep cap above the residual tolerance; its residual is stated"
    if "split" in out and "fp64" in out:
        out["contact_iters_ratio"] = out["split"]["contact_iters_per_s"] / out["fp64"]["contact_iters_per_s"]
    return out, s2, mem


def cpu_at_residual(s2, mem, cfg, a):
    """The CPU oracle (all host threads) on the warm-started pile, the same stop rule, one step."""
    from oracle import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    rule = {"gpu.residual_tol": 1e-6, "pj.max_iterations": a.residual_cap}
    o = oracle.Oracle(s2, dict(cfg, **rule), omp_mode=1, num_threads=threads).set_contacts(mem)
    t0 = time.perf_counter()
    o.step(1)
    ms = (time.perf_counter() - t0) * 1e3
    st = o.stats()
    log(f"at residual 1e-6, cpu oracle: {ms:.0f} ms/step, {st['iterations']} sweeps, residual {st['residual']:.2e}")
    return {"ms_per_step": ms, "sweeps_per_step": st["iterations"], "residual": st["residual"], "steps": 1,
            "contact_iters_per_s": st["num_contacts"] * st["iterations"] / (ms / 1e3), "cores": threads,
            "kind": "port", "sample": "the first step from the warm-started state (one step: the CPU needs seconds)"}


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
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def cpu_baseline(scene, cfg, seconds, steps=None):
    """The CPU oracle on the input state, a bounded number of steps: all host threads (SpMV rows,
    body gathers and projection in OpenMP), and the reference's own threading (OpenMP on the
    projection only, projected_jacobi.cpp:109) for one step."""
    from oracle import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    of = oracle.Oracle(scene, cfg, omp_mode=0, num_threads=threads)
    t0 = time.perf_counter()
    of.step(1)
    faithful_ms = (time.perf_counter() - t0) * 1e3
    o = oracle.Oracle(scene, cfg, omp_mode=1, num_threads=threads)
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
            "sample": f"the first {n} steps from the input state, {st['num_contacts']} contacts at the end",
            "iterations": st["iterations"], "residual": st["residual"],
            "reference_threading": {"value": faithful_ms, "unit": "ms/step", "steps": 1,
                                    "threads": "OpenMP on the projection only, SpMV and gathers on one thread"}}


def other_workloads(flush):
    """The batched scenes, the rotating drum (split form and plain FP64 beside it) and the
    differentiable rollout, each settled or run for a stated number of steps first."""
    import numpy as np
    from cardillocxx_gb300 import PhysicsEngine, scenes
    out = {}
    for name, settle, steps, fp64_steps in (("batch_4096", 1000, 10, 2), ("drum_1m", 2000, 5, 2)):
        t0 = time.time()
        s = scenes.generate(name)
        cfg = scenes.config_for(name)
        state, mem = settle_gpu(s, cfg, settle, "split")
        s2 = with_state(s, state)
        rec = {"bodies": int(s["pos"].shape[0]), "settle_steps": settle, "contacts": int(mem["id_a"].shape[0])}
        for prec, n in (("split", steps), ("fp64", fp64_steps)):
            e = PhysicsEngine(dict(cfg, **{"gpu.precision": prec})).load_scene(s2).set_contacts(mem)
            ms, it, con, res, _ = time_engine(e, n, 1, flush)
            names = PhysicsEngine.split_variants()
            v = e.stats()["contact_variant"]
            e.close()
            rec[prec] = {"ms_per_step": sum(ms) / len(ms), "sweeps": it[-1], "residual": res[-1], "steps": n,
                         "contacts": con[-1], "shape": names[v] if prec == "split" and 0 <= v < len(names) else None}
        rec["fp64_over_split"] = rec["fp64"]["ms_per_step"] / rec["split"]["ms_per_step"]
        if name == "batch_4096":
            rec["at_residual"] = scenes_at_residual(s2, mem, cfg, flush)
        rec["seconds"] = time.time() - t0
        out[name] = rec
        log(f"{name}: split {rec['split']['ms_per_step']:.2f} ms/step, fp64 {rec['fp64']['ms_per_step']:.1f} ms/step")
    t0 = time.time()
    out["diff_256x256"] = rollout("diff_256x256", 1.0, 200, 1, 1)
    out["diff_256x256"]["seconds"] = time.time() - t0
    return out


def scenes_at_residual(s2, mem, cfg, flush, tol=1e-6, cap=2000, steps=5, warmup=8):
    """The batched scenes solved per scene to the residual tolerance: pj.alpha everywhere against
    the autotuner's per-scene alpha (gpu.tune_alpha). The untimed first steps hold the shape
    autotuner's trial steps and the alpha tuner's trial solves."""
    import numpy as np
    from cardillocxx_gb300 import PhysicsEngine
    ns = int(s2["num_scenes"])
    out = {"residual_tol": tol, "sweep_cap": cap}
    for name, over in (("alpha_fixed", {}), ("alpha_tuned", {"gpu.tune_alpha": True})):
        e = PhysicsEngine(dict(cfg, **{"gpu.precision": "split", "gpu.residual_tol": tol, "pj.max_iterations": cap},
                               **over)).load_scene(s2).set_contacts(mem)
        ms, it, con, res, _ = time_engine(e, steps, warmup, flush)
        info = e.scene_solve(ns)
        sw = info["sweeps"]
        out[name] = {"ms_per_step": sum(ms) / len(ms), "residual_max": max(res), "max_sweeps": int(sw.max()),
                     "mean_scene_sweeps": float(sw.mean()), "scenes_at_cap": int((sw >= cap).sum()),
                     "steps": steps, "warmup_steps": warmup}
        if name == "alpha_tuned":
            a = info["alpha"]
            out[name]["alpha_counts"] = {f"{v:g}": int((np.abs(a - v) < 1e-6).sum()) for v in np.unique(a)}
        e.close()
        log(f"batch_4096 at residual {tol:g}, {name}: {out[name]['ms_per_step']:.2f} ms/step, mean scene sweeps "
            f"{out[name]['mean_scene_sweeps']:.1f}, at cap {out[name]['scenes_at_cap']}")
    out["tuned_speedup"] = out["alpha_fixed"]["ms_per_step"] / out["alpha_tuned"]["ms_per_step"]
    return out


def rollout(name, scale, T, warmup, steps, rank=0, world=1):
    """The differentiation workload: forward with checkpoints every 20 steps, a COM loss on the final
    state, gradients w.r.t. the initial state and the per-scene friction through the adjoint (this
    rank's share of the scenes when world > 1)."""
    import numpy as np
    from cardillocxx_gb300 import scenes, shard
    from cardillocxx_gb300.adjoint import Rollout
    s = scenes.generate(name, scale=scale)
    totals = (int(s["num_scenes"]), int(s["pos"].shape[0]))
    keep = np.arange(totals[0])
    if world > 1:
        s, keep, _ = shard.rank_shard(s, rank, world)
    cfg = scenes.config_for(name)
    nsc = int(s["num_scenes"])
    sc, m = s["body_scene"], s["mass"]
    M = np.bincount(sc, weights=m, minlength=nsc)
    target = np.random.default_rng(6).uniform((0.2, 0.2, 0.1), (0.8, 0.8, 0.5), size=(totals[0], 3))[keep]
    R = Rollout(s, cfg, checkpoint_every=20)
    mu = np.full(nsc, 0.3)
    fwd, bwd = [], []
    for k in range(warmup + steps):
        t0 = time.perf_counter()
        xT, _, _ = R.forward(T, s["pos"], s["vel"], s["omega"], mu)
        t1 = time.perf_counter()
        com = np.stack([np.bincount(sc, weights=m * xT[:, q], minlength=nsc) for q in range(3)], 1) / M[:, None]
        gx = 2 * (com - target)[sc] * (m / M[sc])[:, None]
        t2 = time.perf_counter()
        R.backward(gx, np.zeros_like(gx), np.zeros_like(gx))
        t3 = time.perf_counter()
        if k >= warmup:
            fwd.append(1e3 * (t1 - t0))
            bwd.append(1e3 * (t3 - t2))
        log(f"rollout {k}: forward {1e3 * (t1 - t0):.1f} ms, adjoint {1e3 * (t3 - t2):.1f} ms")
    return {"scenes": nsc, "bodies": int(s["pos"].shape[0]), "scenes_total": totals[0], "bodies_total": totals[1],
            "rollout_steps": T, "checkpoint_every": 20, "forward_ms": float(np.median(fwd)),
            "adjoint_ms": float(np.median(bwd)), "info": R.info()}


# ---------------------------------------------------------------------------------------- arms
def run_cdx(a):
    import torch
    from cardillocxx_gb300 import PhysicsEngine, scenes

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    hbm, peak_kind = peaks()
    scene, cfg, desc, input_name = workload_input(a)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    mem = None
    if scene is None:
        # a generated scene: the batched presets shard by scene across ranks (no exchange while they
        # step); a single pile runs as replicas
        scene = scenes.generate(a.scene, scale=a.scale)
        if world > 1 and int(scene.get("num_scenes", 1)) > 1:
            from cardillocxx_gb300 import shard
            scene, _, _ = shard.rank_shard(scene, rank, world)
        settle = a.settle if a.settle is not None else scenes.PRESETS[a.scene]["steps"]
        input_name = f"generated, settled {settle} steps by the split form on the GPU"
        desc = f"seeded {a.scene} (scale {a.scale}) {input_name}"
        if settle > 0:
            # a pinned shape runs the settle too (a profiler then counts its launches exactly)
            pin = None
            if a.sweep_variant is not None:
                names = PhysicsEngine.split_variants()
                pin = {"gpu.sweep_variant": names.index(a.sweep_variant) if a.sweep_variant in names
                       else int(a.sweep_variant)}
            state, mem = settle_gpu(scene, cfg, settle, "split", pin)
            scene = with_state(scene, state)
    N = scene["pos"].shape[0]
    shared = shared_config(a, scene, cfg, input_name)
    run_cfg = dict(cfg, **{"gpu.precision": a.precision, "gpu.graph": not a.no_graph})
    for kv in a.set:
        k, _, v = kv.partition("=")
        run_cfg[k.strip()] = v.strip()
    if a.sweep_variant is not None:
        names = PhysicsEngine.split_variants()
        v = a.sweep_variant
        run_cfg["gpu.sweep_variant"] = names.index(v) if v in names else int(v)
    if world > 1:
        torch.distributed.barrier()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    eng = PhysicsEngine(run_cfg).load_scene(scene)
    if mem is not None:
        eng.set_contacts(mem)
    ms, iters, contacts, res, launches = time_engine(eng, a.steps, a.warmup, flush)
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
    roofline = roofline_of(eng, a.precision, contacts[-1], N, hbm, peak_kind)

    # e2e through the C ABI: state uploaded from pinned host memory and read back every step
    e2e = None
    if not a.no_e2e:
        st0 = eng.state()
        pins = {k: torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy() for k, v in st0.items()}
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

    # plain FP64 GPU method over the same warm-up and timed steps: bit-identical to the oracle, so
    # its final state digest is the reference arm's
    plain = None
    n64 = a.fp64_steps if a.fp64_steps is not None else a.steps
    if a.precision == "split" and n64 > 0:
        e64 = PhysicsEngine(dict(cfg, **{"gpu.precision": "fp64"})).load_scene(scene)
        if mem is not None:
            e64.set_contacts(mem)
        ms64, it64, c64, r64, _ = time_engine(e64, n64, a.warmup, flush)
        m64 = sum(ms64) / len(ms64)
        plain = {"ms_per_step": m64, "steps": n64, "contact_iters_per_s": sum(c * i for c, i in zip(c64, it64)) /
                 (sum(ms64) / 1e3), "iterations": it64[-1], "residual": r64[-1], "contacts": c64[-1],
                 "speedup_of_split": m64 / ms_step, "state_digest": scenes.state_digest(e64.state()),
                 "state_after_steps": a.warmup + n64}
        if c64[-1] > 0:
            t64 = e64.time_sweeps(5)
            plain["contact_kernel_ms"] = t64["ms_contact"]
            plain["contact_kernel_gbs"] = t64["bytes_contact"] / (t64["ms_contact"] * 1e-3) / 1e9
        e64.close()
        log(f"fp64 plain: {m64:.3f} ms/step ({m64 / ms_step:.1f}x the split form), state {plain['state_digest']}")

    serr = None
    at_res, cpu_res, s2m = None, None, None
    if a.scene == "pile_200k" and not a.no_residual_leg and rank == 0:
        at_res, s2, mem2 = at_residual_leg(a, scene, cfg, flush)
        s2m = (s2, mem2)
        if a.precision == "split" and {"split", "fp64"} <= set(a.residual_forms.split(",")):
            serr = split_error(s2, mem2, cfg)
    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cpu = cpu_baseline(scene, cfg, a.cpu_seconds, steps=a.cpu_steps)
        if s2m is not None and "split" in at_res:
            cpu_res = cpu_at_residual(s2m[0], s2m[1], cfg, a)
            at_res["cpu"] = cpu_res
            # one CPU step against the GPU forms' averages: compare the rates of contact-iterations
            at_res["split_over_cpu_contact_iters"] = at_res["split"]["contact_iters_per_s"] / cpu_res["contact_iters_per_s"]
    work = None
    if a.scene == "pile_200k" and not a.no_workloads and rank == 0 and world == 1:
        work = other_workloads(flush)

    sharded = world > 1 and int(scene.get("num_scenes", 1)) > 1
    out = {"metric": METRIC, "value": ms_step, "unit": "ms/step", "n_gpus": world, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": False,
           "scaling": "strong" if sharded else "weak",
           "vs_baseline": None, "dtype": "f32-contact/f64-state" if a.precision == "split" else "f64",
           "data": f"synthetic: {desc}", "config": shared,
           "contacts": contacts[-1], "iterations_per_step": iters[-1], "residual": res[-1],
           "precision": a.precision, "l2": "flushed between timed steps (256 MiB write outside the timed events)",
           "contact_variant": est.get("contact_variant"), "autotune_runs": est.get("autotune_runs"),
           "parallelism": ("scene shards" if sharded else "replicas") if world > 1 else "single",
           "contact_iters_per_s": cit * (world if world > 1 else 1), "roofline": roofline,
           "plain_fp64": plain, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk,
           "split_error": serr, "at_residual": at_res, "workloads": work}
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_reference(a):
    """The reference path's CPU implementation (the oracle port, all host threads) on the same input
    and steps. Loads no code of the GPU library: the scene comes from the input file via NumPy."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from cardillocxx_gb300 import scenes
    scene, cfg, desc, input_name = workload_input(a)
    if scene is None:
        print(json.dumps({"impl": "reference", "unavailable": f"--scene {a.scene} has no committed input; only the "
                          "GPU arm can settle a generated scene"}), flush=True)
        return
    from oracle import oracle
    oracle.build()
    threads = os.cpu_count() or 1
    o = oracle.Oracle(scene, cfg, omp_mode=1, num_threads=threads)
    t0 = time.perf_counter()
    if a.warmup:
        o.step(a.warmup)
    first = o.stats()["num_contacts"]
    t1 = time.perf_counter()
    o.step(a.steps)
    ms = (time.perf_counter() - t1) * 1e3 / a.steps
    st = o.stats()
    digest = scenes.state_digest(o.state())
    log(f"reference (oracle port): {ms:.1f} ms/step, contacts {st['num_contacts']}, state {digest} "
        f"(warm-up {time.perf_counter() - t0 - ms * a.steps / 1e3:.1f} s)")
    out = {"metric": METRIC, "value": ms, "unit": "ms/step", "impl": "reference", "n_gpus": 1, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": f"synthetic: {desc}", "config": shared_config(a, scene, cfg, input_name),
           "contacts": st["num_contacts"], "contacts_after_warmup": first, "iterations_per_step": st["iterations"],
           "residual": st["residual"], "state_digest": digest, "state_after_steps": a.warmup + a.steps,
           "implementation": "CPU restatement of the reference path (the reference needs Eigen, EnTT and coal, "
                             "absent here); OpenMP over all host threads",
           "cpu_baseline": {"value": ms, "unit": "ms/step", "cores": threads, "kind": "port", "cpu_model": cpu_model(),
                            "sample": f"{a.steps} full steps after {a.warmup} warm-up steps"},
           "e2e": {"value": ms, "unit": "ms/step", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_adjoint(a):
    """Only the differentiation workload, as one JSON line. Under torchrun the scenes shard across
    the ranks (they do not interact); every rank rolls out its share and the slowest rank's times
    are the job's."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(0)
        dist.init_process_group("nccl", init_method="env://")
    name = a.scene if a.scene != "pile_200k" else "diff_256x256"
    r = rollout(name, a.scale, a.rollout_steps, a.warmup, a.steps, rank=rank, world=world)
    fwd, adj = r["forward_ms"], r["adjoint_ms"]
    if world > 1:
        t = torch.tensor([fwd, adj], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        fwd, adj = float(t[0]), float(t[1])
    if rank == 0:
        print(json.dumps({"metric": "differentiable rollout ms (forward with checkpoints + adjoint)",
                          "value": fwd + adj, "unit": "ms", "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
                          "higher_is_better": False, "scaling": "strong" if world > 1 else "weak", "dtype": "f64",
                          "data": f"synthetic: seeded {name}",
                          "config": {"workload": name, "scenes": r["scenes_total"], "bodies": r["bodies_total"],
                                     "rollout_steps": r["rollout_steps"], "checkpoint_every": 20,
                                     "parallelism": "scene shards" if world > 1 else "single", "info": r["info"]},
                          "forward_ms": fwd, "adjoint_ms": adj}), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    a = parse()
    if a.gpus > 1 and "LOCAL_RANK" in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]
    if a.impl == "reference":
        run_reference(a)
        return
    import __graft_entry__
    __graft_entry__.build()
    if a.adjoint:
        run_adjoint(a)
    else:
        run_cdx(a)


if __name__ == "__main__":
    main()
