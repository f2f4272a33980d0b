"""CPU-side checks of the C ABI library: it loads, exports every symbol include/cdx.h declares,
parses configs like the reference's ConfigReader, and generates seeded scenes (no GPU calls)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from tests.conftest import HAS_GPU, ROOT


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "cdx.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cdx_[a-z_0-9]+)\s*\(", txt)))


def test_exports_every_declared_symbol(cdxlib):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(cdxlib, s), s


def test_ctypes_bindings_cover_header(cdxlib):
    from cardillocxx_gb300 import _lib
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(header_symbols()) <= bound


def test_struct_sizes_match_header(cdxlib):
    # compile a tiny C program against the header and compare sizeof with the ctypes mirrors
    import subprocess
    import tempfile
    from cardillocxx_gb300 import _lib
    src = '#include <stdio.h>\n#include "cdx.h"\nint main(){printf("%zu %zu %zu %zu\\n", sizeof(cdx_config), ' \
          'sizeof(cdx_scene), sizeof(cdx_stats), sizeof(cdx_gen_params));return 0;}\n'
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "t.c")
        open(p, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), p, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    sizes = [C.sizeof(_lib.CdxConfig), C.sizeof(_lib.CdxScene), C.sizeof(_lib.CdxStats), C.sizeof(_lib.CdxGenParams)]
    assert [int(v) for v in out] == sizes


def test_config_defaults_and_keys(cdxlib):
    from cardillocxx_gb300 import Config
    c = Config()
    # reference defaults (src/config/config.hpp)
    assert c.get("pj_alpha") == 0.3 and c.get("pj_max_iterations") == 200000
    assert c.get("moreau_theta") == 1.0 and c.get("friction_enable") == 0
    assert c.get("sim_gravity") == [0.0, 0.0, -9.81]
    c.set("solver.alpha", "0.5")           # solver. prefix accepted
    c.set("pj.max_iterations", "0")        # clamped to >= 1
    c.set("pj.tol_abs", "garbage")         # unparsable: unchanged
    c.set("friction.enable", "ON")
    c.set("friction.combine", "GEOM")
    c.set("friction.combine", "bogus")     # unknown method: unchanged
    c.set("sim.dt", "-1")                  # must be positive: ignored
    c.set("collision.match_max_dist", "-3")  # clamped at 0
    c.set("some.unknown.key", "1")         # ignored
    c.set("sim.gravity", "0, 0, -1.62")
    assert c.get("pj_alpha") == 0.5 and c.get("pj_max_iterations") == 1
    assert c.get("pj_tol_abs") == 1e-5 and c.get("friction_enable") == 1
    assert c.get("friction_combine") == 2 and c.get("sim_dt") == 1e-3
    assert c.get("collision_match_max_dist") == 0.0
    assert c.get("sim_gravity") == [0.0, 0.0, -1.62]
    # cooperative-solve keys of this build: non-negative integers, 0 = automatic
    assert c.get("gpu_coop_blocks") == 0 and c.get("gpu_coop_smem_contacts") == 0
    c.set("gpu.coop_blocks", "16").set("gpu.coop_smem_contacts", "-5")
    assert c.get("gpu_coop_blocks") == 16 and c.get("gpu_coop_smem_contacts") == 0


def test_config_file_parsing(cdxlib, tmp_path):
    from cardillocxx_gb300 import Config
    p = tmp_path / "scene.config"
    p.write_text("# comment\n  pj.alpha = 0.5   # inline\nmoreau.theta=0.5\nnot a pair\n\n"
                 "pj.relaxation = 0.5\ngpu.precision = split\ngpu.residual_tol = 1e-6\n")
    c = Config.from_file(str(p))
    assert c.get("pj_alpha") == 0.5 and c.get("moreau_theta") == 0.5 and c.get("pj_relaxation") == 0.5
    assert c.get("gpu_precision") == 1 and c.get("gpu_residual_tol") == 1e-6
    missing = Config.from_file(str(tmp_path / "nope.config"))
    assert missing.get("pj_alpha") == 0.3


def test_config_rejects_other_solvers(cdxlib):
    from cardillocxx_gb300 import CdxError, Config, PhysicsEngine
    with pytest.raises(CdxError):
        Config().set("solver.type", "clarabel")
    for name in ("pgs", "projected_gauss_seidel", "ProjectedGaussSeidel"):
        assert Config({"solver.type": name}).get("solver_type") == 2
    c = Config({"solver.type": "condensed"})
    assert c.get("solver_type") == 1 and c.get("condensed_sweep_mode") == 0  # gauss_seidel by default
    assert Config({"condensed.sweep_mode": "colored"}).get("condensed_sweep_mode") == 2
    assert Config({"condensed.sweep_mode": "nonsense"}).get("condensed_sweep_mode") == 0
    # the GPU runs the condensed solver's gauss_seidel, jacobi and colored sweeps in the plain FP64
    # method: the chaotic mode, the split form and its accelerated loops are refused before any
    # device call
    for bad in ({"solver.type": "condensed", "condensed.sweep_mode": "chaotic"},
                {"solver.type": "condensed", "condensed.sweep_mode": "colored", "gpu.precision": "split"},
                {"solver.type": "condensed", "condensed.sweep_mode": "colored", "pj.nesterov": True},
                # projected Gauss-Seidel: its plain loop in the plain FP64 method
                {"solver.type": "pgs", "gpu.precision": "split"},
                {"solver.type": "pgs", "gpu.precision": "fp64", "pj.nesterov": True}):
        with pytest.raises(CdxError) as e:
            PhysicsEngine(bad)
        assert e.value.status == 6


def test_generator_deterministic_and_non_overlapping(cdxlib):
    from cardillocxx_gb300 import scenes
    a = scenes.generate("pile_1k")
    b = scenes.generate("pile_1k")
    for k in ("pos", "radius", "mass"):
        assert np.array_equal(a[k], b[k])
    c = scenes.generate("pile_1k", seed=123)
    assert not np.array_equal(a["pos"], c["pos"])
    p, r = a["pos"], a["radius"]
    d = np.linalg.norm(p[:, None, :] - p[None, :, :], axis=-1)
    np.fill_diagonal(d, np.inf)
    assert (d >= (r[:, None] + r[None, :])).all()
    assert (p[:, 2] >= r).all() and (p[:, :2] >= r[:, None]).all() and (p[:, :2] <= 1 - r[:, None]).all()
    m = a["mass"][0]
    assert m == pytest.approx(1000 * 4 / 3 * np.pi * 0.05 ** 3)
    assert a["inertia"][0] == pytest.approx(0.4 * 0.05 ** 2 * m)
    assert len(a["static_kind"]) == 5


def test_generator_batched_and_drum(cdxlib):
    from cardillocxx_gb300 import scenes
    s = scenes.generate("batch_4096", scale=0.01)
    sc = s["body_scene"]
    assert (np.diff(sc) >= 0).all() and s["num_scenes"] == 41
    counts = np.bincount(sc)
    assert counts.min() >= 16 and counts.max() <= 512
    mus = [s["mu"][sc == k][0] for k in range(s["num_scenes"])]
    assert 0.1 <= min(mus) and max(mus) <= 0.8 and len(set(mus)) > 30
    d = scenes.generate("drum_1m", scale=0.001)
    assert d["static_kind"].tolist() == [1, 0, 0]
    R = d["static_radius"][0]
    rr = np.hypot(d["pos"][:, 1], d["pos"][:, 2]) + d["radius"]
    assert (rr <= R + 1e-12).all()


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device error path")
def test_create_without_device_reports_error(cdxlib):
    from cardillocxx_gb300 import CdxError, PhysicsEngine
    with pytest.raises(CdxError) as e:
        PhysicsEngine({})
    assert "CUDA" in str(e.value) or "cuda" in str(e.value)


def test_acceleration_keys(cdxlib):
    from cardillocxx_gb300.engine import Config
    c = Config()
    assert c.get("pj_nesterov") == 0 and c.get("pj_chebyshev") == 0
    assert c.get("pj_nesterov_beta_threshold") == 1.0 and c.get("pj_nesterov_restart_limit") == 10000
    c.set("pj.nesterov", "on").set("solver.chebyshev", "true").set("pj.nesterov_beta_threshold", 0.9)
    c.set("pj.nesterov_restart_limit", 7)
    assert c.get("pj_nesterov") == 1 and c.get("pj_chebyshev") == 1
    assert c.get("pj_nesterov_beta_threshold") == 0.9 and c.get("pj_nesterov_restart_limit") == 7
    assert c.get("pj_anderson") == 0 and c.get("pj_anderson_m") == 2
    c.set("solver.anderson", "yes").set("pj.anderson_m", 0)
    assert c.get("pj_anderson") == 1 and c.get("pj_anderson_m") == 1  # the window is at least 1
    c.set("pj.anderson_m", 5)
    assert c.get("pj_anderson_m") == 5
    assert c.get("pj_rdiag_true_delassus") == 0
    assert c.set("solver.rdiag_true_delassus", "on").get("pj_rdiag_true_delassus") == 1


def test_split_form_refuses_the_loops_it_does_not_run(cdxlib):
    # the split form runs Nesterov and the standard loop (with its tolerance exit); Chebyshev and
    # Anderson, selected when Nesterov is off (projected_jacobi.cpp:470-491), are refused when the
    # context is created, before any device call, instead of silently running another loop
    from cardillocxx_gb300 import CdxError, PhysicsEngine
    from cardillocxx_gb300._lib import STATUS
    for key in ("pj.chebyshev", "pj.anderson"):
        with pytest.raises(CdxError) as e:
            PhysicsEngine({"gpu.precision": "split", key: True})
        assert e.value.status == 6 and STATUS[6] == "CDX_ERR_UNSUPPORTED"
        assert "plain FP64" in str(e.value)
    from cardillocxx_gb300.engine import Config
    c = Config({"gpu.coop_wait_ns": 5000})
    assert c.get("gpu_coop_wait_ns") == 5000
    assert Config().get("gpu_coop_wait_ns") == 0
    assert Config({"gpu.coop_wait_ns": -1}).get("gpu_coop_wait_ns") == 0  # bad values keep the default


def test_output_keys(cdxlib):
    # output.* keys of the reference (config.hpp:20-23); frames are off unless interval_steps is set
    from cardillocxx_gb300 import CdxError
    from cardillocxx_gb300.engine import Config
    c = Config()
    assert c.get("output_interval_steps") == 0 and c.get("output_write_contact_manifolds") == 1
    assert c.get("output_folder") == b"./vtk_out" and c.get("output_filename_prefix") == b"scene"
    c.set("output.interval_steps", 25).set("output.folder", "/tmp/frames").set("output.filename_prefix", "drum")
    c.set("output.write_contact_manifolds", "off")
    assert c.get("output_interval_steps") == 25 and c.get("output_write_contact_manifolds") == 0
    assert c.get("output_folder") == b"/tmp/frames" and c.get("output_filename_prefix") == b"drum"
    with pytest.raises(CdxError):
        c.set("output.folder", "x" * 300)


def test_reference_adapter_compiles_against_interface_stubs(tmp_path):
    # include/cdx_reference_adapter.hpp only builds inside the reference tree; against stand-ins of
    # the reference interfaces it uses (tests/adapter_stub) it must compile, calls into the C ABI
    # included (syntax only: nothing is linked or run)
    import os
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "adapter_tu.cpp"
    src.write_text('#include "cdx_reference_adapter.hpp"\n'
                   'static cardillo::solver::SolverBase* make(cardillo::physics::DynamicsAssembler& d, '
                   'const cardillo::config::Config& c) { return new cardillo::solver::GpuProjectedJacobiSolver(d, c); }\n'
                   'static cardillo::integration::IntegrationBase* make_int(cardillo::World& w, '
                   'cardillo::solver::SolverBase& s, cardillo::physics::DynamicsAssembler& d, '
                   'cardillo::misc::TimingManager& t, cardillo::config::Config& c) {\n'
                   '  auto* g = new cardillo::integration::GpuMoreauIntegrator(w, s, d, t, c, CDX_PRECISION_SPLIT);\n'
                   '  g->step(1e-3);\n'
                   '  return g; }\n'
                   'int main() { (void)&make; (void)&make_int; return 0; }\n')
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-DCDX_WITH_CARDILLO",
           "-I", os.path.join(root, "include"), "-I", os.path.join(root, "tests", "adapter_stub"), str(src)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
