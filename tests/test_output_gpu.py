"""Frame output (VTK XML PolyData + ParaView collections, tracked CSV) written by the engine's
background writer, read back and compared with the engine's own state and contacts (GPU tests)."""
import base64
import csv
import os
import re
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from cardillocxx_gb300 import PhysicsEngine, scenes

pytestmark = pytest.mark.gpu

TYPES = {"Float32": np.float32, "Int32": np.int32, "Int64": np.int64}


def read_vtp(path):
    """Points, point arrays and cells of a binary-inline (UInt64 header, uncompressed) .vtp file."""
    root = ET.parse(path).getroot()
    assert root.get("type") == "PolyData" and root.get("header_type") == "UInt64"
    piece = root.find("PolyData/Piece")

    def arr(el):
        raw = base64.b64decode(el.text.strip())
        nbytes = int(np.frombuffer(raw[:8], np.uint64)[0])
        assert nbytes == len(raw) - 8
        a = np.frombuffer(raw[8:], TYPES[el.get("type")])
        nc = int(el.get("NumberOfComponents", "1"))
        return a.reshape(-1, nc) if nc > 1 else a

    out = {"npoints": int(piece.get("NumberOfPoints")), "nverts": int(piece.get("NumberOfVerts")),
           "npolys": int(piece.get("NumberOfPolys"))}
    out["points"] = arr(piece.find("Points/DataArray"))
    out["data"] = {el.get("Name"): arr(el) for el in piece.findall("PointData/DataArray")}
    for kind in ("Verts", "Polys"):
        els = {el.get("Name"): arr(el) for el in piece.findall(f"{kind}/DataArray")}
        out[kind.lower()] = (els["connectivity"], els["offsets"])
    return out


def read_pvd(path):
    root = ET.parse(path).getroot()
    return [(float(d.get("timestep")), d.get("file")) for d in root.iter("DataSet")]


@pytest.mark.parametrize("precision", ["fp64", "split"])
def test_frames_collections_and_tracked_csv(gpu, tmp_path, precision):
    s = scenes.generate("pile_1k", scale=0.1)
    dt = 5e-4
    cfg = scenes.config_for("pile_1k", **{"gpu.precision": precision, "output.interval_steps": 5,
                                          "output.folder": str(tmp_path), "output.filename_prefix": "pile",
                                          "sim.dt": dt})
    eng = PhysicsEngine(cfg).load_scene(s)
    eng.track(3, "three")
    eng.track(7, "seven")
    N = s["pos"].shape[0]
    S = len(s["static_kind"])
    states, contacts = {}, {}
    for k in range(12):
        eng.step(1)
        st = eng.state()
        states[k + 1] = st
        if (k + 1) % 5 == 0:
            contacts[k + 1] = eng.contacts()
    eng.flush_output()
    files = sorted(os.listdir(tmp_path))
    assert "pile_static_geo.vtp" in files and "pile_geo.pvd" in files and "pile_tracked.csv" in files
    # frames at steps 0 (before the first step), 5 and 10; the collection lists them with their times
    pvd = read_pvd(tmp_path / "pile_geo.pvd")
    assert [f for _, f in pvd] == ["pile_geo_0000.vtp", "pile_geo_0005.vtp", "pile_geo_0010.vtp"]
    np.testing.assert_allclose([t for t, _ in pvd], [0.0, 5 * dt, 10 * dt], rtol=1e-5)
    f0 = read_vtp(tmp_path / "pile_geo_0000.vtp")
    np.testing.assert_array_equal(f0["points"], s["pos"].astype(np.float32))
    for step in (5, 10):
        g = read_vtp(tmp_path / f"pile_geo_{step:04d}.vtp")
        st = states[step]
        assert g["npoints"] == N and g["nverts"] == N and g["npolys"] == 0
        np.testing.assert_array_equal(g["points"], st["pos"].astype(np.float32))
        np.testing.assert_array_equal(g["data"]["velocity"], st["vel"].astype(np.float32))
        np.testing.assert_array_equal(g["data"]["angular_velocity"], st["omega"].astype(np.float32))
        np.testing.assert_array_equal(g["data"]["entity_id"], np.arange(N) + S)
        np.testing.assert_array_equal(g["data"]["radius"], s["radius"].astype(np.float32))
        conn, off = g["verts"]
        np.testing.assert_array_equal(conn, np.arange(N))
        np.testing.assert_array_equal(off, np.arange(1, N + 1))
        # pressure: the compressive forces over each sphere's area (enrichPressure)
        c = contacts[step]
        force = np.zeros(N)
        pn = np.maximum(c["lambda"][:, 0], 0) / dt
        for ids in (c["id_a"], c["id_b"]):
            m = ids >= S
            np.add.at(force, ids[m] - S, pn[m])
        np.testing.assert_allclose(g["data"]["entity_pressure"], force / (4 * np.pi * s["radius"] ** 2), rtol=1e-5,
                                   atol=1e-3)
        # contact frame
        m = read_vtp(tmp_path / f"pile_contact_manifolds_{step:04d}.vtp")
        assert m["npoints"] == len(c["id_a"])
        np.testing.assert_array_equal(m["points"], c["point"].astype(np.float32))
        np.testing.assert_array_equal(m["data"]["normal"], c["normal"].astype(np.float32))
        np.testing.assert_array_equal(m["data"]["id_a"], c["id_a"])
        np.testing.assert_array_equal(m["data"]["id_b"], c["id_b"])
        np.testing.assert_allclose(m["data"]["pn"], np.maximum(c["lambda"][:, 0], 0), rtol=1e-6)
        t1, t2 = m["data"]["tangent1"], m["data"]["tangent2"]
        np.testing.assert_allclose(np.einsum("ij,ij->i", t1, m["data"]["normal"]), 0, atol=1e-6)
        np.testing.assert_allclose(np.linalg.norm(t2, axis=1), 1, atol=1e-6)
        per = m["data"]["percussion"]
        np.testing.assert_allclose(np.einsum("ij,ij->i", per, m["data"]["normal"]), m["data"]["pn"], rtol=1e-4,
                                   atol=1e-9)
        assert np.all(m["data"]["penetration"] > -0.05)
    # static geometry: one square patch (two triangles) for the ground
    sg = read_vtp(tmp_path / "pile_static_geo.vtp")
    assert sg["npolys"] == 2 * S and sg["npoints"] == 4 * S
    # tracked CSV: header, two rows a step, time and state of the tracked spheres
    rows = list(csv.reader(open(tmp_path / "pile_tracked.csv")))
    assert rows[0] == ["t", "name", "px", "py", "pz", "vx", "vy", "vz", "wx", "wy", "wz",
                       "euler_x", "euler_y", "euler_z"]
    assert len(rows) == 1 + 2 * 12
    for k in range(12):
        for j, (body, name) in enumerate(((3, "three"), (7, "seven"))):
            r = rows[1 + 2 * k + j]
            assert r[1] == name
            assert float(r[0]) == pytest.approx((k + 1) * dt, rel=1e-5)
            st = states[k + 1]
            np.testing.assert_allclose([float(x) for x in r[2:5]], st["pos"][body], rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose([float(x) for x in r[5:8]], st["vel"][body], rtol=1e-5, atol=1e-6)
            np.testing.assert_allclose([float(x) for x in r[8:11]], st["omega"][body], rtol=1e-5, atol=1e-6)


def test_drum_static_geometry_and_no_output_by_default(gpu, tmp_path):
    s = scenes.generate("drum_1m", scale=0.0002)
    cfg = scenes.config_for("drum_1m", **{"output.interval_steps": 3, "output.folder": str(tmp_path / "d"),
                                          "output.write_contact_manifolds": False})
    eng = PhysicsEngine(cfg).load_scene(s)
    eng.step(4)
    eng.flush_output()
    files = sorted(os.listdir(tmp_path / "d"))
    assert files == ["scene_geo.pvd", "scene_geo_0000.vtp", "scene_geo_0003.vtp", "scene_static_geo.vtp"]
    sg = read_vtp(tmp_path / "d" / "scene_static_geo.vtp")
    # the drum wall (64 segments, two triangles each) and the two end walls (two triangles each)
    assert list(s["static_kind"]) == [1, 0, 0]
    assert sg["npolys"] == 128 + 4 and sg["npoints"] == 128 + 8
    np.testing.assert_array_equal(sg["data"]["entity_id"], [0] * 128 + [1] * 4 + [2] * 4)
    R = float(s["static_radius"][0])
    axis = s["static_dir"][0] / np.linalg.norm(s["static_dir"][0])
    r = sg["points"][:128] - s["static_pos"][0]
    radial = np.linalg.norm(r - np.outer(r @ axis, axis), axis=1)
    np.testing.assert_allclose(radial, R, rtol=1e-5)
    # without output.interval_steps nothing is written
    eng2 = PhysicsEngine(scenes.config_for("drum_1m", **{"output.folder": str(tmp_path / "none")})).load_scene(s)
    eng2.step(2)
    eng2.flush_output()
    assert not os.path.exists(tmp_path / "none") or not os.listdir(tmp_path / "none")
