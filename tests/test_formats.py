"""The reference's on-disk formats (checkpoint .sav, contour/curv/mag_pressure.out, collider.out): Python
round trips, and the C++ codec (include/sfgpu_io.hpp) reading and rewriting Python-written files byte for byte."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, pkg


def _fmt():
    import importlib
    return importlib.import_module(pkg().__name__ + ".formats")


def _checkpoint(g, seed):
    F = _fmt()
    rng = np.random.default_rng(seed)
    return F.Checkpoint([rng.standard_normal(g.face_shape(a)) for a in range(3)], rng.standard_normal(g.shape),
                        0.123, -1e-5, 2e-6, 4321, [("Advect", 10, 0.01, 0.02), ("Project", 10, 0.5, 0.75)])


def test_checkpoint_roundtrip(tmp_path):
    F, sf = _fmt(), pkg()
    g = sf.StaggeredGrid.from_origin(1.0 / 9, (9, 7, 5))
    ck = _checkpoint(g, 1)
    F.write_checkpoint(tmp_path / "a.sav", g, ck)
    size = os.path.getsize(tmp_path / "a.sav")
    nfaces = sum(int(np.prod(g.face_shape(a))) for a in range(3))
    assert size == 8 * (nfaces + g.num_cells) + 3 * 8 + 4 + 8 + len(b"Advect\0Project\0") + 2 * (4 + 8 + 8)
    back = F.read_checkpoint(tmp_path / "a.sav", g)
    for a in range(3):
        assert np.array_equal(back.velocity[a], ck.velocity[a])
    assert np.array_equal(back.level_set, ck.level_set)
    assert (back.init_volume, back.cumul_vol_error, back.vol_error, back.max_mesh_size) == (0.123, -1e-5, 2e-6, 4321)
    assert back.timings == ck.timings
    with pytest.raises(ValueError):
        F.read_checkpoint(tmp_path / "a.sav", sf.StaggeredGrid.from_origin(1.0 / 10, (10, 7, 5)))


def test_mesh_and_collider_roundtrip(tmp_path):
    F = _fmt()
    rng = np.random.default_rng(2)
    pos, nrm = rng.random((50, 3)), rng.standard_normal((50, 3))
    idx = rng.integers(0, 50, 60)
    pm = rng.random(50)
    F.write_mesh(tmp_path / "contour.out", pos, nrm, idx)
    F.write_mesh(tmp_path / "mag_pressure.out", pos, nrm, idx, pm)
    c = F.read_mesh(tmp_path / "contour.out", False)
    m = F.read_mesh(tmp_path / "mag_pressure.out", True)
    assert os.path.getsize(tmp_path / "contour.out") == 4 + 50 * 24 + 4 + 60 * 4
    for r in (c, m):
        assert np.array_equal(r.positions, pos.astype(np.float32)) and np.array_equal(r.indices, idx)
    assert c.values is None and np.array_equal(m.values, pm.astype(np.float32))
    F.write_collider(tmp_path / "collider.out", pos[:7], nrm[:7])
    p2, n2 = F.read_collider(tmp_path / "collider.out")
    assert np.array_equal(p2, pos[:7].astype(np.float32)) and np.array_equal(n2, nrm[:7].astype(np.float32))


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs a C++ compiler")
def test_cpp_codec_agrees(tmp_path):
    F, sf = _fmt(), pkg()
    exe = tmp_path / "io_roundtrip"
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "io_roundtrip.cpp"), "-o", str(exe)])
    g = sf.StaggeredGrid.from_origin(1.0 / 6, (6, 5, 4))
    F.write_checkpoint(tmp_path / "in.sav", g, _checkpoint(g, 3))
    rng = np.random.default_rng(4)
    F.write_mesh(tmp_path / "in_mag_pressure.out", rng.random((20, 3)), rng.random((20, 3)),
                 rng.integers(0, 20, 30), rng.random(20))
    subprocess.check_call([str(exe), str(tmp_path), "6", "5", "4"])
    assert open(tmp_path / "in.sav", "rb").read() == open(tmp_path / "out.sav", "rb").read()
    assert open(tmp_path / "in_mag_pressure.out", "rb").read() == \
        open(tmp_path / "out_mag_pressure.out", "rb").read()
