"""The C++ mirror of the reference classes (include/sfgpu.hpp) drives the library the way
core/Simulation.cpp drives the reference: MagneticField::Solve, then SetPressureJump + Project, then
Extrapolation::Solve + Collider::Enforce, and the interface coupling from a surface mesh.  Its results must
match the oracle on the same inputs (bit for bit where no solve is involved)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, oracle_grid, rel_l2, scenes
from test_interface import contour

pytestmark = pytest.mark.gpu


def test_cpp_adapter_matches_oracle(oracle, tmp_path):
    exe = tmp_path / "adapter_demo"
    lib_dir = os.path.join(ROOT, "simferrofluid-cuda_gb300")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "adapter_demo.cpp"), "-L" + lib_dir, "-lsfgpu",
                           "-Wl,-rpath," + lib_dir, "-o", str(exe)])
    n, chi = 24, 1.0
    sc = scenes().pool(n, seed=21, chi=chi)
    sc.phi.tofile(tmp_path / "phi.bin")
    for a in range(3):
        sc.vel[a].tofile(tmp_path / f"vel{a}.bin")
        sc.hext[a].tofile(tmp_path / f"hext{a}.bin")
    marks, pos, nrm, _ = contour(sc.grid.shape, sc.grid.spacing, tuple(sc.grid.origin), sc.phi, 31)
    pos.tofile(tmp_path / "pos.bin")
    nrm.tofile(tmp_path / "nrm.bin")
    for a in range(3):
        marks[a].tofile(tmp_path / f"mark{a}.bin")
    out = subprocess.run([str(exe), str(tmp_path), str(n), str(chi), str(pos.shape[0])], capture_output=True,
                         text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    g = sc.grid
    og = oracle_grid(oracle, g)
    rd = lambda name, shape: np.fromfile(tmp_path / name).reshape(shape)  # noqa: E731
    for a in range(3):
        assert np.array_equal(rd(f"frac{a}.bin", g.face_shape(a)), sc.frac[a])
    # the jump the C++ callback returns on liquid-air faces: 0.01 axis + 0.001 face_y
    jump = []
    for a in range(3):
        J = np.zeros(g.face_shape(a))
        J += 0.01 * a + 0.001 * np.arange(g.face_shape(a)[1])[None, :, None]
        jump.append(J)
    u_or, p_or, _ = oracle.pressure_project(og, sc.phi, sc.frac, sc.vel, jump=jump, tol=1e-13)
    liq = sc.phi <= 0
    p = rd("p.bin", g.shape)
    assert rel_l2(p[liq], p_or[liq]) <= 1e-5
    for a in range(3):
        assert np.abs(rd(f"vel_out{a}.bin", g.face_shape(a)) - u_or[a]).max() <= 1e-5 * np.abs(sc.vel[a]).max()
    psi_or, H_or, _ = oracle.magnetic_solve(og, sc.phi, chi, 2 * g.spacing, sc.hext, tol=1e-13)
    assert rel_l2(rd("psi.bin", g.shape), psi_or) <= 1e-5
    # extrapolation + enforce of the projected velocity, bit for bit, and the collider normals
    ls, frac_or, normal_or = oracle.box_collider(og)
    for a in range(3):
        assert np.array_equal(rd(f"normal{a}.bin", g.face_shape(a)), normal_or[a])
    projected = [rd(f"vel_out{a}.bin", g.face_shape(a)) for a in range(3)]
    want = oracle.collider_enforce(og, oracle.extrapolate_velocity(og, projected, sc.phi, sc.frac), sc.frac, normal_or)
    for a in range(3):
        assert np.array_equal(rd(f"vel_post{a}.bin", g.face_shape(a)), want[a])
    # interface coupling: vertex pressures from the solve's H (bit for bit), then the jump and a projection
    H = [rd(f"H{a}.bin", g.face_shape(a)) for a in range(3)]
    pm_or = oracle.vertex_pressures(og, chi, H, pos, nrm)
    assert np.array_equal(np.fromfile(tmp_path / "pm.bin"), pm_or)
    jump2 = oracle.pressure_jump(og, marks, None, pm_or, 0.0, 1.0, 1e-2)
    u2, p2, _ = oracle.pressure_project(og, sc.phi, sc.frac, sc.vel, jump=jump2, tol=1e-13)
    assert rel_l2(rd("p_mesh.bin", g.shape)[liq], p2[liq]) <= 1e-5
