"""The FP64 form with row activity: rows without an active cell (air in the pressure system) are skipped on every
level by the smoothers, transfers and Krylov kernels, as in the mixed form.  Skipped rows hold zeros in every
vector and would contribute exact zeros to every sum, so the answer is bit-identical to sweeping every row
(full_sweeps = 1), on the pressure (most rows air) and the potential (every row active)."""
import numpy as np
import pytest

from conftest import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [32, 40])
def test_fp64_row_skipping_same_bits(sfpkg, gpu_ctx, n):
    sc = scenes().pool_sphere(n, seed=6)
    out = {}
    for full in (0, 1):
        v = [a.copy() for a in sc.vel]
        P = sfpkg.Pressure(sc.grid, gpu_ctx)
        sp = P.project(v, sc.phi, sc.frac, opts=sfpkg.options("pressure", precision="fp64", full_sweeps=full))
        M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, gpu_ctx)
        sm = M.solve(sc.phi, sc.hext, opts=sfpkg.options("magnetic", precision="fp64", full_sweeps=full,
                                                         warm_start=0))
        assert sp["converged"] == 1 and sm["converged"] == 1
        out[full] = (P.pressure.copy(), [a.copy() for a in v], M.potential.copy(), sp["iters"], sm["iters"])
    assert np.array_equal(out[0][0], out[1][0])
    for a in range(3):
        assert np.array_equal(out[0][1][a], out[1][1][a])
    assert np.array_equal(out[0][2], out[1][2])
    assert out[0][3:] == out[1][3:]
