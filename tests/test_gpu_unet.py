"""GPU tests of the learned part: the U-Net's tensor-core forward and backward kernels against the numpy
reference (oracle/unet_ref.py, with the same BF16 rounding points), training, and the learned solve with its
fallback.  Tolerances: relative L2 1e-2 on outputs and 3e-2 on per-layer gradients (BF16 activations; the
reference accumulates in FP64, the kernels in FP32)."""
import numpy as np
import pytest

from conftest import oracle_grid, rel_l2, scenes

pytestmark = pytest.mark.gpu


def _grid(sf, shape):
    return sf.StaggeredGrid.from_origin(1.0 / shape[0], shape)


@pytest.fixture(scope="module")
def ref():
    from oracle import unet_ref
    return unet_ref


@pytest.mark.parametrize("shape", [(8, 8, 8), (11, 6, 13)])
def test_unet_forward_matches_reference(sfpkg, gpu_ctx, ref, shape):
    import torch
    g = _grid(sfpkg, shape)
    P = ref.init_params(16, seed=3)
    rng = np.random.default_rng(1)
    P["e0a.b"] = rng.normal(0, 0.1, 16).astype(np.float32)
    P["d1a.b"] = rng.normal(0, 0.1, 32).astype(np.float32)
    x = ref.bf16(rng.standard_normal(shape + (16,)))
    out_ref, _ = ref.forward_bf16(P, x)
    net = sfpkg.Network(gpu_ctx)
    assert net.num_params == ref.flatten(P).size
    net.set_params(ref.flatten(P))
    feat = torch.from_numpy(x).to(torch.bfloat16).cuda().contiguous()
    out = torch.zeros(g.num_cells, dtype=torch.float32, device="cuda")
    net.forward(g, feat, out)
    torch.cuda.synchronize()
    assert rel_l2(out.cpu().numpy(), out_ref.ravel()) <= 1e-2
    net.close()


def test_unet_gradients_match_reference(sfpkg, gpu_ctx, ref):
    import torch
    shape = (10, 8, 12)
    g = _grid(sfpkg, shape)
    P = ref.init_params(16, seed=5)
    rng = np.random.default_rng(2)
    x = ref.bf16(rng.standard_normal(shape + (16,)))
    dout = rng.standard_normal(shape).astype(np.float32)
    out_ref, cache = ref.forward_bf16(P, x)
    G = ref.backward_bf16(P, cache, dout.astype(np.float64))
    net = sfpkg.Network(gpu_ctx)
    net.set_params(ref.flatten(P))
    feat = torch.from_numpy(x).to(torch.bfloat16).cuda().contiguous()
    grads = ref.unflatten(net.gradients(g, feat, torch.from_numpy(dout).cuda()))
    for name, *_ in ref.LAYERS:
        for k in (".w", ".b"):
            a, b = grads[name + k], np.asarray(G[name + k]).reshape(grads[name + k].shape)
            if np.linalg.norm(b) == 0:
                continue
            assert rel_l2(a, b) <= 3e-2, (name + k, rel_l2(a, b))
    net.close()


def test_unet_training_reduces_loss(sfpkg, gpu_ctx, ref):
    """Adam on the cosine loss fits a smooth target of the input on one small volume."""
    import torch
    shape = (16, 16, 16)
    g = _grid(sfpkg, shape)
    rng = np.random.default_rng(7)
    x = ref.bf16(rng.standard_normal(shape + (16,)) * 0.5)
    t = (x[..., 0] + 0.5 * np.roll(x[..., 1], 1, axis=0)).astype(np.float32)
    net = sfpkg.Network(gpu_ctx)
    net.set_params(ref.flatten(ref.init_params(16, seed=9)))
    feat = torch.from_numpy(x).to(torch.bfloat16).cuda().contiguous()
    tgt = torch.from_numpy(t).cuda().contiguous()
    losses = [net.train_step(g, feat, tgt, 2e-3) for _ in range(80)]
    assert np.isfinite(losses).all()
    assert losses[-1] < 0.5 * losses[0]
    net.close()


def test_learned_solve_converges_and_falls_back(sfpkg, oracle, gpu_ctx, ref):
    """The learned form reaches the same tolerance and answer as the plain method; a network whose
    prediction is garbage takes no step (SF_STALLED_FALLBACK) and the plain iteration finishes the solve."""
    sc = scenes().pool(32, seed=4)
    og = oracle_grid(oracle, sc.grid)
    u_or, p_or, _ = oracle.pressure_project(og, sc.phi, sc.frac, sc.vel, tol=1e-13)
    liq = sc.phi <= 0
    net = sfpkg.Network(gpu_ctx)
    net.set_params(ref.flatten(ref.init_params(16, seed=1)))
    gpu_ctx.set_network(net)
    P = sfpkg.Pressure(sc.grid, gpu_ctx)
    v = [a.copy() for a in sc.vel]
    st = P.project(v, sc.phi, sc.frac, opts=sfpkg.options("pressure", precision="learned"))
    assert st["converged"] == 1 and st["rel_residual"] <= 1e-8 * 1.01
    assert rel_l2(P.pressure[liq], p_or[liq]) <= 1e-5
    assert st["guess_rel_residual"] >= 0 and st["learned_steps"] >= 1
    assert 0.0 <= st["guess_energy_ratio"] <= 1.0 + 1e-9  # gamma scaling: never worse than zero in A-norm
    # garbage network: huge weights make the prediction overflow to non-finite values -> discarded
    flat = ref.flatten(ref.init_params(16, seed=1))
    flat[:] = 1e30
    net.set_params(flat)
    v = [a.copy() for a in sc.vel]
    st = P.project(v, sc.phi, sc.frac, opts=sfpkg.options("pressure", precision="learned"))
    assert P.status == sfpkg._abi.SF_STALLED_FALLBACK
    assert st["converged"] == 1 and rel_l2(P.pressure[liq], p_or[liq]) <= 1e-5
    assert st["learned_steps"] == 1  # stalled after its first step: the rest is the plain iteration
    gpu_ctx.set_network(None)
    net.close()


def test_trained_network_gain(sfpkg, gpu_ctx, ref):
    """The trained weights (weights/unet.f32) against the same network untrained, on unseen seeded scenes of
    the training distribution (pool of depth U[0.1, 0.3] with spheres, chi U[0.5, 3]) at 64^3: the first learned
    step's A-norm error relative to zero (guess_energy_ratio) is lower with the trained weights on the
    potential, and every learned solve reaches the tolerance.  The measured figures are printed."""
    import os
    S = scenes()
    wpath = os.path.join(os.path.dirname(sfpkg.__file__), "weights", "unet.f32")
    trained = sfpkg.Network(gpu_ctx)
    trained.load(wpath)
    untrained = sfpkg.Network(gpu_ctx)
    untrained.set_params(ref.flatten(ref.init_params(16, seed=5)))
    rows = []
    for seed in (101, 102, 103):
        sc = S.random_scene(64, seed=seed)
        for name, net in (("trained", trained), ("untrained", untrained)):
            gpu_ctx.set_network(net)
            M = sfpkg.MagneticField(sc.grid, sc.chi, sc.band_width, gpu_ctx)
            sm = M.solve(sc.phi, sc.hext, opts=sfpkg.options("magnetic", precision="learned", warm_start=0))
            P = sfpkg.Pressure(sc.grid, gpu_ctx)
            sp = P.project([a.copy() for a in sc.vel], sc.phi, sc.frac,
                           opts=sfpkg.options("pressure", precision="learned"))
            assert sm["converged"] == 1 and sp["converged"] == 1
            rows.append((seed, name, sm["guess_energy_ratio"], sm["iters"], sp["guess_energy_ratio"], sp["iters"]))
    gpu_ctx.set_network(None)
    for r in rows:
        print("seed %d %-9s potential energy ratio %.4f iters %d | pressure energy ratio %.4f iters %d" % r)
    tr = np.mean([r[2] for r in rows if r[1] == "trained"])
    un = np.mean([r[2] for r in rows if r[1] == "untrained"])
    assert tr < un and tr < 1.0, (tr, un)
    trained.close()
    untrained.close()


def test_network_outlives_context(sfpkg):
    """Destroying the context before its network leaves the network handle safe to destroy."""
    ctx = sfpkg.Context(0)
    net = sfpkg.Network(ctx)
    ctx.set_network(net)
    lib = ctx.lib
    h = net.handle
    ctx.close()
    assert lib.sf_unet_num_params(h) == 0  # orphaned: no device state left
    net.close()
