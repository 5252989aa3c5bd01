"""The tcgen05 (TMA + TMEM) forward convolutions against the warp-level MMA ones and the numpy reference.
Both accumulate in FP32 in different orders and round activations to BF16: relative L2 1e-2."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


# (5, 8, 128) and (8, 12, 256) put the 16-channel layers on the line kernel (a 128 x 6 x 4 box fits the grid;
# at (8, 12, 256) also the 16 -> 32 layer of level 1); (5, 8, 64) and the 64^3-type level of (16, 24, 256) (4 x 6
# x 64, 32 and 64 channels) run the 64-long z-line kernel
@pytest.mark.parametrize("shape", [(2, 4, 32), (6, 12, 40), (17, 9, 64), (5, 8, 128), (8, 12, 256), (5, 8, 64),
                                   (16, 24, 256)])
def test_tcgen05_forward_matches_mma(sfpkg, gpu_ctx, shape):
    import torch
    from oracle import unet_ref as ref
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    P = ref.init_params(16, seed=11)
    rng = np.random.default_rng(3)
    for k in P:
        if k.endswith(".b"):
            P[k] = rng.normal(0, 0.05, P[k].shape).astype(np.float32)
    x = ref.bf16(rng.standard_normal(shape + (16,)))
    net = sfpkg.Network(gpu_ctx)
    net.set_params(ref.flatten(P))
    feat = torch.from_numpy(x).to(torch.bfloat16).cuda().contiguous()
    out0 = torch.zeros(g.num_cells, dtype=torch.float32, device="cuda")
    out1 = torch.zeros_like(out0)
    net.set_mode("mma")
    net.forward(g, feat, out0)
    net.set_mode("tcgen05")
    before = net.tc_launches()
    net.forward(g, feat, out1)
    torch.cuda.synchronize()
    assert net.tc_launches() > before  # the tensor-core path ran for the layers whose grid holds a brick
    a, b = out0.cpu().numpy(), out1.cpu().numpy()
    assert np.isfinite(b).all()
    assert rel_l2(b, a) <= 1e-2
    if np.prod(shape) <= 8192:
        out_ref, _ = ref.forward_bf16(P, x)
        assert rel_l2(b, out_ref.ravel()) <= 1e-2
    net.close()


# shapes on the 27-box kernel (no z-line box fits: ny < 6), whose forward equals the warp-MMA kernel's bit for bit
@pytest.mark.parametrize("shape", [(6, 12, 40), (9, 5, 64)])
def test_tcgen05_gradients_match_mma(sfpkg, gpu_ctx, shape):
    """Training with the tcgen05 kernels: the input gradients of every 3x3x3 layer run on tcgen05 (the forward
    convolution with the mirrored, transposed weights, FP32 out); the parameter gradients agree with the
    warp-MMA path's (relative L2 2e-2: BF16 activations, FP32 sums in different orders)."""
    import torch
    from oracle import unet_ref as ref
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    P = ref.init_params(16, seed=12)
    rng = np.random.default_rng(4)
    x = ref.bf16(rng.standard_normal(shape + (16,)))
    net = sfpkg.Network(gpu_ctx)
    net.set_params(ref.flatten(P))
    feat = torch.from_numpy(x).to(torch.bfloat16).cuda().contiguous()
    dout = torch.from_numpy(rng.standard_normal(int(np.prod(shape))).astype(np.float32)).cuda()
    out = torch.zeros(g.num_cells, dtype=torch.float32, device="cuda")
    net.set_mode("mma")
    net.forward(g, feat, out)
    g0 = net.gradients(g, feat, dout)
    net.set_mode("tcgen05")
    before = net.tc_launches()
    net.forward(g, feat, out)
    g1 = net.gradients(g, feat, dout)
    assert net.tc_launches() - before > 8  # forward and input-gradient convolutions on tcgen05
    assert np.isfinite(g1).all()
    assert rel_l2(g1, g0) <= 2e-2, rel_l2(g1, g0)
    # one Adam step in each mode from the same parameters gives close losses and parameters
    tgt = torch.from_numpy(rng.standard_normal(int(np.prod(shape))).astype(np.float32)).cuda()
    net.set_params(ref.flatten(P))
    net.set_mode("mma")
    l0 = net.train_step(g, feat, tgt, 1e-3)
    p0 = net.get_params()
    net.set_params(ref.flatten(P))
    net.set_mode("tcgen05")
    l1 = net.train_step(g, feat, tgt, 1e-3)
    p1 = net.get_params()
    assert abs(l1 - l0) <= 1e-3 * max(abs(l0), 1e-6) + 1e-6
    assert rel_l2(p1, p0) <= 1e-3
    net.close()


@pytest.mark.parametrize("shape", [(6, 12, 40), (9, 8, 64), (16, 20, 96)])
def test_tcgen05_weight_gradient_matches_mma(sfpkg, gpu_ctx, shape):
    """The tcgen05 weight gradient alone (mode "tcgen05_wgrad": forward and input gradients on the warp-MMA
    kernels, so every layer sees the same BF16 dY and X): per-layer weight gradients agree with the warp-MMA
    kernel's to relative L2 1e-4 (the same BF16 products summed in FP32 in a different order); bias gradients and
    the head are computed by the same kernels in both modes and agree exactly."""
    import torch
    from oracle import unet_ref as ref
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    P = ref.init_params(16, seed=13)
    rng = np.random.default_rng(5)
    x = ref.bf16(rng.standard_normal(shape + (16,)))
    net = sfpkg.Network(gpu_ctx)
    net.set_params(ref.flatten(P))
    feat = torch.from_numpy(x).to(torch.bfloat16).cuda().contiguous()
    dout = torch.from_numpy(rng.standard_normal(int(np.prod(shape))).astype(np.float32)).cuda()
    out = torch.zeros(g.num_cells, dtype=torch.float32, device="cuda")
    net.set_mode("mma")
    net.forward(g, feat, out)
    g0 = net.gradients(g, feat, dout)
    net.set_mode("tcgen05_wgrad")
    before = net.tc_launches()
    g1 = net.gradients(g, feat, dout)
    launched = net.tc_launches() - before
    assert launched >= 4  # the level-0 layers at least
    assert np.isfinite(g1).all()
    off = 0
    checked = 0
    for ci, co, taps in [(16, 16, 27), (16, 16, 27), (16, 32, 27), (32, 32, 27), (32, 64, 27), (64, 64, 27),
                         (64, 64, 27), (64, 64, 27), (64, 64, 27), (64, 32, 27), (32, 32, 27), (32, 16, 27),
                         (16, 16, 27), (16, 16, 27), (16, 1, 1)]:
        w = slice(off, off + taps * co * ci)
        b = slice(w.stop, w.stop + co)
        off = b.stop
        if np.abs(g0[w]).max() > 0:
            assert rel_l2(g1[w], g0[w]) <= 1e-4, (ci, co, rel_l2(g1[w], g0[w]))
            checked += 1
        np.testing.assert_array_equal(g1[b], g0[b])
    assert off == g0.size and checked >= 10
    net.close()


@pytest.mark.parametrize("shape", [(4, 6, 128), (8, 12, 256), (5, 8, 64), (16, 24, 256)])
def test_tcgen05_line_gradients_against_oracle(sfpkg, gpu_ctx, shape):
    """Grids that put the 16-channel layers on the line kernel (one halo'd box per z shift for nine taps), whose
    tap order differs from the warp-MMA kernel's, so the BF16 activations of the two paths are no longer bit
    for bit the same and their gradients drift apart by a few percent.  Against the FP64 oracle with the same BF16
    rounding points (oracle/unet_ref.py) the tcgen05 gradients are as close as the warp-MMA ones: per layer the
    relative L2 error is within twice the warp-MMA error or that error + 0.04, and its mean over the layers within
    1.3 times the warp-MMA mean (measured at these shapes: per layer 0.5-1.8 times, means 0.9-1.17 times; both
    paths sit 1-10% from the oracle, a layout error would sit near 100%)."""
    import torch
    from oracle import unet_ref as ref
    g = sfpkg.StaggeredGrid.from_origin(1.0 / shape[0], shape)
    P = ref.init_params(16, seed=5)
    rng = np.random.default_rng(4)
    x = ref.bf16(rng.standard_normal(shape + (16,)))
    dout = rng.standard_normal(shape).astype(np.float32)
    net = sfpkg.Network(gpu_ctx)
    net.set_params(ref.flatten(P))
    feat = torch.from_numpy(x).to(torch.bfloat16).cuda().contiguous()
    out = torch.zeros(g.num_cells, dtype=torch.float32, device="cuda")
    grads = {}
    for mode in ("mma", "tcgen05"):
        net.set_mode(mode)
        before = net.tc_launches()
        net.forward(g, feat, out)
        grads[mode] = ref.unflatten(net.gradients(g, feat, torch.from_numpy(dout).cuda()))
        if mode == "tcgen05":
            assert net.tc_launches() - before >= 8
    _, cache = ref.forward_bf16(P, x)
    G = ref.backward_bf16(P, cache, dout.astype(np.float64))
    errs = []
    for name, *_ in ref.LAYERS:
        for k in (".w", ".b"):
            b = np.asarray(G[name + k]).reshape(grads["mma"][name + k].shape)
            if np.linalg.norm(b) == 0:
                continue
            e_tc, e_mma = rel_l2(grads["tcgen05"][name + k], b), rel_l2(grads["mma"][name + k], b)
            assert np.isfinite(grads["tcgen05"][name + k]).all()
            assert e_tc <= max(2.0 * e_mma, e_mma + 0.04), (name + k, e_tc, e_mma)
            errs.append((e_tc, e_mma))
    assert len(errs) >= 28
    e = np.array(errs)
    assert e[:, 0].mean() <= 1.3 * e[:, 1].mean(), e.mean(axis=0)
    net.close()
