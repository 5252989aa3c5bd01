"""The tcgen05 (TMA + TMEM) forward convolutions against the warp-level MMA ones and the numpy reference.
Both accumulate in FP32 in different orders and round activations to BF16: relative L2 1e-2."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(2, 4, 32), (6, 12, 40), (17, 9, 64)])
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
