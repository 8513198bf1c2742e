"""The learned-proposal network on the tcgen05 tensor cores against its numpy
restatement (oracle/unet_oracle.py): every convolution layer shape in forward, data
gradient and weight gradient, the whole U-Net's loss and parameter gradients, and a
training run that lowers the loss.

Tolerances: FP32 outputs (data / weight gradients) from BF16 operands within 1e-5
relative L2; BF16 forward outputs within 8e-3 (one BF16 rounding); whole-network
parameter gradients within 3e-2 relative L2 per layer (BF16 activations and gradients
are rounded at the same points on both sides, the accumulation orders differ).
"""
import numpy as np
import pytest

import mvrgb300 as M
import unet_oracle as U

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def dev_bf16(a):
    return torch.from_numpy(U.bf16_bits(a).view(np.int16)).cuda()


def host_bf16(t):
    return (t.cpu().numpy().view(np.uint16).astype(np.uint32) << 16).view(np.float32)


@pytest.mark.parametrize("ci,co", U.LAYERS)
def test_conv_layer_forward_dgrad_wgrad(ci, co):
    rng = np.random.default_rng(ci * 100 + co)
    B, X, Y, Z = 2, 12, 8, 4
    x = U.bf16(rng.standard_normal((B, Z, Y, X, ci)))
    w = U.bf16(0.1 * rng.standard_normal((co, 27, ci)))
    b = rng.standard_normal(co).astype(np.float32)
    g = U.bf16(rng.standard_normal((B, Z, Y, X, co)))
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    dims = (X, Y, Z, B)
    # forward with bias and ReLU, BF16 output
    xd, wd = dev_bf16(x), dev_bf16(w)
    bd = torch.from_numpy(b).cuda()
    yd = torch.zeros((B, Z, Y, X, co), dtype=torch.int16, device="cuda")
    M.conv3d_tc(xd.data_ptr(), ci, wd.data_ptr(), co, bd.data_ptr(), 1, 0, yd.data_ptr(), dims, err.data_ptr())
    assert rel(host_bf16(yd), U.conv_fwd(x, w, b, relu=True)) <= 8e-3
    # data gradient with the transposed weights, FP32 output
    gd = dev_bf16(g)
    wtd = dev_bf16(np.ascontiguousarray(w.transpose(2, 1, 0)))
    dxd = torch.zeros((B, Z, Y, X, ci), dtype=torch.float32, device="cuda")
    M.conv3d_tc(gd.data_ptr(), co, wtd.data_ptr(), ci, 0, 0, 1, dxd.data_ptr(), dims, err.data_ptr())
    assert rel(dxd.cpu().numpy(), U.conv_dgrad(g, w)) <= 1e-5
    # weight gradient
    dwd = torch.zeros((co, 27, ci), dtype=torch.float32, device="cuda")
    M.conv3d_tc_wgrad(xd.data_ptr(), ci, gd.data_ptr(), co, dwd.data_ptr(), dims, err.data_ptr())
    assert rel(dwd.cpu().numpy(), U.conv_wgrad(x, g)) <= 1e-5
    assert int(err.item()) == 0


def test_unet_loss_and_gradients_match_numpy():
    rng = np.random.default_rng(11)
    shape = (1, 8, 8, 8)
    psi = rng.uniform(10, 100, shape).astype(np.float32)
    psi_n = (psi * rng.uniform(0.8, 1.25, shape)).astype(np.float32)
    psi_t = (psi * rng.uniform(0.7, 1.4, shape)).astype(np.float32)
    with M.UNet(1, (8, 8, 8), seed=3) as net:
        pd, rd, td = (torch.from_numpy(a).cuda() for a in (psi, psi_n, psi_t))
        net.set_input(pd.data_ptr(), rd.data_ptr(), td.data_ptr())
        params = net.params()
        loss = net.train_step(0.0)  # learning rate 0: gradients only
        grads = net.grads()
        assert np.array_equal(net.params(), params)
    x16 = U.features(psi, psi_n)
    target = np.log(psi_t / psi).astype(np.float64)
    loss_ref, g_ref, _ = U.forward_backward(params, x16, target)
    assert abs(loss - loss_ref) <= 1e-3 * loss_ref
    o = 0
    for ci, co in U.LAYERS:
        nw = co * 27 * ci
        assert rel(grads[o:o + nw], g_ref[o:o + nw]) <= 3e-2, (ci, co)
        o += nw
        assert rel(grads[o:o + co], g_ref[o:o + co]) <= 3e-2, (ci, co, "bias")
        o += co
    assert rel(grads[o:o + 17], g_ref[o:o + 17]) <= 1e-3  # head


def test_unet_training_lowers_the_loss():
    rng = np.random.default_rng(5)
    shape = (2, 16, 16, 16)
    z, y, x = np.meshgrid(*(np.arange(16),) * 3, indexing="ij")
    base = 50 + 40 * np.exp(-((x - 8) ** 2 + (y - 8) ** 2 + (z - 8) ** 2) / 20.0)
    psi = np.stack([base, base[::-1]]).astype(np.float32) * rng.uniform(0.9, 1.1, shape).astype(np.float32)
    ratio = (1.0 + 0.05 * np.sin(x / 3.0)).astype(np.float32)[None].repeat(2, 0)
    psi_n = (psi * ratio).astype(np.float32)
    psi_t = (psi * ratio ** 4).astype(np.float32)  # a structured multi-iteration target
    with M.UNet(2, (16, 16, 16), seed=1) as net:
        pd, rd, td = (torch.from_numpy(a).cuda() for a in (psi, psi_n, psi_t))
        net.set_input(pd.data_ptr(), rd.data_ptr(), td.data_ptr())
        losses = [net.train_step(2e-3) for _ in range(60)]
    assert losses[-1] < 0.3 * losses[0], (losses[0], losses[-1])


def test_fused_decoder_inference_equals_materialised_concat():
    # propose() runs the decoder convolutions straight from [up(low), skip]; forward() builds
    # the concatenated volumes first (as training needs them): the predictions agree exactly
    rng = np.random.default_rng(5)
    dims = (32, 24, 16)
    net = M.UNet(2, dims, seed=3)
    try:
        shape = (2, dims[2], dims[1], dims[0])
        psi = torch.from_numpy(rng.uniform(1, 50, shape).astype(np.float32)).cuda()
        nxt = psi * torch.from_numpy(rng.uniform(0.9, 1.1, shape).astype(np.float32)).cuda()
        pred = torch.empty_like(psi)
        out = torch.empty_like(psi)
        net.set_input(psi.data_ptr(), nxt.data_ptr())
        net.forward(pred.data_ptr())
        net.propose(psi.data_ptr(), out.data_ptr(), 0.5)
        ref = psi * torch.exp(torch.clamp(pred, -0.5, 0.5))
        assert torch.allclose(out, ref, rtol=1e-6, atol=0)
        assert float(pred.abs().max()) > 0
    finally:
        net.close()
