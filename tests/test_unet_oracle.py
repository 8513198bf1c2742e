"""The numpy restatement of the learned-proposal network checked on its own: the data
and weight gradients are the adjoints of the forward convolution, and the whole
network's analytic gradient matches central finite differences (float64, no BF16
rounding)."""
import numpy as np

import unet_oracle as U


def test_conv_adjoints():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((2, 4, 5, 6, 16))
    w = rng.standard_normal((32, 27, 16))
    g = rng.standard_normal((2, 4, 5, 6, 32))
    lhs = float((U.conv_fwd(x, w) * g).sum())
    assert abs(lhs - float((x * U.conv_dgrad(g, w)).sum())) <= 1e-9 * abs(lhs)
    assert abs(lhs - float((w * U.conv_wgrad(x, g)).sum())) <= 1e-9 * abs(lhs)


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159], np.float32)
    r = U.bf16(a)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] + 3.140625) < 1e-6


def test_network_gradient_finite_differences():
    rng = np.random.default_rng(1)
    n = sum(co * 27 * ci + co for ci, co in U.LAYERS) + 17
    params = 0.2 * rng.standard_normal(n)
    x16 = np.zeros((1, 4, 4, 4, 16))
    x16[..., :2] = rng.standard_normal((1, 4, 4, 4, 2))
    target = rng.standard_normal((1, 4, 4, 4))
    loss, g, _ = U.forward_backward(params, x16, target, round_bf16=False)
    for i in rng.choice(n, 25, replace=False).tolist() + [n - 1, n - 2]:
        e = np.zeros(n)
        e[i] = 1e-6
        lp = U.forward_backward(params + e, x16, target, round_bf16=False)[0]
        lm = U.forward_backward(params - e, x16, target, round_bf16=False)[0]
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])
