"""Learned multi-iteration proposals, end to end at a small scale: training pairs from
the plain GPU method, training on the tensor cores, and the likelihood gate.

What the trained network gains over the plain method is measured and printed (NLL
after the same number of steps; it can be negative: the gate compares one step, not
the trajectory).  The assertions are the guarantees: the network learns (its loss falls
below that of predicting no change), an accepted proposal always has a lower FP64
likelihood residual than the plain update from the same iterate, and the gated run
stays within 1e-3 relative NLL of the plain run.
"""
import numpy as np
import pytest

import learned as L

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

DIMS = (64, 64, 64)
PSF = (9, 9, 17)


@pytest.fixture(scope="module")
def trained():
    pairs = L.generate_pairs(n_objects=3, dims=DIMS, crop=(32, 32, 32), iters=16, m=5, pairs_per_object=24,
                             seed0=2000, psf=PSF)
    psi, _, tgt = pairs
    base = float(torch.mean(torch.log(tgt / psi) ** 2))  # loss of predicting "no change"
    params, losses = L.train(pairs, crop=(32, 32, 32), steps=200, batch=4, lr=2e-3, seed=0)
    return params, losses, base


def test_training_learns_the_multi_iteration_update(trained):
    _, losses, base = trained
    late = float(np.mean(losses[-20:]))
    print(f"\nno-change loss {base:.4e}, trained loss {late:.4e}")
    assert late < 0.5 * base


def test_gated_proposals_never_worse_than_plain(trained):
    params = trained[0]
    ds = L.dataset(DIMS, 3000, PSF)
    block = L.one_block(DIMS, PSF)
    plain = L.make_decon(ds, DIMS, block)
    gated = L.make_decon(ds, DIMS, block)
    prop = L.GatedProposer(params, DIMS)
    try:
        n = 8
        h_plain = L.convergence(plain, n)
        steps = []
        for _ in range(n):
            acc, lp, lq = prop.step(gated)
            if acc:
                assert lq < lp
            steps.append(acc)
        nll_gated = gated.likelihood()[0]
    finally:
        prop.close()
        plain.close()
        gated.close()
    nll_plain = h_plain[-1][2]
    print(f"\naccepted {sum(steps)}/{n}; NLL after {n} steps: plain {nll_plain:.6e}, gated {nll_gated:.6e}")
    assert nll_gated <= nll_plain + 1e-3 * abs(nll_plain)


def test_coarse_grid_kernels_against_numpy():
    # mvr_pool2 (2 x 2 x 2 average) and mvr_apply_coarse (trilinear upsampling of the coarse
    # log change beyond the plain step, applied to the full-resolution step)
    import mvrgb300 as M

    rng = np.random.default_rng(9)
    shape = (12, 10, 16)  # [z][y][x]
    dims = (16, 10, 12)
    psi = rng.uniform(1, 5, shape).astype(np.float32)
    nxt = (psi * rng.uniform(0.9, 1.1, shape)).astype(np.float32)
    d_psi, d_nxt = torch.from_numpy(psi).cuda(), torch.from_numpy(nxt).cuda()
    lo = torch.empty((6, 5, 8), dtype=torch.float32, device="cuda")
    lo2 = torch.empty_like(lo)
    M.pool2(d_psi.data_ptr(), dims, lo.data_ptr())
    M.pool2(d_nxt.data_ptr(), dims, lo2.data_ptr())
    torch.cuda.synchronize()
    ref_lo = psi.reshape(6, 2, 5, 2, 8, 2).mean(axis=(1, 3, 5))
    assert np.allclose(lo.cpu().numpy(), ref_lo, rtol=1e-6)
    pred = torch.from_numpy(rng.normal(0, 0.05, (6, 5, 8)).astype(np.float32)).cuda()
    out = torch.empty_like(d_psi)
    M.apply_coarse(d_nxt.data_ptr(), dims, pred.data_ptr(), lo.data_ptr(), lo2.data_ptr(), 1.0, out.data_ptr())
    torch.cuda.synchronize()
    c = pred.cpu().numpy().astype(np.float64) - np.log(lo2.cpu().numpy().astype(np.float64) /
                                                        lo.cpu().numpy().astype(np.float64))

    def up(a, n):  # trilinear along one axis: coarse coordinate x / 2 - 1 / 4, clamped
        u = np.arange(n) / 2.0 - 0.25
        f0 = np.floor(u)
        f = u - f0
        i0 = np.clip(f0.astype(int), 0, a.shape[0] - 1)
        i1 = np.clip(f0.astype(int) + 1, 0, a.shape[0] - 1)
        return a[i0] * (1 - f)[:, None, None] + a[i1] * f[:, None, None]

    cu = up(c, 12)
    cu = np.moveaxis(up(np.moveaxis(cu, 1, 0), 10), 0, 1)
    cu = np.moveaxis(up(np.moveaxis(cu, 2, 0), 16), 0, 2)
    ref = nxt * np.exp(np.clip(cu, -1, 1))
    assert np.allclose(out.cpu().numpy(), ref, rtol=2e-5)
