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
