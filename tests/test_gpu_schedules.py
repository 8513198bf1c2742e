"""The FFT-schedule autotuner of the whole-volume driver (through the C ABI): every schedule
it can pick computes the same iteration, and its trial table lists them.

Tolerances: forced schedules agree with each other to float rounding (relative L2 1e-6
after 2 iterations) and with the oracle within 1e-4.
"""
import numpy as np
import pytest

import mvrgb300 as M
import oracle as O
import synthetic

pytestmark = pytest.mark.gpu
ALL = [M.SCHED_ROWS, M.SCHED_ROWS | M.SCHED_ZPIPE, M.SCHED_PLANE, M.SCHED_PLANE | M.SCHED_ZPIPE,
       M.SCHED_PLANE_PERSIST, M.SCHED_PLANE_PERSIST | M.SCHED_ZPIPE]


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def case():
    rng = np.random.default_rng(21)
    dims = (180, 170, 90)
    shape = dims[::-1]
    psfs = [synthetic.make_psf((9, 9, 15), 1.2, 2.5, a) for a in (0.0, 90.0)]
    imgs = [rng.uniform(5, 200, shape).astype(np.float32) for _ in range(2)]
    ws = [rng.uniform(0.2, 1, shape).astype(np.float32) for _ in range(2)]
    return dims, psfs, imgs, ws


def run(case, code, iters=2):
    dims, psfs, imgs, ws = case
    # 128 x 128 x 64 blocks, circular: a plane-kernel domain with 16-tile Z columns
    with M.Deconvolution(dims, 2, (128, 128, 64), psf_type=M.PSF_OPTIMIZATION_I, lam=0.006,
                         boundary=M.BOUNDARY_CIRCULAR, weight_norm=M.WEIGHTS_AS_GIVEN) as d:
        for v in range(2):
            d.set_view(v, imgs[v], ws[v], psfs[v])
        if code is not None:
            d.set_schedule(code)
        d.prepare()
        used = [d.schedule(v) for v in range(2)]
        trials = d.tuning()
        d.run_iterations(iters)
        run.nll[code] = d.likelihood()[0]  # the plane paths reduce it over the write regions only
        return d.get_psi(), used, trials


run.nll = {}


def test_every_forced_schedule_gives_the_same_psi(case):
    outs = {}
    for code in ALL:
        psi, used, trials = run(case, code)
        assert used == [code, code], M.schedule_name(code)
        assert all(t["code"] == -1 for t in trials)  # no schedule search when forced
        outs[code] = psi
    base = outs[M.SCHED_ROWS]
    for code, psi in outs.items():
        assert rel(psi, base) <= 1e-6, M.schedule_name(code)
        assert run.nll[code] == pytest.approx(run.nll[M.SCHED_ROWS], rel=1e-6)
    dims, psfs, imgs, ws = case
    k1s, k2s = O.psf_init(psfs, O.PSF_OPTIMIZATION_I, 0)
    psi0, mx, _ = O.psi_init_avg(imgs)
    ref, _ = O.decon_run(psi0, imgs, ws, k1s, k2s, (128, 128, 64), 2, lam=0.006, max_intensities=mx)
    assert rel(base, ref) <= 1e-4


def test_autotuner_tries_every_schedule_and_keeps_the_fastest(case):
    psi, used, trials = run(case, None)
    for st in range(2):
        mine = [t for t in trials if t["step"] == st]
        assert sorted(t["code"] for t in mine) == sorted(ALL)
        best = min(mine, key=lambda t: t["ms"])
        assert used[st] == best["code"]
    assert any(t["code"] == -1 for t in trials)  # then the blocks per launch
    forced, _, _ = run(case, used[0]) if used[0] == used[1] else (psi, None, None)
    assert rel(psi, forced) <= 1e-6


def test_schedule_errors():
    with M.Deconvolution((40, 36, 30), 2, (28, 28, 28)) as d:
        with pytest.raises(M.MvrError):
            d.set_schedule(8)
        with pytest.raises(M.MvrError):
            d.set_schedule(-2)
        # a 28^3 block has no plane or pair kernels: forcing them fails at prepare
        d.set_view(0, np.ones((30, 36, 40), np.float32), np.ones((30, 36, 40), np.float32),
                   synthetic.make_psf((5, 5, 7), 1.0, 1.5, 0.0))
        d.set_view(1, np.ones((30, 36, 40), np.float32), np.ones((30, 36, 40), np.float32),
                   synthetic.make_psf((5, 5, 7), 1.0, 1.5, 90.0))
        d.set_schedule(M.SCHED_PAIR)
        with pytest.raises(M.MvrError) as e:
            d.prepare()
        assert e.value.code == M.ERR_UNSUPPORTED
