"""Learned multi-iteration proposals for the multiview RL iteration (no counterpart in
the reference).

* generate_pairs: the plain GPU method itself, run on seeded synthetic objects, yields
  (psi_k, psi_{k+1}, psi_{k+m}) crops.
* train: the tcgen05 U-Net (mvr_unet_*) learns log(psi_{k+m} / psi_k) from
  [log psi_k, log(psi_{k+1} / psi_k)].
* run: each step runs one plain iteration, proposes psi_k * exp(f(...)) from it, and
  keeps the proposal only when the FP64 data-likelihood residual of the proposal is
  below that of the plain update (mvr_decon_likelihood); otherwise the plain update
  stands.

Device buffers are torch tensors (plumbing only); every computation runs in the
library's kernels.
"""
from __future__ import annotations

import math
import time

import numpy as np

import mvrgb300 as M
import synthetic

ANGLES = (0.0, 45.0, 90.0, 135.0)


def _friendly(n: int, even: bool = False) -> int:
    m = n + (1 if even and n % 2 else 0)
    while True:
        k = m
        for r in (2, 3, 5, 7):
            while k % r == 0:
                k //= r
        if k == 1 and (not even or m % 2 == 0):
            return m
        m += 2 if even else 1


def one_block(dims, psf_xyz):
    """FFT-friendly compute block holding the whole volume (effective size >= dims)."""
    return tuple(_friendly(dims[d] + 2 * (psf_xyz[d] - 1), even=(d == 0)) for d in range(3))


def make_decon(ds, dims, block, device=0, lam=0.006, boundary=M.BOUNDARY_CIRCULAR, precision=M.PRECISION_FP32):
    import torch

    d = M.Deconvolution(dims, len(ds.images), block, psf_type=M.PSF_OPTIMIZATION_I, lam=lam, boundary=boundary,
                        precision=precision, weight_norm=M.WEIGHTS_HARD, device=device)
    keep = []
    for v in range(len(ds.images)):
        im = torch.from_numpy(ds.images[v]).to(f"cuda:{device}")
        w = torch.from_numpy(ds.weights[v]).to(f"cuda:{device}")
        keep += [im, w]
        d.set_view_device(v, im.data_ptr(), w.data_ptr(), ds.psfs[v])
    d.prepare()
    d._keep = keep  # the device images must outlive the handle's use
    return d


def dataset(dims, seed, psf=(31, 31, 61), n_beads=None, side_lobes=True):
    nb = n_beads if n_beads is not None else max(8, int(200 * np.prod(dims) / 256 ** 3 * 8))
    return synthetic.make_dataset(dims, ANGLES, psf, n_beads=nb, seed=seed, side_lobes=side_lobes,
                                  weights="cosine")


def _dataset_job(args):
    dims, seed, psf = args
    return dataset(dims, seed, psf)


def synthesize(dims, seeds, psf, workers=None):
    """Seeded synthetic objects, generated in a process pool (spawn context, so it is
    safe in a process that already uses the GPU)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    import os

    workers = workers or max(1, min(len(seeds), (os.cpu_count() or 2) // 2))
    if workers == 1 or len(seeds) == 1:
        return [dataset(dims, s, psf) for s in seeds]
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_dataset_job, [(dims, s, psf) for s in seeds]))


def pool2(vol, device=0):
    """The library's 2 x 2 x 2 average of a device volume [z][y][x] (even dims)."""
    import torch

    out = torch.empty((vol.shape[0] // 2, vol.shape[1] // 2, vol.shape[2] // 2), dtype=torch.float32,
                      device=vol.device)
    M.pool2(vol.data_ptr(), (vol.shape[2], vol.shape[1], vol.shape[0]), out.data_ptr())
    torch.cuda.synchronize(vol.device)
    return out


def generate_pairs(n_objects=50, dims=(128, 128, 128), crop=(64, 64, 64), iters=45, m=5, pairs_per_object=40,
                   seed0=2000, psf=(31, 31, 61), device=0, datasets=None, coarse=True):
    """(psi_k, psi_{k+1}, psi_{k+m}) crops from the plain method on seeded objects (with
    coarse, of the 2 x 2 x 2 averages of the iterates: the grid the coarse proposal runs on).
    Returns three device tensors [P][cz][cy][cx]."""
    import torch

    rng = np.random.default_rng(seed0)
    shape = (dims[2], dims[1], dims[0])
    hshape = tuple(d // 2 for d in shape) if coarse else shape
    block = one_block(dims, psf)
    out = [[], [], []]
    if datasets is None:
        datasets = synthesize(dims, [seed0 + o for o in range(n_objects)], psf)
    for o in range(n_objects):
        ds = datasets[o]
        dec = make_decon(ds, dims, block, device)
        hist = torch.empty((iters + 1,) + hshape, dtype=torch.float32, device=f"cuda:{device}")
        cur = torch.empty(shape, dtype=torch.float32, device=f"cuda:{device}")

        def keep(k):
            dec.get_psi_device(cur.data_ptr() if coarse else hist[k].data_ptr())
            if coarse:
                hist[k].copy_(pool2(cur, device))

        keep(0)
        for k in range(iters):
            dec.run_iterations(1)
            keep(k + 1)
        dec.close()
        shape_c = hshape
        for _ in range(pairs_per_object):
            k = int(rng.integers(0, iters - m))
            z0, y0, x0 = (int(rng.integers(0, shape_c[i] - crop[2 - i] + 1)) for i in range(3))
            sl = (slice(z0, z0 + crop[2]), slice(y0, y0 + crop[1]), slice(x0, x0 + crop[0]))
            out[0].append(hist[k][sl].clone())
            out[1].append(hist[k + 1][sl].clone())
            out[2].append(hist[k + m][sl].clone())
        del hist
    return tuple(torch.stack(x) for x in out)


def train(pairs, crop=(64, 64, 64), steps=1500, batch=4, lr=1e-3, seed=0, device=0):
    """Trains the U-Net on the pairs; returns (parameters, per-step losses)."""
    import torch

    psi, nxt, tgt = pairs
    rng = np.random.default_rng(seed)
    net = M.UNet(batch, crop, seed=seed, device=device)
    shape = (batch, crop[2], crop[1], crop[0])
    bp = torch.empty(shape, dtype=torch.float32, device=f"cuda:{device}")
    bn = torch.empty_like(bp)
    bt = torch.empty_like(bp)
    losses = []
    for s in range(steps):
        idx = torch.from_numpy(rng.integers(0, psi.shape[0], batch)).to(psi.device)
        torch.index_select(psi, 0, idx, out=bp)
        torch.index_select(nxt, 0, idx, out=bn)
        torch.index_select(tgt, 0, idx, out=bt)
        net.set_input(bp.data_ptr(), bn.data_ptr(), bt.data_ptr())
        cur_lr = lr * 0.5 * (1 + math.cos(math.pi * s / steps))  # cosine schedule
        losses.append(net.train_step(cur_lr))
    params = net.params()
    net.close()
    return params, np.array(losses)


class GatedProposer:
    """Likelihood-gated learned proposals on a whole volume.  Every `every`-th step
    proposes (the others are plain iterations); the seconds spent in the network and in
    the gate's likelihood evaluations are accumulated in `timing`."""

    def __init__(self, params, dims, cap=1.0, device=0, every=1, coarse=True):
        import torch

        self.coarse = coarse
        self.dims = tuple(dims)
        ndims = tuple(d // 2 for d in dims) if coarse else tuple(dims)
        self.net = M.UNet(1, ndims, seed=0, device=device)
        self.net.set_params(params)
        shape = (1, dims[2], dims[1], dims[0])
        self.psi = torch.empty(shape, dtype=torch.float32, device=f"cuda:{device}")
        self.nxt = torch.empty_like(self.psi)
        self.prop = torch.empty_like(self.psi)
        if coarse:
            lshape = (ndims[2], ndims[1], ndims[0])
            self.lo_psi = torch.empty(lshape, dtype=torch.float32, device=f"cuda:{device}")
            self.lo_nxt = torch.empty_like(self.lo_psi)
            self.pred = torch.empty_like(self.lo_psi)
        self.cap = cap
        self.every = max(1, int(every))
        self.count = 0
        self.timing = {"plain_s": 0.0, "network_s": 0.0, "gate_s": 0.0}

    def close(self):
        self.net.close()

    def step(self, dec):
        """One step on dec; returns (accepted, nll_plain, nll_proposal) (NaNs for a plain step)."""
        import torch

        self.count += 1
        t0 = time.perf_counter()
        if self.count % self.every:
            dec.run_iterations(1)
            dec.synchronize()
            self.timing["plain_s"] += time.perf_counter() - t0
            return False, float("nan"), float("nan")
        dec.get_psi_device(self.psi.data_ptr())
        dec.run_iterations(1)
        dec.get_psi_device(self.nxt.data_ptr())
        t1 = time.perf_counter()
        if self.coarse:
            # the network on the coarse grid, its prediction applied to the full-resolution step
            M.pool2(self.psi.data_ptr(), self.dims, self.lo_psi.data_ptr())
            M.pool2(self.nxt.data_ptr(), self.dims, self.lo_nxt.data_ptr())
            torch.cuda.synchronize()
            self.net.set_input(self.lo_psi.data_ptr(), self.lo_nxt.data_ptr())
            self.net.forward(self.pred.data_ptr())
            torch.cuda.synchronize()
            M.apply_coarse(self.nxt.data_ptr(), self.dims, self.pred.data_ptr(), self.lo_psi.data_ptr(),
                           self.lo_nxt.data_ptr(), self.cap, self.prop.data_ptr())
        else:
            self.net.set_input(self.psi.data_ptr(), self.nxt.data_ptr())
            self.net.propose(self.psi.data_ptr(), self.prop.data_ptr(), self.cap)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        l_plain = dec.likelihood()[0]
        dec.set_psi_device(self.prop.data_ptr())
        l_prop = dec.likelihood()[0]
        accepted = l_prop < l_plain
        if not accepted:
            dec.set_psi_device(self.nxt.data_ptr())
        dec.synchronize()
        t3 = time.perf_counter()
        self.timing["plain_s"] += t1 - t0
        self.timing["network_s"] += t2 - t1
        self.timing["gate_s"] += t3 - t2
        return accepted, l_plain, l_prop


def convergence(dec, n_steps, ref=None, proposer=None):
    """Runs n_steps plain iterations (or gated steps when proposer is given); returns per
    step (seconds since start, relative L2 to ref or NaN, NLL, accepted)."""
    import torch

    hist = []
    buf = None
    if ref is not None:
        buf = torch.empty_like(ref)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    elapsed = 0.0
    for _ in range(n_steps):
        ts = time.perf_counter()
        if proposer is None:
            dec.run_iterations(1)
            dec.synchronize()
            acc = False
        else:
            acc, _, _ = proposer.step(dec)
        elapsed += time.perf_counter() - ts
        nll = dec.likelihood()[0]  # bookkeeping outside the timed part
        err = float("nan")
        if ref is not None:
            dec.get_psi_device(buf.data_ptr())
            err = float(torch.linalg.vector_norm(buf.double() - ref.double()) / torch.linalg.vector_norm(ref.double()))
        hist.append((elapsed, err, nll, acc))
    _ = t0
    return hist


def first_time(hist, pred):
    for t, err, nll, _ in hist:
        if pred(err, nll):
            return t
    return None


def experiment(ds, dims, block, n_objects=50, train_dims=(128, 128, 128), crop=(64, 64, 64), iters=45, m=5,
               pairs_per_object=40, train_steps=1500, batch=4, lr=1e-3, eval_iters=20, tol=1e-3, device=0,
               datasets=None, everies=(1, 3), coarse=True):
    """Learned + gated vs plain GPU RL on ds: wall time to relative L2 <= tol against the
    FP64 plain result after eval_iters iterations, and to that result's likelihood.  With
    coarse, the network sees and predicts the 2 x 2 x 2 averages (training crops of the
    averaged iterates: the whole 64^3 average of a 128^3 object)."""
    import torch

    t0 = time.perf_counter()
    pairs = generate_pairs(n_objects, train_dims, crop, iters, m, pairs_per_object, psf=ds.psfs[0].shape[::-1],
                           device=device, datasets=datasets, coarse=coarse)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    params, losses = train(pairs, crop, train_steps, batch, lr, device=device)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    psi0, _, tgt0 = pairs
    base = float(torch.mean(torch.log(tgt0 / psi0) ** 2))
    del pairs, psi0, tgt0
    shape = (dims[2], dims[1], dims[0])
    # FP64 plain reference
    d64 = make_decon(ds, dims, block, device, precision=M.PRECISION_FP64)
    d64.run_iterations(eval_iters)
    ref = torch.empty(shape, dtype=torch.float32, device=f"cuda:{device}")
    d64.get_psi_device(ref.data_ptr())
    nll_ref = d64.likelihood()[0]
    d64.close()
    plain = make_decon(ds, dims, block, device)
    h_plain = convergence(plain, eval_iters, ref)
    plain.close()
    runs = {}
    for every in everies:
        gated = make_decon(ds, dims, block, device)
        prop = GatedProposer(params, dims, device=device, every=every, coarse=coarse)
        h = convergence(gated, eval_iters + 10, ref, prop)
        runs[every] = (h, dict(prop.timing))
        prop.close()
        gated.close()

    def summary(h):
        return {"t_err": first_time(h, lambda e, n: e <= tol), "t_nll": first_time(h, lambda e, n: n <= nll_ref),
                "final_err": h[-1][1], "final_nll": h[-1][2], "seconds": h[-1][0],
                "accepted": int(sum(1 for x in h if x[3]))}

    sp = summary(h_plain)
    out = {"pairs": n_objects * pairs_per_object, "objects": n_objects, "m": m, "train_steps": train_steps,
           "train_loss_first": float(np.mean(losses[:20])), "train_loss_last": float(np.mean(losses[-20:])),
           "no_change_loss": base, "gen_s": gen_s, "train_s": train_s, "eval_iters": eval_iters, "tol": tol,
           "nll_fp64_ref": nll_ref, "plain": sp, "trace_plain": [(round(t, 5), e, n) for t, e, n, _ in h_plain]}
    for every, (h, timing) in runs.items():
        sg = summary(h)
        sg["timing"] = timing
        sg["speedup_to_tol"] = sp["t_err"] / sg["t_err"] if sp["t_err"] and sg["t_err"] else None
        sg["speedup_to_nll"] = sp["t_nll"] / sg["t_nll"] if sp["t_nll"] and sg["t_nll"] else None
        sg["trace"] = [(round(t, 5), e, n, a) for t, e, n, a in h]
        out[f"learned_every{every}"] = sg
    return out
