#!/usr/bin/env python3
"""Throughput of the multiview Bayesian (RL-type) deconvolution iteration on GB300.

Workload (the reference's 4-view case): 4 views of 256^3 float32, PSFs 31x31x61
Gaussian-plus-side-lobes rotated 0/45/90/135 degrees about y, Optimization-I compound
kernels, cosine-blended weights normalised with the reference's hard rule, psi from
PsiInitAvgPrecise, Tikhonov lambda 0.006, compute blocks 192^3 (16 per view).
Synthetic seeded data stands in for the reference's microscopy datasets.

A step is one full iteration (all 4 views, all blocks) over the whole volume.
Metric: voxel-iterations/s = 256^3 * steps / seconds.

  value       device-resident inputs, CUDA events on the library's stream around K steps
  e2e         the public C ABI with pinned host buffers: every step uploads the 4 images,
              4 raw weights and psi, runs one iteration and reads psi back
  e2e_block   the per-block plugin call (mvr_block_run_seq, ComputeBlockSeqThread.
              runIteration) with host buffers, 64 calls per iteration from 2 worker threads
  err_vs_fp64 relative L2 of the FP32 iterations against the FP64 run of the same ones
  --impl reference  the float32 CPU restatement of the reference block iteration with its
              padded real-to-complex FFT convolution (oracle/cpu_reference.py, all host
              threads) on a bounded sample of the same workload
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "multiview-reconstruction_gb300")
for _p in (PKG, os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

UNIT = "voxel-iterations/s"


class Workload:
    """A named deconvolution workload: volume, views, compute block, PSF sizes per view."""

    def __init__(self, name, dims, views, block, psfs, lam, make, desc, psf_type=1, weight_norm=1, fp64_iters=None,
                 effective=None):
        # block: one compute block (x, y, z) for every view, or a list with one per view;
        # effective: one effective block for every view (None: block - 2 (k - 1))
        per_view = isinstance(block[0], (tuple, list))
        self.vblocks = [tuple(b) for b in block] if per_view else [tuple(block)] * views
        self.effective = tuple(effective) if effective else None
        block = self.vblocks[0]
        self.name, self.dims, self.views, self.block, self.psfs, self.lam = name, dims, views, block, psfs, lam
        self.make, self.desc = make, desc
        self.psf_type, self.weight_norm = psf_type, weight_norm  # MVR_PSF_*, MVR_WEIGHTS_*
        self.fp64_iters = fp64_iters  # iterations of the FP64 comparison (None: warm-up + timed)
        self.nvox = dims[0] * dims[1] * dims[2]
        self.metric = f"voxel-iterations/s ({views} views)"

    def blocks(self, v):
        """The library's block grid of view v (mvr_block_grid, the whole-volume driver's)."""
        import mvrgb300 as M

        k = self.psfs[v]
        if self.effective:
            # the overlap block - effective + 1 as the doubled kernel 2k' - 1 of a kernel k'
            kk = [self.vblocks[v][d] - self.effective[d] + 1 for d in range(3)]
            assert all(x % 2 == 1 for x in kk), "block - effective must be even"
            k = tuple((x + 1) // 2 for x in kk)
        return M.block_grid(self.dims, k, self.vblocks[v])[0]

    def ref_vblocks(self):
        """The reference's compute block per view for the same effective grid: effective + 2 (k - 1)."""
        if not self.effective:
            return self.vblocks
        return [tuple(self.effective[d] + 2 * (k[d] - 1) for d in range(3)) for k in self.psfs]

    def ref_blocks(self, v):
        import oracle

        return oracle.divide_into_blocks(self.dims, tuple(2 * k - 1 for k in self.psfs[v]), self.ref_vblocks()[v])

    def per_view_blocks(self):
        return len(set(self.vblocks)) > 1

    def setup_blocks(self, d):
        """Per-view compute blocks and the effective block on a Deconvolution handle (before prepare)."""
        if self.per_view_blocks():
            for v in range(self.views):
                d.set_view_block_size(v, self.vblocks[v])
        if self.effective:
            d.set_effective_block_size(-1, self.effective)

    def view_blocks_per_iter(self):
        return sum(len(self.blocks(v)) for v in range(self.views))

    def input_bytes(self):
        return (2 * self.views + 1) * self.nvox * 4

    def flush_l2(self):
        """Inputs below twice the 129 MB L2: the bench flushes L2 before every timed step."""
        return self.input_bytes() < 2 * 129e6

    def config(self, boundary):
        mib = self.input_bytes() / 2**20
        l2 = (f"L2 flushed before every timed step (a 512 MiB write outside the step's events; inputs "
              f"{mib:.0f} MiB)" if self.flush_l2() else
              f"inputs larger than L2 ({self.views} images + {self.views} weights + psi = {mib:.0f} MiB)")
        blk = [list(b) for b in self.vblocks] if self.per_view_blocks() else list(self.block)
        extra = {"effective_block": list(self.effective)} if self.effective else {}
        return {"workload": self.desc, "views": self.views, "dims": list(self.dims), "block": blk, **extra,
                "psf": [list(p) for p in self.psfs] if len(set(self.psfs)) > 1 else list(self.psfs[0]),
                "lambda": self.lam, "iterations_per_step": 1, "boundary": boundary, "l2": l2,
                "data": "seeded synthetic beads + ellipsoid, Poisson, background 10"}


def _make256():
    import synthetic

    return synthetic.config_256()


def _make512():
    import synthetic

    return synthetic.config_512()


def _make_large():
    import torch

    import synthetic

    return synthetic.config_large(torch.cuda.current_device() if torch.cuda.is_available() else "cpu")


def _make_small():
    import synthetic

    return synthetic.config_small()


def _make_pair_case():
    import synthetic

    return synthetic.make_dataset((480, 480, 120), (0.0, 90.0), (21, 21, 15), n_beads=400, seed=1006,
                                  side_lobes=True, weights="cosine")


def _psf_sizes_6():
    import synthetic

    return [tuple(p) for p in synthetic.PSF_SIZES_6]


def friendly(n, even=False):
    """Smallest size >= n with prime factors <= 13 (even when asked): a circular FFT
    domain the library accepts."""
    while True:
        k = n
        for r in (2, 3, 5, 7, 11, 13):
            while k % r == 0:
                k //= r
        if k == 1 and (not even or n % 2 == 0):
            return n
        n += 1


def _blocks_6():
    """128^3 effective blocks: compute block 128 + 2 (k - 1) per axis and view."""
    return [tuple(friendly(128 + 2 * (p[d] - 1), even=d == 0) for d in range(3)) for p in _psf_sizes_6()]


def _blocks_6_plane():
    """The smallest compute blocks at least 128 + 2 (k - 1) per axis with plane kernels:
    x and y 192 (one CTA per plane) or 256 (a pair of CTAs), z a tile-column length."""
    def up(n, sizes):
        return min(s for s in sizes if s >= n)

    return [(up(128 + 2 * (p[0] - 1), (192, 256)), up(128 + 2 * (p[1] - 1), (192, 256)),
             up(128 + 2 * (p[2] - 1), (192, 256, 288))) for p in _psf_sizes_6()]


WORKLOADS = {
    "2view128": lambda: Workload("2view128", (128, 128, 64), 2, (192, 192, 128), [(15, 15, 31)] * 2, 0.0, _make_small,
                                 "2 views 128x128x64 float32, PSF 15x15x31 at 0/90 degrees, efficient-Bayesian, "
                                 "all-one weights, one block (192x192x128 compute block), lambda 0, Seq",
                                 psf_type=2, weight_norm=0),
    "4view256": lambda: Workload("4view256", (256, 256, 256), 4, (192, 192, 192), [(31, 31, 61)] * 4, 0.006, _make256,
                                 "4 views 256^3 float32, PSF 31x31x61 Optimization-I, blocks 192^3, Seq (OSEM-like)"),
    "6view512": lambda: Workload("6view512", (512, 512, 256), 6, _blocks_6_plane(), _psf_sizes_6(), 0.006, _make512,
                                 "6 views 512x512x256 float32, PSFs 21x21x41 ... 41x41x81 per view, "
                                 "Optimization-I, 128^3 effective blocks (4 x 4 x 2 per view, uneven edge blocks) "
                                 "plus overlap: compute blocks 192x192x256 (views 0-3) and 256x256x288 (views 4-5), "
                                 "the smallest plane-kernel shapes >= 128 + 2 (k - 1), Seq", fp64_iters=5,
                                 effective=(128, 128, 128)),
    "6view512tight": lambda: Workload("6view512tight", (512, 512, 256), 6, _blocks_6(), _psf_sizes_6(), 0.006,
                                      _make512,
                                      "6 views 512x512x256 float32, PSFs 21x21x41 ... 41x41x81 per view, "
                                      "Optimization-I, 128^3 effective blocks plus exactly each view's overlap: "
                                      "compute blocks 128 + 2 (k - 1) per axis (168x168x208 ... 208x208x288, rounded "
                                      "up to an FFT-friendly size where needed), 32 blocks per view, Seq", fp64_iters=5),
    "6view512fixed": lambda: Workload("6view512fixed", (512, 512, 256), 6, (192, 192, 256), _psf_sizes_6(), 0.006,
                                      _make512,
                                 "6 views 512x512x256 float32, PSFs 21x21x41 ... 41x41x81 per view, "
                                 "Optimization-I, compute blocks 192x192x256 (effective 112-152 x 112-152 x 96-176, "
                                 "uneven edge blocks), Seq", fp64_iters=5),
    "2view480": lambda: Workload("2view480", (480, 480, 120), 2, (256, 256, 64), [(21, 21, 15)] * 2, 0.006,
                                 _make_pair_case,
                                 "2 views 480x480x120 float32, PSF 21x21x15, compute blocks 256x256x64 (36 per view): "
                                 "a small case of the 256-wide plane kernels, for profiling", fp64_iters=2),
    "8view1024": lambda: Workload("8view1024", (1024, 1024, 512), 8, (256, 256, 256), [(41, 41, 81)] * 8, 0.006,
                                  _make_large,
                                  "8 views 1024x1024x512 (uint16 recorded, converted to float32), 20000 nuclei-like "
                                  "blobs, PSF 41x41x81 at 45 degree steps, compute blocks 256^3 (216 per view), Seq",
                                  fp64_iters=2),
}
W = None  # the workload of this run (set in main)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """DRAM bytes per launch (read + write) from the committed ncu summary: the lines of
    its ```traffic block, 'kernel-family bytes'."""
    path = os.path.join(ROOT, "profiles", "plane_kernels_4view_256cubed.md")
    out, inside = {}, False
    if os.path.exists(path):
        for line in open(path):
            if line.startswith("```"):
                inside = line.strip() == "```traffic"
                continue
            if inside and line.strip():
                k, v = line.split()
                out[k] = float(v)
    return out


def make_data():
    return W.make()


class ClockSampler:
    """nvidia-smi clocks / throttle reasons while the timed region runs."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        try:
            rows = [l.strip().split(",") for l in open(self.path) if l.strip()]
        except Exception:
            rows = []
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, ws):
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist

    on_gpu = torch.cuda.is_available() and dist.get_backend() == "nccl"
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if on_gpu else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def prepare_reference_inputs(ds):
    """Set-up of the CPU sample, outside any timed region: the kernels (DeconViewPSF.init,
    the C oracle), the normalised weights per block and the per-view maxima / psi0
    (PsiInitAvgPrecise).  Host volumes are normalised whole; device volumes (the large
    workload) per sampled block (the rule is per voxel).  Returns (k1s, k2s, weight_block,
    image_block, mx, psi0) with the block functions of cpu_reference.BlockSampler."""
    import cpu_reference as R
    import oracle

    k1s, k2s = oracle.psf_init(ds.psfs, W.psf_type, 0)
    on_dev = not isinstance(ds.images[0], np.ndarray)
    if not on_dev:
        if W.weight_norm == 0:
            ws = [np.ascontiguousarray(w, dtype=np.float32) for w in ds.weights]
        else:
            ws = oracle.normalize_weights(ds.weights, smooth=W.weight_norm == 2)
        psi0, mx, _ = oracle.psi_init_avg(ds.images)
        return (k1s, k2s, (lambda v, off, b: R.extract(ws[v], off, b, "zero")),
                (lambda v, off, b: R.extract(ds.images[v], off, b, "zero")), mx, psi0)

    def box(vol, off, b):
        D = (vol.shape[2], vol.shape[1], vol.shape[0])
        idx = [np.arange(off[d], off[d] + b[d]) for d in range(3)]
        ok = [(idx[d] >= 0) & (idx[d] < D[d]) for d in range(3)]
        out = np.zeros((b[2], b[1], b[0]), dtype=np.float32)
        sub = np.ix_(idx[2][ok[2]], idx[1][ok[1]], idx[0][ok[0]])
        dst = np.ix_(np.nonzero(ok[2])[0], np.nonzero(ok[1])[0], np.nonzero(ok[0])[0])
        out[dst] = _region(vol, sub)
        return out

    def weight_block(v, off, b):
        return oracle.normalize_weights([box(ds.weights[u], off, b) for u in range(W.views)])[v]

    return k1s, k2s, weight_block, (lambda v, off, b: box(ds.images[v], off, b)), None, None


def cpu_sampler(ds, psi, mx, prep):
    import cpu_reference as R

    k1s, k2s, weight_block, image_block, _, _ = prep
    # the reference's own blocks: effective + 2 (k - 1), on the same effective grid
    grids = [W.ref_blocks(v) for v in range(W.views)]
    return R.BlockSampler(psi, None, None, k1s, k2s, grids, W.ref_vblocks(), W.lam, mx, image_block=image_block,
                          weight_block=weight_block)


def cpu_sample_text(steps, sampler):
    P = sampler._convolvers(0)[0].P
    b = W.ref_vblocks()[0]
    return (f"{steps} step(s) of one {b[0]}x{b[1]}x{b[2]} block per view (views in order, effective "
            f"regions pasted back into psi), float32 real-to-complex FFTs at the padded size {P[0]}x{P[1]}x{P[2]} "
            f"(util/FFTConvolution), {sampler.workers} host threads; value = voxel-iterations advanced / seconds")


def _region(vol, sub):
    """vol[sub] as a host array (vol a host array or a device tensor)."""
    if isinstance(vol, np.ndarray):
        return vol[sub]
    import torch

    idx = [torch.as_tensor(np.asarray(i).reshape(-1), device=vol.device) for i in sub]
    return vol.index_select(0, idx[0]).index_select(1, idx[1]).index_select(2, idx[2]).cpu().numpy()


def time_cpu_sampler(sampler, warmup, steps):
    sampler.prepare()
    for _ in range(warmup):
        sampler.step()
    t0 = time.perf_counter()
    adv = 0.0
    for _ in range(steps):
        adv += sampler.step()
    wall = time.perf_counter() - t0
    return adv / wall, wall


def run_reference(args, ws, rank):
    """The reference's CPU block iteration restated in float32 with its padded R2C FFT
    convolution, on all host threads, one block per view per step on real psi."""
    if rank != 0:
        return
    import oracle

    oracle.build()
    ds = make_data()
    prep = prepare_reference_inputs(ds)
    psi0, mx = prep[5], prep[4]
    if psi0 is None:  # device-synthesised volumes: psi0 and the maxima on the host
        import torch

        mx = np.array([float(torch.max(im)) for im in ds.images], dtype=np.float32)
        avg = float(np.mean([float(im[im > 0].mean()) for im in ds.images]))
        psi0 = np.full((W.dims[2], W.dims[1], W.dims[0]), avg, np.float32)
    smp = cpu_sampler(ds, psi0, mx, prep)
    try:
        value, wall = time_cpu_sampler(smp, args.warmup, args.steps)
        sample = cpu_sample_text(args.steps, smp)
        threads = smp.workers
    finally:
        smp.close()
    line = {"impl": "reference", "metric": W.metric, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": W.config("reference (mirror-single / value-1 extension, padded FFT)"),
            "wall_s": wall,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def learned_summary(res):
    """The learned-proposal experiment without its per-step traces, with the metric's second
    half up front: wall time to relative L2 <= 1e-3 of the FP64 plain result (and to that
    result's likelihood), plain vs the best gated form (None: not reached)."""
    out = {k: v for k, v in res.items() if not k.startswith("trace")}
    forms = {}
    for k, v in res.items():
        if k.startswith("learned_every"):
            forms[k] = {kk: vv for kk, vv in v.items() if kk != "trace"}
    out.update(forms)
    best = min((v["t_err"] for v in forms.values() if v.get("t_err")), default=None)
    best_nll = min((v["t_nll"] for v in forms.values() if v.get("t_nll")), default=None)
    p = res["plain"]
    out["time_to_1e-3"] = {"plain_s": p["t_err"], "learned_s": best,
                           "speedup": (p["t_err"] / best) if (best and p["t_err"]) else None}
    out["time_to_fp64_likelihood"] = {"plain_s": p["t_nll"], "learned_s": best_nll,
                                      "speedup": (p["t_nll"] / best_nll) if (best_nll and p["t_nll"]) else None}
    return out


def fp64_error(M, views, n_iter, dev, boundary, d_img, d_w, ds):
    """Relative L2 of n_iter FP32 iterations against n_iter FP64 iterations of the same
    run from the same psi0 (PsiInitAvgPrecise); both through the whole-volume C ABI."""
    out = {}
    for prec in (M.PRECISION_FP32, M.PRECISION_FP64):
        with M.Deconvolution(W.dims, W.views, W.block, mul=False, psf_type=W.psf_type, psf_norm_threads=0, lam=W.lam,
                             boundary=boundary, precision=prec, weight_norm=W.weight_norm, device=dev) as d:
            W.setup_blocks(d)
            for v in range(views):
                d.set_view_device(v, d_img[v].data_ptr(), d_w[v].data_ptr(), ds.psfs[v])
            d.prepare()
            d.run_iterations(n_iter)
            out[prec] = d.get_psi()
    a = out[M.PRECISION_FP32].astype(np.float64)
    b = out[M.PRECISION_FP64].astype(np.float64)
    return {"value": float(np.linalg.norm(a - b) / np.linalg.norm(b)), "iterations": n_iter,
            "what": "relative L2 of psi after the FP32 iterations against the FP64 run of the same iterations "
                    "(same psi0, same kernels, every stage in double)"}


def run_gb300(args, ws, rank, local):
    import torch

    import mvrgb300 as M

    pre_datasets = None
    if args.learned and W.name != "4view256":
        args.learned = False  # the experiment is defined on the 4-view 256^3 setup
    if args.learned and rank == 0:
        # CPU synthesis of the training objects before the first GPU call
        import learned

        pre_datasets = learned.synthesize((128, 128, 128), [2000 + o for o in range(args.learned_objects)],
                                          (31, 31, 61))
    torch.cuda.set_device(local)
    dev = local
    ds = make_data()
    shape = (W.dims[2], W.dims[1], W.dims[0])
    boundary = M.BOUNDARY_CIRCULAR if args.boundary == "circular" else M.BOUNDARY_REFERENCE
    on_dev = torch.is_tensor(ds.images[0])  # synthesised on the device (large workload)
    d_img = ds.images if on_dev else [torch.from_numpy(a).to(f"cuda:{dev}") for a in ds.images]
    d_w = ds.weights if on_dev else [torch.from_numpy(a).to(f"cuda:{dev}") for a in ds.weights]
    dec = M.Deconvolution(W.dims, W.views, W.block, mul=False, psf_type=W.psf_type, psf_norm_threads=0,
                          lam=W.lam, boundary=boundary, precision=M.PRECISION_FP32, weight_norm=W.weight_norm,
                          batch_blocks=args.batch, device=dev)
    W.setup_blocks(dec)
    if args.schedule >= 0:
        dec.set_schedule(args.schedule)
    for v in range(W.views):
        dec.set_view_device(v, d_img[v].data_ptr(), d_w[v].data_ptr(), ds.psfs[v])
    dec.prepare()
    autotune = {"schedules": [M.schedule_name(dec.schedule(v)) for v in range(W.views)],
                "trials": [dict(t, ms=round(t["ms"], 4)) for t in dec.tuning()]}
    dec_max = dec.max_intensities()
    stream = torch.cuda.ExternalStream(dec.stream_ptr(), device=f"cuda:{dev}")
    batch = dec.batch()
    for _ in range(args.warmup):
        dec.run_iterations(1)
    dec.synchronize()

    # ---- value: device-resident, K steps bracketed by barrier + synchronize ----
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier(ws)
    torch.cuda.synchronize()
    launches0 = dec.launch_count()
    flush = W.flush_l2()
    with ClockSampler(dev) as clk:
        if flush:
            # inputs smaller than L2: a 512 MiB write flushes it before every step, outside
            # the per-step event pair
            junk = torch.empty(128 << 20, dtype=torch.float32, device=f"cuda:{dev}")
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
            with torch.cuda.stream(stream):
                for a, b in ev:
                    junk.fill_(1.0)
                    a.record(stream)
                    dec.run_iterations(1)
                    b.record(stream)
        else:
            e0.record(stream)
            for _ in range(args.steps):
                dec.run_iterations(1)
            e1.record(stream)
        torch.cuda.synchronize()
        dec.synchronize()
    launches = dec.launch_count() - launches0
    ms = sum(a.elapsed_time(b) for a, b in ev) if flush else e0.elapsed_time(e1)
    barrier(ws)
    ms = max_over_ranks(ms, ws)
    clocks = clk.summary()
    value = ws * W.nvox * args.steps / (ms / 1e3)

    # ---- the same iterations returning the per-block change statistics (ComputeBlockThread's
    # IterationStatistics): every block voxel is updated and reduced, not only the write regions
    stat_steps = max(1, min(args.steps, 5))
    for _ in range(2):
        dec.run_iterations(1, stats=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(stat_steps):
        dec.run_iterations(1, stats=True)
    e1.record(stream)
    torch.cuda.synchronize()
    stats_ms = max_over_ranks(e0.elapsed_time(e1), ws) / stat_steps

    # ---- roofline: per-kernel CUDA events on the library stream, same workload ----
    dec.set_profiling(True)
    prof_steps = max(1, min(args.steps, 3))
    for _ in range(prof_steps):
        dec.run_iterations(1)
    prof = dec.profile()
    dec.set_profiling(False)
    total_ms = sum(v[0] for v in prof.values()) or 1.0
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    dname, (dms, dlaunch, dbytes) = dom
    peak, peak_kind = load_peaks()
    achieved = (dbytes / dlaunch) / (dms / dlaunch / 1e3) / 1e9 if dlaunch else 0.0
    # the committed ncu capture is of the 4-view 256^3 workload
    traffic = ncu_traffic().get(dname) if W.name == "4view256" else None
    kernels = {k: {"share": v[0] / total_ms, "launches": v[1],
                   "gbs": (v[2] / (v[0] / 1e3) / 1e9) if v[0] > 0 else None} for k, v in prof.items() if v[1]}
    path_bytes = sum(v[2] for v in prof.values())
    roofline = {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": traffic, "bytes_per_launch": dbytes / max(1, dlaunch),
                "path_achieved": path_bytes / (total_ms / 1e3) / 1e9, "kernels": kernels}
    # the whole path against the algorithmic byte model of one view-block, 28 N + 48 Pc
    # (N block voxels, Pc = (bx / 2 + 1) by bz spectrum values), over the timed steps
    b_it = 0.0
    for v in range(W.views):
        b = W.vblocks[v]
        bn = b[0] * b[1] * b[2]
        bpc = (b[0] // 2 + 1) * b[1] * b[2]
        b_it += len(W.blocks(v)) * (28.0 * bn + 48.0 * bpc)
    roofline["model_bytes_per_iteration"] = b_it
    roofline["model_achieved"] = b_it * args.steps / (ms / 1e3) / 1e9
    roofline["model_frac"] = roofline["model_achieved"] / peak

    # ---- e2e: public C ABI with pinned host buffers, copies inside the timed region ----
    if args.no_e2e or on_dev:
        e2e = None  # the large workload keeps its volumes on the device only
        e2e_block = None
    else:
        e2e = run_e2e(args, ws, dev, ds, dec, shape, boundary)
        # one block worker size: the per-block path of one-block-size workloads
        e2e_block = None if W.per_view_blocks() else run_e2e_block(args, ws, dev, ds, dec, dec_max)
    psi_now = dec.get_psi()
    dec.close()
    # ---- every result's error against an FP64 run of the same iterations ----
    n64 = W.fp64_iters if W.fp64_iters is not None else args.warmup + args.steps
    err64 = fp64_error(M, W.views, n64, dev, boundary, d_img, d_w, ds) if not args.no_fp64 else None
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        import oracle

        oracle.build()
        prep = prepare_reference_inputs(ds)
        smp = cpu_sampler(ds, psi_now, dec_max, prep)  # the GPU run's psi: real data, not a constant
        try:
            cval, _ = time_cpu_sampler(smp, 0, args.cpu_steps)
            cpu = {"value": cval, "unit": UNIT, "cores": smp.workers, "kind": "port",
                   "sample": cpu_sample_text(args.cpu_steps, smp)}
        finally:
            smp.close()
    learned_res = None
    if args.learned and rank == 0:
        import learned

        learned_res = learned.experiment(ds, W.dims, W.block, n_objects=args.learned_objects,
                                         train_steps=args.learned_steps, pairs_per_object=30, device=dev,
                                         datasets=pre_datasets)
    if rank == 0:
        line = {"metric": W.metric, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(W.config(args.boundary), batch_blocks=batch), "clocks": clocks, "autotune": autotune,
                "gpu_launches": launches, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "with_statistics": {"ms_per_step": stats_ms, "value": ws * W.nvox / (stats_ms / 1e3),
                                    "steps": stat_steps,
                                    "note": "iterations that also return the per-block change statistics: every "
                                            "block voxel updated and reduced (value and ms_per_step above skip the "
                                            "voxels outside the write regions, which the reference discards)"}}
        if learned_res is not None:
            line["learned"] = learned_summary(learned_res)
        if e2e_block is not None:
            line["e2e_block"] = e2e_block
        if err64 is not None:
            line["err_vs_fp64"] = err64
        print(json.dumps(line), flush=True)


def run_e2e(args, ws, dev, ds, dec, shape, boundary):
    """The public C ABI with pinned host buffers: every step uploads psi, runs one iteration
    and reads psi back, and uploads the images and raw weights of the next step while its
    iteration runs (mvr_decon_run_host_next; the first timed step's set came up during the
    last warm-up step, the last timed step's set is uploaded inside the timed region)."""
    import torch

    import mvrgb300 as M

    h_img = [torch.from_numpy(a).pin_memory() for a in ds.images]
    h_w = [torch.from_numpy(a).pin_memory() for a in ds.weights]
    h_psi = torch.empty(shape, dtype=torch.float32).pin_memory()
    h_psi.copy_(torch.from_numpy(dec.get_psi()))
    e2e_dec = M.Deconvolution(W.dims, W.views, W.block, mul=False, psf_type=W.psf_type,
                              psf_norm_threads=0, lam=W.lam, boundary=boundary, precision=M.PRECISION_FP32,
                              weight_norm=W.weight_norm, device=dev)
    W.setup_blocks(e2e_dec)
    for v in range(W.views):
        e2e_dec.set_view(v, h_img[v].numpy(), h_w[v].numpy(), ds.psfs[v])
    e2e_dec.prepare()
    out = h_psi.numpy()
    e2e_steps = max(1, min(args.steps, 10))
    imgs = [a.numpy() for a in h_img]
    wts = [a.numpy() for a in h_w]
    for _ in range(min(2, args.warmup)):
        e2e_dec.run_host(1, imgs, wts, out, imgs, wts)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        # mvr_decon_run_host_next: psi up, one iteration, psi back; the next step's images and
        # raw weights upload during this step's iteration (every step uploads one full set)
        e2e_dec.run_host(1, imgs, wts, out, imgs, wts)
    e2e_dec.synchronize()  # the last step's uploads are inside the timed region
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    e2e_value = ws * W.nvox * e2e_steps / e2e_s
    h2d = W.views * 2 * W.nvox * 4 + W.nvox * 4
    d2h = W.nvox * 4
    e2e_dec.close()
    return {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": e2e_steps}


def run_e2e_block(args, ws, dev, ds, dec, dec_max, workers=2, iters=2):
    """The drop-in per-block path: mvr_block_run_seq (ComputeBlockSeqThread.runIteration,
    ComputeBlockSeqThread.java:54-61) with host buffers, one call per view-block as the
    reference's driver issues them (MultiViewDeconvolutionSeq.java:91-150), from `workers`
    host threads with one block worker each (numParallelBlocks = 2, so one worker's copies
    overlap the other's kernels).  Like the reference's CUDA block thread, every worker keeps
    its own psi, image and weight arrays and the driver copies each block into them
    (Block.copyBlock) before the call and the psi block out after it (pasteBlock); those host
    copies are the driver's work and run untimed.  A call uploads the three arrays, runs the
    iteration and returns the psi block and its statistics.  Timed: the calls; a view-step
    counts the longest of the workers' summed call times (the workers run concurrently)."""
    import concurrent.futures as cf

    import cpu_reference as R
    import mvrgb300 as M

    psi = dec.get_psi()
    wts = [dec.weights(v) for v in range(W.views)]
    boundary = M.BOUNDARY_CIRCULAR
    shape = (W.block[2], W.block[1], W.block[0])
    wk = [M.BlockWorker(W.block, 1e-4, W.lam, W.views, boundary, dev) for _ in range(workers)]
    hot = [[np.zeros(shape, np.float32) for _ in range(3)] for _ in range(workers)]  # psi, img, weight per worker
    try:
        for w in wk:
            for v in range(W.views):
                k1, k2 = dec.kernels(v, ds.psfs[v].shape)
                w.set_kernels(v, k1, k2)
        grids = [W.blocks(v) for v in range(W.views)]
        inputs = [[(R.extract(ds.images[v], bl["offset"], W.block, "zero"),
                    R.extract(wts[v], bl["offset"], W.block, "zero")) for bl in grids[v]] for v in range(W.views)]
        pool = cf.ThreadPoolExecutor(max_workers=workers)
        calls = 0
        step_s = []
        per_call = []
        for it in range(1 + iters):
            t_it = 0.0
            for v in range(W.views):
                pb = [R.extract(psi, bl["offset"], W.block, "mirror") for bl in grids[v]]

                def run(r, v=v, pb=pb):
                    hp, hi, hw = hot[r]
                    spent = []
                    for j in range(r, len(pb), workers):
                        np.copyto(hp, pb[j])
                        np.copyto(hi, inputs[v][j][0])
                        np.copyto(hw, inputs[v][j][1])
                        c0 = time.perf_counter()
                        wk[r].run_iteration(v, hp, hi, hw, float(dec_max[v]))
                        spent.append(time.perf_counter() - c0)
                        np.copyto(pb[j], hp)
                    return spent

                spents = list(pool.map(run, range(workers)))
                t_it += max(sum(x) for x in spents)
                for j, bl in enumerate(grids[v]):
                    R.paste(psi, pb[j], bl["eff_offset"], bl["eff_size"], bl["eff_local"])
                if it:
                    calls += len(pb)
                    per_call += [x for sp in spents for x in sp]
            if it:
                step_s.append(t_it)
        pool.shutdown()
    finally:
        for w in wk:
            w.close()
    t = float(np.mean(step_s))
    nb = 4 * W.block[0] * W.block[1] * W.block[2]
    return {"value": ws * W.nvox / t, "unit": UNIT, "h2d_bytes_per_step": 3 * nb * calls // iters,
            "d2h_bytes_per_step": nb * calls // iters, "calls_per_step": calls // iters, "steps": iters,
            "workers": workers, "ms_per_call": 1e3 * float(np.mean(per_call)) if per_call else None,
            "boundary": "circular (the pasted effective regions are the reference boundary's; "
                        "the per-block statistics differ)",
            "note": "timed: the mvr_block_run_seq calls (pageable host arrays kept per worker, as the reference's "
                    "CUDA block thread keeps its float[] arrays); the driver's block copies into / out of them and "
                    "into the volumes run untimed"}


def run_psf(args):
    """PSF preparation on one GPU: PSFExtraction.extractPSFLocal of 2000 beads (PSF 31x31x61)
    from one 1024x1024x512 float view on the device, and PSFPreparation.loadGroupTransformPSFs
    of 8 views in 4 groups.  The oracle's extraction on the host cores is the CPU baseline
    (a bounded sample of beads, scaled per bead)."""
    import numpy as np
    import torch

    import mvrgb300 as M

    dev = 0
    torch.cuda.set_device(dev)
    dims, nloc, size = (1024, 1024, 512), 2000, (31, 31, 61)
    g = torch.Generator(device=f"cuda:{dev}")
    g.manual_seed(1005)
    img = torch.rand((dims[2], dims[1], dims[0]), generator=g, device=f"cuda:{dev}", dtype=torch.float32) * 100
    rng = np.random.default_rng(1005)
    loc = rng.uniform(0, 1, (nloc, 3)) * np.array(dims, dtype=np.float64)
    out = torch.empty((size[2], size[1], size[0]), dtype=torch.float32, device=f"cuda:{dev}")
    for _ in range(args.warmup):
        M.psf_extract(img.data_ptr(), dims, loc, size, out.data_ptr(), dev)
    steps = max(1, min(args.steps, 10))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        M.psf_extract(img.data_ptr(), dims, loc, size, out.data_ptr(), dev)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    psf = out.cpu().numpy()
    views = [(psf, np.hstack([np.eye(3) * (1.0, 1.0, 1.0 + 0.1 * v), np.zeros((3, 1))])) for v in range(8)]
    groups = [views[2 * k:2 * k + 2] for k in range(4)]
    M.load_group_transform_psfs(groups, True, dev)
    t0 = time.perf_counter()
    M.load_group_transform_psfs(groups, True, dev)
    prep_ms = (time.perf_counter() - t0) * 1e3
    cpu = None
    if not args.no_cpu:
        import oracle

        himg = img[:128, :128, :128].cpu().numpy()
        sample = 8
        sl = rng.uniform(0, 128, (sample, 3))
        t0 = time.perf_counter()
        oracle.psf_extract(himg, sl, size)
        per = (time.perf_counter() - t0) / sample
        cpu = {"value": 1.0 / per, "unit": "beads/s", "cores": 1, "kind": "port",
               "sample": f"{sample} beads, PSF 31x31x61, numpy restatement of extractPSFLocal on one core"}
    line = {"metric": "PSF bead neighbourhoods extracted/s", "value": nloc / (ms / 1e3), "unit": "beads/s",
            "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "dtype": "f32 data, f64 positions and weights", "data": "synthetic",
            "config": {"workload": "PSF extraction, 2000 beads, PSF 31x31x61, view 1024x1024x512 float32 on the device",
                       "group_preparation": "8 views in 4 groups: normalise, transform, average, same size"},
            "group_preparation_ms": prep_ms, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="4view256",
                    help="4view256: 4 views 256^3 (the headline case); 6view512: 6 views 512x512x256 with "
                         "per-view PSF sizes and uneven edge blocks; 8view1024: 8 views 1024x1024x512, 256^3 "
                         "blocks (volumes synthesised on the device, no e2e line)")
    ap.add_argument("--boundary", choices=["circular", "reference"], default="circular")
    ap.add_argument("--schedule", type=int, default=-1,
                    help="force one FFT schedule code for every view (mvr_decon_set_schedule); -1 = autotuned")
    ap.add_argument("--batch", type=int, default=0,
                    help="blocks per batched launch (1..16); 0 = autotuned")
    ap.add_argument("--cpu-steps", type=int, default=2,
                    help="steps of the CPU baseline sample (one block per view each)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-learned", dest="learned", action="store_false",
                    help="skip the learned-proposal experiment (training + gated runs vs plain; on by default "
                         "for the 4-view 256^3 workload)")
    ap.add_argument("--learned-objects", type=int, default=24)
    ap.add_argument("--learned-steps", type=int, default=800, help="training steps of the learned proposal")
    ap.add_argument("--psf", action="store_true",
                    help="time the PSF preparation instead (bead extraction from a 1024x1024x512 view)")
    args = ap.parse_args()
    if args.psf:
        run_psf(args)
        return
    global W
    W = WORKLOADS[args.workload]()
    ws, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        run_gb300(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
