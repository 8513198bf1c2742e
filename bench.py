#!/usr/bin/env python3
"""Throughput of the multiview Bayesian (RL-type) deconvolution iteration on GB300.

Workload (the reference's 4-view case): 4 views of 256^3 float32, PSFs 31x31x61
Gaussian-plus-side-lobes rotated 0/45/90/135 degrees about y, Optimization-I compound
kernels, cosine-blended weights normalised with the reference's hard rule, psi from
PsiInitAvgPrecise, Tikhonov lambda 0.006, compute blocks 192^3 (16 per view).
Synthetic seeded data stands in for the reference's microscopy datasets.

A step is one full iteration (all 4 views, all blocks) over the whole volume.
Metric: voxel-iterations/s = 256^3 * steps / seconds.

  value  device-resident inputs, CUDA events on the library's stream around K steps
  e2e    the public C ABI with pinned host buffers: every step uploads the 4 images,
         4 raw weights and psi, runs one iteration and reads psi back
  --impl reference  the CPU restatement of the reference block iteration (oracle/,
         all host threads) on a bounded sample of the same workload
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

    def __init__(self, name, dims, views, block, psfs, lam, make, desc):
        self.name, self.dims, self.views, self.block, self.psfs, self.lam = name, dims, views, block, psfs, lam
        self.make, self.desc = make, desc
        self.nvox = dims[0] * dims[1] * dims[2]
        self.metric = f"voxel-iterations/s ({views} views)"

    def blocks(self, v):
        import oracle

        kk = tuple(2 * k - 1 for k in self.psfs[v])
        return oracle.divide_into_blocks(self.dims, kk, self.block)

    def view_blocks_per_iter(self):
        return sum(len(self.blocks(v)) for v in range(self.views))

    def config(self, boundary):
        return {"workload": self.desc, "views": self.views, "dims": list(self.dims), "block": list(self.block),
                "psf": [list(p) for p in self.psfs] if len(set(self.psfs)) > 1 else list(self.psfs[0]),
                "lambda": self.lam, "iterations_per_step": 1, "boundary": boundary,
                "l2": f"inputs larger than L2 ({self.views} images + {self.views} weights + psi = "
                      f"{(2 * self.views + 1) * self.nvox * 4 / 2**20:.0f} MiB)",
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


def _psf_sizes_6():
    import synthetic

    return [tuple(p) for p in synthetic.PSF_SIZES_6]


WORKLOADS = {
    "4view256": lambda: Workload("4view256", (256, 256, 256), 4, (192, 192, 192), [(31, 31, 61)] * 4, 0.006, _make256,
                                 "4 views 256^3 float32, PSF 31x31x61 Optimization-I, blocks 192^3, Seq (OSEM-like)"),
    "6view512": lambda: Workload("6view512", (512, 512, 256), 6, (192, 192, 256), _psf_sizes_6(), 0.006, _make512,
                                 "6 views 512x512x256 float32, PSFs 21x21x41 ... 41x41x81 per view, "
                                 "Optimization-I, compute blocks 192x192x256 (effective 112-152 x 112-152 x 96-176, "
                                 "uneven edge blocks), Seq"),
    "8view1024": lambda: Workload("8view1024", (1024, 1024, 512), 8, (256, 256, 256), [(41, 41, 81)] * 8, 0.006,
                                  _make_large,
                                  "8 views 1024x1024x512 (uint16 recorded, converted to float32), 20000 nuclei-like "
                                  "blobs, PSF 41x41x81 at 45 degree steps, compute blocks 256^3 (216 per view), Seq"),
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


def cpu_block_sample(ds, k1s, k2s, mx, n_blocks):
    """Times the oracle (reference-faithful CPU block iteration) on n_blocks view-blocks
    of the workload; returns (seconds per view-block, threads)."""
    import oracle

    D = W.dims
    B = W.block
    times = []
    for i in range(n_blocks):
        v = i % W.views
        blocks = W.blocks(v)
        bl = blocks[(5 + i) % len(blocks)]
        off = bl["offset"]
        idx = [np.arange(off[d], off[d] + B[d]) for d in range(3)]
        psi = np.full((B[2], B[1], B[0]), 50.0, np.float32)
        img = np.zeros_like(psi)
        w = np.zeros_like(psi)
        ok = [(idx[d] >= 0) & (idx[d] < D[d]) for d in range(3)]
        sub = np.ix_(idx[2][ok[2]], idx[1][ok[1]], idx[0][ok[0]])
        dst = np.ix_(np.nonzero(ok[2])[0], np.nonzero(ok[1])[0], np.nonzero(ok[0])[0])
        img[dst] = _region(ds.images[v], sub)
        if isinstance(ds.weights[v], np.ndarray):
            w[dst] = ds.weights[v][sub]
        else:  # raw device weights: normalise this region with the hard rule
            raw = [_region(ds.weights[u], sub) for u in range(W.views)]
            w[dst] = oracle.normalize_weights(raw)[v]
        t0 = time.perf_counter()
        oracle.block_seq(psi, img, w, k1s[v], k2s[v], W.lam, 1e-4, float(mx[v]))
        times.append(time.perf_counter() - t0)
    return float(np.mean(times)), oracle.num_threads()


def cpu_sample_text(n):
    dom = "x".join(str(W.block[d] + W.psfs[0][d] - 1) for d in range(3))
    return (f"{n} view-block(s) of {W.block[0]}x{W.block[1]}x{W.block[2]} (reference boundary, FFT domain about "
            f"{dom}), extrapolated to the {W.view_blocks_per_iter()} view-blocks of one iteration")


def prepare_reference_inputs(ds, mx=None):
    """Kernels, normalised weights and per-view maxima for the CPU sample.  For device
    volumes (the large workload) the weights are normalised per sampled block (the hard
    rule is per voxel) and the maxima come from the GPU run (mx)."""
    import oracle

    k1s, k2s = oracle.psf_init(ds.psfs, oracle.PSF_OPTIMIZATION_I, 0)
    if mx is None:
        ws = oracle.normalize_weights(ds.weights)
        _, mx, _ = oracle.psi_init_avg(ds.images)
        ds.weights = ws
    return k1s, k2s, mx


def _region(vol, sub, normalise_with=None):
    """vol[sub] as a host array (vol a host array or a device tensor)."""
    if isinstance(vol, np.ndarray):
        return vol[sub]
    import torch

    idx = [torch.as_tensor(np.asarray(i).reshape(-1), device=vol.device) for i in sub]
    return vol.index_select(0, idx[0]).index_select(1, idx[1]).index_select(2, idx[2]).cpu().numpy()


def run_reference(args, ws, rank):
    if rank != 0:
        return
    import oracle

    oracle.build()
    ds = make_data()
    k1s, k2s, mx = prepare_reference_inputs(ds)
    threads = oracle.num_threads()
    for _ in range(args.warmup):
        cpu_block_sample(ds, k1s, k2s, mx, 1)
    t0 = time.perf_counter()
    per_vb = []
    for _ in range(args.steps):
        t, _ = cpu_block_sample(ds, k1s, k2s, mx, 1)
        per_vb.append(t)
    wall = time.perf_counter() - t0
    t_vb = float(np.mean(per_vb))
    nvb = W.view_blocks_per_iter()
    value = W.nvox / (t_vb * nvb)
    sample = cpu_sample_text(1) + " (one view-block per step)"
    line = {"impl": "reference", "metric": W.metric, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_vb * nvb,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": W.config("reference (mirror-single / value-1 extension)"),
            "wall_s": wall,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gb300(args, ws, rank, local):
    import torch

    import mvrgb300 as M

    pre_datasets = None
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
    dec = M.Deconvolution(W.dims, W.views, W.block, mul=False, psf_type=M.PSF_OPTIMIZATION_I, psf_norm_threads=0,
                          lam=W.lam, boundary=boundary, precision=M.PRECISION_FP32, weight_norm=M.WEIGHTS_HARD,
                          batch_blocks=args.batch, device=dev)
    for v in range(W.views):
        dec.set_view_device(v, d_img[v].data_ptr(), d_w[v].data_ptr(), ds.psfs[v])
    dec.prepare()
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
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            dec.run_iterations(1)
        e1.record(stream)
        torch.cuda.synchronize()
        dec.synchronize()
    launches = dec.launch_count() - launches0
    ms = e0.elapsed_time(e1)
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
    bn = W.block[0] * W.block[1] * W.block[2]
    bpc = (W.block[0] // 2 + 1) * W.block[1] * W.block[2]
    b_it = W.view_blocks_per_iter() * (28.0 * bn + 48.0 * bpc)
    roofline["model_bytes_per_iteration"] = b_it
    roofline["model_achieved"] = b_it * args.steps / (ms / 1e3) / 1e9
    roofline["model_frac"] = roofline["model_achieved"] / peak

    # ---- e2e: public C ABI with pinned host buffers, copies inside the timed region ----
    if args.no_e2e or on_dev:
        e2e = None  # the large workload keeps its volumes on the device only
    else:
        e2e = run_e2e(args, ws, dev, ds, dec, shape, boundary)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        import oracle

        oracle.build()
        k1s, k2s, mx = prepare_reference_inputs(ds, dec_max if on_dev else None)
        t_vb, threads = cpu_block_sample(ds, k1s, k2s, mx, args.cpu_blocks)
        cpu = {"value": W.nvox / (t_vb * W.view_blocks_per_iter()), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": cpu_sample_text(args.cpu_blocks)}
    dec.close()
    learned_res = None
    if args.learned and rank == 0:
        import learned

        learned_res = learned.experiment(ds, W.dims, W.block, n_objects=args.learned_objects, device=dev,
                                         datasets=pre_datasets)
    if rank == 0:
        line = {"metric": W.metric, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": dict(W.config(args.boundary), batch_blocks=batch), "clocks": clocks,
                "gpu_launches": launches, "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu,
                "with_statistics": {"ms_per_step": stats_ms, "value": ws * W.nvox / (stats_ms / 1e3),
                                    "steps": stat_steps,
                                    "note": "iterations that also return the per-block change statistics: every "
                                            "block voxel updated and reduced (value and ms_per_step above skip the "
                                            "voxels outside the write regions, which the reference discards)"}}
        if learned_res is not None:
            line["learned"] = learned_res
        print(json.dumps(line), flush=True)


def run_e2e(args, ws, dev, ds, dec, shape, boundary):
    """The public C ABI with pinned host buffers: every step uploads the 4 images, the 4
    raw weights and psi, runs one iteration and reads psi back."""
    import torch

    import mvrgb300 as M

    h_img = [torch.from_numpy(a).pin_memory() for a in ds.images]
    h_w = [torch.from_numpy(a).pin_memory() for a in ds.weights]
    h_psi = torch.empty(shape, dtype=torch.float32).pin_memory()
    h_psi.copy_(torch.from_numpy(dec.get_psi()))
    e2e_dec = M.Deconvolution(W.dims, W.views, W.block, mul=False, psf_type=M.PSF_OPTIMIZATION_I,
                              psf_norm_threads=0, lam=W.lam, boundary=boundary, precision=M.PRECISION_FP32, weight_norm=M.WEIGHTS_HARD,
                              device=dev)
    for v in range(W.views):
        e2e_dec.set_view(v, h_img[v].numpy(), h_w[v].numpy(), ds.psfs[v])
    e2e_dec.prepare()
    out = h_psi.numpy()
    e2e_steps = max(1, min(args.steps, 10))
    for _ in range(min(2, args.warmup)):
        for v in range(W.views):
            e2e_dec.update_images(v, h_img[v].numpy(), h_w[v].numpy())
        e2e_dec.set_psi(out)
        e2e_dec.run_iterations(1)
        e2e_dec.get_psi(out)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for v in range(W.views):
            e2e_dec.update_images(v, h_img[v].numpy(), h_w[v].numpy())
        e2e_dec.set_psi(out)
        e2e_dec.run_iterations(1)
        e2e_dec.get_psi(out)
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    e2e_value = ws * W.nvox * e2e_steps / e2e_s
    h2d = W.views * 2 * W.nvox * 4 + W.nvox * 4
    d2h = W.nvox * 4
    e2e_dec.close()
    return {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": e2e_steps}


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
    ap.add_argument("--batch", type=int, default=0,
                    help="blocks per batched launch (1..16); 0 = autotuned")
    ap.add_argument("--cpu-blocks", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--learned", action="store_true",
                    help="also run the learned-proposal experiment (training + gated run vs plain)")
    ap.add_argument("--learned-objects", type=int, default=50)
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
