"""Python mirror of the reference's per-block plugin surface over the C ABI
(include/mvr_gb300.h), loaded with ctypes from the in-tree libmvrgb300.so.

Reference interfaces (paths relative to src/main/java/ of PreibischLab/multiview-reconstruction,
MV = net/preibisch/mvrecon/process/deconvolution):

* ``ComputeBlockThreadFactory.create`` (MV/iteration/ComputeBlockThreadFactory.java:25-29)
  -> :class:`BlockWorker`
* ``ComputeBlockSeqThread.runIteration`` (MV/iteration/sequential/ComputeBlockSeqThread.java:54-61)
  -> :meth:`BlockWorker.run_iteration`
* ``ComputeBlockMulThread.runIteration`` (MV/iteration/mul/ComputeBlockMulThread.java:56-62)
  -> :meth:`BlockWorker.run_iteration_mul`
* ``ComputeBlockThread.IterationStatistics`` (MV/iteration/ComputeBlockThread.java:64-68)
  -> :class:`IterationStatistics`

There is no CPU fallback: loading fails with an exception when the library was not
built, and every call raises :class:`MvrError` on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmvrgb300.so")

OK, ERR_ARG, ERR_CUDA, ERR_OOM, ERR_UNSUPPORTED, ERR_STATE = 0, 1, 2, 3, 4, 5
PRECISION_FP32, PRECISION_FP64 = 0, 1
WEIGHTS_AS_GIVEN, WEIGHTS_HARD, WEIGHTS_SMOOTH = 0, 1, 2
KERNEL_KINDS = 11
BOUNDARY_REFERENCE, BOUNDARY_CIRCULAR = 0, 1
PSF_OPTIMIZATION_II, PSF_OPTIMIZATION_I, PSF_EFFICIENT_BAYESIAN, PSF_INDEPENDENT = 0, 1, 2, 3
PSI_INIT_AVG_PRECISE, PSI_INIT_AVG_APPROX, PSI_INIT_BLURRED_FUSED = 0, 1, 2

# every symbol include/mvr_gb300.h declares
EXPORTS = [
    "mvr_block_create", "mvr_block_destroy", "mvr_block_last_error", "mvr_block_set_kernels",
    "mvr_block_run_seq", "mvr_block_run_mul", "mvr_block_run_seq_device", "mvr_block_synchronize",
    "mvr_decon_create", "mvr_decon_destroy", "mvr_decon_last_error", "mvr_decon_set_view",
    "mvr_decon_set_view_device", "mvr_decon_set_view_block_size", "mvr_decon_set_effective_block_size",
    "mvr_decon_update_images", "mvr_decon_prepare", "mvr_decon_set_psi",
    "mvr_decon_set_psi_device", "mvr_decon_get_psi", "mvr_decon_get_psi_device", "mvr_decon_run", "mvr_decon_get_kernels",
    "mvr_decon_get_max", "mvr_decon_get_weights", "mvr_decon_psi_device", "mvr_decon_synchronize",
    "mvr_decon_stream", "mvr_decon_launch_count", "mvr_decon_set_profiling", "mvr_decon_get_profile",
    "mvr_kernel_name", "mvr_convolve_static", "mvr_decon_batch", "mvr_decon_likelihood",
    "mvr_decon_set_graphs", "mvr_decon_graphs_captured", "mvr_decon_set_schedule", "mvr_decon_schedule",
    "mvr_decon_tuning", "mvr_decon_run_host", "mvr_decon_run_host_next", "mvr_export_tiff", "mvr_export_n5", "mvr_pool2",
    "mvr_apply_coarse", "mvr_decon_init_psi", "mvr_fuse_group",
    "mvr_fuse_last_error", "mvr_psf_extract", "mvr_psf_transformed_dims", "mvr_psf_transform_normalized",
    "mvr_psf_average", "mvr_psf_make_same_size", "mvr_psf_projection", "mvr_psf_remove_min_projections",
    "mvr_psf_last_error", "mvr_block_grid",
    "mvr_unet_create", "mvr_unet_destroy", "mvr_unet_last_error", "mvr_unet_num_params", "mvr_unet_get_params",
    "mvr_unet_set_params", "mvr_unet_get_grads", "mvr_unet_set_input", "mvr_unet_forward", "mvr_unet_train_step",
    "mvr_unet_propose", "mvr_conv3d_tc", "mvr_conv3d_tc_wgrad", "mvr_conv3d_tc_last_error",
    "convolution3DfftCUDA", "convolution3DfftCUDAInPlace", "getNumDevicesCUDA", "getNameDeviceCUDA",
    "getMemDeviceCUDA", "getFreeMemDeviceCUDA", "getCUDAcomputeCapabilityMajorVersion",
    "getCUDAcomputeCapabilityMinorVersion", "mvr_free",
]


SCHED_ROWS, SCHED_PLANE, SCHED_PLANE_PERSIST, SCHED_PAIR, SCHED_ZPIPE = 0, 1, 2, 3, 4


def schedule_name(code: int) -> str:
    if code < 0:
        return "batch trial"
    path = {SCHED_ROWS: "row/column kernels", SCHED_PLANE: "plane kernels, one CTA per plane",
            SCHED_PLANE_PERSIST: "plane kernels, persistent",
            SCHED_PAIR: "pair plane kernels (two CTAs per plane), persistent"}[code & 3]
    return path + (" + persistent Z pass" if code & SCHED_ZPIPE else "")


class MvrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class _BlockParams(C.Structure):
    _fields_ = [("block_size", C.c_int * 3), ("min_value", C.c_float), ("lambda_", C.c_float),
                ("num_views", C.c_int), ("boundary", C.c_int), ("device", C.c_int)]


class _DeconParams(C.Structure):
    _fields_ = [("dims", C.c_int * 3), ("num_views", C.c_int), ("block_size", C.c_int * 3), ("mul", C.c_int),
                ("psf_type", C.c_int), ("psf_norm_threads", C.c_int), ("lambda_", C.c_float),
                ("min_value", C.c_float), ("boundary", C.c_int), ("precision", C.c_int),
                ("filter_blocks", C.c_int), ("weight_norm", C.c_int), ("osem_speedup", C.c_float),
                ("max_diff_range", C.c_float), ("scaling_range", C.c_float), ("batch_blocks", C.c_int),
                ("device", C.c_int)]


_lib = None


def load() -> C.CDLL:
    """Loads libmvrgb300.so (raises if it was not built: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} not built; run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    L.mvr_block_create.argtypes = [C.POINTER(_BlockParams), C.POINTER(P)]
    L.mvr_block_destroy.argtypes = [P]
    L.mvr_block_destroy.restype = None
    L.mvr_block_last_error.argtypes = [P]
    L.mvr_block_last_error.restype = C.c_char_p
    L.mvr_block_set_kernels.argtypes = [P, C.c_int, P, P, P]
    L.mvr_block_run_seq.argtypes = [P, C.c_int, P, P, P, C.c_float, P]
    L.mvr_block_run_mul.argtypes = [P, P, P, P, P, P]
    L.mvr_block_run_seq_device.argtypes = [P, C.c_int, P, P, P, C.c_float, P]
    L.mvr_block_synchronize.argtypes = [P]
    L.convolution3DfftCUDAInPlace.argtypes = [P, P, P, P, C.c_int]
    L.convolution3DfftCUDAInPlace.restype = None
    L.convolution3DfftCUDA.argtypes = [P, P, P, P, C.c_int]
    L.convolution3DfftCUDA.restype = C.POINTER(C.c_float)
    L.mvr_free.argtypes = [P]
    L.mvr_free.restype = None
    L.getNumDevicesCUDA.restype = C.c_int
    L.getNameDeviceCUDA.argtypes = [C.c_int, C.c_char_p]
    L.getNameDeviceCUDA.restype = None
    L.getMemDeviceCUDA.argtypes = [C.c_int]
    L.getMemDeviceCUDA.restype = C.c_longlong
    L.getFreeMemDeviceCUDA.argtypes = [C.c_int]
    L.getFreeMemDeviceCUDA.restype = C.c_longlong
    L.getCUDAcomputeCapabilityMajorVersion.argtypes = [C.c_int]
    L.getCUDAcomputeCapabilityMinorVersion.argtypes = [C.c_int]
    L.mvr_decon_create.argtypes = [C.POINTER(_DeconParams), C.POINTER(P)]
    L.mvr_decon_destroy.argtypes = [P]
    L.mvr_decon_destroy.restype = None
    L.mvr_decon_last_error.argtypes = [P]
    L.mvr_decon_last_error.restype = C.c_char_p
    L.mvr_decon_set_view.argtypes = [P, C.c_int, P, P, P, P]
    L.mvr_decon_set_view_device.argtypes = [P, C.c_int, P, P, P, P]
    L.mvr_decon_update_images.argtypes = [P, C.c_int, P, P]
    L.mvr_decon_set_view_block_size.argtypes = [P, C.c_int, P]
    L.mvr_decon_set_effective_block_size.argtypes = [P, C.c_int, P]
    L.mvr_decon_set_schedule.argtypes = [P, C.c_int]
    L.mvr_decon_schedule.argtypes = [P, C.c_int]
    L.mvr_decon_tuning.argtypes = [P, C.c_int, P, P, P, P]
    L.mvr_decon_run_host.argtypes = [P, C.c_int, P, P, P]
    L.mvr_decon_run_host_next.argtypes = [P, C.c_int, P, P, P, P, P]
    L.mvr_export_tiff.argtypes = [C.c_char_p, P, P, C.c_int, P, C.c_char_p, C.c_char_p, C.c_int]
    L.mvr_pool2.argtypes = [P, P, P, P]
    L.mvr_apply_coarse.argtypes = [P, P, P, P, P, C.c_float, P, P]
    L.mvr_export_n5.argtypes = [C.c_char_p, C.c_char_p, P, P, C.c_int, P, C.c_char_p, C.c_int]
    L.mvr_decon_prepare.argtypes = [P]
    L.mvr_decon_set_psi.argtypes = [P, P]
    L.mvr_decon_set_psi_device.argtypes = [P, P]
    L.mvr_decon_get_psi.argtypes = [P, P]
    L.mvr_decon_get_psi_device.argtypes = [P, P]
    L.mvr_decon_run.argtypes = [P, C.c_int, P]
    L.mvr_decon_get_kernels.argtypes = [P, C.c_int, P, P]
    L.mvr_decon_get_max.argtypes = [P, P]
    L.mvr_decon_get_weights.argtypes = [P, C.c_int, P]
    L.mvr_decon_psi_device.argtypes = [P]
    L.mvr_decon_psi_device.restype = C.c_void_p
    L.mvr_decon_synchronize.argtypes = [P]
    L.mvr_decon_stream.argtypes = [P]
    L.mvr_decon_stream.restype = C.c_void_p
    L.mvr_decon_launch_count.argtypes = [P]
    L.mvr_decon_launch_count.restype = C.c_longlong
    L.mvr_decon_set_profiling.argtypes = [P, C.c_int]
    L.mvr_decon_get_profile.argtypes = [P, P, P, P]
    L.mvr_kernel_name.argtypes = [C.c_int]
    L.mvr_kernel_name.restype = C.c_char_p
    L.mvr_convolve_static.argtypes = [P, P, P, P, P, P, C.c_char_p, C.c_int]
    L.mvr_decon_batch.argtypes = [P]
    L.mvr_decon_set_graphs.argtypes = [P, C.c_int]
    L.mvr_decon_init_psi.argtypes = [P, C.c_int, C.c_double, P]
    L.mvr_fuse_group.argtypes = [P, C.c_int, P, P, P, P, C.c_int, P]
    L.mvr_fuse_last_error.restype = C.c_char_p
    L.mvr_psf_extract.argtypes = [P, P, P, C.c_int, P, P, C.c_int, P]
    L.mvr_psf_transformed_dims.argtypes = [P, P, P]
    L.mvr_psf_transform_normalized.argtypes = [P, P, P, P, P, C.c_int, P]
    L.mvr_psf_average.argtypes = [P, P, C.c_int, C.c_int, P, P, C.c_int, P]
    L.mvr_psf_make_same_size.argtypes = [P, P, P, P, C.c_int, P]
    L.mvr_psf_projection.argtypes = [P, P, C.c_int, C.c_int, P, P, C.c_int, P]
    L.mvr_psf_remove_min_projections.argtypes = [P, P, C.c_int, P]
    L.mvr_psf_last_error.restype = C.c_char_p
    L.mvr_block_grid.argtypes = [P, P, P, C.c_int, P, C.c_int, P]
    L.mvr_decon_graphs_captured.argtypes = [P]
    L.mvr_decon_likelihood.argtypes = [P, P, P]
    L.mvr_unet_create.argtypes = [C.c_int, P, C.c_uint, C.c_int, C.POINTER(P)]
    L.mvr_unet_destroy.argtypes = [P]
    L.mvr_unet_destroy.restype = None
    L.mvr_unet_last_error.argtypes = [P]
    L.mvr_unet_last_error.restype = C.c_char_p
    L.mvr_unet_num_params.argtypes = [P]
    L.mvr_unet_num_params.restype = C.c_longlong
    for f in ("mvr_unet_get_params", "mvr_unet_set_params", "mvr_unet_get_grads"):
        getattr(L, f).argtypes = [P, P]
    L.mvr_unet_set_input.argtypes = [P, P, P, P]
    L.mvr_unet_forward.argtypes = [P, P]
    L.mvr_unet_train_step.argtypes = [P, C.c_float, P]
    L.mvr_unet_propose.argtypes = [P, P, P, C.c_float]
    L.mvr_conv3d_tc.argtypes = [P, C.c_int, P, C.c_int, P, C.c_int, C.c_int, P, P, P, P]
    L.mvr_conv3d_tc_wgrad.argtypes = [P, C.c_int, P, C.c_int, P, P, P, P]
    L.mvr_conv3d_tc_last_error.restype = C.c_char_p
    _lib = L
    return L


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _size_xyz(a: np.ndarray):
    return (C.c_int * 3)(a.shape[2], a.shape[1], a.shape[0])


@dataclass
class IterationStatistics:
    """ComputeBlockThread.IterationStatistics: signed sum and max of the change."""
    sum_change: float = 0.0
    max_change: float = -1.0


class BlockWorker:
    """One block worker (ComputeBlockSeqThread / ComputeBlockMulThread) on one GPU.

    ``block_size`` is (x, y, z); arrays are float32 [z][y][x]."""

    def __init__(self, block_size, min_value: float = 1e-4, lam: float = 0.0, num_views: int = 1,
                 boundary: int = BOUNDARY_REFERENCE, device: int = 0):
        self._lib = load()
        prm = _BlockParams((C.c_int * 3)(*block_size), min_value, lam, num_views, boundary, device)
        h = C.c_void_p()
        rc = self._lib.mvr_block_create(C.byref(prm), C.byref(h))
        if rc != OK:
            raise MvrError(rc, self._lib.mvr_block_last_error(None).decode())
        self._h = h
        self.block_size = tuple(block_size)
        self.min_value = min_value
        self.num_views = num_views

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mvr_block_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != OK:
            raise MvrError(rc, self._lib.mvr_block_last_error(self._h).decode())

    @property
    def shape(self):
        return (self.block_size[2], self.block_size[1], self.block_size[0])

    def set_kernels(self, view: int, kernel1, kernel2):
        k1, k2 = _f32(kernel1), _f32(kernel2)
        if k1.shape != k2.shape:
            raise ValueError("kernel1 and kernel2 must have the same shape")
        self._check(self._lib.mvr_block_set_kernels(self._h, view, _p(k1), _p(k2), _size_xyz(k1)))

    def run_iteration(self, view: int, psi_block, img_block, weight_block, max_intensity: float):
        """ComputeBlockSeqThread.runIteration; psi_block (float32) is updated in place."""
        if psi_block.dtype != np.float32 or not psi_block.flags.c_contiguous or psi_block.shape != self.shape:
            raise ValueError("psi_block must be a C-contiguous float32 array of the block shape")
        img, w = _f32(img_block), _f32(weight_block)
        if img.shape != self.shape or w.shape != self.shape:
            raise ValueError("img/weight blocks must have the block shape")
        st = np.zeros(2, dtype=np.float64)
        self._check(self._lib.mvr_block_run_seq(self._h, view, _p(psi_block), _p(img), _p(w),
                                                float(max_intensity), _p(st)))
        return IterationStatistics(float(st[0]), float(st[1]))

    def run_iteration_mul(self, psi_block, img_blocks, weight_blocks, max_intensities):
        """ComputeBlockMulThread.runIteration over all views; psi_block updated in place."""
        if psi_block.dtype != np.float32 or not psi_block.flags.c_contiguous or psi_block.shape != self.shape:
            raise ValueError("psi_block must be a C-contiguous float32 array of the block shape")
        imgs = [_f32(a) for a in img_blocks]
        ws = [_f32(a) for a in weight_blocks]
        if len(imgs) != self.num_views or len(ws) != self.num_views:
            raise ValueError("one image and one weight block per view")
        ip = (C.c_void_p * self.num_views)(*[a.ctypes.data for a in imgs])
        wp = (C.c_void_p * self.num_views)(*[a.ctypes.data for a in ws])
        mx = np.asarray(max_intensities, dtype=np.float32)
        st = np.zeros(2, dtype=np.float64)
        self._check(self._lib.mvr_block_run_mul(self._h, _p(psi_block), ip, wp, _p(mx), _p(st)))
        return IterationStatistics(float(st[0]), float(st[1]))

    def run_iteration_device(self, view: int, psi_ptr: int, img_ptr: int, w_ptr: int, max_intensity: float,
                             stats_ptr: int = 0):
        """Queues one iteration on device buffers (raw device addresses)."""
        self._check(self._lib.mvr_block_run_seq_device(self._h, view, C.c_void_p(psi_ptr), C.c_void_p(img_ptr),
                                                       C.c_void_p(w_ptr), float(max_intensity),
                                                       C.c_void_p(stats_ptr) if stats_ptr else None))

    def synchronize(self):
        self._check(self._lib.mvr_block_synchronize(self._h))


class Deconvolution:
    """Device-resident MultiViewDeconvolutionSeq / MultiViewDeconvolutionMul
    (MultiViewDeconvolution.java:90-200) with DeconViews/DeconViewPSF.init, the block grid,
    weight normalisation and PsiInitAvgPrecise.  Volumes are float32 [z][y][x]; sizes (x, y, z)."""

    def __init__(self, dims, num_views, block_size, mul=False, psf_type=PSF_OPTIMIZATION_I,
                 psf_norm_threads=0, lam=0.006, min_value=1e-4, boundary=BOUNDARY_REFERENCE,
                 precision=PRECISION_FP32, filter_blocks=True, weight_norm=WEIGHTS_AS_GIVEN, osem_speedup=1.0,
                 max_diff_range=0.1, scaling_range=0.05, batch_blocks=0, device=0):
        self._lib = load()
        prm = _DeconParams((C.c_int * 3)(*dims), num_views, (C.c_int * 3)(*block_size), int(mul), psf_type,
                           psf_norm_threads, lam, min_value, boundary, precision, int(filter_blocks), weight_norm,
                           osem_speedup, max_diff_range, scaling_range, batch_blocks, device)
        h = C.c_void_p()
        rc = self._lib.mvr_decon_create(C.byref(prm), C.byref(h))
        if rc != OK:
            raise MvrError(rc, self._lib.mvr_decon_last_error(None).decode())
        self._h = h
        self.dims = tuple(dims)
        self.num_views = num_views
        self.mul = bool(mul)
        self._keep = {}

    @property
    def shape(self):
        return (self.dims[2], self.dims[1], self.dims[0])

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mvr_decon_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != OK:
            raise MvrError(rc, self._lib.mvr_decon_last_error(self._h).decode())

    def set_view(self, view, img, weight, psf):
        img, w, k = _f32(img), _f32(weight), _f32(psf)
        if img.shape != self.shape or w.shape != self.shape:
            raise ValueError("image/weight must have the volume shape")
        self._check(self._lib.mvr_decon_set_view(self._h, view, _p(img), _p(w), _p(k), _size_xyz(k)))

    def set_view_device(self, view, img_ptr: int, weight_ptr: int, psf):
        k = _f32(psf)
        self._check(self._lib.mvr_decon_set_view_device(self._h, view, C.c_void_p(img_ptr), C.c_void_p(weight_ptr),
                                                        _p(k), _size_xyz(k)))

    def set_schedule(self, code: int):
        """Forces an FFT schedule (SCHED_* code) for every view, -1 = autotuned; before prepare()."""
        self._check(self._lib.mvr_decon_set_schedule(self._h, int(code)))

    def schedule(self, view: int = 0) -> int:
        c = self._lib.mvr_decon_schedule(self._h, view)
        if c < 0:
            raise MvrError(-c, "schedule: view out of range")
        return c

    def tuning(self):
        """The autotuner's trials: dicts {step, code, schedule, batch, ms} (step and code -1
        for a blocks-per-launch trial)."""
        n = self._lib.mvr_decon_tuning(self._h, 0, None, None, None, None)
        st, cd, bt = (np.zeros(max(n, 1), np.int32) for _ in range(3))
        ms = np.zeros(max(n, 1), np.float32)
        self._lib.mvr_decon_tuning(self._h, n, _p(st), _p(cd), _p(bt), _p(ms))
        return [{"step": int(st[i]), "code": int(cd[i]), "schedule": schedule_name(int(cd[i])),
                 "batch": int(bt[i]), "ms": float(ms[i])} for i in range(n)]

    def set_view_block_size(self, view, block_size):
        """Compute block size (x, y, z) of one view (None: the handle's), before prepare()."""
        self._check(self._lib.mvr_decon_set_view_block_size(self._h, view,
                                                            (C.c_int * 3)(*block_size) if block_size else None))

    def set_effective_block_size(self, view, effective):
        """Effective block size (x, y, z) of one view (view -1: every view; None: block - 2 (k - 1)),
        before prepare(): the compute block then carries block - effective of overlap."""
        self._check(self._lib.mvr_decon_set_effective_block_size(self._h, view,
                                                                (C.c_int * 3)(*effective) if effective else None))

    def update_images(self, view, img, weight):
        img, w = _f32(img), _f32(weight)
        self._check(self._lib.mvr_decon_update_images(self._h, view, _p(img), _p(w)))

    def prepare(self):
        self._check(self._lib.mvr_decon_prepare(self._h))

    def set_psi(self, psi):
        psi = _f32(psi)
        self._check(self._lib.mvr_decon_set_psi(self._h, _p(psi)))

    def set_psi_device(self, ptr: int):
        self._check(self._lib.mvr_decon_set_psi_device(self._h, C.c_void_p(ptr)))

    def get_psi(self, out=None):
        if out is None:
            out = np.empty(self.shape, dtype=np.float32)
        self._check(self._lib.mvr_decon_get_psi(self._h, _p(out)))
        return out

    def get_psi_device(self, ptr: int):
        """Copies psi (float) into the device buffer at ptr."""
        self._check(self._lib.mvr_decon_get_psi_device(self._h, C.c_void_p(ptr)))

    def run_host(self, n: int, imgs, weights, psi, next_imgs=None, next_weights=None):
        """mvr_decon_run_host: uploads the host images, raw weights and psi (float32 [z][y][x],
        C-contiguous), runs n iterations and writes psi back in place.  With next_imgs /
        next_weights (mvr_decon_run_host_next) the next call's images and weights upload during
        these iterations; they must be C-contiguous float32 arrays of the volume shape and stay
        unchanged until the next call returns (the handle keeps references to them)."""
        arrs = [_f32(a) for a in list(imgs) + list(weights)]
        if any(a.shape != self.shape for a in arrs) or psi.dtype != np.float32 or psi.shape != self.shape \
                or not psi.flags.c_contiguous:
            raise ValueError("volumes must be C-contiguous float32 of the volume shape")
        nv = self.num_views
        ip = (C.c_void_p * nv)(*[a.ctypes.data for a in arrs[:nv]])
        wp = (C.c_void_p * nv)(*[a.ctypes.data for a in arrs[nv:]])
        if next_imgs is None and next_weights is None:
            self._check(self._lib.mvr_decon_run_host(self._h, int(n), ip, wp, _p(psi)))
            self._next_keep = None
            return psi
        nxt = list(next_imgs) + list(next_weights)
        if len(nxt) != 2 * nv or any(not isinstance(a, np.ndarray) or a.dtype != np.float32 or a.shape != self.shape
                                     or not a.flags.c_contiguous for a in nxt):
            raise ValueError("next images and weights: one C-contiguous float32 volume per view each")
        nip = (C.c_void_p * nv)(*[a.ctypes.data for a in nxt[:nv]])
        nwp = (C.c_void_p * nv)(*[a.ctypes.data for a in nxt[nv:]])
        self._check(self._lib.mvr_decon_run_host_next(self._h, int(n), ip, wp, _p(psi), nip, nwp))
        self._next_keep = nxt  # read by the copies in flight until the next call returns
        return psi

    def run_iterations(self, n: int, stats: bool = False):
        """runIterations; returns per (iteration, view-step) [sumChange, maxChange] if asked."""
        steps = 1 if self.mul else self.num_views
        st = np.zeros((n * steps, 2), dtype=np.float64) if stats else None
        self._check(self._lib.mvr_decon_run(self._h, n, _p(st) if stats else None))
        return st

    def kernels(self, view, shape):
        k1 = np.empty(shape, dtype=np.float32)
        k2 = np.empty(shape, dtype=np.float32)
        self._check(self._lib.mvr_decon_get_kernels(self._h, view, _p(k1), _p(k2)))
        return k1, k2

    def max_intensities(self):
        m = np.zeros(self.num_views, dtype=np.float32)
        self._check(self._lib.mvr_decon_get_max(self._h, _p(m)))
        return m

    def weights(self, view):
        w = np.empty(self.shape, dtype=np.float32)
        self._check(self._lib.mvr_decon_get_weights(self._h, view, _p(w)))
        return w

    def psi_device_ptr(self) -> int:
        return int(self._lib.mvr_decon_psi_device(self._h) or 0)

    def synchronize(self):
        self._check(self._lib.mvr_decon_synchronize(self._h))

    def stream_ptr(self) -> int:
        """cudaStream_t of the handle (for torch.cuda.ExternalStream / events)."""
        return int(self._lib.mvr_decon_stream(self._h) or 0)

    def likelihood(self):
        """Poisson NLL of the current psi: (total, per-view array), FP64 sums."""
        tot = np.zeros(1, np.float64)
        pv = np.zeros(self.num_views, np.float64)
        self._check(self._lib.mvr_decon_likelihood(self._h, _p(tot), _p(pv)))
        return float(tot[0]), pv

    def batch(self) -> int:
        """Blocks per batched launch in use."""
        return int(self._lib.mvr_decon_batch(self._h))

    def init_psi(self, method=PSI_INIT_BLURRED_FUSED, sigma: float = 5.0) -> float:
        """PsiInit on the device (PsiInitAvgPrecise / PsiInitAvgApprox / PsiInitBlurredFused);
        returns the average intensity (PsiInit.getAvg)."""
        avg = np.zeros(1, np.float64)
        self._check(self._lib.mvr_decon_init_psi(self._h, int(method), float(sigma), _p(avg)))
        return float(avg[0])

    def set_graphs(self, on: bool):
        """Whole iterations as CUDA graphs (default on); off launches eagerly."""
        self._check(self._lib.mvr_decon_set_graphs(self._h, int(on)))

    def graphs_captured(self) -> int:
        return int(self._lib.mvr_decon_graphs_captured(self._h))

    def launch_count(self) -> int:
        return int(self._lib.mvr_decon_launch_count(self._h))

    def set_profiling(self, on: bool):
        self._check(self._lib.mvr_decon_set_profiling(self._h, int(on)))

    def profile(self):
        """{kernel family: (ms, launches, algorithmic bytes)} accumulated while profiling."""
        n = KERNEL_KINDS
        ms = np.zeros(n, np.float64)
        la = np.zeros(n, np.int64)
        by = np.zeros(n, np.float64)
        self._check(self._lib.mvr_decon_get_profile(self._h, _p(ms), _p(la), _p(by)))
        return {self._lib.mvr_kernel_name(k).decode(): (float(ms[k]), int(la[k]), float(by[k])) for k in range(n)}


class UNet:
    """The learned-proposal network (3-level 3D U-Net, tcgen05 BF16 kernels) on device
    volumes given as raw addresses of float32 [batch][z][y][x] tensors."""

    def __init__(self, batch, dims, seed=0, device=0):
        self._lib = load()
        h = C.c_void_p()
        rc = self._lib.mvr_unet_create(batch, (C.c_int * 3)(*dims), seed, device, C.byref(h))
        if rc != OK:
            raise MvrError(rc, self._lib.mvr_unet_last_error(None).decode())
        self._h = h
        self.batch = batch
        self.dims = tuple(dims)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mvr_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc != OK:
            raise MvrError(rc, self._lib.mvr_unet_last_error(self._h).decode())

    @property
    def num_params(self) -> int:
        return int(self._lib.mvr_unet_num_params(self._h))

    def params(self):
        p = np.empty(self.num_params, np.float32)
        self._check(self._lib.mvr_unet_get_params(self._h, _p(p)))
        return p

    def set_params(self, p):
        p = _f32(p)
        self._check(self._lib.mvr_unet_set_params(self._h, _p(p)))

    def grads(self):
        g = np.empty(self.num_params, np.float32)
        self._check(self._lib.mvr_unet_get_grads(self._h, _p(g)))
        return g

    def set_input(self, psi_ptr: int, next_ptr: int = 0, target_ptr: int = 0):
        """psi_k, psi_{k+1} (network input) and psi_{k+m} (training target) device volumes."""
        self._check(self._lib.mvr_unet_set_input(self._h, C.c_void_p(psi_ptr), C.c_void_p(next_ptr) if next_ptr else None,
                                                 C.c_void_p(target_ptr) if target_ptr else None))

    def forward(self, pred_ptr: int = 0):
        self._check(self._lib.mvr_unet_forward(self._h, C.c_void_p(pred_ptr) if pred_ptr else None))

    def train_step(self, lr: float) -> float:
        loss = np.zeros(1, np.float64)
        self._check(self._lib.mvr_unet_train_step(self._h, lr, _p(loss)))
        return float(loss[0])

    def propose(self, psi_ptr: int, out_ptr: int, cap: float = 1.0):
        self._check(self._lib.mvr_unet_propose(self._h, C.c_void_p(psi_ptr), C.c_void_p(out_ptr), cap))


def pool2(in_ptr: int, dims, out_ptr: int, stream: int = 0):
    """mvr_pool2: 2 x 2 x 2 average of a device float volume of even dims (x, y, z)."""
    rc = load().mvr_pool2(C.c_void_p(in_ptr), (C.c_int * 3)(*dims), C.c_void_p(out_ptr), _sp(stream))
    if rc != OK:
        raise MvrError(rc, "mvr_pool2")


def apply_coarse(psi_next_ptr: int, dims, pred_low_ptr: int, psi_low_ptr: int, next_low_ptr: int, cap: float,
                 out_ptr: int, stream: int = 0):
    """mvr_apply_coarse: the coarse prediction applied to the full-resolution plain step."""
    rc = load().mvr_apply_coarse(C.c_void_p(psi_next_ptr), (C.c_int * 3)(*dims), C.c_void_p(pred_low_ptr),
                                 C.c_void_p(psi_low_ptr), C.c_void_p(next_low_ptr), float(cap), C.c_void_p(out_ptr),
                                 _sp(stream))
    if rc != OK:
        raise MvrError(rc, "mvr_apply_coarse")


def conv3d_tc(act_ptr, c_act, w_ptr, n_out, bias_ptr, relu, transposed, out_ptr, dims_xyzb, err_ptr, stream=0):
    """One tensor-core 3x3x3 convolution layer (forward or data gradient) on device buffers."""
    L = load()
    rc = L.mvr_conv3d_tc(C.c_void_p(act_ptr), c_act, C.c_void_p(w_ptr), n_out,
                         C.c_void_p(bias_ptr) if bias_ptr else None, int(relu), int(transposed), C.c_void_p(out_ptr),
                         (C.c_int * 4)(*dims_xyzb), C.c_void_p(err_ptr), C.c_void_p(stream) if stream else None)
    if rc != OK:
        raise MvrError(rc, L.mvr_conv3d_tc_last_error().decode())


def conv3d_tc_wgrad(x_ptr, c_in, g_ptr, c_out, dw_ptr, dims_xyzb, err_ptr, stream=0):
    L = load()
    rc = L.mvr_conv3d_tc_wgrad(C.c_void_p(x_ptr), c_in, C.c_void_p(g_ptr), c_out, C.c_void_p(dw_ptr),
                               (C.c_int * 4)(*dims_xyzb), C.c_void_p(err_ptr), C.c_void_p(stream) if stream else None)
    if rc != OK:
        raise MvrError(rc, L.mvr_conv3d_tc_last_error().decode())


def convolution3d_fft_cuda_in_place(im, kernel, device: int = 0) -> np.ndarray:
    """The reference's JNA call CUDAFourierConvolution.convolution3DfftCUDAInPlace with
    reversed dims; returns the convolved copy of ``im``."""
    L = load()
    a = np.array(im, dtype=np.float32, order="C")
    k = _f32(kernel)
    imdim = (C.c_int * 3)(*a.shape)  # reversed: {z, y, x}
    kdim = (C.c_int * 3)(*k.shape)
    L.convolution3DfftCUDAInPlace(_p(a), imdim, _p(k), kdim, device)
    return a


def convolve_static(img_ptr: int, img_size, kernel_ptr: int, kernel_size, out_ptr: int, stream: int = 0):
    """mvr_convolve_static on device buffers (raw addresses, sizes (x, y, z)); queued on
    `stream` without waiting.  Raises MvrError with the library's message on failure."""
    L = load()
    err = C.create_string_buffer(256)
    rc = L.mvr_convolve_static(C.c_void_p(img_ptr), (C.c_int * 3)(*img_size), C.c_void_p(kernel_ptr),
                               (C.c_int * 3)(*kernel_size), C.c_void_p(out_ptr), C.c_void_p(stream) if stream else None,
                               err, len(err))
    if rc != OK:
        raise MvrError(rc, err.value.decode())


def export_tiff(path, volume, calibration=(1.0, 1.0, 1.0), unit="px", dims=None):
    """mvr_export_tiff (Save3dTIFF): volume a float32 [z][y][x] host array, or a device address
    with dims (x, y, z)."""
    L = load()
    err = C.create_string_buffer(256)
    if isinstance(volume, np.ndarray):
        v = _f32(volume)
        ptr, on_dev, d = _p(v), 0, (v.shape[2], v.shape[1], v.shape[0])
    else:
        ptr, on_dev, d = C.c_void_p(volume), 1, dims
    rc = L.mvr_export_tiff(str(path).encode(), ptr, (C.c_longlong * 3)(*d), on_dev, (C.c_double * 3)(*calibration),
                           unit.encode(), err, len(err))
    if rc != OK:
        raise MvrError(rc, err.value.decode())


def export_n5(root, dataset, volume, block_size=(64, 64, 64), dims=None):
    """mvr_export_n5 (ExportN5Api, N5, raw blocks): volume a float32 [z][y][x] host array, or a
    device address with dims (x, y, z)."""
    L = load()
    err = C.create_string_buffer(256)
    if isinstance(volume, np.ndarray):
        v = _f32(volume)
        ptr, on_dev, d = _p(v), 0, (v.shape[2], v.shape[1], v.shape[0])
    else:
        ptr, on_dev, d = C.c_void_p(volume), 1, dims
    rc = L.mvr_export_n5(str(root).encode(), dataset.encode(), ptr, (C.c_longlong * 3)(*d), on_dev,
                         (C.c_int * 3)(*block_size), err, len(err))
    if rc != OK:
        raise MvrError(rc, err.value.decode())


def device_info(device: int = 0) -> dict:
    L = load()
    name = C.create_string_buffer(256)
    L.getNameDeviceCUDA(device, name)
    return dict(count=L.getNumDevicesCUDA(), name=name.value.decode(), mem=L.getMemDeviceCUDA(device),
                free=L.getFreeMemDeviceCUDA(device), major=L.getCUDAcomputeCapabilityMajorVersion(device),
                minor=L.getCUDAcomputeCapabilityMinorVersion(device))


class _FuseView(C.Structure):
    _fields_ = [("img", C.c_void_p), ("dims", C.c_int * 3), ("model", C.c_double * 12), ("fusion_blend", C.c_int),
                ("fusion_border", C.c_float * 3), ("fusion_range", C.c_float * 3), ("decon_blend", C.c_int),
                ("decon_border", C.c_float * 3), ("decon_range", C.c_float * 3), ("intensity_adjust", C.c_int),
                ("intensity", C.c_double * 2)]


def fuse_group(views, bb_min, bb_dims, image_out_ptr: int, weight_out_ptr: int, device: int = 0, stream: int = 0):
    """ProcessInputImages.fuseGroups for one group on the device.  views: dicts with
    'img_ptr' (device float volume), 'dims' (x, y, z), 'model' (3 x 4 view -> world) and
    optional 'fusion' / 'decon' blendings as (border xyz, range xyz).  Writes the fused image
    and the summed deconvolution weight of the bounding box (device float volumes).  An optional
    'intensity' = (m00, m01) applies the view's intensity adjustment v m00 + m01."""
    L = load()
    arr = (_FuseView * len(views))()
    for k, v in enumerate(views):
        a = arr[k]
        a.img = v["img_ptr"]
        a.dims = (C.c_int * 3)(*v["dims"])
        a.model = (C.c_double * 12)(*np.asarray(v["model"], dtype=np.float64).reshape(12))
        for key, flag, border, rng in (("fusion", "fusion_blend", "fusion_border", "fusion_range"),
                                       ("decon", "decon_blend", "decon_border", "decon_range")):
            b = v.get(key)
            setattr(a, flag, 0 if b is None else 1)
            if b is not None:
                setattr(a, border, (C.c_float * 3)(*b[0]))
                setattr(a, rng, (C.c_float * 3)(*b[1]))
        if v.get("intensity") is not None:
            a.intensity_adjust = 1
            a.intensity = (C.c_double * 2)(*v["intensity"])
    rc = L.mvr_fuse_group(C.cast(arr, C.c_void_p), len(views), (C.c_longlong * 3)(*bb_min), (C.c_int * 3)(*bb_dims),
                          C.c_void_p(image_out_ptr), C.c_void_p(weight_out_ptr), device,
                          C.c_void_p(stream) if stream else None)
    if rc != OK:
        raise MvrError(rc, L.mvr_fuse_last_error().decode())


# ---- PSF preparation (MV/process/psf, deconvolution/util/PSFPreparation.java) -----------
# Pointer arguments are device float volumes [z][y][x]; sizes are (x, y, z).

def _psf_check(rc):
    if rc != OK:
        raise MvrError(rc, load().mvr_psf_last_error().decode())


def _sp(stream):
    return C.c_void_p(stream) if stream else None


def psf_extract(img_ptr: int, img_dims, locations, psf_dims, psf_out_ptr: int, device: int = 0, stream: int = 0):
    """PSFExtraction.extractPSFLocal on the periodic image: the sum over the locations
    (n x 3 array of x, y, z) of the linearly interpolated neighbourhoods of size psf_dims."""
    loc = np.ascontiguousarray(np.asarray(locations, dtype=np.float64).reshape(-1, 3))
    _psf_check(load().mvr_psf_extract(C.c_void_p(img_ptr), (C.c_longlong * 3)(*img_dims), _p(loc) if len(loc) else None,
                                      len(loc), (C.c_int * 3)(*psf_dims), C.c_void_p(psf_out_ptr), device,
                                      _sp(stream)))


def psf_transformed_dims(dims, model):
    """Size (x, y, z) of PSFExtraction.transformPSF's output for the 3 x 4 model."""
    out = (C.c_int * 3)()
    m = np.ascontiguousarray(np.asarray(model, dtype=np.float64).reshape(12))
    _psf_check(load().mvr_psf_transformed_dims((C.c_int * 3)(*dims), _p(m), out))
    return tuple(out)


def psf_transform_normalized(psf_ptr: int, dims, model, out_ptr: int, out_dims, device: int = 0, stream: int = 0):
    """PSFExtraction.getTransformedNormalizedPSF (the input PSF is left unchanged)."""
    m = np.ascontiguousarray(np.asarray(model, dtype=np.float64).reshape(12))
    _psf_check(load().mvr_psf_transform_normalized(C.c_void_p(psf_ptr), (C.c_int * 3)(*dims), _p(m),
                                                   C.c_void_p(out_ptr), (C.c_int * 3)(*out_dims), device,
                                                   _sp(stream)))


def psf_average_dims(dims_list, max_size: bool):
    f = max if max_size else min
    return tuple(f(int(d[k]) for d in dims_list) for k in range(3))


def psf_average(psf_ptrs, dims_list, max_size: bool, out_ptr: int, device: int = 0, stream: int = 0):
    """PSFCombination.computeAverageImage; returns the output size (x, y, z)."""
    n = len(psf_ptrs)
    ptrs = (C.c_void_p * n)(*psf_ptrs)
    dims = (C.c_int * (3 * n))(*[int(v) for d in dims_list for v in d])
    out = (C.c_int * 3)()
    _psf_check(load().mvr_psf_average(C.cast(ptrs, C.c_void_p), C.cast(dims, C.c_void_p), n, 1 if max_size else 0,
                                      C.c_void_p(out_ptr), out, device, _sp(stream)))
    return tuple(out)


def psf_make_same_size(psf_ptr: int, dims, size, out_ptr: int, device: int = 0, stream: int = 0):
    """PSFCombination.makeSameSize."""
    _psf_check(load().mvr_psf_make_same_size(C.c_void_p(psf_ptr), (C.c_int * 3)(*dims), (C.c_int * 3)(*size),
                                             C.c_void_p(out_ptr), device, _sp(stream)))


def psf_projection(psf_ptr: int, dims, dim: int, use_max: bool, out_ptr: int, device: int = 0, stream: int = 0):
    """PSFCombination.computeProjection; returns the projected axis."""
    used = C.c_int(-1)
    _psf_check(load().mvr_psf_projection(C.c_void_p(psf_ptr), (C.c_int * 3)(*dims), dim, 1 if use_max else 0,
                                         C.c_void_p(out_ptr), C.byref(used), device, _sp(stream)))
    return used.value


def psf_remove_min_projections(psf_ptr: int, dims, device: int = 0, stream: int = 0):
    """PSFExtraction.removeMinProjections, in place."""
    _psf_check(load().mvr_psf_remove_min_projections(C.c_void_p(psf_ptr), (C.c_int * 3)(*dims), device, _sp(stream)))


def load_group_transform_psfs(groups, same_size_for_all: bool = True, device: int = 0):
    """PSFPreparation.loadGroupTransformPSFs (deconvolution/util/PSFPreparation.java:41-91) on
    the device.  groups: list of groups, each a list of (psf [z][y][x] float array, 3 x 4 model
    of its view, downsampling included).  Per group the views' normalised transformed PSFs
    are averaged on their smallest common size; with same_size_for_all every group's PSF
    is then centred in the largest size (extended with its minimum).  Returns float32
    arrays [z][y][x], one per group."""
    import torch

    dev = f"cuda:{device}"

    def vol(d):
        return torch.empty((d[2], d[1], d[0]), dtype=torch.float32, device=dev)

    out = []
    for grp in groups:
        tr, dims = [], []
        for psf, model in grp:
            p = torch.from_numpy(np.ascontiguousarray(psf, dtype=np.float32)).to(dev)
            pd = (p.shape[2], p.shape[1], p.shape[0])
            td = psf_transformed_dims(pd, model)
            t = vol(td)
            psf_transform_normalized(p.data_ptr(), pd, model, t.data_ptr(), td, device)
            tr.append(t)
            dims.append(td)
        ad = psf_average_dims(dims, False)
        avg = vol(ad)
        psf_average([t.data_ptr() for t in tr], dims, False, avg.data_ptr(), device)
        out.append(avg)
    if same_size_for_all:
        mx = tuple(max(a.shape[2 - k] for a in out) for k in range(3))
        res = []
        for a in out:
            d = (a.shape[2], a.shape[1], a.shape[0])
            r = vol(mx)
            psf_make_same_size(a.data_ptr(), d, mx, r.data_ptr(), device)
            res.append(r)
        out = res
    torch.cuda.synchronize(device)
    return [a.cpu().numpy() for a in out]


def block_grid(dims, kernel_size, block_size, min_required: int = 1):
    """BlockGeneratorFixedSizePrecise.divideIntoBlocks + BlockSorter's slab dimension (host):
    returns (blocks as dicts with offset / eff_offset / eff_size / eff_local, each (x, y, z),
    slab dimension)."""
    L = load()
    d = (C.c_longlong * 3)(*dims)
    k = (C.c_int * 3)(*kernel_size)
    b = (C.c_int * 3)(*block_size)
    n = L.mvr_block_grid(d, k, b, min_required, None, 0, None)
    if n < 0:
        raise MvrError(-n, "mvr_block_grid: bad sizes or a block smaller than the doubled kernel")
    out = np.zeros((max(n, 1), 12), dtype=np.int64)
    sd = C.c_int(-1)
    L.mvr_block_grid(d, k, b, min_required, _p(out), n, C.byref(sd))
    return [dict(offset=tuple(int(v) for v in r[0:3]), eff_offset=tuple(int(v) for v in r[3:6]),
                 eff_size=tuple(int(v) for v in r[6:9]), eff_local=tuple(int(v) for v in r[9:12]))
            for r in out[:n]], sd.value

