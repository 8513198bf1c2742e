/*
 * mvr_gb300.h -- C ABI of the GB300 multiview Bayesian (Richardson-Lucy type)
 * deconvolution block iteration.
 *
 * Drop-in boundary: the entry points replace the per-block plugin surface of
 * PreibischLab/multiview-reconstruction (paths relative to src/main/java/ of that
 * project, MV = net/preibisch/mvrecon/process):
 *
 *   ComputeBlockThreadFactory.create / numParallelBlocks
 *       MV/deconvolution/iteration/ComputeBlockThreadFactory.java:25-29
 *   ComputeBlockSeqThread.runIteration
 *       MV/deconvolution/iteration/sequential/ComputeBlockSeqThread.java:54-61
 *   ComputeBlockMulThread.runIteration / getNumViews
 *       MV/deconvolution/iteration/mul/ComputeBlockMulThread.java:40-62
 *   ComputeBlockThread.IterationStatistics
 *       MV/deconvolution/iteration/ComputeBlockThread.java:64-68
 *   DeconViewPSF.getKernel1FFT / getKernel2FFT (kernel spectra cached per view)
 *       MV/deconvolution/DeconViewPSF.java:79-111
 * and the native library bound through JNA by the reference's CUDA option
 *   CUDAFourierConvolution  MV/cuda/CUDAFourierConvolution.java:26-33
 *   CUDAStandardFunctions   MV/cuda/CUDAStandardFunctions.java:27-46
 *
 * Conventions: every volume / block is float32, x fastest ([z][y][x]); sizes are
 * given as {x, y, z}.  Functions return 0 (MVR_OK) or an MVR_ERR_* code; the
 * message of the last failure of a handle is mvr_block_last_error().  A handle is
 * used by one host thread at a time (the reference runs one ComputeBlockThread per
 * Java thread).  There is no CPU fallback: without a usable GB300 (sm_103a) the
 * create calls fail with MVR_ERR_CUDA.
 *
 * FP32 FFT domains with Px, Py in {128, 192} run on the plane kernels (x and y transforms
 * fused per z-plane); the environment variable MVR_PLANE_KERNELS=0, read when kernels are
 * set or a deconvolution is prepared, selects the row / column kernels instead (for
 * comparisons; results agree to float rounding).
 */
#ifndef MVR_GB300_H
#define MVR_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define MVR_API __attribute__((visibility("default")))
#else
#define MVR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define MVR_OK 0
#define MVR_ERR_ARG 1
#define MVR_ERR_CUDA 2
#define MVR_ERR_OOM 3
#define MVR_ERR_UNSUPPORTED 4
#define MVR_ERR_STATE 5

/* Boundary handling of the two convolutions of one block iteration.
 * MVR_BOUNDARY_REFERENCE: FFT domain >= block + kernel - 1 with the reference's
 *   extensions (mirror-single for psi, value 1 for the quotient), so the whole
 *   updated block and its statistics match ComputeBlockSeqThreadCPU
 *   (ComputeBlockSeqThreadCPU.java:171-209, util/FFTConvolution.java:508-603).
 * MVR_BOUNDARY_CIRCULAR: FFT domain == block (sizes with prime factors <= 13, x
 *   even).  The effective region a driver pastes is identical (the block overlap is
 *   2k-1, DeconView.java:155-157); the margin and the statistics differ. */
#define MVR_BOUNDARY_REFERENCE 0
#define MVR_BOUNDARY_CIRCULAR 1

typedef struct mvr_block_params {
    int block_size[3]; /* ComputeBlockThread.getBlockSize(), {x, y, z} */
    float min_value;   /* ComputeBlockThread.getMinValue(), reference default 1e-4 */
    float lambda;      /* Tikhonov lambda, 0 disables it (DeconvolutionMethods.java:336) */
    int num_views;     /* views of a multiplicative block (getNumViews), 1..16 */
    int boundary;      /* MVR_BOUNDARY_* */
    int device;        /* CUDA device ordinal */
} mvr_block_params;

typedef struct mvr_block mvr_block;

/* ComputeBlockThreadFactory.create(id): a block worker with its device buffers.
 * On failure *out is NULL and the return code says why. */
MVR_API int mvr_block_create(const mvr_block_params *params, mvr_block **out);
MVR_API void mvr_block_destroy(mvr_block *h);
/* Message of the last failed call on h (or of the last failed create when h is NULL). */
MVR_API const char *mvr_block_last_error(const mvr_block *h);

/* Uploads view `view`'s kernel1 / kernel2 (DeconViewPSF.getKernel1/getKernel2, same
 * size) and computes their spectra for this block size, as getKernel1FFT /
 * getKernel2FFT do once per (PSF, block size). */
MVR_API int mvr_block_set_kernels(mvr_block *h, int view, const float *kernel1, const float *kernel2,
                          const int kernel_size[3]);

/* ComputeBlockSeqThread.runIteration: one sequential iteration of view `view` on one
 * block.  psi_block (in/out, block_size voxels) is psiBlockTmp, updated in place;
 * img_block / weight_block are the zero-extended image and weight over the block.
 * stats[0] = sumChange, stats[1] = maxChange (IterationStatistics). */
MVR_API int mvr_block_run_seq(mvr_block *h, int view, float *psi_block, const float *img_block,
                      const float *weight_block, float max_intensity, double stats[2]);

/* ComputeBlockMulThread.runIteration: views 0..num_views-1 of one block, one
 * multiplicative update (ComputeBlockMulThreadCPU.java:87-188).  max_intensities has
 * num_views entries; their mean is used as in the reference. */
MVR_API int mvr_block_run_mul(mvr_block *h, float *psi_block, const float *const *img_blocks,
                      const float *const *weight_blocks, const float *max_intensities, double stats[2]);

/* Device-resident form of mvr_block_run_seq: all pointers are device pointers of
 * block_size voxels, work is queued on the handle's stream and the call returns
 * without synchronising (stats_device: 2 doubles, or NULL). */
MVR_API int mvr_block_run_seq_device(mvr_block *h, int view, float *psi_block, const float *img_block,
                             const float *weight_block, float max_intensity, double *stats_device);
/* Waits for the work queued on the handle's stream. */
MVR_API int mvr_block_synchronize(mvr_block *h);

/* ---- whole-volume deconvolution (device resident) ---------------------------------
 * MultiViewDeconvolutionSeq / MultiViewDeconvolutionMul with their set-up:
 *   MV/deconvolution/MultiViewDeconvolution.java:90-200 (constructor, runIterations)
 *   MV/deconvolution/MultiViewDeconvolutionSeq.java:57-180, MultiViewDeconvolutionMul.java:116-245
 *   MV/deconvolution/DeconView.java:118-184 (block grid with the doubled kernel 2k-1)
 *   MV/deconvolution/DeconViews.java:44-71 + DeconViewPSF.java:119-254 (PSF preparation)
 *   MV/deconvolution/normalization/NormalizingRandomAccess.java:76-109 (weights)
 *   MV/deconvolution/init/PsiInitAvgPrecise.java:52-110 (psi initialisation, max per view)
 * Images, weights and psi stay on the device between calls.  Sizes are {x, y, z}. */
#define MVR_PSF_OPTIMIZATION_II 0
#define MVR_PSF_OPTIMIZATION_I 1
#define MVR_PSF_EFFICIENT_BAYESIAN 2
#define MVR_PSF_INDEPENDENT 3

#define MVR_PRECISION_FP32 0
#define MVR_PRECISION_FP64 1

#define MVR_WEIGHTS_AS_GIVEN 0 /* weights are used as passed */
#define MVR_WEIGHTS_HARD 1     /* NormalizingRandomAccess hardWeights */
#define MVR_WEIGHTS_SMOOTH 2   /* NormalizingRandomAccess smoothWeights */

typedef struct mvr_decon_params {
    int dims[3];          /* volume size {x, y, z} */
    int num_views;        /* 1..16 */
    int block_size[3];    /* compute block size (DeconView blockSize) */
    int mul;              /* 0: sequential (OSEM-like), 1: multiplicative */
    int psf_type;         /* MVR_PSF_* (DeconViewPSF.PSFTYPE) */
    int psf_norm_threads; /* thread count T of AdjustInput.sumImg: the first of T portions is
                             counted twice in the PSF sum as in the reference; 0 = plain sum */
    float lambda;         /* Tikhonov lambda, 0 = off */
    float min_value;      /* psi floor, reference 1e-4 */
    int boundary;         /* MVR_BOUNDARY_* */
    int precision;        /* MVR_PRECISION_*: FP64 runs every stage in double */
    int filter_blocks;    /* drop blocks whose weight is all zero (DeconView.filterBlocksForContent) */
    int weight_norm;      /* MVR_WEIGHTS_* */
    float osem_speedup;   /* OSEM speed-up of the weight normalisation (1 = none) */
    float max_diff_range; /* smoothWeights parameters (reference 0.1, 0.05) */
    float scaling_range;
    int batch_blocks;     /* blocks per batched launch, 1..16; 0 = autotuned in mvr_decon_prepare */
    int device;           /* CUDA device ordinal */
} mvr_decon_params;

typedef struct mvr_decon mvr_decon;

MVR_API int mvr_decon_create(const mvr_decon_params *params, mvr_decon **out);
MVR_API void mvr_decon_destroy(mvr_decon *h);
MVR_API const char *mvr_decon_last_error(const mvr_decon *h);
/* DeconView(image, weight, psf): host arrays, copied to the device. */
MVR_API int mvr_decon_set_view(mvr_decon *h, int view, const float *img, const float *weight, const float *psf,
                               const int psf_size[3]);
/* The same with device-resident image and weight (borrowed, not copied; they must
 * outlive the handle). */
MVR_API int mvr_decon_set_view_device(mvr_decon *h, int view, const float *img, const float *weight,
                                      const float *psf, const int psf_size[3]);
/* The compute block size of one view ({x, y, z}; NULL restores the handle's block_size),
 * before mvr_decon_prepare.  DeconView takes its block size per view
 * (MV/deconvolution/DeconView.java:118-184): with per-view PSF sizes, a block of
 * E + 2 (k_v - 1) per axis gives every view effective blocks of E (the doubled kernel
 * 2 k_v - 1).  Multiplicative mode needs one grid: equal block sizes. */
MVR_API int mvr_decon_set_view_block_size(mvr_decon *h, int view, const int block_size[3]);
/* Effective block size of a view (view -1: every view; NULL: back to block - 2 (k - 1)).
 * No counterpart in the reference, whose effective block is always the block size minus
 * the doubled kernel (DeconView.java:155-157): here a view's compute block may carry more
 * overlap than its kernel needs, so that views with different PSF sizes split the volume on
 * one grid of effective blocks while their compute blocks take FFT shapes with plane
 * kernels.  block - effective + 1 must be at least 2k - 1 on every axis (checked at
 * prepare); the effective region of every block sees only voxels within its overlap, so
 * the result equals the reference's grid of the same effective size. */
MVR_API int mvr_decon_set_effective_block_size(mvr_decon *h, int view, const int effective[3]);
/* Replaces a view's image and raw weight (host) without redoing the PSF preparation. */
MVR_API int mvr_decon_update_images(mvr_decon *h, int view, const float *img, const float *weight);
/* DeconViews + DeconViewPSF.init, weight normalisation, block grids, PsiInitAvgPrecise. */
MVR_API int mvr_decon_prepare(mvr_decon *h);
/* PsiInitFromRAI: replace psi (host or device float volume). */
MVR_API int mvr_decon_set_psi(mvr_decon *h, const float *psi);
MVR_API int mvr_decon_set_psi_device(mvr_decon *h, const float *psi);
MVR_API int mvr_decon_get_psi(mvr_decon *h, float *psi);
/* Copy of psi as float into a device buffer of the volume's size (queued on the handle's
 * stream, then synchronised). */
MVR_API int mvr_decon_get_psi_device(mvr_decon *h, float *psi_device);
/* The block grid of one view (host arithmetic, no device work): BlockGeneratorFixedSizePrecise
 * .divideIntoBlocks (MV/cuda/BlockGeneratorFixedSizePrecise.java:59-131) for the doubled kernel
 * 2 kernel_size - 1 (DeconView.java:155-157), in x-fastest block order, and BlockSorter's slab
 * dimension for min_required blocks per slab (MV/cuda/BlockSorter.java:55-143).  blocks receives
 * up to `capacity` records of 12 values {offset[3], effective offset[3], effective size[3],
 * effective offset inside the block[3]} ({x, y, z} each).  Returns the number of blocks, or
 * -MVR_ERR_ARG (also when the block is smaller than the doubled kernel). */
MVR_API int mvr_block_grid(const long long dims[3], const int kernel_size[3], const int block_size[3],
                           int min_required, long long *blocks, int capacity, int *sort_dim);
/* runIterations: `iterations` more iterations.  stats (or NULL) receives per iteration
 * and view-step {sumChange, maxChange} (Seq: num_views steps, Mul: 1 step).  With stats NULL
 * the block voxels outside the regions written back to psi (which the reference computes
 * and discards) are not computed; psi is bit-identical either way. */
MVR_API int mvr_decon_run(mvr_decon *h, int iterations, double *stats);
/* runIterations with the inputs on the host (no reference counterpart as one call: the
 * reference driver holds images, weights and psi in host memory and copies blocks per call):
 * uploads every view's image and raw weight and psi (host arrays of the volume's size, views
 * set with mvr_decon_set_view), normalises the weights, runs `iterations` iterations and
 * writes psi back.  The uploads run on a copy stream, weights and psi first, then the images
 * in view order, and view-step v of the first iteration waits only for image v, so the image
 * uploads overlap the computation; page-locked host buffers keep the copies asynchronous. */
MVR_API int mvr_decon_run_host(mvr_decon *h, int iterations, const float *const *imgs, const float *const *weights,
                               float *psi);
/* mvr_decon_run_host that also starts uploading the NEXT call's images and raw weights
 * (next_images / next_weights, one host array per view) into a second set of device buffers
 * while this call's iterations run; a later call given those same host arrays as its images
 * and weights then uploads only psi before its first view-step (a time series of views, or
 * repeated steps on the same arrays).  The next arrays are read asynchronously until the next
 * call on the handle (or mvr_decon_synchronize) returns: keep them alive and unchanged until
 * then.  NULL next arrays: the same as mvr_decon_run_host.  No counterpart in the reference,
 * whose driver holds its images in host memory for the whole run
 * (MultiViewDeconvolution.java:144-200). */
MVR_API int mvr_decon_run_host_next(mvr_decon *h, int iterations, const float *const *images,
                                    const float *const *weights, float *psi, const float *const *next_images,
                                    const float *const *next_weights);
/* Prepared kernel1 / kernel2 of a view (DeconViewPSF.getKernel1/getKernel2). */
MVR_API int mvr_decon_get_kernels(mvr_decon *h, int view, float *kernel1, float *kernel2);
/* Maximum intensity per view (PsiInit.getMax). */
MVR_API int mvr_decon_get_max(mvr_decon *h, float *max_per_view);
/* Normalised weight of a view (host copy). */
MVR_API int mvr_decon_get_weights(mvr_decon *h, int view, float *weight);
/* Device address of psi (float for FP32, double for FP64), valid until the next run. */
MVR_API const void *mvr_decon_psi_device(const mvr_decon *h);
MVR_API int mvr_decon_synchronize(mvr_decon *h);
/* The cudaStream_t (as void *) all of the handle's work is queued on. */
MVR_API void *mvr_decon_stream(mvr_decon *h);
/* Number of kernel launches the handle has queued so far. */
MVR_API long long mvr_decon_launch_count(const mvr_decon *h);
/* Per-kernel-family timing with CUDA events on the handle's stream (off by default). */
#define MVR_KERNEL_KINDS 11
MVR_API int mvr_decon_set_profiling(mvr_decon *h, int on);
/* Accumulated {ms, launches, algorithmic bytes} per family (MVR_KERNEL_KINDS entries each);
 * synchronises the stream. */
MVR_API int mvr_decon_get_profile(mvr_decon *h, double *ms, long long *launches, double *bytes);
MVR_API const char *mvr_kernel_name(int kind);
/* Blocks per batched launch in use (chosen by the autotuner unless fixed). */
MVR_API int mvr_decon_batch(const mvr_decon *h);
/* Whole iterations of mvr_decon_run as CUDA graphs (on by default; the batched form of
 * the iteration loop MultiViewDeconvolution.runIterations, MultiViewDeconvolution.java:
 * 160-200).  An iteration in a new state (psi buffer, statistics slots, batch size,
 * scratch allocation, image/weight pointers) runs eagerly; the next one in that state is
 * captured and later ones replay it.  Results are identical to the eager launches.
 * on = 0 drops the graphs and launches eagerly.  While profiling is on, iterations run
 * eagerly. */
MVR_API int mvr_decon_set_graphs(mvr_decon *h, int on);
/* Number of captured iteration graphs held by the handle. */
MVR_API int mvr_decon_graphs_captured(const mvr_decon *h);
/* FFT schedules.  mvr_decon_prepare times, per view-step, every schedule the step's FFT
 * domain admits and keeps the fastest (then the blocks per launch, unless batch_blocks fixes
 * it); the batched, autotuned form of the iteration loop (no reference counterpart: the
 * reference's FFT has one fixed schedule).  Codes: MVR_SCHED_ROWS (row and column kernels),
 * MVR_SCHED_PLANE (x and y fused per z-plane, one CTA per plane), MVR_SCHED_PLANE_PERSIST
 * (the same with one CTA per SM walking the planes), MVR_SCHED_PAIR (a cluster of two CTAs per
 * plane, each holding half of its rows, exchanging the radix-2 stage of the y transform through
 * distributed shared memory: planes of 192 x 192 and 256 x 256), plus MVR_SCHED_ZPIPE when the Z pass
 * runs the persistent double-buffered column kernel.  Every schedule computes the same
 * iteration (results agree to float rounding).
 * mvr_decon_set_schedule (before prepare): force `code` for every view, -1 = autotune.
 * mvr_decon_schedule: the code in use for a view (negative on error).
 * mvr_decon_tuning: the autotuner's trials, up to `capacity` of them into the arrays (any may
 * be NULL): view-step (-1 for a batch trial), code (-1 for a batch trial), blocks per launch,
 * ms per view-step; returns the number of trials. */
#define MVR_SCHED_ROWS 0
#define MVR_SCHED_PLANE 1
#define MVR_SCHED_PLANE_PERSIST 2
#define MVR_SCHED_PAIR 3
#define MVR_SCHED_ZPIPE 4
MVR_API int mvr_decon_set_schedule(mvr_decon *h, int code);
MVR_API int mvr_decon_schedule(const mvr_decon *h, int view);
MVR_API int mvr_decon_tuning(const mvr_decon *h, int capacity, int *step, int *code, int *batch, float *ms);

/* PsiInit (MV/deconvolution/init/): re-initialise psi and the per-view maxima on the
 * device after mvr_decon_prepare (which runs MVR_PSI_INIT_AVG_PRECISE).
 *   MVR_PSI_INIT_AVG_PRECISE   PsiInitAvgPrecise.java:52-110
 *   MVR_PSI_INIT_AVG_APPROX    PsiInitAvgApprox.java:49-106, PsiInitAvgApproxThread.java:57-84
 *   MVR_PSI_INIT_BLURRED_FUSED PsiInitBlurredFused.java:66-127 (non-zero weighted fusion with
 *                              the normalised weights, then a Gaussian of `sigma` on every
 *                              axis, mirror-single extension; the reference default is 5)
 * avg (or NULL) receives the average intensity (PsiInit.getAvg). */
#define MVR_PSI_INIT_AVG_PRECISE 0
#define MVR_PSI_INIT_AVG_APPROX 1
#define MVR_PSI_INIT_BLURRED_FUSED 2
MVR_API int mvr_decon_init_psi(mvr_decon *h, int method, double sigma, double *avg);
/* Data-likelihood residual of the current psi (no reference counterpart; the reference
 * logs only the change statistics): the Poisson negative log-likelihood
 * sum_v sum_x w_v (conv1_v - img_v ln conv1_v) over img_v > 0, each voxel once, reduced
 * in FP64.  per_view (or NULL) receives num_views partial sums. */
MVR_API int mvr_decon_likelihood(mvr_decon *h, double *total, double *per_view);

/* ---- input preparation: transformed, fused views (device) ------------------------------
 * ProcessInputImages.fuseGroups (MV/deconvolution/util/ProcessInputImages.java:279-399) for
 * one group: every view is transformed into the bounding box with linear interpolation
 * (TransformView.transformView with minValueImg 1 inside and 0 outside the view,
 * TransformedInputRandomAccess.get), weighted by its cosine blending
 * (TransformWeight.transformBlending, BlendingRealRandomAccess.computeWeight) and averaged
 * (FusedRandomAccess, Fusion.AVG); the deconvolution weight is the sum of the views'
 * deconvolution blendings (CombineWeightsSumRandomAccess).  The result is the image and the
 * raw weight of one DeconView (mvr_decon_set_view_device). */
typedef struct mvr_fuse_view {
    const float *img;         /* device pointer: the view's image, x fastest */
    int dims[3];              /* its size {x, y, z} */
    double model[12];         /* view pixel -> world, row-packed 3 x 4 (AffineTransform3D.getRowPackedCopy) */
    int fusion_blend;         /* 0: fusion weight 1 (no blending), 1: blending with the two arrays below */
    float fusion_border[3];   /* pixels skipped at each face before blending (x, y, z) */
    float fusion_range[3];    /* pixels over which the weight rises from 0 to 1 */
    int decon_blend;          /* the same for the deconvolution weight */
    float decon_border[3];
    float decon_range[3];
    int intensity_adjust;     /* 1: every image value v becomes (float)(v m00 + m01) before the
                                 interpolation (IntensityAdjuster, intensity[] = {m00, m01}) */
    double intensity[2];
} mvr_fuse_view;
/* bb_min: world coordinate of the box's first voxel; bb_dims {x, y, z}; image_out and
 * weight_out: device float volumes of the box.  Synchronous on `stream`. */
MVR_API int mvr_fuse_group(const mvr_fuse_view *views, int num_views, const long long bb_min[3], const int bb_dims[3],
                           float *image_out, float *weight_out, int device, void *stream);
MVR_API const char *mvr_fuse_last_error(void);

/* ---- PSF preparation (MV/process/psf, deconvolution/util/PSFPreparation.java:41-91) ------
 * Device float volumes, x fastest, sizes {x, y, z}; synchronous on `stream`.
 *
 * mvr_psf_extract: PSFExtraction.extractPSFLocal (PSFExtraction.java:234-269) on the
 * periodic extension of the image (the RandomAccessibleInterval constructors, :112-120):
 * psf(p) = sum over the locations, in their order, of the linear interpolation of the image
 * at p - psf_dims / 2 + location.  locations: host array of num_locations {x, y, z} doubles
 * (0 locations: a zero PSF, hadDetections false). */
MVR_API int mvr_psf_extract(const float *img, const long long img_dims[3], const double *locations, int num_locations,
                            const int psf_dims[3], float *psf_out, int device, void *stream);
/* The size of PSFExtraction.transformPSF's output (:367-409): the bounding box of the
 * transformed PSF, (int) extent + 1, made odd.  model: row-packed 3 x 4. */
MVR_API int mvr_psf_transformed_dims(const int dims[3], const double model[12], int out_dims[3]);
/* PSFExtraction.getTransformedNormalizedPSF (:182-188): the PSF normalised to [0, 1]
 * (normalize, :453-471; the input is not modified) and transformed with the view's model,
 * its centre voxel dims / 2 kept at the output centre (transform, :411-451; linear
 * interpolation, zero outside).  out_dims must equal mvr_psf_transformed_dims. */
MVR_API int mvr_psf_transform_normalized(const float *psf, const int dims[3], const double model[12], float *out,
                                         const int out_dims[3], int device, void *stream);
/* PSFCombination.computeAverageImage (PSFCombination.java:74-138): the PSFs (1..64, dims
 * num_psfs x {x, y, z}) centred and averaged on the largest (max_size 1) or smallest
 * (max_size 0) size per axis, returned in out_dims; out holds that many voxels (at most the
 * largest size on every axis). */
MVR_API int mvr_psf_average(const float *const *psfs, const int *dims, int num_psfs, int max_size, float *out,
                            int out_dims[3], int device, void *stream);
/* PSFCombination.makeSameSize (:182-210): the PSF centred in `size`, extended with its minimum. */
MVR_API int mvr_psf_make_same_size(const float *psf, const int dims[3], const int size[3], float *out, int device,
                                   void *stream);
/* PSFCombination.computeMaxProjection (:228-296): max (use_max 1) or min projection along
 * axis dim (dim < 0: the smallest axis, returned in used_dim); the output keeps the other
 * two axes in order. */
MVR_API int mvr_psf_projection(const float *psf, const int dims[3], int dim, int use_max, float *out, int *used_dim,
                               int device, void *stream);
/* PSFExtraction.removeMinProjections (:190-229): for axis 0, 1, 2 in turn, subtract the min
 * projection along that axis (in place). */
MVR_API int mvr_psf_remove_min_projections(float *psf, const int dims[3], int device, void *stream);
MVR_API const char *mvr_psf_last_error(void);

/* ---- export of the deconvolved volume (Image_Deconvolution's ImgExport, MV/export) -----
 * volume: float32 [z][y][x] of dims {x, y, z}, in host memory (on_device 0) or device memory
 * (on_device 1, read back in slabs).  err (may be NULL) receives a message on failure.
 * mvr_export_tiff: Save3dTIFF (MV/export/Save3dTIFF.java:86-160): an ImageJ stack of 32-bit
 *   float slices (big-endian TIFF, one strip per slice, ImageJ description with the slice
 *   count, unit, z spacing and the display range 0..255 of DisplayImage), calibration {x, y,
 *   z} per pixel (NULL: 1) and unit (NULL: "px"); stacks beyond the 4 GB offsets of a TIFF
 *   file return MVR_ERR_UNSUPPORTED.
 * mvr_export_n5: ExportN5Api with the N5 format and no compression (MV/export/ExportN5Api.java):
 *   dataset `dataset` under the container directory `root`, float32, raw blocks of
 *   block_size {x, y, z} (clipped at the border), one file per grid position bx/by/bz. */
MVR_API int mvr_export_tiff(const char *path, const float *volume, const long long dims[3], int on_device,
                            const double calibration[3], const char *unit, char *err, int err_len);
MVR_API int mvr_export_n5(const char *root, const char *dataset, const float *volume, const long long dims[3],
                          int on_device, const int block_size[3], char *err, int err_len);

/* ---- learned multi-iteration proposal (no counterpart in the reference) ---------------
 * A 3-level 3D U-Net (16/32/64 channels, 3x3x3 convolutions, BF16 weights and
 * activations, FP32 accumulation on the tcgen05 tensor cores) with its own forward and
 * backward kernels and Adam, for patches [batch][z][y][x] of sizes {x, y, z} (multiples
 * of 4).  Inputs are device float volumes: psi_k and the plain method's next iterate
 * psi_{k+1} (the network sees the ratio psi_{k+1} / psi_k); it predicts
 * log(psi_{k+m} / psi_k).  Callers gate its proposals with mvr_decon_likelihood. */
typedef struct mvr_unet mvr_unet;
MVR_API int mvr_unet_create(int batch, const int dims[3], unsigned seed, int device, mvr_unet **out);
MVR_API void mvr_unet_destroy(mvr_unet *h);
MVR_API const char *mvr_unet_last_error(const mvr_unet *h);
MVR_API long long mvr_unet_num_params(const mvr_unet *h);
/* FP32 master parameters (host copies): per layer W[co][27][ci] then b[co], head w[16], b. */
MVR_API int mvr_unet_get_params(mvr_unet *h, float *params);
MVR_API int mvr_unet_set_params(mvr_unet *h, const float *params);
/* Gradients of the last training step (same layout as the parameters). */
MVR_API int mvr_unet_get_grads(mvr_unet *h, float *grads);
/* Features from psi_k and psi_{k+1} (device, may be NULL) and the target
 * log(psi_target / psi_k) (psi_target may be NULL for inference). */
MVR_API int mvr_unet_set_input(mvr_unet *h, const float *psi, const float *psi_next, const float *psi_target);
/* Forward pass; pred (device, or NULL) receives the predicted log-ratio. */
MVR_API int mvr_unet_forward(mvr_unet *h, float *pred);
/* Forward, mean-squared-error loss against the target, backward, one Adam step. */
MVR_API int mvr_unet_train_step(mvr_unet *h, float lr, double *loss);
/* Forward and psi_out = psi * exp(clamp(pred, -cap, cap)) (device volumes). */
MVR_API int mvr_unet_propose(mvr_unet *h, const float *psi, float *psi_out, float cap);
/* One 3x3x3 convolution layer on the tensor cores (device BF16 [B][z][y][x][C] volumes,
 * dims {x, y, z, B}): transposed == 0 is the forward pass (weights [n_out][27][c_act],
 * bias, ReLU, BF16 output), transposed == 1 the data gradient (weights transposed
 * [n_out][27][c_act], FP32 output).  err_dev: device int, set on a tensor-core timeout. */
MVR_API int mvr_conv3d_tc(const void *act, int c_act, const void *weights, int n_out, const float *bias, int relu,
                          int transposed, void *out, const int dims[4], int *err_dev, void *stream);
/* Weight gradient dw[c_out][27][c_in] += sum_n g[n][c_out] x[n + off][c_in] (FP32). */
MVR_API int mvr_conv3d_tc_wgrad(const void *x, int c_in, const void *g, int c_out, float *dw, const int dims[4],
                                int *err_dev, void *stream);
MVR_API const char *mvr_conv3d_tc_last_error(void);
/* The coarse form of the proposal: the network runs on the 2 x 2 x 2 averages of psi_k and
 * psi_{k+1} (mvr_pool2: device float volume of even dims {x, y, z} -> dims / 2, queued on
 * `stream`), and mvr_apply_coarse applies its prediction at full resolution:
 * out = psi_next * exp(clamp(up(pred_low - log(next_low / psi_low)), -cap, cap)), up = trilinear
 * interpolation of the coarse grid (cell centres), i.e. the plain step at full resolution
 * plus the predicted further change of the coarse scales. */
MVR_API int mvr_pool2(const float *in, const int dims[3], float *out, void *stream);
MVR_API int mvr_apply_coarse(const float *psi_next, const int dims[3], const float *pred_low, const float *psi_low,
                             const float *next_low, float cap, float *out, void *stream);

/* ---- convolution without device allocation ------------------------------------------
 * No counterpart in the reference: an addition for callers that cannot call
 * cudaMalloc -- code running inside another framework's CUDA context whose caching
 * allocator owns the device memory, or latency-critical paths that cannot take the
 * implicit device synchronisation of cudaMalloc / cudaFree.
 *
 * The same convolution as convolution3DfftCUDA (linear, zero extension, output over
 * the image; sizes here are {x, y, z}, not reversed), but every intermediate lives in
 * one fixed device array compiled into the library (16 MiB + 24 KiB, held by every
 * GPU that loads the library until the process exits).  img, kernel and out are
 * device pointers supplied by the caller; the work is queued on `stream` (a
 * cudaStream_t, NULL = legacy default stream) and the call does not wait for it.
 * Limits: the FFT domain (img + kernel - 1 per axis, rounded up to an even size with
 * prime factors <= 13) must be <= 1024 per axis and (x/2 + 1) * y * z <= 1048576;
 * larger sizes return MVR_ERR_UNSUPPORTED with the reason in err.
 * Every call resolves the array's device address in the calling thread's current
 * context (cudaGetSymbolAddress) and computes its twiddle tables on the device, so
 * nothing is cached across contexts or device resets and nothing is staged in host
 * memory.  The first call on a device also loads the library's module there; make
 * that first call before any stream capture.  All calls share the one
 * array and it keeps the last call's contents (every value is written before it is
 * read, nothing needs clearing); calls whose work overlaps on the GPU -- from
 * different streams or threads -- race on it.  It calls no cudaMalloc, cudaFree or
 * other allocating routine.  err (may be NULL) receives a message on failure. */
MVR_API int mvr_convolve_static(const float *img, const int img_size[3], const float *kernel,
                                const int kernel_size[3], float *out, void *stream, char *err, int err_len);

/* ---- the reference's JNA library (CUDAFourierConvolution / CUDAStandardFunctions) ----
 * Exported under the reference's own symbol names so that the unchanged
 * ComputeBlockSeqThreadCUDA can load this library.  Dimensions arrive reversed
 * ({z, y, x}, CUDATools.getCUDACoordinates, CUDATools.java:41-49).  The convolution
 * is linear with zero extension, output over the image. */
MVR_API float *convolution3DfftCUDA(float *im, int *imDim, float *kernel, int *kernelDim, int devCUDA);
MVR_API void convolution3DfftCUDAInPlace(float *im, int *imDim, float *kernel, int *kernelDim, int devCUDA);
MVR_API int getNumDevicesCUDA(void);
MVR_API void getNameDeviceCUDA(int devCUDA, char *name);
MVR_API long long getMemDeviceCUDA(int devCUDA);
MVR_API long long getFreeMemDeviceCUDA(int devCUDA);
MVR_API int getCUDAcomputeCapabilityMajorVersion(int devCUDA);
MVR_API int getCUDAcomputeCapabilityMinorVersion(int devCUDA);
/* Frees a result of convolution3DfftCUDA (the reference leaves this to JNA). */
MVR_API void mvr_free(void *p);

#ifdef __cplusplus
}
#endif

#endif /* MVR_GB300_H */
