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
