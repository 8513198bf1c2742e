// Input preparation on the device: the views of one group transformed into the
// deconvolution bounding box and fused, with the fusion and deconvolution blending weights
// (ProcessInputImages.fuseGroups, deconvolution/util/ProcessInputImages.java:279-399).
//
// Per output voxel p of the bounding box (world coordinate s = p + bb_min) and view v:
//   t = model_v^-1 s                                  (double, AffineTransform3D.applyInverse)
//   image  I_v = max(1, linear interpolation of the view at t) when t lies strictly inside
//                the view (min < t < max on every axis), else 0
//                (TransformView.transformView with minValueImg 1 / outsideValueImg 0,
//                 TransformedInputRandomAccess.get, AbstractTransformedImgRandomAccess)
//   weights wf_v, wd_v = the cosine blending of the view's interval at t (as float) with the
//                fusion / deconvolution border and range, or 1 without blending
//                (TransformWeight.transformBlending, TransformedRasteredRandomAccess.applyInverse,
//                 BlendingRealRandomAccess.computeWeight)
//   fused image = sum(I_v wf_v) / sum(wf_v) over wf_v != 0, 0 when the sum is 0
//                (FusedRandomAccess.get, Fusion.AVG)
//   deconvolution weight = sum(wd_v) (CombineWeightsSumRandomAccess.get)
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/mvr_gb300.h"
#include "affine.cuh"

namespace mvr {
namespace {

constexpr int kFuseMaxViews = 16;

struct FuseView {
    const float *img;
    int dims[3];
    double inv[12];  // world -> view pixel, row-packed 3 x 4
    float fb[3], fr[3], db[3], dr[3];
    int fblend, dblend;
    int adjust;        // intensity adjustment v -> v m00 + m01 (double, stored as float)
    double m00, m01;
};

struct FuseViews {
    FuseView v[kFuseMaxViews];
    int n;
};

// BlendingRealRandomAccess.computeWeight on an interval [0, dims - 1] at a float location
// (float arithmetic as in the reference, the look-up table product in double).
__device__ __forceinline__ float blend_weight(const float *loc, const int *dims, const float *border,
                                              const float *range, const double *lut)
{
    float tmp[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float l = loc[d];
        const float a = __fsub_rn(l, border[d]);
        const float b = __fsub_rn(__fsub_rn((float)(dims[d] - 1), l), border[d]);
        tmp[d] = a < b ? a : b;
        if (tmp[d] <= 0.0f) return 0.0f;
    }
    float w = 1.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        const float rel = __fdiv_rn(tmp[d], range[d]);
        if (rel < 1.0f) w = (float)((double)w * lut[(int)((double)rel * 1000.0 + 0.5)]);
    }
    return w;
}

// Linear interpolation of a float volume at t (all eight neighbours exist: t is strictly
// inside), the interpolator of the reference's views (NLinearInterpolator3D order); with
// `adjust` every neighbour goes through the intensity adjustment first
// (IntensityAdjuster.apply, fusion/intensityadjust/IntensityAdjuster.java: v m00 + m01 in
// double, stored as float).
__device__ __forceinline__ float trilinear(const FuseView &v, const double *t)
{
    const double f[3] = {floor(t[0]), floor(t[1]), floor(t[2])};
    const double w[3] = {__dsub_rn(t[0], f[0]), __dsub_rn(t[1], f[1]), __dsub_rn(t[2], f[2])};
    const long long sy = v.dims[0], sz = (long long)v.dims[0] * v.dims[1];
    const float *p = v.img + (long long)f[2] * sz + (long long)f[1] * sy + (long long)f[0];
    return nlinear3(w, [&](int dx, int dy, int dz) {
        const float x = __ldg(p + dz * sz + dy * sy + dx);
        return v.adjust ? __double2float_rn(__dadd_rn(__dmul_rn((double)x, v.m00), v.m01)) : x;
    });
}

__global__ void k_fuse_group(FuseViews fv, long long bx, long long by, long long bz, int nx, int ny, int nz,
                             float *__restrict__ out_img, float *__restrict__ out_w, const double *__restrict__ lut)
{
    const long long n = (long long)nx * ny * nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % nx);
        const int y = (int)((i / nx) % ny);
        const int z = (int)(i / ((long long)nx * ny));
        const double s0 = (double)(x + bx), s1 = (double)(y + by), s2 = (double)(z + bz);
        double sumI = 0.0, sumW = 0.0, sumD = 0.0;
        for (int k = 0; k < fv.n; ++k) {
            const FuseView &v = fv.v[k];
            const double sp[3] = {s0, s1, s2};
            double t[3];
            apply_affine(v.inv, sp, t);
            const float tf[3] = {(float)t[0], (float)t[1], (float)t[2]};
            const float wf = v.fblend ? blend_weight(tf, v.dims, v.fb, v.fr, lut) : 1.0f;
            const float wd = v.dblend ? blend_weight(tf, v.dims, v.db, v.dr, lut) : 1.0f;
            sumD += (double)wd;
            if (wf == 0.0f) continue;
            float val = 0.0f;  // outsideValueImg
            if (t[0] > 0.0 && t[1] > 0.0 && t[2] > 0.0 && t[0] < v.dims[0] - 1 && t[1] < v.dims[1] - 1 &&
                t[2] < v.dims[2] - 1)
                val = fmaxf(1.0f, trilinear(v, t));  // minValueImg
            sumI += (double)val * (double)wf;
            sumW += (double)wf;
        }
        out_img[i] = sumW > 0.0 ? (float)(sumI / sumW) : 0.0f;
        out_w[i] = (float)sumD;
    }
}

thread_local std::string g_fuse_err;

int fuse_fail(int code, const std::string &m)
{
    g_fuse_err = m;
    return code;
}

}  // namespace
}  // namespace mvr

using namespace mvr;

extern "C" MVR_API const char *mvr_fuse_last_error(void) { return g_fuse_err.c_str(); }

extern "C" MVR_API int mvr_fuse_group(const mvr_fuse_view *views, int num_views, const long long bb_min[3],
                                      const int bb_dims[3], float *image_out, float *weight_out, int device,
                                      void *stream)
{
    if (!views || num_views < 1 || num_views > kFuseMaxViews || !bb_min || !bb_dims || !image_out || !weight_out)
        return fuse_fail(MVR_ERR_ARG, "mvr_fuse_group: 1..16 views, bounding box and outputs are required");
    for (int d = 0; d < 3; ++d)
        if (bb_dims[d] < 1) return fuse_fail(MVR_ERR_ARG, "mvr_fuse_group: empty bounding box");
    FuseViews fv{};
    fv.n = num_views;
    for (int k = 0; k < num_views; ++k) {
        const mvr_fuse_view &s = views[k];
        FuseView &v = fv.v[k];
        if (!s.img) return fuse_fail(MVR_ERR_ARG, "mvr_fuse_group: a view image is NULL");
        for (int d = 0; d < 3; ++d) {
            if (s.dims[d] < 2) return fuse_fail(MVR_ERR_ARG, "mvr_fuse_group: view sizes must be >= 2");
            v.dims[d] = s.dims[d];
            v.fb[d] = s.fusion_border[d];
            v.fr[d] = s.fusion_range[d];
            v.db[d] = s.decon_border[d];
            v.dr[d] = s.decon_range[d];
        }
        v.fblend = s.fusion_blend;
        v.dblend = s.decon_blend;
        v.adjust = s.intensity_adjust ? 1 : 0;
        v.m00 = s.intensity[0];
        v.m01 = s.intensity[1];
        v.img = s.img;
        if (!invert_affine(s.model, v.inv)) return fuse_fail(MVR_ERR_ARG, "mvr_fuse_group: a view model is singular");
    }
    // the blending look-up table of BlendingRealRandomAccess: d runs from 0 in steps of 0.001
    // (accumulated in double, as there), entry (int)(d * 1000 + 0.5) = (cos((1 - d) pi) + 1) / 2
    std::vector<double> lut(1001, 0.0);
    for (double d = 0; d <= 1.0001; d = d + 0.001) lut[(int)(d * 1000.0 + 0.5)] = (std::cos((1 - d) * M_PI) + 1) / 2;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return fuse_fail(MVR_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double *dlut = nullptr;
    e = cudaMalloc(&dlut, sizeof(double) * lut.size());
    if (e != cudaSuccess) return fuse_fail(e == cudaErrorMemoryAllocation ? MVR_ERR_OOM : MVR_ERR_CUDA, cudaGetErrorString(e));
    e = cudaMemcpyAsync(dlut, lut.data(), sizeof(double) * lut.size(), cudaMemcpyHostToDevice, s);
    const long long n = (long long)bb_dims[0] * bb_dims[1] * bb_dims[2];
    if (e == cudaSuccess) {
        const int grid = (int)std::min<long long>((n + 255) / 256, 152LL * 16);
        k_fuse_group<<<grid, 256, 0, s>>>(fv, bb_min[0], bb_min[1], bb_min[2], bb_dims[0], bb_dims[1], bb_dims[2],
                                          image_out, weight_out, dlut);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dlut);
    if (e != cudaSuccess) return fuse_fail(MVR_ERR_CUDA, std::string("mvr_fuse_group: ") + cudaGetErrorString(e));
    return MVR_OK;
}
