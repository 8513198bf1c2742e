// PSF preparation on the device (MV/process/psf and the deconvolution's PSF loading,
// deconvolution/util/PSFPreparation.java:41-91):
//   mvr_psf_extract               PSFExtraction.extractPSFLocal (PSFExtraction.java:234-269) on the
//                                 periodic extension of the image (PSFExtraction.java:112-120)
//   mvr_psf_transformed_dims /    PSFExtraction.getTransformedNormalizedPSF (:182-188):
//   mvr_psf_transform_normalized  normalize (:453-471) then transformPSF / transform (:367-451)
//   mvr_psf_average               PSFCombination.computeAverageImage (PSFCombination.java:74-138)
//   mvr_psf_make_same_size        PSFCombination.makeSameSize (:182-210)
//   mvr_psf_projection            PSFCombination.computeProjection / computeMaxProjection (:212-296)
//   mvr_psf_remove_min_projections PSFExtraction.removeMinProjections / subtractProjection (:190-229)
// Volumes are float32 [z][y][x] (x fastest) in device memory; sizes are given as (x, y, z).
// The PSFs are small (a few 10^4 .. 10^6 voxels): one thread per output voxel, the bead
// locations of the extraction summed in their given order per voxel, as the reference does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/mvr_gb300.h"
#include "affine.cuh"

namespace mvr {
namespace {

thread_local std::string g_psf_err;

int psf_fail(int code, const std::string &m)
{
    g_psf_err = m;
    return code;
}

int psf_cuda(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return MVR_OK;
    return psf_fail(e == cudaErrorMemoryAllocation ? MVR_ERR_OOM : MVR_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
}

#define PSF_TRY(x)                  \
    do {                            \
        const int rc_ = (x);        \
        if (rc_ != MVR_OK) return rc_; \
    } while (0)

inline unsigned grid_of(long long n) { return (unsigned)std::max<long long>(1, (n + 255) / 256); }

__device__ __forceinline__ long long dwrap(long long i, long long n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

// extractPSFLocal: psf(p) = sum over the locations l, in order, of the linear interpolation of
// the periodic image at p - size / 2 + l; each sum step psf + value in double, stored as float.
__global__ void k_psf_extract(const float *__restrict__ img, long long D0, long long D1, long long D2,
                              const double *__restrict__ loc, int nloc, int s0, int s1, int s2,
                              float *__restrict__ psf)
{
    const long long n = (long long)s0 * s1 * s2;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % s0), y = (int)((i / s0) % s1), z = (int)(i / ((long long)s0 * s1));
    const double r0 = (double)(x - s0 / 2), r1 = (double)(y - s1 / 2), r2 = (double)(z - s2 / 2);
    float acc = 0.0f;
    for (int l = 0; l < nloc; ++l) {
        const double t0 = __dadd_rn(r0, __ldg(loc + 3 * l)), t1 = __dadd_rn(r1, __ldg(loc + 3 * l + 1)),
                     t2 = __dadd_rn(r2, __ldg(loc + 3 * l + 2));
        const double f0 = floor(t0), f1 = floor(t1), f2 = floor(t2);
        const double w[3] = {__dsub_rn(t0, f0), __dsub_rn(t1, f1), __dsub_rn(t2, f2)};
        const long long x0 = dwrap((long long)f0, D0), y0 = dwrap((long long)f1, D1), z0 = dwrap((long long)f2, D2);
        const long long xs[2] = {x0, x0 + 1 == D0 ? 0 : x0 + 1};
        const long long ys[2] = {y0 * D0, (y0 + 1 == D1 ? 0 : y0 + 1) * D0};
        const long long zs[2] = {z0 * D1 * D0, (z0 + 1 == D2 ? 0 : z0 + 1) * D1 * D0};
        const float v = nlinear3(w, [&](int dx, int dy, int dz) { return __ldg(img + zs[dz] + ys[dy] + xs[dx]); });
        acc = __double2float_rn(__dadd_rn((double)acc, (double)v));
    }
    psf[i] = acc;
}

// Minimum and maximum (double) of a small volume, one CTA; NaN values are skipped.
__global__ void k_psf_minmax(const float *__restrict__ a, long long n, double *out)
{
    __shared__ double smin[256], smax[256];
    double mn = DBL_MAX, mx = -DBL_MAX;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = (double)a[i];
        if (v < mn) mn = v;
        if (v > mx) mx = v;
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            if (smin[threadIdx.x + h] < smin[threadIdx.x]) smin[threadIdx.x] = smin[threadIdx.x + h];
            if (smax[threadIdx.x + h] > smax[threadIdx.x]) smax[threadIdx.x] = smax[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = smin[0];
        out[1] = smax[0];
    }
}

struct Affine {
    double m[12];
};

// transform() of the normalised PSF: out(p) = linear interpolation of the zero-extended
// normalised PSF at model^-1 (p + offset); normalize maps v to (v - min) / (max - min).
__global__ void k_psf_transform(const float *__restrict__ psf, int d0, int d1, int d2,
                                const double *__restrict__ minmax, Affine inv, double o0, double o1, double o2,
                                int n0, int n1, int n2, float *__restrict__ out)
{
    const long long n = (long long)n0 * n1 * n2;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % n0), y = (int)((i / n0) % n1), z = (int)(i / ((long long)n0 * n1));
    const double mn = minmax[0], rng = __dsub_rn(minmax[1], minmax[0]);
    const double s[3] = {__dadd_rn((double)x, o0), __dadd_rn((double)y, o1), __dadd_rn((double)z, o2)};
    double t[3];
    apply_affine(inv.m, s, t);
    const double f[3] = {floor(t[0]), floor(t[1]), floor(t[2])};
    const double w[3] = {__dsub_rn(t[0], f[0]), __dsub_rn(t[1], f[1]), __dsub_rn(t[2], f[2])};
    const long long bx = (long long)f[0], by = (long long)f[1], bz = (long long)f[2];
    out[i] = nlinear3(w, [&](int dx, int dy, int dz) {
        const long long xx = bx + dx, yy = by + dy, zz = bz + dz;
        if (xx < 0 || yy < 0 || zz < 0 || xx >= d0 || yy >= d1 || zz >= d2) return 0.0f;  // extendZero
        const double v = (double)__ldg(psf + (zz * d1 + yy) * d0 + xx);
        return __double2float_rn(__ddiv_rn(__dsub_rn(v, mn), rng));
    });
}

constexpr int kMaxPsfs = 64;
struct PsfList {
    const float *p[kMaxPsfs];
    int d[kMaxPsfs][3];
    int n;
};

// computeAverageImage: the PSFs centred on the average image (centre = size / 2), summed in
// float in list order, then divided by their number (double, stored as float).
__global__ void k_psf_average(PsfList L, int a0, int a1, int a2, float *__restrict__ out)
{
    const long long n = (long long)a0 * a1 * a2;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % a0), y = (int)((i / a0) % a1), z = (int)(i / ((long long)a0 * a1));
    float acc = 0.0f;
    for (int k = 0; k < L.n; ++k) {
        const int *d = L.d[k];
        const int px = x - a0 / 2 + d[0] / 2, py = y - a1 / 2 + d[1] / 2, pz = z - a2 / 2 + d[2] / 2;
        if (px < 0 || py < 0 || pz < 0 || px >= d[0] || py >= d[1] || pz >= d[2]) continue;
        acc = __fadd_rn(acc, __ldg(L.p[k] + ((long long)pz * d[1] + py) * d[0] + px));
    }
    out[i] = __double2float_rn(__ddiv_rn((double)acc, (double)L.n));
}

// makeSameSize: the image centred in the new size, extended with its minimum.
__global__ void k_psf_same_size(const float *__restrict__ img, int d0, int d1, int d2, const double *minmax, int n0,
                                int n1, int n2, float *__restrict__ out)
{
    const long long n = (long long)n0 * n1 * n2;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int x = (int)(i % n0), y = (int)((i / n0) % n1), z = (int)(i / ((long long)n0 * n1));
    const int px = x - n0 / 2 + d0 / 2, py = y - n1 / 2 + d1 / 2, pz = z - n2 / 2 + d2 / 2;
    out[i] = (px < 0 || py < 0 || pz < 0 || px >= d0 || py >= d1 || pz >= d2)
                 ? __double2float_rn(minmax[0])
                 : __ldg(img + ((long long)pz * d1 + py) * d0 + px);
}

// computeMaxProjection: the extreme (max or min, double, starting at -+DBL_MAX) along axis
// `dim`; the output keeps the other axes in order.
__global__ void k_psf_project(const float *__restrict__ a, int d0, int d1, int d2, int dim, int use_max,
                              float *__restrict__ out)
{
    const int dd[3] = {d0, d1, d2};
    const int q0 = dim == 0 ? 1 : 0, q1 = dim == 2 ? 1 : 2;  // the kept axes
    const long long n = (long long)dd[q0] * dd[q1];
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int c[3];
    c[q0] = (int)(i % dd[q0]);
    c[q1] = (int)(i / dd[q0]);
    const long long st[3] = {1, d0, (long long)d0 * d1};
    double ext = use_max ? -DBL_MAX : DBL_MAX;
    c[dim] = 0;
    const float *p = a + c[0] * st[0] + c[1] * st[1] + c[2] * st[2];
    for (int k = 0; k < dd[dim]; ++k) {
        const double v = (double)p[k * st[dim]];
        if (use_max ? v > ext : v < ext) ext = v;
    }
    out[i] = __double2float_rn(ext);
}

// subtractProjection: a(p) -= proj(p without axis dim), float.
__global__ void k_psf_subtract(float *__restrict__ a, int d0, int d1, int d2, int dim, const float *__restrict__ proj)
{
    const long long n = (long long)d0 * d1 * d2;
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c[3] = {(int)(i % d0), (int)((i / d0) % d1), (int)(i / ((long long)d0 * d1))};
    const int dd[3] = {d0, d1, d2};
    const int q0 = dim == 0 ? 1 : 0, q1 = dim == 2 ? 1 : 2;
    a[i] = __fsub_rn(a[i], proj[(long long)c[q1] * dd[q0] + c[q0]]);
}

bool dims_ok(const int *d)
{
    return d && d[0] >= 1 && d[1] >= 1 && d[2] >= 1 && (long long)d[0] * d[1] * d[2] < (1LL << 31);
}

// Device scratch of two doubles for the min / max reductions.
struct Scratch {
    double *p = nullptr;
    ~Scratch() { cudaFree(p); }
};

int setup(int device, Scratch *sc)
{
    PSF_TRY(psf_cuda(cudaSetDevice(device), "cudaSetDevice"));
    if (sc) PSF_TRY(psf_cuda(cudaMalloc(&sc->p, 2 * sizeof(double)), "cudaMalloc"));
    return MVR_OK;
}

int finish(cudaStream_t s, const char *what)
{
    PSF_TRY(psf_cuda(cudaGetLastError(), what));
    return psf_cuda(cudaStreamSynchronize(s), what);
}

// transformPSF's output size and offset: the bounding box of the transformed corners of
// [0, dims - 1] (AffineTransform3D.estimateBounds), size (int)(max - min) + 1 made odd, and
// the offset that maps the PSF centre dims / 2 onto the output centre size / 2.
bool transformed_geometry(const int *dims, const double *model, int *out, double *offset)
{
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (int c = 0; c < 8; ++c) {
        const double s[3] = {(c & 1) ? (double)(dims[0] - 1) : 0.0, (c & 2) ? (double)(dims[1] - 1) : 0.0,
                             (c & 4) ? (double)(dims[2] - 1) : 0.0};
        double t[3];
        apply_affine(model, s, t);
        for (int d = 0; d < 3; ++d) {
            lo[d] = std::min(lo[d], t[d]);
            hi[d] = std::max(hi[d], t[d]);
        }
    }
    const double center[3] = {(double)(dims[0] / 2), (double)(dims[1] / 2), (double)(dims[2] / 2)};
    double tc[3];
    apply_affine(model, center, tc);
    for (int d = 0; d < 3; ++d) {
        const double size = hi[d] - lo[d];
        if (!std::isfinite(size) || size < 0 || size > 1e7) return false;
        long long ns = (long long)(int)size + 1;
        if (ns % 2 == 0) ++ns;
        out[d] = (int)ns;
        offset[d] = tc[d] - (double)(ns / 2);
    }
    return true;
}

}  // namespace
}  // namespace mvr

using namespace mvr;

extern "C" MVR_API const char *mvr_psf_last_error(void) { return g_psf_err.c_str(); }

extern "C" MVR_API int mvr_psf_extract(const float *img, const long long img_dims[3], const double *locations,
                                       int num_locations, const int psf_dims[3], float *psf_out, int device,
                                       void *stream)
{
    if (!img || !img_dims || !psf_out || !dims_ok(psf_dims) || num_locations < 0 || (num_locations > 0 && !locations))
        return psf_fail(MVR_ERR_ARG, "mvr_psf_extract: image, PSF size (>= 1) and output are required");
    for (int d = 0; d < 3; ++d)
        if (img_dims[d] < 1) return psf_fail(MVR_ERR_ARG, "mvr_psf_extract: empty image");
    PSF_TRY(setup(device, nullptr));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    double *dloc = nullptr;
    if (num_locations > 0) {
        PSF_TRY(psf_cuda(cudaMalloc(&dloc, sizeof(double) * 3 * (size_t)num_locations), "cudaMalloc"));
        const cudaError_t e = cudaMemcpyAsync(dloc, locations, sizeof(double) * 3 * (size_t)num_locations,
                                              cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            cudaFree(dloc);
            return psf_cuda(e, "mvr_psf_extract");
        }
    }
    const long long n = (long long)psf_dims[0] * psf_dims[1] * psf_dims[2];
    k_psf_extract<<<grid_of(n), 256, 0, s>>>(img, img_dims[0], img_dims[1], img_dims[2], dloc, num_locations,
                                             psf_dims[0], psf_dims[1], psf_dims[2], psf_out);
    const int rc = finish(s, "mvr_psf_extract");
    cudaFree(dloc);
    return rc;
}

extern "C" MVR_API int mvr_psf_transformed_dims(const int dims[3], const double model[12], int out_dims[3])
{
    if (!dims_ok(dims) || !model || !out_dims) return psf_fail(MVR_ERR_ARG, "mvr_psf_transformed_dims: bad arguments");
    double off[3];
    if (!transformed_geometry(dims, model, out_dims, off))
        return psf_fail(MVR_ERR_ARG, "mvr_psf_transformed_dims: the model does not give a finite PSF size");
    return MVR_OK;
}

extern "C" MVR_API int mvr_psf_transform_normalized(const float *psf, const int dims[3], const double model[12],
                                                    float *out, const int out_dims[3], int device, void *stream)
{
    if (!psf || !dims_ok(dims) || !model || !out || !out_dims)
        return psf_fail(MVR_ERR_ARG, "mvr_psf_transform_normalized: bad arguments");
    int nd[3];
    double off[3];
    if (!transformed_geometry(dims, model, nd, off))
        return psf_fail(MVR_ERR_ARG, "mvr_psf_transform_normalized: the model does not give a finite PSF size");
    if (nd[0] != out_dims[0] || nd[1] != out_dims[1] || nd[2] != out_dims[2])
        return psf_fail(MVR_ERR_ARG, "mvr_psf_transform_normalized: out_dims differ from mvr_psf_transformed_dims");
    Affine inv;
    if (!invert_affine(model, inv.m)) return psf_fail(MVR_ERR_ARG, "mvr_psf_transform_normalized: singular model");
    Scratch sc;
    PSF_TRY(setup(device, &sc));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const long long n = (long long)dims[0] * dims[1] * dims[2];
    k_psf_minmax<<<1, 256, 0, s>>>(psf, n, sc.p);
    const long long no = (long long)nd[0] * nd[1] * nd[2];
    k_psf_transform<<<grid_of(no), 256, 0, s>>>(psf, dims[0], dims[1], dims[2], sc.p, inv, off[0], off[1], off[2],
                                                nd[0], nd[1], nd[2], out);
    return finish(s, "mvr_psf_transform_normalized");
}

extern "C" MVR_API int mvr_psf_average(const float *const *psfs, const int *dims, int num_psfs, int max_size,
                                       float *out, int out_dims[3], int device, void *stream)
{
    if (!psfs || !dims || !out || !out_dims || num_psfs < 1 || num_psfs > kMaxPsfs)
        return psf_fail(MVR_ERR_ARG, "mvr_psf_average: 1..64 PSFs and an output are required");
    PsfList L{};
    L.n = num_psfs;
    int a[3];
    for (int d = 0; d < 3; ++d) a[d] = max_size ? 0 : INT32_MAX;
    for (int k = 0; k < num_psfs; ++k) {
        if (!psfs[k] || !dims_ok(dims + 3 * k)) return psf_fail(MVR_ERR_ARG, "mvr_psf_average: bad PSF");
        L.p[k] = psfs[k];
        for (int d = 0; d < 3; ++d) {
            L.d[k][d] = dims[3 * k + d];
            a[d] = max_size ? std::max(a[d], dims[3 * k + d]) : std::min(a[d], dims[3 * k + d]);
        }
    }
    for (int d = 0; d < 3; ++d) out_dims[d] = a[d];
    PSF_TRY(setup(device, nullptr));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const long long n = (long long)a[0] * a[1] * a[2];
    k_psf_average<<<grid_of(n), 256, 0, s>>>(L, a[0], a[1], a[2], out);
    return finish(s, "mvr_psf_average");
}

extern "C" MVR_API int mvr_psf_make_same_size(const float *psf, const int dims[3], const int size[3], float *out,
                                              int device, void *stream)
{
    if (!psf || !dims_ok(dims) || !dims_ok(size) || !out)
        return psf_fail(MVR_ERR_ARG, "mvr_psf_make_same_size: bad arguments");
    Scratch sc;
    PSF_TRY(setup(device, &sc));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    k_psf_minmax<<<1, 256, 0, s>>>(psf, (long long)dims[0] * dims[1] * dims[2], sc.p);
    const long long n = (long long)size[0] * size[1] * size[2];
    k_psf_same_size<<<grid_of(n), 256, 0, s>>>(psf, dims[0], dims[1], dims[2], sc.p, size[0], size[1], size[2], out);
    return finish(s, "mvr_psf_make_same_size");
}

extern "C" MVR_API int mvr_psf_projection(const float *psf, const int dims[3], int dim, int use_max, float *out,
                                          int *used_dim, int device, void *stream)
{
    if (!psf || !dims_ok(dims) || !out || dim > 2) return psf_fail(MVR_ERR_ARG, "mvr_psf_projection: bad arguments");
    if (dim < 0) {  // the smallest axis (the first of equal ones)
        dim = 0;
        for (int d = 1; d < 3; ++d)
            if (dims[d] < dims[dim]) dim = d;
    }
    if (used_dim) *used_dim = dim;
    PSF_TRY(setup(device, nullptr));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const long long n = (long long)dims[0] * dims[1] * dims[2] / dims[dim];
    k_psf_project<<<grid_of(n), 256, 0, s>>>(psf, dims[0], dims[1], dims[2], dim, use_max ? 1 : 0, out);
    return finish(s, "mvr_psf_projection");
}

extern "C" MVR_API int mvr_psf_remove_min_projections(float *psf, const int dims[3], int device, void *stream)
{
    if (!psf || !dims_ok(dims)) return psf_fail(MVR_ERR_ARG, "mvr_psf_remove_min_projections: bad arguments");
    PSF_TRY(setup(device, nullptr));
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    const long long n = (long long)dims[0] * dims[1] * dims[2];
    float *proj = nullptr;
    const long long np = n / std::min(dims[0], std::min(dims[1], dims[2]));
    PSF_TRY(psf_cuda(cudaMalloc(&proj, sizeof(float) * (size_t)np), "cudaMalloc"));
    for (int d = 0; d < 3; ++d) {
        k_psf_project<<<grid_of(n / dims[d]), 256, 0, s>>>(psf, dims[0], dims[1], dims[2], d, 0, proj);
        k_psf_subtract<<<grid_of(n), 256, 0, s>>>(psf, dims[0], dims[1], dims[2], d, proj);
    }
    const int rc = finish(s, "mvr_psf_remove_min_projections");
    cudaFree(proj);
    return rc;
}
