// Device-resident whole-volume deconvolution: the GB300 counterpart of
// MultiViewDeconvolution{Seq,Mul} with DeconViews / DeconViewPSF.init, the block
// grid (BlockGeneratorFixedSizePrecise, BlockSorter, DeconView.filterBlocksForContent),
// weight normalisation (NormalizingRandomAccess) and PsiInitAvgPrecise.
//
// Reference files (relative to src/main/java/net/preibisch/mvrecon/process/):
//   deconvolution/MultiViewDeconvolutionSeq.java:57-180, MultiViewDeconvolutionMul.java:116-245
//   deconvolution/DeconViewPSF.java:119-284, deconvolution/normalization/AdjustInput.java:52-122,
//   deconvolution/util/Mirror.java:55-132, cuda/BlockGeneratorFixedSizePrecise.java:59-131,
//   cuda/BlockSorter.java:55-143, deconvolution/DeconView.java:118-274,
//   deconvolution/normalization/NormalizingRandomAccess.java:76-214,
//   deconvolution/init/PsiInitAvgPrecise.java:52-110
#include "wdiv.h"
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mvr_gb300.h"
#include "engine.cuh"

namespace mvr {

// ---- small device kernels -----------------------------------------------------------
namespace {

// sum over all and over the first `first` elements (AdjustInput.sumImg 115-119), FP64,
// one CTA in a fixed order
__global__ void k_sum_first(const float *__restrict__ k, long long n, long long first, double *out)
{
    __shared__ double sa[256], sf[256];
    double a = 0.0, f = 0.0;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = (double)k[i];
        a += v;
        if (i < first) f += v;
    }
    sa[threadIdx.x] = a;
    sf[threadIdx.x] = f;
    __syncthreads();
    for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            sa[threadIdx.x] += sa[threadIdx.x + h];
            sf[threadIdx.x] += sf[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sa[0];
        out[1] = sf[0];
    }
}

__global__ void k_div(float *k, long long n, const double *sums, int quirk)
{
    const double s = sums[0] + (quirk ? sums[1] : 0.0);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        k[i] = (float)((double)k[i] / s);
}

// out[z][y][x] = in[pz[z]][py[y]][px[x]]
__global__ void k_gather(const float *__restrict__ in, float *__restrict__ out, int kx, int ky, int kz,
                         const int *__restrict__ perm)
{
    const long long n = (long long)kx * ky * kz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % kx);
        const long long t = i / kx;
        const int y = (int)(t % ky), z = (int)(t / ky);
        const int sx = perm[x], sy = perm[kx + y], sz = perm[kx + ky + z];
        out[i] = in[((long long)sz * ky + sy) * kx + sx];
    }
}

__global__ void k_mul_into(float *tmp, const float *__restrict__ o, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        tmp[i] = __fmul_rn(o[i], tmp[i]);
}

// DeconViewPSF.pow 276-284: value^power by repeated float multiplication
__global__ void k_pow_views(const float *__restrict__ k, float *e, long long n, int power)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float r = k[i];
        for (int j = 1; j < power; ++j) r = __fmul_rn(r, k[i]);
        e[i] = r;
    }
}

struct WeightPtrs {
    const float *raw[kMaxViews];
    float *out[kMaxViews];
};

// NormalizingRandomAccess.get 76-109 (hardWeights 211-214, smoothWeights 183-200), one voxel
// at a time through mvr_wd_normalize: float operations that round as the reference's double
// sum and division do (the double operations only next to a float rounding boundary).  The
// views' weights sit in registers (loops over MAXV >= nv views, unrolled), and every thread
// loads U voxels before normalising any, so that more loads are in flight.
template <int MAXV, int U = (MAXV <= 8 ? 2 : 1)>
__global__ void k_normalize_weights(WeightPtrs wp, int nv, long long n, double osem, int smooth, float maxDiffRange,
                                    float scalingRange)
{
    const int osem_one = osem == 1.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; i0 < n; i0 += U * stride) {
        float w[U][MAXV], o[MAXV];
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const long long i = i0 + k * stride;
#pragma unroll
            for (int v = 0; v < MAXV; ++v) w[k][v] = (v < nv && i < n) ? fminf(1.0f, wp.raw[v][i]) : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < U; ++k) {
            const long long i = i0 + k * stride;
            if (i >= n) break;
            mvr_wd_normalize(w[k], nv, MAXV, osem_one, osem, smooth, maxDiffRange, scalingRange, o);
#pragma unroll
            for (int v = 0; v < MAXV; ++v)
                if (v < nv) wp.out[v][i] = o[v];
        }
    }
}

struct ImgPtrs {
    const float *img[kMaxViews];
};

// Optional fused output of PsiInitBlurredFused: the weighted average over the views with
// data, FusedNonZeroRandomAccess.get (deconvolution/util/FusedNonZeroRandomAccess.java
// 63-102): sum(I w) / sum(w) over I > 0, 0 where no weight.
struct FusePtrs {
    const float *w[kMaxViews];
    void *out;  // T volume, or NULL
};

// PsiInitAvgPreciseThread.compatibleLoop 127-160 (and the statistics of
// FusedNonZeroRandomAccess, which are the same), per-CTA partials
template <typename T>
__global__ void k_psi_avg_partials(ImgPtrs ip, FusePtrs fp, int nv, long long n, double *psum, long long *pcnt,
                                   float *pmax)
{
    __shared__ double ss[256];
    __shared__ long long sc[256];
    __shared__ float sm[256];
    double s = 0.0;
    long long c = 0;
    float mx[kMaxViews];
    for (int v = 0; v < nv; ++v) mx[v] = 0.0f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        double sum = 0.0, sumI = 0.0, sumW = 0.0;
        int cnt = 0;
        for (int v = 0; v < nv; ++v) {
            const float x = ip.img[v][i];
            if (x > 0.0f) {
                mx[v] = fmaxf(mx[v], x);
                sum += x;
                ++cnt;
                if (fp.out) {
                    const double wv = (double)fp.w[v][i];
                    sumI += (double)x * wv;
                    sumW += wv;
                }
            }
        }
        if (fp.out) reinterpret_cast<T *>(fp.out)[i] = sumW > 0.0 ? (T)(float)(sumI / sumW) : (T)0;
        if (cnt > 0) {
            s += sum / cnt;
            ++c;
        }
    }
    ss[threadIdx.x] = s;
    sc[threadIdx.x] = c;
    __syncthreads();
    for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            ss[threadIdx.x] += ss[threadIdx.x + h];
            sc[threadIdx.x] += sc[threadIdx.x + h];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        psum[blockIdx.x] = ss[0];
        pcnt[blockIdx.x] = sc[0];
    }
    for (int v = 0; v < nv; ++v) {
        sm[threadIdx.x] = mx[v];
        __syncthreads();
        for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
            if (threadIdx.x < h) sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + h]);
            __syncthreads();
        }
        if (threadIdx.x == 0) pmax[blockIdx.x * kMaxViews + v] = sm[0];
        __syncthreads();
    }
}

__global__ void k_psi_avg_final(const double *psum, const long long *pcnt, const float *pmax, int nparts, int nv,
                                double *avg_out, float *max_out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    long long c = 0;
    for (int i = 0; i < nparts; ++i) {
        s += psum[i];
        c += pcnt[i];
    }
    double avg = s / (double)c;
    if (isnan(avg)) avg = 1.0;
    *avg_out = avg;
    for (int v = 0; v < nv; ++v) {
        float m = 0.0f;
        for (int i = 0; i < nparts; ++i) m = fmaxf(m, pmax[i * kMaxViews + v]);
        max_out[v] = m;
    }
}

template <typename T>
__global__ void k_fill_avg(T *psi, long long n, const double *avg)
{
    const T v = (T)(float)(*avg);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        psi[i] = v;
}

// One separable pass of Gauss3.gauss (imglib2-algorithm, net.imglib2.algorithm.gauss3,
// called by PsiInitBlurredFused.java:117): out = sum_k h[|k|] in[mirror-single(i + k)]
// along `axis`, h the normalised half kernel of length hs.
template <typename T>
__global__ void k_gauss_axis(const T *__restrict__ in, T *__restrict__ out, long long D0, long long D1, long long D2,
                             int axis, const double *__restrict__ h, int hs)
{
    const long long n = D0 * D1 * D2;
    const long long len = axis == 0 ? D0 : (axis == 1 ? D1 : D2);
    const long long stride = axis == 0 ? 1 : (axis == 1 ? D0 : D0 * D1);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long c = (i / stride) % len;
        const long long base = i - c * stride;
        double acc = h[0] * (double)in[i];
        for (int k = 1; k < hs; ++k)
            acc += h[k] * ((double)in[base + mirror1(c - k, len) * stride] + (double)in[base + mirror1(c + k, len) * stride]);
        out[i] = (T)acc;
    }
}

// PsiInitAvgApproxThread.call 57-84: min / max / mean of each view's y-z slice at
// x = D0 / 2 (the reference iterates that same slice once per dimension, which leaves
// the mean unchanged).  One CTA per view: out[3 v .. 3 v + 2] = {sum, max, count}.
__global__ void k_slice_stats(ImgPtrs ip, long long D0, long long D1, long long D2, double *out)
{
    __shared__ double ss[256];
    __shared__ float sm[256];
    const float *img = ip.img[blockIdx.x];
    const long long x0 = D0 / 2, n = D1 * D2;
    double s = 0.0;
    float mx = -3.402823466e38f;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        const float v = img[i * D0 + x0];
        s += (double)v;
        mx = fmaxf(mx, v);
    }
    ss[threadIdx.x] = s;
    sm[threadIdx.x] = mx;
    __syncthreads();
    for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            ss[threadIdx.x] += ss[threadIdx.x + h];
            sm[threadIdx.x] = fmaxf(sm[threadIdx.x], sm[threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[3 * blockIdx.x] = ss[0];
        out[3 * blockIdx.x + 1] = (double)sm[0];
        out[3 * blockIdx.x + 2] = (double)n;
    }
}

template <typename A, typename B>
__global__ void k_convert(const A *__restrict__ in, B *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (B)in[i];
}

// DeconView.filterBlocksForContent (DeconView.java:204-274): flags[b] = 1 when block b's
// box (offsets offs[3 b .. 3 b + 2], size bx x by x bz, zero outside the volume) holds a
// non-zero weight.  One launch covers every block of a step (blockIdx.y = block).
__global__ void k_block_content(const float *__restrict__ w, long long D0, long long D1, long long D2,
                                const long long *__restrict__ offs, int bx, int by, int bz, int *flags)
{
    const int blk = blockIdx.y;
    const long long ox = offs[3 * blk], oy = offs[3 * blk + 1], oz = offs[3 * blk + 2];
    const long long n = (long long)bx * by * bz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long x = ox + i % bx;
        const long long t = i / bx;
        const long long y = oy + t % by, z = oz + t / by;
        if (x < 0 || y < 0 || z < 0 || x >= D0 || y >= D1 || z >= D2) continue;
        if (w[(z * D1 + y) * D0 + x] != 0.0f) {
            flags[blk] = 1;
            return;
        }
    }
}

int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 16)); }

}  // namespace

// ---- host helpers ---------------------------------------------------------------------
struct BlockDesc {
    long long off[3];
    long long eoff[3];
    int esize[3];
    int eloc[3];
    int batch;
};

// BlockGeneratorFixedSizePrecise.divideIntoBlocks + BlockSorter slab dimension; the
// doubled kernel kk = 2k-1 (DeconView 155-157).  Returns false when the block is
// smaller than the doubled kernel.
static bool divide_blocks(const long long D[3], const int kk[3], const int b[3], std::vector<BlockDesc> &out,
                          int &sort_dim, int min_required = 1)
{
    long long eff[3], nb[3];
    for (int d = 0; d < 3; ++d) {
        eff[d] = b[d] - kk[d] + 1;
        if (eff[d] <= 0) return false;
        nb[d] = D[d] / eff[d] + (D[d] % eff[d] != 0);
    }
    // BlockSorter: product of the other dims' counts; equal products keep the last dim
    long long sz[3];
    for (int d = 0; d < 3; ++d) {
        sz[d] = 1;
        for (int e = 0; e < 3; ++e)
            if (e != d) sz[d] *= nb[e];
    }
    long long srt[3] = {sz[0], sz[1], sz[2]};
    std::sort(srt, srt + 3);
    sort_dim = 2;
    for (int i = 0; i < 3; ++i) {
        if (srt[i] >= min_required || i == 2) {
            for (int d = 0; d < 3; ++d)
                if (sz[d] == srt[i]) sort_dim = d;  // last d with this product
            break;
        }
    }
    out.clear();
    for (long long z = 0; z < nb[2]; ++z)
        for (long long y = 0; y < nb[1]; ++y)
            for (long long x = 0; x < nb[0]; ++x) {
                const long long cb[3] = {x, y, z};
                BlockDesc bd{};
                for (int d = 0; d < 3; ++d) {
                    bd.eoff[d] = cb[d] * eff[d];
                    long long es = eff[d];
                    if (bd.eoff[d] + es > D[d]) es = D[d] - bd.eoff[d];
                    bd.esize[d] = (int)es;
                    bd.off[d] = bd.eoff[d] - kk[d] / 2;
                    bd.eloc[d] = kk[d] / 2;
                }
                bd.batch = (int)cb[sort_dim];
                out.push_back(bd);
            }
    return true;
}

// permutation of Mirror.mirror along one axis: swaps p <= n/2 with n-1-p in order
static std::vector<int> mirror_perm(int n)
{
    std::vector<int> p(n);
    for (int i = 0; i < n; ++i) p[i] = i;
    for (int i = 0; i < n; ++i)
        if (i <= n / 2) std::swap(p[i], p[n - 1 - i]);
    return p;
}

// FusionTools.divideIntoPortions 1287-1329: length of the first portion for T threads
static long long first_portion(long long size, int T)
{
    if (size == 0 || T <= 0) return 0;
    long long np = size <= T ? size : std::max<long long>(T, size / (64LL * 64 * 64));
    long long chunk = size / np;
    while (chunk == 0) {
        --np;
        chunk = size / np;
    }
    return np == 1 ? size : chunk;
}

class DeconBase {
public:
    virtual ~DeconBase() = default;
    virtual int set_images(int v, const float *img, const float *w, bool on_device) = 0;
    virtual int set_psf(int v, const float *psf, const int dims[3]) = 0;
    virtual int set_view_block(int v, const int block[3]) = 0;
    virtual int set_view_effective(int v, const int eff[3]) = 0;
    virtual int prepare() = 0;
    virtual int set_psi(const float *psi, bool on_device) = 0;
    virtual int get_psi(float *psi) = 0;
    virtual int get_psi_device(float *psi) = 0;
    virtual int run(int iterations, double *stats) = 0;
    virtual int run_host(int iterations, const float *const *imgs, const float *const *ws, float *psi,
                         const float *const *next_imgs, const float *const *next_ws) = 0;
    virtual int get_kernels(int v, float *k1, float *k2) = 0;
    virtual int get_max(float *mx) = 0;
    virtual int get_weights(int v, float *w) = 0;
    virtual const void *psi_device() const = 0;
    virtual int synchronize() = 0;
    virtual int num_steps() const = 0;
    virtual const std::string &error() const = 0;
    virtual void *stream() = 0;
    virtual long long launches() const = 0;
    virtual void set_profiling(bool on) = 0;
    virtual int profile(KernelProfile &out) = 0;
    virtual int batch() const = 0;
    virtual int likelihood(double *total, double *per_view) = 0;
    virtual int set_graphs(bool on) = 0;
    virtual int psi_init(int method, double sigma, double *avg) = 0;
    virtual int graphs_captured() const = 0;
    virtual int set_schedule(int code) = 0;
    virtual int schedule(int view) const = 0;
    virtual int tuning(int capacity, int *step, int *code, int *batch, float *ms) const = 0;
};

template <typename T>
class Decon : public DeconBase {
public:
    explicit Decon(const mvr_decon_params &p) : p_(p) {}
    ~Decon() override;
    int init();
    int set_images(int v, const float *img, const float *w, bool on_device) override;
    int set_psf(int v, const float *psf, const int dims[3]) override;
    int set_view_block(int v, const int block[3]) override;
    int set_view_effective(int v, const int eff[3]) override;
    int prepare() override;
    int set_psi(const float *psi, bool on_device) override;
    int get_psi(float *psi) override;
    int get_psi_device(float *psi) override;
    int run(int iterations, double *stats) override;
    int run_host(int iterations, const float *const *imgs, const float *const *ws, float *psi,
                 const float *const *next_imgs, const float *const *next_ws) override;
    int get_kernels(int v, float *k1, float *k2) override;
    int get_max(float *mx) override;
    int get_weights(int v, float *w) override;
    const void *psi_device() const override { return psi_; }
    int synchronize() override;
    int num_steps() const override { return p_.mul ? 1 : p_.num_views; }
    const std::string &error() const override { return err_; }
    void *stream() override { return (void *)engine_.stream(); }
    long long launches() const override { return engine_.launches(); }
    void set_profiling(bool on) override { engine_.set_profiling(on); }
    int profile(KernelProfile &out) override { return eng(engine_.profile_collect(out)); }
    int batch() const override { return batch_; }
    int likelihood(double *total, double *per_view) override;

private:
    struct View {
        float *img = nullptr, *w = nullptr, *w_raw = nullptr;
        bool own_img = false, own_w = false;
        std::vector<float> psf;
        int kd[3] = {0, 0, 0};
        int block[3] = {0, 0, 0};            // compute block size of this view (0: the handle's)
        int eff[3] = {0, 0, 0};              // effective block size (0: block - 2 (k - 1))
        float *k1 = nullptr, *k2 = nullptr;  // device, prepared kernels
        Plan<T> plan;
        const int *bsize(const int *dflt) const { return block[0] > 0 ? block : dflt; }
    };
    int fail(int c, const std::string &m)
    {
        err_ = m;
        return c;
    }
    int cuda(cudaError_t e, const char *what)
    {
        if (e == cudaSuccess) return MVR_OK;
        err_ = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? MVR_ERR_OOM : MVR_ERR_CUDA;
    }
    int eng(int rc)
    {
        if (rc != MVR_OK) err_ = engine_.error();
        return rc;
    }
    int norm_to_sum1(float *k, long long n);
    int invert(const float *in, float *out, const int kd[3]);
    int conv_zero(const float *in, const int id[3], const float *k, const int kd[3], float *out);
    int psf_init();
    int run_step(int s, double *stats_slot, bool trial, int batch);
    int run_iteration(double *stats_base, size_t stats_stride);
    int init_psi(int method, double sigma, double *avg_out);
    int autotune();
    // Whole iterations captured as CUDA graphs, one per starting state: the psi buffer
    // (the Jacobi path swaps psi and the staging volume every view-step), the stats
    // slots, the batch size and the engine's scratch allocation.  The first iteration in
    // a new state runs eagerly (it may allocate scratch); when the next one starts in the
    // same state it is captured, and every later one replays the graph.
    struct IterGraph {
        const T *psi_start = nullptr;
        const double *stats = nullptr;
        int batch = 0;
        long long epoch = -1;
        long long inputs = -1;
        int set = 0;  // which of the two input buffer sets of mvr_decon_run_host_next is in use
        cudaGraphExec_t exec = nullptr;
        T *psi_end = nullptr, *stage_end = nullptr;
        long long launches = 0;
        bool same(const IterGraph &o) const
        {
            return psi_start == o.psi_start && stats == o.stats && batch == o.batch && epoch == o.epoch &&
                   inputs == o.inputs && set == o.set;
        }
    };
    std::vector<IterGraph> graphs_;
    std::vector<IterGraph> seen_;  // states of recent eager iterations (psi alternates between two buffers)
    bool graphs_on_ = true;
    long long inputs_epoch_ = 0;  // bumped when image/weight pointers or the set-up change
    void drop_graphs();

public:
    int set_graphs(bool on) override
    {
        graphs_on_ = on;
        if (!on) drop_graphs();
        return MVR_OK;
    }
    int graphs_captured() const override { return (int)graphs_.size(); }
    int set_schedule(int code) override;
    int schedule(int view) const override;
    int tuning(int capacity, int *step, int *code, int *batch, float *ms) const override;
    int psi_init(int method, double sigma, double *avg) override;

private:
    int normalize_weights();
    int batch_ = 1;
    struct Trial {
        int step;   // view-step of a schedule trial, -1 for a batch trial
        int code;   // FFT schedule (SCHED_*), -1 for a batch trial
        int batch;  // blocks per launch
        float ms;   // one view-step
    };
    std::vector<Trial> tune_;
    int force_sched_ = -1;  // FFT schedule forced for every view, -1: autotuned
    bool weights_dirty_ = false;

    mvr_decon_params p_;
    Engine<T> engine_;
    std::vector<View> views_;
    long long n_ = 0;
    T *psi_ = nullptr, *stage_ = nullptr;
    std::vector<std::vector<BlockDesc>> blocks_;  // per step
    std::vector<int> sort_dim_;
    std::vector<int> jacobi_;
    std::vector<float> max_;
    double *d_scratch_ = nullptr;  // reductions
    int *d_perm_ = nullptr;
    double *d_stats_ = nullptr;
    long long stats_cap_ = 0;
    cudaStream_t copy_ = nullptr;              // uploads of mvr_decon_run_host
    cudaEvent_t ev_w_ = nullptr;               // weights and psi uploaded
    std::vector<cudaEvent_t> ev_img_;          // image of view v uploaded
    // the next call's images and raw weights, uploaded during this call's iterations into a
    // second set of device buffers (mvr_decon_run_host_next)
    std::vector<float *> alt_img_, alt_w_;
    std::vector<const float *> pre_img_, pre_w_;  // the host arrays the second set holds
    bool pre_valid_ = false;
    int cur_set_ = 0;               // flips with every swap of the two sets
    cudaEvent_t ev_pre_ = nullptr;  // the second set uploaded
    bool prepared_ = false;
    std::string err_;
};

#define D_TRY(expr)                   \
    do {                              \
        int rc__ = (expr);            \
        if (rc__ != MVR_OK) return rc__; \
    } while (0)
#define D_CUDA(expr) D_TRY(cuda((expr), #expr))

template <typename T>
Decon<T>::~Decon()
{
    cudaSetDevice(p_.device);
    for (auto &v : views_) {
        if (v.own_img) cudaFree(v.img);
        if (v.own_w) cudaFree(v.w_raw);
        if (v.w != v.w_raw) cudaFree(v.w);
        cudaFree(v.k1);
        cudaFree(v.k2);
        engine_.free_plan(v.plan);
    }
    cudaFree(psi_);
    cudaFree(stage_);
    cudaFree(d_scratch_);
    cudaFree(d_perm_);
    cudaFree(d_stats_);
    if (copy_) cudaStreamSynchronize(copy_);  // a prefetch may still read host arrays
    for (float *a : alt_img_) cudaFree(a);
    for (float *a : alt_w_) cudaFree(a);
    for (cudaEvent_t e : ev_img_) cudaEventDestroy(e);
    if (ev_w_) cudaEventDestroy(ev_w_);
    if (ev_pre_) cudaEventDestroy(ev_pre_);
    if (copy_) cudaStreamDestroy(copy_);
    drop_graphs();
}

template <typename T>
void Decon<T>::drop_graphs()
{
    for (auto &g : graphs_)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    graphs_.clear();
    seen_.clear();
}

template <typename T>
int Decon<T>::init()
{
    for (int d = 0; d < 3; ++d)
        if (p_.dims[d] < 1 || p_.block_size[d] < 1) return fail(MVR_ERR_ARG, "dims and block_size must be >= 1");
    if (p_.num_views < 1 || p_.num_views > kMaxViews) return fail(MVR_ERR_ARG, "num_views must be 1..16");
    if (p_.psf_type < 0 || p_.psf_type > 3) return fail(MVR_ERR_ARG, "unknown psf_type");
    if (p_.boundary != MVR_BOUNDARY_REFERENCE && p_.boundary != MVR_BOUNDARY_CIRCULAR)
        return fail(MVR_ERR_ARG, "unknown boundary");
    D_TRY(eng(engine_.init(p_.device, p_.boundary, (double)p_.lambda, p_.min_value)));
    n_ = (long long)p_.dims[0] * p_.dims[1] * p_.dims[2];
    views_.resize(p_.num_views);
    D_CUDA(cudaMalloc(&psi_, sizeof(T) * (size_t)n_));
    D_CUDA(cudaMalloc(&stage_, sizeof(T) * (size_t)n_));
    D_CUDA(cudaMalloc(&d_scratch_, sizeof(double) * 2 * 4096 + sizeof(long long) * 4096 + sizeof(float) * 4096 * kMaxViews));
    return MVR_OK;
}

template <typename T>
int Decon<T>::set_images(int v, const float *img, const float *w, bool on_device)
{
    if (v < 0 || v >= p_.num_views) return fail(MVR_ERR_ARG, "view out of range");
    if (!img || !w) return fail(MVR_ERR_ARG, "image and weight must not be NULL");
    D_CUDA(cudaSetDevice(p_.device));
    View &vw = views_[v];
    cudaStream_t s = engine_.stream();
    ++inputs_epoch_;
    if (on_device) {
        if (vw.own_img) cudaFree(vw.img);
        if (vw.own_w) cudaFree(vw.w_raw);
        vw.img = const_cast<float *>(img);
        vw.w_raw = const_cast<float *>(w);
        vw.own_img = vw.own_w = false;
    } else {
        if (!vw.own_img) {
            vw.img = nullptr;
            D_CUDA(cudaMalloc(&vw.img, sizeof(float) * (size_t)n_));
            vw.own_img = true;
        }
        if (!vw.own_w) {
            vw.w_raw = nullptr;
            D_CUDA(cudaMalloc(&vw.w_raw, sizeof(float) * (size_t)n_));
            vw.own_w = true;
        }
        D_CUDA(cudaMemcpyAsync(vw.img, img, sizeof(float) * (size_t)n_, cudaMemcpyHostToDevice, s));
        D_CUDA(cudaMemcpyAsync(vw.w_raw, w, sizeof(float) * (size_t)n_, cudaMemcpyHostToDevice, s));
    }
    if (p_.weight_norm == MVR_WEIGHTS_AS_GIVEN) {
        if (vw.w != vw.w_raw && vw.w) cudaFree(vw.w);
        vw.w = vw.w_raw;
    } else if (prepared_) {
        weights_dirty_ = true;  // weights depend on all views: renormalised before the next use
    }
    return MVR_OK;
}

template <typename T>
int Decon<T>::set_psf(int v, const float *psf, const int dims[3])
{
    if (v < 0 || v >= p_.num_views) return fail(MVR_ERR_ARG, "view out of range");
    if (!psf || !dims || dims[0] < 1 || dims[1] < 1 || dims[2] < 1) return fail(MVR_ERR_ARG, "bad psf");
    View &vw = views_[v];
    const long long kn = (long long)dims[0] * dims[1] * dims[2];
    vw.psf.assign(psf, psf + kn);
    std::memcpy(vw.kd, dims, sizeof(vw.kd));
    prepared_ = false;
    return MVR_OK;
}

template <typename T>
int Decon<T>::set_view_block(int v, const int block[3])
{
    if (v < 0 || v >= p_.num_views) return fail(MVR_ERR_ARG, "view out of range");
    if (!block) {
        std::memset(views_[v].block, 0, sizeof(views_[v].block));
    } else {
        for (int d = 0; d < 3; ++d)
            if (block[d] < 1) return fail(MVR_ERR_ARG, "block sizes must be >= 1");
        std::memcpy(views_[v].block, block, sizeof(views_[v].block));
    }
    prepared_ = false;
    return MVR_OK;
}

template <typename T>
int Decon<T>::set_view_effective(int v, const int eff[3])
{
    if (v < -1 || v >= p_.num_views) return fail(MVR_ERR_ARG, "view out of range");
    for (int u = (v < 0 ? 0 : v); u < (v < 0 ? p_.num_views : v + 1); ++u) {
        if (!eff) {
            std::memset(views_[u].eff, 0, sizeof(views_[u].eff));
        } else {
            for (int d = 0; d < 3; ++d)
                if (eff[d] < 1) return fail(MVR_ERR_ARG, "effective block sizes must be >= 1");
            std::memcpy(views_[u].eff, eff, sizeof(views_[u].eff));
        }
    }
    prepared_ = false;
    return MVR_OK;
}

template <typename T>
int Decon<T>::norm_to_sum1(float *k, long long n)
{
    const long long first = p_.psf_norm_threads > 0 ? first_portion(n, p_.psf_norm_threads) : 0;
    cudaStream_t s = engine_.stream();
    k_sum_first<<<1, 256, 0, s>>>(k, n, first, d_scratch_);
    D_CUDA(cudaGetLastError());
    k_div<<<grid_for(n), 256, 0, s>>>(k, n, d_scratch_, p_.psf_norm_threads > 0);
    D_CUDA(cudaGetLastError());
    return MVR_OK;
}

template <typename T>
int Decon<T>::invert(const float *in, float *out, const int kd[3])
{
    std::vector<int> perm;
    for (int d = 0; d < 3; ++d) {
        std::vector<int> p = mirror_perm(kd[d]);
        perm.insert(perm.end(), p.begin(), p.end());
    }
    cudaFree(d_perm_);
    d_perm_ = nullptr;
    D_CUDA(cudaMalloc(&d_perm_, sizeof(int) * perm.size()));
    cudaStream_t s = engine_.stream();
    D_CUDA(cudaMemcpyAsync(d_perm_, perm.data(), sizeof(int) * perm.size(), cudaMemcpyHostToDevice, s));
    const long long n = (long long)kd[0] * kd[1] * kd[2];
    k_gather<<<grid_for(n), 256, 0, s>>>(in, out, kd[0], kd[1], kd[2], d_perm_);
    D_CUDA(cudaGetLastError());
    D_CUDA(cudaStreamSynchronize(s));  // perm buffer is reused
    return MVR_OK;
}

// FFTConvolution(extendZero(in), in, extendZero(k), k, out): linear, zero extension,
// output over `in`, rounded to float.
template <typename T>
int Decon<T>::conv_zero(const float *in, const int id[3], const float *k, const int kd[3], float *out)
{
    Engine<float> e;
    D_TRY(e.init(p_.device, BOUNDARY_REFERENCE, 0.0, 0.0f) == MVR_OK ? MVR_OK : fail(MVR_ERR_CUDA, e.error()));
    D_CUDA(cudaStreamSynchronize(engine_.stream()));
    Plan<float> pl;
    int rc = e.make_plan(pl, id, k, kd, nullptr, nullptr, true);
    if (rc == MVR_OK) rc = e.convolve(pl, in, SRC_ZERO, out);
    if (rc == MVR_OK) rc = e.cuda_check(cudaStreamSynchronize(e.stream()), "conv_zero");
    if (rc != MVR_OK) err_ = e.error();
    e.free_plan(pl);
    return rc;
}

// DeconViewPSF.init 119-254 for all views in order.
template <typename T>
int Decon<T>::psf_init()
{
    const int nv = p_.num_views;
    cudaStream_t s = engine_.stream();
    for (auto &vw : views_) {
        const long long kn = (long long)vw.kd[0] * vw.kd[1] * vw.kd[2];
        cudaFree(vw.k1);
        cudaFree(vw.k2);
        vw.k1 = vw.k2 = nullptr;
        D_CUDA(cudaMalloc(&vw.k1, sizeof(float) * (size_t)kn));
        D_CUDA(cudaMalloc(&vw.k2, sizeof(float) * (size_t)kn));
        D_CUDA(cudaMemcpyAsync(vw.k1, vw.psf.data(), sizeof(float) * (size_t)kn, cudaMemcpyHostToDevice, s));
    }
    for (int v = 0; v < nv; ++v) {
        View &vw = views_[v];
        const long long n = (long long)vw.kd[0] * vw.kd[1] * vw.kd[2];
        D_TRY(norm_to_sum1(vw.k1, n));
        if (nv == 1 || p_.psf_type == MVR_PSF_INDEPENDENT) {
            D_TRY(invert(vw.k1, vw.k2, vw.kd));
            continue;
        }
        float *tmp = nullptr, *a = nullptr, *b = nullptr, *c = nullptr;
        D_CUDA(cudaMalloc(&tmp, sizeof(float) * (size_t)n));
        D_CUDA(cudaMalloc(&a, sizeof(float) * (size_t)n));
        D_CUDA(cudaMalloc(&b, sizeof(float) * (size_t)n));
        int rc = MVR_OK;
        if (p_.psf_type == MVR_PSF_EFFICIENT_BAYESIAN) {
            rc = invert(vw.k1, tmp, vw.kd);
            for (int w = 0; w < nv && rc == MVR_OK; ++w) {
                if (w == v) continue;
                View &ww = views_[w];
                const long long nw = (long long)ww.kd[0] * ww.kd[1] * ww.kd[2];
                c = nullptr;
                if (cudaMalloc(&c, sizeof(float) * (size_t)nw) != cudaSuccess) { rc = fail(MVR_ERR_OOM, "psf scratch"); break; }
                rc = invert(vw.k1, a, vw.kd);
                if (rc == MVR_OK) rc = conv_zero(a, vw.kd, ww.k1, ww.kd, b);
                if (rc == MVR_OK) rc = invert(ww.k1, c, ww.kd);
                if (rc == MVR_OK) rc = conv_zero(b, vw.kd, c, ww.kd, a);
                if (rc == MVR_OK) {
                    k_mul_into<<<grid_for(n), 256, 0, s>>>(tmp, a, n);
                    rc = cuda(cudaGetLastError(), "k_mul_into");
                }
                cudaStreamSynchronize(s);
                cudaFree(c);
            }
            if (rc == MVR_OK) rc = norm_to_sum1(tmp, n);
            if (rc == MVR_OK) rc = cuda(cudaMemcpyAsync(vw.k2, tmp, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, s), "copy");
        } else if (p_.psf_type == MVR_PSF_OPTIMIZATION_I) {
            rc = cuda(cudaMemcpyAsync(tmp, vw.k1, sizeof(float) * (size_t)n, cudaMemcpyDeviceToDevice, s), "copy");
            for (int w = 0; w < nv && rc == MVR_OK; ++w) {
                if (w == v) continue;
                View &ww = views_[w];
                const long long nw = (long long)ww.kd[0] * ww.kd[1] * ww.kd[2];
                c = nullptr;
                if (cudaMalloc(&c, sizeof(float) * (size_t)nw) != cudaSuccess) { rc = fail(MVR_ERR_OOM, "psf scratch"); break; }
                rc = invert(ww.k1, c, ww.kd);
                if (rc == MVR_OK) rc = conv_zero(vw.k1, vw.kd, c, ww.kd, a);
                if (rc == MVR_OK) {
                    k_mul_into<<<grid_for(n), 256, 0, s>>>(tmp, a, n);
                    rc = cuda(cudaGetLastError(), "k_mul_into");
                }
                cudaStreamSynchronize(s);
                cudaFree(c);
            }
            if (rc == MVR_OK) rc = norm_to_sum1(tmp, n);
            if (rc == MVR_OK) rc = invert(tmp, vw.k2, vw.kd);
        } else {  // OPTIMIZATION_II
            k_pow_views<<<grid_for(n), 256, 0, s>>>(vw.k1, tmp, n, nv);
            rc = cuda(cudaGetLastError(), "k_pow_views");
            if (rc == MVR_OK) rc = norm_to_sum1(tmp, n);
            if (rc == MVR_OK) rc = invert(tmp, vw.k2, vw.kd);
        }
        cudaStreamSynchronize(s);
        cudaFree(tmp);
        cudaFree(a);
        cudaFree(b);
        D_TRY(rc);
    }
    return MVR_OK;
}

template <typename T>
int Decon<T>::prepare()
{
    D_CUDA(cudaSetDevice(p_.device));
    ++inputs_epoch_;
    drop_graphs();
    cudaStream_t s = engine_.stream();
    const int nv = p_.num_views;
    for (int v = 0; v < nv; ++v) {
        if (!views_[v].img || !views_[v].w_raw) return fail(MVR_ERR_STATE, "images/weights missing for a view");
        if (views_[v].psf.empty()) return fail(MVR_ERR_STATE, "psf missing for a view");
    }
    if (p_.mul) {
        for (int v = 1; v < nv; ++v)
            if (std::memcmp(views_[v].kd, views_[0].kd, sizeof(views_[0].kd)) != 0)
                return fail(MVR_ERR_ARG, "multiplicative mode needs one block grid: equal PSF sizes "
                                         "(MultiViewDeconvolutionMul.testBlockIntegrity)");
        for (int v = 1; v < nv; ++v)
            if (std::memcmp(views_[v].bsize(p_.block_size), views_[0].bsize(p_.block_size), 3 * sizeof(int)) != 0 ||
                std::memcmp(views_[v].eff, views_[0].eff, sizeof(views_[0].eff)) != 0)
                return fail(MVR_ERR_ARG, "multiplicative mode needs one block grid: equal block sizes");
    }
    // weights
    if (p_.weight_norm != MVR_WEIGHTS_AS_GIVEN) {
        for (int v = 0; v < nv; ++v) {
            if (views_[v].w == nullptr || views_[v].w == views_[v].w_raw) {
                views_[v].w = nullptr;
                D_CUDA(cudaMalloc(&views_[v].w, sizeof(float) * (size_t)n_));
            }
        }
        D_TRY(normalize_weights());
    } else {
        for (auto &vw : views_) vw.w = vw.w_raw;
    }
    // PSFs and their spectra for this block size
    D_TRY(psf_init());
    for (auto &vw : views_)
        D_TRY(eng(engine_.make_plan(vw.plan, vw.bsize(p_.block_size), vw.k1, vw.kd, vw.k2, vw.kd, true)));
    // block grids per step
    const long long D[3] = {p_.dims[0], p_.dims[1], p_.dims[2]};
    const int steps = num_steps();
    blocks_.assign(steps, {});
    sort_dim_.assign(steps, 2);
    jacobi_.assign(steps, 1);
    for (int st = 0; st < steps; ++st) {
        const View &vw = views_[st];
        std::vector<BlockDesc> all;
        const int *bs = vw.bsize(p_.block_size);
        // the grid's overlap: the doubled kernel 2k-1, or block - effective + 1 when an
        // effective block size is set (at least the doubled kernel)
        int kk[3];
        for (int d = 0; d < 3; ++d) {
            kk[d] = 2 * vw.kd[d] - 1;
            if (vw.eff[0] > 0) {
                if (bs[d] - vw.eff[d] + 1 < kk[d])
                    return fail(MVR_ERR_ARG, "effective block leaves less overlap than the doubled kernel (2k-1)");
                kk[d] = bs[d] - vw.eff[d] + 1;
            }
        }
        if (!divide_blocks(D, kk, bs, all, sort_dim_[st]))
            return fail(MVR_ERR_ARG, "block size smaller than the doubled kernel (2k-1)");
        const float *wcheck = views_[st].w;  // Mul: view 0's grid and weight
        std::vector<int> keep(all.size(), 1);
        if (p_.filter_blocks && !all.empty()) {
            // one launch over all blocks of the step, one copy of the flags back.  The region
            // checked is the reference's block, effective + 2 (k - 1) around the effective
            // region (the compute block itself unless an effective size is set)
            const int nb = (int)all.size();
            int cs[3];
            for (int d = 0; d < 3; ++d) cs[d] = vw.eff[0] > 0 ? vw.eff[d] + 2 * (vw.kd[d] - 1) : bs[d];
            std::vector<long long> offs(3 * (size_t)nb);
            for (int b = 0; b < nb; ++b)
                for (int d = 0; d < 3; ++d) offs[3 * (size_t)b + d] = all[b].eoff[d] - (vw.kd[d] - 1);
            long long *d_offs = nullptr;
            int *d_flags = nullptr;
            D_CUDA(cudaMalloc(&d_offs, sizeof(long long) * offs.size()));
            const cudaError_t ea = cudaMalloc(&d_flags, sizeof(int) * (size_t)nb);
            if (ea != cudaSuccess) {
                cudaFree(d_offs);
                D_CUDA(ea);
            }
            cudaError_t e = cudaMemcpyAsync(d_offs, offs.data(), sizeof(long long) * offs.size(),
                                            cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(d_flags, 0, sizeof(int) * (size_t)nb, s);
            if (e == cudaSuccess) {
                const long long bn = (long long)cs[0] * cs[1] * cs[2];
                const int gx = (int)std::max<long long>(1, std::min<long long>((bn + 255) / 256, 64));
                k_block_content<<<dim3(gx, nb), 256, 0, s>>>(wcheck, D[0], D[1], D[2], d_offs, cs[0], cs[1], cs[2],
                                                            d_flags);
                e = cudaGetLastError();
            }
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(keep.data(), d_flags, sizeof(int) * (size_t)nb, cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            cudaFree(d_offs);
            cudaFree(d_flags);
            D_CUDA(e);
        }
        for (size_t b = 0; b < all.size(); ++b)
            if (keep[b]) blocks_[st].push_back(all[b]);
        // every block of a batch reads psi before the step when the slab's effective
        // size >= k-1 (deferred write-back, MultiViewDeconvolutionSeq 79-162)
        const int sd = sort_dim_[st];
        const long long eff = bs[sd] - kk[sd] + 1;
        jacobi_[st] = (eff >= vw.kd[sd] - 1 && blocks_[st].size() == all.size()) ? 1 : 0;
    }
    // psi init: PsiInitAvgPrecise (average over views with data) and max per view
    D_TRY(init_psi(MVR_PSI_INIT_AVG_PRECISE, 0.0, nullptr));
    D_CUDA(cudaStreamSynchronize(s));
    D_TRY(autotune());
    prepared_ = true;
    return MVR_OK;
}

template <typename T>
int Decon<T>::psi_init(int method, double sigma, double *avg)
{
    if (!prepared_) return fail(MVR_ERR_STATE, "mvr_decon_prepare was not called");
    D_CUDA(cudaSetDevice(p_.device));
    if (weights_dirty_) D_TRY(normalize_weights());
    return init_psi(method, sigma, avg);
}

// PsiInit (deconvolution/init/): psi and the per-view maxima used by the update.
//   AVG_PRECISE    PsiInitAvgPrecise.java:52-110: psi = mean over voxels with data of the
//                  mean of the views with data; max = per-view maximum
//   AVG_APPROX     PsiInitAvgApprox.java:49-106 with PsiInitAvgApproxThread.java:57-84:
//                  psi = mean over views of the mean of the y-z slice at x = D0 / 2; max =
//                  that slice's maximum
//   BLURRED_FUSED  PsiInitBlurredFused.java:66-127: psi = the non-zero weighted fusion
//                  (normalised weights), then Gauss3 with sigma on all axes and mirror-single
//                  extension; avg / max as AVG_PRECISE
template <typename T>
int Decon<T>::init_psi(int method, double sigma, double *avg_out)
{
    cudaStream_t s = engine_.stream();
    const int nv = p_.num_views;
    ImgPtrs ip{};
    for (int v = 0; v < nv; ++v) ip.img[v] = views_[v].img;
    double avg_h = 0.0;
    if (method == MVR_PSI_INIT_AVG_PRECISE || method == MVR_PSI_INIT_BLURRED_FUSED) {
        const int parts = 1024;
        double *psum = d_scratch_;
        long long *pcnt = reinterpret_cast<long long *>(d_scratch_ + 2 * 4096);
        float *pmax = reinterpret_cast<float *>(pcnt + 4096);
        FusePtrs fp{};
        if (method == MVR_PSI_INIT_BLURRED_FUSED) {
            for (int v = 0; v < nv; ++v) fp.w[v] = views_[v].w;
            fp.out = psi_;
        }
        k_psi_avg_partials<T><<<parts, 256, 0, s>>>(ip, fp, nv, n_, psum, pcnt, pmax);
        D_CUDA(cudaGetLastError());
        double *avg = d_scratch_ + 4096;
        float *mx = reinterpret_cast<float *>(d_scratch_ + 4097);
        k_psi_avg_final<<<1, 1, 0, s>>>(psum, pcnt, pmax, parts, nv, avg, mx);
        D_CUDA(cudaGetLastError());
        if (method == MVR_PSI_INIT_AVG_PRECISE) {
            k_fill_avg<T><<<grid_for(n_), 256, 0, s>>>(psi_, n_, avg);
            D_CUDA(cudaGetLastError());
        } else {
            // Gauss3.halfkernel: h[0] = 1, h[x] = exp(-x^2 / (2 sigma^2)) for x < hs =
            // max(2, (int)(3 sigma + 0.5) + 1), normalised so that h[0] + 2 sum h[x>0] = 1
            if (!(sigma > 0.0) || sigma > 1000.0) return fail(MVR_ERR_ARG, "sigma must be in (0, 1000]");
            const int hs = std::max(2, (int)(3.0 * sigma + 0.5) + 1);
            std::vector<double> h(hs);
            h[0] = 1.0;
            double sum = 0.5;
            for (int x = 1; x < hs; ++x) {
                h[x] = std::exp(-(double)(x * x) / (2.0 * sigma * sigma));
                sum += h[x];
            }
            sum *= 2.0;
            for (double &v : h) v /= sum;
            double *dh = nullptr;
            D_CUDA(cudaMalloc(&dh, sizeof(double) * hs));
            int rc = cuda(cudaMemcpyAsync(dh, h.data(), sizeof(double) * hs, cudaMemcpyHostToDevice, s), "gauss kernel");
            const long long D0 = p_.dims[0], D1 = p_.dims[1], D2 = p_.dims[2];
            T *a = psi_, *b = stage_;
            for (int axis = 0; axis < 3 && rc == MVR_OK; ++axis) {
                k_gauss_axis<T><<<grid_for(n_), 256, 0, s>>>(a, b, D0, D1, D2, axis, dh, hs);
                rc = cuda(cudaGetLastError(), "k_gauss_axis");
                std::swap(a, b);
            }
            if (rc == MVR_OK) rc = cuda(cudaStreamSynchronize(s), "gauss");
            cudaFree(dh);
            D_TRY(rc);
            psi_ = a;  // the result of the third pass
            stage_ = b;
        }
        max_.assign(nv, 0.0f);
        D_CUDA(cudaMemcpyAsync(max_.data(), mx, sizeof(float) * nv, cudaMemcpyDeviceToHost, s));
        D_CUDA(cudaMemcpyAsync(&avg_h, avg, sizeof(double), cudaMemcpyDeviceToHost, s));
    } else if (method == MVR_PSI_INIT_AVG_APPROX) {
        double *st = d_scratch_;
        k_slice_stats<<<nv, 256, 0, s>>>(ip, p_.dims[0], p_.dims[1], p_.dims[2], st);
        D_CUDA(cudaGetLastError());
        std::vector<double> hs(3 * nv);
        D_CUDA(cudaMemcpyAsync(hs.data(), st, sizeof(double) * 3 * nv, cudaMemcpyDeviceToHost, s));
        D_CUDA(cudaStreamSynchronize(s));
        max_.assign(nv, 0.0f);
        for (int v = 0; v < nv; ++v) {
            avg_h += hs[3 * v] / hs[3 * v + 2];
            max_[v] = (float)hs[3 * v + 1];
        }
        avg_h /= (double)nv;
        if (std::isnan(avg_h)) avg_h = 1.0;
        double *avg = d_scratch_ + 4096;
        D_CUDA(cudaMemcpyAsync(avg, &avg_h, sizeof(double), cudaMemcpyHostToDevice, s));
        k_fill_avg<T><<<grid_for(n_), 256, 0, s>>>(psi_, n_, avg);
        D_CUDA(cudaGetLastError());
    } else {
        return fail(MVR_ERR_ARG, "unknown psi initialisation");
    }
    D_CUDA(cudaStreamSynchronize(s));
    if (avg_out) *avg_out = avg_h;
    ++inputs_epoch_;  // max_ and possibly the psi buffer changed: captured graphs are stale
    drop_graphs();
    return MVR_OK;
}

template <typename T>
int Decon<T>::normalize_weights()
{
    WeightPtrs wp{};
    for (int v = 0; v < p_.num_views; ++v) {
        wp.raw[v] = views_[v].w_raw;
        wp.out[v] = views_[v].w;
    }
    const int nv = p_.num_views, sm = p_.weight_norm == MVR_WEIGHTS_SMOOTH;
    const double osem = (double)p_.osem_speedup;
    cudaStream_t s = engine_.stream();
    if (nv <= 4)
        k_normalize_weights<4><<<grid_for(n_), 256, 0, s>>>(wp, nv, n_, osem, sm, p_.max_diff_range, p_.scaling_range);
    else if (nv <= 8)
        k_normalize_weights<8><<<grid_for(n_), 256, 0, s>>>(wp, nv, n_, osem, sm, p_.max_diff_range, p_.scaling_range);
    else
        k_normalize_weights<16><<<grid_for(n_), 256, 0, s>>>(wp, nv, n_, osem, sm, p_.max_diff_range,
                                                             p_.scaling_range);
    D_CUDA(cudaGetLastError());
    weights_dirty_ = false;
    return MVR_OK;
}

template <typename T>
int Decon<T>::set_psi(const float *psi, bool on_device)
{
    if (!psi) return fail(MVR_ERR_ARG, "psi must not be NULL");
    D_CUDA(cudaSetDevice(p_.device));
    cudaStream_t s = engine_.stream();
    if (sizeof(T) == sizeof(float)) {
        D_CUDA(cudaMemcpyAsync(psi_, psi, sizeof(float) * (size_t)n_,
                               on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
        return MVR_OK;
    }
    const float *src = psi;
    if (!on_device) {
        float *tmp = reinterpret_cast<float *>(stage_);
        D_CUDA(cudaMemcpyAsync(tmp, psi, sizeof(float) * (size_t)n_, cudaMemcpyHostToDevice, s));
        float *hold = nullptr;
        D_CUDA(cudaMalloc(&hold, sizeof(float) * (size_t)n_));
        D_CUDA(cudaMemcpyAsync(hold, tmp, sizeof(float) * (size_t)n_, cudaMemcpyDeviceToDevice, s));
        k_convert<float, T><<<grid_for(n_), 256, 0, s>>>(hold, psi_, n_);
        D_CUDA(cudaGetLastError());
        D_CUDA(cudaStreamSynchronize(s));
        cudaFree(hold);
        return MVR_OK;
    }
    k_convert<float, T><<<grid_for(n_), 256, 0, s>>>(src, psi_, n_);
    D_CUDA(cudaGetLastError());
    return MVR_OK;
}

template <typename T>
int Decon<T>::get_psi(float *psi)
{
    if (!psi) return fail(MVR_ERR_ARG, "psi must not be NULL");
    D_CUDA(cudaSetDevice(p_.device));
    cudaStream_t s = engine_.stream();
    if (sizeof(T) == sizeof(float)) {
        D_CUDA(cudaMemcpyAsync(psi, psi_, sizeof(float) * (size_t)n_, cudaMemcpyDeviceToHost, s));
    } else {
        float *tmp = reinterpret_cast<float *>(stage_);
        k_convert<T, float><<<grid_for(n_), 256, 0, s>>>(psi_, tmp, n_);
        D_CUDA(cudaGetLastError());
        D_CUDA(cudaMemcpyAsync(psi, tmp, sizeof(float) * (size_t)n_, cudaMemcpyDeviceToHost, s));
    }
    D_CUDA(cudaStreamSynchronize(s));
    return MVR_OK;
}

template <typename T>
int Decon<T>::get_psi_device(float *psi)
{
    if (!psi) return fail(MVR_ERR_ARG, "psi must not be NULL");
    D_CUDA(cudaSetDevice(p_.device));
    cudaStream_t s = engine_.stream();
    if (sizeof(T) == sizeof(float)) {
        D_CUDA(cudaMemcpyAsync(psi, psi_, sizeof(float) * (size_t)n_, cudaMemcpyDeviceToDevice, s));
    } else {
        k_convert<T, float><<<grid_for(n_), 256, 0, s>>>(psi_, psi, n_);
        D_CUDA(cudaGetLastError());
    }
    D_CUDA(cudaStreamSynchronize(s));
    return MVR_OK;
}

template <typename T>
int Decon<T>::get_kernels(int v, float *k1, float *k2)
{
    if (v < 0 || v >= p_.num_views || !prepared_) return fail(MVR_ERR_STATE, "not prepared or view out of range");
    const View &vw = views_[v];
    const size_t kn = (size_t)vw.kd[0] * vw.kd[1] * vw.kd[2];
    cudaStream_t s = engine_.stream();
    if (k1) D_CUDA(cudaMemcpyAsync(k1, vw.k1, sizeof(float) * kn, cudaMemcpyDeviceToHost, s));
    if (k2) D_CUDA(cudaMemcpyAsync(k2, vw.k2, sizeof(float) * kn, cudaMemcpyDeviceToHost, s));
    D_CUDA(cudaStreamSynchronize(s));
    return MVR_OK;
}

template <typename T>
int Decon<T>::get_max(float *mx)
{
    if (!prepared_ || !mx) return fail(MVR_ERR_STATE, "not prepared");
    std::memcpy(mx, max_.data(), sizeof(float) * max_.size());
    return MVR_OK;
}

template <typename T>
int Decon<T>::get_weights(int v, float *w)
{
    if (v < 0 || v >= p_.num_views || !prepared_ || !w) return fail(MVR_ERR_STATE, "not prepared or view out of range");
    if (weights_dirty_) D_TRY(normalize_weights());
    cudaStream_t s = engine_.stream();
    D_CUDA(cudaMemcpyAsync(w, views_[v].w, sizeof(float) * (size_t)n_, cudaMemcpyDeviceToHost, s));
    D_CUDA(cudaStreamSynchronize(s));
    return MVR_OK;
}

template <typename T>
int Decon<T>::synchronize()
{
    D_CUDA(cudaSetDevice(p_.device));
    D_CUDA(cudaStreamSynchronize(engine_.stream()));
    if (copy_) D_CUDA(cudaStreamSynchronize(copy_));
    return MVR_OK;
}

// One view-step (Seq) or one iteration (Mul): blocks in slab batches, each slab in
// launches of up to batch_ blocks.  trial: time-only run for the autotuner (psi is
// read, the staging volume written, nothing pasted or swapped).
template <typename T>
int Decon<T>::run_step(int st, double *stats_slot, bool trial, int batch)
{
    cudaStream_t s = engine_.stream();
    const std::vector<BlockDesc> &bl = blocks_[st];
    const long long D[3] = {p_.dims[0], p_.dims[1], p_.dims[2]};
    int nb = 0;
    for (const auto &b : bl) nb = std::max(nb, b.batch + 1);
    const bool jac = jacobi_[st] != 0;
    auto place = [&](const BlockDesc &b) {
        BlockPlace bp;
        bp.psi_src = psi_;
        bp.psi_dst = stage_;
        for (int d = 0; d < 3; ++d) {
            bp.D[d] = D[d];
            bp.off[d] = b.off[d];
            bp.OD[d] = D[d];
            bp.ooff[d] = b.off[d];
            bp.wlo[d] = b.eloc[d];
            bp.whi[d] = b.eloc[d] + b.esize[d];
        }
        return bp;
    };
    auto paste = [&](const BlockDesc &b) -> int {
        const long long nvx = (long long)b.esize[0] * b.esize[1] * b.esize[2];
        D_TRY(eng(engine_.prof_begin(KK_PASTE, 2.0 * sizeof(T) * (double)nvx)));
        k_paste<T><<<grid_for(nvx), 256, 0, s>>>(stage_, psi_, D[0], D[1], b.eoff[0], b.eoff[1], b.eoff[2], b.esize[0],
                                                 b.esize[1], b.esize[2]);
        D_TRY(cuda(cudaGetLastError(), "k_paste"));
        return eng(engine_.prof_end());
    };
    auto run_blocks = [&](const std::vector<const BlockDesc *> &grp, double *sd) -> int {
        std::vector<BlockPlace> bps;
        for (const BlockDesc *b : grp) bps.push_back(place(*b));
        if (!p_.mul) {
            const View &vw = views_[st];
            return eng(engine_.run_seq(vw.plan, bps.data(), (int)bps.size(), vw.img, vw.w, max_[st], sd));
        }
        std::vector<const Plan<T> *> pls;
        std::vector<const float *> imgs, ws;
        double miv = 0.0;
        for (auto &vw : views_) {
            pls.push_back(&vw.plan);
            imgs.push_back(vw.img);
            ws.push_back(vw.w);
        }
        for (float m : max_) miv += m;
        miv /= (double)max_.size();
        return eng(engine_.run_mul(pls, bps.data(), (int)bps.size(), imgs.data(), ws.data(), (float)miv, sd));
    };
    int slot = 0;
    std::vector<const BlockDesc *> prev;
    // Jacobi: every block reads psi before the step, so all slabs go out together
    const int nslabs = jac ? 1 : nb;
    for (int j = 0; j < nslabs; ++j) {
        std::vector<const BlockDesc *> cur;
        for (const auto &b : bl)
            if (jac || b.batch == j) cur.push_back(&b);
        for (size_t i0 = 0; i0 < cur.size(); i0 += (size_t)batch) {
            std::vector<const BlockDesc *> grp(cur.begin() + i0, cur.begin() + std::min(cur.size(), i0 + batch));
            D_TRY(run_blocks(grp, stats_slot ? stats_slot + 2 * slot : nullptr));
            slot += (int)grp.size();
        }
        if (!jac && !trial) {
            for (const BlockDesc *b : prev) D_TRY(paste(*b));
            prev = cur;
        }
    }
    if (trial) return MVR_OK;
    if (jac) std::swap(psi_, stage_);
    else
        for (const BlockDesc *b : prev) D_TRY(paste(*b));
    return MVR_OK;
}

// One iteration (all view-steps): replayed from a captured graph when one exists for
// the current state, captured when the previous iteration ran in the same state, else
// run eagerly.  With profiling on, every iteration runs eagerly (the profiler brackets
// launches with events).
template <typename T>
int Decon<T>::run_iteration(double *stats_base, size_t stats_stride)
{
    const int steps = num_steps();
    auto eager = [&]() -> int {
        for (int st = 0; st < steps; ++st)
            D_TRY(run_step(st, stats_base ? stats_base + (size_t)st * stats_stride : nullptr, false, batch_));
        return MVR_OK;
    };
    if (!graphs_on_ || engine_.profiling()) return eager();
    cudaStream_t s = engine_.stream();
    IterGraph key;
    key.psi_start = psi_;
    key.stats = stats_base;
    key.batch = batch_;
    key.epoch = engine_.alloc_epoch();
    key.inputs = inputs_epoch_;
    key.set = cur_set_;
    for (const auto &g : graphs_) {
        if (!g.same(key)) continue;
        D_CUDA(cudaGraphLaunch(g.exec, s));
        psi_ = g.psi_end;
        stage_ = g.stage_end;
        engine_.count_replayed(g.launches);
        return MVR_OK;
    }
    bool seen = false;
    for (const auto &k : seen_) seen = seen || k.same(key);
    if (!seen) {
        D_TRY(eager());
        if (seen_.size() >= 4) seen_.erase(seen_.begin());
        seen_.push_back(key);
        return MVR_OK;
    }
    // capture this iteration; the captured work runs when the graph is launched
    T *psi0 = psi_, *stage0 = stage_;
    const long long l0 = engine_.launches();
    D_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const int rc = eager();
    cudaGraph_t graph = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (rc != MVR_OK || ce != cudaSuccess || graph == nullptr) {
        if (graph) cudaGraphDestroy(graph);
        psi_ = psi0;
        stage_ = stage0;
        if (rc != MVR_OK) return rc;
        return cuda(ce == cudaSuccess ? cudaErrorStreamCaptureInvalidated : ce, "cudaStreamEndCapture");
    }
    key.psi_end = psi_;
    key.stage_end = stage_;
    key.launches = engine_.launches() - l0;
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
        psi_ = psi0;
        stage_ = stage0;
        return cuda(ie, "cudaGraphInstantiate");
    }
    key.exec = exec;
    if (graphs_.size() >= 8) {  // keep the most recent states
        cudaGraphExecDestroy(graphs_.front().exec);
        graphs_.erase(graphs_.begin());
    }
    graphs_.push_back(key);
    D_CUDA(cudaGraphLaunch(exec, s));
    return MVR_OK;
}

// The autotuner, at prepare: per view-step, the FFT schedule (row / column kernels, plane
// kernels with one CTA per plane or persistent, and the Z pass with the one-tile-per-CTA or the
// persistent double-buffered column kernel) that runs the step fastest at the largest batch;
// then the blocks per launch (1, 2, 4, 8, 16) with those schedules.  Every candidate runs the
// step twice (warm, then timed with CUDA events on the engine stream) as a trial that reads
// psi and writes only the staging volume.  A forced schedule (mvr_decon_set_schedule) or one
// of the environment switches MVR_PLANE_KERNELS / MVR_XY_PERSIST / MVR_COLS_PIPE skips the
// schedule search; a fixed batch_blocks skips the batch search.
namespace {
bool sched_env_forced()
{
    for (const char *v : {"MVR_PLANE_KERNELS", "MVR_XY_PERSIST", "MVR_COLS_PIPE"})
        if (std::getenv(v)) return true;
    return false;
}
}  // namespace

template <typename T>
int Decon<T>::autotune()
{
    size_t maxb = 1;
    for (auto &b : blocks_) maxb = std::max(maxb, b.size());
    const int cap = (int)std::min<size_t>(maxb, kMaxBatch);
    cudaStream_t s = engine_.stream();
    cudaEvent_t a, b;
    D_CUDA(cudaEventCreate(&a));
    const cudaError_t eb = cudaEventCreate(&b);
    if (eb != cudaSuccess) {
        cudaEventDestroy(a);
        D_CUDA(eb);
    }
    tune_.clear();
    auto time_step = [&](int st, int batch, float &ms) -> int {
        D_TRY(run_step(st, nullptr, true, batch));  // warm (allocates the batch's scratch)
        D_CUDA(cudaEventRecord(a, s));
        D_TRY(run_step(st, nullptr, true, batch));
        D_CUDA(cudaEventRecord(b, s));
        D_CUDA(cudaEventSynchronize(b));
        D_CUDA(cudaEventElapsedTime(&ms, a, b));
        return MVR_OK;
    };
    auto body = [&]() -> int {
        const int bt = p_.batch_blocks > 0 ? std::min(p_.batch_blocks, kMaxBatch) : cap;
        const bool env = sched_env_forced();
        for (int st = 0; st < num_steps(); ++st) {
            std::vector<View *> vs;
            if (p_.mul)
                for (auto &vw : views_) vs.push_back(&vw);
            else vs.push_back(&views_[st]);
            if (force_sched_ >= 0) {
                for (View *vw : vs) D_TRY(eng(engine_.set_schedule(vw->plan, force_sched_)));
                continue;
            }
            const std::vector<int> cands = engine_.schedule_candidates(vs[0]->plan);
            if (env || cands.size() <= 1 || blocks_[st].empty()) continue;
            float best = 1e30f;
            int bestc = engine_.schedule(vs[0]->plan);
            for (int c : cands) {
                for (View *vw : vs) D_TRY(eng(engine_.set_schedule(vw->plan, c)));
                float ms = 0.0f;
                D_TRY(time_step(st, bt, ms));
                tune_.push_back({st, c, bt, ms});
                if (ms < best) {
                    best = ms;
                    bestc = c;
                }
            }
            for (View *vw : vs) D_TRY(eng(engine_.set_schedule(vw->plan, bestc)));
        }
        if (p_.batch_blocks > 0) {
            batch_ = std::min(p_.batch_blocks, kMaxBatch);
            return MVR_OK;
        }
        batch_ = 1;
        if (cap <= 1 || !jacobi_[0]) return MVR_OK;
        float best = 1e30f;
        for (int cand = 1; cand <= cap; cand *= 2) {
            float ms = 0.0f;
            D_TRY(time_step(0, cand, ms));
            tune_.push_back({-1, -1, cand, ms});
            if (ms < best) {
                best = ms;
                batch_ = cand;
            }
        }
        return MVR_OK;
    };
    const int rc = body();
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return rc;
}

template <typename T>
int Decon<T>::set_schedule(int code)
{
    if (code < -1 || code > (SCHED_PAIR | SCHED_ZPIPE))
        return fail(MVR_ERR_ARG, "unknown FFT schedule code");
    force_sched_ = code;
    prepared_ = false;
    return MVR_OK;
}

template <typename T>
int Decon<T>::schedule(int view) const
{
    if (view < 0 || view >= p_.num_views) return -MVR_ERR_ARG;
    return engine_.schedule(views_[view].plan);
}

template <typename T>
int Decon<T>::tuning(int capacity, int *step, int *code, int *batch, float *ms) const
{
    const int n = (int)tune_.size();
    for (int i = 0; i < n && i < capacity; ++i) {
        if (step) step[i] = tune_[i].step;
        if (code) code[i] = tune_[i].code;
        if (batch) batch[i] = tune_[i].batch;
        if (ms) ms[i] = tune_[i].ms;
    }
    return n;
}

// runIterations with host-resident inputs (MultiViewDeconvolution.runIterations on images,
// raw weights and psi held by the caller): the uploads go out on a copy stream in the order
// weights, psi, image 0, 1, ...; the weight normalisation waits for the weights and psi, and
// view-step v of the first iteration for image v, so the image uploads overlap the first
// view-steps.  psi comes back at the end.  With page-locked host buffers the copies run
// asynchronously to the host; pageable buffers work but may serialise them.
template <typename T>
int Decon<T>::run_host(int iterations, const float *const *imgs, const float *const *ws, float *psi,
                       const float *const *next_imgs, const float *const *next_ws)
{
    if (!prepared_) return fail(MVR_ERR_STATE, "mvr_decon_prepare was not called");
    if (!imgs || !ws || !psi || iterations < 1) return fail(MVR_ERR_ARG, "inputs must not be NULL, iterations >= 1");
    if ((next_imgs == nullptr) != (next_ws == nullptr))
        return fail(MVR_ERR_ARG, "next images and next weights: both or neither");
    const int nv = p_.num_views;
    for (int v = 0; v < nv; ++v) {
        if (!imgs[v] || !ws[v]) return fail(MVR_ERR_ARG, "image and weight pointers must not be NULL");
        if (next_imgs && (!next_imgs[v] || !next_ws[v]))
            return fail(MVR_ERR_ARG, "next image and weight pointers must not be NULL");
        if (!views_[v].own_img || !views_[v].own_w)
            return fail(MVR_ERR_STATE, "mvr_decon_run_host needs views set with mvr_decon_set_view (host arrays)");
    }
    D_CUDA(cudaSetDevice(p_.device));
    cudaStream_t s = engine_.stream();
    if (!copy_) D_CUDA(cudaStreamCreateWithFlags(&copy_, cudaStreamNonBlocking));
    if (!ev_w_) D_CUDA(cudaEventCreateWithFlags(&ev_w_, cudaEventDisableTiming));
    if (!ev_pre_) D_CUDA(cudaEventCreateWithFlags(&ev_pre_, cudaEventDisableTiming));
    while ((int)ev_img_.size() < nv) {
        cudaEvent_t e = nullptr;
        D_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ev_img_.push_back(e);
    }
    const size_t bytes = sizeof(float) * (size_t)n_;
    // this call's images and weights were uploaded by the previous call when it was given
    // the same host arrays as its next ones
    bool pre = pre_valid_;
    for (int v = 0; pre && v < nv; ++v) pre = imgs[v] == pre_img_[v] && ws[v] == pre_w_[v];
    pre_valid_ = false;
    // the copy stream starts after the work already queued on the compute stream (earlier
    // iterations still read the buffers it overwrites)
    D_CUDA(cudaEventRecord(ev_w_, s));
    D_CUDA(cudaStreamWaitEvent(copy_, ev_w_, 0));
    if (pre) {
        for (int v = 0; v < nv; ++v) {
            std::swap(views_[v].img, alt_img_[v]);
            std::swap(views_[v].w_raw, alt_w_[v]);
            if (p_.weight_norm == MVR_WEIGHTS_AS_GIVEN) views_[v].w = views_[v].w_raw;
        }
        cur_set_ ^= 1;  // captured iterations are kept per set
        D_CUDA(cudaStreamWaitEvent(s, ev_pre_, 0));
    } else {
        for (int v = 0; v < nv; ++v)
            D_CUDA(cudaMemcpyAsync(views_[v].w_raw, ws[v], bytes, cudaMemcpyHostToDevice, copy_));
    }
    float *psi_up = sizeof(T) == sizeof(float) ? reinterpret_cast<float *>(psi_) : reinterpret_cast<float *>(stage_);
    D_CUDA(cudaMemcpyAsync(psi_up, psi, bytes, cudaMemcpyHostToDevice, copy_));
    D_CUDA(cudaEventRecord(ev_w_, copy_));
    if (!pre) {
        for (int v = 0; v < nv; ++v) {
            D_CUDA(cudaMemcpyAsync(views_[v].img, imgs[v], bytes, cudaMemcpyHostToDevice, copy_));
            D_CUDA(cudaEventRecord(ev_img_[v], copy_));
        }
    }
    if (next_imgs) {
        // the next call's inputs into the second set, behind this call's uploads on the copy
        // stream and concurrent with this call's iterations (the second set's last reader was
        // the previous call, which has returned)
        if (alt_img_.empty()) {
            alt_img_.assign(nv, nullptr);
            alt_w_.assign(nv, nullptr);
            for (int v = 0; v < nv; ++v) {
                D_CUDA(cudaMalloc(&alt_img_[v], bytes));
                D_CUDA(cudaMalloc(&alt_w_[v], bytes));
            }
        }
        for (int v = 0; v < nv; ++v) {
            D_CUDA(cudaMemcpyAsync(alt_w_[v], next_ws[v], bytes, cudaMemcpyHostToDevice, copy_));
            D_CUDA(cudaMemcpyAsync(alt_img_[v], next_imgs[v], bytes, cudaMemcpyHostToDevice, copy_));
        }
        D_CUDA(cudaEventRecord(ev_pre_, copy_));
        pre_img_.assign(next_imgs, next_imgs + nv);
        pre_w_.assign(next_ws, next_ws + nv);
        pre_valid_ = true;
    }
    // prefetched raw weights are already on the device (the compute stream waited for the
    // second set above): normalise them while psi is still uploading
    const bool norm = p_.weight_norm != MVR_WEIGHTS_AS_GIVEN;
    if (pre && norm) D_TRY(normalize_weights());
    D_CUDA(cudaStreamWaitEvent(s, ev_w_, 0));
    if (sizeof(T) != sizeof(float)) {
        // FP64 run: the uploaded float psi (in the staging volume) converted into psi
        float *hold = nullptr;
        D_CUDA(cudaMalloc(&hold, bytes));
        D_CUDA(cudaMemcpyAsync(hold, psi_up, bytes, cudaMemcpyDeviceToDevice, s));
        k_convert<float, T><<<grid_for(n_), 256, 0, s>>>(hold, psi_, n_);
        D_CUDA(cudaGetLastError());
        D_CUDA(cudaStreamSynchronize(s));
        cudaFree(hold);
    }
    if (!pre && norm) D_TRY(normalize_weights());
    int it = 0;
    if (!pre) {
        // the first iteration eagerly, each view-step after its image
        const int steps = num_steps();
        for (int st = 0; st < steps; ++st) {
            if (p_.mul)
                for (int v = 0; v < nv; ++v) D_CUDA(cudaStreamWaitEvent(s, ev_img_[v], 0));
            else D_CUDA(cudaStreamWaitEvent(s, ev_img_[st], 0));
            D_TRY(run_step(st, nullptr, false, batch_));
        }
        it = 1;
    }
    // (with every input already on the device, all iterations take the captured-graph path)
    for (; it < iterations; ++it) D_TRY(run_iteration(nullptr, 0));
    return get_psi(psi);
}

template <typename T>
int Decon<T>::run(int iterations, double *stats)
{
    if (!prepared_) return fail(MVR_ERR_STATE, "mvr_decon_prepare was not called");
    if (iterations < 0) return fail(MVR_ERR_ARG, "iterations must be >= 0");
    D_CUDA(cudaSetDevice(p_.device));
    if (weights_dirty_) D_TRY(normalize_weights());
    const int steps = num_steps();
    size_t maxb = 1;
    for (auto &b : blocks_) maxb = std::max(maxb, b.size());
    const long long need = (long long)steps * (long long)maxb * 2;
    if (stats && need > stats_cap_) {
        cudaFree(d_stats_);
        d_stats_ = nullptr;
        stats_cap_ = 0;
        D_CUDA(cudaMalloc(&d_stats_, sizeof(double) * (size_t)need));
        stats_cap_ = need;
    }
    std::vector<double> hs;
    for (int it = 0; it < iterations; ++it) {
        D_TRY(run_iteration(stats ? d_stats_ : nullptr, maxb * 2));
        if (stats) {
            hs.resize((size_t)need);
            D_CUDA(cudaMemcpyAsync(hs.data(), d_stats_, sizeof(double) * (size_t)need, cudaMemcpyDeviceToHost,
                                   engine_.stream()));
            D_CUDA(cudaStreamSynchronize(engine_.stream()));
            for (int st = 0; st < steps; ++st) {
                double sum = 0.0, mx = -1.0;
                for (size_t b = 0; b < blocks_[st].size(); ++b) {
                    sum += hs[((size_t)st * maxb + b) * 2];
                    mx = std::max(mx, hs[((size_t)st * maxb + b) * 2 + 1]);
                }
                stats[((size_t)it * steps + st) * 2] = sum;
                stats[((size_t)it * steps + st) * 2 + 1] = mx;
            }
        }
    }
    return MVR_OK;
}

// Poisson negative log-likelihood of the current psi, summed over views in FP64:
// sum_v sum_x w_v (conv1_v - img_v ln conv1_v) over img_v > 0 (each voxel once).
template <typename T>
int Decon<T>::likelihood(double *total, double *per_view)
{
    if (!prepared_) return fail(MVR_ERR_STATE, "mvr_decon_prepare was not called");
    D_CUDA(cudaSetDevice(p_.device));
    if (weights_dirty_) D_TRY(normalize_weights());
    cudaStream_t s = engine_.stream();
    const long long D[3] = {p_.dims[0], p_.dims[1], p_.dims[2]};
    size_t maxb = 1;
    for (auto &b : blocks_) maxb = std::max(maxb, b.size());
    const long long need = (long long)p_.num_views * (long long)maxb * 2;
    if (need > stats_cap_) {
        cudaFree(d_stats_);
        d_stats_ = nullptr;
        stats_cap_ = 0;
        D_CUDA(cudaMalloc(&d_stats_, sizeof(double) * (size_t)need));
        stats_cap_ = need;
    }
    for (int v = 0; v < p_.num_views; ++v) {
        const std::vector<BlockDesc> &bl = blocks_[p_.mul ? 0 : v];
        const View &vw = views_[v];
        for (size_t i0 = 0; i0 < bl.size(); i0 += (size_t)batch_) {
            std::vector<BlockPlace> bps;
            for (size_t i = i0; i < std::min(bl.size(), i0 + (size_t)batch_); ++i) {
                const BlockDesc &b = bl[i];
                BlockPlace bp;
                bp.psi_src = psi_;
                for (int d = 0; d < 3; ++d) {
                    bp.D[d] = D[d];
                    bp.off[d] = b.off[d];
                    bp.OD[d] = D[d];
                    bp.ooff[d] = b.off[d];
                    bp.wlo[d] = b.eloc[d];
                    bp.whi[d] = b.eloc[d] + b.esize[d];
                }
                bps.push_back(bp);
            }
            D_TRY(eng(engine_.likelihood(vw.plan, bps.data(), (int)bps.size(), vw.img, vw.w,
                                         d_stats_ + ((size_t)v * maxb + i0) * 2)));
        }
    }
    std::vector<double> hs((size_t)need);
    D_CUDA(cudaMemcpyAsync(hs.data(), d_stats_, sizeof(double) * (size_t)need, cudaMemcpyDeviceToHost, s));
    D_CUDA(cudaStreamSynchronize(s));
    double tot = 0.0;
    for (int v = 0; v < p_.num_views; ++v) {
        double sv = 0.0;
        for (size_t b = 0; b < blocks_[p_.mul ? 0 : v].size(); ++b) sv += hs[((size_t)v * maxb + b) * 2];
        if (per_view) per_view[v] = sv;
        tot += sv;
    }
    if (total) *total = tot;
    return MVR_OK;
}

template class Decon<float>;
template class Decon<double>;

}  // namespace mvr

// ---- C ABI ---------------------------------------------------------------------------
struct mvr_decon {
    std::unique_ptr<mvr::DeconBase> impl;
};

namespace {
thread_local std::string g_decon_create_error;
}

extern "C" int mvr_decon_create(const mvr_decon_params *p, mvr_decon **out)
{
    if (!out) return MVR_ERR_ARG;
    *out = nullptr;
    if (!p) {
        g_decon_create_error = "params is NULL";
        return MVR_ERR_ARG;
    }
    std::unique_ptr<mvr_decon> h(new mvr_decon());
    int rc;
    if (p->precision == MVR_PRECISION_FP64) {
        auto *d = new mvr::Decon<double>(*p);
        h->impl.reset(d);
        rc = d->init();
    } else if (p->precision == MVR_PRECISION_FP32) {
        auto *d = new mvr::Decon<float>(*p);
        h->impl.reset(d);
        rc = d->init();
    } else {
        g_decon_create_error = "unknown precision";
        return MVR_ERR_ARG;
    }
    if (rc != MVR_OK) {
        g_decon_create_error = h->impl->error();
        return rc;
    }
    *out = h.release();
    return MVR_OK;
}

extern "C" void mvr_decon_destroy(mvr_decon *h) { delete h; }

extern "C" const char *mvr_decon_last_error(const mvr_decon *h)
{
    return h ? h->impl->error().c_str() : g_decon_create_error.c_str();
}

extern "C" int mvr_decon_set_view(mvr_decon *h, int view, const float *img, const float *weight, const float *psf,
                                  const int psf_size[3])
{
    if (!h) return MVR_ERR_ARG;
    int rc = h->impl->set_images(view, img, weight, false);
    return rc != MVR_OK ? rc : h->impl->set_psf(view, psf, psf_size);
}

extern "C" int mvr_decon_set_view_device(mvr_decon *h, int view, const float *img, const float *weight,
                                         const float *psf, const int psf_size[3])
{
    if (!h) return MVR_ERR_ARG;
    int rc = h->impl->set_images(view, img, weight, true);
    return rc != MVR_OK ? rc : h->impl->set_psf(view, psf, psf_size);
}

extern "C" int mvr_decon_run_host_next(mvr_decon *h, int iterations, const float *const *images,
                                       const float *const *weights, float *psi, const float *const *next_images,
                                       const float *const *next_weights)
{
    return h ? h->impl->run_host(iterations, images, weights, psi, next_images, next_weights) : MVR_ERR_ARG;
}

extern "C" int mvr_decon_run_host(mvr_decon *h, int iterations, const float *const *imgs, const float *const *weights,
                                  float *psi)
{
    return h ? h->impl->run_host(iterations, imgs, weights, psi, nullptr, nullptr) : MVR_ERR_ARG;
}

extern "C" int mvr_decon_set_schedule(mvr_decon *h, int code)
{
    return h ? h->impl->set_schedule(code) : MVR_ERR_ARG;
}

extern "C" int mvr_decon_schedule(const mvr_decon *h, int view)
{
    return h ? h->impl->schedule(view) : -MVR_ERR_ARG;
}

extern "C" int mvr_decon_tuning(const mvr_decon *h, int capacity, int *step, int *code, int *batch, float *ms)
{
    if (!h || capacity < 0) return -MVR_ERR_ARG;
    return h->impl->tuning(capacity, step, code, batch, ms);
}

extern "C" int mvr_decon_set_view_block_size(mvr_decon *h, int view, const int block_size[3])
{
    return h ? h->impl->set_view_block(view, block_size) : MVR_ERR_ARG;
}

extern "C" int mvr_decon_set_effective_block_size(mvr_decon *h, int view, const int effective[3])
{
    return h ? h->impl->set_view_effective(view, effective) : MVR_ERR_ARG;
}

extern "C" int mvr_decon_update_images(mvr_decon *h, int view, const float *img, const float *weight)
{
    return h ? h->impl->set_images(view, img, weight, false) : MVR_ERR_ARG;
}

extern "C" int mvr_decon_prepare(mvr_decon *h) { return h ? h->impl->prepare() : MVR_ERR_ARG; }
extern "C" int mvr_decon_set_psi(mvr_decon *h, const float *psi) { return h ? h->impl->set_psi(psi, false) : MVR_ERR_ARG; }
extern "C" int mvr_decon_set_psi_device(mvr_decon *h, const float *psi)
{
    return h ? h->impl->set_psi(psi, true) : MVR_ERR_ARG;
}
extern "C" int mvr_decon_get_psi(mvr_decon *h, float *psi) { return h ? h->impl->get_psi(psi) : MVR_ERR_ARG; }
extern "C" int mvr_decon_get_psi_device(mvr_decon *h, float *psi)
{
    return h ? h->impl->get_psi_device(psi) : MVR_ERR_ARG;
}
extern "C" int mvr_decon_run(mvr_decon *h, int iterations, double *stats)
{
    return h ? h->impl->run(iterations, stats) : MVR_ERR_ARG;
}
extern "C" int mvr_decon_get_kernels(mvr_decon *h, int view, float *k1, float *k2)
{
    return h ? h->impl->get_kernels(view, k1, k2) : MVR_ERR_ARG;
}
extern "C" int mvr_decon_get_max(mvr_decon *h, float *mx) { return h ? h->impl->get_max(mx) : MVR_ERR_ARG; }
extern "C" int mvr_decon_get_weights(mvr_decon *h, int view, float *w)
{
    return h ? h->impl->get_weights(view, w) : MVR_ERR_ARG;
}
extern "C" const void *mvr_decon_psi_device(const mvr_decon *h) { return h ? h->impl->psi_device() : nullptr; }
extern "C" int mvr_decon_synchronize(mvr_decon *h) { return h ? h->impl->synchronize() : MVR_ERR_ARG; }

extern "C" void *mvr_decon_stream(mvr_decon *h) { return h ? h->impl->stream() : nullptr; }
extern "C" long long mvr_decon_launch_count(const mvr_decon *h) { return h ? h->impl->launches() : -1; }
extern "C" int mvr_decon_set_profiling(mvr_decon *h, int on)
{
    if (!h) return MVR_ERR_ARG;
    h->impl->set_profiling(on != 0);
    return MVR_OK;
}
extern "C" int mvr_decon_get_profile(mvr_decon *h, double *ms, long long *launches, double *bytes)
{
    if (!h) return MVR_ERR_ARG;
    mvr::KernelProfile p{};
    const int rc = h->impl->profile(p);
    if (rc != MVR_OK) return rc;
    for (int k = 0; k < mvr::KK_COUNT; ++k) {
        if (ms) ms[k] = p.ms[k];
        if (launches) launches[k] = p.launches[k];
        if (bytes) bytes[k] = p.bytes[k];
    }
    return MVR_OK;
}
extern "C" const char *mvr_kernel_name(int kind) { return mvr::kernel_kind_name(kind); }
extern "C" int mvr_decon_batch(const mvr_decon *h) { return h ? h->impl->batch() : -1; }
extern "C" int mvr_decon_set_graphs(mvr_decon *h, int on) { return h ? h->impl->set_graphs(on != 0) : MVR_ERR_ARG; }
extern "C" int mvr_decon_graphs_captured(const mvr_decon *h) { return h ? h->impl->graphs_captured() : -1; }
extern "C" int mvr_decon_init_psi(mvr_decon *h, int method, double sigma, double *avg)
{
    return h ? h->impl->psi_init(method, sigma, avg) : MVR_ERR_ARG;
}
extern "C" int mvr_decon_likelihood(mvr_decon *h, double *total, double *per_view)
{
    return h ? h->impl->likelihood(total, per_view) : MVR_ERR_ARG;
}

// BlockGeneratorFixedSizePrecise.divideIntoBlocks (MV/cuda/BlockGeneratorFixedSizePrecise.java:
// 59-131) with the doubled kernel 2k-1 of DeconView (MV/deconvolution/DeconView.java:155-157)
// and BlockSorter's slab dimension (MV/cuda/BlockSorter.java:55-143): host arithmetic only.
extern "C" MVR_API int mvr_block_grid(const long long dims[3], const int kernel_size[3], const int block_size[3],
                                      int min_required, long long *blocks, int capacity, int *sort_dim)
{
    if (!dims || !kernel_size || !block_size || capacity < 0 || (capacity > 0 && !blocks)) return -MVR_ERR_ARG;
    long long D[3];
    int kk[3];
    for (int d = 0; d < 3; ++d) {
        if (dims[d] < 1 || kernel_size[d] < 1 || block_size[d] < 1) return -MVR_ERR_ARG;
        D[d] = dims[d];
        kk[d] = 2 * kernel_size[d] - 1;
    }
    std::vector<mvr::BlockDesc> all;
    int sd = 2;
    if (!mvr::divide_blocks(D, kk, block_size, all, sd, min_required < 1 ? 1 : min_required)) return -MVR_ERR_ARG;
    if (sort_dim) *sort_dim = sd;
    for (size_t i = 0; i < all.size() && (long long)i < capacity; ++i)
        for (int d = 0; d < 3; ++d) {
            blocks[12 * i + d] = all[i].off[d];
            blocks[12 * i + 3 + d] = all[i].eoff[d];
            blocks[12 * i + 6 + d] = all[i].esize[d];
            blocks[12 * i + 9 + d] = all[i].eloc[d];
        }
    return (int)all.size();
}
