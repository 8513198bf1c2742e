// extern "C" entry points of the block worker and of the reference's JNA library
// (declared in include/mvr_gb300.h).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/mvr_gb300.h"
#include "engine.cuh"

using mvr::Engine;
using mvr::Plan;

namespace {
thread_local std::string g_create_error;

// Host <-> device copies of the block buffers.  A block buffer of the Java driver (or any
// caller) is ordinary pageable memory that changes from call to call; a DMA copy of it first
// pins every page, which for freshly allocated buffers costs more than the transfer.  Where
// the GPU reads and writes pageable host memory through the host's page tables
// (cudaDevAttrPageableMemoryAccessUsesHostPageTables, e.g. NVLink-C2C systems), a copy kernel
// moves the buffer instead; elsewhere cudaMemcpyAsync.  MVR_HOST_COPY=dma forces the DMA copy.
__global__ void k_copy_words(float4 *__restrict__ dst, const float4 *__restrict__ src, long long n4)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n4; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}
__global__ void k_copy_floats(float *__restrict__ dst, const float *__restrict__ src, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

bool kernel_host_copy(int dev)
{
    static int cached[64] = {0};  // 0 unknown, 1 kernel, 2 DMA
    if (dev < 0 || dev >= 64) return false;
    if (!cached[dev]) {
        const char *e = std::getenv("MVR_HOST_COPY");
        int ht = 0;
        if (cudaDeviceGetAttribute(&ht, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) != cudaSuccess) ht = 0;
        cached[dev] = (ht == 1 && !(e && std::strcmp(e, "dma") == 0)) ? 1 : 2;
    }
    return cached[dev] == 1;
}

cudaError_t host_copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, int dev, cudaStream_t s)
{
    if (!kernel_host_copy(dev)) return cudaMemcpyAsync(dst, src, bytes, kind, s);
    const bool vec = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src) | bytes) & 15) == 0;
    if (vec)
        k_copy_words<<<608, 256, 0, s>>>(static_cast<float4 *>(dst), static_cast<const float4 *>(src),
                                         (long long)(bytes / 16));
    else
        k_copy_floats<<<608, 256, 0, s>>>(static_cast<float *>(dst), static_cast<const float *>(src),
                                          (long long)(bytes / 4));
    return cudaGetLastError();
}
}  // namespace

struct mvr_block {
    Engine<float> eng;
    int b[3] = {0, 0, 0};
    long long nvox = 0;
    int nviews = 1;
    std::vector<Plan<float>> plans;
    float *d_psi = nullptr;
    std::vector<float *> d_img, d_w;
    double *d_stats = nullptr;
    std::string err;

    ~mvr_block()
    {
        cudaSetDevice(eng.device() >= 0 ? eng.device() : 0);
        for (auto &p : plans) eng.free_plan(p);
        cudaFree(d_psi);
        for (float *p : d_img) cudaFree(p);
        for (float *p : d_w) cudaFree(p);
        cudaFree(d_stats);
    }
    int fail(int code, const std::string &m)
    {
        err = m;
        return code;
    }
    int from_engine(int rc)
    {
        if (rc != MVR_OK) err = eng.error();
        return rc;
    }
    int cuda(cudaError_t e, const char *what)
    {
        if (e == cudaSuccess) return MVR_OK;
        err = std::string(what) + ": " + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? MVR_ERR_OOM : MVR_ERR_CUDA;
    }
};

#define BLK_CUDA(h, expr)                              \
    do {                                               \
        int rc__ = (h)->cuda((expr), #expr);           \
        if (rc__ != MVR_OK) return rc__;               \
    } while (0)

extern "C" int mvr_block_create(const mvr_block_params *p, mvr_block **out)
{
    if (!out) return MVR_ERR_ARG;
    *out = nullptr;
    if (!p) {
        g_create_error = "params is NULL";
        return MVR_ERR_ARG;
    }
    for (int d = 0; d < 3; ++d)
        if (p->block_size[d] < 1) {
            g_create_error = "block_size must be >= 1";
            return MVR_ERR_ARG;
        }
    if (p->num_views < 1 || p->num_views > mvr::kMaxViews) {
        g_create_error = "num_views must be 1..16";
        return MVR_ERR_ARG;
    }
    if (p->boundary != MVR_BOUNDARY_REFERENCE && p->boundary != MVR_BOUNDARY_CIRCULAR) {
        g_create_error = "unknown boundary";
        return MVR_ERR_ARG;
    }
    std::unique_ptr<mvr_block> h(new mvr_block());
    int rc = h->eng.init(p->device, p->boundary, (double)p->lambda, p->min_value);
    if (rc != MVR_OK) {
        g_create_error = h->eng.error();
        return rc;
    }
    for (int d = 0; d < 3; ++d) h->b[d] = p->block_size[d];
    h->nvox = (long long)h->b[0] * h->b[1] * h->b[2];
    h->nviews = p->num_views;
    h->plans.resize(p->num_views);
    h->d_img.assign(p->num_views, nullptr);
    h->d_w.assign(p->num_views, nullptr);
    const size_t bytes = sizeof(float) * (size_t)h->nvox;
    cudaError_t e = cudaMalloc(&h->d_psi, bytes);
    for (int v = 0; v < p->num_views && e == cudaSuccess; ++v) {
        e = cudaMalloc(&h->d_img[v], bytes);
        if (e == cudaSuccess) e = cudaMalloc(&h->d_w[v], bytes);
    }
    if (e == cudaSuccess) e = cudaMalloc(&h->d_stats, 2 * sizeof(double));
    if (e != cudaSuccess) {
        g_create_error = std::string("device allocation: ") + cudaGetErrorString(e);
        return e == cudaErrorMemoryAllocation ? MVR_ERR_OOM : MVR_ERR_CUDA;
    }
    *out = h.release();
    return MVR_OK;
}

extern "C" void mvr_block_destroy(mvr_block *h) { delete h; }

extern "C" const char *mvr_block_last_error(const mvr_block *h)
{
    return h ? h->err.c_str() : g_create_error.c_str();
}

extern "C" int mvr_block_set_kernels(mvr_block *h, int view, const float *k1, const float *k2, const int ks[3])
{
    if (!h) return MVR_ERR_ARG;
    if (view < 0 || view >= h->nviews) return h->fail(MVR_ERR_ARG, "view out of range");
    if (!k1 || !k2 || !ks) return h->fail(MVR_ERR_ARG, "kernel pointers must not be NULL");
    BLK_CUDA(h, cudaSetDevice(h->eng.device()));
    return h->from_engine(h->eng.make_plan(h->plans[view], h->b, k1, ks, k2, ks));
}

static int run_seq_impl(mvr_block *h, int view, const float *psi_src, float *psi_dst, const float *img,
                        const float *w, float maxI, double *stats_dev)
{
    mvr::BlockPlace bp;
    bp.psi_src = psi_src;
    bp.psi_dst = psi_dst;
    for (int d = 0; d < 3; ++d) {
        bp.D[d] = h->b[d];
        bp.OD[d] = h->b[d];
        bp.whi[d] = h->b[d];
    }
    return h->from_engine(h->eng.run_seq(h->plans[view], &bp, 1, img, w, maxI, stats_dev));
}

extern "C" int mvr_block_run_seq(mvr_block *h, int view, float *psi, const float *img, const float *w, float maxI,
                                 double stats[2])
{
    if (!h) return MVR_ERR_ARG;
    if (view < 0 || view >= h->nviews) return h->fail(MVR_ERR_ARG, "view out of range");
    if (!psi || !img || !w) return h->fail(MVR_ERR_ARG, "block pointers must not be NULL");
    if (!h->plans[view].k1h) return h->fail(MVR_ERR_STATE, "mvr_block_set_kernels was not called for this view");
    BLK_CUDA(h, cudaSetDevice(h->eng.device()));
    cudaStream_t s = h->eng.stream();
    const size_t bytes = sizeof(float) * (size_t)h->nvox;
    const int dev = h->eng.device();
    BLK_CUDA(h, host_copy(h->d_psi, psi, bytes, cudaMemcpyHostToDevice, dev, s));
    BLK_CUDA(h, host_copy(h->d_img[0], img, bytes, cudaMemcpyHostToDevice, dev, s));
    BLK_CUDA(h, host_copy(h->d_w[0], w, bytes, cudaMemcpyHostToDevice, dev, s));
    int rc = run_seq_impl(h, view, h->d_psi, h->d_psi, h->d_img[0], h->d_w[0], maxI, h->d_stats);
    if (rc != MVR_OK) return rc;
    BLK_CUDA(h, host_copy(psi, h->d_psi, bytes, cudaMemcpyDeviceToHost, dev, s));
    double st[2] = {0.0, -1.0};
    BLK_CUDA(h, cudaMemcpyAsync(st, h->d_stats, sizeof(st), cudaMemcpyDeviceToHost, s));
    BLK_CUDA(h, cudaStreamSynchronize(s));
    if (stats) {
        stats[0] = st[0];
        stats[1] = st[1];
    }
    return MVR_OK;
}

extern "C" int mvr_block_run_seq_device(mvr_block *h, int view, float *psi, const float *img, const float *w,
                                        float maxI, double *stats_dev)
{
    if (!h) return MVR_ERR_ARG;
    if (view < 0 || view >= h->nviews) return h->fail(MVR_ERR_ARG, "view out of range");
    if (!psi || !img || !w) return h->fail(MVR_ERR_ARG, "block pointers must not be NULL");
    if (!h->plans[view].k1h) return h->fail(MVR_ERR_STATE, "mvr_block_set_kernels was not called for this view");
    BLK_CUDA(h, cudaSetDevice(h->eng.device()));
    return run_seq_impl(h, view, psi, psi, img, w, maxI, stats_dev);
}

extern "C" int mvr_block_synchronize(mvr_block *h)
{
    if (!h) return MVR_ERR_ARG;
    BLK_CUDA(h, cudaSetDevice(h->eng.device()));
    BLK_CUDA(h, cudaStreamSynchronize(h->eng.stream()));
    return MVR_OK;
}

extern "C" int mvr_block_run_mul(mvr_block *h, float *psi, const float *const *imgs, const float *const *ws,
                                 const float *maxIs, double stats[2])
{
    if (!h) return MVR_ERR_ARG;
    if (!psi || !imgs || !ws || !maxIs) return h->fail(MVR_ERR_ARG, "pointers must not be NULL");
    std::vector<const Plan<float> *> pls;
    for (int v = 0; v < h->nviews; ++v) {
        if (!imgs[v] || !ws[v]) return h->fail(MVR_ERR_ARG, "block pointers must not be NULL");
        if (!h->plans[v].k1h) return h->fail(MVR_ERR_STATE, "mvr_block_set_kernels was not called for every view");
        pls.push_back(&h->plans[v]);
    }
    BLK_CUDA(h, cudaSetDevice(h->eng.device()));
    cudaStream_t s = h->eng.stream();
    const size_t bytes = sizeof(float) * (size_t)h->nvox;
    const int dev = h->eng.device();
    BLK_CUDA(h, host_copy(h->d_psi, psi, bytes, cudaMemcpyHostToDevice, dev, s));
    for (int v = 0; v < h->nviews; ++v) {
        BLK_CUDA(h, host_copy(h->d_img[v], imgs[v], bytes, cudaMemcpyHostToDevice, dev, s));
        BLK_CUDA(h, host_copy(h->d_w[v], ws[v], bytes, cudaMemcpyHostToDevice, dev, s));
    }
    // ComputeBlockMulThreadCPU.java:144-149: mean of the maxima in double, then float
    double miv = 0.0;
    for (int v = 0; v < h->nviews; ++v) miv += maxIs[v];
    miv /= (double)h->nviews;
    mvr::BlockPlace bp;
    bp.psi_src = h->d_psi;
    bp.psi_dst = h->d_psi;
    for (int d = 0; d < 3; ++d) {
        bp.D[d] = h->b[d];
        bp.OD[d] = h->b[d];
        bp.whi[d] = h->b[d];
    }
    std::vector<const float *> di(h->d_img.begin(), h->d_img.end()), dw(h->d_w.begin(), h->d_w.end());
    int rc = h->from_engine(h->eng.run_mul(pls, &bp, 1, di.data(), dw.data(), (float)miv, h->d_stats));
    if (rc != MVR_OK) return rc;
    BLK_CUDA(h, host_copy(psi, h->d_psi, bytes, cudaMemcpyDeviceToHost, dev, s));
    double st[2] = {0.0, -1.0};
    BLK_CUDA(h, cudaMemcpyAsync(st, h->d_stats, sizeof(st), cudaMemcpyDeviceToHost, s));
    BLK_CUDA(h, cudaStreamSynchronize(s));
    if (stats) {
        stats[0] = st[0];
        stats[1] = st[1];
    }
    return MVR_OK;
}

// ---- the reference's JNA library ----------------------------------------------------
namespace {
struct ConvCache {  // one engine per device, plans keyed by (image, kernel) sizes
    std::unique_ptr<Engine<float>> eng;
    std::map<std::tuple<int, int, int, int, int, int>, std::unique_ptr<Plan<float>>> plans;
    float *d_img = nullptr;
    float *d_out = nullptr;
    long long cap = 0;
};
std::mutex g_conv_mutex;
std::map<int, ConvCache> g_conv;

int conv3d(float *im, const int *imDim, const float *kernel, const int *kernelDim, int dev, float *out)
{
    if (!im || !imDim || !kernel || !kernelDim || !out) return MVR_ERR_ARG;
    // reversed dimensions: {z, y, x}
    const int b[3] = {imDim[2], imDim[1], imDim[0]};
    const int kd[3] = {kernelDim[2], kernelDim[1], kernelDim[0]};
    std::lock_guard<std::mutex> lock(g_conv_mutex);
    ConvCache &c = g_conv[dev];
    if (!c.eng) {
        c.eng.reset(new Engine<float>());
        if (c.eng->init(dev, mvr::BOUNDARY_REFERENCE, 0.0, 0.0f) != MVR_OK) {
            c.eng.reset();
            return MVR_ERR_CUDA;
        }
    }
    if (cudaSetDevice(dev) != cudaSuccess) return MVR_ERR_CUDA;
    auto key = std::make_tuple(b[0], b[1], b[2], kd[0], kd[1], kd[2]);
    auto it = c.plans.find(key);
    Plan<float> *pl = nullptr;
    if (it == c.plans.end()) {
        std::unique_ptr<Plan<float>> p(new Plan<float>());
        if (c.eng->make_plan(*p, b, kernel, kd, nullptr, nullptr) != MVR_OK) return MVR_ERR_CUDA;
        pl = p.get();
        c.plans[key] = std::move(p);
    } else {
        pl = it->second.get();
        // the kernel may change between calls with the same sizes
        if (c.eng->make_plan(*pl, b, kernel, kd, nullptr, nullptr) != MVR_OK) return MVR_ERR_CUDA;
    }
    const long long n = (long long)b[0] * b[1] * b[2];
    if (n > c.cap) {
        cudaFree(c.d_img);
        cudaFree(c.d_out);
        c.d_img = c.d_out = nullptr;
        c.cap = 0;
        if (cudaMalloc(&c.d_img, sizeof(float) * (size_t)n) != cudaSuccess) return MVR_ERR_OOM;
        if (cudaMalloc(&c.d_out, sizeof(float) * (size_t)n) != cudaSuccess) return MVR_ERR_OOM;
        c.cap = n;
    }
    cudaStream_t s = c.eng->stream();
    if (host_copy(c.d_img, im, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, dev, s) != cudaSuccess)
        return MVR_ERR_CUDA;
    if (c.eng->convolve(*pl, c.d_img, mvr::SRC_ZERO, c.d_out) != MVR_OK) return MVR_ERR_CUDA;
    if (host_copy(out, c.d_out, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, dev, s) != cudaSuccess)
        return MVR_ERR_CUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? MVR_OK : MVR_ERR_CUDA;
}
}  // namespace

extern "C" void convolution3DfftCUDAInPlace(float *im, int *imDim, float *kernel, int *kernelDim, int devCUDA)
{
    conv3d(im, imDim, kernel, kernelDim, devCUDA, im);
}

extern "C" float *convolution3DfftCUDA(float *im, int *imDim, float *kernel, int *kernelDim, int devCUDA)
{
    if (!imDim) return nullptr;
    const long long n = (long long)imDim[0] * imDim[1] * imDim[2];
    float *out = (float *)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    if (!out) return nullptr;
    if (conv3d(im, imDim, kernel, kernelDim, devCUDA, out) != MVR_OK) {
        free(out);
        return nullptr;
    }
    return out;
}

extern "C" void mvr_free(void *p) { free(p); }

extern "C" int getNumDevicesCUDA(void)
{
    int n = 0;
    return cudaGetDeviceCount(&n) == cudaSuccess ? n : -1;
}

extern "C" void getNameDeviceCUDA(int dev, char *name)
{
    if (!name) return;
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
        name[0] = 0;
        return;
    }
    std::strncpy(name, p.name, 255);
    name[255] = 0;
}

extern "C" long long getMemDeviceCUDA(int dev)
{
    cudaDeviceProp p;
    return cudaGetDeviceProperties(&p, dev) == cudaSuccess ? (long long)p.totalGlobalMem : -1;
}

extern "C" long long getFreeMemDeviceCUDA(int dev)
{
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess || cudaSetDevice(dev) != cudaSuccess) return -1;
    size_t f = 0, t = 0;
    const cudaError_t e = cudaMemGetInfo(&f, &t);
    cudaSetDevice(cur);
    return e == cudaSuccess ? (long long)f : -1;
}

extern "C" int getCUDAcomputeCapabilityMajorVersion(int dev)
{
    cudaDeviceProp p;
    return cudaGetDeviceProperties(&p, dev) == cudaSuccess ? p.major : -1;
}

extern "C" int getCUDAcomputeCapabilityMinorVersion(int dev)
{
    cudaDeviceProp p;
    return cudaGetDeviceProperties(&p, dev) == cudaSuccess ? p.minor : -1;
}
