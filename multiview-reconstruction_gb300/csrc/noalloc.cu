// mvr_convolve_static: the block convolution (linear, zero extension, output over
// the image) with all of its scratch in a fixed device array, for callers that
// cannot allocate device memory.  See include/mvr_gb300.h for the contract.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/mvr_gb300.h"
#include "engine.cuh"

namespace {

using namespace mvr;

// Limits of the fixed scratch: two half spectra of at most kMaxPc complex values
// (the kernel's and the image's) and one twiddle table per axis.
constexpr long long kMaxPc = 1LL << 20;   // complex values per spectrum (8 MiB as float2)
constexpr int kMaxAxis = 1024;            // FFT length per axis
constexpr long long kScratchLen = 2 * kMaxPc + 3LL * kMaxAxis;

// The scratch itself: 16 MiB + 24 KiB, resident on every device that loads the library.
static __device__ __align__(256) float2 g_static_scratch[kScratchLen];

std::mutex g_mutex;

void put_error(char *err, int len, const char *msg)
{
    if (err && len > 0) std::snprintf(err, (size_t)len, "%s", msg);
}

// Twiddle tables exp(-2 pi i k / n) of the three axes, written straight into the scratch
// array: nothing is staged in host memory, so a call queues device work only.
__global__ void k_static_twiddles(float2 *tw, int n0, int n1, int n2)
{
    const int axis = blockIdx.y;
    const int n = axis == 0 ? n0 : (axis == 1 ? n1 : n2);
    float2 *t = tw + (size_t)axis * kMaxAxis;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        double s, c;
        sincospi(-2.0 * (double)k / (double)n, &s, &c);
        t[k] = make_float2((float)c, (float)s);
    }
}

// Resolves the scratch array's device address in the current context and raises the
// dynamic shared-memory limit of the kernels this entry point launches.  Done on every
// call (both are cheap and allocate nothing), so a new context or a reset device never
// sees an address or a limit left over from an earlier one.
int setup_device(float2 **scratch, char *err, int err_len)
{
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    const int m = 227 * 1024;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rows_fwd<float, SrcKernel, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rows_fwd<float, SrcZero<float>, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 m);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cols<float, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cols<float, 1, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_cols<float, 2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rows_update<float, EPI_STORE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    if (e != cudaSuccess) {
        put_error(err, err_len, cudaGetErrorString(e));
        return MVR_ERR_CUDA;
    }
    *scratch = static_cast<float2 *>(p);
    return MVR_OK;
}

void col_shape(int n, int &NP, size_t &smem)
{
    NP = 16;
    while (NP > 1 && sizeof(float2) * (size_t)n * (1 + 2 * NP) > 72 * 1024) NP >>= 1;
    smem = sizeof(float2) * (size_t)n * (1 + 2 * NP);
}

}  // namespace

extern "C" int mvr_convolve_static(const float *img, const int img_size[3], const float *kernel,
                                   const int kernel_size[3], float *out, void *stream, char *err, int err_len)
{
    if (!img || !img_size || !kernel || !kernel_size || !out) {
        put_error(err, err_len, "img, img_size, kernel, kernel_size and out must not be NULL");
        return MVR_ERR_ARG;
    }
    int b[3], kd[3], P[3];
    for (int d = 0; d < 3; ++d) {
        b[d] = img_size[d];
        kd[d] = kernel_size[d];
        if (b[d] < 1 || kd[d] < 1) {
            put_error(err, err_len, "sizes must be >= 1");
            return MVR_ERR_ARG;
        }
        P[d] = (int)next_friendly_even((long long)b[d] + kd[d] - 1);
    }
    const long long Hx = P[0] / 2 + 1;
    const long long Pc = Hx * P[1] * P[2];
    if (P[0] > kMaxAxis || P[1] > kMaxAxis || P[2] > kMaxAxis || Pc > kMaxPc) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "size too large for the static scratch: FFT domain %dx%dx%d (%lld complex values) exceeds "
                      "%d per axis or %lld values",
                      P[0], P[1], P[2], Pc, kMaxAxis, kMaxPc);
        put_error(err, err_len, msg);
        return MVR_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    float2 *scr = nullptr;
    int rc = setup_device(&scr, err, err_len);
    if (rc != MVR_OK) return rc;
    cudaError_t e;
    float2 *Sk = scr;           // kernel spectrum
    float2 *S = scr + kMaxPc;   // image spectrum
    float2 *tw[3] = {scr + 2 * kMaxPc, scr + 2 * kMaxPc + kMaxAxis, scr + 2 * kMaxPc + 2 * kMaxAxis};
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_static_twiddles<<<dim3(4, 3), 256, 0, s>>>(tw[0], P[0], P[1], P[2]);
    const FftDesc dx = make_desc(P[0] / 2), dy = make_desc(P[1]), dz = make_desc(P[2]);
    const int m = P[0] / 2;
    int RP = 16;
    const size_t per_row = 2 * sizeof(float2) * (size_t)(m + 1), tws = sizeof(float2) * (size_t)P[0];
    while (RP > 1 && tws + RP * per_row > 48 * 1024) RP >>= 1;
    const size_t smem_row = tws + RP * per_row;
    int NPy, NPz;
    size_t smem_y, smem_z;
    col_shape(P[1], NPy, smem_y);
    col_shape(P[2], NPz, smem_z);
    const long long nrows = (long long)P[1] * P[2];
    const unsigned grid_rows = (unsigned)((nrows + RP - 1) / RP);
    const dim3 gy((unsigned)((Hx + NPy - 1) / NPy), (unsigned)P[2]);
    const dim3 gz((unsigned)((Hx + NPz - 1) / NPz), (unsigned)P[1]);
    const long long ey = Hx, oy = (long long)P[1] * Hx, ez = (long long)P[1] * Hx, oz = Hx;

    BlockMaps kms{};  // the kernel's spectrum: whole domain
    BlockMaps bms{};  // the image: block at the origin, k-1-k/2 wrapped before it
    BlockMap &km = kms.m[0];
    BlockMap &bm = bms.m[0];
    for (int d = 0; d < 3; ++d) {
        km.P[d] = km.b[d] = P[d];
        km.D[d] = P[d];
        bm.P[d] = P[d];
        bm.b[d] = b[d];
        bm.L[d] = kd[d] - 1 - kd[d] / 2;
        bm.D[d] = b[d];
        bm.OD[d] = b[d];
        bm.whi[d] = b[d];
    }
    const double scale = 1.0 / ((double)P[0] * P[1] * P[2]);
    k_rows_fwd<float, SrcKernel, true><<<grid_rows, 256, smem_row, s>>>(SrcKernel{kernel, {kd[0], kd[1], kd[2]}, scale}, Sk,
                                                                 kms, Pc, dx, tw[0], RP);
    k_cols<float, 0, true><<<gy, 256, smem_y, s>>>(Sk, Sk, nullptr, (int)Hx, ey, oy, NPy, Pc, dy, tw[1]);
    k_cols<float, 0, true><<<gz, 256, smem_z, s>>>(Sk, Sk, nullptr, (int)Hx, ez, oz, NPz, Pc, dz, tw[2]);
    k_rows_fwd<float, SrcZero<float>, true><<<grid_rows, 256, smem_row, s>>>(SrcZero<float>{img}, S, bms, Pc, dx, tw[0], RP);
    k_cols<float, 0, true><<<gy, 256, smem_y, s>>>(S, S, nullptr, (int)Hx, ey, oy, NPy, Pc, dy, tw[1]);
    k_cols<float, 2, true><<<gz, 256, smem_z, s>>>(S, S, Sk, (int)Hx, ez, oz, NPz, Pc, dz, tw[2]);
    k_cols<float, 1, true><<<gy, 256, smem_y, s>>>(S, S, nullptr, (int)Hx, ey, oy, NPy, Pc, dy, tw[1]);
    UpdateArgs ua{};
    ua.store = out;
    k_rows_update<float, EPI_STORE, true><<<grid_rows, 256, smem_row, s>>>(S, ua, bms, Pc, dx, tw[0], RP);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        put_error(err, err_len, cudaGetErrorString(e));
        return MVR_ERR_CUDA;
    }
    return MVR_OK;
}
