// Learned multi-iteration proposal: a 3-level 3D U-Net (16/32/64 channels, 3x3x3
// convolutions, BF16 weights and activations, FP32 accumulation on the tcgen05 tensor
// cores) trained with its own forward and backward kernels, and its C ABI.
//
// No counterpart in the reference: the proposal is gated by the plain method's own
// data-likelihood residual (mvr_decon_likelihood) by the caller.
//
// Network (input [psi_k, ratio_k] features, output log(psi_{k+m} / psi_k)):
//   e1 = relu(conv(in, 16 -> 16))                level 1 (D, H, W)
//   e2 = relu(conv(pool(e1), 16 -> 32))          level 2 (D/2 ...)
//   b3 = relu(conv(pool(e2), 32 -> 64))          level 3 (D/4 ...)
//   d2 = relu(conv([up(b3), e2], 96 -> 32))      level 2
//   d1 = relu(conv([up(d2), e1], 48 -> 16))      level 1
//   out = head(d1) (1x1x1, 16 -> 1)
// Input features: channel 0 = log(psi_k / mean psi_k), channel 1 = log(ratio_k) with
// ratio_k = psi_{k+1} / psi_k the plain method's one-iteration update, the
// other 14 input channels are zero (the tensor-core K step is 16 channels).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include <cudaTypedefs.h>

#include "../../include/mvr_gb300.h"
#include "conv3d_tc.cuh"
#include "conv3d_tma.cuh"
#include "fsum.cuh"

namespace mvr {
namespace {

typedef __nv_bfloat16 bf16;

int gsize(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)); }

// ---- tcgen05 convolution launchers --------------------------------------------------
template <int N, int C>
size_t conv_smem() { return 2 * (128 * C * 2 + N * C * 2); }
template <int N>
size_t wgrad_smem() { return 2 * (128 * 64 * 2 + N * 64 * 2); }

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder()
{
    static const PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

// MVR_CONV_TMA=0 keeps every convolution on k_conv3d_shift
bool conv_tma_enabled()
{
    const char *e = std::getenv("MVR_CONV_TMA");
    return !(e && e[0] == '0');
}

// The persistent TMA convolution (k_conv3d_tma) of a shape that fits: the tensor map of the
// [B][D][H][W][C] input with a box of 8 channels x 10 x 18 x 3 voxels, one CTA per SM slot.
// cudaErrorNotSupported when no encoder is available (the caller falls back).
template <int N, int C, int OUT>
cudaError_t launch_conv_tma(const bf16 *act, const bf16 *w, const float *bias, void *out, const ConvGeom &g, int sign,
                            int relu, int *err, cudaStream_t s)
{
    const PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return cudaErrorNotSupported;
    CUtensorMap map;
    const cuuint64_t dims[5] = {(cuuint64_t)C, (cuuint64_t)g.W, (cuuint64_t)g.H, (cuuint64_t)g.D, (cuuint64_t)g.B};
    const cuuint64_t strides[4] = {(cuuint64_t)C * 2, (cuuint64_t)g.W * C * 2, (cuuint64_t)g.H * g.W * C * 2,
                                   (cuuint64_t)g.D * g.H * g.W * C * 2};
    const cuuint32_t box[5] = {8, (cuuint32_t)kShHX, (cuuint32_t)kShHY, (cuuint32_t)kShHZ, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<bf16 *>(act), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorInvalidValue;
    const size_t sm = conv_tma_smem<N, C>();
    cudaError_t e =
        cudaFuncSetAttribute(k_conv3d_tma<N, C, OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_conv3d_tma<N, C, OUT>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess) return e;
    int per = 0, dev = 0, nsm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_conv3d_tma<N, C, OUT>, 128, sm)) != cudaSuccess)
        return e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    const long long bricks =
        (long long)((g.W + kShX - 1) / kShX) * ((g.H + kShY - 1) / kShY) * g.D * g.B;
    const long long grid = std::min<long long>(bricks, (long long)nsm * std::max(1, per));
    k_conv3d_tma<N, C, OUT><<<(unsigned)grid, 128, sm, s>>>(map, w, bias, out, g, sign, relu, err);
    return cudaGetLastError();
}

// Forward and data-gradient convolutions run on 8 x 16 x 1 output bricks with the input
// halo staged once in shared memory and one descriptor per tap: the persistent TMA kernel
// where its buffers fit and N + C >= 48 (k_conv3d_tma), else k_conv3d_shift; k_conv3d_brick
// (halo, per-tap copies) and k_conv3d_tc (gathered per tap) are earlier forms of the same
// product.  Measured on the 128^3 grid (ncu, serialised): 16 <- 48 channels 632 against
// 680 us, 32 <- 16 (64^3) 40 against 49 us, 64 <- 32 (32^3) 20 against 28 us, but 16 <- 16
// 251 against 193 us: the halo's tiles have a 16-byte inner extent (one K group of one voxel),
// which the copy engine moves as that many small rows, and the threads' 16-byte
// asynchronous copies of k_conv3d_shift keep up with it when the tile is small.
template <int N, int C, int OUT>
cudaError_t launch_conv(const bf16 *act, const bf16 *w, const float *bias, void *out, const ConvGeom &g, int sign,
                        int relu, int *err, cudaStream_t s)
{
    if constexpr (conv_tma_fits<N, C>() && N + C >= 48) {
        if (conv_tma_enabled()) {
            const cudaError_t e = launch_conv_tma<N, C, OUT>(act, w, bias, out, g, sign, relu, err, s);
            if (e != cudaErrorNotSupported) return e;
        }
    }
    const size_t sm = conv_shift_smem<N, C>();
    cudaError_t e =
        cudaFuncSetAttribute(k_conv3d_shift<N, C, OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const long long bricks =
        (long long)((g.W + kShX - 1) / kShX) * ((g.H + kShY - 1) / kShY) * g.D * g.B;
    k_conv3d_shift<N, C, OUT><<<(unsigned)bricks, 128, sm, s>>>(act, w, bias, out, g, sign, relu, err);
    return cudaGetLastError();
}

// Decoder convolution (bias, ReLU, BF16 out) on the concatenation [up(low) (CU channels),
// skip (C - CU channels)] without materialising it.
template <int N, int C, int CU>
cudaError_t launch_conv_concat(const bf16 *low, const bf16 *skip, const bf16 *w, const float *bias, void *out,
                               const ConvGeom &g, int *err, cudaStream_t s)
{
    const size_t sm = conv_shift_smem<N, C>();
    cudaError_t e =
        cudaFuncSetAttribute(k_conv3d_shift<N, C, 0, CU>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const long long bricks =
        (long long)((g.W + kShX - 1) / kShX) * ((g.H + kShY - 1) / kShY) * g.D * g.B;
    k_conv3d_shift<N, C, 0, CU><<<(unsigned)bricks, 128, sm, s>>>(low, w, bias, out, g, 1, 1, err, skip);
    return cudaGetLastError();
}

template <int N, int C>
cudaError_t launch_wgrad(const bf16 *X, const bf16 *G, float *dW, const ConvGeom &g, int *err, cudaStream_t s)
{
    const size_t sm = wgrad_smem<N>();
    cudaError_t e = cudaFuncSetAttribute(k_wgrad_tc<N, C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    const int mt = (27 * C + 127) / 128;
    // split the voxels so that about 4 waves of CTAs run
    long long splits = std::max<long long>(1, (152LL * 4) / mt);
    long long vpc = (g.nvox + splits - 1) / splits;
    vpc = ((vpc + 63) / 64) * 64;
    splits = (g.nvox + vpc - 1) / vpc;
    k_wgrad_tc<N, C><<<dim3((unsigned)mt, (unsigned)splits), 128, sm, s>>>(X, G, dW, g, vpc, err);
    return cudaGetLastError();
}

// forward (N = Cout, C = Cin) and dgrad (N = Cin, C = Cout) shapes of the five layers
cudaError_t conv_any(int N, int C, int out_mode, const bf16 *act, const bf16 *w, const float *bias, void *out,
                     const ConvGeom &g, int sign, int relu, int *err, cudaStream_t s)
{
#define MVR_CONV_CASE(NN, CC)                                                                              \
    if (N == NN && C == CC)                                                                                \
        return out_mode == 0 ? launch_conv<NN, CC, 0>(act, w, bias, out, g, sign, relu, err, s)            \
                             : launch_conv<NN, CC, 1>(act, w, bias, out, g, sign, relu, err, s);
    MVR_CONV_CASE(16, 16)
    MVR_CONV_CASE(32, 16)
    MVR_CONV_CASE(64, 32)
    MVR_CONV_CASE(32, 96)
    MVR_CONV_CASE(16, 48)
    MVR_CONV_CASE(16, 32)
    MVR_CONV_CASE(32, 64)
    MVR_CONV_CASE(96, 32)
    MVR_CONV_CASE(48, 16)
#undef MVR_CONV_CASE
    return cudaErrorInvalidValue;
}

cudaError_t wgrad_any(int N, int C, const bf16 *X, const bf16 *G, float *dW, const ConvGeom &g, int *err,
                      cudaStream_t s)
{
    if (N == 16 && C == 16) return launch_wgrad<16, 16>(X, G, dW, g, err, s);
    if (N == 32 && C == 16) return launch_wgrad<32, 16>(X, G, dW, g, err, s);
    if (N == 64 && C == 32) return launch_wgrad<64, 32>(X, G, dW, g, err, s);
    if (N == 32 && C == 96) return launch_wgrad<32, 96>(X, G, dW, g, err, s);
    if (N == 16 && C == 48) return launch_wgrad<16, 48>(X, G, dW, g, err, s);
    return cudaErrorInvalidValue;
}

// ---- elementwise kernels ------------------------------------------------------------
// per-patch mean of psi: kMeanParts CTAs per patch sum their slices as compensated float
// pairs (one double per CTA), then one thread per patch adds the parts in FP64
constexpr int kMeanParts = 256;

__global__ void k_patch_partials(const float *psi, long long per, double *parts)
{
    __shared__ float sh[256], sl[256];
    const float *p = psi + (long long)blockIdx.y * per;
    const long long chunk = (per + kMeanParts - 1) / kMeanParts;
    const long long i0 = (long long)blockIdx.x * chunk, i1 = min(per, i0 + chunk);
    float hi = 0.0f, lo = 0.0f;
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) pair_add(hi, lo, p[i], 0.0f);
    sh[threadIdx.x] = hi;
    sl[threadIdx.x] = lo;
    __syncthreads();
    for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            float a = sh[threadIdx.x], b = sl[threadIdx.x];
            pair_add(a, b, sh[threadIdx.x + h], sl[threadIdx.x + h]);
            sh[threadIdx.x] = a;
            sl[threadIdx.x] = b;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) parts[(long long)blockIdx.y * kMeanParts + blockIdx.x] = (double)sh[0] + (double)sl[0];
}

__global__ void k_patch_mean(const double *parts, long long per, int B, double *mean)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    double s = 0.0;
    for (int k = 0; k < kMeanParts; ++k) s += parts[(long long)b * kMeanParts + k];
    mean[b] = s / (double)per;
}

// features: [log(psi / mean), log(psi_next / psi), 0 x 14] as BF16; target log(psi_m / psi)
__global__ void k_features(const float *psi, const float *psi_next, const float *psi_m, long long n, long long per,
                           const double *mean, bf16 *in16, float *target)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float p = fmaxf(psi[i], 1e-12f);
        const float m = (float)mean[i / per];
        __align__(16) bf16 f[16];
        f[0] = __float2bfloat16(logf(p / fmaxf(m, 1e-12f)));
        f[1] = __float2bfloat16(psi_next ? logf(fmaxf(psi_next[i], 1e-12f) / p) : 0.0f);
#pragma unroll
        for (int c = 2; c < 16; ++c) f[c] = __float2bfloat16(0.0f);
        uint4 *o = reinterpret_cast<uint4 *>(in16 + i * 16);
        o[0] = reinterpret_cast<const uint4 *>(f)[0];
        o[1] = reinterpret_cast<const uint4 *>(f)[1];
        if (target && psi_m) target[i] = logf(fmaxf(psi_m[i], 1e-12f) / p);
    }
}

// 2x2x2 average pooling, channels-last BF16
__global__ void k_pool(const bf16 *in, bf16 *out, ConvGeom lo, int C)
{
    const long long n = lo.nvox * C;
    const int W2 = lo.W * 2, H2 = lo.H * 2, D2 = lo.D * 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        int x, y, z, b;
        vox_coords(lo, i / C, x, y, z, b);
        float s = 0.0f;
        for (int q = 0; q < 8; ++q) {
            const long long src = (((long long)b * D2 + 2 * z + (q >> 2)) * H2 + 2 * y + ((q >> 1) & 1)) * W2 + 2 * x + (q & 1);
            s += __bfloat162float(in[src * C + c]);
        }
        out[i] = __float2bfloat16(0.125f * s);
    }
}

// out[n] = [up(low)[n] (Cu channels), skip[n] (Cs channels)], nearest upsampling x2, in
// chunks of 8 channels (16 bytes); Cu and Cs are multiples of 8
__global__ void k_up_concat(const bf16 *low, const bf16 *skip, bf16 *out, ConvGeom hi, int Cu, int Cs)
{
    const int Ct = Cu + Cs, K = Ct / 8, Ku = Cu / 8;
    const long long n = hi.nvox * K;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c8 = (int)(i % K);
        const long long v = i / K;
        uint4 val;
        if (c8 < Ku) {
            int x, y, z, b;
            vox_coords(hi, v, x, y, z, b);
            const long long lv = (((long long)b * (hi.D / 2) + z / 2) * (hi.H / 2) + y / 2) * (hi.W / 2) + x / 2;
            val = reinterpret_cast<const uint4 *>(low + lv * Cu)[c8];
        } else {
            val = reinterpret_cast<const uint4 *>(skip + v * Cs)[c8 - Ku];
        }
        reinterpret_cast<uint4 *>(out + v * Ct)[c8] = val;
    }
}

// head: out[n] = sum_c wh[c] d1[n][c] + bh
__global__ void k_head(const bf16 *d1, const float *wh, const float *bh, float *out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        float s = bh[0];
#pragma unroll
        for (int c = 0; c < 16; ++c) s += wh[c] * __bfloat162float(d1[i * 16 + c]);
        out[i] = s;
    }
}

// loss sum (FP64 atomics per CTA), gout = 2 (out - target) / n, head gradients,
// G5 = gout * wh * (d1 > 0) as BF16
__global__ void k_head_back(const float *out, const float *target, const bf16 *d1, const float *wh, long long n,
                            double *loss, float *gwh, float *gbh, bf16 *G5, float *db5)
{
    __shared__ float swh[17], sdb[16];
    __shared__ double sl;
    if (threadIdx.x < 17) swh[threadIdx.x] = 0.0f;
    if (threadIdx.x < 16) sdb[threadIdx.x] = 0.0f;
    if (threadIdx.x == 0) sl = 0.0;
    __syncthreads();
    float lw[16] = {0}, ldb[16] = {0}, lb = 0.0f;
    double ll = 0.0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float d = out[i] - target[i];
        ll += (double)d * d;
        const float g = 2.0f * d / (float)n;
        lb += g;
        __align__(16) bf16 gg[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            const float a = __bfloat162float(d1[i * 16 + c]);
            lw[c] += g * a;
            const float gc = a > 0.0f ? g * wh[c] : 0.0f;
            ldb[c] += gc;
            gg[c] = __float2bfloat16(gc);
        }
        uint4 *o = reinterpret_cast<uint4 *>(G5 + i * 16);
        o[0] = reinterpret_cast<const uint4 *>(gg)[0];
        o[1] = reinterpret_cast<const uint4 *>(gg)[1];
    }
    for (int c = 0; c < 16; ++c) {
        atomicAdd(&swh[c], lw[c]);
        atomicAdd(&sdb[c], ldb[c]);
    }
    atomicAdd(&swh[16], lb);
    atomicAdd(&sl, ll);
    __syncthreads();
    if (threadIdx.x < 16) {
        atomicAdd(&gwh[threadIdx.x], swh[threadIdx.x]);
        atomicAdd(&db5[threadIdx.x], sdb[threadIdx.x]);
    }
    if (threadIdx.x == 16) atomicAdd(gbh, swh[16]);
    if (threadIdx.x == 0) atomicAdd(loss, sl);
}

// G[n][c] = (gsk[n][coff + c] + gpool) * (act[n][c] > 0) as BF16, with gpool the
// gradient of the pooled copy (glo[parent][c] / 8; glo may be NULL), and the bias
// gradient db[c] += sum_n G[n][c].
__global__ void k_mask_grad(const float *gsk, int gsk_stride, int coff, const float *glo, ConvGeom hi, const bf16 *act,
                            int C, bf16 *G, float *db)
{
    extern __shared__ float sdb[];
    for (int c = threadIdx.x; c < C; c += blockDim.x) sdb[c] = 0.0f;
    __syncthreads();
    const long long n = hi.nvox * C;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long v = i / C;
        float g = gsk ? gsk[v * gsk_stride + coff + c] : 0.0f;
        if (glo) {
            int x, y, z, b;
            vox_coords(hi, v, x, y, z, b);
            const long long lv = (((long long)b * (hi.D / 2) + z / 2) * (hi.H / 2) + y / 2) * (hi.W / 2) + x / 2;
            g += 0.125f * glo[lv * C + c];
        }
        const float r = __bfloat162float(act[i]) > 0.0f ? g : 0.0f;
        G[i] = __float2bfloat16(r);
        atomicAdd(&sdb[c], r);
    }
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) atomicAdd(&db[c], sdb[c]);
}

// gradient of up(low) inside a concat gradient: glow[lv][c] = sum over the 8 children
// of gcat[child][c], c < Cu
__global__ void k_up_back(const float *gcat, int Ct, ConvGeom lo, int Cu, float *glow)
{
    const long long n = lo.nvox * Cu;
    const int W2 = lo.W * 2, H2 = lo.H * 2, D2 = lo.D * 2;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % Cu);
        int x, y, z, b;
        vox_coords(lo, i / Cu, x, y, z, b);
        float s = 0.0f;
        for (int q = 0; q < 8; ++q) {
            const long long src = (((long long)b * D2 + 2 * z + (q >> 2)) * H2 + 2 * y + ((q >> 1) & 1)) * W2 + 2 * x + (q & 1);
            s += gcat[src * Ct + c];
        }
        glow[i] = s;
    }
}

// BF16 copies of the FP32 master weights: W[co][t][ci] and its transpose WT[ci][t][co]
__global__ void k_weights_bf16(const float *w, int Co, int Ci, bf16 *wt, bf16 *wtt)
{
    const long long n = (long long)Co * 27 * Ci;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(i % Ci);
        const long long r = i / Ci;
        const int t = (int)(r % 27), co = (int)(r / 27);
        const bf16 v = __float2bfloat16(w[i]);
        wt[i] = v;
        if (wtt) wtt[((long long)ci * 27 + t) * Co + co] = v;
    }
}

// Adam (bias corrected), FP32 master parameters
__global__ void k_adam(float *p, const float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

// psi' = psi * exp(clamp(pred, -cap, cap))
__global__ void k_propose(const float *psi, const float *pred, float *out, long long n, float cap)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = psi[i] * expf(fminf(fmaxf(pred[i], -cap), cap));
}

// 2 x 2 x 2 average of a float volume [z][y][x] of even dims (the coarse grid of the proposal)
__global__ void k_pool2_f32(const float *__restrict__ in, long long X, long long Y, long long Z, float *__restrict__ out)
{
    const long long x2 = X / 2, y2 = Y / 2, n = x2 * y2 * (Z / 2);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long x = i % x2, t = i / x2, y = t % y2, z = t / y2;
        const float *p = in + ((2 * z) * Y + 2 * y) * X + 2 * x;
        const float s = (p[0] + p[1]) + (p[X] + p[X + 1]) + ((p[X * Y] + p[X * Y + 1]) + (p[X * Y + X] + p[X * Y + X + 1]));
        out[i] = 0.125f * s;
    }
}

// The coarse proposal applied at full resolution: c = pred - log(next_low / psi_low) on the
// coarse grid (the predicted log change beyond the plain step), trilinearly interpolated at
// full-resolution voxel x (coarse coordinate x / 2 - 1 / 4, clamped at the borders), and
// out = psi_next * exp(clamp(c, -cap, cap)).
__device__ __forceinline__ float coarse_c(const float *pred, const float *lo_psi, const float *lo_next, long long i)
{
    return pred[i] - logf(fmaxf(lo_next[i], 1e-12f) / fmaxf(lo_psi[i], 1e-12f));
}
__global__ void k_apply_coarse(const float *__restrict__ psi_next, long long X, long long Y, long long Z,
                               const float *__restrict__ pred, const float *__restrict__ lo_psi,
                               const float *__restrict__ lo_next, float cap, float *__restrict__ out)
{
    const long long x2 = X / 2, y2 = Y / 2, z2 = Z / 2, n = X * Y * Z;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const long long x = i % X, t = i / X, y = t % Y, z = t / Y;
        long long c0[3], c1[3];
        float f[3];
        const long long dim[3] = {x2, y2, z2}, pos[3] = {x, y, z};
        for (int d = 0; d < 3; ++d) {
            const float u = 0.5f * (float)pos[d] - 0.25f;
            const float fl = floorf(u);
            long long a = (long long)fl, b = a + 1;
            f[d] = u - fl;
            if (a < 0) a = 0;
            if (b > dim[d] - 1) b = dim[d] - 1;
            c0[d] = a;
            c1[d] = b;
        }
        float acc = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long cx = (k & 1) ? c1[0] : c0[0], cy = (k & 2) ? c1[1] : c0[1], cz = (k & 4) ? c1[2] : c0[2];
            const float w = ((k & 1) ? f[0] : 1.0f - f[0]) * ((k & 2) ? f[1] : 1.0f - f[1]) * ((k & 4) ? f[2] : 1.0f - f[2]);
            acc += w * coarse_c(pred, lo_psi, lo_next, (cz * y2 + cy) * x2 + cx);
        }
        out[i] = psi_next[i] * expf(fminf(fmaxf(acc, -cap), cap));
    }
}

}  // namespace

// ---- the network ----------------------------------------------------------------------
struct LayerSpec {
    int ci, co;
};
constexpr LayerSpec kLayers[5] = {{16, 16}, {16, 32}, {32, 64}, {96, 32}, {48, 16}};

class UNet {
public:
    UNet(int batch, const int dims[3], unsigned seed, int device) : B_(batch), dev_(device), seed_(seed)
    {
        for (int d = 0; d < 3; ++d) dims_[d] = dims[d];
    }
    ~UNet();
    int init();
    int set_input(const float *psi, const float *psi_next, const float *psi_target);
    int forward(float *pred, bool fused = false);
    int train_step(float lr, double *loss);
    int propose(const float *psi, float *out, float cap);
    long long num_params() const { return nparams_; }
    int get_params(float *host);
    int set_params(const float *host);
    int get_grads(float *host);
    const std::string &error() const { return err_; }

private:
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
    int check_err();
    int refresh_weights();
    template <typename P>
    int alloc(P *&p, long long n)
    {
        p = nullptr;
        const cudaError_t e = cudaMalloc(&p, sizeof(P) * (size_t)std::max<long long>(1, n));
        if (e == cudaSuccess) allocs_.push_back((void *)p);
        return cuda(e, "cudaMalloc");
    }

    int B_, dev_;
    unsigned seed_;
    int dims_[3];
    ConvGeom g1_{}, g2_{}, g3_{};
    cudaStream_t s_ = nullptr;
    std::vector<void *> allocs_;
    long long nparams_ = 0;
    long long woff_[5], boff_[5], whoff_ = 0, bhoff_ = 0;
    float *params_ = nullptr, *grads_ = nullptr, *am_ = nullptr, *av_ = nullptr;
    bf16 *wt_[5] = {}, *wtt_[5] = {};
    bf16 *in16_ = nullptr, *e1_ = nullptr, *p1_ = nullptr, *e2_ = nullptr, *p2_ = nullptr, *b3_ = nullptr;
    bf16 *c2_ = nullptr, *d2_ = nullptr, *c1_ = nullptr, *d1_ = nullptr;
    bf16 *G_ = nullptr;  // BF16 gradient scratch (largest: level 1 x 16 or level 2 x 32)
    float *out_ = nullptr, *target_ = nullptr;
    float *gc1_ = nullptr, *gc2_ = nullptr, *gd2_ = nullptr, *gb3_ = nullptr, *gp2_ = nullptr, *gp1_ = nullptr;
    double *mean_ = nullptr, *meanp_ = nullptr, *loss_ = nullptr;
    int *err_dev_ = nullptr;
    int step_ = 0;
    bool weights_fresh_ = false;
    std::string err_;
};

UNet::~UNet()
{
    cudaSetDevice(dev_);
    if (s_) cudaStreamSynchronize(s_);
    for (void *p : allocs_) cudaFree(p);
    if (s_) cudaStreamDestroy(s_);
}

int UNet::init()
{
    if (B_ < 1) return fail(MVR_ERR_ARG, "batch must be >= 1");
    for (int d = 0; d < 3; ++d)
        if (dims_[d] < 4 || dims_[d] % 4) return fail(MVR_ERR_ARG, "patch sizes must be multiples of 4");
    int D_ = MVR_OK;
    if ((D_ = cuda(cudaSetDevice(dev_), "cudaSetDevice")) != MVR_OK) return D_;
    if ((D_ = cuda(cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking), "stream")) != MVR_OK) return D_;
    g1_ = ConvGeom{B_, dims_[2], dims_[1], dims_[0], (long long)B_ * dims_[0] * dims_[1] * dims_[2]};
    g2_ = ConvGeom{B_, dims_[2] / 2, dims_[1] / 2, dims_[0] / 2, g1_.nvox / 8};
    g3_ = ConvGeom{B_, dims_[2] / 4, dims_[1] / 4, dims_[0] / 4, g1_.nvox / 64};
    // parameter layout: per layer W[co][27][ci] then b[co]; head wh[16], bh
    long long o = 0;
    for (int l = 0; l < 5; ++l) {
        woff_[l] = o;
        o += (long long)kLayers[l].co * 27 * kLayers[l].ci;
        boff_[l] = o;
        o += kLayers[l].co;
    }
    whoff_ = o;
    o += 16;
    bhoff_ = o;
    o += 1;
    nparams_ = o;
    int rc;
#define A_(p, n) \
    if ((rc = alloc(p, n)) != MVR_OK) return rc;
    A_(params_, nparams_) A_(grads_, nparams_) A_(am_, nparams_) A_(av_, nparams_)
    for (int l = 0; l < 5; ++l) {
        A_(wt_[l], (long long)kLayers[l].co * 27 * kLayers[l].ci)
        A_(wtt_[l], (long long)kLayers[l].co * 27 * kLayers[l].ci)
    }
    const long long n1 = g1_.nvox, n2 = g2_.nvox, n3 = g3_.nvox;
    A_(in16_, n1 * 16) A_(e1_, n1 * 16) A_(p1_, n2 * 16) A_(e2_, n2 * 32) A_(p2_, n3 * 32) A_(b3_, n3 * 64)
    A_(c2_, n2 * 96) A_(d2_, n2 * 32) A_(c1_, n1 * 48) A_(d1_, n1 * 16)
    A_(G_, std::max(n1 * 16, n2 * 32)) A_(out_, n1) A_(target_, n1)
    A_(gc1_, n1 * 48) A_(gc2_, n2 * 96) A_(gd2_, n2 * 32) A_(gb3_, n3 * 64) A_(gp2_, n3 * 32) A_(gp1_, n2 * 16)
    A_(mean_, B_) A_(meanp_, (long long)B_ * kMeanParts) A_(loss_, 1) A_(err_dev_, 1)
#undef A_
    // He initialisation from a seeded generator (host), zero biases
    std::vector<float> h((size_t)nparams_, 0.0f);
    std::mt19937 rng(seed_);
    for (int l = 0; l < 5; ++l) {
        const int fan_in = 27 * (l == 0 ? 2 : kLayers[l].ci);
        std::normal_distribution<float> nd(0.0f, std::sqrt(2.0f / fan_in));
        for (long long i = 0; i < (long long)kLayers[l].co * 27 * kLayers[l].ci; ++i) h[(size_t)(woff_[l] + i)] = nd(rng);
    }
    std::normal_distribution<float> nh(0.0f, 0.01f);  // small head: proposals start near the identity
    for (int c = 0; c < 16; ++c) h[(size_t)(whoff_ + c)] = nh(rng);
    if ((rc = cuda(cudaMemcpyAsync(params_, h.data(), sizeof(float) * (size_t)nparams_, cudaMemcpyHostToDevice, s_),
                   "params")) != MVR_OK)
        return rc;
    if ((rc = cuda(cudaMemsetAsync(am_, 0, sizeof(float) * (size_t)nparams_, s_), "memset")) != MVR_OK) return rc;
    if ((rc = cuda(cudaMemsetAsync(av_, 0, sizeof(float) * (size_t)nparams_, s_), "memset")) != MVR_OK) return rc;
    if ((rc = cuda(cudaMemsetAsync(err_dev_, 0, sizeof(int), s_), "memset")) != MVR_OK) return rc;
    return cuda(cudaStreamSynchronize(s_), "init");
}

int UNet::check_err()
{
    int h = 0;
    int rc = cuda(cudaMemcpyAsync(&h, err_dev_, sizeof(int), cudaMemcpyDeviceToHost, s_), "err");
    if (rc != MVR_OK) return rc;
    if ((rc = cuda(cudaStreamSynchronize(s_), "sync")) != MVR_OK) return rc;
    if (h) return fail(MVR_ERR_CUDA, "tensor-core wait timed out");
    return MVR_OK;
}

int UNet::refresh_weights()
{
    if (weights_fresh_) return MVR_OK;
    for (int l = 0; l < 5; ++l) {
        const long long n = (long long)kLayers[l].co * 27 * kLayers[l].ci;
        k_weights_bf16<<<gsize(n), 256, 0, s_>>>(params_ + woff_[l], kLayers[l].co, kLayers[l].ci, wt_[l], wtt_[l]);
    }
    weights_fresh_ = true;
    return cuda(cudaGetLastError(), "k_weights_bf16");
}

int UNet::set_input(const float *psi, const float *psi_next, const float *psi_target)
{
    if (!psi) return fail(MVR_ERR_ARG, "psi must not be NULL");
    cudaSetDevice(dev_);
    const long long per = g1_.nvox / B_;
    k_patch_partials<<<dim3(kMeanParts, B_), 256, 0, s_>>>(psi, per, meanp_);
    k_patch_mean<<<(B_ + 127) / 128, 128, 0, s_>>>(meanp_, per, B_, mean_);
    k_features<<<gsize(g1_.nvox), 256, 0, s_>>>(psi, psi_next, psi_target, g1_.nvox, per, mean_, in16_,
                                                psi_target ? target_ : nullptr);
    return cuda(cudaGetLastError(), "k_features");
}

int UNet::forward(float *pred, bool fused)
{
    cudaSetDevice(dev_);
    int rc = refresh_weights();
    if (rc != MVR_OK) return rc;
    const long long n1 = g1_.nvox, n2 = g2_.nvox;
#define C_(expr)                                         \
    if ((rc = cuda((expr), #expr)) != MVR_OK) return rc;
    C_(conv_any(16, 16, 0, in16_, wt_[0], params_ + boff_[0], e1_, g1_, 1, 1, err_dev_, s_))
    k_pool<<<gsize(n2 * 16), 256, 0, s_>>>(e1_, p1_, g2_, 16);
    C_(conv_any(32, 16, 0, p1_, wt_[1], params_ + boff_[1], e2_, g2_, 1, 1, err_dev_, s_))
    k_pool<<<gsize(g3_.nvox * 32), 256, 0, s_>>>(e2_, p2_, g3_, 32);
    C_(conv_any(64, 32, 0, p2_, wt_[2], params_ + boff_[2], b3_, g3_, 1, 1, err_dev_, s_))
    if (fused) {  // inference: the decoder convolutions read [up(low), skip] directly
        // (materialising [up(d2), e1] for the TMA kernel costs more than that kernel saves:
        // 82 + 632 against 680 us on the 128^3 grid)
        C_((launch_conv_concat<32, 96, 64>(b3_, e2_, wt_[3], params_ + boff_[3], d2_, g2_, err_dev_, s_)))
        C_((launch_conv_concat<16, 48, 32>(d2_, e1_, wt_[4], params_ + boff_[4], d1_, g1_, err_dev_, s_)))
    } else {  // training: the concatenations are kept for the backward pass
        k_up_concat<<<gsize(n2 * 12), 256, 0, s_>>>(b3_, e2_, c2_, g2_, 64, 32);
        C_(conv_any(32, 96, 0, c2_, wt_[3], params_ + boff_[3], d2_, g2_, 1, 1, err_dev_, s_))
        k_up_concat<<<gsize(n1 * 6), 256, 0, s_>>>(d2_, e1_, c1_, g1_, 32, 16);
        C_(conv_any(16, 48, 0, c1_, wt_[4], params_ + boff_[4], d1_, g1_, 1, 1, err_dev_, s_))
    }
    k_head<<<gsize(n1), 256, 0, s_>>>(d1_, params_ + whoff_, params_ + bhoff_, out_, n1);
    C_(cudaGetLastError())
    if (pred) C_(cudaMemcpyAsync(pred, out_, sizeof(float) * (size_t)n1, cudaMemcpyDeviceToDevice, s_))
#undef C_
    return check_err();
}

int UNet::train_step(float lr, double *loss)
{
    int rc = forward(nullptr);
    if (rc != MVR_OK) return rc;
    const long long n1 = g1_.nvox, n2 = g2_.nvox, n3 = g3_.nvox;
#define C_(expr)                                         \
    if ((rc = cuda((expr), #expr)) != MVR_OK) return rc;
    C_(cudaMemsetAsync(grads_, 0, sizeof(float) * (size_t)nparams_, s_))
    C_(cudaMemsetAsync(loss_, 0, sizeof(double), s_))
    float *dW[5], *db[5];
    for (int l = 0; l < 5; ++l) {
        dW[l] = grads_ + woff_[l];
        db[l] = grads_ + boff_[l];
    }
    // head, d1: G5 and the layer-5 bias gradient
    k_head_back<<<gsize(n1), 256, 0, s_>>>(out_, target_, d1_, params_ + whoff_, n1, loss_, grads_ + whoff_,
                                          grads_ + bhoff_, G_, db[4]);
    C_(cudaGetLastError())
    // layer 5: 48 -> 16 on c1 = [up(d2), e1]
    C_(wgrad_any(16, 48, c1_, G_, dW[4], g1_, err_dev_, s_))
    C_(conv_any(48, 16, 1, G_, wtt_[4], nullptr, gc1_, g1_, -1, 0, err_dev_, s_))
    k_up_back<<<gsize(n2 * 32), 256, 0, s_>>>(gc1_, 48, g2_, 32, gd2_);
    k_mask_grad<<<gsize(n2 * 32), 256, 32 * sizeof(float), s_>>>(gd2_, 32, 0, nullptr, g2_, d2_, 32, G_, db[3]);
    C_(cudaGetLastError())
    // layer 4: 96 -> 32 on c2 = [up(b3), e2]
    C_(wgrad_any(32, 96, c2_, G_, dW[3], g2_, err_dev_, s_))
    C_(conv_any(96, 32, 1, G_, wtt_[3], nullptr, gc2_, g2_, -1, 0, err_dev_, s_))
    k_up_back<<<gsize(n3 * 64), 256, 0, s_>>>(gc2_, 96, g3_, 64, gb3_);
    k_mask_grad<<<gsize(n3 * 64), 256, 64 * sizeof(float), s_>>>(gb3_, 64, 0, nullptr, g3_, b3_, 64, G_, db[2]);
    C_(cudaGetLastError())
    // layer 3: 32 -> 64 on pool(e2)
    C_(wgrad_any(64, 32, p2_, G_, dW[2], g3_, err_dev_, s_))
    C_(conv_any(32, 64, 1, G_, wtt_[2], nullptr, gp2_, g3_, -1, 0, err_dev_, s_))
    // e2: skip gradient (channels 64..95 of c2) + pooled gradient from level 3
    k_mask_grad<<<gsize(n2 * 32), 256, 32 * sizeof(float), s_>>>(gc2_, 96, 64, gp2_, g2_, e2_, 32, G_, db[1]);
    C_(cudaGetLastError())
    // layer 2: 16 -> 32 on pool(e1)
    C_(wgrad_any(32, 16, p1_, G_, dW[1], g2_, err_dev_, s_))
    C_(conv_any(16, 32, 1, G_, wtt_[1], nullptr, gp1_, g2_, -1, 0, err_dev_, s_))
    // e1: skip gradient (channels 32..47 of c1) + pooled gradient from level 2
    k_mask_grad<<<gsize(n1 * 16), 256, 16 * sizeof(float), s_>>>(gc1_, 48, 32, gp1_, g1_, e1_, 16, G_, db[0]);
    C_(cudaGetLastError())
    // layer 1: 16 -> 16 on the input features
    C_(wgrad_any(16, 16, in16_, G_, dW[0], g1_, err_dev_, s_))
    // Adam
    ++step_;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, (float)step_), c2 = 1.0f - std::pow(b2, (float)step_);
    k_adam<<<gsize(nparams_), 256, 0, s_>>>(params_, grads_, am_, av_, nparams_, lr, b1, b2, 1e-8f, c1, c2);
    C_(cudaGetLastError())
    weights_fresh_ = false;
    double l = 0.0;
    C_(cudaMemcpyAsync(&l, loss_, sizeof(double), cudaMemcpyDeviceToHost, s_))
#undef C_
    rc = check_err();
    if (rc == MVR_OK && loss) *loss = l / (double)n1;
    return rc;
}

int UNet::propose(const float *psi, float *out, float cap)
{
    int rc = forward(nullptr, true);
    if (rc != MVR_OK) return rc;
    k_propose<<<gsize(g1_.nvox), 256, 0, s_>>>(psi, out_, out, g1_.nvox, cap);
    if ((rc = cuda(cudaGetLastError(), "k_propose")) != MVR_OK) return rc;
    return cuda(cudaStreamSynchronize(s_), "propose");
}

int UNet::get_params(float *host)
{
    cudaSetDevice(dev_);
    int rc = cuda(cudaMemcpyAsync(host, params_, sizeof(float) * (size_t)nparams_, cudaMemcpyDeviceToHost, s_), "get");
    return rc != MVR_OK ? rc : cuda(cudaStreamSynchronize(s_), "get");
}

int UNet::get_grads(float *host)
{
    cudaSetDevice(dev_);
    int rc = cuda(cudaMemcpyAsync(host, grads_, sizeof(float) * (size_t)nparams_, cudaMemcpyDeviceToHost, s_), "grads");
    return rc != MVR_OK ? rc : cuda(cudaStreamSynchronize(s_), "grads");
}

int UNet::set_params(const float *host)
{
    cudaSetDevice(dev_);
    int rc = cuda(cudaMemcpyAsync(params_, host, sizeof(float) * (size_t)nparams_, cudaMemcpyHostToDevice, s_), "set");
    weights_fresh_ = false;
    return rc != MVR_OK ? rc : cuda(cudaStreamSynchronize(s_), "set");
}

// ---- layer-level entry points (used by the gradient checks) ----------------------------
namespace {
thread_local std::string g_tc_error;
int tc_status(cudaError_t e, int *err_dev, cudaStream_t s)
{
    if (e != cudaSuccess) {
        g_tc_error = cudaGetErrorString(e);
        return MVR_ERR_CUDA;
    }
    int h = 0;
    e = cudaMemcpyAsync(&h, err_dev, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        g_tc_error = cudaGetErrorString(e);
        return MVR_ERR_CUDA;
    }
    if (h) {
        g_tc_error = "tensor-core wait timed out";
        return MVR_ERR_CUDA;
    }
    return MVR_OK;
}
}  // namespace

}  // namespace mvr

// ---- C ABI ----------------------------------------------------------------------------
struct mvr_unet {
    std::unique_ptr<mvr::UNet> net;
};

namespace {
thread_local std::string g_unet_create_error;
}

extern "C" int mvr_unet_create(int batch, const int dims[3], unsigned seed, int device, mvr_unet **out)
{
    if (!out || !dims) return MVR_ERR_ARG;
    *out = nullptr;
    std::unique_ptr<mvr_unet> h(new mvr_unet());
    h->net.reset(new mvr::UNet(batch, dims, seed, device));
    const int rc = h->net->init();
    if (rc != MVR_OK) {
        g_unet_create_error = h->net->error();
        return rc;
    }
    *out = h.release();
    return MVR_OK;
}

extern "C" void mvr_unet_destroy(mvr_unet *h) { delete h; }
extern "C" const char *mvr_unet_last_error(const mvr_unet *h)
{
    return h ? h->net->error().c_str() : g_unet_create_error.c_str();
}
extern "C" long long mvr_unet_num_params(const mvr_unet *h) { return h ? h->net->num_params() : -1; }
extern "C" int mvr_unet_get_params(mvr_unet *h, float *p) { return h && p ? h->net->get_params(p) : MVR_ERR_ARG; }
extern "C" int mvr_unet_set_params(mvr_unet *h, const float *p) { return h && p ? h->net->set_params(p) : MVR_ERR_ARG; }
extern "C" int mvr_unet_get_grads(mvr_unet *h, float *g) { return h && g ? h->net->get_grads(g) : MVR_ERR_ARG; }
extern "C" int mvr_unet_set_input(mvr_unet *h, const float *psi, const float *psi_next, const float *psi_target)
{
    return h ? h->net->set_input(psi, psi_next, psi_target) : MVR_ERR_ARG;
}
// inference: the decoder convolutions read [up(low), skip] directly (the training step keeps the
// concatenations for its backward pass)
extern "C" int mvr_unet_forward(mvr_unet *h, float *pred) { return h ? h->net->forward(pred, true) : MVR_ERR_ARG; }
extern "C" int mvr_unet_train_step(mvr_unet *h, float lr, double *loss)
{
    return h ? h->net->train_step(lr, loss) : MVR_ERR_ARG;
}
extern "C" int mvr_unet_propose(mvr_unet *h, const float *psi, float *out, float cap)
{
    return h && psi && out ? h->net->propose(psi, out, cap) : MVR_ERR_ARG;
}

extern "C" int mvr_conv3d_tc(const void *act, int c_act, const void *weights, int n_out, const float *bias, int relu,
                             int transposed, void *out, const int dims[4], int *err_dev, void *stream)
{
    if (!act || !weights || !out || !dims || !err_dev) return MVR_ERR_ARG;
    mvr::ConvGeom g{dims[3], dims[2], dims[1], dims[0], (long long)dims[0] * dims[1] * dims[2] * dims[3]};
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const cudaError_t e =
        mvr::conv_any(n_out, c_act, transposed ? 1 : 0, static_cast<const __nv_bfloat16 *>(act),
                      static_cast<const __nv_bfloat16 *>(weights), bias, out, g, transposed ? -1 : 1, relu, err_dev, s);
    if (e == cudaErrorInvalidValue) {
        mvr::g_tc_error = "unsupported channel pair";
        return MVR_ERR_UNSUPPORTED;
    }
    return mvr::tc_status(e, err_dev, s);
}

extern "C" int mvr_conv3d_tc_wgrad(const void *x, int c_in, const void *g, int c_out, float *dw, const int dims[4],
                                   int *err_dev, void *stream)
{
    if (!x || !g || !dw || !dims || !err_dev) return MVR_ERR_ARG;
    mvr::ConvGeom gg{dims[3], dims[2], dims[1], dims[0], (long long)dims[0] * dims[1] * dims[2] * dims[3]};
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const cudaError_t e = mvr::wgrad_any(c_out, c_in, static_cast<const __nv_bfloat16 *>(x),
                                         static_cast<const __nv_bfloat16 *>(g), dw, gg, err_dev, s);
    if (e == cudaErrorInvalidValue) {
        mvr::g_tc_error = "unsupported channel pair";
        return MVR_ERR_UNSUPPORTED;
    }
    return mvr::tc_status(e, err_dev, s);
}

extern "C" const char *mvr_conv3d_tc_last_error(void) { return mvr::g_tc_error.c_str(); }

extern "C" int mvr_pool2(const float *in, const int dims[3], float *out, void *stream)
{
    if (!in || !dims || !out || dims[0] < 2 || dims[1] < 2 || dims[2] < 2 || (dims[0] | dims[1] | dims[2]) & 1)
        return MVR_ERR_ARG;
    const long long n = (long long)(dims[0] / 2) * (dims[1] / 2) * (dims[2] / 2);
    mvr::k_pool2_f32<<<mvr::gsize(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(in, dims[0], dims[1], dims[2], out);
    return cudaGetLastError() == cudaSuccess ? MVR_OK : MVR_ERR_CUDA;
}

extern "C" int mvr_apply_coarse(const float *psi_next, const int dims[3], const float *pred_low, const float *psi_low,
                                const float *next_low, float cap, float *out, void *stream)
{
    if (!psi_next || !dims || !pred_low || !psi_low || !next_low || !out || dims[0] < 2 || dims[1] < 2 ||
        dims[2] < 2 || (dims[0] | dims[1] | dims[2]) & 1)
        return MVR_ERR_ARG;
    const long long n = (long long)dims[0] * dims[1] * dims[2];
    mvr::k_apply_coarse<<<mvr::gsize(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        psi_next, dims[0], dims[1], dims[2], pred_low, psi_low, next_low, cap, out);
    return cudaGetLastError() == cudaSuccess ? MVR_OK : MVR_ERR_CUDA;
}
