// Column passes (y or z axis) with one warp per column and warp-shuffle butterflies, for
// column lengths n = R * 32 (R = 2, 3, 4, 5, 6, 8: n = 64 ... 256).
//
// A column is held in registers as a[k1] = c[lane + 32 k1].  The forward transform is
//   1. R-point DFT of the lane's registers,
//   2. twiddle by W_n^(lane k1),
//   3. 32-point decimation-in-frequency FFT across the lanes (__shfl_xor, spans 16..1),
// after which register k1 of lane l holds frequency k1 + R * bitrev5(l).  The spectrum
// is stored in exactly that register layout: storage position p = l + 32 k1 holds
// frequency k1 + R bitrev5(l) ("lane-major order").  The inverse transform is the exact
// algebraic inverse of the three steps in reverse order (decimation-in-time butterflies
// with conjugate twiddles, spans 1..16; conjugate twiddle; inverse R-point DFT), so it
// reads lane-major order and returns natural order, unnormalised (n times the inverse).
//
// Every spectrum along an axis that uses these kernels (the data and the kernel
// spectra K1^, K2^) is produced by the same forward pass, so the spectral product is
// taken position by position and no reordering pass exists anywhere.
//
// A CTA of 8 warps takes NP consecutive x' columns at one index of the other axis (as
// the shared-memory kernels do): the tile is loaded with coalesced NP-wide row segments
// into shared memory (row stride NP + 1), every warp moves its columns between shared
// memory and registers, and the tile is stored back coalesced.
#pragma once
#include "kernels.cuh"

namespace mvr {

template <bool INV>
__device__ __forceinline__ void dft6(float2 *v)
{
    // 6 = 3 x 2 (Cooley-Tukey): inner 3-point DFTs over q = 2 q1 + q2, twiddle
    // W6^(q2 k1), outer 2-point DFTs; output k = k1 + 3 k2.
    float2 e[3] = {v[0], v[2], v[4]}, o[3] = {v[1], v[3], v[5]};
    dft3<INV>(e);
    dft3<INV>(o);
    const float h = 0.8660254037844386f;  // sin(pi/3)
    const float2 w1 = make_float2(0.5f, INV ? h : -h), w2 = make_float2(-0.5f, INV ? h : -h);
    o[1] = cmul(o[1], w1);
    o[2] = cmul(o[2], w2);
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
        v[k1] = cadd(e[k1], o[k1]);
        v[k1 + 3] = csub(e[k1], o[k1]);
    }
}

template <int R, bool INV>
__device__ __forceinline__ void rdft(float2 (&a)[R])
{
    if constexpr (R == 2) dft2<INV>(a);
    else if constexpr (R == 3) dft3<INV>(a);
    else if constexpr (R == 4) dft4<INV>(a);
    else if constexpr (R == 5) dft5<INV>(a);
    else if constexpr (R == 6) dft6<INV>(a);
    else dft8<INV>(a);
}

template <int R>
struct ColTw {
    float2 stage[5];  // W_{2 span}^(lane & (span-1)), span = 16 >> st
    float2 inner[R];  // W_n^(lane k1)
};

template <int R>
__device__ __forceinline__ void col_tw_init(ColTw<R> &t, const float2 *__restrict__ tw, int lane)
{
    constexpr int n = 32 * R;  // tw[j] = exp(-2 pi i j / n)
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int span = 16 >> st;
        t.stage[st] = __ldg(&tw[(lane & (span - 1)) * (n / (2 * span))]);
    }
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) t.inner[k1] = __ldg(&tw[lane * k1]);
}

// natural order -> lane-major spectrum (forward, unnormalised)
template <int R>
__device__ __forceinline__ void col_fwd(float2 (&a)[R], const ColTw<R> &t, int lane)
{
    rdft<R, false>(a);
#pragma unroll
    for (int k1 = 1; k1 < R; ++k1) a[k1] = cmul(a[k1], t.inner[k1]);
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int span = 16 >> st;
        const bool upper = (lane & span) != 0;
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) {
            const float2 o = shfl_x(a[k1], span);
            a[k1] = upper ? cmul(csub(o, a[k1]), t.stage[st]) : cadd(a[k1], o);
        }
    }
}

// lane-major spectrum -> natural order (inverse of col_fwd's steps, times n)
template <int R>
__device__ __forceinline__ void col_inv(float2 (&a)[R], const ColTw<R> &t, int lane)
{
#pragma unroll
    for (int st = 4; st >= 0; --st) {
        const int span = 16 >> st;
        const bool upper = (lane & span) != 0;
        const float2 w = cconj(t.stage[st]);
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) {
            // lower lane holds u = a + b, upper lane v = (a - b) w:  a = u + v w*, b = u - v w*
            const float2 mine = upper ? cmul(a[k1], w) : a[k1];
            const float2 o = shfl_x(mine, span);
            a[k1] = upper ? csub(o, mine) : cadd(mine, o);
        }
    }
#pragma unroll
    for (int k1 = 1; k1 < R; ++k1) a[k1] = cmul(a[k1], cconj(t.inner[k1]));
    rdft<R, true>(a);
}

constexpr int kWColNP = 16;  // columns per tile
constexpr int kWColCPW = kWColNP / 8;  // columns per warp

// MODE 0: forward (natural -> lane-major), 1: inverse (lane-major -> natural),
// 2: forward, multiply by Kh (lane-major), inverse.
template <int R, int MODE>
__global__ void __launch_bounds__(256) k_wcols(const float2 *src, float2 *dst, const float2 *__restrict__ Kh, int Hx,
                                               long long estride, long long ostride, long long Pc,
                                               const float2 *__restrict__ twg)
{
    constexpr int n = 32 * R, NP = kWColNP, PS = NP + 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *A = reinterpret_cast<float2 *>(smem_raw);  // [n][PS]
    float2 *K = A + n * PS;                             // MODE 2: [n][PS]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int x0 = blockIdx.x * NP;
    const long long base = (long long)blockIdx.y * ostride + x0;
    src += (long long)blockIdx.z * Pc;
    dst += (long long)blockIdx.z * Pc;
    const int np = min(NP, Hx - x0);
    ColTw<R> t;
    col_tw_init<R>(t, twg, lane);
    constexpr int tot = n * NP;
    constexpr int step = 256 * kLoadBatch;
    for (int t0 = threadIdx.x; t0 < tot; t0 += step) {
        float2 r[kLoadBatch], k[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int e = t0 + u * 256;
            const int p = e % NP, i = e / NP;
            const bool ok = e < tot && p < np;
            r[u] = ok ? src[base + i * estride + p] : make_float2(0.0f, 0.0f);
            if (MODE == 2) k[u] = ok ? __ldg(&Kh[base + i * estride + p]) : make_float2(0.0f, 0.0f);
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int e = t0 + u * 256;
            if (e < tot) {
                const int p = e % NP, i = e / NP;
                A[i * PS + p] = r[u];
                if (MODE == 2) K[i * PS + p] = k[u];
            }
        }
    }
    __syncthreads();
    // kWColCPW columns per warp, transformed together for instruction-level parallelism
    float2 a[kWColCPW][R];
#pragma unroll
    for (int j = 0; j < kWColCPW; ++j) {
        const int c = warp + 8 * j;
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) a[j][k1] = A[(lane + 32 * k1) * PS + c];
    }
    if (MODE != 1) {
#pragma unroll
        for (int j = 0; j < kWColCPW; ++j) col_fwd<R>(a[j], t, lane);
    }
    if (MODE == 2) {
#pragma unroll
        for (int j = 0; j < kWColCPW; ++j) {
            const int c = warp + 8 * j;
#pragma unroll
            for (int k1 = 0; k1 < R; ++k1) a[j][k1] = cmul(a[j][k1], K[(lane + 32 * k1) * PS + c]);
        }
    }
    if (MODE != 0) {
#pragma unroll
        for (int j = 0; j < kWColCPW; ++j) col_inv<R>(a[j], t, lane);
    }
#pragma unroll
    for (int j = 0; j < kWColCPW; ++j) {
        const int c = warp + 8 * j;
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) A[(lane + 32 * k1) * PS + c] = a[j][k1];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < tot; e += 256) {
        const int p = e % NP, i = e / NP;
        if (p < np) dst[base + i * estride + p] = A[i * PS + p];
    }
}

// Shared memory of k_wcols<R, MODE>.
inline size_t wcols_smem(int R, int mode) { return sizeof(float2) * (size_t)(32 * R) * (kWColNP + 1) * (mode == 2 ? 2 : 1); }

}  // namespace mvr
