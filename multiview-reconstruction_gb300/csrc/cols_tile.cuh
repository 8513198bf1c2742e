// Column passes (y or z axis) as a two-phase register FFT over a shared-memory tile, for
// FP32 column lengths n = V * 16 (V = 4, 6, 8, 12, 16, 18: n = 64 ... 288).
//
// With n = V * T (T = 16), column element i = t + T v (t < T, v < V):
//   phase 1, item (column, t):  V-point DFT over v of x[t + T v], times W_n^(t k1),
//                               written back in place to positions t + T k1;
//   phase 2, item (column, k1): T-point DFT over t of positions t + T k1, written back in
//                               place: position k2 + T k1 holds frequency k1 + V k2.
// Every thread keeps its V or T values in registers; the exchange between the phases is
// one pass through shared memory.  The spectrum stays in that order ("tile order"), and
// every spectrum along the axis (data and kernel spectra K1^, K2^) is produced by the
// same forward pass, so the spectral product is taken position by position.  The
// inverse runs the exact inverse of each phase in reverse order and returns natural
// order, unnormalised (n times the inverse DFT).
//
// A CTA of 256 threads takes 16 consecutive x' columns at one index of the other axis;
// the tile moves between HBM and shared memory in coalesced 16-wide row segments.
// MODE 2 multiplies by K^ in phase 2, reading it from L2 (every block of a batch shares
// one K^) or, with MVR_TCOLS_KS=1, from a staged shared-memory tile.  A gathered tile (pstride > 1)
// takes one x' column at 16 consecutive indices of the other axis instead: the last
// column of a spectrum with Hx = 16 q + 1 (the Nyquist column) goes that way, so no
// CTA works on a tile with a single live column.
#pragma once
#include "cols_warp.cuh"
#include "pdl.cuh"

namespace mvr {

// 12 = 4 x 3 (Cooley-Tukey): inner 4-point DFTs over q = 3 q1 + q2, twiddle
// W12^(q2 k1), outer 3-point DFTs; output k = k1 + 4 k2.
template <bool INV>
__device__ __forceinline__ void dft12(float2 *v)
{
    float2 u[3][4];
#pragma unroll
    for (int q2 = 0; q2 < 3; ++q2) {
#pragma unroll
        for (int q1 = 0; q1 < 4; ++q1) u[q2][q1] = v[3 * q1 + q2];
        dft4<INV>(u[q2]);
    }
    const float h = 0.8660254037844386f;  // cos(pi/6) = sin(pi/3)
    const float sg = INV ? 1.0f : -1.0f;
    // W12^1 = (h, -1/2), W12^2 = (1/2, -h), W12^3 = -i, W12^4 = (-1/2, -h), W12^6 = -1
    u[1][1] = cmul(u[1][1], make_float2(h, sg * 0.5f));
    u[1][2] = cmul(u[1][2], make_float2(0.5f, sg * h));
    u[1][3] = mul_j<INV>(u[1][3]);
    u[2][1] = cmul(u[2][1], make_float2(0.5f, sg * h));
    u[2][2] = cmul(u[2][2], make_float2(-0.5f, sg * h));
    u[2][3] = make_float2(-u[2][3].x, -u[2][3].y);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        float2 w[3] = {u[0][k1], u[1][k1], u[2][k1]};
        dft3<INV>(w);
#pragma unroll
        for (int k2 = 0; k2 < 3; ++k2) v[k1 + 4 * k2] = w[k2];
    }
}

// 16 = 4 x 4: inner 4-point DFTs over q = 4 q1 + q2, twiddle W16^(q2 k1), outer 4-point
// DFTs; output k = k1 + 4 k2.
template <bool INV>
__device__ __forceinline__ void dft16(float2 *v)
{
    float2 u[4][4];
#pragma unroll
    for (int q2 = 0; q2 < 4; ++q2) {
#pragma unroll
        for (int q1 = 0; q1 < 4; ++q1) u[q2][q1] = v[4 * q1 + q2];
        dft4<INV>(u[q2]);
    }
    const float c = 0.92387953251128674f, s = 0.38268343236508977f, r = 0.70710678118654752f;
    const float sg = INV ? 1.0f : -1.0f;
    // W16^j = (cos(2 pi j / 16), -+ sin(2 pi j / 16))
    const float2 w1 = make_float2(c, sg * s), w2 = make_float2(r, sg * r), w3 = make_float2(s, sg * c);
    const float2 w6 = make_float2(-r, sg * r), w9 = make_float2(-c, -sg * s);
    u[1][1] = cmul(u[1][1], w1);
    u[1][2] = cmul(u[1][2], w2);
    u[1][3] = cmul(u[1][3], w3);
    u[2][1] = cmul(u[2][1], w2);
    u[2][2] = mul_j<INV>(u[2][2]);
    u[2][3] = cmul(u[2][3], w6);
    u[3][1] = cmul(u[3][1], w3);
    u[3][2] = cmul(u[3][2], w6);
    u[3][3] = cmul(u[3][3], w9);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        float2 w[4] = {u[0][k1], u[1][k1], u[2][k1], u[3][k1]};
        dft4<INV>(w);
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = w[k2];
    }
}

// 9 = 3 x 3 (Cooley-Tukey): inner 3-point DFTs over q = 3 q1 + q2, twiddle W9^(q2 k1), outer
// 3-point DFTs; output k = k1 + 3 k2.
template <bool INV>
__device__ __forceinline__ void dft9(float2 *v)
{
    float2 u[3][3];
#pragma unroll
    for (int q2 = 0; q2 < 3; ++q2) {
#pragma unroll
        for (int q1 = 0; q1 < 3; ++q1) u[q2][q1] = v[3 * q1 + q2];
        dft3<INV>(u[q2]);
    }
    const float sg = INV ? 1.0f : -1.0f;
    // W9^j = (cos(2 pi j / 9), -+ sin(2 pi j / 9)), j = 1, 2, 4
    const float2 w1 = make_float2(0.76604444311897804f, sg * 0.64278760968653933f);
    const float2 w2 = make_float2(0.17364817766693035f, sg * 0.98480775301220806f);
    const float2 w4 = make_float2(-0.93969262078590838f, sg * 0.34202014332566873f);
    u[1][1] = cmul(u[1][1], w1);
    u[1][2] = cmul(u[1][2], w2);
    u[2][1] = cmul(u[2][1], w2);
    u[2][2] = cmul(u[2][2], w4);
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
        float2 w[3] = {u[0][k1], u[1][k1], u[2][k1]};
        dft3<INV>(w);
#pragma unroll
        for (int k2 = 0; k2 < 3; ++k2) v[k1 + 3 * k2] = w[k2];
    }
}

// 18 = 2 x 9: the 9-point DFTs of the even and odd inputs, X[k] = E[k] + W18^k O[k],
// X[k + 9] = E[k] - W18^k O[k].
template <bool INV>
__device__ __forceinline__ void dft18(float2 *v)
{
    float2 e[9], o[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        e[j] = v[2 * j];
        o[j] = v[2 * j + 1];
    }
    dft9<INV>(e);
    dft9<INV>(o);
    const float sg = INV ? 1.0f : -1.0f;
    // W18^k = (cos(pi k / 9), -+ sin(pi k / 9)), k = 1 .. 8
    const float c[8] = {0.93969262078590838f, 0.76604444311897804f, 0.5f, 0.17364817766693035f,
                        -0.17364817766693035f, -0.5f, -0.76604444311897804f, -0.93969262078590838f};
    const float sn[8] = {0.34202014332566873f, 0.64278760968653933f, 0.86602540378443865f, 0.98480775301220806f,
                         0.98480775301220806f, 0.86602540378443865f, 0.64278760968653933f, 0.34202014332566873f};
#pragma unroll
    for (int k = 1; k < 9; ++k) o[k] = cmul(o[k], make_float2(c[k - 1], sg * sn[k - 1]));
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        v[k] = cadd(e[k], o[k]);
        v[k + 9] = csub(e[k], o[k]);
    }
}

template <int N, bool INV>
__device__ __forceinline__ void sdft(float2 (&a)[N])
{
    if constexpr (N == 4) dft4<INV>(a);
    else if constexpr (N == 6) dft6<INV>(a);
    else if constexpr (N == 8) dft8<INV>(a);
    else if constexpr (N == 12) dft12<INV>(a);
    else if constexpr (N == 18) dft18<INV>(a);
    else dft16<INV>(a);
}

constexpr int kTColT = 16;   // phase-2 length
constexpr int kTColNP = 16;  // columns per tile

// Build-time knobs: MVR_TCOLS_KS=1 stages the K^ tile in shared memory with the data tile
// (MODE 2) instead of reading K^ from L2 in phase 2, and MVR_TCOLS_MINB sets the register
// budget (CTAs per SM).  Measured on GB300 for the 192-long Z pass: K^ from L2 at 3 CTAs per
// SM 4.99 TB/s, staged 4.80 TB/s, from L2 at 4 CTAs per SM (64 registers) 4.54 TB/s.
#ifndef MVR_TCOLS_KS
#define MVR_TCOLS_KS 0
#endif
#ifndef MVR_TCOLS_MINB
#define MVR_TCOLS_MINB 3
#endif

// NP columns per tile with 16 NP threads (NP = 16: 256 threads, 3 CTAs per SM).  Measured on
// GB300 for the 192-long Z pass: 32-column tiles (512 threads, 256-byte row segments, 2 CTAs
// per SM) ran at 3.5 TB/s against 4.5 TB/s for 16-column tiles.
// The 288-long columns (V = 18) take 2 CTAs per SM: at 3 the 18-point transforms spill.
template <int V, int MODE, int NP = kTColNP>
__global__ void __launch_bounds__(16 * NP, (NP == 16 && V <= 16) ? MVR_TCOLS_MINB : 2)
    k_tcols(const float2 *src, float2 *dst, const float2 *__restrict__ Kh, int Hx, long long estride,
            long long ostride, long long Pc, const float2 *__restrict__ twg, int gather, int nother, int rlo, int rhi,
            int olo, int llo, int lhi)
{
    constexpr int T = kTColT, n = V * T, NT = 16 * NP;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *A = reinterpret_cast<float2 *>(smem_raw);  // [n][NP]
    float2 *tw = A + n * NP;                            // [n]: exp(-2 pi i j / n)
    float2 *KA = tw + n;                                // MODE 2: [n][NP] tile of K^
    pdl_trigger();
    for (int i = threadIdx.x; i < n; i += NT) tw[i] = __ldg(&twg[i]);
    // tile column p of row i at base + i * estride + p * pstride.  The grid covers the
    // other-axis indices olo + blockIdx.y < nother.  With gather, the last x tile of the grid
    // is the gathered tile of the last column (Hx - 1) at the other-axis indices
    // olo + 16 blockIdx.y ...; the other tiles cover columns < Hx - 1.
    const bool gtile = gather && blockIdx.x == gridDim.x - 1;
    if (gtile && olo + (int)blockIdx.y * NP >= nother) return;  // the whole CTA, before any barrier
    long long base, pstride;
    int np;
    if (!gtile) {
        const int x0 = blockIdx.x * NP;
        base = (long long)(olo + blockIdx.y) * ostride + x0;
        np = min(NP, (gather ? Hx - 1 : Hx) - x0);
        pstride = 1;
    } else {
        const int o0 = olo + blockIdx.y * NP;
        base = (long long)o0 * ostride + (Hx - 1);
        np = min(NP, nother - o0);
        pstride = ostride;
    }
    src += (long long)blockIdx.z * Pc;
    dst += (long long)blockIdx.z * Pc;
    constexpr int tot = n * NP;
    // every thread keeps one column p = threadIdx % NP and the rows threadIdx / NP + 16 j,
    // j < R, loaded in batches of LB with all loads of a batch in flight
    constexpr int R = tot / NT, LB = (R % 8 == 0) ? 8 : ((R % 6 == 0) ? 6 : 4);
    static_assert(R % LB == 0, "load batches");
    const int pc = threadIdx.x % NP;
    const bool plive = pc < np;
    const long long coff = base + (long long)pc * pstride + (long long)(threadIdx.x / NP) * estride;
    const long long rstep = (long long)(NT / NP) * estride;
    pdl_wait();  // the spectra are the predecessor's output
    {
        const float2 *sp = src + coff;
        const float2 *kp = Kh + coff;
#pragma unroll
        for (int j0 = 0; j0 < R; j0 += LB) {
            float2 r[LB], q[LB];
#pragma unroll
            for (int u = 0; u < LB; ++u) {
                // rows outside [llo, lhi) are read as zeros (the caller's input is zero there)
                const int row = (int)(threadIdx.x / NP) + (NT / NP) * (j0 + u);
                r[u] = (plive && row >= llo && row < lhi) ? sp[(j0 + u) * rstep] : make_float2(0.0f, 0.0f);
                if (MODE == 2 && MVR_TCOLS_KS) q[u] = plive ? __ldg(kp + (j0 + u) * rstep) : make_float2(0.0f, 0.0f);
            }
#pragma unroll
            for (int u = 0; u < LB; ++u) {
                A[threadIdx.x + (j0 + u) * NT] = r[u];
                if (MODE == 2 && MVR_TCOLS_KS) KA[threadIdx.x + (j0 + u) * NT] = q[u];
            }
        }
    }
    __syncthreads();
    const int c = threadIdx.x % NP;
    // items of columns beyond the domain (the last tile of Hx = 16 q + 1 columns holds
    // one) skip their transforms
    const bool live = c < np;
    if (MODE != 1 && live) {  // phase 1 forward: item (c, t)
        const int t = threadIdx.x / NP;
        float2 a[V];
#pragma unroll
        for (int v = 0; v < V; ++v) a[v] = A[(t + T * v) * NP + c];
        sdft<V, false>(a);
#pragma unroll
        for (int k1 = 1; k1 < V; ++k1) a[k1] = cmul(a[k1], tw[t * k1]);
#pragma unroll
        for (int k1 = 0; k1 < V; ++k1) A[(t + T * k1) * NP + c] = a[k1];
    }
    if (MODE != 1) __syncthreads();
    // phase 2: items (c, k1), k1 = threadIdx / NP, + NT / NP, ... (more than one round for V > 16)
    for (int k1 = threadIdx.x / NP; k1 < V; k1 += NT / NP) {
        if (live) {
            float2 b[T];
#pragma unroll
            for (int t = 0; t < T; ++t) b[t] = A[(t + T * k1) * NP + c];
            if (MODE != 1) sdft<T, false>(b);
            if (MODE == 2) {
                if (MVR_TCOLS_KS) {
#pragma unroll
                    for (int k2 = 0; k2 < T; ++k2) b[k2] = cmul(b[k2], KA[(k2 + T * k1) * NP + c]);
                } else {
                    const float2 *kq = Kh + base + (long long)c * pstride + (long long)(T * k1) * estride;
#pragma unroll
                    for (int k2 = 0; k2 < T; ++k2) b[k2] = cmul(b[k2], __ldg(kq + (long long)k2 * estride));
                }
            }
            if (MODE != 0) sdft<T, true>(b);
#pragma unroll
            for (int t = 0; t < T; ++t) A[(t + T * k1) * NP + c] = b[t];
        }
    }
    __syncthreads();
    if (MODE != 0 && live) {  // phase 1 inverse: item (c, t)
        const int t = threadIdx.x / NP;
        float2 a[V];
#pragma unroll
        for (int k1 = 0; k1 < V; ++k1) a[k1] = A[(t + T * k1) * NP + c];
#pragma unroll
        for (int k1 = 1; k1 < V; ++k1) a[k1] = cmul(a[k1], cconj(tw[t * k1]));
        sdft<V, true>(a);
#pragma unroll
        for (int v = 0; v < V; ++v) A[(t + T * v) * NP + c] = a[v];
    }
    if (MODE != 0) __syncthreads();
    // rows [rlo, rhi) of the transformed axis are stored (all of them unless the caller
    // reads only a sub-range)
    if (plive) {
        float2 *dp = dst + coff;
        const int prow = threadIdx.x / NP;
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const int row = prow + (NT / NP) * j;
            if (row >= rlo && row < rhi) dp[j * rstep] = A[threadIdx.x + j * NT];
        }
    }
}

// data tile + twiddles (+ the K^ tile of MODE 2)
inline size_t tcols_smem(int V, int mode = 2, int np = kTColNP)
{
    const size_t n = (size_t)V * kTColT;
    return sizeof(float2) * (n * np + n + (mode == 2 && MVR_TCOLS_KS ? n * np : 0));
}

}  // namespace mvr
