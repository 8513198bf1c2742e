// Row passes with one warp per x-row and warp-shuffle butterflies, for half lengths
// m = R * 32 (R = 2, 3, 4: rows of 128, 192, 256 reals).
//
// Forward m-point FFT of z[0..m) held as a[s] = z[lane + 32 s] (Cooley-Tukey with
// m = R * 32, input index q = lane + 32 q1, output index k = k1 + R k2):
//   1. R-point DFT of the lane's registers:   b[k1] = sum_q1 a[q1] W_R^(q1 k1)
//   2. twiddle:                               b[k1] *= W_m^(lane k1)
//   3. 32-point decimation-in-frequency FFT across the lanes of each b[k1] with
//      __shfl_xor (radix 2, spans 16..1), leaving lane l with Z[k1 + R bitrev5(l)].
// The inverse uses conjugate twiddles.  A per-warp shared row puts the result back in
// natural order.  No block-wide barrier is involved, and all twiddles that do not
// depend on the row are computed once per thread.
#pragma once
#include "kernels.cuh"

namespace mvr {

template <int R>
struct WarpTw {
    float2 stage[5];   // W_{2 span}^(lane & (span-1)), span = 16 >> st
    float2 inner[R];   // W_m^(lane k1)
    float2 post[R];    // W_{2m}^(lane + 32 s): packed-real split
};

template <int R>
__device__ __forceinline__ void warp_tw_init(WarpTw<R> &t, const float2 *__restrict__ tw, int Px, int lane)
{
    // tw[j] = exp(-2 pi i j / Px), Px = 2m = 64 R
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int span = 16 >> st;
        t.stage[st] = __ldg(&tw[(lane & (span - 1)) * (Px / (2 * span))]);
    }
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) t.inner[k1] = __ldg(&tw[2 * lane * k1]);
#pragma unroll
    for (int s = 0; s < R; ++s) t.post[s] = __ldg(&tw[lane + 32 * s]);
}

__device__ __forceinline__ float2 shfl_x(float2 v, int m)
{
    return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

__device__ __forceinline__ int bitrev5(int l) { return (int)(__brev((unsigned)l) >> 27); }

template <int R, bool INV>
__device__ __forceinline__ void warp_fft(float2 (&a)[R], const WarpTw<R> &t, int lane)
{
    if constexpr (R == 2) dft2<INV>(a);
    else if constexpr (R == 3) dft3<INV>(a);
    else dft4<INV>(a);
#pragma unroll
    for (int k1 = 1; k1 < R; ++k1) a[k1] = cmul(a[k1], INV ? cconj(t.inner[k1]) : t.inner[k1]);
#pragma unroll
    for (int st = 0; st < 5; ++st) {
        const int span = 16 >> st;
        const bool upper = (lane & span) != 0;
        const float2 w = INV ? cconj(t.stage[st]) : t.stage[st];
#pragma unroll
        for (int k1 = 0; k1 < R; ++k1) {
            const float2 o = shfl_x(a[k1], span);
            a[k1] = upper ? cmul(csub(o, a[k1]), w) : cadd(a[k1], o);
        }
    }
}

// Result of warp_fft into the warp's shared row, natural order.
template <int R>
__device__ __forceinline__ void warp_store_natural(const float2 (&a)[R], float2 *row, int lane)
{
    const int br = bitrev5(lane);
#pragma unroll
    for (int k1 = 0; k1 < R; ++k1) row[k1 + R * br] = a[k1];
    __syncwarp();
}

// Packed-real split of the natural-order FFT in `row` into X[0..m] of S row `out`.
template <int R>
__device__ __forceinline__ void warp_r2c_post(const float2 *row, float2 *__restrict__ out, const WarpTw<R> &t, int lane)
{
    constexpr int m = 32 * R;
#pragma unroll
    for (int s = 0; s < R; ++s) {
        const int k = lane + 32 * s;
        const float2 zk = row[k];
        const float2 zc = cconj(row[k == 0 ? 0 : m - k]);
        const float2 e = cscale(cadd(zk, zc), 0.5f);
        const float2 dd = cscale(csub(zk, zc), 0.5f);
        out[k] = cadd(e, cmul(t.post[s], make_float2(dd.y, -dd.x)));
    }
    if (lane == 0) {  // Nyquist bin k = m: Re Z0 - Im Z0
        const float2 z0 = row[0];
        out[m] = make_float2(z0.x - z0.y, 0.0f);
    }
    __syncwarp();
}

// S row -> packed Z' in registers (natural order a[s] = Z'[lane + 32 s]).
template <int R>
__device__ __forceinline__ void warp_c2r_pre(const float2 *__restrict__ in, float2 (&a)[R], const WarpTw<R> &t, int lane)
{
    constexpr int m = 32 * R;
    float2 xk[R], xc[R];
#pragma unroll
    for (int s = 0; s < R; ++s) {
        const int k = lane + 32 * s;
        xk[s] = in[k];
        xc[s] = in[m - k];
    }
#pragma unroll
    for (int s = 0; s < R; ++s) {
        const float2 c = cconj(xc[s]);
        const float2 e = cadd(xk[s], c);
        const float2 o = cmul(csub(xk[s], c), cconj(t.post[s]));
        a[s] = make_float2(e.x - o.y, e.y + o.x);
    }
}

// Row-invariant x mappings, computed once per CTA into shared memory: the volume x of
// every domain x depends on the block only, not on the row.
struct RowX {
    int mir[256];  // psi: volume x under the mirror mapping
    int zx[256];   // img / weight: volume x of a block voxel inside the volume, else -1
};

// domain_ext: x is a domain index (extension wraps to negative block x); otherwise a
// block index.  Ends with a CTA barrier.
__device__ __forceinline__ void row_x_init(RowX &rx, const BlockMap &bm, int Px, bool domain_ext)
{
    for (int x = threadIdx.x; x < Px; x += blockDim.x) {
        rx.mir[x] = (int)mirror_x(bm, x);
        const int bx = domain_ext ? ext_e(x, bm.P[0], bm.L[0]) : x;
        const long long gx = bm.off[0] + bx;
        rx.zx[x] = (bx >= 0 && bx < bm.b[0] && gx >= 0 && gx < bm.D[0]) ? (int)gx : -1;
    }
    __syncthreads();
}

// ---- forward: extract psi (mirror-single) + R2C -----------------------------------------
template <int R>
__global__ void __launch_bounds__(256) k_wrows_fwd(const float *__restrict__ psi, float2 *__restrict__ S,
                                                   const BlockMaps bms, long long Pc, const float2 *__restrict__ twg)
{
    constexpr int m = 32 * R;
    __shared__ float2 srow[8][m + 1];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const BlockMap &bm = bms.m[blockIdx.y];
    float2 *Sb = S + (long long)blockIdx.y * Pc;
    WarpTw<R> t;
    warp_tw_init<R>(t, twg, 2 * m, lane);
    __shared__ RowX rx;
    row_x_init(rx, bm, 2 * m, true);
    const long long nrows = (long long)bm.P[1] * bm.P[2];
    for (long long row = (long long)blockIdx.x * 8 + wib; row < nrows; row += (long long)gridDim.x * 8) {
        const int z = (int)((unsigned)row / (unsigned)bm.P[1]), y = (int)row - z * bm.P[1];  // rows < 2^31
        const float *pr = psi + mirror_row(bm, y, z).base;
        float2 a[R];
#pragma unroll
        for (int s = 0; s < R; ++s) {
            const int x = 2 * (lane + 32 * s);
            a[s] = make_float2(__ldg(pr + rx.mir[x]), __ldg(pr + rx.mir[x + 1]));
        }
        warp_fft<R, false>(a, t, lane);
        warp_store_natural<R>(a, srow[wib], lane);
        warp_r2c_post<R>(srow[wib], Sb + row * (m + 1), t, lane);
    }
}

// ---- C2R -> quotient -> R2C ----------------------------------------------------------
// DeconvolutionMethods.java:71-74: img > 0 ? img / conv1 : 1.  Voxels outside the
// block (the value-1 extension) and outside the volume (img zero-extended) both give 1,
// so they are read as img = 0.
template <int R>
__global__ void __launch_bounds__(256) k_wrows_ratio(float2 *__restrict__ S, const float *__restrict__ img,
                                                     const BlockMaps bms, long long Pc, const float2 *__restrict__ twg)
{
    constexpr int m = 32 * R;
    __shared__ float2 srow[8][m + 1];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const BlockMap &bm = bms.m[blockIdx.y];
    float2 *Sb = S + (long long)blockIdx.y * Pc;
    WarpTw<R> t;
    warp_tw_init<R>(t, twg, 2 * m, lane);
    __shared__ RowX rx;
    row_x_init(rx, bm, 2 * m, true);
    const long long nrows = (long long)bm.P[1] * bm.P[2];
    for (long long row = (long long)blockIdx.x * 8 + wib; row < nrows; row += (long long)gridDim.x * 8) {
        float2 *Srow = Sb + row * (m + 1);
        float2 a[R];
        warp_c2r_pre<R>(Srow, a, t, lane);
        const int z = (int)((unsigned)row / (unsigned)bm.P[1]), y = (int)row - z * bm.P[1];  // rows < 2^31
        const int ey = ext_e(y, bm.P[1], bm.L[1]), ez = ext_e(z, bm.P[2], bm.L[2]);
        const bool rin = ey >= 0 && ey < bm.b[1] && ez >= 0 && ez < bm.b[2];
        const long long zb = rin ? zero_row(bm, ey, ez).base : -1;
        float im[R][2];
#pragma unroll
        for (int s = 0; s < R; ++s)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int gx = rx.zx[2 * (lane + 32 * s) + h];
                im[s][h] = (zb >= 0 && gx >= 0) ? __ldg(img + zb + gx) : 0.0f;
            }
        warp_fft<R, true>(a, t, lane);
        warp_store_natural<R>(a, srow[wib], lane);
#pragma unroll
        for (int s = 0; s < R; ++s) {
            const float2 c = srow[wib][lane + 32 * s];  // conv1 at x = 2q, 2q+1
            a[s] = make_float2(quotient_fast(im[s][0], c.x), quotient_fast(im[s][1], c.y));
        }
        __syncwarp();
        warp_fft<R, false>(a, t, lane);
        warp_store_natural<R>(a, srow[wib], lane);
        warp_r2c_post<R>(srow[wib], Srow, t, lane);
    }
}

// ---- C2R -> sequential update (FP64 block statistics) ---------------------------------
template <int R>
__global__ void __launch_bounds__(256) k_wrows_update(float2 *__restrict__ S, UpdateArgs ua, const BlockMaps bms,
                                                      long long Pc, const float2 *__restrict__ twg)
{
    constexpr int m = 32 * R;
    __shared__ float2 srow[8][m + 1];
    __shared__ double red_s[8], red_m[8];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const BlockMap &bm = bms.m[blockIdx.y];
    float2 *Sb = S + (long long)blockIdx.y * Pc;
    WarpTw<R> t;
    warp_tw_init<R>(t, twg, 2 * m, lane);
    __shared__ RowX rx;
    row_x_init(rx, bm, 2 * m, false);
    unsigned inb = 0, wr = 0;  // bit (2s+h): x inside the block / inside the written region
#pragma unroll
    for (int s = 0; s < R; ++s)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int x = 2 * (lane + 32 * s) + h;
            if (x < bm.b[0]) inb |= 1u << (2 * s + h);
            if (x < bm.b[0] && x >= bm.wlo[0] && x < bm.whi[0]) wr |= 1u << (2 * s + h);
        }
    const float *psrc = reinterpret_cast<const float *>(ua.psi_src);
    float *pdst = reinterpret_cast<float *>(ua.psi_dst);
    const float *wgt = ua.weight[0];
    UpdConst uc;
    uc.minI = ua.minI;
    uc.maxI = ua.maxI;
    uc.inv_maxI = 1.0f / ua.maxI;
    uc.two_lambda = ua.two_lambda;
    uc.tik = ua.tik != 0;
    float ksum = 0.0f, kcomp = 0.0f, kmax = -1.0f;
    // all rows, or (prune) the rows of the write region's planes
    const long long r0 = ua.prune ? (long long)bm.wlo[2] * bm.P[1] : 0;
    const long long nrows = ua.prune ? (long long)bm.whi[2] * bm.P[1] : (long long)bm.P[1] * bm.P[2];
    for (long long row = r0 + (long long)blockIdx.x * 8 + wib; row < nrows; row += (long long)gridDim.x * 8) {
        const int z = (int)((unsigned)row / (unsigned)bm.P[1]), y = (int)row - z * bm.P[1];  // rows < 2^31
        if (y >= bm.b[1] || z >= bm.b[2]) continue;  // extension rows carry no block voxels
        const bool wrow = y >= bm.wlo[1] && y < bm.whi[1] && z >= bm.wlo[2] && z < bm.whi[2];
        if (ua.prune && !wrow) continue;
        float2 a[R];
        warp_c2r_pre<R>(Sb + row * (m + 1), a, t, lane);
        const float *pr = psrc + mirror_row(bm, y, z).base;
        const long long zb = zero_row(bm, y, z).base;
        float lastv[R][2], wv[R][2];
#pragma unroll
        for (int s = 0; s < R; ++s)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = 2 * (lane + 32 * s) + h;
                const bool ok = (inb >> (2 * s + h)) & 1u;
                const int gx = rx.zx[x];
                lastv[s][h] = ok ? __ldg(pr + rx.mir[x]) : 0.0f;
                wv[s][h] = (ok && zb >= 0 && gx >= 0) ? __ldg(wgt + zb + gx) : 0.0f;
            }
        warp_fft<R, true>(a, t, lane);
        warp_store_natural<R>(a, srow[wib], lane);
        float *orow = pdst + ((bm.ooff[2] + z) * bm.OD[1] + (bm.ooff[1] + y)) * bm.OD[0] + bm.ooff[0];
#pragma unroll
        for (int s = 0; s < R; ++s) {
            const float2 c = srow[wib][lane + 32 * s];
            const float cv[2] = {c.x, c.y};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (!((inb >> (2 * s + h)) & 1u)) continue;
                const float last = lastv[s][h];
                const float next = next_value_fast(last, cv[h], wv[s][h], uc);
                const float ch = next - last;  // signed change (DeconvolutionMethods.java:308)
                const float ky = ch - kcomp;
                const float kt = ksum + ky;
                kcomp = (kt - ksum) - ky;
                ksum = kt;
                kmax = kmax > ch ? kmax : ch;
                if (wrow && ((wr >> (2 * s + h)) & 1u)) orow[2 * (lane + 32 * s) + h] = next;
            }
        }
        __syncwarp();
    }
    if (!ua.prune)
        stats_to_partials(ksum, kcomp, kmax, red_s, red_m, ua.partials, (long long)blockIdx.y * gridDim.x + blockIdx.x);
}

}  // namespace mvr
