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

// ---- forward: extract + R2C ----------------------------------------------------------
template <int R, class Src>
__global__ void __launch_bounds__(256) k_wrows_fwd(Src src, float2 *__restrict__ S, const BlockMaps bms, long long Pc,
                                                   const float2 *__restrict__ twg)
{
    constexpr int m = 32 * R;
    __shared__ float2 srow[8][m + 1];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const BlockMap &bm = bms.m[blockIdx.y];
    float2 *Sb = S + (long long)blockIdx.y * Pc;
    WarpTw<R> t;
    warp_tw_init<R>(t, twg, 2 * m, lane);
    const long long nrows = (long long)bm.P[1] * bm.P[2];
    for (long long row = (long long)blockIdx.x * 8 + wib; row < nrows; row += (long long)gridDim.x * 8) {
        const int y = (int)(row % bm.P[1]), z = (int)(row / bm.P[1]);
        const typename Src::Row Rw = src.row(bm, y, z);
        float2 a[R];
#pragma unroll
        for (int s = 0; s < R; ++s) {
            const int q = lane + 32 * s;
            a[s] = make_float2(src.template at<float>(Rw, bm, 2 * q), src.template at<float>(Rw, bm, 2 * q + 1));
        }
        warp_fft<R, false>(a, t, lane);
        warp_store_natural<R>(a, srow[wib], lane);
        warp_r2c_post<R>(srow[wib], Sb + row * (m + 1), t, lane);
    }
}

// ---- C2R -> quotient -> R2C ----------------------------------------------------------
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
    const long long nrows = (long long)bm.P[1] * bm.P[2];
    for (long long row = (long long)blockIdx.x * 8 + wib; row < nrows; row += (long long)gridDim.x * 8) {
        float2 *Srow = Sb + row * (m + 1);
        float2 a[R];
        warp_c2r_pre<R>(Srow, a, t, lane);
        warp_fft<R, true>(a, t, lane);
        warp_store_natural<R>(a, srow[wib], lane);
        const int y = (int)(row % bm.P[1]), z = (int)(row / bm.P[1]);
        const int ey = ext_e(y, bm.P[1], bm.L[1]), ez = ext_e(z, bm.P[2], bm.L[2]);
        const bool rin = ey >= 0 && ey < bm.b[1] && ez >= 0 && ez < bm.b[2];
        const ZeroRow zr = rin ? zero_row(bm, ey, ez) : ZeroRow{-1};
        float im[R][2];
#pragma unroll
        for (int s = 0; s < R; ++s) {
            const int q = lane + 32 * s;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int ex = ext_e(2 * q + h, bm.P[0], bm.L[0]);
                im[s][h] = (rin && ex >= 0 && ex < bm.b[0]) ? zero_at(img, bm, zr, ex) : -1.0f;
            }
        }
#pragma unroll
        for (int s = 0; s < R; ++s) {
            const float2 c = srow[wib][lane + 32 * s];  // conv1 at x = 2q, 2q+1
            a[s] = make_float2(im[s][0] < 0.0f ? 1.0f : quotient(im[s][0], c.x),
                               im[s][1] < 0.0f ? 1.0f : quotient(im[s][1], c.y));
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
    const float *psrc = reinterpret_cast<const float *>(ua.psi_src);
    float *pdst = reinterpret_cast<float *>(ua.psi_dst);
    float ksum = 0.0f, kcomp = 0.0f, kmax = -1.0f;
    const long long nrows = (long long)bm.P[1] * bm.P[2];
    for (long long row = (long long)blockIdx.x * 8 + wib; row < nrows; row += (long long)gridDim.x * 8) {
        const int y = (int)(row % bm.P[1]), z = (int)(row / bm.P[1]);
        if (y >= bm.b[1] || z >= bm.b[2]) continue;  // extension rows carry no block voxels
        float2 a[R];
        warp_c2r_pre<R>(Sb + row * (m + 1), a, t, lane);
        warp_fft<R, true>(a, t, lane);
        warp_store_natural<R>(a, srow[wib], lane);
        const ZeroRow zr = zero_row(bm, y, z);
        const MirrorRow mr = mirror_row(bm, y, z);
        const bool wrow = y >= bm.wlo[1] && y < bm.whi[1] && z >= bm.wlo[2] && z < bm.whi[2];
        const long long orow = ((bm.ooff[2] + z) * bm.OD[1] + (bm.ooff[1] + y)) * bm.OD[0] + bm.ooff[0];
        float lastv[R][2], wv[R][2];
#pragma unroll
        for (int s = 0; s < R; ++s) {
            const int q = lane + 32 * s;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = 2 * q + h;
                const bool ok = x < bm.b[0];
                lastv[s][h] = ok ? psrc[mr.base + mirror_x(bm, x)] : 0.0f;
                wv[s][h] = ok ? zero_at(ua.weight[0], bm, zr, x) : 0.0f;
            }
        }
#pragma unroll
        for (int s = 0; s < R; ++s) {
            const int q = lane + 32 * s;
            const float2 c = srow[wib][q];
            const float cv[2] = {c.x, c.y};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = 2 * q + h;
                if (x >= bm.b[0]) continue;
                const float last = lastv[s][h];
                const float next = next_value(last, cv[h], wv[s][h], ua.lambda, ua.minI, ua.maxI);
                const float ch = next - last;
                const float ky = ch - kcomp;
                const float kt = ksum + ky;
                kcomp = (kt - ksum) - ky;
                ksum = kt;
                kmax = kmax > ch ? kmax : ch;
                if (wrow && x >= bm.wlo[0] && x < bm.whi[0]) pdst[orow + x] = next;
            }
        }
        __syncwarp();
    }
    double lsum = (double)ksum - (double)kcomp, lmax = (double)kmax;
    for (int o = 16; o > 0; o >>= 1) {
        lsum += __shfl_down_sync(0xffffffffu, lsum, o);
        lmax = fmax(lmax, __shfl_down_sync(0xffffffffu, lmax, o));
    }
    if (lane == 0) {
        red_s[wib] = lsum;
        red_m[wib] = lmax;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0, mx = -1.0;
        for (int w = 0; w < 8; ++w) {
            s += red_s[w];
            mx = fmax(mx, red_m[w]);
        }
        const long long slot = (long long)blockIdx.y * gridDim.x + blockIdx.x;
        ua.partials[2 * slot] = s;
        ua.partials[2 * slot + 1] = mx;
    }
}

}  // namespace mvr
