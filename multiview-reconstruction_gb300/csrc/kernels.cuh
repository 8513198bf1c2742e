// Pass kernels of one block iteration.  The spectrum of a block lives in HBM as
// complex [Pz][Py][Hx], Hx = Px/2 + 1 (half spectrum along x).  One iteration of one
// view on one block is:
//
//   k_rows_fwd      extract psi (mirror-single, from the volume) + R2C along x
//   k_cols   Y fwd
//   k_cols   Z fwd -> x K1^ -> Z inv      (spectral multiply fused between the passes)
//   k_cols   Y inv
//   k_rows_ratio    C2R along x -> conv1 -> quotient img/conv1 -> R2C along x
//   k_cols   Y fwd
//   k_cols   Z fwd -> x K2^ -> Z inv
//   k_cols   Y inv
//   k_rows_update   C2R along x -> conv2 -> multiplicative update, FP64 stats,
//                   effective region written to the output volume
//
// Reference semantics (cited relative to src/main/java/ of the reference):
//   quotient   net/preibisch/mvrecon/process/deconvolution/iteration/sequential/DeconvolutionMethods.java:71-74
//   update     .../DeconvolutionMethods.java:320-358 (Seq), 370-419 (Mul), tikhonov 421
//   extension  .../ComputeBlockSeqThreadCPU.java:171-209 (mirror-single for conv1, 1 for conv2)
//   extract    net/preibisch/mvrecon/process/deconvolution/MultiViewDeconvolutionSeq.java:115
//              (Views.extendMirrorSingle(psi)), img/weight zero-extended (:122-123)
#pragma once
#include "fft_device.cuh"
#include "fsum.cuh"

namespace mvr {

constexpr int kMaxViews = 16;

// Where a block sits: FFT domain, block, volume, and the region written back.
struct BlockMap {
    int P[3];            // FFT domain (x, y, z)
    int b[3];            // block size
    int L[3];            // wrapped left extension: domain index j >= P-L is block coordinate j-P
    long long off[3];    // block offset in volume coordinates (may be negative)
    long long D[3];      // volume dims
    int wlo[3], whi[3];  // block-local region written to the output volume [lo, hi)
    long long ooff[3];   // volume coordinate of block-local (0,0,0) in the output volume
    long long OD[3];     // output volume dims
    int fast_x;          // 1: domain x == block x and the block row lies inside the volume
};

// The blocks of one batched launch: blockIdx.y (rows) / blockIdx.z (columns) picks
// the block; block i's spectrum starts at i * Pc.
constexpr int kMaxBatch = 16;
struct BlockMaps {
    BlockMap m[kMaxBatch];
};

// 1 when every domain x maps to volume x = off + x without extension or mirroring.
inline int block_fast_x(const BlockMap &m)
{
    return (m.L[0] == 0 && m.P[0] == m.b[0] && m.off[0] >= 0 && m.off[0] + m.b[0] <= m.D[0]) ? 1 : 0;
}

__device__ __forceinline__ int ext_e(int j, int P, int L) { return j >= P - L ? j - P : j; }

__device__ __forceinline__ long long mirror1(long long i, long long n)
{
    if (i >= 0 && i < n) return i;  // inside: no reflection
    if (n <= 1) return 0;
    const int p = (int)(2 * n - 2);
    int j = (int)(i % p);
    if (j < 0) j += p;
    return j >= n ? p - j : j;
}

// Volume index of block coordinate (bx, by, bz) under mirror-single on the volume.
struct MirrorRow {
    long long base;  // (gz * D1 + gy) * D0
};
__device__ __forceinline__ MirrorRow mirror_row(const BlockMap &m, int y, int z)
{
    const int ey = ext_e(y, m.P[1], m.L[1]), ez = ext_e(z, m.P[2], m.L[2]);
    const long long by = mirror1(ey, m.b[1]), bz = mirror1(ez, m.b[2]);
    const long long gy = mirror1(m.off[1] + by, m.D[1]), gz = mirror1(m.off[2] + bz, m.D[2]);
    MirrorRow r;
    r.base = (gz * m.D[1] + gy) * m.D[0];
    return r;
}
__device__ __forceinline__ long long mirror_x(const BlockMap &m, int x)
{
    if (m.fast_x) return m.off[0] + x;
    const int ex = ext_e(x, m.P[0], m.L[0]);
    return mirror1(m.off[0] + mirror1(ex, m.b[0]), m.D[0]);
}

// Zero-extended access to img / weight volumes for block voxels.
struct ZeroRow {
    long long base;  // -1 when the row lies outside the volume
};
__device__ __forceinline__ ZeroRow zero_row(const BlockMap &m, int by, int bz)
{
    const long long gy = m.off[1] + by, gz = m.off[2] + bz;
    ZeroRow r;
    r.base = (gy < 0 || gy >= m.D[1] || gz < 0 || gz >= m.D[2]) ? -1 : (gz * m.D[1] + gy) * m.D[0];
    return r;
}
__device__ __forceinline__ float zero_at(const float *__restrict__ v, const BlockMap &m, ZeroRow r, int bx)
{
    const long long gx = m.off[0] + bx;
    if (r.base < 0 || (!m.fast_x && (gx < 0 || gx >= m.D[0]))) return 0.0f;
    return __ldg(v + r.base + gx);
}

// ---- row sources for the forward pass ----------------------------------------------
template <typename TS>
struct SrcMirror {  // psi (or any volume) under the block's mirror mapping
    const TS *vol;
    typedef MirrorRow Row;
    __device__ __forceinline__ Row row(const BlockMap &m, int y, int z) const { return mirror_row(m, y, z); }
    template <typename T>
    __device__ __forceinline__ T at(const Row &r, const BlockMap &m, int x) const { return (T)vol[r.base + mirror_x(m, x)]; }
};

template <typename TS>
struct SrcZero {  // a block buffer [b] with zero outside it (FFTConvolution with extendZero)
    const TS *blk;
    struct Row { long long base; };
    __device__ __forceinline__ Row row(const BlockMap &m, int y, int z) const
    {
        const int ey = ext_e(y, m.P[1], m.L[1]), ez = ext_e(z, m.P[2], m.L[2]);
        Row r;
        r.base = (ey >= 0 && ey < m.b[1] && ez >= 0 && ez < m.b[2]) ? ((long long)ez * m.b[1] + ey) * m.b[0] : -1;
        return r;
    }
    template <typename T>
    __device__ __forceinline__ T at(const Row &r, const BlockMap &m, int x) const
    {
        const int ex = ext_e(x, m.P[0], m.L[0]);
        if (r.base < 0 || ex < 0 || ex >= m.b[0]) return (T)0;
        return (T)blk[r.base + ex];
    }
};

struct SrcKernel {  // kernel placed with its centre (k/2) at the origin, wrapped, scaled
    const float *k;
    int kd[3];
    double scale;
    struct Row { long long base; };
    __device__ __forceinline__ Row row(const BlockMap &m, int y, int z) const
    {
        const int ty = (y + kd[1] / 2) % m.P[1], tz = (z + kd[2] / 2) % m.P[2];
        Row r;
        r.base = (ty < kd[1] && tz < kd[2]) ? ((long long)tz * kd[1] + ty) * kd[0] : -1;
        return r;
    }
    template <typename T>
    __device__ __forceinline__ T at(const Row &r, const BlockMap &m, int x) const
    {
        const int tx = (x + kd[0] / 2) % m.P[0];
        if (r.base < 0 || tx >= kd[0]) return (T)0;
        return (T)((double)k[r.base + tx] * scale);
    }
};

// ---- shared helpers of the row kernels ----------------------------------------------
template <typename V>
__device__ __forceinline__ void load_twiddles(V *tw, const V *__restrict__ twg, int n)
{
    for (int i = threadIdx.x; i < n; i += blockDim.x) tw[i] = twg[i];
}

// Z (m-point FFT of packed rows) -> half spectrum X[0..m], stored to S rows.
template <typename V>
__device__ __forceinline__ void r2c_post_store(const V *Z, int ps, V *__restrict__ S, long long row0, int nr, int m,
                                               const V *tw)
{
    typedef typename Re<V>::t T;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = warp; r < nr; r += nw) {
        const V *z = Z + r * ps;
        V *out = S + (row0 + r) * (long long)(m + 1);
        for (int k = lane; k <= m; k += 32) {
            const V zk = z[k == m ? 0 : k];
            const V zc = cconj(z[k == 0 ? 0 : m - k]);
            const V e = cscale(cadd(zk, zc), (T)0.5);
            const V dd = cscale(csub(zk, zc), (T)0.5);
            const V o = cx<V>(dd.y, -dd.x);  // -i * dd
            out[k] = cadd(e, cmul(tw[k], o));
        }
    }
}

// S rows -> packed Z' for the inverse m-point FFT (yields Px * x after it).  A warp
// takes a row; each lane keeps its loads of one 256-wide chunk in registers.
constexpr int kRowBatch = 8;  // 8 x 32 lanes = 256 values per chunk

template <typename V>
__device__ __forceinline__ void c2r_pre_load(const V *__restrict__ S, V *A, int ps, long long row0, int nr, int m,
                                             const V *tw)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = warp; r < nr; r += nw) {
        const V *in = S + (row0 + r) * (long long)(m + 1);
        V *a = A + r * ps;
        for (int c0 = 0; c0 < m; c0 += 32 * kRowBatch) {
            V xk[kRowBatch], xc[kRowBatch];
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) {
                const int k = c0 + lane + 32 * u;
                if (k < m) {
                    xk[u] = in[k];
                    xc[u] = in[m - k];
                }
            }
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) {
                const int k = c0 + lane + 32 * u;
                if (k < m) {
                    const V e = cadd(xk[u], cconj(xc[u]));
                    const V o = cmul(csub(xk[u], cconj(xc[u])), cconj(tw[k]));
                    a[k] = cx<V>(e.x - o.y, e.y + o.x);  // e + i*o
                }
            }
        }
    }
}

// ---- forward row pass with a fused source -------------------------------------------
template <typename T, class Src, bool BIG>
__global__ void __launch_bounds__(256) k_rows_fwd(Src src, typename Cx<T>::t *__restrict__ S, const BlockMaps bms,
                                                  long long Pc, FftDesc d, const typename Cx<T>::t *__restrict__ twg,
                                                  int RP)
{
    typedef typename Cx<T>::t V;
    const BlockMap &bm = bms.m[blockIdx.y];
    S += (long long)blockIdx.y * Pc;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Px = bm.P[0], m = Px >> 1, ps = m + 1;
    V *tw = reinterpret_cast<V *>(smem_raw);
    V *A = tw + Px;
    V *B = A + RP * ps;
    const long long nrows = (long long)bm.P[1] * bm.P[2];
    const long long row0 = (long long)blockIdx.x * RP;
    const int nr = (int)min((long long)RP, nrows - row0);
    load_twiddles(tw, twg, Px);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = warp; r < nr; r += nw) {
        const long long row = row0 + r;
        const int z = (int)((unsigned)row / (unsigned)bm.P[1]), y = (int)row - z * bm.P[1];  // rows < 2^31
        const typename Src::Row R = src.row(bm, y, z);
        for (int c0 = 0; c0 < m; c0 += 32 * kRowBatch) {
            T v0[kRowBatch], v1[kRowBatch];
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) {
                const int q = c0 + lane + 32 * u;
                if (q < m) {
                    v0[u] = src.template at<T>(R, bm, 2 * q);
                    v1[u] = src.template at<T>(R, bm, 2 * q + 1);
                }
            }
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) {
                const int q = c0 + lane + 32 * u;
                if (q < m) A[r * ps + q] = cx<V>(v0[u], v1[u]);
            }
        }
    }
    __syncthreads();
    V *Z = fft_run<false, false, BIG>(A, B, nr, ps, 1, d, tw, 2);
    r2c_post_store(Z, ps, S, row0, nr, m, tw);
}

// ---- column passes (y or z axis) ----------------------------------------------------
// MODE 0: forward, 1: inverse, 2: forward, multiply by Kh, inverse.  NP (a power of
// two) consecutive x' columns at one other-axis index form the tile; every thread
// keeps kLoadBatch independent global accesses in flight.
constexpr int kLoadBatch = 8;

template <typename T, int MODE, bool BIG>
__global__ void __launch_bounds__(256) k_cols(const typename Cx<T>::t *src, typename Cx<T>::t *dst,
                                              const typename Cx<T>::t *__restrict__ Kh, int Hx, long long estride,
                                              long long ostride, int NP, long long Pc, FftDesc d,
                                              const typename Cx<T>::t *__restrict__ twg)
{
    typedef typename Cx<T>::t V;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = d.n;
    V *tw = reinterpret_cast<V *>(smem_raw);
    V *A = tw + n;
    V *B = A + n * NP;
    load_twiddles(tw, twg, n);
    const int x0 = blockIdx.x * NP;
    const long long base = (long long)blockIdx.y * ostride + x0;
    src += (long long)blockIdx.z * Pc;
    dst += (long long)blockIdx.z * Pc;
    const int np = min(NP, Hx - x0);
    const int tot = n * NP;
    const int lg = __ffs(NP) - 1;
    const int step = blockDim.x * kLoadBatch;
    for (int t0 = threadIdx.x; t0 < tot; t0 += step) {
        V r[kLoadBatch];
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int t = t0 + u * blockDim.x;
            const int p = t & (NP - 1), i = t >> lg;
            r[u] = (t < tot && p < np) ? src[base + i * estride + p] : cx<V>((T)0, (T)0);
        }
#pragma unroll
        for (int u = 0; u < kLoadBatch; ++u) {
            const int t = t0 + u * blockDim.x;
            if (t < tot) A[t] = r[u];
        }
    }
    __syncthreads();
    V *R = fft_run<MODE == 1, true, BIG>(A, B, NP, 1, NP, d, tw, 1);
    if (MODE == 2) {
        for (int t0 = threadIdx.x; t0 < tot; t0 += step) {
            V k[kLoadBatch];
#pragma unroll
            for (int u = 0; u < kLoadBatch; ++u) {
                const int t = t0 + u * blockDim.x;
                const int p = t & (NP - 1), i = t >> lg;
                k[u] = (t < tot && p < np) ? __ldg(&Kh[base + i * estride + p]) : cx<V>((T)0, (T)0);
            }
#pragma unroll
            for (int u = 0; u < kLoadBatch; ++u) {
                const int t = t0 + u * blockDim.x;
                if (t < tot) R[t] = cmul(R[t], k[u]);
            }
        }
        __syncthreads();
        R = fft_run<true, true, BIG>(R, R == A ? B : A, NP, 1, NP, d, tw, 1);
    }
    for (int t = threadIdx.x; t < tot; t += blockDim.x) {
        const int p = t & (NP - 1), i = t >> lg;
        if (p < np) dst[base + i * estride + p] = R[t];
    }
}

// ---- pointwise rules ------------------------------------------------------------------
// DeconvolutionMethods.java:71-74: img > 0 ? img / blurred : 1 (float division).
__device__ __forceinline__ float quotient(float img, float blurred) { return img > 0.0f ? __fdiv_rn(img, blurred) : 1.0f; }
__device__ __forceinline__ double quotient(float img, double blurred) { return img > 0.0f ? (double)img / blurred : 1.0; }

// tikhonov (DeconvolutionMethods.java:421), double, no contraction
__device__ __forceinline__ double tikhonov(double v, double lambda)
{
    return __ddiv_rn(__dsub_rn(__dsqrt_rn(__dadd_rn(1.0, __dmul_rn(__dmul_rn(2.0, lambda), v))), 1.0), lambda);
}

// The Tikhonov factor in float, from the algebraically equal form without the
// cancellation of sqrt(1+x)-1: (sqrt(1 + 2 l v) - 1) / l == 2 v / (sqrt(1 + 2 l v) + 1).
// Within a few float ulp of the reference's double evaluation rounded to float (the
// reference rounds it to float too); the GPU's double rate is a small fraction of its
// float rate, so the double form would dominate the whole iteration.
__device__ __forceinline__ float tikhonov_f(float v, float two_lambda)
{
    const float r = __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(two_lambda, v)));
    return __fdiv_rn(__fmul_rn(2.0f, v), __fadd_rn(r, 1.0f));
}

// computeNextValue (DeconvolutionMethods.java:320-358) in float: every operation the
// reference does in float is done in float here with IEEE rounding and no contraction.
// two_lambda = (float)(2 lambda) and tik = lambda > 0 come from the host (no FP64 here).
__device__ __forceinline__ float next_value(float last, float integral, float weight, float two_lambda, int tik,
                                            float minI, float maxI)
{
    const float value = __fmul_rn(last, integral);
    float adjusted;
    if (value > 0.0f)
        adjusted = tik ? __fmul_rn(tikhonov_f(__fdiv_rn(value, maxI), two_lambda), maxI) : value;
    else adjusted = minI;
    const float next = isnan(adjusted) ? minI : (minI >= adjusted ? minI : adjusted);
    return __fadd_rn(last, __fmul_rn(__fsub_rn(next, last), weight));
}
// The plane kernels' form of the same rule: the division by maxI becomes a product with
// its reciprocal, the Tikhonov factor takes the hardware reciprocal square root and the
// approximate division (each within 2 ulp), the rest is as above.  The difference to
// the IEEE form is a few float ulp per voxel, far inside the FFT rounding.
struct UpdConst {
    float minI, maxI, inv_maxI, two_lambda;
    bool tik;
};
__device__ __forceinline__ float next_value_fast(float last, float integral, float weight, const UpdConst &c)
{
    const float value = __fmul_rn(last, integral);
    float adjusted;
    if (value > 0.0f) {
        if (c.tik) {
            const float v = value * c.inv_maxI;
            const float s = fmaf(c.two_lambda, v, 1.0f);
            const float r = s * rsqrtf(s);
            adjusted = __fdividef(2.0f * v, r + 1.0f) * c.maxI;
        } else {
            adjusted = value;
        }
    } else {
        adjusted = c.minI;
    }
    const float next = isnan(adjusted) ? c.minI : (c.minI >= adjusted ? c.minI : adjusted);
    return __fadd_rn(last, __fmul_rn(__fsub_rn(next, last), weight));
}
// Quotient with the approximate division (within 2 ulp of img / blurred).
__device__ __forceinline__ float quotient_fast(float img, float blurred)
{
    return img > 0.0f ? __fdividef(img, blurred) : 1.0f;
}
// The same rule in double (FP64 run).
__device__ __forceinline__ double next_value(double last, double integral, double weight, double lambda, double minI,
                                             double maxI)
{
    const double value = __dmul_rn(last, integral);
    double adjusted;
    if (value > 0.0) adjusted = lambda > 0 ? __dmul_rn(tikhonov(__ddiv_rn(value, maxI), lambda), maxI) : value;
    else adjusted = minI;
    const double next = isnan(adjusted) ? minI : (minI >= adjusted ? minI : adjusted);
    return __dadd_rn(last, __dmul_rn(__dsub_rn(next, last), weight));
}

// ---- C2R -> quotient -> R2C (conv1 of one view, then the input of conv2) -------------
template <typename T, bool BIG>
__global__ void __launch_bounds__(256) k_rows_ratio(typename Cx<T>::t *__restrict__ S, const float *__restrict__ img,
                                                    const BlockMaps bms, long long Pc, FftDesc d,
                                                    const typename Cx<T>::t *__restrict__ twg, int RP)
{
    typedef typename Cx<T>::t V;
    const BlockMap &bm = bms.m[blockIdx.y];
    S += (long long)blockIdx.y * Pc;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int Px = bm.P[0], m = Px >> 1, ps = m + 1;
    V *tw = reinterpret_cast<V *>(smem_raw);
    V *A = tw + Px;
    V *B = A + RP * ps;
    const long long nrows = (long long)bm.P[1] * bm.P[2];
    const long long row0 = (long long)blockIdx.x * RP;
    const int nr = (int)min((long long)RP, nrows - row0);
    load_twiddles(tw, twg, Px);
    __syncthreads();
    c2r_pre_load(S, A, ps, row0, nr, m, tw);
    __syncthreads();
    V *Z = fft_run<true, false, BIG>(A, B, nr, ps, 1, d, tw, 2);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = warp; r < nr; r += nw) {
        const long long row = row0 + r;
        const int z = (int)((unsigned)row / (unsigned)bm.P[1]), y = (int)row - z * bm.P[1];  // rows < 2^31
        const int ey = ext_e(y, bm.P[1], bm.L[1]), ez = ext_e(z, bm.P[2], bm.L[2]);
        const bool rin = ey >= 0 && ey < bm.b[1] && ez >= 0 && ez < bm.b[2];
        const ZeroRow zr = rin ? zero_row(bm, ey, ez) : ZeroRow{-1};
        V *zz = Z + r * ps;
        for (int c0 = 0; c0 < m; c0 += 32 * kRowBatch) {
            float im[kRowBatch][2];
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) {
                const int q = c0 + lane + 32 * u;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int ex = ext_e(2 * q + h, Px, bm.L[0]);
                    im[u][h] = (q < m && rin && ex >= 0 && ex < bm.b[0]) ? zero_at(img, bm, zr, ex) : -1.0f;
                }
            }
#pragma unroll
            for (int u = 0; u < kRowBatch; ++u) {
                const int q = c0 + lane + 32 * u;
                if (q >= m) continue;
                const V c = zz[q];  // conv1 at x = 2q, 2q+1 (kernel spectrum carries 1/(Px Py Pz))
                T out[2] = {c.x, c.y};
#pragma unroll
                for (int h = 0; h < 2; ++h)  // -1 marks the value-1 extension outside the block
                    out[h] = im[u][h] < 0.0f ? (T)1 : (T)quotient(im[u][h], out[h]);
                zz[q] = cx<V>(out[0], out[1]);
            }
        }
    }
    __syncthreads();
    V *Z2 = fft_run<false, false, BIG>(Z, Z == A ? B : A, nr, ps, 1, d, tw, 2);
    r2c_post_store(Z2, ps, S, row0, nr, m, tw);
}

// ---- the running product of the Mul update ---------------------------------------------
// computeNextValueMul (DeconvolutionMethods.java:370-387) multiplies the views' conv2
// values in double and takes pow(prod, 1 / V).  A float product of 4-16 factors can leave
// the float range where the double one does not (a tiny blurred value makes one factor
// huge), so the float path keeps the product as a float mantissa in [0.5, 1) and a
// power-of-two exponent (stored as a float pair, 8 bytes per voxel; every factor is split
// with frexpf first, so no partial product under- or overflows).  Zero, signed, Inf and NaN
// factors propagate as in the double product.
__device__ __forceinline__ float2 mulprod_first(float c)
{
    int e;
    const float m = frexpf(c, &e);
    return make_float2(m, (float)e);
}
__device__ __forceinline__ float2 mulprod_acc(float2 p, float c)
{
    int ec, e2;
    const float mc = frexpf(c, &ec);
    const float m = frexpf(__fmul_rn(p.x, mc), &e2);
    return make_float2(m, p.y + (float)(ec + e2));
}
// pow(prod, 1 / V) rounded to float: 2^(e / V) split into an integer power q and a
// remainder r < V, so the float power function only sees m 2^r in [0.5, 2^(V-1)).
// Math.pow of a negative base with the non-integer exponent 1 / V (V >= 2) is NaN.
__device__ __forceinline__ float mulprod_root(float2 p, int V)
{
    const float m = p.x;
    const int e = (int)p.y;
    if (V == 1) return ldexpf(m, e);
    if (m == 0.0f) return 0.0f;
    if (!(m > 0.0f)) return __int_as_float(0x7fc00000);  // negative or NaN
    if (isinf(m)) return m;
    const int q = e >= 0 ? e / V : -((V - 1 - e) / V);
    const int r = e - q * V;
    const float x = ldexpf(m, r);
    const float y = V == 2 ? __fsqrt_rn(x) : powf(x, 1.0f / (float)V);
    return ldexpf(y, q);
}

// ---- C2R -> update -------------------------------------------------------------------
enum { EPI_SEQ = 0, EPI_MUL_FIRST = 1, EPI_MUL_ACC = 2, EPI_MUL_FINAL = 3, EPI_STORE = 4, EPI_NLL = 5 };

struct UpdateArgs {
    const void *psi_src;  // T volume, read under the mirror mapping
    void *psi_dst;        // T output volume (write region only)
    const float *weight[kMaxViews];
    int nviews;
    void *prod;           // Mul: running product over views, block layout [bz][by][bx], 8 bytes a
                          // voxel (double for the FP64 path, mulprod_* float pairs for FP32)
    float *store;         // EPI_STORE: conv result, block layout
    const float *img;     // EPI_NLL: the view's image (zero outside the volume)
    double lambda;
    float two_lambda;     // (float)(2 lambda), for the float update
    int tik;              // lambda > 0
    float minI;
    float maxI;
    double *partials;     // per CTA {sum, max}
    int prune;            // plane kernels: only the planes and rows of the write region, no
                          // statistics (voxels outside the write region are discarded)
};

// The update epilogue of one block row (C2R result zz: natural-order packed values,
// zz[q] = (x = 2q, x = 2q + 1)), shared by the row kernels and the plane kernels.
// ua.prod / ua.store are already offset to the block.  One warp per row, lanes over x.
template <typename T, int EPI>
__device__ __forceinline__ void update_row(const typename Cx<T>::t *zz, int m, const BlockMap &bm,
                                           const UpdateArgs &ua, int y, int z, int lane, T &ksum, T &kcomp, T &kmax)
{
    typedef typename Cx<T>::t V;
    const T *psrc = reinterpret_cast<const T *>(ua.psi_src);
    T *pdst = reinterpret_cast<T *>(ua.psi_dst);
    const ZeroRow zr = zero_row(bm, y, z);
    const MirrorRow mr = mirror_row(bm, y, z);
    const bool wrow = y >= bm.wlo[1] && y < bm.whi[1] && z >= bm.wlo[2] && z < bm.whi[2];
    const long long orow = ((bm.ooff[2] + z) * bm.OD[1] + (bm.ooff[1] + y)) * bm.OD[0] + bm.ooff[0];
    const long long brow = ((long long)z * bm.b[1] + y) * bm.b[0];
    constexpr int UB = kRowBatch / 2;
    for (int c0 = 0; c0 < m; c0 += 32 * UB) {
        T lastv[UB][2];
        float wv[UB][2];
        if (EPI == EPI_SEQ || EPI == EPI_MUL_FINAL) {  // psi and the first weight, batched
#pragma unroll
            for (int u = 0; u < UB; ++u) {
                const int q = c0 + lane + 32 * u;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int x = 2 * q + h;
                    const bool ok = q < m && x < bm.b[0];
                    lastv[u][h] = ok ? psrc[mr.base + mirror_x(bm, x)] : (T)0;
                    wv[u][h] = (ok && EPI == EPI_SEQ) ? zero_at(ua.weight[0], bm, zr, x) : 0.0f;
                }
            }
        }
#pragma unroll
        for (int u = 0; u < UB; ++u) {
            const int q = c0 + lane + 32 * u;
            if (q >= m) continue;
            const V c = zz[q];
            const T cv[2] = {c.x, c.y};
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int x = 2 * q + h;
                if (x >= bm.b[0]) continue;
                const T integral = cv[h];
                if (EPI == EPI_STORE) {
                    ua.store[brow + x] = (float)integral;
                    continue;
                }
                if (EPI == EPI_MUL_FIRST) {
                    if constexpr (sizeof(T) == sizeof(float))
                        reinterpret_cast<float2 *>(ua.prod)[brow + x] = mulprod_first((float)integral);
                    else reinterpret_cast<T *>(ua.prod)[brow + x] = integral;
                    continue;
                }
                if (EPI == EPI_NLL) {
                    // Poisson negative log-likelihood w * (conv1 - img ln conv1) over img > 0,
                    // each volume voxel once (write region of its block)
                    if (!(wrow && x >= bm.wlo[0] && x < bm.whi[0])) continue;
                    const float im = zero_at(ua.img, bm, zr, x);
                    const float wt = zero_at(ua.weight[0], bm, zr, x);
                    if (!(im > 0.0f) || !(integral > (T)0)) continue;
                    const T lg = sizeof(T) == sizeof(float) ? (T)logf((float)integral) : (T)log((double)integral);
                    const T term = (T)wt * (integral - (T)im * lg);
                    const T ky = term - kcomp;
                    const T kt = ksum + ky;
                    kcomp = (kt - ksum) - ky;
                    ksum = kt;
                    continue;
                }
                if (EPI == EPI_MUL_ACC) {
                    if constexpr (sizeof(T) == sizeof(float)) {
                        float2 *pp = reinterpret_cast<float2 *>(ua.prod) + brow + x;
                        *pp = mulprod_acc(*pp, (float)integral);
                    } else {
                        reinterpret_cast<T *>(ua.prod)[brow + x] *= integral;
                    }
                    continue;
                }
                const T last = lastv[u][h];
                T next;
                if (EPI == EPI_SEQ) {
                    if constexpr (sizeof(T) == sizeof(float))
                        next = next_value((float)last, (float)integral, (float)wv[u][h], ua.two_lambda, ua.tik, ua.minI,
                                          ua.maxI);
                    else
                        next = next_value(last, integral, (T)wv[u][h], ua.lambda, (T)ua.minI, (T)ua.maxI);
                } else {  // EPI_MUL_FINAL: DeconvolutionMethods.computeNextValueMul 370-419
                    // the weight sum in T (the reference uses double; the float sum of V
                    // weights in [0, 1] stays within an ulp), the product as above
                    T sumW = 0;
                    for (int v = 0; v < ua.nviews; ++v) sumW += (T)zero_at(ua.weight[v], bm, zr, x);
                    T root;
                    if constexpr (sizeof(T) == sizeof(double)) {
                        const T prod = (ua.nviews == 1 ? (T)1 : reinterpret_cast<const T *>(ua.prod)[brow + x]) * integral;
                        root = (T)pow((double)prod, 1.0 / ua.nviews);
                    } else {
                        const float2 p = ua.nviews == 1 ? mulprod_first((float)integral)
                                                        : mulprod_acc(reinterpret_cast<const float2 *>(ua.prod)[brow + x],
                                                                      (float)integral);
                        root = (T)mulprod_root(p, ua.nviews);
                    }
                    sumW = sumW < (T)1 ? sumW : (T)1;
                    if constexpr (sizeof(T) == sizeof(float))
                        next = next_value((float)last, (float)root, (float)sumW, ua.two_lambda, ua.tik, ua.minI, ua.maxI);
                    else
                        next = next_value(last, root, sumW, ua.lambda, (T)ua.minI, (T)ua.maxI);
                }
                const T ch = next - last;  // signed change (DeconvolutionMethods.java:308)
                const T ky = ch - kcomp;
                const T kt = ksum + ky;
                kcomp = (kt - ksum) - ky;
                ksum = kt;
                kmax = kmax > ch ? kmax : ch;
                if (wrow && x >= bm.wlo[0] && x < bm.whi[0]) pdst[orow + x] = next;
            }
        }
    }
}

// Deterministic CTA reduction of the per-thread statistics into ua.partials[slot]
// (sum from the compensated per-thread sums as float pairs, converted to double once per
// CTA; max).  Every thread must call it.
template <typename T>
__device__ __forceinline__ void stats_to_partials(T ksum, T kcomp, T kmax, double *red_s, double *red_m,
                                                  double *partials, long long slot)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    if constexpr (sizeof(T) == sizeof(float)) {
        float hi = ksum, lo = -kcomp, mx = kmax;
        for (int o = 16; o > 0; o >>= 1) {
            const float bh = __shfl_down_sync(0xffffffffu, hi, o), bl = __shfl_down_sync(0xffffffffu, lo, o);
            pair_add(hi, lo, bh, bl);
            mx = fmaxf(mx, __shfl_down_sync(0xffffffffu, mx, o));
        }
        float *rs = reinterpret_cast<float *>(red_s);  // [hi, lo] per warp
        float *rm = reinterpret_cast<float *>(red_m);
        if (lane == 0) {
            rs[2 * warp] = hi;
            rs[2 * warp + 1] = lo;
            rm[warp] = mx;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float sh = 0.0f, sl = 0.0f, m = -1.0f;
            for (int w = 0; w < nw; ++w) {
                pair_add(sh, sl, rs[2 * w], rs[2 * w + 1]);
                m = fmaxf(m, rm[w]);
            }
            partials[2 * slot] = (double)sh + (double)sl;
            partials[2 * slot + 1] = (double)m;
        }
    } else {
        double lsum = (double)ksum - (double)kcomp, lmax = (double)kmax;
        for (int o = 16; o > 0; o >>= 1) {
            lsum += __shfl_down_sync(0xffffffffu, lsum, o);
            lmax = fmax(lmax, __shfl_down_sync(0xffffffffu, lmax, o));
        }
        if (lane == 0) { red_s[warp] = lsum; red_m[warp] = lmax; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0, mx = -1.0;
            for (int w = 0; w < nw; ++w) { s += red_s[w]; mx = fmax(mx, red_m[w]); }
            partials[2 * slot] = s;
            partials[2 * slot + 1] = mx;
        }
    }
}

template <typename T, int EPI, bool BIG>
__global__ void __launch_bounds__(256) k_rows_update(typename Cx<T>::t *__restrict__ S, UpdateArgs ua,
                                                     const BlockMaps bms, long long Pc, FftDesc d,
                                                     const typename Cx<T>::t *__restrict__ twg, int RP)
{
    typedef typename Cx<T>::t V;
    const BlockMap &bm = bms.m[blockIdx.y];
    S += (long long)blockIdx.y * Pc;
    const long long bvox = (long long)bm.b[0] * bm.b[1] * bm.b[2];
    if (ua.prod) ua.prod = reinterpret_cast<double *>(ua.prod) + (long long)blockIdx.y * bvox;  // 8 bytes a voxel
    if (ua.store) ua.store += (long long)blockIdx.y * bvox;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red_s[32], red_m[32];
    const int Px = bm.P[0], m = Px >> 1, ps = m + 1;
    V *tw = reinterpret_cast<V *>(smem_raw);
    V *A = tw + Px;
    V *B = A + RP * ps;
    const long long nrows = (long long)bm.P[1] * bm.P[2];
    const long long row0 = (long long)blockIdx.x * RP;
    const int nr = (int)min((long long)RP, nrows - row0);
    load_twiddles(tw, twg, Px);
    __syncthreads();
    c2r_pre_load(S, A, ps, row0, nr, m, tw);
    __syncthreads();
    V *Z = fft_run<true, false, BIG>(A, B, nr, ps, 1, d, tw, 2);
    // signed-change statistics: per thread in T with Kahan compensation (T = float:
    // the double rate is a small fraction of the float rate), per block in double
    T ksum = 0, kcomp = 0, kmax = (T)-1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    for (int r = warp; r < nr; r += nw) {
        const long long row = row0 + r;
        const int z = (int)((unsigned)row / (unsigned)bm.P[1]), y = (int)row - z * bm.P[1];  // rows < 2^31
        if (y >= bm.b[1] || z >= bm.b[2]) continue;  // extension rows carry no block voxels
        update_row<T, EPI>(Z + r * ps, m, bm, ua, y, z, lane, ksum, kcomp, kmax);
    }
    if (EPI == EPI_SEQ || EPI == EPI_MUL_FINAL || EPI == EPI_NLL)
        stats_to_partials(ksum, kcomp, kmax, red_s, red_m, ua.partials, (long long)blockIdx.y * gridDim.x + blockIdx.x);
}

// Sum / max of per-CTA partials in a fixed order (one CTA), into out[0..1].
template <typename D>
__global__ void k_reduce_stats(const D *__restrict__ partials, int n, D *out)
{
    partials += 2LL * n * blockIdx.x;  // block of the batch
    out += 2 * blockIdx.x;
    __shared__ double s_s[1024], s_m[1024];
    double s = 0.0, mx = -1.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) { s += partials[2 * i]; mx = fmax(mx, partials[2 * i + 1]); }
    s_s[threadIdx.x] = s;
    s_m[threadIdx.x] = mx;
    __syncthreads();
    for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
        if (threadIdx.x < h) {
            s_s[threadIdx.x] += s_s[threadIdx.x + h];
            s_m[threadIdx.x] = fmax(s_m[threadIdx.x], s_m[threadIdx.x + h]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) { out[0] = s_s[0]; out[1] = s_m[0]; }
}

// Copy the effective region of a block from one volume to another (paste,
// Block.java:357-403).
template <typename T>
__global__ void k_paste(const T *__restrict__ src, T *__restrict__ dst, long long D0, long long D1, long long ox,
                        long long oy, long long oz, int sx, int sy, int sz)
{
    const long long n = (long long)sx * sy * sz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % sx);
        const long long t = i / sx;
        const int y = (int)(t % sy), z = (int)(t / sy);
        const long long g = ((oz + z) * D1 + (oy + y)) * D0 + (ox + x);
        dst[g] = src[g];
    }
}

}  // namespace mvr
