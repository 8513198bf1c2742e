// Plane kernels: the x and y transforms of one z-plane of a block, fused with the
// extract / quotient / update work of the iteration, with the whole plane spectrum
// held in shared memory.
//
// For FFT domains Px = 32 VX (real x rows of m = 16 VX packed complex values) and
// Py = 16 VY, a CTA works on one z-plane of one block at a time (k_xy_fwd and k_xy_ratio are
// persistent: one CTA per SM walks the (block, plane) items; k_xy_update takes one plane):
//   k_xy_fwd     rows from the source (psi under the mirror mapping, a zero-extended
//                block, or a wrapped kernel) -> R2C along x -> FFT along y -> plane of S
//   k_xy_ratio   plane of S -> inverse y -> C2R along x -> quotient img / conv1
//                (DeconvolutionMethods.java:71-74) -> R2C along x -> FFT along y -> S
//   k_xy_update  plane of S -> inverse y -> C2R along x -> the row epilogue of the
//                update (update_row: Seq / Mul update, FP64-reduced statistics,
//                likelihood, or a plain store)
// so one view-step is fwd, Z (x K1^), ratio, Z (x K2^), update: five passes over the
// spectra instead of nine.
//
// Both axes use the two-phase register FFT of the tile column kernels (n = 16 V):
// phase 1, item (pencil, t): V-point DFT of elements t + 16 v, twiddle W_n^(t k1),
// written back to t + 16 k1; phase 2, item (pencil, k1): 16-point DFT of elements
// t + 16 k1, written back in place, so position k2 + 16 k1 holds frequency k1 + V k2
// ("tile order").  The x spectrum of a real row (m + 1 values) therefore sits in tile
// order too: frequency f < m at position pos(f) = f / VX + 16 (f % VX), the Nyquist
// value at position m.  Every spectrum the products use (data, K1^, K2^) comes from the
// same forward kernels, so the spectral product is taken position by position; the
// inverse phases undo the forward ones exactly and return natural order (times n).
//
// Shared memory: the plane as [y][c] with row stride m + 1 (odd: pencil-fastest
// items touch distinct banks both along rows and along columns), which is also the
// layout of the plane in S ([z][y][c], c < m + 1), so the plane moves between HBM and
// shared memory as one contiguous 16-byte-vectorised copy.
#pragma once
#include "rows_warp.cuh"
#include "cols_tile.cuh"
#include "pdl.cuh"

namespace mvr {

constexpr long long kNoRow = -(1LL << 62);

// CTA size of the 192 x 192 plane kernels (a build-time tuning knob; 1024 measured best)
#ifndef MVR_XY_THREADS_192
#define MVR_XY_THREADS_192 1024
#endif

template <int VX, int VY>
struct XYShape {
    static constexpr int m = 16 * VX;     // packed complex values per real x row
    static constexpr int Px = 2 * m;      // real x length
    static constexpr int Py = 16 * VY;
    static constexpr int SR = m + 1;      // row stride (x spectrum incl. Nyquist)
    static constexpr int plane = Py * SR; // complex values per plane
    // threads per CTA and CTAs per SM: 1024 x 1 for the 155 KB plane of 192 x 192,
    // 512 x 2 for the planes of at most 100 KB (the latency of the shared-memory FFT
    // phases is hidden by warps, not by per-thread interleaving)
    static constexpr int NT = (VX == 6 && VY == 12) ? MVR_XY_THREADS_192 : 512;
    static constexpr int MINB = (VX == 6 && VY == 12) ? 1 : 2;
    // rounds of the row items (y, t) of the fused x phase 1
    static constexpr int RX = Py * 16 / NT;
    static_assert((Py * 16) % NT == 0, "row items must fill whole rounds");
};

// Bytes of dynamic shared memory of the plane kernels of shape (VX, VY).
template <int VX, int VY>
constexpr size_t xy_smem_bytes()
{
    typedef XYShape<VX, VY> S;
    return sizeof(float2) * (size_t)(S::plane + S::Px + S::Py) + 3 * sizeof(long long) * S::Py +
           sizeof(int) * (size_t)(3 * S::Px + S::m + S::Py);
}

// ---- two-phase FFT on pencils in shared memory -------------------------------------
// Element i of pencil p at A[p * PS + i * ES]; tw[j * TWM] = exp(-2 pi i j / (16 V)).
// Items run pencil-fastest so that a warp touches consecutive pencils.
template <int V, int NPEN, int PS, int ES, bool INV, int NT>
__device__ __forceinline__ void tp_phase1(float2 *A, const float2 *tw, int twm)
{
    constexpr int T = 16, items = NPEN * T;
    for (int it = threadIdx.x; it < items; it += NT) {
        const int t = it / NPEN, p = it - t * NPEN;
        float2 *a0 = A + p * PS + t * ES;
        float2 a[V];
#pragma unroll
        for (int v = 0; v < V; ++v) a[v] = a0[T * v * ES];
        if (!INV) {
            sdft<V, false>(a);
#pragma unroll
            for (int k1 = 1; k1 < V; ++k1) a[k1] = cmul(a[k1], tw[t * k1 * twm]);
        } else {
#pragma unroll
            for (int k1 = 1; k1 < V; ++k1) a[k1] = cmul(a[k1], cconj(tw[t * k1 * twm]));
            sdft<V, true>(a);
        }
#pragma unroll
        for (int v = 0; v < V; ++v) a0[T * v * ES] = a[v];
    }
}

template <int V, int NPEN, int PS, int ES, bool INV, int NT>
__device__ __forceinline__ void tp_phase2(float2 *A)
{
    constexpr int T = 16, items = NPEN * V;
    for (int it = threadIdx.x; it < items; it += NT) {
        const int k1 = it / NPEN, p = it - k1 * NPEN;
        float2 *b0 = A + p * PS + T * k1 * ES;
        float2 b[T];
#pragma unroll
        for (int t = 0; t < T; ++t) b[t] = b0[t * ES];
        sdft<T, INV>(b);
#pragma unroll
        for (int t = 0; t < T; ++t) b0[t * ES] = b[t];
    }
}

// x phase 1 of one row item (y, t) on registers: a[v] <-> positions t + 16 v of row y.
// Forward: natural-order values in, twiddled phase-1 output out; inverse the reverse.
template <int VX, bool INV>
__device__ __forceinline__ void xrow_p1(float2 (&a)[VX], const float2 *twx, int t)
{
    if (!INV) {
        sdft<VX, false>(a);
#pragma unroll
        for (int k1 = 1; k1 < VX; ++k1) a[k1] = cmul(a[k1], twx[2 * t * k1]);
    } else {
#pragma unroll
        for (int k1 = 1; k1 < VX; ++k1) a[k1] = cmul(a[k1], cconj(twx[2 * t * k1]));
        sdft<VX, true>(a);
    }
}

// x phase 2 with the packed-real split (forward) or merge (inverse) fused in registers.
// Item (row y, k1) holds the frequencies f = k1 + V k2 (k2 < 16) at positions k2 + 16 k1; the
// split pairs f with m - f, which item (y, V - k1) holds at slot 15 - k2 (k1 = 0: the same
// item at slot 16 - k2; k1 = V / 2: the same item at slot 15 - k2).  A warp takes 16 rows:
// lanes 0-15 item k1, lanes 16-31 the partner item V - k1 of the same rows, so the partner
// values come over one shuffle; the last pair group is (0, V / 2), both self-paired.
//   forward: X[f] = E + W_Px^f (-i D), E = (Z[f] + conj Z[m-f]) / 2, D = (Z[f] - conj Z[m-f]) / 2,
//            the DC and Nyquist values (both real) packed as (X[0], X[m]) at position 0;
//   inverse: a[f] = e + i o, e = X[f] + conj X[m-f], o = (X[f] - conj X[m-f]) conj(W_Px^f),
//            then the inverse 16-point DFT.
template <int VX, int VY, bool INV>
__device__ __forceinline__ float2 xy_split_one(float2 zf, float2 zg, int f, const float2 *twx)
{
    const float2 zc = cconj(zg);
    if (f == 0) return make_float2(zf.x + zf.y, zf.x - zf.y);
    if (!INV) {
        const float2 e = cscale(cadd(zf, zc), 0.5f), dd = cscale(csub(zf, zc), 0.5f);
        return cadd(e, cmul(twx[f], make_float2(dd.y, -dd.x)));
    }
    const float2 e = cadd(zf, zc), q = cmul(csub(zf, zc), cconj(twx[f]));
    return make_float2(e.x - q.y, e.y + q.x);
}

// One item (y, k1) of x phase 2 with the split / merge: b holds its 16 values, read from b0;
// the results go back to b0.  All 32 lanes of the warp take part (the partner item's values
// come over shuffles).
template <int VX, int VY, bool INV>
__device__ __forceinline__ void xy_x_p2_item(float2 (&b)[16], float2 *b0, int k1, int h, bool selfgrp,
                                             const float2 *twx)
{
    constexpr int T = 16;
    if (!INV) sdft<T, false>(b);  // b[k2] = Z[k1 + V k2]
    if (!selfgrp) {
        // partner item V - k1 in lane ^ 16: frequency m - f sits at its slot 15 - k2
#pragma unroll
        for (int k2 = 0; k2 < T / 2; ++k2) {
            const int k3 = T - 1 - k2;
            float2 ga, gb;
            ga.x = __shfl_xor_sync(0xffffffffu, b[k3].x, 16);
            ga.y = __shfl_xor_sync(0xffffffffu, b[k3].y, 16);
            gb.x = __shfl_xor_sync(0xffffffffu, b[k2].x, 16);
            gb.y = __shfl_xor_sync(0xffffffffu, b[k2].y, 16);
            const float2 oa = xy_split_one<VX, VY, INV>(b[k2], ga, k1 + VX * k2, twx);
            const float2 ob = xy_split_one<VX, VY, INV>(b[k3], gb, k1 + VX * k3, twx);
            if (INV) {
                b[k2] = oa;
                b[k3] = ob;
            } else {  // forward: straight back to shared memory
                b0[k2] = oa;
                b0[k3] = ob;
            }
        }
    } else if (h == 0) {  // k1 = 0: f = V k2 pairs with slot 16 - k2; slot 8 is m / 2
        const float2 o0 = xy_split_one<VX, VY, INV>(b[0], b[0], 0, twx);
        const float2 o8 = xy_split_one<VX, VY, INV>(b[8], b[8], VX * 8, twx);
        if (INV) {
            b[0] = o0;
            b[8] = o8;
        } else {
            b0[0] = o0;
            b0[8] = o8;
        }
#pragma unroll
        for (int k2 = 1; k2 < T / 2; ++k2) {
            const int k3 = T - k2;
            const float2 oa = xy_split_one<VX, VY, INV>(b[k2], b[k3], VX * k2, twx);
            const float2 ob = xy_split_one<VX, VY, INV>(b[k3], b[k2], VX * k3, twx);
            if (INV) {
                b[k2] = oa;
                b[k3] = ob;
            } else {  // forward: straight back to shared memory
                b0[k2] = oa;
                b0[k3] = ob;
            }
        }
    } else {  // k1 = V / 2: slot k2 pairs with slot 15 - k2
#pragma unroll
        for (int k2 = 0; k2 < T / 2; ++k2) {
            const int k3 = T - 1 - k2;
            const float2 oa = xy_split_one<VX, VY, INV>(b[k2], b[k3], VX / 2 + VX * k2, twx);
            const float2 ob = xy_split_one<VX, VY, INV>(b[k3], b[k2], VX / 2 + VX * k3, twx);
            if (INV) {
                b[k2] = oa;
                b[k3] = ob;
            } else {  // forward: straight back to shared memory
                b0[k2] = oa;
                b0[k3] = ob;
            }
        }
    }
    if (INV) {
        sdft<T, true>(b);
#pragma unroll
        for (int t = 0; t < T; ++t) b0[t] = b[t];
    }
}

// x phase 2 items of the rows [y0, y0 + 16 RB): item it (warp-aligned) is row y of a block of
// 16 rows; half-warp h holds k1, the other half its partner V - k1 (or the self-paired k1 = 0
// and V / 2 in the last group), for threads i0, i0 + step, ... of the items.
template <int VX, int VY, bool INV>
__device__ __forceinline__ void xy_x_p2_rows_n(float2 *A, const float2 *twx, int y0, int RB, int i0, int step)
{
    typedef XYShape<VX, VY> S;
    constexpr int T = 16;
    static_assert(VX % 2 == 0 && (16 * VX) % 32 == 0, "whole warps of row pairs");
    const int items = 16 * RB * VX;
    for (int it = i0; it < items; it += step) {
        const int l = it & 31, grp = it >> 5;
        const int h = l >> 4, jp = grp / RB;
        const int y = y0 + (grp - jp * RB) * 16 + (l & 15);
        const bool selfgrp = jp == VX / 2 - 1;  // the same for the whole warp
        const int k1 = selfgrp ? (h ? VX / 2 : 0) : (h ? VX - 1 - jp : 1 + jp);
        float2 *b0 = A + y * S::SR + T * k1;
        float2 b[T];
#pragma unroll
        for (int t = 0; t < T; ++t) b[t] = b0[t];
        xy_x_p2_item<VX, VY, INV>(b, b0, k1, h, selfgrp, twx);
    }
}

// the same for a compile-time row count NR
template <int VX, int VY, bool INV, int NR>
__device__ __forceinline__ void xy_x_p2_rows(float2 *A, const float2 *twx, int y0, int i0, int step)
{
    static_assert(NR % 16 == 0, "whole blocks of 16 rows");
    xy_x_p2_rows_n<VX, VY, INV>(A, twx, y0, NR / 16, i0, step);
}

template <int VX, int VY, bool INV>
__device__ __forceinline__ void xy_x_p2_split(float2 *A, const float2 *twx)
{
    typedef XYShape<VX, VY> S;
    static_assert(S::NT % 32 == 0, "whole warps");
    xy_x_p2_rows<VX, VY, INV, S::Py>(A, twx, 0, threadIdx.x, S::NT);
}

// x phase 2 (forward), then the packed-real split in tile order.  The DC and Nyquist
// values of a row (both real) are packed as one complex value at position 0, so that the
// y transforms run on m columns.
template <int VX, int VY>
__device__ __forceinline__ void xy_x_forward_p2(float2 *A, const float2 *twx, const int *)
{
    xy_x_p2_split<VX, VY, false>(A, twx);
    __syncthreads();
}

// Packed-real merge in tile order, then x phase 2 inverse (x phase 1 inverse follows in
// the caller).  Position 0 holds (X[0], X[m]).
template <int VX, int VY>
__device__ __forceinline__ void xy_x_inverse_p2(float2 *A, const float2 *twx, const int *)
{
    xy_x_p2_split<VX, VY, true>(A, twx);
    __syncthreads();
}

// y transforms of the m columns.  Forward: column 0 holds X[0] + i X[m] per row (two real
// sequences); afterwards it is split into the spectra of both (Hermitian in y), X[0]'s
// to column 0 and X[m]'s to column m.  Inverse: the two columns are recombined as
// Y0 + i Ym before the transform, and column 0 returns X[0] + i X[m] per row.
template <int VX, int VY, bool INV>
__device__ __forceinline__ void xy_y(float2 *A, const float2 *twy, const int *posy)
{
    typedef XYShape<VX, VY> S;
    constexpr int m = S::m, Py = S::Py, NT = S::NT;
    if (!INV) {
        tp_phase1<VY, m, 1, S::SR, false, NT>(A, twy, 1);
        __syncthreads();
        tp_phase2<VY, m, 1, S::SR, false, NT>(A);
        __syncthreads();
        for (int k = threadIdx.x; k <= Py / 2; k += NT) {
            const int g = (Py - k) % Py, pk = posy[k], pg = posy[g];
            const float2 P = A[pk * S::SR], Q = A[pg * S::SR];
            // Y0[k] = (P + conj Q) / 2, Ym[k] = -i (P - conj Q) / 2, and the same for g
            const float2 y0k = cscale(cadd(P, cconj(Q)), 0.5f), dk = cscale(csub(P, cconj(Q)), 0.5f);
            const float2 y0g = cscale(cadd(Q, cconj(P)), 0.5f), dg = cscale(csub(Q, cconj(P)), 0.5f);
            A[pk * S::SR] = y0k;
            A[pk * S::SR + m] = make_float2(dk.y, -dk.x);
            if (g != k) {
                A[pg * S::SR] = y0g;
                A[pg * S::SR + m] = make_float2(dg.y, -dg.x);
            }
        }
    } else {
        // phase 2 inverse; the items of column 0 first recombine Y0 + i Ym from columns 0 and m
        constexpr int T = 16, items = m * VY;
        for (int it = threadIdx.x; it < items; it += NT) {
            const int k1 = it / m, p = it - k1 * m;
            float2 *b0 = A + p + T * k1 * S::SR;
            float2 b[T];
#pragma unroll
            for (int t = 0; t < T; ++t) b[t] = b0[t * S::SR];
            if (p == 0) {
#pragma unroll
                for (int t = 0; t < T; ++t) {
                    const float2 c = b0[t * S::SR + m];
                    b[t] = make_float2(b[t].x - c.y, b[t].y + c.x);
                }
            }
            sdft<T, true>(b);
#pragma unroll
            for (int t = 0; t < T; ++t) b0[t * S::SR] = b[t];
        }
        __syncthreads();
        tp_phase1<VY, m, 1, S::SR, true, NT>(A, twy, 1);
    }
    __syncthreads();
}

// Shared-memory carve-up and the per-CTA tables.
template <int VX, int VY>
struct XYSmem {
    typedef XYShape<VX, VY> S;
    float2 *A, *twx, *twy;
    long long *rowb, *rowb2, *rowb3;  // per domain row: volume / block row bases (or -1)
    int *colx, *colx2, *colx3;        // per domain x: volume x of the row's voxel (or -1)
    int *posx;                        // tile position of x frequency f < m
    int *posy;                        // tile position of y frequency k < Py
    __device__ __forceinline__ XYSmem(unsigned char *raw)
    {
        A = reinterpret_cast<float2 *>(raw);
        twx = A + S::plane;
        twy = twx + S::Px;
        rowb = reinterpret_cast<long long *>(twy + S::Py);
        rowb2 = rowb + S::Py;
        rowb3 = rowb2 + S::Py;
        colx = reinterpret_cast<int *>(rowb3 + S::Py);
        colx2 = colx + S::Px;
        colx3 = colx2 + S::Px;
        posx = colx3 + S::Px;
        posy = posx + S::m;
    }
    __device__ __forceinline__ void load_tables(const float2 *__restrict__ gtwx, const float2 *__restrict__ gtwy)
    {
        for (int i = threadIdx.x; i < S::Px; i += blockDim.x) twx[i] = __ldg(&gtwx[i]);
        for (int i = threadIdx.x; i < S::Py; i += blockDim.x) twy[i] = __ldg(&gtwy[i]);
        for (int f = threadIdx.x; f < S::m; f += blockDim.x) posx[f] = f / VX + 16 * (f % VX);
        for (int k = threadIdx.x; k < S::Py; k += blockDim.x) posy[k] = k / VY + 16 * (k % VY);
    }
};

// The plane from HBM: every thread issues all its (at most 12) 16-byte loads before the
// first store, so the copy costs one memory latency.
template <int VX, int VY>
__device__ __forceinline__ void xy_load_plane(float2 *A, const float2 *__restrict__ Sp)
{
    typedef XYShape<VX, VY> SH;
    constexpr int n4 = SH::plane / 2, NT = SH::NT;
    constexpr int U = (n4 + NT - 1) / NT < 12 ? (n4 + NT - 1) / NT : 12;
    const float4 *src = reinterpret_cast<const float4 *>(Sp);
    float4 *dst = reinterpret_cast<float4 *>(A);
    for (int i0 = threadIdx.x; i0 < n4; i0 += NT * U) {
        float4 r[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = i0 + u * NT;
            if (i < n4) r[u] = __ldg(src + i);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int i = i0 + u * NT;
            if (i < n4) dst[i] = r[u];
        }
    }
}

template <int VX, int VY>
__device__ __forceinline__ void xy_store_plane(float2 *__restrict__ Sp, const float2 *A)
{
    constexpr int n4 = XYShape<VX, VY>::plane / 2;
    const float4 *src = reinterpret_cast<const float4 *>(A);
    float4 *dst = reinterpret_cast<float4 *>(Sp);
    for (int i = threadIdx.x; i < n4; i += blockDim.x) dst[i] = src[i];
}

// L2 prefetch of item `next`'s plane (persistent plane kernels): one 128-byte line per
// thread and step, issued before the current plane is transformed.
template <int VX, int VY>
__device__ __forceinline__ void xy_prefetch_next(const float2 *S, long long Pc, int z0, int nzb, int next,
                                                 int nitems)
{
    if (next >= nitems) return;
    constexpr int bytes = XYShape<VX, VY>::plane * (int)sizeof(float2), NT = XYShape<VX, VY>::NT;
    const int nb = next / nzb, nz = z0 + (next - nb * nzb);
    const char *p = reinterpret_cast<const char *>(S + (long long)nb * Pc + (long long)nz * XYShape<VX, VY>::plane);
    for (int off = threadIdx.x * 128; off < bytes; off += NT * 128)
        asm volatile("prefetch.global.L2 [%0];" ::"l"(p + off));
}

// ---- forward: source rows -> R2C x -> FFT y ---------------------------------------------
template <typename Src>
struct XYSrcTraits { static constexpr bool mirror = false; };
template <>
struct XYSrcTraits<SrcMirror<float>> { static constexpr bool mirror = true; };

// Row items (y, t) of the fused x phase 1: thread k of the CTA takes item
// it = k + r NT (r < RX), t = it % 16 (a half-warp covers 32 consecutive x of one row).
template <int VX, int VY, class Src>
__global__ void __launch_bounds__(XYShape<VX, VY>::NT, XYShape<VX, VY>::MINB)
    k_xy_fwd(Src src, float2 *__restrict__ S, const BlockMaps bms, long long Pc, const float2 *__restrict__ gtwx,
             const float2 *__restrict__ gtwy, int Pz, int nitems)
{
    typedef XYShape<VX, VY> SH;
    constexpr int NT = SH::NT, RX = SH::RX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    XYSmem<VX, VY> sm(smem_raw);
    pdl_trigger();
    sm.load_tables(gtwx, gtwy);
    constexpr bool MIR = XYSrcTraits<Src>::mirror;
    pdl_wait();  // the source volume is the predecessor's output
    // persistent: the CTA walks the (block, plane) items blockIdx.x, + gridDim.x, ...
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int bi = item / Pz, z = item - bi * Pz;
        const BlockMap &bm = bms.m[bi];
        float2 *Sp = S + (long long)bi * Pc + (long long)z * SH::plane;
        for (int y = threadIdx.x; y < SH::Py; y += NT) {
            const typename Src::Row r = src.row(bm, y, z);
            sm.rowb[y] = r.base;
        }
        if (MIR)
            for (int x = threadIdx.x; x < SH::Px; x += NT) sm.colx[x] = (int)mirror_x(bm, x);
        __syncthreads();
        // all loads of the thread's row items first, then their x phase 1
        float2 a[RX][VX];
#pragma unroll
        for (int r = 0; r < RX; ++r) {
            const int it = threadIdx.x + r * NT, t = it & 15, y = it >> 4;
#pragma unroll
            for (int v = 0; v < VX; ++v) {
                const int x = 2 * (t + 16 * v);
                if constexpr (MIR) {
                    const float *pr = src.vol + sm.rowb[y];
                    const int2 cx = *reinterpret_cast<const int2 *>(sm.colx + x);  // x even: one 8-byte read
                    a[r][v] = make_float2(__ldg(pr + cx.x), __ldg(pr + cx.y));
                } else {
                    typename Src::Row row;
                    row.base = sm.rowb[y];
                    a[r][v] = make_float2(src.template at<float>(row, bm, x), src.template at<float>(row, bm, x + 1));
                }
            }
        }
#pragma unroll
        for (int r = 0; r < RX; ++r) {
            const int it = threadIdx.x + r * NT, t = it & 15, y = it >> 4;
            xrow_p1<VX, false>(a[r], sm.twx, t);
#pragma unroll
            for (int v = 0; v < VX; ++v) sm.A[y * SH::SR + t + 16 * v] = a[r][v];
        }
        __syncthreads();
        xy_x_forward_p2<VX, VY>(sm.A, sm.twx, sm.posx);
        xy_y<VX, VY, false>(sm.A, sm.twy, sm.posy);
        xy_store_plane<VX, VY>(Sp, sm.A);
        __syncthreads();  // the next item rewrites the plane and the row / column tables
    }
}

// ---- C2R -> quotient -> R2C ----------------------------------------------------------
// The CTAs walk the planes [z0, z0 + nzb) of every block of the batch (items nb * nzb).
// DeconvolutionMethods.java:71-74: img > 0 ? img / conv1 : 1.  Domain voxels outside the
// block (the value-1 extension) and outside the volume (img zero-extended) read img = 0.
// x phase 1 inverse, the quotient and x phase 1 forward run on registers per row item.
template <int VX, int VY>
__global__ void __launch_bounds__(XYShape<VX, VY>::NT, XYShape<VX, VY>::MINB)
    k_xy_ratio(float2 *__restrict__ S, const float *__restrict__ img, const BlockMaps bms, long long Pc,
               const float2 *__restrict__ gtwx, const float2 *__restrict__ gtwy, int z0, int nzb, int nitems)
{
    typedef XYShape<VX, VY> SH;
    constexpr int NT = SH::NT, RX = SH::RX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    XYSmem<VX, VY> sm(smem_raw);
    pdl_trigger();
    sm.load_tables(gtwx, gtwy);
    pdl_wait();
    // persistent: the CTA walks the (block, plane) items blockIdx.x, + gridDim.x, ...
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int bi = item / nzb, z = z0 + (item - bi * nzb);
        const BlockMap &bm = bms.m[bi];
        float2 *Sp = S + (long long)bi * Pc + (long long)z * SH::plane;
        const int ez = ext_e(z, bm.P[2], bm.L[2]);
        for (int y = threadIdx.x; y < SH::Py; y += NT) {
            const int ey = ext_e(y, bm.P[1], bm.L[1]);
            const bool rin = ey >= 0 && ey < bm.b[1] && ez >= 0 && ez < bm.b[2];
            sm.rowb[y] = rin ? zero_row(bm, ey, ez).base : -1;
        }
        for (int x = threadIdx.x; x < SH::Px; x += NT) {
            const int bx = ext_e(x, bm.P[0], bm.L[0]);
            const long long gx = bm.off[0] + bx;
            sm.colx[x] = (bx >= 0 && bx < bm.b[0] && gx >= 0 && gx < bm.D[0]) ? (int)gx : -1;
        }
        xy_load_plane<VX, VY>(sm.A, Sp);
        __syncthreads();
        xy_y<VX, VY, true>(sm.A, sm.twy, sm.posy);
        xy_x_inverse_p2<VX, VY>(sm.A, sm.twx, sm.posx);
#pragma unroll 1
        for (int r = 0; r < RX; ++r) {
            const int it = threadIdx.x + r * NT, t = it & 15, y = it >> 4;
            const long long rb = sm.rowb[y];
            float im[VX][2];
#pragma unroll
            for (int v = 0; v < VX; ++v) {
                const int2 cx = *reinterpret_cast<const int2 *>(sm.colx + 2 * (t + 16 * v));
                im[v][0] = (rb >= 0 && cx.x >= 0) ? __ldg(img + rb + cx.x) : 0.0f;
                im[v][1] = (rb >= 0 && cx.y >= 0) ? __ldg(img + rb + cx.y) : 0.0f;
            }
            float2 a[VX];
            float2 *row = sm.A + y * SH::SR + t;
#pragma unroll
            for (int v = 0; v < VX; ++v) a[v] = row[16 * v];
            xrow_p1<VX, true>(a, sm.twx, t);  // natural order: a[v] = conv1 at x = 2 (t + 16 v) + {0, 1}
#pragma unroll
            for (int v = 0; v < VX; ++v)
                a[v] = make_float2(quotient_fast(im[v][0], a[v].x), quotient_fast(im[v][1], a[v].y));
            xrow_p1<VX, false>(a, sm.twx, t);
#pragma unroll
            for (int v = 0; v < VX; ++v) row[16 * v] = a[v];
        }
        // the next item's plane into L2 while this one is transformed forward
        xy_prefetch_next<VX, VY>(S, Pc, z0, nzb, item + gridDim.x, nitems);
        __syncthreads();
        xy_x_forward_p2<VX, VY>(sm.A, sm.twx, sm.posx);
        xy_y<VX, VY, false>(sm.A, sm.twy, sm.posy);
        xy_store_plane<VX, VY>(Sp, sm.A);
        __syncthreads();  // the next item rewrites the plane and the row / column tables
    }
}

// ---- C2R -> update epilogue --------------------------------------------------------------
// WR (with EPI_SEQ, for runs without statistics, ua.prune): only the write region's voxels are
// updated, through the x transform of its rows alone, and only their psi and weight are read;
// a separate instantiation, so that the form with statistics keeps its own register budget.
template <int VX, int VY, int EPI, bool WR = false>
__global__ void __launch_bounds__(XYShape<VX, VY>::NT, XYShape<VX, VY>::MINB)
    k_xy_update(float2 *__restrict__ S, UpdateArgs ua, const BlockMaps bms, long long Pc,
                const float2 *__restrict__ gtwx, const float2 *__restrict__ gtwy)
{
    typedef XYShape<VX, VY> SH;
    constexpr int NT = SH::NT, RX = SH::RX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red_s[32], red_m[32];
    XYSmem<VX, VY> sm(smem_raw);
    pdl_trigger();
    const BlockMap &bm = bms.m[blockIdx.y];
    int z = blockIdx.x;
    if (ua.prune) {  // the grid covers the deepest write region of the batch
        z += bm.wlo[2];
        if (z >= bm.whi[2]) return;
    }
    float2 *Sp = S + (long long)blockIdx.y * Pc + (long long)z * SH::plane;
    const long long bvox = (long long)bm.b[0] * bm.b[1] * bm.b[2];
    if (ua.prod) ua.prod = reinterpret_cast<float2 *>(ua.prod) + (long long)blockIdx.y * bvox;  // mulprod_* pairs
    if (ua.store) ua.store += (long long)blockIdx.y * bvox;
    sm.load_tables(gtwx, gtwy);
    float ksum = 0.0f, kcomp = 0.0f, kmax = -1.0f;
    if constexpr (EPI == EPI_SEQ) {
        // Seq epilogue (computeFinalValues / computeNextValue, DeconvolutionMethods.java
        // 103-182, 320-358) fused with x phase 1 inverse on the row items
        const bool zin = z < bm.b[2];  // extension planes carry no block voxels
        const bool zw = z >= bm.wlo[2] && z < bm.whi[2];
        for (int y = threadIdx.x; y < SH::Py; y += NT) {
            const bool in = zin && y < bm.b[1];
            sm.rowb[y] = in ? mirror_row(bm, y, z).base : -1;
            sm.rowb2[y] = in ? zero_row(bm, y, z).base : -1;
            // output row base (negative for blocks left of the volume; rows outside the
            // write region carry kNoRow)
            sm.rowb3[y] = (in && zw && y >= bm.wlo[1] && y < bm.whi[1])
                              ? ((bm.ooff[2] + z) * bm.OD[1] + (bm.ooff[1] + y)) * bm.OD[0] + bm.ooff[0]
                              : kNoRow;
        }
        for (int x = threadIdx.x; x < SH::Px; x += NT) {
            const bool in = x < bm.b[0];
            const long long gx = bm.off[0] + x;
            sm.colx[x] = in ? (int)mirror_x(bm, x) : -1;
            sm.colx2[x] = (in && gx >= 0 && gx < bm.D[0]) ? (int)gx : -1;
            sm.colx3[x] = (in && x >= bm.wlo[0] && x < bm.whi[0]) ? x : -1;
        }
        pdl_wait();
        xy_load_plane<VX, VY>(sm.A, Sp);
        __syncthreads();
        xy_y<VX, VY, true>(sm.A, sm.twy, sm.posy);
        if constexpr (WR) {
            // only the rows of the write region go on through the x transform (in whole
            // blocks of 16 rows)
            const int y0 = bm.wlo[1] & ~15, y1 = min(SH::Py, (bm.whi[1] + 15) & ~15);
            if (y1 > y0) xy_x_p2_rows_n<VX, VY, true>(sm.A, sm.twx, y0, (y1 - y0) >> 4, threadIdx.x, NT);
            __syncthreads();
        } else {
            xy_x_inverse_p2<VX, VY>(sm.A, sm.twx, sm.posx);
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
        // ST: every block voxel is updated and its change summed (the statistics)
        constexpr bool ST = !WR;
        {
#pragma unroll 1
            for (int r = 0; r < RX; ++r) {
                const int it = threadIdx.x + r * NT, t = it & 15, y = it >> 4;
                const long long pb = sm.rowb[y], wb = sm.rowb2[y], ob = sm.rowb3[y];
                // not a block row / not written
                if (pb < 0 || ((!ST || ua.prune) && ob == kNoRow)) continue;
                float pv[VX][2], wv[VX][2];
#pragma unroll
                for (int v = 0; v < VX; ++v) {
                    const int x = 2 * (t + 16 * v);  // even: the pair of table entries is one 8-byte read
                    const int2 mx = *reinterpret_cast<const int2 *>(sm.colx + x);
                    const int2 gx = *reinterpret_cast<const int2 *>(sm.colx2 + x);
                    const int2 c3 = *reinterpret_cast<const int2 *>(sm.colx3 + x);
                    const bool u0 = mx.x >= 0 && (ST || c3.x >= 0), u1 = mx.y >= 0 && (ST || c3.y >= 0);
                    pv[v][0] = u0 ? __ldg(psrc + pb + mx.x) : 0.0f;
                    pv[v][1] = u1 ? __ldg(psrc + pb + mx.y) : 0.0f;
                    wv[v][0] = (u0 && wb >= 0 && gx.x >= 0) ? __ldg(wgt + wb + gx.x) : 0.0f;
                    wv[v][1] = (u1 && wb >= 0 && gx.y >= 0) ? __ldg(wgt + wb + gx.y) : 0.0f;
                }
                float2 a[VX];
                const float2 *row = sm.A + y * SH::SR + t;
#pragma unroll
                for (int v = 0; v < VX; ++v) a[v] = row[16 * v];
                xrow_p1<VX, true>(a, sm.twx, t);  // natural order: conv2 at x = 2 (t + 16 v) + {0, 1}
#pragma unroll
                for (int v = 0; v < VX; ++v) {
                    const float cv[2] = {a[v].x, a[v].y};
                    const int2 cx = *reinterpret_cast<const int2 *>(sm.colx + 2 * (t + 16 * v));
                    const int2 c3 = *reinterpret_cast<const int2 *>(sm.colx3 + 2 * (t + 16 * v));
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int x = 2 * (t + 16 * v) + h;
                        if ((h ? cx.y : cx.x) < 0) continue;  // beyond the block
                        const bool w = ob != kNoRow && (h ? c3.y : c3.x) >= 0;
                        if (!ST && !w) continue;
                        const float last = pv[v][h];
                        const float next = next_value_fast(last, cv[h], wv[v][h], uc);
                        if constexpr (ST) {
                            const float ch = next - last;  // signed change (DeconvolutionMethods.java:308)
                            const float ky = ch - kcomp;
                            const float kt = ksum + ky;
                            kcomp = (kt - ksum) - ky;
                            ksum = kt;
                            kmax = kmax > ch ? kmax : ch;
                        }
                        if (w) pdst[ob + x] = next;
                    }
                }
            }
        }
    } else {
        pdl_wait();
        xy_load_plane<VX, VY>(sm.A, Sp);
        __syncthreads();
        xy_y<VX, VY, true>(sm.A, sm.twy, sm.posy);
        xy_x_inverse_p2<VX, VY>(sm.A, sm.twx, sm.posx);
        tp_phase1<VX, SH::Py, SH::SR, 1, true, NT>(sm.A, sm.twx, 2);
        __syncthreads();
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = NT >> 5;
        const int ylo = ua.prune ? bm.wlo[1] : 0, yhi = ua.prune ? bm.whi[1] : bm.b[1];
        if (z < bm.b[2])  // extension planes carry no block voxels
            for (int y = ylo + warp; y < yhi && y < SH::Py; y += nw)
                update_row<float, EPI>(sm.A + y * SH::SR, SH::m, bm, ua, y, z, lane, ksum, kcomp, kmax);
    }
    // pruned runs skip the statistics, but the likelihood is reduced over the write region
    if ((EPI == EPI_SEQ || EPI == EPI_MUL_FINAL || EPI == EPI_NLL) && (!ua.prune || EPI == EPI_NLL))
        stats_to_partials(ksum, kcomp, kmax, red_s, red_m, ua.partials, (long long)blockIdx.y * gridDim.x + blockIdx.x);
}

}  // namespace mvr
