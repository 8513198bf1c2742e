// Pair plane kernels: the x and y transforms of one z-plane on a cluster of two CTAs, each
// holding half of the plane's rows in its shared memory, for planes too large for one CTA
// (256 x 256: 264 KB) or, at half the shared memory per CTA, with two CTAs per SM.
//
// CTA r of the pair (r = %cluster_ctarank) holds the H = Py / 2 rows [r H, r H + H) for the x
// transforms (rows are local).  The y transform of length Py = 2 H is split as
//   forward (decimation in frequency): u_j = a_j + a_{j+H},  v_j = (a_j - a_{j+H}) W_Py^j,
//            then the H-point FFTs of u (CTA 0: the even frequencies X[2k]) and of v (CTA 1:
//            the odd frequencies X[2k + 1]);
//   inverse (decimation in time): the H-point inverse FFTs of each CTA's half spectrum, then
//            a_j = u_j + W_Py^-j v_j, a_{j+H} = u_j - W_Py^-j v_j,
// so the only exchange between the two CTAs is the radix-2 butterfly, read from the
// partner's shared memory (distributed shared memory) between two cluster barriers.  The
// H-point FFTs are the two-phase register FFTs of the single-CTA plane kernels (H = 16 VH,
// tile order: frequency k' at row k' / VH + 16 (k' % VH)), fused with the butterfly on the
// phase-1 items.  A CTA's half spectrum is stored at rows [r H, r H + H) of the plane in S, so
// the spectrum's y order is (k mod 2, tile position of k / 2); every spectrum (data, K1^, K2^)
// comes from the same kernels, so the spectral product stays position by position.
//
// The packed-real column 0 (X[0] + i X[m] of every row) is split after the y transform into
// the spectra of its two real columns; frequency k pairs with Py - k, which lies in the same
// half (k' <-> (H - k') mod H for even k, k' <-> H - 1 - k' for odd k).
#pragma once
#include "xy_plane.cuh"

namespace mvr {

// ---- cluster primitives (PTX) --------------------------------------------------------
__device__ __forceinline__ unsigned cluster_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// Every thread of both CTAs; orders shared-memory writes before the barrier with reads after.
__device__ __forceinline__ void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
// The address of the same shared-memory variable in CTA `rank` of the cluster.
__device__ __forceinline__ unsigned map_cluster(unsigned local, unsigned rank)
{
    unsigned r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(local), "r"(rank));
    return r;
}
__device__ __forceinline__ float2 ld_cluster(unsigned addr)
{
    float2 v;
    asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
    return v;
}

template <int VX, int VH>
struct PairShape {
    static constexpr int m = 16 * VX;      // packed complex values per real x row
    static constexpr int Px = 2 * m;
    static constexpr int H = 16 * VH;      // rows per CTA
    static constexpr int Py = 2 * H;
    static constexpr int SR = m + 1;       // row stride
    static constexpr int half = H * SR;    // complex values per CTA
    static constexpr int plane = Py * SR;  // complex values per plane in S
    // 512 threads and two CTAs per SM for the 192-wide planes (83 KB each), 1024 threads and
    // one CTA per SM for 256 (143 KB)
    static constexpr int NT = (VX >= 8 || VH >= 8) ? 1024 : 512;
    static constexpr int MINB = NT == 1024 ? 1 : 2;
    static constexpr int RX = H * 16 / NT;  // rounds of the x phase-1 row items (y, t)
    static constexpr int RY = m * 16 / NT;  // rounds of the y phase-1 column items (p, t)
    static_assert((H * 16) % NT == 0 && (m * 16) % NT == 0, "whole rounds");
};

template <int VX, int VH>
constexpr size_t pair_smem_bytes()
{
    typedef PairShape<VX, VH> S;
    return sizeof(float2) * (size_t)(S::half + S::Px + S::Py) + 3 * sizeof(long long) * S::H +
           sizeof(int) * (size_t)(3 * S::Px + S::m + S::H);
}

template <int VX, int VH>
struct PairSmem {
    typedef PairShape<VX, VH> S;
    float2 *A, *twx, *twy;
    long long *rowb, *rowb2, *rowb3;
    int *colx, *colx2, *colx3;
    int *posx, *posh;
    __device__ __forceinline__ PairSmem(unsigned char *raw)
    {
        A = reinterpret_cast<float2 *>(raw);
        twx = A + S::half;
        twy = twx + S::Px;
        rowb = reinterpret_cast<long long *>(twy + S::Py);
        rowb2 = rowb + S::H;
        rowb3 = rowb2 + S::H;
        colx = reinterpret_cast<int *>(rowb3 + S::H);
        colx2 = colx + S::Px;
        colx3 = colx2 + S::Px;
        posx = colx3 + S::Px;
        posh = posx + S::m;
    }
    __device__ __forceinline__ void load_tables(const float2 *__restrict__ gtwx, const float2 *__restrict__ gtwy)
    {
        for (int i = threadIdx.x; i < S::Px; i += blockDim.x) twx[i] = __ldg(&gtwx[i]);
        for (int i = threadIdx.x; i < S::Py; i += blockDim.x) twy[i] = __ldg(&gtwy[i]);
        for (int f = threadIdx.x; f < S::m; f += blockDim.x) posx[f] = f / VX + 16 * (f % VX);
        for (int k = threadIdx.x; k < S::H; k += blockDim.x) posh[k] = k / VH + 16 * (k % VH);
    }
};

// x phase 2 with the packed-real split / merge over the CTA's H rows (the row items of
// xy_x_p2_split on a row count of H): lanes 0-15 item k1, lanes 16-31 the partner item
// VX - k1 of the same 16 rows; the pair group (0, VX / 2) is self-paired.
template <int VX, int VH, bool INV>
__device__ __forceinline__ void pair_x_p2(float2 *A, const float2 *twx)
{
    typedef PairShape<VX, VH> S;
    constexpr int T = 16, NT = S::NT, RB = S::H / 16, items = S::H * VX;
    static_assert(VX % 2 == 0 && items % 32 == 0, "whole warps of row pairs");
    for (int it = threadIdx.x; it < items; it += NT) {
        const int l = it & 31, grp = it >> 5;
        const int h = l >> 4, jp = grp / RB;
        const int y = (grp - jp * RB) * 16 + (l & 15);
        const bool selfgrp = jp == VX / 2 - 1;
        const int k1 = selfgrp ? (h ? VX / 2 : 0) : (h ? VX - 1 - jp : 1 + jp);
        float2 *b0 = A + y * S::SR + T * k1;
        float2 b[T];
#pragma unroll
        for (int t = 0; t < T; ++t) b[t] = b0[t];
        if (!INV) sdft<T, false>(b);
        if (!selfgrp) {
#pragma unroll
            for (int k2 = 0; k2 < T / 2; ++k2) {
                const int k3 = T - 1 - k2;
                float2 ga, gb;
                ga.x = __shfl_xor_sync(0xffffffffu, b[k3].x, 16);
                ga.y = __shfl_xor_sync(0xffffffffu, b[k3].y, 16);
                gb.x = __shfl_xor_sync(0xffffffffu, b[k2].x, 16);
                gb.y = __shfl_xor_sync(0xffffffffu, b[k2].y, 16);
                const float2 oa = xy_split_one<VX, VH, INV>(b[k2], ga, k1 + VX * k2, twx);
                const float2 ob = xy_split_one<VX, VH, INV>(b[k3], gb, k1 + VX * k3, twx);
                if (INV) {
                    b[k2] = oa;
                    b[k3] = ob;
                } else {
                    b0[k2] = oa;
                    b0[k3] = ob;
                }
            }
        } else if (h == 0) {
            const float2 o0 = xy_split_one<VX, VH, INV>(b[0], b[0], 0, twx);
            const float2 o8 = xy_split_one<VX, VH, INV>(b[8], b[8], VX * 8, twx);
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
                const float2 oa = xy_split_one<VX, VH, INV>(b[k2], b[k3], VX * k2, twx);
                const float2 ob = xy_split_one<VX, VH, INV>(b[k3], b[k2], VX * k3, twx);
                if (INV) {
                    b[k2] = oa;
                    b[k3] = ob;
                } else {
                    b0[k2] = oa;
                    b0[k3] = ob;
                }
            }
        } else {
#pragma unroll
            for (int k2 = 0; k2 < T / 2; ++k2) {
                const int k3 = T - 1 - k2;
                const float2 oa = xy_split_one<VX, VH, INV>(b[k2], b[k3], VX / 2 + VX * k2, twx);
                const float2 ob = xy_split_one<VX, VH, INV>(b[k3], b[k2], VX / 2 + VX * k3, twx);
                if (INV) {
                    b[k2] = oa;
                    b[k3] = ob;
                } else {
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
    __syncthreads();
}

// Forward y transform of the pair (after both CTAs' x passes; starts with a cluster barrier):
// the radix-2 butterfly with the partner's rows fused into phase 1 of the H-point FFT, then
// phase 2 and the split of the packed column 0 into columns 0 and m.
template <int VX, int VH>
__device__ __forceinline__ void pair_y_forward(float2 *A, const float2 *twy, const int *posh, unsigned rank)
{
    typedef PairShape<VX, VH> S;
    constexpr int m = S::m, H = S::H, SR = S::SR, NT = S::NT, RY = S::RY;
    cluster_sync();  // both halves hold their x spectra
    const unsigned rbase = map_cluster(smem_addr(A), rank ^ 1u);
    float2 a[RY][VH];
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        const int it = threadIdx.x + r * NT, t = it / m, p = it - t * m;
#pragma unroll
        for (int v = 0; v < VH; ++v) {
            const int idx = (t + 16 * v) * SR + p;
            const float2 own = A[idx], rem = ld_cluster(rbase + 8u * (unsigned)idx);
            a[r][v] = rank == 0 ? cadd(own, rem) : csub(rem, own);
        }
    }
    cluster_sync();  // the partner has read this half
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        const int it = threadIdx.x + r * NT, t = it / m, p = it - t * m;
        if (rank)
#pragma unroll
            for (int v = 0; v < VH; ++v) a[r][v] = cmul(a[r][v], twy[t + 16 * v]);  // W_Py^j, j = t + 16 v
        sdft<VH, false>(a[r]);
#pragma unroll
        for (int k1 = 1; k1 < VH; ++k1) a[r][k1] = cmul(a[r][k1], twy[2 * t * k1]);  // W_H^(t k1)
#pragma unroll
        for (int v = 0; v < VH; ++v) A[(t + 16 * v) * SR + p] = a[r][v];
    }
    __syncthreads();
    tp_phase2<VH, m, 1, SR, false, NT>(A);
    __syncthreads();
    // column 0 holds Z[k] = Y0[k] + i Ym[k] (k = 2 k' + rank): Y0 to column 0, Ym to column m
    for (int kp = threadIdx.x; kp < H; kp += NT) {
        const int kq = rank == 0 ? (H - kp) % H : H - 1 - kp;
        if (kq < kp) continue;  // every pair once
        const int pk = posh[kp], pg = posh[kq];
        const float2 P = A[pk * SR], Q = A[pg * SR];
        const float2 y0k = cscale(cadd(P, cconj(Q)), 0.5f), dk = cscale(csub(P, cconj(Q)), 0.5f);
        const float2 y0g = cscale(cadd(Q, cconj(P)), 0.5f), dg = cscale(csub(Q, cconj(P)), 0.5f);
        A[pk * SR] = y0k;
        A[pk * SR + m] = make_float2(dk.y, -dk.x);
        if (kq != kp) {
            A[pg * SR] = y0g;
            A[pg * SR + m] = make_float2(dg.y, -dg.x);
        }
    }
    __syncthreads();
}

// Inverse y transform of the pair: phase 2 inverse (column 0 first recombines Y0 + i Ym from
// columns 0 and m), phase 1 inverse, then the radix-2 butterfly with the partner's values.
template <int VX, int VH>
__device__ __forceinline__ void pair_y_inverse(float2 *A, const float2 *twy, unsigned rank)
{
    typedef PairShape<VX, VH> S;
    constexpr int m = S::m, SR = S::SR, NT = S::NT, RY = S::RY, T = 16, items = m * VH;
    for (int it = threadIdx.x; it < items; it += NT) {
        const int k1 = it / m, p = it - k1 * m;
        float2 *b0 = A + p + T * k1 * SR;
        float2 b[T];
#pragma unroll
        for (int t = 0; t < T; ++t) b[t] = b0[t * SR];
        if (p == 0) {
#pragma unroll
            for (int t = 0; t < T; ++t) {
                const float2 c = b0[t * SR + m];
                b[t] = make_float2(b[t].x - c.y, b[t].y + c.x);
            }
        }
        sdft<T, true>(b);
#pragma unroll
        for (int t = 0; t < T; ++t) b0[t * SR] = b[t];
    }
    __syncthreads();
    float2 a[RY][VH];
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        const int it = threadIdx.x + r * NT, t = it / m, p = it - t * m;
#pragma unroll
        for (int v = 0; v < VH; ++v) a[r][v] = A[(t + 16 * v) * SR + p];
#pragma unroll
        for (int k1 = 1; k1 < VH; ++k1) a[r][k1] = cmul(a[r][k1], cconj(twy[2 * t * k1]));
        sdft<VH, true>(a[r]);  // natural order: a[r][v] = u (CTA 0) or v (CTA 1) at row t + 16 v
#pragma unroll
        for (int v = 0; v < VH; ++v) A[(t + 16 * v) * SR + p] = a[r][v];
    }
    cluster_sync();  // both halves hold u / v
    const unsigned rbase = map_cluster(smem_addr(A), rank ^ 1u);
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        const int it = threadIdx.x + r * NT, t = it / m, p = it - t * m;
#pragma unroll
        for (int v = 0; v < VH; ++v) {
            const int idx = (t + 16 * v) * SR + p;
            const float2 rem = ld_cluster(rbase + 8u * (unsigned)idx);
            const float2 w = cconj(twy[t + 16 * v]);
            a[r][v] = rank == 0 ? cadd(a[r][v], cmul(w, rem)) : csub(rem, cmul(w, a[r][v]));
        }
    }
    cluster_sync();  // the partner has read this half
#pragma unroll
    for (int r = 0; r < RY; ++r) {
        const int it = threadIdx.x + r * NT, t = it / m, p = it - t * m;
#pragma unroll
        for (int v = 0; v < VH; ++v) A[(t + 16 * v) * SR + p] = a[r][v];
    }
    __syncthreads();
}

template <int VX, int VH>
__device__ __forceinline__ void pair_load(float2 *A, const float2 *__restrict__ Sp)
{
    typedef PairShape<VX, VH> SH;
    constexpr int n4 = SH::half / 2, NT = SH::NT;
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

template <int VX, int VH>
__device__ __forceinline__ void pair_store(float2 *__restrict__ Sp, const float2 *A)
{
    constexpr int n4 = PairShape<VX, VH>::half / 2;
    const float4 *src = reinterpret_cast<const float4 *>(A);
    float4 *dst = reinterpret_cast<float4 *>(Sp);
    for (int i = threadIdx.x; i < n4; i += blockDim.x) dst[i] = src[i];
}

// ---- forward: source rows -> R2C x -> FFT y (persistent: a cluster walks the planes) -----
template <int VX, int VH, class Src>
__global__ void __launch_bounds__(PairShape<VX, VH>::NT, PairShape<VX, VH>::MINB)
    k_xy2_fwd(Src src, float2 *__restrict__ S, const BlockMaps bms, long long Pc, const float2 *__restrict__ gtwx,
              const float2 *__restrict__ gtwy, int Pz, int nitems)
{
    typedef PairShape<VX, VH> SH;
    constexpr int NT = SH::NT, RX = SH::RX, H = SH::H;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PairSmem<VX, VH> sm(smem_raw);
    const unsigned rank = cluster_rank();
    const int y0 = (int)rank * H;
    pdl_trigger();
    sm.load_tables(gtwx, gtwy);
    constexpr bool MIR = XYSrcTraits<Src>::mirror;
    pdl_wait();
    const int nclusters = gridDim.x >> 1;
    for (int item = blockIdx.x >> 1; item < nitems; item += nclusters) {
        const int bi = item / Pz, z = item - bi * Pz;
        const BlockMap &bm = bms.m[bi];
        float2 *Sp = S + (long long)bi * Pc + (long long)z * SH::plane + (long long)rank * SH::half;
        for (int y = threadIdx.x; y < H; y += NT) sm.rowb[y] = src.row(bm, y0 + y, z).base;
        if (MIR)
            for (int x = threadIdx.x; x < SH::Px; x += NT) sm.colx[x] = (int)mirror_x(bm, x);
        __syncthreads();
        float2 a[RX][VX];
#pragma unroll
        for (int r = 0; r < RX; ++r) {
            const int it = threadIdx.x + r * NT, t = it & 15, y = it >> 4;
#pragma unroll
            for (int v = 0; v < VX; ++v) {
                const int x = 2 * (t + 16 * v);
                if constexpr (MIR) {
                    const float *pr = src.vol + sm.rowb[y];
                    const int2 cx = *reinterpret_cast<const int2 *>(sm.colx + x);
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
        pair_x_p2<VX, VH, false>(sm.A, sm.twx);
        pair_y_forward<VX, VH>(sm.A, sm.twy, sm.posh, rank);
        pair_store<VX, VH>(Sp, sm.A);
        __syncthreads();
    }
}

// ---- C2R -> quotient -> R2C --------------------------------------------------------------
template <int VX, int VH>
__global__ void __launch_bounds__(PairShape<VX, VH>::NT, PairShape<VX, VH>::MINB)
    k_xy2_ratio(float2 *__restrict__ S, const float *__restrict__ img, const BlockMaps bms, long long Pc,
                const float2 *__restrict__ gtwx, const float2 *__restrict__ gtwy, int z0, int nzb, int nitems)
{
    typedef PairShape<VX, VH> SH;
    constexpr int NT = SH::NT, RX = SH::RX, H = SH::H;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PairSmem<VX, VH> sm(smem_raw);
    const unsigned rank = cluster_rank();
    const int y0 = (int)rank * H;
    pdl_trigger();
    sm.load_tables(gtwx, gtwy);
    pdl_wait();
    const int nclusters = gridDim.x >> 1;
    for (int item = blockIdx.x >> 1; item < nitems; item += nclusters) {
        const int bi = item / nzb, z = z0 + (item - bi * nzb);
        const BlockMap &bm = bms.m[bi];
        float2 *Sp = S + (long long)bi * Pc + (long long)z * SH::plane + (long long)rank * SH::half;
        const int ez = ext_e(z, bm.P[2], bm.L[2]);
        for (int y = threadIdx.x; y < H; y += NT) {
            const int ey = ext_e(y0 + y, bm.P[1], bm.L[1]);
            const bool rin = ey >= 0 && ey < bm.b[1] && ez >= 0 && ez < bm.b[2];
            sm.rowb[y] = rin ? zero_row(bm, ey, ez).base : -1;
        }
        for (int x = threadIdx.x; x < SH::Px; x += NT) {
            const int bx = ext_e(x, bm.P[0], bm.L[0]);
            const long long gx = bm.off[0] + bx;
            sm.colx[x] = (bx >= 0 && bx < bm.b[0] && gx >= 0 && gx < bm.D[0]) ? (int)gx : -1;
        }
        pair_load<VX, VH>(sm.A, Sp);
        __syncthreads();
        pair_y_inverse<VX, VH>(sm.A, sm.twy, rank);
        pair_x_p2<VX, VH, true>(sm.A, sm.twx);
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
            xrow_p1<VX, true>(a, sm.twx, t);
#pragma unroll
            for (int v = 0; v < VX; ++v)
                a[v] = make_float2(quotient_fast(im[v][0], a[v].x), quotient_fast(im[v][1], a[v].y));
            xrow_p1<VX, false>(a, sm.twx, t);
#pragma unroll
            for (int v = 0; v < VX; ++v) row[16 * v] = a[v];
        }
        // the next item's half plane into L2 while this one is transformed forward
        {
            const int next = item + nclusters;
            if (next < nitems) {
                const int nbi = next / nzb, nz = z0 + (next - nbi * nzb);
                const char *np = reinterpret_cast<const char *>(S + (long long)nbi * Pc + (long long)nz * SH::plane +
                                                                (long long)rank * SH::half);
                for (int off = threadIdx.x * 128; off < SH::half * (int)sizeof(float2); off += NT * 128)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(np + off));
            }
        }
        __syncthreads();
        pair_x_p2<VX, VH, false>(sm.A, sm.twx);
        pair_y_forward<VX, VH>(sm.A, sm.twy, sm.posh, rank);
        pair_store<VX, VH>(Sp, sm.A);
        __syncthreads();
    }
}

// ---- C2R -> update epilogue (one cluster per plane: blockIdx.x = 2 z + rank) ------------
template <int VX, int VH, int EPI>
__global__ void __launch_bounds__(PairShape<VX, VH>::NT, PairShape<VX, VH>::MINB)
    k_xy2_update(float2 *__restrict__ S, UpdateArgs ua, const BlockMaps bms, long long Pc,
                 const float2 *__restrict__ gtwx, const float2 *__restrict__ gtwy)
{
    typedef PairShape<VX, VH> SH;
    constexpr int NT = SH::NT, RX = SH::RX, H = SH::H;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red_s[32], red_m[32];
    PairSmem<VX, VH> sm(smem_raw);
    const unsigned rank = cluster_rank();
    const int y0 = (int)rank * H;
    pdl_trigger();
    const BlockMap &bm = bms.m[blockIdx.y];
    int z = blockIdx.x >> 1;
    if (ua.prune) z += bm.wlo[2];  // the grid covers the deepest write region of the batch
    // both CTAs of the pair take the same z; a plane beyond this block's write region has no
    // work, and both leave before any cluster barrier
    if (ua.prune && z >= bm.whi[2]) return;
    float2 *Sp = S + (long long)blockIdx.y * Pc + (long long)z * SH::plane + (long long)rank * SH::half;
    const long long bvox = (long long)bm.b[0] * bm.b[1] * bm.b[2];
    if (ua.prod) ua.prod = reinterpret_cast<float2 *>(ua.prod) + (long long)blockIdx.y * bvox;
    if (ua.store) ua.store += (long long)blockIdx.y * bvox;
    sm.load_tables(gtwx, gtwy);
    float ksum = 0.0f, kcomp = 0.0f, kmax = -1.0f;
    if constexpr (EPI == EPI_SEQ) {
        const bool zin = z < bm.b[2];
        const bool zw = z >= bm.wlo[2] && z < bm.whi[2];
        for (int yl = threadIdx.x; yl < H; yl += NT) {
            const int y = y0 + yl;
            const bool in = zin && y < bm.b[1];
            sm.rowb[yl] = in ? mirror_row(bm, y, z).base : -1;
            sm.rowb2[yl] = in ? zero_row(bm, y, z).base : -1;
            sm.rowb3[yl] = (in && zw && y >= bm.wlo[1] && y < bm.whi[1])
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
        pair_load<VX, VH>(sm.A, Sp);
        __syncthreads();
        pair_y_inverse<VX, VH>(sm.A, sm.twy, rank);
        pair_x_p2<VX, VH, true>(sm.A, sm.twx);
        const float *psrc = reinterpret_cast<const float *>(ua.psi_src);
        float *pdst = reinterpret_cast<float *>(ua.psi_dst);
        const float *wgt = ua.weight[0];
        UpdConst uc;
        uc.minI = ua.minI;
        uc.maxI = ua.maxI;
        uc.inv_maxI = 1.0f / ua.maxI;
        uc.two_lambda = ua.two_lambda;
        uc.tik = ua.tik != 0;
#pragma unroll 1
        for (int r = 0; r < RX; ++r) {
            const int it = threadIdx.x + r * NT, t = it & 15, y = it >> 4;
            const long long pb = sm.rowb[y], wb = sm.rowb2[y], ob = sm.rowb3[y];
            if (pb < 0 || (ua.prune && ob == kNoRow)) continue;
            float pv[VX][2], wv[VX][2];
#pragma unroll
            for (int v = 0; v < VX; ++v) {
                const int x = 2 * (t + 16 * v);
                const int2 mx = *reinterpret_cast<const int2 *>(sm.colx + x);
                const int2 gx = *reinterpret_cast<const int2 *>(sm.colx2 + x);
                pv[v][0] = mx.x >= 0 ? __ldg(psrc + pb + mx.x) : 0.0f;
                pv[v][1] = mx.y >= 0 ? __ldg(psrc + pb + mx.y) : 0.0f;
                wv[v][0] = (wb >= 0 && gx.x >= 0) ? __ldg(wgt + wb + gx.x) : 0.0f;
                wv[v][1] = (wb >= 0 && gx.y >= 0) ? __ldg(wgt + wb + gx.y) : 0.0f;
            }
            float2 a[VX];
            const float2 *row = sm.A + y * SH::SR + t;
#pragma unroll
            for (int v = 0; v < VX; ++v) a[v] = row[16 * v];
            xrow_p1<VX, true>(a, sm.twx, t);
#pragma unroll
            for (int v = 0; v < VX; ++v) {
                const float cv[2] = {a[v].x, a[v].y};
                const int2 cx = *reinterpret_cast<const int2 *>(sm.colx + 2 * (t + 16 * v));
                const int2 c3 = *reinterpret_cast<const int2 *>(sm.colx3 + 2 * (t + 16 * v));
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int x = 2 * (t + 16 * v) + h;
                    if ((h ? cx.y : cx.x) < 0) continue;
                    const float last = pv[v][h];
                    const float next = next_value_fast(last, cv[h], wv[v][h], uc);
                    const float ch = next - last;  // signed change (DeconvolutionMethods.java:308)
                    const float ky = ch - kcomp;
                    const float kt = ksum + ky;
                    kcomp = (kt - ksum) - ky;
                    ksum = kt;
                    kmax = kmax > ch ? kmax : ch;
                    if (ob != kNoRow && (h ? c3.y : c3.x) >= 0) pdst[ob + x] = next;
                }
            }
        }
    } else {
        pdl_wait();
        pair_load<VX, VH>(sm.A, Sp);
        __syncthreads();
        pair_y_inverse<VX, VH>(sm.A, sm.twy, rank);
        pair_x_p2<VX, VH, true>(sm.A, sm.twx);
        tp_phase1<VX, H, SH::SR, 1, true, NT>(sm.A, sm.twx, 2);
        __syncthreads();
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = NT >> 5;
        const int ylo = ua.prune ? bm.wlo[1] : 0, yhi = ua.prune ? bm.whi[1] : bm.b[1];
        if (z < bm.b[2])
            for (int yl = warp; yl < H; yl += nw) {
                const int y = y0 + yl;
                if (y >= ylo && y < yhi)
                    update_row<float, EPI>(sm.A + yl * SH::SR, SH::m, bm, ua, y, z, lane, ksum, kcomp, kmax);
            }
    }
    // pruned runs skip the statistics, but the likelihood is reduced over the write region
    if ((EPI == EPI_SEQ || EPI == EPI_MUL_FINAL || EPI == EPI_NLL) && (!ua.prune || EPI == EPI_NLL))
        stats_to_partials(ksum, kcomp, kmax, red_s, red_m, ua.partials, (long long)blockIdx.y * gridDim.x + blockIdx.x);
}

}  // namespace mvr
