// Persistent, double-buffered form of the tile column pass (k_tcols, cols_tile.cuh).
//
// Each CTA walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ... of the whole batch.  While
// it transforms one tile in shared memory, the next tile (and, for the Z pass, the same
// tile of K^) streams into the second stage with cp.async, so the HBM reads of tile t + 1
// overlap the FFT work and the stores of tile t.  The transform itself is the two-phase
// register FFT of k_tcols, item for item.
//
// The spectra have an odd row length (Hx = P / 2 + 1 complex values), so a tile row starts
// on an 8-byte boundary only: the copies are 8-byte cp.async (one complex value), columns
// beyond the domain are zero-filled by a source size of 0.
#pragma once
#include "cols_tile.cuh"

namespace mvr {

__device__ __forceinline__ void cp_async8(void *smem, const void *gmem, bool ok)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(ok ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Tiles of one launch: per block of the batch, hmain x tiles at each of ny other-axis
// indices (olo + ty), then gtiles gathered tiles of the last column (x = Hx - 1).
struct PipeGeom {
    int hmain;      // x tiles
    int ny;         // other-axis indices
    int gtiles;     // gathered tiles per block (0 without gather)
    int per_block;  // hmain * ny + gtiles
    int ntiles;     // per_block * blocks
};

// Build-time tuning knobs: K^ staged in shared memory for the Z pass up to this V (else
// read from L2 in phase 2), and the CTAs per SM the register budget is sized for.  Measured
// on GB300: staging K^ (two CTAs of 100 KB per SM) and more CTAs per SM (80 or 64 registers)
// were both slower.
#ifndef MVR_PIPE_KS_MAXV
#define MVR_PIPE_KS_MAXV 0
#endif
#ifndef MVR_PIPE_MINB
#define MVR_PIPE_MINB 2
#endif

template <int V, int MODE>
__host__ __device__ constexpr bool pipe_kstage()
{
    return MODE == 2 && V <= MVR_PIPE_KS_MAXV;
}

template <int V, int MODE>
__host__ __device__ constexpr size_t pipe_smem()
{
    constexpr size_t n = (size_t)V * kTColT, tot = n * kTColNP;
    return sizeof(float2) * (n + 2 * tot * (pipe_kstage<V, MODE>() ? 2 : 1));
}

template <int V, int MODE>
__global__ void __launch_bounds__(256, MVR_PIPE_MINB)
    k_tcols_pipe(const float2 *src, float2 *dst, const float2 *__restrict__ Kh, int Hx, long long estride,
                 long long ostride, long long Pc, const float2 *__restrict__ twg, int gather, int nother, int rlo,
                 int rhi, int olo, PipeGeom pg, int llo, int lhi)
{
    constexpr int T = kTColT, NP = kTColNP, n = V * T, tot = n * NP;
    constexpr bool KS = pipe_kstage<V, MODE>();
    constexpr int SS = tot * (KS ? 2 : 1);  // float2 per stage
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw);
    float2 *stages = tw + n;
    pdl_trigger();
    for (int i = threadIdx.x; i < n; i += 256) tw[i] = __ldg(&twg[i]);
    pdl_wait();  // the spectra are the predecessor's output
    const int pc = threadIdx.x % NP;  // this thread's column in the copies and the stores
    const int prow = threadIdx.x / NP;
    // tile -> (block offset, base of column 0 at row 0, column stride, live columns)
    auto geom = [&](int tile, long long &boff, long long &base, long long &pstride, int &np) {
        const int b = tile / pg.per_block, r = tile - b * pg.per_block;
        boff = (long long)b * Pc;
        if (r < pg.hmain * pg.ny) {
            const int ty = r / pg.hmain, tx = r - ty * pg.hmain;
            const int x0 = tx * NP;
            base = (long long)(olo + ty) * ostride + x0;
            np = min(NP, (gather ? Hx - 1 : Hx) - x0);
            pstride = 1;
        } else {
            const int o0 = olo + (r - pg.hmain * pg.ny) * NP;
            base = (long long)o0 * ostride + (Hx - 1);
            np = min(NP, nother - o0);
            pstride = ostride;
        }
    };
    auto issue = [&](int tile, float2 *st) {
        long long boff, base, pstride;
        int np;
        geom(tile, boff, base, pstride, np);
        const bool live = pc < np;
        const long long c0 = base + (live ? (long long)pc * pstride : 0) + (long long)prow * estride;
        const long long rs = (long long)(256 / NP) * estride;
#pragma unroll
        for (int u = 0; u < tot / 256; ++u) {
            const long long o = c0 + u * rs;
            // rows outside [llo, lhi) are zero-filled (the caller's input is zero there)
            const int row = prow + (256 / NP) * u;
            cp_async8(st + threadIdx.x + 256 * u, src + boff + o, live && row >= llo && row < lhi);
            if (KS) cp_async8(st + tot + threadIdx.x + 256 * u, Kh + o, live);
        }
    };
    int it = 0;
    if ((int)blockIdx.x < pg.ntiles) issue(blockIdx.x, stages);
    cp_async_commit();
    for (int tile = blockIdx.x; tile < pg.ntiles; tile += gridDim.x, ++it) {
        float2 *A = stages + (it & 1) * SS;
        const int tn = tile + gridDim.x;
        if (tn < pg.ntiles) issue(tn, stages + ((it + 1) & 1) * SS);
        cp_async_commit();
        cp_async_wait1();  // every group but the one just issued: this tile is in A
        __syncthreads();
        const float2 *KA = A + tot;
        long long boff, base, pstride;
        int np;
        geom(tile, boff, base, pstride, np);
        const int c = threadIdx.x % NP;
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
        // phase 2: items (c, k1), k1 = threadIdx / NP, + 256 / NP, ... (more than one round for V > 16)
        for (int k1 = threadIdx.x / NP; k1 < V; k1 += 256 / NP) {
            if (live) {
                float2 b[T];
#pragma unroll
                for (int t = 0; t < T; ++t) b[t] = A[(t + T * k1) * NP + c];
                if (MODE != 1) sdft<T, false>(b);
                if (MODE == 2) {
                    if (KS) {
#pragma unroll
                        for (int k2 = 0; k2 < T; ++k2) b[k2] = cmul(b[k2], KA[(k2 + T * k1) * NP + c]);
                    } else {
                        const float2 *kp = Kh + base + (long long)c * pstride;
#pragma unroll
                        for (int k2 = 0; k2 < T; ++k2) b[k2] = cmul(b[k2], __ldg(kp + (long long)(k2 + T * k1) * estride));
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
        // rows [rlo, rhi) of the transformed axis go back to HBM
        if (pc < np) {
            float2 *cb = dst + boff + base + (long long)pc * pstride;
            for (int e = threadIdx.x + rlo * NP; e < rhi * NP; e += 256) cb[(long long)(e / NP) * estride] = A[e];
        }
        __syncthreads();  // the next iteration refills this stage
    }
    // no copy is left in flight: the last committed group was empty or waited for
}

}  // namespace mvr
