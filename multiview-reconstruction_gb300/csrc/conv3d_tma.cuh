// Persistent TMA form of the shifted convolution (k_conv3d_shift, conv3d_tc.cuh): the same
// 8 x 16 x 1 output bricks, the same K-group-major halo (the 16-byte chunk of channels
// 8j..8j+7 of halo voxel h = hx + 10 hy + 180 hz at byte j * LBO + 16 h) and the same one
// descriptor per tap, but
//   - the halo of a brick arrives by tensor-memory-access copies: one 5-D tile per K group
//     (box 8 channels x 10 x 18 x 3 voxels of the [B][D][H][W][C] volume), which lands in
//     exactly that layout; coordinates outside the volume read as zeros;
//   - the CTA is persistent: the weights of all 27 taps stay in shared memory, two halo
//     buffers and two tensor-memory accumulators rotate, and while the epilogue of brick i
//     runs on all warps, the products of brick i + 1 run on the tensor core and the halo of
//     brick i + 2 streams in.
// Thread 0 issues the copies and the products; every wait is bounded, and a run-out stops
// all threads together and drains the copies and products in flight before the tensor
// memory is released.
#pragma once
#include <cuda.h>

#include "conv3d_tc.cuh"

namespace mvr {

constexpr int kTmaLbo = 544 * 16;  // K-group stride of a halo buffer (540 rows, 128-byte aligned)

__host__ __device__ constexpr size_t tma_round1k(size_t b) { return (b + 1023) / 1024 * 1024; }

template <int N, int C>
__host__ __device__ constexpr size_t conv_tma_smem()
{
    return 2 * tma_round1k((size_t)C / 8 * kTmaLbo) + 27 * (size_t)N * C * 2;
}

// shapes whose two halo buffers and 27 weight taps fit next to each other
template <int N, int C>
__host__ __device__ constexpr bool conv_tma_fits()
{
    return conv_tma_smem<N, C>() <= 200 * 1024 && C % 16 == 0 && N % 16 == 0 && 2 * N <= 256;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(mbar)), "r"(bytes)
                 : "memory");
}

// 5-D tile copy global -> shared, completion counted on mbar (bytes)
__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t *mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
        "%6}], [%7];" ::"r"(tc::smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(tc::smem_u32(mbar))
        : "memory");
}

template <int N, int C, int OUT_MODE>
__global__ void __launch_bounds__(128, 1) k_conv3d_tma(const __grid_constant__ CUtensorMap act_map,
                                                       const __nv_bfloat16 *__restrict__ wk,
                                                       const float *__restrict__ bias, void *out, ConvGeom g, int sign,
                                                       int relu, int *err)
{
    static_assert(conv_tma_fits<N, C>(), "tile shape");
    constexpr int CH = C / 8;
    constexpr size_t HB = tma_round1k((size_t)CH * kTmaLbo);
    constexpr int B_TAP = N * C * 2;
    constexpr uint32_t TX = CH * kShRows * 16;  // bytes of one brick's halo
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *halo[2] = {smem, smem + HB};
    uint8_t *sB = smem + 2 * HB;
    __shared__ __align__(8) uint64_t full[2], done[2];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t ncols = TmemCols<2 * N>::value;  // two accumulators of N columns
    if (warp == 0) tc::tmem_alloc(&tbase, ncols);
    if (tid == 0) {
        for (int s = 0; s < 2; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&done[s], 1);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const int nbx = (g.W + kShX - 1) / kShX, nby = (g.H + kShY - 1) / kShY;
    const long long nbricks = (long long)nbx * nby * g.D * g.B;
    const long long q0 = blockIdx.x;
    const int nmine = q0 < nbricks ? (int)((nbricks - 1 - q0) / gridDim.x + 1) : 0;
    auto place = [&](int i, int &x0, int &y0, int &z0, int &b) {
        long long q = q0 + (long long)i * gridDim.x;
        x0 = (int)(q % nbx) * kShX;
        q /= nbx;
        y0 = (int)(q % nby) * kShY;
        q /= nby;
        z0 = (int)(q % g.D);
        b = (int)(q / g.D);
    };
    // thread 0: the halo of brick i into buffer i & 1
    uint32_t issued_full[2] = {0, 0}, issued_done[2] = {0, 0};
    auto issue = [&](int i) {
        const int s = i & 1;
        int x0, y0, z0, b;
        place(i, x0, y0, z0, b);
        mbar_expect_tx(&full[s], TX);
#pragma unroll
        for (int j = 0; j < CH; ++j) tma_load_5d(halo[s] + j * kTmaLbo, &act_map, 8 * j, x0 - 1, y0 - 1, z0 - 1, b, &full[s]);
        ++issued_full[s];
    };
    if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (nmine > 0) issue(0);
        if (nmine > 1) issue(1);
    }
    // the weights of all taps, canonical K-major per tap, once
    for (int s = tid; s < 27 * N * CH; s += 128) {
        const int t = s / (N * CH), rem = s - t * (N * CH), r = rem / CH, j = rem - r * CH;
        cp_async16(sB + t * B_TAP + tc::core_offset(r, 8 * j, C),
                   reinterpret_cast<const uint4 *>(wk + ((long long)r * 27 + t) * C) + j, true);
    }
    cp_async_wait_all();
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    const uint32_t idesc = tc::idesc_bf16(128, N);
    const uint32_t bbase = tc::smem_u32(sB);
    // thread 0: the products of brick i into accumulator i & 1 (false: its halo never came)
    auto mma = [&](int i) -> bool {
        const int s = i & 1;
        if (!tc::mbar_wait(&full[s], (uint32_t)(i >> 1) & 1u, kTcWaitIter)) return false;
        tc::fence_after_sync();
        const uint32_t hb = tc::smem_u32(halo[s]);
        for (int t = 0; t < 27; ++t) {
            const int dz = (t / 9 - 1) * sign, dy = ((t / 3) % 3 - 1) * sign, dx = (t % 3 - 1) * sign;
            const uint32_t a0 = hb + 16u * (uint32_t)((1 + dx) + kShHX * (1 + dy) + kShHX * kShHY * (1 + dz));
            const uint32_t b0 = bbase + (uint32_t)(t * B_TAP);
#pragma unroll
            for (int k = 0; k < C / 16; ++k) {
                const uint64_t ad = tc::smem_desc(a0 + (uint32_t)(2 * k) * kTmaLbo, kTmaLbo, kShHX * 16);
                const uint64_t bd = tc::smem_desc(b0 + k * 256, 128, C * 16);
                tc::mma_bf16(tmem + (uint32_t)(s * N), ad, bd, idesc, (t > 0 || k > 0) ? 1 : 0);
            }
        }
        tc::mma_commit(&done[s]);
        ++issued_done[s];
        return true;
    };
    bool ok = true;
    if (tid == 0 && nmine > 0) ok = mma(0);
    const int lx = tid & 7, ly = tid >> 3;
    for (int i = 0; i < nmine; ++i) {
        const int s = i & 1;
        // brick i's products done: its halo buffer is free and its accumulator readable
        const bool w = ok && tc::mbar_wait(&done[s], (uint32_t)(i >> 1) & 1u, kTcWaitIter);
        if (!__syncthreads_and(w)) {
            ok = false;
            break;
        }
        tc::fence_after_sync();
        if (tid == 0) {
            if (i + 2 < nmine) issue(i + 2);
            if (i + 1 < nmine) ok = mma(i + 1);
        }
        __syncwarp();
        int x0, y0, z0, b;
        place(i, x0, y0, z0, b);
        const int x = x0 + lx, y = y0 + ly;
        const bool rv = x < g.W && y < g.H;
        const long long n = rv ? (((long long)b * g.D + z0) * g.H + y) * g.W + x : 0;
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(s * N);
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(trow + c0, v);
            if (!rv) continue;
            if (OUT_MODE == 0) {
                __align__(16) __nv_bfloat16 o[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    float a = v[j] + (bias ? bias[c0 + j] : 0.0f);
                    if (relu) a = fmaxf(a, 0.0f);
                    o[j] = __float2bfloat16(a);
                }
                uint4 *op = reinterpret_cast<uint4 *>(reinterpret_cast<__nv_bfloat16 *>(out) + n * N + c0);
                op[0] = reinterpret_cast<const uint4 *>(o)[0];
                op[1] = reinterpret_cast<const uint4 *>(o)[1];
            } else {
                float4 *op = reinterpret_cast<float4 *>(reinterpret_cast<float *>(out) + n * N + c0);
#pragma unroll
                for (int j = 0; j < 4; ++j) op[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
            }
        }
        // accumulator s is read before brick i + 2's products (issued after this barrier) write it
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    }
    if (!ok) {
        // a wait ran out: let every copy and product in flight finish (bounded) before the
        // tensor memory goes back
        if (tid == 0) {
            atomicExch(err, 1);
            for (int s = 0; s < 2; ++s) {
                if (issued_full[s]) tc::mbar_wait(&full[s], (issued_full[s] - 1) & 1u, kTcWaitIter);
                if (issued_done[s]) tc::mbar_wait(&done[s], (issued_done[s] - 1) & 1u, kTcWaitIter);
            }
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

}  // namespace mvr
