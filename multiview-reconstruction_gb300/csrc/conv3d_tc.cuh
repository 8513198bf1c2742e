// 3x3x3 convolution (stride 1, zero padding 1) on channels-last BF16 volumes as
// implicit GEMMs on the tcgen05 tensor cores, FP32 accumulation in tensor memory.
//
//   forward  Y[n][co] = act( sum_{t,ci} X[n + off(t)][ci] W[co][t][ci] + b[co] )
//            M = 128 voxels per CTA, N = C_out, K = 27 C_in, one tap per stage
//   dgrad    dX[n][ci] = sum_{t,co} G[n - off(t)][co] W[co][t][ci]
//            the same kernel with the offsets negated and WT[ci][t][co] as B
//   wgrad    dW[co][t][ci] += sum_n G[n][co] X[n + off(t)][ci]
//            M = 128 (t, ci) rows per CTA, N = C_out, K = voxels (split over CTAs,
//            FP32 atomics into dW)
//
// Volumes are [B][D][H][W][C] (x fastest, then y, z, batch), C a multiple of 16.
// Stages are double buffered: the gather of tap t+1 overlaps the MMAs of tap t; a
// buffer is refilled only after the mbarrier of its previous MMAs completed.  Every
// wait is bounded and reports a timeout through err instead of hanging.
#pragma once
#include "tcgen05.cuh"

namespace mvr {

struct ConvGeom {
    int B, D, H, W;
    long long nvox;  // B * D * H * W
};

constexpr long long kTcWaitIter = 1LL << 24;

__device__ __forceinline__ void vox_coords(const ConvGeom &g, long long n, int &x, int &y, int &z, int &b)
{
    x = (int)(n % g.W);
    long long t = n / g.W;
    y = (int)(t % g.H);
    t /= g.H;
    z = (int)(t % g.D);
    b = (int)(t / g.D);
}

// Index of the neighbour of (x,y,z,b) at tap t (offsets in {-1,0,1}, times sign), or
// -1 outside the volume.
__device__ __forceinline__ long long neighbour(const ConvGeom &g, int x, int y, int z, int b, int t, int sign)
{
    const int dz = (t / 9 - 1) * sign, dy = ((t / 3) % 3 - 1) * sign, dx = (t % 3 - 1) * sign;
    const int xx = x + dx, yy = y + dy, zz = z + dz;
    if (xx < 0 || yy < 0 || zz < 0 || xx >= g.W || yy >= g.H || zz >= g.D) return -1;
    return (((long long)b * g.D + zz) * g.H + yy) * g.W + xx;
}

// 16-byte asynchronous copy global -> shared (L2 only); ok == false writes 16 zero bytes
// (source size 0, the source address not read)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool ok)
{
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(ok ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

template <int N>
struct TmemCols {
    static constexpr uint32_t value = N <= 32 ? 32 : (N <= 64 ? 64 : (N <= 128 ? 128 : 256));
};

// OUT_MODE 0: BF16 output with bias (+ReLU when relu != 0); 1: FP32 output, no bias.
template <int N, int C, int OUT_MODE>
__global__ void __launch_bounds__(128) k_conv3d_tc(const __nv_bfloat16 *__restrict__ act,
                                                   const __nv_bfloat16 *__restrict__ wk, const float *__restrict__ bias,
                                                   void *out, ConvGeom g, int sign, int relu, int *err)
{
    static_assert(N % 16 == 0 && N <= 256 && C % 16 == 0 && C <= 128, "tile shape");
    constexpr int A_BYTES = 128 * C * 2, B_BYTES = N * C * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA[2] = {smem, smem + A_BYTES};
    uint8_t *sB[2] = {smem + 2 * A_BYTES, smem + 2 * A_BYTES + B_BYTES};
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t ncols = TmemCols<N>::value;
    if (warp == 0) tc::tmem_alloc(&tbase, ncols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    const long long n = (long long)blockIdx.x * 128 + tid;  // this thread's row (voxel)
    int x = 0, y = 0, z = 0, b = 0;
    const bool rv = n < g.nvox;
    if (rv) vox_coords(g, n, x, y, z, b);
    const uint32_t idesc = tc::idesc_bf16(128, N);
    bool ok = true;
    uint32_t uses[2] = {0, 0};
    for (int t = 0; t < 27; ++t) {
        const int buf = t & 1;
        if (t >= 2) {  // the MMAs that last read this buffer must be done; on a timeout
                       // every thread stops before it writes the buffer again
            if (!__syncthreads_and(tc::mbar_wait(&mbar[buf], (uses[buf] - 1) & 1, kTcWaitIter))) {
                ok = false;
                break;
            }
        }
        // A: this thread's row, C channels of the neighbour at tap t
        const long long src = rv ? neighbour(g, x, y, z, b, t, sign) : -1;
        const uint4 *ap = reinterpret_cast<const uint4 *>(act + (src < 0 ? 0 : src * C));
#pragma unroll
        for (int j = 0; j < C / 8; ++j) {
            const uint4 v = src < 0 ? make_uint4(0, 0, 0, 0) : __ldg(ap + j);
            *reinterpret_cast<uint4 *>(sA[buf] + tc::core_offset(tid, 8 * j, C)) = v;
        }
        // B: N rows of K = (t, 0..C-1)
        for (int s = tid; s < N * (C / 8); s += 128) {
            const int r = s / (C / 8), j = s % (C / 8);
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(wk + ((long long)r * 27 + t) * C) + j);
            *reinterpret_cast<uint4 *>(sB[buf] + tc::core_offset(r, 8 * j, C)) = v;
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0 && ok) {
            tc::fence_after_sync();
#pragma unroll
            for (int c = 0; c < C / 16; ++c) {
                const uint64_t ad = tc::smem_desc(tc::smem_u32(sA[buf]) + c * 256, 128, C * 16);
                const uint64_t bd = tc::smem_desc(tc::smem_u32(sB[buf]) + c * 256, 128, C * 16);
                tc::mma_bf16(tmem, ad, bd, idesc, (t > 0 || c > 0) ? 1 : 0);
            }
            tc::mma_commit(&mbar[buf]);
        }
        ++uses[buf];
    }
    // drain: both buffers' last commits
    for (int bb = 0; bb < 2; ++bb)
        if (uses[bb]) ok = tc::mbar_wait(&mbar[bb], (uses[bb] - 1) & 1, kTcWaitIter) && ok;
    tc::fence_after_sync();
    ok = __syncthreads_and(ok) != 0;  // one outcome for the whole CTA (the TMEM loads are warp-wide)
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
    } else {
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
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
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// The same convolution on output bricks of 8 x 4 x 4 voxels (x, y, z): the brick's
// input halo (10 x 6 x 6 voxels, zero outside the volume) is loaded into shared memory
// once, and the A operand of every tap is copied from it (shared to shared) instead of
// being gathered 27 times from L1/L2.  Row r of the 128-row tile is voxel
// (r % 8, (r / 8) % 4, r / 32) of the brick.  Shared memory: halo, two A stages, two B
// stages.
constexpr int kBrickX = 8, kBrickY = 4, kBrickZ = 4;
constexpr int kHaloX = kBrickX + 2, kHaloY = kBrickY + 2, kHaloZ = kBrickZ + 2;
constexpr int kHaloVox = kHaloX * kHaloY * kHaloZ;

template <int N, int C>
constexpr size_t conv_brick_smem()
{
    return (size_t)kHaloVox * C * 2 + 2 * (128 * C * 2 + N * C * 2);
}

// CU > 0: the input is the concatenation [nearest x2 upsampling of `act` (CU channels,
// a volume of half the size), act2 (C - CU channels)] read straight into the halo, so the
// decoder layers need no concatenated copy.
template <int N, int C, int OUT_MODE, int CU = 0>
__global__ void __launch_bounds__(128) k_conv3d_brick(const __nv_bfloat16 *__restrict__ act,
                                                      const __nv_bfloat16 *__restrict__ wk,
                                                      const float *__restrict__ bias, void *out, ConvGeom g, int sign,
                                                      int relu, int *err, const __nv_bfloat16 *__restrict__ act2 = nullptr)
{
    static_assert(CU % 8 == 0 && CU < C, "concatenated channel split");
    static_assert(N % 16 == 0 && N <= 256 && C % 16 == 0 && C <= 128, "tile shape");
    constexpr int A_BYTES = 128 * C * 2, B_BYTES = N * C * 2, H_BYTES = kHaloVox * C * 2;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA[2] = {smem, smem + A_BYTES};
    uint8_t *sB[2] = {smem + 2 * A_BYTES, smem + 2 * A_BYTES + B_BYTES};
    uint8_t *halo = smem + 2 * A_BYTES + 2 * B_BYTES;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t ncols = TmemCols<N>::value;
    if (warp == 0) tc::tmem_alloc(&tbase, ncols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // brick coordinates
    const int nbx = (g.W + kBrickX - 1) / kBrickX, nby = (g.H + kBrickY - 1) / kBrickY,
              nbz = (g.D + kBrickZ - 1) / kBrickZ;
    long long q = blockIdx.x;
    const int ibx = (int)(q % nbx);
    q /= nbx;
    const int iby = (int)(q % nby);
    q /= nby;
    const int ibz = (int)(q % nbz);
    const int b = (int)(q / nbz);
    const int x0 = ibx * kBrickX, y0 = iby * kBrickY, z0 = ibz * kBrickZ;
    // halo: C / 8 chunks of 16 bytes per voxel, zero outside the volume
    constexpr int CH = C / 8;
    for (int k = tid; k < kHaloVox * CH; k += 128) {
        const int hv = k / CH, j = k - hv * CH;
        const int hx = hv % kHaloX, hy = (hv / kHaloX) % kHaloY, hz = hv / (kHaloX * kHaloY);
        const int xx = x0 - 1 + hx, yy = y0 - 1 + hy, zz = z0 - 1 + hz;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (xx >= 0 && yy >= 0 && zz >= 0 && xx < g.W && yy < g.H && zz < g.D) {
            if constexpr (CU == 0) {
                v = __ldg(reinterpret_cast<const uint4 *>(act + ((((long long)b * g.D + zz) * g.H + yy) * g.W + xx) * C) + j);
            } else if (j < CU / 8) {
                const long long lv = (((long long)b * (g.D / 2) + zz / 2) * (g.H / 2) + yy / 2) * (g.W / 2) + xx / 2;
                v = __ldg(reinterpret_cast<const uint4 *>(act + lv * CU) + j);
            } else {
                const long long hv2 = (((long long)b * g.D + zz) * g.H + yy) * g.W + xx;
                v = __ldg(reinterpret_cast<const uint4 *>(act2 + hv2 * (C - CU)) + (j - CU / 8));
            }
        }
        *reinterpret_cast<uint4 *>(halo + (size_t)hv * C * 2 + 16 * j) = v;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    const int lx = tid & 7, ly = (tid >> 3) & 3, lz = tid >> 5;
    const int x = x0 + lx, y = y0 + ly, z = z0 + lz;
    const bool rv = x < g.W && y < g.H && z < g.D;
    const long long n = rv ? (((long long)b * g.D + z) * g.H + y) * g.W + x : 0;
    const uint32_t idesc = tc::idesc_bf16(128, N);
    bool ok = true;
    uint32_t uses[2] = {0, 0};
    for (int t = 0; t < 27; ++t) {
        const int buf = t & 1;
        if (t >= 2) {  // the MMAs that last read this buffer must be done; on a timeout
                       // every thread stops before it writes the buffer again
            if (!__syncthreads_and(tc::mbar_wait(&mbar[buf], (uses[buf] - 1) & 1, kTcWaitIter))) {
                ok = false;
                break;
            }
        }
        // A: this thread's row from the halo at tap t
        const int dz = (t / 9 - 1) * sign, dy = ((t / 3) % 3 - 1) * sign, dx = (t % 3 - 1) * sign;
        const int hv = ((lz + 1 + dz) * kHaloY + (ly + 1 + dy)) * kHaloX + (lx + 1 + dx);
        const uint4 *hp = reinterpret_cast<const uint4 *>(halo + (size_t)hv * C * 2);
#pragma unroll
        for (int j = 0; j < CH; ++j)
            *reinterpret_cast<uint4 *>(sA[buf] + tc::core_offset(tid, 8 * j, C)) = hp[j];
        // B: N rows of K = (t, 0..C-1)
        for (int s = tid; s < N * CH; s += 128) {
            const int r = s / CH, j = s % CH;
            const uint4 v = __ldg(reinterpret_cast<const uint4 *>(wk + ((long long)r * 27 + t) * C) + j);
            *reinterpret_cast<uint4 *>(sB[buf] + tc::core_offset(r, 8 * j, C)) = v;
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0 && ok) {
            tc::fence_after_sync();
#pragma unroll
            for (int c = 0; c < C / 16; ++c) {
                const uint64_t ad = tc::smem_desc(tc::smem_u32(sA[buf]) + c * 256, 128, C * 16);
                const uint64_t bd = tc::smem_desc(tc::smem_u32(sB[buf]) + c * 256, 128, C * 16);
                tc::mma_bf16(tmem, ad, bd, idesc, (t > 0 || c > 0) ? 1 : 0);
            }
            tc::mma_commit(&mbar[buf]);
        }
        ++uses[buf];
    }
    for (int bb = 0; bb < 2; ++bb)
        if (uses[bb]) ok = tc::mbar_wait(&mbar[bb], (uses[bb] - 1) & 1, kTcWaitIter) && ok;
    tc::fence_after_sync();
    ok = __syncthreads_and(ok) != 0;  // one outcome for the whole CTA (the TMEM loads are warp-wide)
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
    } else {
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
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
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// The same convolution with no per-tap copies at all: the output tile is a brick of 8 x 16 x 1
// voxels (x, y, z), row r = x + 8 y, and the input halo (10 x 18 x 3 voxels) is stored in
// shared memory "K-group major": the 16-byte chunk of channels 8j..8j+7 of halo voxel
// h = hx + 10 hy + 180 hz at byte j * LBO + 16 h.  Eight x-consecutive halo voxels then form
// one canonical core matrix (8 rows x 16 bytes), the next y line of the brick is 10 rows
// (160 bytes) further, and the A operand of tap (dx, dy, dz) is the same layout started
// 16 ((1 + dx) + 10 (1 + dy) + 180 (1 + dz)) bytes later: one shared-memory descriptor per
// tap over the halo loaded once.  B (all taps of the weights, canonical K-major per tap) is
// staged in chunks of G taps through two buffers.
constexpr int kShX = 8, kShY = 16;                     // brick
constexpr int kShHX = kShX + 2, kShHY = kShY + 2, kShHZ = 3;
constexpr int kShRows = kShHX * kShHY * kShHZ;         // 540 halo voxels
constexpr int kShLbo = (kShRows + 1) * 16;             // K-group stride (one padding row: distinct banks)

template <int N, int C>
__host__ __device__ constexpr size_t shift_halo_bytes()
{
    return ((size_t)C / 8 * kShLbo + 1023) / 1024 * 1024;  // B starts 1 KB aligned
}

// taps of B per staged chunk: all 27 in one buffer when they fit next to the halo in
// 220 KB, else chunks of 9, else of 3, through two buffers
template <int N, int C>
__host__ __device__ constexpr int shift_taps_per_chunk()
{
    return (shift_halo_bytes<N, C>() + 27 * (size_t)N * C * 2 <= 220 * 1024)      ? 27
           : (shift_halo_bytes<N, C>() + 2 * 9 * (size_t)N * C * 2 <= 220 * 1024) ? 9
                                                                                   : 3;
}

template <int N, int C>
__host__ __device__ constexpr size_t conv_shift_smem()
{
    constexpr int G = shift_taps_per_chunk<N, C>();
    return shift_halo_bytes<N, C>() + (G == 27 ? 1 : 2) * (size_t)G * N * C * 2;
}

template <int N, int C, int OUT_MODE, int CU = 0>
__global__ void __launch_bounds__(128) k_conv3d_shift(const __nv_bfloat16 *__restrict__ act,
                                                      const __nv_bfloat16 *__restrict__ wk,
                                                      const float *__restrict__ bias, void *out, ConvGeom g, int sign,
                                                      int relu, int *err, const __nv_bfloat16 *__restrict__ act2 = nullptr)
{
    static_assert(N % 16 == 0 && N <= 256 && C % 16 == 0 && C <= 128, "tile shape");
    static_assert(CU % 8 == 0 && CU < C, "concatenated channel split");
    constexpr int G = shift_taps_per_chunk<N, C>(), NCH = 27 / G;
    constexpr int B_TAP = N * C * 2, B_BYTES = G * B_TAP;
    constexpr size_t H_BYTES = shift_halo_bytes<N, C>();
    constexpr int CH = C / 8;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *halo = smem;
    uint8_t *sB[2] = {smem + H_BYTES, smem + H_BYTES + (NCH > 1 ? B_BYTES : 0)};
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t ncols = TmemCols<N>::value;
    if (warp == 0) tc::tmem_alloc(&tbase, ncols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    const int nbx = (g.W + kShX - 1) / kShX, nby = (g.H + kShY - 1) / kShY;
    long long q = blockIdx.x;
    const int ibx = (int)(q % nbx);
    q /= nbx;
    const int iby = (int)(q % nby);
    q /= nby;
    const int z0 = (int)(q % g.D);
    const int b = (int)(q / g.D);
    const int x0 = ibx * kShX, y0 = iby * kShY;
    // halo, channel chunk fastest (coalesced reads), zero outside the volume; every copy is
    // asynchronous, so a thread's copies are all in flight together
    for (int k = tid; k < kShRows * CH; k += 128) {
        const int h = k / CH, j = k - h * CH;
        const int hx = h % kShHX, hy = (h / kShHX) % kShHY, hz = h / (kShHX * kShHY);
        const int xx = x0 - 1 + hx, yy = y0 - 1 + hy, zz = z0 - 1 + hz;
        const bool in = xx >= 0 && yy >= 0 && zz >= 0 && xx < g.W && yy < g.H && zz < g.D;
        const uint4 *src = reinterpret_cast<const uint4 *>(act);
        if (in) {
            if constexpr (CU == 0) {
                src = reinterpret_cast<const uint4 *>(act + ((((long long)b * g.D + zz) * g.H + yy) * g.W + xx) * C) + j;
            } else if (j < CU / 8) {
                const long long lv = (((long long)b * (g.D / 2) + zz / 2) * (g.H / 2) + yy / 2) * (g.W / 2) + xx / 2;
                src = reinterpret_cast<const uint4 *>(act + lv * CU) + j;
            } else {
                const long long hv2 = (((long long)b * g.D + zz) * g.H + yy) * g.W + xx;
                src = reinterpret_cast<const uint4 *>(act2 + hv2 * (C - CU)) + (j - CU / 8);
            }
        }
        cp_async16(halo + (size_t)j * kShLbo + 16 * h, src, in);
    }
    // B chunk c (taps G c .. G c + G - 1) into buffer `buf`, canonical K-major per tap
    auto load_b = [&](int c, int buf) {
        for (int s = tid; s < G * N * CH; s += 128) {
            const int tt = s / (N * CH), rem = s - tt * (N * CH), r = rem / CH, j = rem - r * CH;
            cp_async16(sB[buf] + tt * B_TAP + tc::core_offset(r, 8 * j, C),
                       reinterpret_cast<const uint4 *>(wk + ((long long)r * 27 + G * c + tt) * C) + j, true);
        }
        cp_async_wait_all();
    };
    load_b(0, 0);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    const uint32_t idesc = tc::idesc_bf16(128, N);
    const uint32_t hbase = tc::smem_u32(halo);
    bool ok = true;
    uint32_t uses[2] = {0, 0};
    for (int c = 0; c < NCH; ++c) {
        const int buf = c & 1;
        if (tid == 0 && ok) {
            tc::fence_after_sync();
            for (int tt = 0; tt < G; ++tt) {
                const int t = G * c + tt;
                const int dz = (t / 9 - 1) * sign, dy = ((t / 3) % 3 - 1) * sign, dx = (t % 3 - 1) * sign;
                const uint32_t a0 = hbase + 16u * (uint32_t)((1 + dx) + kShHX * (1 + dy) + kShHX * kShHY * (1 + dz));
                const uint32_t b0 = tc::smem_u32(sB[buf] + tt * B_TAP);
#pragma unroll
                for (int k = 0; k < C / 16; ++k) {
                    const uint64_t ad = tc::smem_desc(a0 + (uint32_t)(2 * k) * kShLbo, kShLbo, kShHX * 16);
                    const uint64_t bd = tc::smem_desc(b0 + k * 256, 128, C * 16);
                    tc::mma_bf16(tmem, ad, bd, idesc, (t > 0 || k > 0) ? 1 : 0);
                }
            }
            tc::mma_commit(&mbar[buf]);
        }
        ++uses[buf];
        if (c + 1 < NCH) {
            const int nb = (c + 1) & 1;
            if (c + 1 >= 2 && !__syncthreads_and(tc::mbar_wait(&mbar[nb], (uses[nb] - 1) & 1, kTcWaitIter))) {
                ok = false;  // every thread stops before it writes the buffer again
                break;
            }
            load_b(c + 1, nb);
            tc::fence_proxy_async();
            tc::fence_before_sync();
            __syncthreads();
            tc::fence_after_sync();
        }
    }
    for (int bb = 0; bb < 2; ++bb)
        if (uses[bb]) ok = tc::mbar_wait(&mbar[bb], (uses[bb] - 1) & 1, kTcWaitIter) && ok;
    tc::fence_after_sync();
    ok = __syncthreads_and(ok) != 0;  // one outcome for the whole CTA (the TMEM loads are warp-wide)
    const int lx = tid & 7, ly = tid >> 3;
    const int x = x0 + lx, y = y0 + ly;
    const bool rv = x < g.W && y < g.H;
    const long long n = rv ? (((long long)b * g.D + z0) * g.H + y) * g.W + x : 0;
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
    } else {
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
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
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

// wgrad: D[(t,ci) rows][co] over the voxels [blockIdx.y * vpc, +vpc), atomically added
// to dW[co][t][ci] (FP32).
template <int N, int C>
__global__ void __launch_bounds__(128) k_wgrad_tc(const __nv_bfloat16 *__restrict__ X,
                                                  const __nv_bfloat16 *__restrict__ G, float *dW, ConvGeom g,
                                                  long long vpc, int *err)
{
    constexpr int KT = 64;  // voxels per stage
    constexpr int A_BYTES = 128 * KT * 2, B_BYTES = N * KT * 2;
    constexpr int ROWS = 27 * C;
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA[2] = {smem, smem + A_BYTES};
    uint8_t *sB[2] = {smem + 2 * A_BYTES, smem + 2 * A_BYTES + B_BYTES};
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tbase;
    const int tid = threadIdx.x, warp = tid >> 5;
    constexpr uint32_t ncols = TmemCols<N>::value;
    if (warp == 0) tc::tmem_alloc(&tbase, ncols);
    if (tid == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tbase;
    const int row0 = blockIdx.x * 128;
    const long long n0 = (long long)blockIdx.y * vpc;
    const long long n1 = n0 + vpc < g.nvox ? n0 + vpc : g.nvox;
    const uint32_t idesc = tc::idesc_bf16(128, N);
    bool ok = true;
    uint32_t uses[2] = {0, 0};
    int stage = 0;
    for (long long k0 = n0; k0 < n1; k0 += KT, ++stage) {
        const int buf = stage & 1;
        if (stage >= 2 && !__syncthreads_and(tc::mbar_wait(&mbar[buf], (uses[buf] - 1) & 1, kTcWaitIter))) {
            ok = false;  // every thread stops before it writes the buffer again
            break;
        }
        // A: 16 row groups x KT voxels; a row group is 8 channels of one tap
        for (int s = tid; s < 16 * KT; s += 128) {
            const int rg = s / KT, k = s % KT;
            const int r = row0 + 8 * rg;
            const long long nn = k0 + k;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (r < ROWS && nn < n1) {
                const int t = r / C, ci = r % C;
                int x, y, z, b;
                vox_coords(g, nn, x, y, z, b);
                const long long src = neighbour(g, x, y, z, b, t, 1);
                if (src >= 0) v = __ldg(reinterpret_cast<const uint4 *>(X + src * C + ci));
            }
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                *reinterpret_cast<__nv_bfloat16 *>(sA[buf] + tc::core_offset(8 * rg + q, k, KT)) = e[q];
        }
        // B: N channels of G at KT voxels
        for (int s = tid; s < (N / 8) * KT; s += 128) {
            const int cg = s / KT, k = s % KT;
            const long long nn = k0 + k;
            uint4 v = make_uint4(0, 0, 0, 0);
            if (nn < n1) v = __ldg(reinterpret_cast<const uint4 *>(G + nn * N + 8 * cg));
            const __nv_bfloat16 *e = reinterpret_cast<const __nv_bfloat16 *>(&v);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                *reinterpret_cast<__nv_bfloat16 *>(sB[buf] + tc::core_offset(8 * cg + q, k, KT)) = e[q];
        }
        tc::fence_proxy_async();
        __syncthreads();
        if (tid == 0 && ok) {
            tc::fence_after_sync();
#pragma unroll
            for (int c = 0; c < KT / 16; ++c) {
                const uint64_t ad = tc::smem_desc(tc::smem_u32(sA[buf]) + c * 256, 128, KT * 16);
                const uint64_t bd = tc::smem_desc(tc::smem_u32(sB[buf]) + c * 256, 128, KT * 16);
                tc::mma_bf16(tmem, ad, bd, idesc, (stage > 0 || c > 0) ? 1 : 0);
            }
            tc::mma_commit(&mbar[buf]);
        }
        ++uses[buf];
    }
    for (int bb = 0; bb < 2; ++bb)
        if (uses[bb]) ok = tc::mbar_wait(&mbar[bb], (uses[bb] - 1) & 1, kTcWaitIter) && ok;
    tc::fence_after_sync();
    ok = __syncthreads_and(ok) != 0;  // one outcome for the whole CTA (the TMEM loads are warp-wide)
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
    } else if (stage > 0) {
        const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
        const int r = row0 + tid;  // (t, ci)
#pragma unroll
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc::tmem_ld16(trow + c0, v);
            if (r < ROWS)
#pragma unroll
                for (int j = 0; j < 16; ++j) atomicAdd(&dW[(long long)(c0 + j) * ROWS + r], v[j]);
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, ncols);
}

}  // namespace mvr
