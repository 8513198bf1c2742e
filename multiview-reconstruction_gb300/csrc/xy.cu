// Launchers of the plane kernels (see xy_plane.cuh).
#include "xy.cuh"
#include "xy_pair.cuh"
#include "xy_plane.cuh"

#include <algorithm>
#include <cstdlib>
#include <mutex>

namespace mvr {

// Shapes with compiled plane kernels: Px in {128, 192}, Py in {128, 192}.
#define XY_DISPATCH(combo, ...)                    \
    switch (combo) {                               \
    case 408: {                                    \
        constexpr int VX_ = 4, VY_ = 8;            \
        __VA_ARGS__;                               \
    } break;                                       \
    case 412: {                                    \
        constexpr int VX_ = 4, VY_ = 12;           \
        __VA_ARGS__;                               \
    } break;                                       \
    case 608: {                                    \
        constexpr int VX_ = 6, VY_ = 8;            \
        __VA_ARGS__;                               \
    } break;                                       \
    case 612: {                                    \
        constexpr int VX_ = 6, VY_ = 12;           \
        __VA_ARGS__;                               \
    } break;                                       \
    default: return cudaErrorInvalidValue;         \
    }

// Shapes with compiled pair kernels (two CTAs per plane): Px = Py = 192 or 256.  A pair
// shape code is 10000 + 100 VX + VH with Px = 32 VX, Py = 32 VH.
#define PAIR_DISPATCH(combo, ...)                  \
    switch (combo) {                               \
    case 10606: {                                  \
        constexpr int VX_ = 6, VH_ = 6;            \
        __VA_ARGS__;                               \
    } break;                                       \
    case 10808: {                                  \
        constexpr int VX_ = 8, VH_ = 8;            \
        __VA_ARGS__;                               \
    } break;                                       \
    default: return cudaErrorInvalidValue;         \
    }

int xy_pair_combo(const int P[3])
{
    if (P[0] % 32 || P[1] % 32) return 0;
    const int c = 10000 + (P[0] / 32) * 100 + P[1] / 32;
    return (c == 10606 || c == 10808) ? c : 0;
}

int xy_partial_slots(int combo, int planes) { return combo >= 10000 ? 2 * planes : planes; }

int xy_combo(const int P[3])
{
    if (P[0] % 32 || P[1] % 16) return 0;
    const int c = (P[0] / 32) * 100 + P[1] / 16;
    return (c == 408 || c == 412 || c == 608 || c == 612) ? c : 0;
}

size_t xy_smem(int combo)
{
    switch (combo) {
    case 10606: return pair_smem_bytes<6, 6>();
    case 10808: return pair_smem_bytes<8, 8>();
    case 408: return xy_smem_bytes<4, 8>();
    case 412: return xy_smem_bytes<4, 12>();
    case 608: return xy_smem_bytes<6, 8>();
    case 612: return xy_smem_bytes<6, 12>();
    default: return 0;
    }
}

namespace {

template <int VX, int VY>
void set_limits_one()
{
    const int m = (int)xy_smem_bytes<VX, VY>();
    cudaFuncSetAttribute(k_xy_fwd<VX, VY, SrcMirror<float>>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_fwd<VX, VY, SrcZero<float>>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_fwd<VX, VY, SrcKernel>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_ratio<VX, VY>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_update<VX, VY, EPI_SEQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_update<VX, VY, EPI_SEQ, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_update<VX, VY, EPI_MUL_FIRST>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_update<VX, VY, EPI_MUL_ACC>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_update<VX, VY, EPI_MUL_FINAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_update<VX, VY, EPI_STORE>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy_update<VX, VY, EPI_NLL>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
}

// CTAs of the persistent plane kernels: one per SM (MVR_XY_PERSIST=0: one per plane).
int persist_ctas()
{
    static int n = 0;
    if (!n) {
        const char *e = std::getenv("MVR_XY_PERSIST");
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        n = (e && e[0] == '0') ? (1 << 30) : std::max(1, sms);
    }
    return n;
}

template <int VX, int VH>
void set_limits_pair()
{
    const int m = (int)pair_smem_bytes<VX, VH>();
    cudaFuncSetAttribute(k_xy2_fwd<VX, VH, SrcMirror<float>>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_fwd<VX, VH, SrcZero<float>>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_fwd<VX, VH, SrcKernel>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_ratio<VX, VH>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_update<VX, VH, EPI_SEQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_update<VX, VH, EPI_MUL_FIRST>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_update<VX, VH, EPI_MUL_ACC>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_update<VX, VH, EPI_MUL_FINAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_update<VX, VH, EPI_STORE>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_xy2_update<VX, VH, EPI_NLL>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
}

// A launch of a cluster-pair kernel: clusters of two CTAs along x, with programmatic
// dependent launch as launch_pdl.
template <typename... KArgs, typename... Args>
cudaError_t launch_pair(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[2];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[1].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
    cfg.attrs = at;
    cfg.numAttrs = 2;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Clusters of the persistent pair kernels: as many as the SMs hold at once.
template <int VX, int VH>
int pair_clusters()
{
    static int n = 0;
    if (!n) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        n = std::max(1, sms * PairShape<VX, VH>::MINB / 2);
    }
    return n;
}

void set_limits()
{
    static std::once_flag once;
    std::call_once(once, [] {
        set_limits_pair<6, 6>();
        set_limits_pair<8, 8>();
        set_limits_one<4, 8>();
        set_limits_one<4, 12>();
        set_limits_one<6, 8>();
        set_limits_one<6, 12>();
    });
}

template <class Src>
cudaError_t fwd(int combo, const Src &src, float2 *S, const BlockMaps &bms, int nb, int Pz, long long Pc,
                const float2 *twx, const float2 *twy, cudaStream_t s, bool persist)
{
    set_limits();
    const int nitems = Pz * nb;
    if (combo >= 10000) {
        PAIR_DISPATCH(combo, return launch_pair(k_xy2_fwd<VX_, VH_, Src>,
                                                dim3(2 * (unsigned)std::min(nitems, pair_clusters<VX_, VH_>())),
                                                PairShape<VX_, VH_>::NT, pair_smem_bytes<VX_, VH_>(), s, src, S, bms,
                                                Pc, twx, twy, Pz, nitems));
        return cudaGetLastError();
    }
    const dim3 grid((unsigned)(persist ? std::min(nitems, persist_ctas()) : nitems));
    XY_DISPATCH(combo, return launch_pdl(k_xy_fwd<VX_, VY_, Src>, grid, XYShape<VX_, VY_>::NT,
                                         xy_smem_bytes<VX_, VY_>(), s, src, S, bms, Pc, twx, twy, Pz, nitems));
    return cudaGetLastError();
}

}  // namespace

cudaError_t xy_fwd_mirror(int combo, const float *psi, float2 *S, const BlockMaps &bms, int nb, int Pz, long long Pc,
                          const float2 *twx, const float2 *twy, cudaStream_t s, bool persist)
{
    return fwd(combo, SrcMirror<float>{psi}, S, bms, nb, Pz, Pc, twx, twy, s, persist);
}

cudaError_t xy_fwd_zero(int combo, const float *blk, float2 *S, const BlockMaps &bms, int nb, int Pz, long long Pc,
                        const float2 *twx, const float2 *twy, cudaStream_t s, bool persist)
{
    return fwd(combo, SrcZero<float>{blk}, S, bms, nb, Pz, Pc, twx, twy, s, persist);
}

cudaError_t xy_fwd_kernel(int combo, const SrcKernel &src, float2 *S, const BlockMaps &bms, int nb, int Pz,
                          long long Pc, const float2 *twx, const float2 *twy, cudaStream_t s, bool persist)
{
    return fwd(combo, src, S, bms, nb, Pz, Pc, twx, twy, s, persist);
}

cudaError_t xy_ratio(int combo, float2 *S, const float *img, const BlockMaps &bms, int nb, int z0, int nzb,
                     long long Pc, const float2 *twx, const float2 *twy, cudaStream_t s, bool persist)
{
    set_limits();
    const int nitems = nzb * nb;
    if (combo >= 10000) {
        PAIR_DISPATCH(combo, return launch_pair(k_xy2_ratio<VX_, VH_>,
                                                dim3(2 * (unsigned)std::min(nitems, pair_clusters<VX_, VH_>())),
                                                PairShape<VX_, VH_>::NT, pair_smem_bytes<VX_, VH_>(), s, S, img, bms,
                                                Pc, twx, twy, z0, nzb, nitems));
        return cudaGetLastError();
    }
    const dim3 grid((unsigned)(persist ? std::min(nitems, persist_ctas()) : nitems));
    XY_DISPATCH(combo, return launch_pdl(k_xy_ratio<VX_, VY_>, grid, XYShape<VX_, VY_>::NT, xy_smem_bytes<VX_, VY_>(),
                                         s, S, img, bms, Pc, twx, twy, z0, nzb, nitems));
    return cudaGetLastError();
}

cudaError_t xy_update(int combo, int epi, float2 *S, const UpdateArgs &ua, const BlockMaps &bms, int nb, int Pz,
                      long long Pc, const float2 *twx, const float2 *twy, cudaStream_t s)
{
    set_limits();
    int planes = Pz;
    if (ua.prune) {
        if (epi == EPI_STORE) return cudaErrorInvalidValue;
        planes = 0;
        for (int i = 0; i < nb; ++i) planes = std::max(planes, bms.m[i].whi[2] - bms.m[i].wlo[2]);
        if (planes < 1) return cudaSuccess;
    }
    if (combo >= 10000) {
        const dim3 pgrid(2 * (unsigned)planes, (unsigned)nb);
#define XY2_UPD(E)                                                                                             \
    PAIR_DISPATCH(combo, return launch_pair(k_xy2_update<VX_, VH_, E>, pgrid, PairShape<VX_, VH_>::NT,            \
                                            pair_smem_bytes<VX_, VH_>(), s, S, ua, bms, Pc, twx, twy))
        switch (epi) {
        case EPI_SEQ: XY2_UPD(EPI_SEQ); break;
        case EPI_MUL_FIRST: XY2_UPD(EPI_MUL_FIRST); break;
        case EPI_MUL_ACC: XY2_UPD(EPI_MUL_ACC); break;
        case EPI_MUL_FINAL: XY2_UPD(EPI_MUL_FINAL); break;
        case EPI_NLL: XY2_UPD(EPI_NLL); break;
        case EPI_STORE: XY2_UPD(EPI_STORE); break;
        default: return cudaErrorInvalidValue;
        }
#undef XY2_UPD
        return cudaGetLastError();
    }
    const dim3 grid((unsigned)planes, (unsigned)nb);
#define XY_UPD(...)                                                                                         \
    XY_DISPATCH(combo, return launch_pdl(k_xy_update<VX_, VY_, __VA_ARGS__>, grid, XYShape<VX_, VY_>::NT,    \
                                         xy_smem_bytes<VX_, VY_>(), s, S, ua, bms, Pc, twx, twy))
    switch (epi) {
    case EPI_SEQ:
        if (ua.prune) {
            XY_UPD(EPI_SEQ, true);  // the write regions alone
        } else {
            XY_UPD(EPI_SEQ);
        }
        break;
    case EPI_MUL_FIRST: XY_UPD(EPI_MUL_FIRST); break;
    case EPI_MUL_ACC: XY_UPD(EPI_MUL_ACC); break;
    case EPI_MUL_FINAL: XY_UPD(EPI_MUL_FINAL); break;
    case EPI_NLL: XY_UPD(EPI_NLL); break;
    case EPI_STORE: XY_UPD(EPI_STORE); break;
    default: return cudaErrorInvalidValue;
    }
#undef XY_UPD
    return cudaGetLastError();
}

}  // namespace mvr
