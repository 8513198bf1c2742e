// Launchers of the plane kernels (see xy_plane.cuh).
#include "xy.cuh"
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

int xy_combo(const int P[3])
{
    if (P[0] % 32 || P[1] % 16) return 0;
    const int c = (P[0] / 32) * 100 + P[1] / 16;
    return (c == 408 || c == 412 || c == 608 || c == 612) ? c : 0;
}

size_t xy_smem(int combo)
{
    switch (combo) {
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

void set_limits()
{
    static std::once_flag once;
    std::call_once(once, [] {
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

cudaError_t xy_ratio(int combo, float2 *S, const float *img, const BlockMaps &bms, int nb, int Pz, long long Pc,
                     const float2 *twx, const float2 *twy, cudaStream_t s, bool persist)
{
    set_limits();
    const int nitems = Pz * nb;
    const dim3 grid((unsigned)(persist ? std::min(nitems, persist_ctas()) : nitems));
    XY_DISPATCH(combo, return launch_pdl(k_xy_ratio<VX_, VY_>, grid, XYShape<VX_, VY_>::NT, xy_smem_bytes<VX_, VY_>(),
                                         s, S, img, bms, Pc, twx, twy, Pz, nitems));
    return cudaGetLastError();
}

cudaError_t xy_update(int combo, int epi, float2 *S, const UpdateArgs &ua, const BlockMaps &bms, int nb, int Pz,
                      long long Pc, const float2 *twx, const float2 *twy, cudaStream_t s)
{
    set_limits();
    int planes = Pz;
    if (ua.prune) {
        if (epi == EPI_NLL || epi == EPI_STORE) return cudaErrorInvalidValue;
        planes = 0;
        for (int i = 0; i < nb; ++i) planes = std::max(planes, bms.m[i].whi[2] - bms.m[i].wlo[2]);
        if (planes < 1) return cudaSuccess;
    }
    const dim3 grid((unsigned)planes, (unsigned)nb);
#define XY_UPD(E)                                                                                           \
    XY_DISPATCH(combo, return launch_pdl(k_xy_update<VX_, VY_, E>, grid, XYShape<VX_, VY_>::NT,              \
                                         xy_smem_bytes<VX_, VY_>(), s, S, ua, bms, Pc, twx, twy))
    switch (epi) {
    case EPI_SEQ: XY_UPD(EPI_SEQ); break;
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
