// Host side of the block iteration (see engine.cuh).
#include "engine.cuh"
#include "rows_warp.cuh"
#include "cols_warp.cuh"
#include "cols_tile.cuh"
#include "cols_pipe.cuh"
#include "xy.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

namespace mvr {

namespace {
constexpr int kThreads = 256;
constexpr int kRadices[] = {8, 4, 2, 3, 5, 7, 11, 13};
constexpr size_t kRowSmemTarget = 48 * 1024;
constexpr size_t kColSmemTarget = 72 * 1024;
constexpr size_t kSmemMax = 227 * 1024;
}  // namespace

const char *kernel_kind_name(int k)
{
    static const char *names[KK_COUNT] = {"rows_fwd_extract", "cols_y_fwd", "cols_y_inv", "cols_z_fwd_mul_inv",
                                          "rows_c2r_ratio_r2c", "rows_c2r_update", "reduce_stats", "paste",
                                          "xy_fwd_extract", "xy_c2r_ratio_r2c", "xy_c2r_update"};
    return (k >= 0 && k < KK_COUNT) ? names[k] : "?";
}

bool fft_friendly(long long n)
{
    if (n < 1) return false;
    for (int r : {2, 3, 5, 7, 11, 13})
        while (n % r == 0) n /= r;
    return n == 1;
}

long long next_friendly_even(long long n)
{
    long long m = std::max<long long>(2, n);
    if (m & 1) ++m;
    while (!fft_friendly(m)) m += 2;
    return m;
}

FftDesc make_desc(int n)
{
    FftDesc d{};
    d.n = n;
    d.ns = 0;
    int m = n;
    // powers of two first: Ns stays a power of two up to the first odd radix
    for (int r : kRadices)
        while (m % r == 0 && d.ns < kMaxStages) {
            d.radix[d.ns++] = r;
            m /= r;
        }
    int Ns = 1;
    for (int s = 0; s < d.ns; ++s) {
        const int R = d.radix[s];
        d.Ns[s] = Ns;
        d.twstep[s] = n / (Ns * R);
        d.ns_magic[s] = (unsigned)((0x100000000ULL + Ns - 1) / Ns);
        const unsigned nb = (unsigned)(n / R);
        d.nb_magic[s] = (unsigned)((0x100000000ULL + nb - 1) / nb);
        Ns *= R;
    }
    return d;
}

template <typename T>
int Engine<T>::fail(int code, const std::string &msg)
{
    err_ = msg;
    return code;
}

template <typename T>
int Engine<T>::cuda_check(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return OK;
    err_ = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? ERR_OOM : ERR_CUDA;
}

#define MVR_TRY(expr)                      \
    do {                                   \
        int rc__ = (expr);                 \
        if (rc__ != OK) return rc__;       \
    } while (0)
#define MVR_CUDA(expr) MVR_TRY(cuda_check((expr), #expr))
#define MVR_LAUNCHED(name) MVR_TRY(cuda_check(cudaGetLastError(), name))
// Launches the kernel expression with B = the plan's radix set (see fft_run).
#define MVR_WITH_BIG(big, ...)            \
    do {                                  \
        if (big) {                        \
            constexpr bool B = true;      \
            __VA_ARGS__;                  \
        } else {                          \
            constexpr bool B = false;     \
            __VA_ARGS__;                  \
        }                                 \
    } while (0)

// Launches the kernel expression with R_ = the warp-row radix (Px = 64 R_).
#define WARP_ROWS(wr, ...)                                                   \
    do {                                                                     \
        if ((wr) == 2) {                                                     \
            constexpr int R_ = 2;                                            \
            __VA_ARGS__;                                                     \
        } else if ((wr) == 3) {                                              \
            constexpr int R_ = 3;                                            \
            __VA_ARGS__;                                                     \
        } else {                                                             \
            constexpr int R_ = 4;                                            \
            __VA_ARGS__;                                                     \
        }                                                                    \
    } while (0)

// Launches the kernel expression with R_ = the warp-column radix (n = 32 R_).
#define WARP_COLS(wc, ...)                    \
    do {                                      \
        switch (wc) {                         \
        case 2: {                             \
            constexpr int R_ = 2;             \
            __VA_ARGS__;                      \
        } break;                              \
        case 3: {                             \
            constexpr int R_ = 3;             \
            __VA_ARGS__;                      \
        } break;                              \
        case 4: {                             \
            constexpr int R_ = 4;             \
            __VA_ARGS__;                      \
        } break;                              \
        case 5: {                             \
            constexpr int R_ = 5;             \
            __VA_ARGS__;                      \
        } break;                              \
        case 6: {                             \
            constexpr int R_ = 6;             \
            __VA_ARGS__;                      \
        } break;                              \
        default: {                            \
            constexpr int R_ = 8;             \
            __VA_ARGS__;                      \
        } break;                              \
        }                                     \
    } while (0)

// Launches the kernel expression with V_ = the tile column length (n = 16 V_).
#define TILE_COLS(tc, ...)                    \
    do {                                      \
        switch (tc) {                         \
        case 4: {                             \
            constexpr int V_ = 4;             \
            __VA_ARGS__;                      \
        } break;                              \
        case 6: {                             \
            constexpr int V_ = 6;             \
            __VA_ARGS__;                      \
        } break;                              \
        case 8: {                             \
            constexpr int V_ = 8;             \
            __VA_ARGS__;                      \
        } break;                              \
        case 12: {                            \
            constexpr int V_ = 12;            \
            __VA_ARGS__;                      \
        } break;                              \
        case 18: {                            \
            constexpr int V_ = 18;            \
            __VA_ARGS__;                      \
        } break;                              \
        default: {                            \
            constexpr int V_ = 16;            \
            __VA_ARGS__;                      \
        } break;                              \
        }                                     \
    } while (0)

namespace {
template <typename V>
V *dev_twiddles_impl(int n, cudaStream_t s, std::string &err)
{
    typedef typename Re<V>::t T;
    std::vector<V> h(n);
    for (int k = 0; k < n; ++k) {
        // exp(-2 pi i k / n), exact angle reduction by symmetry before the libm call
        const double a = -2.0 * M_PI * (double)k / (double)n;
        h[k].x = (T)std::cos(a);
        h[k].y = (T)std::sin(a);
    }
    V *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(V) * (size_t)n);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); return nullptr; }
    e = cudaMemcpyAsync(d, h.data(), sizeof(V) * (size_t)n, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { err = cudaGetErrorString(e); cudaFree(d); return nullptr; }
    return d;
}

template <typename T, bool B>
void set_smem_limits_big(int m)
{
    cudaFuncSetAttribute(k_rows_fwd<T, SrcMirror<T>, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_fwd<T, SrcZero<T>, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_fwd<T, SrcKernel, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_cols<T, 0, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_cols<T, 1, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_cols<T, 2, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_ratio<T, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_update<T, EPI_SEQ, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_update<T, EPI_MUL_FIRST, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_update<T, EPI_MUL_ACC, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_update<T, EPI_MUL_FINAL, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_update<T, EPI_STORE, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_rows_update<T, EPI_NLL, B>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
}

template <int R>
void set_smem_limits_wcols(int m)
{
    cudaFuncSetAttribute(k_wcols<R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_wcols<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_wcols<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
}

template <int V>
void set_smem_limits_tcols(int m)
{
    cudaFuncSetAttribute(k_tcols<V, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_tcols<V, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_tcols<V, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_tcols_pipe<V, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_tcols_pipe<V, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
    cudaFuncSetAttribute(k_tcols_pipe<V, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, m);
}

// Resident CTAs of the persistent column pass on the whole device (SMs x CTAs per SM).
template <int V, int MODE>
int pipe_resident()
{
    static int cached = 0;
    if (!cached) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_tcols_pipe<V, MODE>, kThreads, pipe_smem<V, MODE>());
        cached = std::max(1, sms * std::max(1, per));
    }
    return cached;
}

// The persistent column pass is used for the Z pass of 256-long columns, where it measured
// 4.6 TB/s against 3.3 TB/s of the one-tile-per-CTA pass; for the other lengths and the Y
// passes the one-tile-per-CTA pass is as fast or faster.  MVR_COLS_PIPE=0 disables it.
inline bool cols_pipe_enabled()
{
    static const bool on = [] {
        const char *e = std::getenv("MVR_COLS_PIPE");
        return !(e && e[0] == '0');
    }();
    return on;
}

template <typename T>
void set_smem_limits()
{
    // allow every instantiation to use up to the opt-in maximum; launches size it exactly
    static std::once_flag once;
    std::call_once(once, [] {
        const int m = (int)kSmemMax;
        set_smem_limits_big<T, false>(m);
        set_smem_limits_big<T, true>(m);
        set_smem_limits_wcols<2>(m);
        set_smem_limits_wcols<3>(m);
        set_smem_limits_wcols<4>(m);
        set_smem_limits_wcols<5>(m);
        set_smem_limits_wcols<6>(m);
        set_smem_limits_wcols<8>(m);
        set_smem_limits_tcols<4>(m);
        set_smem_limits_tcols<6>(m);
        set_smem_limits_tcols<8>(m);
        set_smem_limits_tcols<12>(m);
        set_smem_limits_tcols<16>(m);
        set_smem_limits_tcols<18>(m);
    });
}

// Two-phase tile column length V (n = 16 V) for an FP32 axis of length n (0: none).
template <typename T>
int tile_col_v(int n)
{
    if (sizeof(T) != sizeof(float) || n % 16) return 0;
    const int v = n / 16;
    return (v == 4 || v == 6 || v == 8 || v == 12 || v == 16 || v == 18) ? v : 0;
}

// Warp-shuffle column radix for an FP32 axis of length n (0: shared-memory kernels).
template <typename T>
int warp_col_radix(int n)
{
    if (sizeof(T) != sizeof(float) || n % 32) return 0;
    const int r = n / 32;
    return (r == 2 || r == 3 || r == 4 || r == 5 || r == 6 || r == 8) ? r : 0;
}
}  // namespace

template <typename T>
Engine<T>::~Engine()
{
    if (device_ >= 0) cudaSetDevice(device_);
    cudaFree(S0_);
    cudaFree(S1_);
    cudaFree(prod_);
    cudaFree(partials_);
    cudaFree(kbuf_);
    for (auto &p : pending_) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : event_pool_) cudaEventDestroy(e);
    if (stream_) cudaStreamDestroy(stream_);
}

template <typename T>
int Engine<T>::prof_begin(int kind, double bytes)
{
    ++launches_;
    if (!prof_on_) return OK;
    Pending p{kind, bytes, nullptr, nullptr};
    for (cudaEvent_t *e : {&p.a, &p.b}) {
        if (!event_pool_.empty()) {
            *e = event_pool_.back();
            event_pool_.pop_back();
        } else {
            MVR_CUDA(cudaEventCreate(e));
        }
    }
    MVR_CUDA(cudaEventRecord(p.a, stream_));
    pending_.push_back(p);
    return OK;
}

template <typename T>
int Engine<T>::prof_end()
{
    if (!prof_on_ || pending_.empty()) return OK;
    MVR_CUDA(cudaEventRecord(pending_.back().b, stream_));
    return OK;
}

template <typename T>
int Engine<T>::profile_collect(KernelProfile &out)
{
    MVR_CUDA(cudaStreamSynchronize(stream_));
    for (auto &p : pending_) {
        float ms = 0.0f;
        MVR_CUDA(cudaEventElapsedTime(&ms, p.a, p.b));
        acc_.ms[p.kind] += ms;
        acc_.launches[p.kind] += 1;
        acc_.bytes[p.kind] += p.bytes;
        event_pool_.push_back(p.a);
        event_pool_.push_back(p.b);
    }
    pending_.clear();
    out = acc_;
    return OK;
}

template <typename T>
int Engine<T>::init(int device, int boundary, double lambda, float min_value)
{
    int n = 0;
    MVR_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return fail(ERR_ARG, "device ordinal out of range");
    device_ = device;
    boundary_ = boundary;
    lambda_ = lambda;
    min_value_ = min_value;
    MVR_CUDA(cudaSetDevice(device));
    MVR_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    set_smem_limits<T>();
    return OK;
}

template <typename T>
int Engine<T>::reserve(long long Pc, long long nvox_block, long long rows, int nb)
{
    if (nb < 1) nb = 1;
    if (Pc * nb > Scap_) {
        cudaFree(S0_);
        cudaFree(S1_);
        S0_ = S1_ = nullptr;
        Scap_ = 0;
        MVR_CUDA(cudaMalloc(&S0_, sizeof(V) * (size_t)(Pc * nb)));
        MVR_CUDA(cudaMalloc(&S1_, sizeof(V) * (size_t)(Pc * nb)));
        Scap_ = Pc * nb;
        ++alloc_epoch_;
    }
    if (rows * nb > partcap_) {
        cudaFree(partials_);
        partials_ = nullptr;
        partcap_ = 0;
        MVR_CUDA(cudaMalloc(&partials_, sizeof(double) * 2 * (size_t)(rows * nb)));
        partcap_ = rows * nb;
        ++alloc_epoch_;
    }
    (void)nvox_block;
    return OK;
}

template <typename T>
int Engine<T>::reserve_prod(long long n)
{
    if (n > prodcap_) {
        cudaFree(prod_);
        prod_ = nullptr;
        prodcap_ = 0;
        MVR_CUDA(cudaMalloc(&prod_, sizeof(double) * (size_t)n));
        prodcap_ = n;
        ++alloc_epoch_;
    }
    return OK;
}

template <typename T>
void Engine<T>::free_plan(Plan<T> &pl)
{
    cudaFree(pl.twx);
    cudaFree(pl.twy);
    cudaFree(pl.twz);
    cudaFree(pl.k1h);
    cudaFree(pl.k2h);
    pl.twx = pl.twy = pl.twz = pl.k1h = pl.k2h = nullptr;
}

template <typename T>
std::vector<int> Engine<T>::schedule_candidates(const Plan<T> &pl) const
{
    std::vector<int> paths = {SCHED_ROWS};
    if (pl.xy_cap) {
        paths.push_back(SCHED_PLANE);
        paths.push_back(SCHED_PLANE_PERSIST);
    }
    if (pl.pair_cap) paths.push_back(SCHED_PAIR);
    std::vector<int> out;
    for (int p : paths) {
        out.push_back(p);
        if (sizeof(T) == sizeof(float) && pl.tcz) out.push_back(p | SCHED_ZPIPE);
    }
    return out;
}

template <typename T>
int Engine<T>::schedule(const Plan<T> &pl) const
{
    const int path = pl.xy >= 10000 ? SCHED_PAIR : (pl.xy ? (pl.persist ? SCHED_PLANE_PERSIST : SCHED_PLANE) : SCHED_ROWS);
    const bool zp = pl.zpipe >= 0 ? pl.zpipe == 1 : (cols_pipe_enabled() && pl.tcz == 16);
    return path | (zp && sizeof(T) == sizeof(float) && pl.tcz ? SCHED_ZPIPE : 0);
}

template <typename T>
int Engine<T>::set_schedule(Plan<T> &pl, int code)
{
    const int path = code & 3;
    if (code < 0 || code > (SCHED_PAIR | SCHED_ZPIPE)) return fail(ERR_ARG, "unknown FFT schedule");
    if ((path == SCHED_PLANE || path == SCHED_PLANE_PERSIST) && !pl.xy_cap)
        return fail(ERR_UNSUPPORTED, "no plane kernels for this FFT domain");
    if (path == SCHED_PAIR && !pl.pair_cap) return fail(ERR_UNSUPPORTED, "no pair kernels for this FFT domain");
    if ((code & SCHED_ZPIPE) && !(sizeof(T) == sizeof(float) && pl.tcz))
        return fail(ERR_UNSUPPORTED, "no tile column kernels for this Z length");
    const int xy = path == SCHED_ROWS ? 0 : (path == SCHED_PAIR ? pl.pair_cap : pl.xy_cap);
    if (xy != pl.kspec_xy && !pl.ksrc1)
        return fail(ERR_STATE, "the plan's kernels are not on the device: its path cannot change");
    pl.xy = xy;
    pl.persist = path == SCHED_PLANE_PERSIST || path == SCHED_PAIR ? 1 : 0;
    pl.zpipe = (code & SCHED_ZPIPE) ? 1 : 0;
    if (pl.xy != pl.kspec_xy) return kernel_spectra(pl, pl.ksrc1, pl.ksrc2, true);  // another spectrum layout
    return OK;
}

template <typename T>
int Engine<T>::make_plan(Plan<T> &pl, const int b[3], const float *k1, const int kd1[3], const float *k2,
                         const int kd2[3], bool k_on_device)
{
    if (stream_ == nullptr) return fail(ERR_STATE, "engine not initialised");
    for (int d = 0; d < 3; ++d) {
        if (b[d] < 1 || kd1[d] < 1) return fail(ERR_ARG, "block and kernel sizes must be >= 1");
        if (k2 && kd2[d] != kd1[d]) return fail(ERR_ARG, "kernel1 and kernel2 must have the same size");
        if (kd1[d] > b[d] && boundary_ == BOUNDARY_CIRCULAR)
            return fail(ERR_ARG, "kernel larger than the block under circular boundary");
    }
    free_plan(pl);
    for (int d = 0; d < 3; ++d) {
        pl.b[d] = b[d];
        pl.kd[d] = kd1[d];
        if (boundary_ == BOUNDARY_CIRCULAR) {
            pl.P[d] = b[d];
            pl.L[d] = 0;
            if (!fft_friendly(b[d]) || (d == 0 && (b[d] & 1)))
                return fail(ERR_UNSUPPORTED, "circular boundary needs block sizes with prime factors <= 13 (even along x)");
        } else {
            pl.P[d] = (int)next_friendly_even(b[d] + kd1[d] - 1);
            pl.L[d] = kd1[d] - 1 - kd1[d] / 2;
        }
    }
    if (pl.P[0] > 4096 || pl.P[1] > 2048 || pl.P[2] > 2048)
        return fail(ERR_UNSUPPORTED, "FFT domain larger than 4096 x 2048 x 2048");
    pl.Hx = pl.P[0] / 2 + 1;
    pl.Pc = (long long)pl.Hx * pl.P[1] * pl.P[2];
    pl.dx = make_desc(pl.P[0] / 2);
    pl.dy = make_desc(pl.P[1]);
    pl.dz = make_desc(pl.P[2]);
    pl.big = false;
    for (const FftDesc *dd : {&pl.dx, &pl.dy, &pl.dz})
        for (int st = 0; st < dd->ns; ++st)
            if (dd->radix[st] == 7 || dd->radix[st] == 11 || dd->radix[st] == 13) pl.big = true;
    std::string e;
    pl.twx = dev_twiddles_impl<V>(pl.P[0], stream_, e);
    pl.twy = dev_twiddles_impl<V>(pl.P[1], stream_, e);
    pl.twz = dev_twiddles_impl<V>(pl.P[2], stream_, e);
    if (!pl.twx || !pl.twy || !pl.twz) return fail(ERR_CUDA, "twiddle upload: " + e);
    // launch shapes
    const int m = pl.P[0] / 2;
    const size_t per_row = 2 * sizeof(V) * (size_t)(m + 1);
    const size_t tws = sizeof(V) * (size_t)pl.P[0];
    int RP = 16;
    while (RP > 1 && tws + RP * per_row > kRowSmemTarget) RP >>= 1;
    if (tws + RP * per_row > kSmemMax) return fail(ERR_UNSUPPORTED, "row too long for shared memory");
    pl.RP = RP;
    pl.smem_row = tws + RP * per_row;
    pl.wr = (sizeof(T) == sizeof(float) && (pl.P[0] == 128 || pl.P[0] == 192 || pl.P[0] == 256)) ? pl.P[0] / 64 : 0;
    pl.tcy = tile_col_v<T>(pl.P[1]);
    pl.tcz = tile_col_v<T>(pl.P[2]);
    {
        // plane kernels: FP32, z along the tile column kernels; MVR_PLANE_KERNELS=0 turns them off
        const char *env = std::getenv("MVR_PLANE_KERNELS");
        const bool allow = !(env && env[0] == '0');
        pl.xy_cap = (sizeof(T) == sizeof(float) && pl.tcz) ? xy_combo(pl.P) : 0;
        pl.pair_cap = (sizeof(T) == sizeof(float) && pl.tcz) ? xy_pair_combo(pl.P) : 0;
        pl.xy = allow ? pl.xy_cap : 0;
        // the pair kernels for the domains without single-CTA plane kernels (MVR_PAIR_KERNELS=1)
        const char *pe = std::getenv("MVR_PAIR_KERNELS");
        if (allow && !pl.xy && pl.pair_cap && pe && pe[0] == '1') pl.xy = pl.pair_cap;
        pl.persist = 1;
        pl.zpipe = -1;
    }
    pl.wcy = pl.tcy ? 0 : warp_col_radix<T>(pl.P[1]);
    pl.wcz = pl.tcz ? 0 : warp_col_radix<T>(pl.P[2]);
    auto col_np = [&](int n, int &NP, size_t &smem) -> bool {
        NP = 16;
        while (NP > 1 && sizeof(V) * (size_t)n * (1 + 2 * NP) > kColSmemTarget) NP >>= 1;
        smem = sizeof(V) * (size_t)n * (1 + 2 * NP);
        return smem <= kSmemMax;
    };
    if (!col_np(pl.P[1], pl.NPy, pl.smem_coly) || !col_np(pl.P[2], pl.NPz, pl.smem_colz))
        return fail(ERR_UNSUPPORTED, "column too long for shared memory");
    const long long nrows = (long long)pl.P[1] * pl.P[2];
    MVR_TRY(reserve(pl.Pc, (long long)b[0] * b[1] * b[2], (nrows + pl.RP - 1) / pl.RP, 1));
    // kernel spectra, scaled by 1 / (Px Py Pz) so that the inverse needs no scaling
    MVR_CUDA(cudaMalloc(&pl.k1h, sizeof(V) * (size_t)pl.Pc));
    if (k2) MVR_CUDA(cudaMalloc(&pl.k2h, sizeof(V) * (size_t)pl.Pc));
    pl.ksrc1 = k_on_device ? k1 : nullptr;
    pl.ksrc2 = k_on_device ? k2 : nullptr;
    return kernel_spectra(pl, k1, k2, k_on_device);
}

// The kernel spectra K1^, K2^ of a plan, computed by the forward kernels of the plan's path
// (the plane kernels leave x and y in tile order, the row / column kernels in natural order;
// every product is taken position by position, so K^ must come from the same path).
template <typename T>
int Engine<T>::kernel_spectra(Plan<T> &pl, const float *k1, const float *k2, bool k_on_device)
{
    const int *kd1 = pl.kd;
    const long long nrows = (long long)pl.P[1] * pl.P[2];
    const long long kn = (long long)kd1[0] * kd1[1] * kd1[2];
    if (!k_on_device && kn > kcap_) {
        cudaFree(kbuf_);
        kbuf_ = nullptr;
        kcap_ = 0;
        MVR_CUDA(cudaMalloc(&kbuf_, sizeof(float) * (size_t)kn));
        kcap_ = kn;
    }
    BlockMaps bms{};
    BlockMap &bm = bms.m[0];
    for (int d = 0; d < 3; ++d) {
        bm.P[d] = pl.P[d];
        bm.b[d] = pl.P[d];
        bm.D[d] = pl.P[d];
    }
    bm.fast_x = block_fast_x(bm);
    const double scale = 1.0 / ((double)pl.P[0] * pl.P[1] * pl.P[2]);
    pl.kspec_xy = pl.xy;
    for (int which = 0; which < (k2 ? 2 : 1); ++which) {
        const float *kh = which == 0 ? k1 : k2;
        const float *kdev = kh;
        if (!k_on_device) {
            MVR_CUDA(cudaMemcpyAsync(kbuf_, kh, sizeof(float) * (size_t)kn, cudaMemcpyHostToDevice, stream_));
            kdev = kbuf_;
        }
        SrcKernel src{kdev, {kd1[0], kd1[1], kd1[2]}, scale};
        if constexpr (sizeof(T) == sizeof(float)) {
            if (pl.xy) {
                ++launches_;
                MVR_CUDA(xy_fwd_kernel(pl.xy, src, S0_, bms, 1, pl.P[2], pl.Pc, pl.twx, pl.twy, stream_, pl.persist != 0));
                MVR_TRY(launch_cols(pl, 2, 0, S0_, which == 0 ? pl.k1h : pl.k2h, nullptr, 1));
                continue;
            }
        }
        const dim3 grid((unsigned)((nrows + pl.RP - 1) / pl.RP), 1);
        MVR_WITH_BIG(pl.big, (k_rows_fwd<T, SrcKernel, B><<<grid, kThreads, pl.smem_row, stream_>>>(
                                 src, S0_, bms, pl.Pc, pl.dx, pl.twx, pl.RP)));
        MVR_LAUNCHED("k_rows_fwd(kernel)");
        MVR_TRY(launch_cols(pl, 1, 0, S0_, S0_, nullptr, 1));
        MVR_TRY(launch_cols(pl, 2, 0, S0_, which == 0 ? pl.k1h : pl.k2h, nullptr, 1));
    }
    MVR_CUDA(cudaStreamSynchronize(stream_));
    return OK;
}

template <typename T>
int Engine<T>::launch_cols(const Plan<T> &pl, int axis, int mode, const V *src, V *dst, const V *Kh, int nb, int rlo,
                           int rhi, int olo, int ohi, int llo, int lhi)
{
    const int Hx = pl.Hx;
    long long estride, ostride;
    int nother, NP;
    size_t smem;
    const FftDesc *d;
    if (axis == 1) {
        estride = Hx;
        ostride = (long long)pl.P[1] * Hx;
        nother = pl.P[2];
        NP = pl.NPy;
        smem = pl.smem_coly;
        d = &pl.dy;
    } else {
        estride = (long long)pl.P[1] * Hx;
        ostride = Hx;
        nother = pl.P[1];
        NP = pl.NPz;
        smem = pl.smem_colz;
        d = &pl.dz;
    }
    const V *tw = axis == 1 ? pl.twy : pl.twz;
    const dim3 grid((unsigned)((Hx + NP - 1) / NP), (unsigned)nother, (unsigned)nb);
    const double cb = (double)sizeof(V) * (double)pl.Pc * nb;
    const int kind = mode == 2 ? KK_COLS_ZMUL : (mode == 1 ? KK_COLS_INV : KK_COLS_FWD);
    const int nax = pl.P[axis];
    const bool tiled = sizeof(T) == sizeof(float) && (axis == 1 ? pl.tcy : pl.tcz);
    if (rhi < 0 || rhi > nax || !tiled) rhi = nax;
    if (rlo < 0 || rlo > rhi || rhi == nax) rlo = 0;
    if (lhi < 0 || lhi > nax) lhi = nax;
    if (llo < 0 || llo > lhi) llo = 0;
    if ((llo > 0 || lhi < nax) && !tiled) return fail(ERR_STATE, "a partial input band needs a tile pass");
    if (ohi < 0 || ohi > nother || !tiled) ohi = nother;
    if (olo < 0 || olo >= ohi) olo = 0;
    const double stored = (double)(rhi - rlo) / nax, loaded = (double)(lhi - llo) / nax;
    const double part = (double)(ohi - olo) / nother;
    MVR_TRY(prof_begin(kind, part * (mode == 2 ? (1.0 + loaded + stored) * cb : (loaded + stored) * cb)));
    const long long Pc = pl.Pc;
    const int wc = axis == 1 ? pl.wcy : pl.wcz;
    const int tc = axis == 1 ? pl.tcy : pl.tcz;
    if constexpr (sizeof(T) == sizeof(float)) {
        if (tc) {
            // Hx = 16 q + 1: q full tiles, and the last column in gathered tiles of 16
            // other-axis indices (an extra x tile of the same grid)
            const int gather = (Hx > 1 && Hx % kTColNP == 1) ? 1 : 0;
            const int hmain = gather ? Hx - 1 : Hx;
            const bool pipe = pl.zpipe >= 0 ? (pl.zpipe == 1 && axis == 2 && mode == 2)
                                            : (cols_pipe_enabled() && tc == 16 && mode == 2);
            if (pipe) {
                PipeGeom pg;
                pg.hmain = (hmain + kTColNP - 1) / kTColNP;
                pg.ny = ohi - olo;
                pg.gtiles = gather ? (pg.ny + kTColNP - 1) / kTColNP : 0;
                pg.per_block = pg.hmain * pg.ny + pg.gtiles;
                pg.ntiles = pg.per_block * nb;
                TILE_COLS(tc, {
                    const size_t ps = pipe_smem<V_, 0>();
                    if (mode == 0)
                        k_tcols_pipe<V_, 0><<<std::min(pg.ntiles, pipe_resident<V_, 0>()), kThreads, ps, stream_>>>(
                            src, dst, Kh, Hx, estride, ostride, Pc, tw, gather, ohi, rlo, rhi, olo, pg, llo, lhi);
                    else if (mode == 1)
                        k_tcols_pipe<V_, 1><<<std::min(pg.ntiles, pipe_resident<V_, 1>()), kThreads, ps, stream_>>>(
                            src, dst, Kh, Hx, estride, ostride, Pc, tw, gather, ohi, rlo, rhi, olo, pg, llo, lhi);
                    else
                        MVR_CUDA(launch_pdl(k_tcols_pipe<V_, 2>, std::min(pg.ntiles, pipe_resident<V_, 2>()), kThreads,
                                            pipe_smem<V_, 2>(), stream_, src, dst, Kh, Hx, estride, ostride, Pc, tw,
                                            gather, ohi, rlo, rhi, olo, pg, llo, lhi));
                });
                MVR_LAUNCHED("k_tcols_pipe");
                return prof_end();
            }
            const size_t ts = tcols_smem(tc, mode);
            const dim3 tgrid((unsigned)((hmain + kTColNP - 1) / kTColNP + gather), (unsigned)(ohi - olo), (unsigned)nb);
            TILE_COLS(tc, {
                if (mode == 0)
                    MVR_CUDA(launch_pdl(k_tcols<V_, 0>, tgrid, kThreads, ts, stream_, src, dst, Kh, Hx, estride, ostride, Pc, tw,
                                       gather, ohi, rlo, rhi, olo, llo, lhi));
                else if (mode == 1)
                    MVR_CUDA(launch_pdl(k_tcols<V_, 1>, tgrid, kThreads, ts, stream_, src, dst, Kh, Hx, estride, ostride, Pc, tw,
                                       gather, ohi, rlo, rhi, olo, llo, lhi));
                else
                    MVR_CUDA(launch_pdl(k_tcols<V_, 2>, tgrid, kThreads, ts, stream_, src, dst, Kh, Hx, estride, ostride, Pc, tw,
                                       gather, ohi, rlo, rhi, olo, llo, lhi));
            });
            MVR_LAUNCHED("k_tcols");
            return prof_end();
        }
        if (wc) {
            const dim3 wgrid((unsigned)((Hx + kWColNP - 1) / kWColNP), (unsigned)nother, (unsigned)nb);
            const size_t ws = wcols_smem(wc, mode);
            WARP_COLS(wc, {
                if (mode == 0)
                    k_wcols<R_, 0><<<wgrid, kThreads, ws, stream_>>>(src, dst, Kh, Hx, estride, ostride, Pc, tw);
                else if (mode == 1)
                    k_wcols<R_, 1><<<wgrid, kThreads, ws, stream_>>>(src, dst, Kh, Hx, estride, ostride, Pc, tw);
                else
                    k_wcols<R_, 2><<<wgrid, kThreads, ws, stream_>>>(src, dst, Kh, Hx, estride, ostride, Pc, tw);
            });
            MVR_LAUNCHED("k_wcols");
            return prof_end();
        }
    }
    MVR_WITH_BIG(pl.big, {
        if (mode == 0)
            k_cols<T, 0, B><<<grid, kThreads, smem, stream_>>>(src, dst, Kh, Hx, estride, ostride, NP, Pc, *d, tw);
        else if (mode == 1)
            k_cols<T, 1, B><<<grid, kThreads, smem, stream_>>>(src, dst, Kh, Hx, estride, ostride, NP, Pc, *d, tw);
        else
            k_cols<T, 2, B><<<grid, kThreads, smem, stream_>>>(src, dst, Kh, Hx, estride, ostride, NP, Pc, *d, tw);
    });
    MVR_LAUNCHED("k_cols");
    return prof_end();
}

template <typename T>
BlockMaps Engine<T>::block_maps(const Plan<T> &pl, const BlockPlace *bps, int nb) const
{
    BlockMaps bms{};
    for (int i = 0; i < nb; ++i) {
        BlockMap &bm = bms.m[i];
        const BlockPlace &bp = bps[i];
        for (int d = 0; d < 3; ++d) {
            bm.P[d] = pl.P[d];
            bm.b[d] = pl.b[d];
            bm.L[d] = pl.L[d];
            bm.off[d] = bp.off[d];
            bm.D[d] = bp.D[d];
            bm.wlo[d] = bp.wlo[d];
            bm.whi[d] = bp.whi[d];
            bm.ooff[d] = bp.ooff[d];
            bm.OD[d] = bp.OD[d];
        }
        bm.fast_x = block_fast_x(bm);
    }
    return bms;
}

template <typename T>
int Engine<T>::launch_fwd_mirror(const Plan<T> &pl, const BlockMaps &bms, int nb, const T *src, V *S)
{
    const long long nrows = (long long)pl.P[1] * pl.P[2];
    const dim3 grid((unsigned)((nrows + pl.RP - 1) / pl.RP), (unsigned)nb);
    const double nv = (double)pl.b[0] * pl.b[1] * pl.b[2];
    MVR_TRY(prof_begin(KK_ROWS_FWD, nb * (sizeof(T) * nv + sizeof(V) * (double)pl.Pc)));
    if constexpr (sizeof(T) == sizeof(float)) {
        if (pl.wr) {
            WARP_ROWS(pl.wr, (k_wrows_fwd<R_><<<grid, kThreads, 0, stream_>>>(src, S, bms, pl.Pc, pl.twx)));
            MVR_LAUNCHED("k_wrows_fwd");
            return prof_end();
        }
    }
    MVR_WITH_BIG(pl.big, (k_rows_fwd<T, SrcMirror<T>, B><<<grid, kThreads, pl.smem_row, stream_>>>(
                             SrcMirror<T>{src}, S, bms, pl.Pc, pl.dx, pl.twx, pl.RP)));
    MVR_LAUNCHED("k_rows_fwd");
    return prof_end();
}

template <typename T>
int Engine<T>::launch_ratio(const Plan<T> &pl, const BlockMaps &bms, int nb, V *S, const float *img)
{
    const long long nrows = (long long)pl.P[1] * pl.P[2];
    const dim3 grid((unsigned)((nrows + pl.RP - 1) / pl.RP), (unsigned)nb);
    const double nv = (double)pl.b[0] * pl.b[1] * pl.b[2];
    MVR_TRY(prof_begin(KK_ROWS_RATIO, nb * (2.0 * sizeof(V) * (double)pl.Pc + 4.0 * nv)));
    if constexpr (sizeof(T) == sizeof(float)) {
        if (pl.wr) {
            WARP_ROWS(pl.wr, (k_wrows_ratio<R_><<<grid, kThreads, 0, stream_>>>(S, img, bms, pl.Pc, pl.twx)));
            MVR_LAUNCHED("k_wrows_ratio");
            return prof_end();
        }
    }
    MVR_WITH_BIG(pl.big, (k_rows_ratio<T, B><<<grid, kThreads, pl.smem_row, stream_>>>(S, img, bms, pl.Pc, pl.dx,
                                                                                          pl.twx, pl.RP)));
    MVR_LAUNCHED("k_rows_ratio");
    return prof_end();
}

template <typename T>
int Engine<T>::launch_update(const Plan<T> &pl, const BlockMaps &bms, int nb, V *S, const UpdateArgs &ua, int epi,
                             double bytes, double *stats_dev)
{
    long long nrows = (long long)pl.P[1] * pl.P[2];
    if (ua.prune) {  // k_wrows_update over the rows of the write regions' planes
        if (!(sizeof(T) == sizeof(float) && pl.wr && epi == EPI_SEQ)) return fail(ERR_STATE, "pruned update");
        int depth = 0;
        for (int i = 0; i < nb; ++i) depth = std::max(depth, bms.m[i].whi[2] - bms.m[i].wlo[2]);
        nrows = (long long)pl.P[1] * depth;
    }
    const unsigned gx = (unsigned)std::max(1LL, (nrows + pl.RP - 1) / pl.RP);
    const dim3 grid(gx, (unsigned)nb);
    MVR_TRY(prof_begin(KK_ROWS_UPDATE, bytes));
    bool warp_done = false;
    if constexpr (sizeof(T) == sizeof(float)) {
        if (pl.wr && epi == EPI_SEQ) {
            WARP_ROWS(pl.wr, (k_wrows_update<R_><<<grid, kThreads, 0, stream_>>>(S, ua, bms, pl.Pc, pl.twx)));
            MVR_LAUNCHED("k_wrows_update");
            warp_done = true;
        }
    }
    if (!warp_done) MVR_WITH_BIG(pl.big, {
        switch (epi) {
        case EPI_SEQ:
            k_rows_update<T, EPI_SEQ, B><<<grid, kThreads, pl.smem_row, stream_>>>(S, ua, bms, pl.Pc, pl.dx, pl.twx, pl.RP);
            break;
        case EPI_MUL_FIRST:
            k_rows_update<T, EPI_MUL_FIRST, B><<<grid, kThreads, pl.smem_row, stream_>>>(S, ua, bms, pl.Pc, pl.dx,
                                                                                         pl.twx, pl.RP);
            break;
        case EPI_MUL_ACC:
            k_rows_update<T, EPI_MUL_ACC, B><<<grid, kThreads, pl.smem_row, stream_>>>(S, ua, bms, pl.Pc, pl.dx, pl.twx,
                                                                                       pl.RP);
            break;
        case EPI_MUL_FINAL:
            k_rows_update<T, EPI_MUL_FINAL, B><<<grid, kThreads, pl.smem_row, stream_>>>(S, ua, bms, pl.Pc, pl.dx,
                                                                                         pl.twx, pl.RP);
            break;
        case EPI_NLL:
            k_rows_update<T, EPI_NLL, B><<<grid, kThreads, pl.smem_row, stream_>>>(S, ua, bms, pl.Pc, pl.dx, pl.twx,
                                                                                   pl.RP);
            break;
        default:
            k_rows_update<T, EPI_STORE, B><<<grid, kThreads, pl.smem_row, stream_>>>(S, ua, bms, pl.Pc, pl.dx, pl.twx,
                                                                                     pl.RP);
            break;
        }
    });
    MVR_LAUNCHED("k_rows_update");
    MVR_TRY(prof_end());
    if (stats_dev && (epi == EPI_SEQ || epi == EPI_MUL_FINAL || epi == EPI_NLL)) {
        MVR_TRY(prof_begin(KK_REDUCE, 16.0 * gx * nb));
        k_reduce_stats<double><<<nb, 1024, 0, stream_>>>(partials_, (int)gx, stats_dev);
        MVR_LAUNCHED("k_reduce_stats");
        MVR_TRY(prof_end());
    }
    return OK;
}

// ---- plane kernels (FP32 plans with pl.xy) ---------------------------------------------
template <typename T>
int Engine<T>::launch_xy_fwd(const Plan<T> &pl, const BlockMaps &bms, int nb, const T *src, V *S)
{
    if constexpr (sizeof(T) == sizeof(float)) {
        const double nv = (double)pl.b[0] * pl.b[1] * pl.b[2];
        MVR_TRY(prof_begin(KK_XY_FWD, nb * (sizeof(T) * nv + sizeof(V) * (double)pl.Pc)));
        MVR_CUDA(xy_fwd_mirror(pl.xy, src, S, bms, nb, pl.P[2], pl.Pc, pl.twx, pl.twy, stream_, pl.persist != 0));
        return prof_end();
    }
    return fail(ERR_STATE, "plane kernels are FP32 only");
}

// The second convolution's output on the planes [zlo, zhi) reads its input on
// [zlo - r, zhi + r) only, r = kd / 2 + 1 covering the kernel's reach on either side of its
// centre.  When that band lies inside the domain (no circular wrap) and is shorter than it, the
// first convolution's Z pass stores the band alone, the quotient pass works on it, and the
// second convolution's Z pass reads it with zeros for the other planes: those carry no weight
// in the outputs that are kept.
// MVR_RATIO_BAND=0 keeps the quotient pass on every plane
static bool ratio_band_off()
{
    const char *e = std::getenv("MVR_RATIO_BAND");
    return e && e[0] == '0';
}

template <typename T>
bool Engine<T>::ratio_band(const Plan<T> &pl, int zlo, int zhi, int &lo, int &hi) const
{
    lo = 0;
    hi = pl.P[2];
    if (sizeof(T) != sizeof(float) || !pl.tcz || zhi <= zlo || ratio_band_off()) return false;
    const int r = pl.kd[2] / 2 + 1;
    if (zlo - r < 0 || zhi + r > pl.P[2] || zhi - zlo + 2 * r >= pl.P[2]) return false;
    lo = zlo - r;
    hi = zhi + r;
    return true;
}

template <typename T>
int Engine<T>::launch_xy_ratio(const Plan<T> &pl, const BlockMaps &bms, int nb, V *S, const float *img, int zlo,
                               int zhi)
{
    if constexpr (sizeof(T) == sizeof(float)) {
        if (zhi < 0 || zhi > pl.P[2]) zhi = pl.P[2];
        if (zlo < 0 || zlo >= zhi) zlo = 0;
        const double part = (double)(zhi - zlo) / pl.P[2];
        const double nv = (double)pl.b[0] * pl.b[1] * pl.b[2];
        MVR_TRY(prof_begin(KK_XY_RATIO, part * nb * (2.0 * sizeof(V) * (double)pl.Pc + 4.0 * nv)));
        MVR_CUDA(xy_ratio(pl.xy, S, img, bms, nb, zlo, zhi - zlo, pl.Pc, pl.twx, pl.twy, stream_, pl.persist != 0));
        return prof_end();
    }
    return fail(ERR_STATE, "plane kernels are FP32 only");
}

template <typename T>
int Engine<T>::launch_xy_update(const Plan<T> &pl, const BlockMaps &bms, int nb, V *S, const UpdateArgs &ua, int epi,
                                double bytes, double *stats_dev)
{
    if constexpr (sizeof(T) == sizeof(float)) {
        MVR_TRY(prof_begin(KK_XY_UPDATE, bytes));
        // partial slots per block: one per CTA of the update grid (planes of the deepest write
        // region when pruned; a pruned likelihood leaves the slots of shallower blocks' extra
        // planes at zero)
        int planes = pl.P[2];
        if (ua.prune) {
            planes = 0;
            for (int i = 0; i < nb; ++i) planes = std::max(planes, bms.m[i].whi[2] - bms.m[i].wlo[2]);
        }
        const int slots = xy_partial_slots(pl.xy, planes);
        if (ua.prune && epi == EPI_NLL && stats_dev)
            MVR_CUDA(cudaMemsetAsync(partials_, 0, sizeof(double) * 2 * (size_t)slots * nb, stream_));
        MVR_CUDA(xy_update(pl.xy, epi, S, ua, bms, nb, pl.P[2], pl.Pc, pl.twx, pl.twy, stream_));
        MVR_TRY(prof_end());
        if (stats_dev && (epi == EPI_SEQ || epi == EPI_MUL_FINAL || epi == EPI_NLL)) {
            MVR_TRY(prof_begin(KK_REDUCE, 16.0 * slots * nb));
            k_reduce_stats<double><<<nb, 1024, 0, stream_>>>(partials_, slots, stats_dev);
            MVR_LAUNCHED("k_reduce_stats");
            MVR_TRY(prof_end());
        }
        return OK;
    }
    return fail(ERR_STATE, "plane kernels are FP32 only");
}

// The planes [zlo, zhi) and rows [ylo, yhi) holding every write region of a batch.
inline void write_region(const BlockPlace *bps, int nb, int &zlo, int &zhi, int &ylo, int &yhi)
{
    zlo = bps[0].wlo[2];
    zhi = bps[0].whi[2];
    ylo = bps[0].wlo[1];
    yhi = bps[0].whi[1];
    for (int i = 1; i < nb; ++i) {
        zlo = std::min(zlo, bps[i].wlo[2]);
        zhi = std::max(zhi, bps[i].whi[2]);
        ylo = std::min(ylo, bps[i].wlo[1]);
        yhi = std::max(yhi, bps[i].whi[1]);
    }
}

template <typename T>
int Engine<T>::run_seq(const Plan<T> &pl, const BlockPlace *bps, int nb, const float *img, const float *w, float maxI,
                       double *stats_dev)
{
    if (!pl.k1h || !pl.k2h) return fail(ERR_STATE, "kernels not set for this view");
    if (nb < 1 || nb > kMaxBatch) return fail(ERR_ARG, "batch of 1..16 blocks");
    const long long nrows = (long long)pl.P[1] * pl.P[2];
    MVR_TRY(reserve(pl.Pc, (long long)pl.b[0] * pl.b[1] * pl.b[2], (nrows + pl.RP - 1) / pl.RP, nb));
    const BlockMaps bms = block_maps(pl, bps, nb);
    // without statistics only the write regions are needed after the second convolution
    // (the plane kernels, or the warp-row update of the row / column path)
    const bool prune = !stats_dev && (pl.xy || (sizeof(T) == sizeof(float) && pl.wr));
    int zlo = 0, zhi = -1, ylo = 0, yhi = -1;
    if (prune) write_region(bps, nb, zlo, zhi, ylo, yhi);
    if (pl.xy) {
        int blo = 0, bhi = -1;
        if (prune) ratio_band(pl, zlo, zhi, blo, bhi);
        MVR_TRY(launch_xy_fwd(pl, bms, nb, reinterpret_cast<const T *>(bps[0].psi_src), S0_));
        // the first convolution stores the band, the quotient pass works on it, and the second
        // convolution reads it (the planes outside it are zeros to the transform)
        MVR_TRY(launch_cols(pl, 2, 2, S0_, S0_, pl.k1h, nb, blo, bhi));
        MVR_TRY(launch_xy_ratio(pl, bms, nb, S0_, img, blo, bhi));
        MVR_TRY(launch_cols(pl, 2, 2, S0_, S0_, pl.k2h, nb, zlo, zhi, 0, -1, blo, bhi));
    } else {
        MVR_TRY(launch_fwd_mirror(pl, bms, nb, reinterpret_cast<const T *>(bps[0].psi_src), S0_));
        MVR_TRY(launch_cols(pl, 1, 0, S0_, S0_, nullptr, nb));
        MVR_TRY(launch_cols(pl, 2, 2, S0_, S0_, pl.k1h, nb));
        MVR_TRY(launch_cols(pl, 1, 1, S0_, S0_, nullptr, nb));
        MVR_TRY(launch_ratio(pl, bms, nb, S0_, img));
        MVR_TRY(launch_cols(pl, 1, 0, S0_, S0_, nullptr, nb));
        // Z: store the write planes; Y inverse: those planes only, storing the write rows
        MVR_TRY(launch_cols(pl, 2, 2, S0_, S0_, pl.k2h, nb, zlo, zhi));
        MVR_TRY(launch_cols(pl, 1, 1, S0_, S0_, nullptr, nb, ylo, yhi, zlo, zhi < 0 ? -1 : zhi));
    }
    UpdateArgs ua{};
    ua.psi_src = bps[0].psi_src;
    ua.psi_dst = bps[0].psi_dst;
    ua.weight[0] = w;
    ua.nviews = 1;
    ua.lambda = lambda_;
    ua.two_lambda = (float)(2.0 * lambda_);
    ua.tik = lambda_ > 0 ? 1 : 0;
    ua.minI = min_value_;
    ua.maxI = maxI;
    ua.partials = partials_;
    // without statistics the voxels outside the write region are not needed: the plane
    // kernels skip their planes and rows
    ua.prune = prune ? 1 : 0;
    const double nv = (double)pl.b[0] * pl.b[1] * pl.b[2];
    double bytes = 0.0;
    for (int i = 0; i < nb; ++i) {
        const BlockPlace &bp = bps[i];
        const double ez = bp.whi[2] - bp.wlo[2], ey = bp.whi[1] - bp.wlo[1];
        const double neff = (double)(bp.whi[0] - bp.wlo[0]) * ey * ez;
        if (ua.prune)
            bytes += sizeof(V) * (double)pl.Pc * ez / pl.P[2] * (pl.xy ? 1.0 : ey / pl.P[1]) +
                     (sizeof(T) + 4.0) * pl.b[0] * ey * ez + sizeof(T) * neff;
        else
            bytes += sizeof(V) * (double)pl.Pc + (sizeof(T) + 4.0) * nv + sizeof(T) * neff;
    }
    if (pl.xy) return launch_xy_update(pl, bms, nb, S0_, ua, EPI_SEQ, bytes, stats_dev);
    return launch_update(pl, bms, nb, S0_, ua, EPI_SEQ, bytes, stats_dev);
}

template <typename T>
int Engine<T>::run_mul(const std::vector<const Plan<T> *> &pls, const BlockPlace *bps, int nb,
                       const float *const *imgs, const float *const *ws, float maxI, double *stats_dev)
{
    const int nv = (int)pls.size();
    if (nv < 1 || nv > kMaxViews) return fail(ERR_ARG, "number of views must be 1..16");
    if (nb < 1 || nb > kMaxBatch) return fail(ERR_ARG, "batch of 1..16 blocks");
    UpdateArgs ua{};
    ua.psi_src = bps[0].psi_src;
    ua.psi_dst = bps[0].psi_dst;
    for (int v = 0; v < nv; ++v) ua.weight[v] = ws[v];
    ua.nviews = nv;
    ua.lambda = lambda_;
    ua.two_lambda = (float)(2.0 * lambda_);
    ua.tik = lambda_ > 0 ? 1 : 0;
    ua.minI = min_value_;
    ua.maxI = maxI;
    const Plan<T> *prev = nullptr;
    for (int v = 0; v < nv; ++v) {
        const Plan<T> &pl = *pls[v];
        if (!pl.k1h || !pl.k2h) return fail(ERR_STATE, "kernels not set for a view");
        const long long nrows = (long long)pl.P[1] * pl.P[2];
        const long long bvox = (long long)pl.b[0] * pl.b[1] * pl.b[2];
        MVR_TRY(reserve(pl.Pc, bvox, (nrows + pl.RP - 1) / pl.RP, nb));
        if (nv > 1) MVR_TRY(reserve_prod(bvox * nb));
        ua.prod = prod_;
        ua.partials = partials_;
        ua.prune = (!stats_dev && pl.xy) ? 1 : 0;
        const BlockMaps bms = block_maps(pl, bps, nb);
        if (!prev || std::memcmp(prev->P, pl.P, sizeof(pl.P)) != 0 || std::memcmp(prev->L, pl.L, sizeof(pl.L)) != 0 ||
            prev->xy != pl.xy) {
            // FFT of psi along x and y, shared by every view with this domain
            if (pl.xy) {
                MVR_TRY(launch_xy_fwd(pl, bms, nb, reinterpret_cast<const T *>(bps[0].psi_src), S0_));
            } else {
                MVR_TRY(launch_fwd_mirror(pl, bms, nb, reinterpret_cast<const T *>(bps[0].psi_src), S0_));
                MVR_TRY(launch_cols(pl, 1, 0, S0_, S0_, nullptr, nb));
            }
        }
        prev = &pl;
        int zlo = 0, zhi = -1, ylo, yhi, blo = 0, bhi = -1;
        if (pl.xy && !stats_dev) write_region(bps, nb, zlo, zhi, ylo, yhi);
        const bool band = pl.xy && !stats_dev && ratio_band(pl, zlo, zhi, blo, bhi);
        MVR_TRY(launch_cols(pl, 2, 2, S0_, S1_, pl.k1h, nb, band ? blo : 0, band ? bhi : -1));
        if (pl.xy) {
            MVR_TRY(launch_xy_ratio(pl, bms, nb, S1_, imgs[v], band ? blo : 0, band ? bhi : -1));
            MVR_TRY(launch_cols(pl, 2, 2, S1_, S1_, pl.k2h, nb, zlo, zhi, 0, -1, band ? blo : 0, band ? bhi : -1));
        } else {
            MVR_TRY(launch_cols(pl, 1, 1, S1_, S1_, nullptr, nb));
            MVR_TRY(launch_ratio(pl, bms, nb, S1_, imgs[v]));
            MVR_TRY(launch_cols(pl, 1, 0, S1_, S1_, nullptr, nb));
            MVR_TRY(launch_cols(pl, 2, 2, S1_, S1_, pl.k2h, nb));
            MVR_TRY(launch_cols(pl, 1, 1, S1_, S1_, nullptr, nb));
        }
        const double sb = (double)sizeof(V) * (double)pl.Pc;
        const double bytes = nb * (v == nv - 1 ? sb + (sizeof(T) + 12.0 + 4.0 * nv) * bvox + sizeof(T) * bvox
                                               : sb + (v == 0 ? 8.0 : 16.0) * bvox);
        const int epi = v == nv - 1 ? EPI_MUL_FINAL : (v == 0 ? EPI_MUL_FIRST : EPI_MUL_ACC);
        if (pl.xy) MVR_TRY(launch_xy_update(pl, bms, nb, S1_, ua, epi, bytes, stats_dev));
        else MVR_TRY(launch_update(pl, bms, nb, S1_, ua, epi, bytes, stats_dev));
    }
    return OK;
}

template <typename T>
int Engine<T>::likelihood(const Plan<T> &pl, const BlockPlace *bps, int nb, const float *img, const float *w,
                          double *stats_dev)
{
    if (!pl.k1h) return fail(ERR_STATE, "kernels not set for this view");
    if (nb < 1 || nb > kMaxBatch) return fail(ERR_ARG, "batch of 1..16 blocks");
    const long long nrows = (long long)pl.P[1] * pl.P[2];
    MVR_TRY(reserve(pl.Pc, (long long)pl.b[0] * pl.b[1] * pl.b[2], (nrows + pl.RP - 1) / pl.RP, nb));
    const BlockMaps bms = block_maps(pl, bps, nb);
    // plane kernels: only the write regions (each volume voxel once) are transformed back
    int zlo = 0, zhi = -1, ylo = 0, yhi = -1;
    if (pl.xy) {
        write_region(bps, nb, zlo, zhi, ylo, yhi);
        MVR_TRY(launch_xy_fwd(pl, bms, nb, reinterpret_cast<const T *>(bps[0].psi_src), S0_));
        MVR_TRY(launch_cols(pl, 2, 2, S0_, S0_, pl.k1h, nb, zlo, zhi));
    } else {
        MVR_TRY(launch_fwd_mirror(pl, bms, nb, reinterpret_cast<const T *>(bps[0].psi_src), S0_));
        MVR_TRY(launch_cols(pl, 1, 0, S0_, S0_, nullptr, nb));
        MVR_TRY(launch_cols(pl, 2, 2, S0_, S0_, pl.k1h, nb));
        MVR_TRY(launch_cols(pl, 1, 1, S0_, S0_, nullptr, nb));
    }
    UpdateArgs ua{};
    ua.prune = pl.xy ? 1 : 0;
    ua.psi_src = bps[0].psi_src;
    ua.img = img;
    ua.weight[0] = w;
    ua.nviews = 1;
    ua.partials = partials_;
    const double nv = (double)pl.b[0] * pl.b[1] * pl.b[2];
    const double bytes = nb * (sizeof(V) * (double)pl.Pc + 8.0 * nv);
    if (pl.xy) return launch_xy_update(pl, bms, nb, S0_, ua, EPI_NLL, bytes, stats_dev);
    return launch_update(pl, bms, nb, S0_, ua, EPI_NLL, bytes, stats_dev);
}

template <typename T>
int Engine<T>::convolve(const Plan<T> &pl, const T *blk, int src_kind, float *out)
{
    BlockMaps bms{};
    BlockMap &bm = bms.m[0];
    for (int d = 0; d < 3; ++d) {
        bm.P[d] = pl.P[d];
        bm.b[d] = pl.b[d];
        bm.L[d] = pl.L[d];
        bm.D[d] = pl.b[d];
        bm.OD[d] = pl.b[d];
        bm.whi[d] = pl.b[d];
    }
    bm.fast_x = block_fast_x(bm);
    if constexpr (sizeof(T) == sizeof(float)) {
        if (pl.xy) {
            ++launches_;
            if (src_kind == SRC_ZERO)
                MVR_CUDA(xy_fwd_zero(pl.xy, blk, S0_, bms, 1, pl.P[2], pl.Pc, pl.twx, pl.twy, stream_));
            else MVR_CUDA(xy_fwd_mirror(pl.xy, blk, S0_, bms, 1, pl.P[2], pl.Pc, pl.twx, pl.twy, stream_));
            MVR_TRY(launch_cols(pl, 2, 2, S0_, S0_, pl.k1h, 1));
            UpdateArgs ua{};
            ua.store = out;
            ua.partials = partials_;
            return launch_xy_update(pl, bms, 1, S0_, ua, EPI_STORE, 0.0, nullptr);
        }
    }
    const long long nrows = (long long)pl.P[1] * pl.P[2];
    const dim3 grid((unsigned)((nrows + pl.RP - 1) / pl.RP), 1);
    if (src_kind == SRC_ZERO)
        MVR_WITH_BIG(pl.big, (k_rows_fwd<T, SrcZero<T>, B><<<grid, kThreads, pl.smem_row, stream_>>>(
                                 SrcZero<T>{blk}, S0_, bms, pl.Pc, pl.dx, pl.twx, pl.RP)));
    else
        MVR_WITH_BIG(pl.big, (k_rows_fwd<T, SrcMirror<T>, B><<<grid, kThreads, pl.smem_row, stream_>>>(
                                 SrcMirror<T>{blk}, S0_, bms, pl.Pc, pl.dx, pl.twx, pl.RP)));
    MVR_LAUNCHED("k_rows_fwd(conv)");
    MVR_TRY(launch_cols(pl, 1, 0, S0_, S0_, nullptr, 1));
    MVR_TRY(launch_cols(pl, 2, 2, S0_, S0_, pl.k1h, 1));
    MVR_TRY(launch_cols(pl, 1, 1, S0_, S0_, nullptr, 1));
    UpdateArgs ua{};
    ua.store = out;
    ua.partials = partials_;
    return launch_update(pl, bms, 1, S0_, ua, EPI_STORE, 0.0, nullptr);
}

template class Engine<float>;
template class Engine<double>;

}  // namespace mvr
