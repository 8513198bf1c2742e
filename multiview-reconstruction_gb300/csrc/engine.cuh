// Host side of the block iteration: FFT plans, kernel spectra, scratch and the
// per-block Seq / Mul pipelines.  One Engine belongs to one device and one stream.
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "kernels.cuh"

namespace mvr {

enum Status { OK = 0, ERR_ARG = 1, ERR_CUDA = 2, ERR_OOM = 3, ERR_UNSUPPORTED = 4, ERR_STATE = 5 };
enum Boundary { BOUNDARY_REFERENCE = 0, BOUNDARY_CIRCULAR = 1 };
enum SrcKind { SRC_MIRROR = 0, SRC_ZERO = 1 };

// Kernel families timed by the optional profiler (CUDA events on the engine stream).
enum KernelKind {
    KK_ROWS_FWD = 0,   // extract + R2C along x
    KK_COLS_FWD,       // y forward
    KK_COLS_INV,       // y inverse
    KK_COLS_ZMUL,      // z forward, spectral multiply, z inverse
    KK_ROWS_RATIO,     // C2R, quotient, R2C
    KK_ROWS_UPDATE,    // C2R, update, stats partials
    KK_REDUCE,         // stats reduction
    KK_PASTE,          // effective-region copy
    KK_XY_FWD,         // plane: extract + R2C along x + FFT along y
    KK_XY_RATIO,       // plane: inverse y, C2R, quotient, R2C, FFT y
    KK_XY_UPDATE,      // plane: inverse y, C2R, update, stats partials
    KK_COUNT
};
const char *kernel_kind_name(int k);

struct KernelProfile {
    double ms[KK_COUNT];
    long long launches[KK_COUNT];
    double bytes[KK_COUNT];  // algorithmic bytes moved by those launches
};

bool fft_friendly(long long n);
long long next_friendly_even(long long n);
FftDesc make_desc(int n);

// FFT domain of one (block size, kernel size) pair and the spectra of its kernels.
template <typename T>
struct Plan {
    typedef typename Cx<T>::t V;
    int b[3] = {0, 0, 0};
    int kd[3] = {0, 0, 0};
    int P[3] = {0, 0, 0};
    int L[3] = {0, 0, 0};
    int Hx = 0;
    long long Pc = 0;
    FftDesc dx{}, dy{}, dz{};
    V *twx = nullptr, *twy = nullptr, *twz = nullptr;
    V *k1h = nullptr, *k2h = nullptr;
    int RP = 1, NPy = 1, NPz = 1;
    bool big = false;  // some axis needs radix 7, 11 or 13
    int wr = 0;        // FP32 rows of Px = 64 wr reals (wr = 2, 3, 4) take the warp-shuffle row kernels
    int wcy = 0, wcz = 0;  // FP32 columns of 32 wc (wc = 2, 3, 4, 5, 6, 8) take the warp-shuffle column kernels
    int tcy = 0, tcz = 0;  // FP32 columns of 16 tc (tc = 4, 6, 8, 12, 16, 18) take the two-phase tile kernels (preferred)
    int xy = 0;            // plane kernels (x and y fused per z-plane): shape code, 0 = row / column kernels
    size_t smem_row = 0, smem_coly = 0, smem_colz = 0;
    // FFT schedule (chosen by the autotuner of the whole-volume driver, or forced):
    int xy_cap = 0;        // the plane-kernel shape this domain allows (0: none)
    int pair_cap = 0;      // the pair-kernel shape (two CTAs per plane) this domain allows (0: none)
    int persist = 1;       // plane kernels: forward / quotient passes as one CTA per SM walking the planes
                           // (1) or one CTA per plane (0)
    int zpipe = -1;        // Z pass of the tile column kernels: persistent double-buffered (1), one tile per
                           // CTA (0), or -1: the built-in choice (persistent for 256-long columns only)
    int kspec_xy = 0;      // the path (plane shape or 0) K1^ / K2^ were computed with
    const float *ksrc1 = nullptr, *ksrc2 = nullptr;  // device kernels (whole-volume driver), for recomputing K^
};

// FFT schedule codes (Engine::schedule_candidates / set_schedule):
//   path: 0 row / column kernels, 1 plane kernels one CTA per plane, 2 plane kernels persistent;
//   + 4 when the Z pass of the convolutions uses the persistent double-buffered column kernel.
//   path 3: the pair kernels (a cluster of two CTAs per plane, persistent).
enum { SCHED_ROWS = 0, SCHED_PLANE = 1, SCHED_PLANE_PERSIST = 2, SCHED_PAIR = 3, SCHED_ZPIPE = 4 };

// Where the block's output goes (volume driver) or the block itself (block API).
struct BlockPlace {
    const void *psi_src = nullptr;  // T volume (mirror-single read)
    long long D[3] = {0, 0, 0};     // its dims
    long long off[3] = {0, 0, 0};   // block offset
    void *psi_dst = nullptr;        // T output volume
    long long OD[3] = {0, 0, 0};
    long long ooff[3] = {0, 0, 0};  // volume coordinate of block-local origin in the output
    int wlo[3] = {0, 0, 0}, whi[3] = {0, 0, 0};
};

template <typename T>
class Engine {
public:
    typedef typename Cx<T>::t V;
    Engine() = default;
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    // Binds the engine to a device and creates its stream.
    int init(int device, int boundary, double lambda, float min_value);
    // Plan for (block b, kernel kd); k1/k2 are host arrays (k2 may be null). Kernel
    // spectra are computed on the device.
    int make_plan(Plan<T> &pl, const int b[3], const float *k1, const int kd1[3], const float *k2,
                  const int kd2[3], bool k_on_device = false);
    void free_plan(Plan<T> &pl);
    // The FFT schedules a plan admits (codes SCHED_*), and the one in use.
    int kernel_spectra(Plan<T> &pl, const float *k1, const float *k2, bool k_on_device);
    std::vector<int> schedule_candidates(const Plan<T> &pl) const;
    int schedule(const Plan<T> &pl) const;
    int set_schedule(Plan<T> &pl, int code);

    // One sequential iteration (ComputeBlockSeqThread.runIteration) of view plan pl on
    // nb (1..16) blocks in one batched launch per pass; all blocks read the same psi
    // source and write the same output volume.  stats_dev: 2 doubles per block.
    int run_seq(const Plan<T> &pl, const BlockPlace *bps, int nb, const float *img, const float *w, float maxI,
                double *stats_dev);
    // One multiplicative iteration over views (ComputeBlockMulThread.runIteration).
    int run_mul(const std::vector<const Plan<T> *> &pls, const BlockPlace *bps, int nb, const float *const *imgs,
                const float *const *ws, float maxI, double *stats_dev);
    // Poisson negative log-likelihood of psi under view pl: per block (stats_dev, 2
    // doubles each, [0] = sum) the FP64 sum over the block's write region of
    // w * (conv1 - img ln conv1) where img > 0.
    int likelihood(const Plan<T> &pl, const BlockPlace *bps, int nb, const float *img, const float *w,
                   double *stats_dev);
    // Linear convolution of a T block (mirror or zero extension) with pl's k1, result
    // to a float block of the same size.
    int convolve(const Plan<T> &pl, const T *blk, int src_kind, float *out);

    cudaStream_t stream() const { return stream_; }
    // launch accounting: every kernel launch of the engine (and of its owner through
    // count_launch) is counted; with profiling on, each is bracketed by CUDA events
    long long launches() const { return launches_; }
    // adds launches replayed from a captured graph to the count
    void count_replayed(long long n) { launches_ += n; }
    // changes whenever the engine's scratch buffers are reallocated (captured graphs
    // that use them are then stale)
    long long alloc_epoch() const { return alloc_epoch_; }
    bool profiling() const { return prof_on_; }
    void set_profiling(bool on) { prof_on_ = on; }
    int prof_begin(int kind, double bytes);
    int prof_end();
    int profile_collect(KernelProfile &out);  // synchronises, then adds the pending times
    int device() const { return device_; }
    const std::string &error() const { return err_; }
    int fail(int code, const std::string &msg);
    int cuda_check(cudaError_t e, const char *what);
    int reserve(long long Pc, long long nvox_block, long long rows, int nb);
    int reserve_prod(long long n);

private:
    int launch_fwd_mirror(const Plan<T> &pl, const BlockMaps &bms, int nb, const T *src, V *S);
    int launch_xy_fwd(const Plan<T> &pl, const BlockMaps &bms, int nb, const T *src, V *S);
    // the quotient pass over the planes [zlo, zhi) of each block (zhi < 0: all)
    int launch_xy_ratio(const Plan<T> &pl, const BlockMaps &bms, int nb, V *S, const float *img, int zlo = 0,
                        int zhi = -1);
    int launch_xy_update(const Plan<T> &pl, const BlockMaps &bms, int nb, V *S, const UpdateArgs &ua, int epi,
                         double bytes, double *stats_dev);
    // rows [rlo, rhi) of the transformed axis are stored, and only the other-axis indices
    // [olo, ohi) are transformed (negative hi: all; tile kernels only, the others do all);
    // the input rows outside [llo, lhi) are taken as zeros without being read (tile kernels)
    int launch_cols(const Plan<T> &pl, int axis, int mode, const V *src, V *dst, const V *Kh, int nb, int rlo = 0,
                    int rhi = -1, int olo = 0, int ohi = -1, int llo = 0, int lhi = -1);
    // the planes [lo, hi) that the second convolution reads for a write region [zlo, zhi) (its
    // kernel's reach either side); false when pruning does not apply (lo = 0, hi = P)
    bool ratio_band(const Plan<T> &pl, int zlo, int zhi, int &lo, int &hi) const;
    int launch_ratio(const Plan<T> &pl, const BlockMaps &bms, int nb, V *S, const float *img);
    int launch_update(const Plan<T> &pl, const BlockMaps &bms, int nb, V *S, const UpdateArgs &ua, int epi,
                      double bytes, double *stats_dev);
    BlockMaps block_maps(const Plan<T> &pl, const BlockPlace *bps, int nb) const;

    int device_ = -1;
    int boundary_ = BOUNDARY_REFERENCE;
    double lambda_ = 0.0;
    float min_value_ = 1e-4f;
    cudaStream_t stream_ = nullptr;
    V *S0_ = nullptr, *S1_ = nullptr;
    long long Scap_ = 0;
    double *prod_ = nullptr;
    long long prodcap_ = 0;
    double *partials_ = nullptr;
    long long partcap_ = 0;
    float *kbuf_ = nullptr;
    long long kcap_ = 0;
    std::string err_;
    long long launches_ = 0;
    long long alloc_epoch_ = 0;
    bool prof_on_ = false;
    struct Pending {
        int kind;
        double bytes;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending_;
    std::vector<cudaEvent_t> event_pool_;
    KernelProfile acc_{};
};

extern template class Engine<float>;
extern template class Engine<double>;

}  // namespace mvr
