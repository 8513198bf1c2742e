// Device FFT engine: mixed-radix Stockham autosort transforms of many pencils held
// in shared memory, ping-ponging between two buffers (one barrier per stage).
//
// A stage of radix R with Ns = product of the previous radices maps butterfly j
// (0 <= j < n/R) of pencil p as (Stockham autosort, Govindaraju et al., SC08):
//   inputs   a[j + r*n/R],  r = 0..R-1, twiddled by exp(-+2 pi i r k / (Ns R)), k = j mod Ns
//   outputs  b[(j / Ns) * Ns * R + k + r*Ns] = R-point DFT of the inputs
// which leaves the result in natural order after the last stage.
//
// Element (p, i) of the pencil set lives at s[p*ps + i*es]: rows use ps = n+pad,
// es = 1 and a j-fastest thread mapping; column tiles use ps = 1, es = NP and a
// p-fastest mapping so that a warp touches consecutive words.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mvr {

constexpr int kMaxStages = 24;

// Stage list of one transform length, passed by value in kernel parameters.  For
// stage s: radix[s], Ns[s] = product of the previous radices, twstep[s] = n / (Ns R),
// and exact reciprocals for division by Ns[s] and by n / radix[s] of any index below
// 2^16 (q = umulhi(j, magic) with magic = ceil(2^32 / divisor)).
struct FftDesc {
    int n;
    int ns;
    int radix[kMaxStages];
    int Ns[kMaxStages];
    int twstep[kMaxStages];
    unsigned ns_magic[kMaxStages];
    unsigned nb_magic[kMaxStages];
};

template <typename T> struct Cx;
template <> struct Cx<float> { typedef float2 t; };
template <> struct Cx<double> { typedef double2 t; };

template <typename V> struct Re;
template <> struct Re<float2> { typedef float t; };
template <> struct Re<double2> { typedef double t; };

template <typename V>
__device__ __forceinline__ V cx(typename Re<V>::t a, typename Re<V>::t b) { V r; r.x = a; r.y = b; return r; }
template <typename V> __device__ __forceinline__ V cadd(V a, V b) { return cx<V>(a.x + b.x, a.y + b.y); }
template <typename V> __device__ __forceinline__ V csub(V a, V b) { return cx<V>(a.x - b.x, a.y - b.y); }
template <typename V> __device__ __forceinline__ V cscale(V a, typename Re<V>::t s) { return cx<V>(a.x * s, a.y * s); }
template <typename V> __device__ __forceinline__ V cconj(V a) { return cx<V>(a.x, -a.y); }
template <typename V>
__device__ __forceinline__ V cmul(V a, V b) { return cx<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename V>
__device__ __forceinline__ V mul_j(V a) { return INV ? cx<V>(-a.y, a.x) : cx<V>(a.y, -a.x); }

// FP32 complex additions and real scalings on the paired FP32 instructions of sm_100 and
// later (one instruction for both components, rounded to nearest like the scalar ones).
// MVR_PAIRED_FP=0 keeps the scalar forms.
#ifndef MVR_PAIRED_FP
#define MVR_PAIRED_FP 1
#endif
#if MVR_PAIRED_FP && defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) { return __fadd2_rn(a, b); }
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b)
{
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
}
template <> __device__ __forceinline__ float2 cscale<float2>(float2 a, float s)
{
    return __fmul2_rn(a, make_float2(s, s));
}
// a - s b with one fused paired instruction
__device__ __forceinline__ float2 csub_scaled(float2 a, float2 b, float s)
{
    return __ffma2_rn(b, make_float2(-s, -s), a);
}
#endif
template <typename V>
__device__ __forceinline__ V csub_scaled(V a, V b, typename Re<V>::t s) { return csub(a, cscale(b, s)); }

// t +- (-+i) d component-wise (the rotated operand never forms a swizzled pair):
// returns t + mul_j(d) in p and t - mul_j(d) in q
template <bool INV, typename V>
__device__ __forceinline__ void add_sub_j(V t, V d, V &p, V &q)
{
    if (INV) {
        p = cx<V>(t.x - d.y, t.y + d.x);
        q = cx<V>(t.x + d.y, t.y - d.x);
    } else {
        p = cx<V>(t.x + d.y, t.y - d.x);
        q = cx<V>(t.x - d.y, t.y + d.x);
    }
}

// ---- small DFTs (constants are the exact roots of unity of each radix) -------------
template <bool INV, typename V> __device__ __forceinline__ void dft2(V *v)
{
    V a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}

template <bool INV, typename V> __device__ __forceinline__ void dft3(V *v)
{
    typedef typename Re<V>::t T;
    const T s3 = (T)0.86602540378443864676;  // sin(2 pi / 3)
    V t1 = cadd(v[1], v[2]);
    V m = csub_scaled(v[0], t1, (T)0.5);
    V e = csub(v[1], v[2]);
    v[0] = cadd(v[0], t1);
    // m +- s3 mul_j(e), component-wise
    if (INV) {
        v[1] = cx<V>(m.x - s3 * e.y, m.y + s3 * e.x);
        v[2] = cx<V>(m.x + s3 * e.y, m.y - s3 * e.x);
    } else {
        v[1] = cx<V>(m.x + s3 * e.y, m.y - s3 * e.x);
        v[2] = cx<V>(m.x - s3 * e.y, m.y + s3 * e.x);
    }
}

template <bool INV, typename V> __device__ __forceinline__ void dft4(V *v)
{
    V t0 = cadd(v[0], v[2]), t1 = csub(v[0], v[2]);
    V t2 = cadd(v[1], v[3]), d = csub(v[1], v[3]);
    v[0] = cadd(t0, t2);
    v[2] = csub(t0, t2);
    add_sub_j<INV>(t1, d, v[1], v[3]);
}

template <bool INV, typename V> __device__ __forceinline__ void dft5(V *v)
{
    typedef typename Re<V>::t T;
    const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;   // cos 2pi/5, cos 4pi/5
    const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;    // sin 2pi/5, sin 4pi/5
    V a1 = cadd(v[1], v[4]), a2 = cadd(v[2], v[3]);
    V b1 = csub(v[1], v[4]), b2 = csub(v[2], v[3]);
    V m1 = cadd(v[0], cadd(cscale(a1, c1), cscale(a2, c2)));
    V m2 = cadd(v[0], cadd(cscale(a1, c2), cscale(a2, c1)));
    V n1 = mul_j<INV>(cadd(cscale(b1, s1), cscale(b2, s2)));
    V n2 = mul_j<INV>(csub(cscale(b1, s2), cscale(b2, s1)));
    v[0] = cadd(v[0], cadd(a1, a2));
    v[1] = cadd(m1, n1);
    v[4] = csub(m1, n1);
    v[2] = cadd(m2, n2);
    v[3] = csub(m2, n2);
}

template <bool INV, typename V> __device__ __forceinline__ void dft8(V *v)
{
    typedef typename Re<V>::t T;
    const T r = (T)0.70710678118654752440;  // 1/sqrt(2)
    V a[4], b[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) { a[j] = cadd(v[j], v[j + 4]); b[j] = csub(v[j], v[j + 4]); }
    // b_j *= exp(-+2 pi i j / 8)
    if (INV) {
        b[1] = cx<V>((b[1].x - b[1].y) * r, (b[1].x + b[1].y) * r);
        b[3] = cx<V>((-b[3].x - b[3].y) * r, (b[3].x - b[3].y) * r);
    } else {
        b[1] = cx<V>((b[1].x + b[1].y) * r, (b[1].y - b[1].x) * r);
        b[3] = cx<V>((b[3].y - b[3].x) * r, (-b[3].x - b[3].y) * r);
    }
    b[2] = mul_j<INV>(b[2]);
    dft4<INV>(a);
    dft4<INV>(b);
#pragma unroll
    for (int m = 0; m < 4; ++m) { v[2 * m] = a[m]; v[2 * m + 1] = b[m]; }
}

// Generic odd prime radix from the length-n twiddle table (table[t*twmul] = exp(-2 pi i t / n)).
template <int R, bool INV, typename V>
__device__ __forceinline__ void dftg(V *v, const V *tw, int n, int twmul)
{
    V o[R];
    const int step = (n / R) * twmul;
#pragma unroll
    for (int u = 0; u < R; ++u) {
        V acc = v[0];
#pragma unroll
        for (int q = 1; q < R; ++q) {
            V w = tw[((q * u) % R) * step];
            if (INV) w.y = -w.y;
            acc = cadd(acc, cmul(v[q], w));
        }
        o[u] = acc;
    }
#pragma unroll
    for (int u = 0; u < R; ++u) v[u] = o[u];
}

template <int R, bool INV, typename V>
__device__ __forceinline__ void dft(V *v, const V *tw, int n, int twmul)
{
    if (R == 2) dft2<INV>(v);
    else if (R == 3) dft3<INV>(v);
    else if (R == 4) dft4<INV>(v);
    else if (R == 5) dft5<INV>(v);
    else if (R == 8) dft8<INV>(v);
    else dftg<R, INV>(v, tw, n, twmul);
}

// One butterfly of one stage: group q = j / Ns, position k = j mod Ns.
template <int R, bool INV, typename V>
__device__ __forceinline__ void stage_bfly(const V *__restrict__ src, V *__restrict__ dst, int p, int j, int q, int k,
                                           int Ns, int n, int twstep, int ps, int es, const V *__restrict__ tw,
                                           int twmul)
{
    const int nR = n / R;
    V v[R];
    const V *s = src + p * ps;
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = s[(j + r * nR) * es];
    if (Ns > 1) {
        const int step = k * twstep * twmul;
#pragma unroll
        for (int r = 1; r < R; ++r) {
            V w = tw[r * step];
            if (INV) w.y = -w.y;
            v[r] = cmul(v[r], w);
        }
    }
    dft<R, INV>(v, tw, n, twmul);
    const int idxD = q * Ns * R + k;
    V *d = dst + p * ps;
#pragma unroll
    for (int r = 0; r < R; ++r) d[(idxD + r * Ns) * es] = v[r];
}

// All butterflies of stage s on npen pencils, without integer division.
template <int R, bool INV, bool PFAST, typename V>
__device__ __forceinline__ void stage_loop(const V *__restrict__ a, V *__restrict__ b, int npen, int ps, int es,
                                           const FftDesc &d, int s, const V *__restrict__ tw, int twmul)
{
    const int nb = d.n / R;
    const int total = nb * npen;
    const int Ns = d.Ns[s];
    const int twstep = d.twstep[s];
    const unsigned nsm = d.ns_magic[s];
    if (PFAST) {  // npen is a power of two
        const int lg = __ffs(npen) - 1;
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int p = t & (npen - 1);
            const int j = t >> lg;
            const int q = Ns == 1 ? j : (int)__umulhi((unsigned)j, nsm);
            stage_bfly<R, INV>(a, b, p, j, q, j - q * Ns, Ns, d.n, twstep, ps, es, tw, twmul);
        }
    } else {
        const unsigned nbm = d.nb_magic[s];
        for (int t = threadIdx.x; t < total; t += blockDim.x) {
            const int p = nb == 1 ? t : (int)__umulhi((unsigned)t, nbm);
            const int j = t - p * nb;
            const int q = Ns == 1 ? j : (int)__umulhi((unsigned)j, nsm);
            stage_bfly<R, INV>(a, b, p, j, q, j - q * Ns, Ns, d.n, twstep, ps, es, tw, twmul);
        }
    }
}

// Run all stages on npen pencils.  Input in a (synchronised by the caller); returns
// the buffer that holds the result (a or b).  PFAST: thread index runs over pencils
// first (column tiles, npen a power of two), else over butterflies first (rows).
// BIG: the stage list may contain radix 7, 11 or 13 (generic DFT, many registers);
// otherwise only 2, 3, 4, 5, 8 occur and the kernel stays lean.
template <bool INV, bool PFAST, bool BIG, typename V>
__device__ V *fft_run(V *a, V *b, int npen, int ps, int es, const FftDesc &d, const V *__restrict__ tw,
                      int twmul)
{
    for (int s = 0; s < d.ns; ++s) {
        switch (d.radix[s]) {
        case 2: stage_loop<2, INV, PFAST>(a, b, npen, ps, es, d, s, tw, twmul); break;
        case 3: stage_loop<3, INV, PFAST>(a, b, npen, ps, es, d, s, tw, twmul); break;
        case 4: stage_loop<4, INV, PFAST>(a, b, npen, ps, es, d, s, tw, twmul); break;
        case 5: stage_loop<5, INV, PFAST>(a, b, npen, ps, es, d, s, tw, twmul); break;
        case 8: stage_loop<8, INV, PFAST>(a, b, npen, ps, es, d, s, tw, twmul); break;
        default:
            if (BIG) {
                if (d.radix[s] == 7) stage_loop<7, INV, PFAST>(a, b, npen, ps, es, d, s, tw, twmul);
                else if (d.radix[s] == 11) stage_loop<11, INV, PFAST>(a, b, npen, ps, es, d, s, tw, twmul);
                else stage_loop<13, INV, PFAST>(a, b, npen, ps, es, d, s, tw, twmul);
            }
            break;
        }
        __syncthreads();
        V *t = a;
        a = b;
        b = t;
    }
    return a;
}

}  // namespace mvr
