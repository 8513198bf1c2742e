/*
 * mvr_oracle.c -- CPU restatement of the multiview Bayesian (Richardson-Lucy type)
 * deconvolution block iteration of PreibischLab/multiview-reconstruction.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA path and the
 * timed CPU baseline; the product library never links, loads or calls it.
 *
 * Parity status: UNPINNED by the reference.  The reference is Java (no JVM in this
 * build environment, Maven dependencies need the network) and ships no tests, no
 * golden vectors and no fixtures for deconvolution.  This restatement is pinned
 * instead by (a) an independent numpy restatement of the same semantics
 * (tests/golden/make_golden.py, committed fixtures), (b) direct spatial
 * convolution for small kernels and (c) analytic known-answer cases
 * (delta PSF, constant-image fixed point, Seq==Mul for one view).
 *
 * Two numeric modes:
 *   fp64 == 0  "reference-faithful FP32": every value the Java code stores in a
 *              FloatType is rounded to float at the same place, the update runs in
 *              float arithmetic exactly as DeconvolutionMethods does (no FMA
 *              contraction: build with -ffp-contract=off), stats in double.  The
 *              FFT convolution itself is computed in double and rounded once
 *              (the reference's float FFT differs from it by O(1e-7) relative).
 *   fp64 == 1  every stage in double: the FP64 run of the same iteration that GPU
 *              results state their error against.
 *
 * Reference files are cited relative to src/main/java/ of the reference project:
 *   DM  = net/preibisch/mvrecon/process/deconvolution/iteration/sequential/DeconvolutionMethods.java
 *   FFC = util/FFTConvolution.java
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

/* ------------------------------------------------------------------------- */
/* Mixed-radix complex FFT (recursive decimation in time), any length >= 1.   */
/* ------------------------------------------------------------------------- */

typedef struct {
    int n;
    int nf;
    int fac[64];
    cplx *tw; /* tw[k] = exp(-2 pi i k / n) */
} orc_fftplan;

static void plan_init(orc_fftplan *p, int n)
{
    p->n = n;
    p->nf = 0;
    int m = n;
    while (m % 4 == 0) { p->fac[p->nf++] = 4; m /= 4; }
    while (m % 2 == 0) { p->fac[p->nf++] = 2; m /= 2; }
    for (int f = 3; m > 1; f += 2) {
        while (m % f == 0) { p->fac[p->nf++] = f; m /= f; }
        if (f * f > m && m > 1) { p->fac[p->nf++] = m; m = 1; }
    }
    if (p->nf == 0) p->fac[p->nf++] = 1;
    p->tw = (cplx *)malloc(sizeof(cplx) * (size_t)(n > 0 ? n : 1));
    for (int k = 0; k < n; ++k) {
        double a = -2.0 * M_PI * (double)k / (double)n;
        p->tw[k] = cos(a) + I * sin(a);
    }
}

static void plan_free(orc_fftplan *p) { free(p->tw); p->tw = NULL; }

static inline cplx twv(const orc_fftplan *p, long idx, int sign)
{
    cplx w = p->tw[idx % p->n];
    return sign < 0 ? w : conj(w);
}

/* out (contiguous, length n) = DFT of in[0], in[s], ..., in[(n-1)s].
 * sign -1: forward exp(-2 pi i ...), +1: unnormalised inverse. */
static void fft_rec(cplx *out, const cplx *in, int n, long s, const int *fac,
                    const orc_fftplan *p, long twstep, int sign, cplx *scr)
{
    const int r = fac[0];
    const int m = n / r;
    if (m == 1) {
        for (int q = 0; q < r; ++q) out[q] = in[q * s];
    } else {
        for (int q = 0; q < r; ++q)
            fft_rec(out + (long)q * m, in + q * s, m, s * r, fac + 1, p, twstep * r, sign, scr);
    }
    if (r == 1) return;
    if (r == 2) {
        for (int k = 0; k < m; ++k) {
            cplx a = out[k];
            cplx b = out[k + m] * twv(p, (long)k * twstep, sign);
            out[k] = a + b;
            out[k + m] = a - b;
        }
        return;
    }
    if (r == 4) {
        const cplx jj = sign < 0 ? -I : I; /* exp(sign * i pi / 2) */
        for (int k = 0; k < m; ++k) {
            cplx a0 = out[k];
            cplx a1 = out[k + m] * twv(p, (long)k * twstep, sign);
            cplx a2 = out[k + 2 * m] * twv(p, 2L * k * twstep, sign);
            cplx a3 = out[k + 3 * m] * twv(p, 3L * k * twstep, sign);
            cplx t0 = a0 + a2, t1 = a0 - a2, t2 = a1 + a3, t3 = (a1 - a3) * jj;
            out[k] = t0 + t2;
            out[k + m] = t1 + t3;
            out[k + 2 * m] = t0 - t2;
            out[k + 3 * m] = t1 - t3;
        }
        return;
    }
    /* generic radix r: W_r = W_n^{twstep * m} over the full-length table */
    const long wr = twstep * m;
    for (int k = 0; k < m; ++k) {
        for (int q = 0; q < r; ++q)
            scr[q] = out[k + (long)q * m] * twv(p, (long)q * k * twstep, sign);
        for (int u = 0; u < r; ++u) {
            cplx acc = 0;
            for (int q = 0; q < r; ++q)
                acc += scr[q] * twv(p, (long)((q * u) % r) * wr, sign);
            out[k + (long)u * m] = acc;
        }
    }
}

static int max_factor(const orc_fftplan *p)
{
    int mx = 1;
    for (int i = 0; i < p->nf; ++i) if (p->fac[i] > mx) mx = p->fac[i];
    return mx;
}

/* In-place 3D complex FFT of a[z][y][x] (dims P[0]=x, P[1]=y, P[2]=z). */
static void fft3d(cplx *a, const int P[3], int sign)
{
    const long px = P[0], py = P[1], pz = P[2];
    for (int ax = 0; ax < 3; ++ax) {
        orc_fftplan pl;
        plan_init(&pl, P[ax]);
        const int n = P[ax];
        const long stride = ax == 0 ? 1 : (ax == 1 ? px : px * py);
        const long npencil = (px * py * pz) / n;
        const int mf = max_factor(&pl);
#pragma omp parallel
        {
            cplx *tmp = (cplx *)malloc(sizeof(cplx) * (size_t)n);
            cplx *scr = (cplx *)malloc(sizeof(cplx) * (size_t)mf);
#pragma omp for schedule(static)
            for (long q = 0; q < npencil; ++q) {
                long base;
                if (ax == 0) base = q * px;
                else if (ax == 1) base = (q / px) * px * py + (q % px);
                else base = q;
                fft_rec(tmp, a + base, n, stride, pl.fac, &pl, 1, sign, scr);
                for (int i = 0; i < n; ++i) a[base + (long)i * stride] = tmp[i];
            }
            free(tmp);
            free(scr);
        }
        plan_free(&pl);
    }
}

/* Public 1D FFT (for tests): in/out interleaved re,im doubles. */
void orc_fft1d(double *data, int n, int inverse)
{
    orc_fftplan pl;
    plan_init(&pl, n);
    cplx *in = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    cplx *out = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    cplx *scr = (cplx *)malloc(sizeof(cplx) * (size_t)max_factor(&pl));
    for (int i = 0; i < n; ++i) in[i] = data[2 * i] + I * data[2 * i + 1];
    fft_rec(out, in, n, 1, pl.fac, &pl, 1, inverse ? 1 : -1, scr);
    for (int i = 0; i < n; ++i) { data[2 * i] = creal(out[i]); data[2 * i + 1] = cimag(out[i]); }
    free(in); free(out); free(scr);
    plan_free(&pl);
}

/* ------------------------------------------------------------------------- */
/* Extensions and linear convolution                                          */
/* ------------------------------------------------------------------------- */

enum { ORC_EXT_ZERO = 0, ORC_EXT_MIRROR_SINGLE = 1, ORC_EXT_VALUE = 2 };

/* imglib2 Views.extendMirrorSingle: the border voxel is not repeated, period 2n-2. */
long orc_mirror_single(long i, long n)
{
    if (n <= 1) return 0;
    const long p = 2 * n - 2;
    i %= p;
    if (i < 0) i += p;
    return i >= n ? p - i : i;
}

/* Kernel spectrum on a P domain: Kp[(t - k/2) mod P] = K[t] (kernel centre at the
 * origin via periodic wrap), FFC computeKernelFFT 560-582 with setupFFTs 537-541. */
static cplx *kernel_spectrum(const float *k, const int kd[3], const int P[3])
{
    const long px = P[0], py = P[1], pz = P[2];
    cplx *a = (cplx *)calloc((size_t)(px * py * pz), sizeof(cplx));
    for (int z = 0; z < kd[2]; ++z)
        for (int y = 0; y < kd[1]; ++y)
            for (int x = 0; x < kd[0]; ++x) {
                long X = ((x - kd[0] / 2) % px + px) % px;
                long Y = ((y - kd[1] / 2) % py + py) % py;
                long Z = ((z - kd[2] / 2) % pz + pz) % pz;
                a[(Z * py + Y) * px + X] += (double)k[((long)z * kd[1] + y) * kd[0] + x];
            }
    fft3d(a, P, -1);
    return a;
}

/* Linear convolution of the extended block with a kernel whose centre is index
 * kd/2, output over the block: FFC convolve 490-506 / setupFFTs 508-544 /
 * computeConvolution 584-603.  The padded domain is P = b + k - 1 per axis with the
 * block at the origin, `c = k/2` extension voxels after it and `k-1-c` wrapped
 * before it; any padded size >= b + k - 1 gives the same linear convolution, which
 * is why the reference's "fast" FFT size is irrelevant to the result. */
static void convolve_ext(const double *in, const int b[3], int ext_mode, double ext_value,
                         const float *k, const int kd[3], const cplx *khat_opt, double *out)
{
    int P[3];
    for (int d = 0; d < 3; ++d) P[d] = b[d] + kd[d] - 1;
    const long px = P[0], py = P[1], pz = P[2];
    const long bx = b[0], by = b[1], bz = b[2];
    cplx *a = (cplx *)malloc(sizeof(cplx) * (size_t)(px * py * pz));
    const int R[3] = {kd[0] / 2, kd[1] / 2, kd[2] / 2};
#pragma omp parallel for schedule(static)
    for (long Z = 0; Z < pz; ++Z)
        for (long Y = 0; Y < py; ++Y)
            for (long X = 0; X < px; ++X) {
                long c[3] = {X, Y, Z};
                const long bb[3] = {bx, by, bz};
                int inside = 1;
                for (int d = 0; d < 3; ++d) {
                    if (c[d] >= bb[d] + R[d]) c[d] -= P[d]; /* wrapped left extension */
                    if (c[d] < 0 || c[d] >= bb[d]) inside = 0;
                }
                double v;
                if (inside) v = in[(c[2] * by + c[1]) * bx + c[0]];
                else if (ext_mode == ORC_EXT_MIRROR_SINGLE) {
                    long mx = orc_mirror_single(c[0], bx), my = orc_mirror_single(c[1], by),
                         mz = orc_mirror_single(c[2], bz);
                    v = in[(mz * by + my) * bx + mx];
                } else if (ext_mode == ORC_EXT_VALUE) v = ext_value;
                else v = 0.0;
                a[(Z * py + Y) * px + X] = v;
            }
    fft3d(a, P, -1);
    cplx *kh = khat_opt ? (cplx *)khat_opt : kernel_spectrum(k, kd, P);
    const long np = px * py * pz;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < np; ++i) a[i] *= kh[i];
    if (!khat_opt) free(kh);
    fft3d(a, P, +1);
    const double s = 1.0 / (double)np;
#pragma omp parallel for schedule(static)
    for (long z = 0; z < bz; ++z)
        for (long y = 0; y < by; ++y)
            for (long x = 0; x < bx; ++x)
                out[(z * by + y) * bx + x] = creal(a[(z * py + y) * px + x]) * s;
    free(a);
}

/* Public: conv of a float block, result in double (tests) */
void orc_convolve(const float *in, const int b[3], int ext_mode, double ext_value,
                  const float *k, const int kd[3], double *out)
{
    const long n = (long)b[0] * b[1] * b[2];
    double *d = (double *)malloc(sizeof(double) * (size_t)n);
    for (long i = 0; i < n; ++i) d[i] = in[i];
    convolve_ext(d, b, ext_mode, ext_value, k, kd, NULL, out);
    free(d);
}

/* ------------------------------------------------------------------------- */
/* Pointwise update rules (DM)                                                */
/* ------------------------------------------------------------------------- */

/* DM tikhonov 421 */
static inline double tikhonov(double value, double lambda)
{
    return (sqrt(1.0 + 2.0 * lambda * value) - 1.0) / lambda;
}

/* DM computeNextValue 320-358, float arithmetic exactly as Java evaluates it. */
static inline float next_value_f32(float last, float integral, float weight, double lambda,
                                   float minI, float maxI)
{
    const float value = last * integral;
    float adjusted;
    if (value > 0) {
        if (lambda > 0) adjusted = (float)tikhonov((double)(value / maxI), lambda) * maxI;
        else adjusted = value;
    } else adjusted = minI;
    float next;
    if (isnan(adjusted)) next = minI;
    else next = (minI >= adjusted) ? minI : adjusted; /* Math.max(float, float), no NaN here */
    return last + ((next - last) * weight);
}

/* The same rule in double (FP64 run). */
static inline double next_value_f64(double last, double integral, double weight, double lambda,
                                    double minI, double maxI)
{
    const double value = last * integral;
    double adjusted;
    if (value > 0) adjusted = lambda > 0 ? tikhonov(value / maxI, lambda) * maxI : value;
    else adjusted = minI;
    double next = isnan(adjusted) ? minI : (minI >= adjusted ? minI : adjusted);
    return last + (next - last) * weight;
}

/* DM computeNextValueMul 370-419: product and pow in double, sumW capped at 1. */
static inline float next_value_mul_f32(float last, const float *integral, const float *weight,
                                       int nv, double lambda, float minI, float maxI)
{
    double sumW = 0, prod = 1;
    for (int i = 0; i < nv; ++i) { prod *= (double)integral[i]; sumW += (double)weight[i]; }
    prod = pow(prod, 1.0 / nv);
    sumW = sumW < 1.0 ? sumW : 1.0;
    const float value = last * (float)prod;
    float adjusted;
    if (value > 0) {
        if (lambda > 0) adjusted = (float)tikhonov((double)(value / maxI), lambda) * maxI;
        else adjusted = value;
    } else adjusted = minI;
    float next;
    if (isnan(adjusted)) next = minI;
    else next = (minI >= adjusted) ? minI : adjusted;
    return last + ((next - last) * (float)sumW);
}

static inline double next_value_mul_f64(double last, const double *integral, const double *weight,
                                        int nv, double lambda, double minI, double maxI)
{
    double sumW = 0, prod = 1;
    for (int i = 0; i < nv; ++i) { prod *= integral[i]; sumW += weight[i]; }
    prod = pow(prod, 1.0 / nv);
    sumW = sumW < 1.0 ? sumW : 1.0;
    const double value = last * prod;
    double adjusted;
    if (value > 0) adjusted = lambda > 0 ? tikhonov(value / maxI, lambda) * maxI : value;
    else adjusted = minI;
    double next = isnan(adjusted) ? minI : (minI >= adjusted ? minI : adjusted);
    return last + (next - last) * sumW;
}

/* ------------------------------------------------------------------------- */
/* Kernel-spectrum cache (DeconViewPSF.getKernel1FFT/getKernel2FFT 79-111)    */
/* ------------------------------------------------------------------------- */

typedef struct {
    int b[3];
    int k1d[3], k2d[3];
    cplx *k1hat, *k2hat; /* on P = b + k - 1 */
} orc_view_cache;

static void cache_build(orc_view_cache *c, const int b[3], const float *k1, const int k1d[3],
                        const float *k2, const int k2d[3])
{
    int P1[3], P2[3];
    for (int d = 0; d < 3; ++d) {
        c->b[d] = b[d]; c->k1d[d] = k1d[d]; c->k2d[d] = k2d[d];
        P1[d] = b[d] + k1d[d] - 1; P2[d] = b[d] + k2d[d] - 1;
    }
    c->k1hat = kernel_spectrum(k1, k1d, P1);
    c->k2hat = kernel_spectrum(k2, k2d, P2);
}

static void cache_free(orc_view_cache *c) { free(c->k1hat); free(c->k2hat); }

/* ------------------------------------------------------------------------- */
/* Block iterations                                                           */
/* ------------------------------------------------------------------------- */

/* One sequential block iteration:
 * ComputeBlockSeqThreadCPU.runIteration 79-169 (convolve1 171-189: mirror-single
 * extension; convolve2 191-209: value-1 extension), DM computeQuotient 46-98 and
 * computeFinalValues 103-182.  psi (float, in/out) or psi64 (double, in/out, fp64
 * mode) holds the whole block, updated in place.  stats[0] = sum of signed change,
 * stats[1] = max signed change (initial -1, ComputeBlockThread 64-68). */
static void block_seq_impl(float *psi, double *psi64, const float *img, const float *w,
                           const int b[3], const float *k1, const int k1d[3], const float *k2,
                           const int k2d[3], const orc_view_cache *cache, double lambda,
                           float minI, float maxI, int fp64, double *stats)
{
    const long n = (long)b[0] * b[1] * b[2];
    double *t = (double *)malloc(sizeof(double) * (size_t)n);
    double *u = (double *)malloc(sizeof(double) * (size_t)n);
    if (fp64) memcpy(t, psi64, sizeof(double) * (size_t)n);
    else for (long i = 0; i < n; ++i) t[i] = psi[i];
    /* conv1: psi >> tmp1 (stored as FloatType in the reference) */
    convolve_ext(t, b, ORC_EXT_MIRROR_SINGLE, 0.0, k1, k1d, cache ? cache->k1hat : NULL, u);
    /* quotient: tmp1 = img > 0 ? img / tmp1 : 1 (DM 71-74) */
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        if (fp64) u[i] = img[i] > 0 ? (double)img[i] / u[i] : 1.0;
        else {
            const float blurred = (float)u[i];
            u[i] = img[i] > 0 ? (double)(img[i] / blurred) : 1.0;
        }
    }
    /* conv2: tmp1 >> tmp2, outside value 1 */
    convolve_ext(u, b, ORC_EXT_VALUE, 1.0, k2, k2d, cache ? cache->k2hat : NULL, t);
    double sum = 0, mx = -1;
    for (long i = 0; i < n; ++i) {
        if (fp64) {
            const double last = psi64[i];
            const double next = next_value_f64(last, t[i], (double)w[i], lambda, (double)minI, (double)maxI);
            psi64[i] = next;
            const double ch = next - last;
            sum += ch;
            if (ch > mx) mx = ch;
        } else {
            const float last = psi[i];
            const float next = next_value_f32(last, (float)t[i], w[i], lambda, minI, maxI);
            psi[i] = next;
            const float ch = next - last; /* DM change 308: signed */
            sum += ch;
            if ((double)ch > mx) mx = ch;
        }
    }
    stats[0] = sum;
    stats[1] = mx;
    free(t);
    free(u);
}

void orc_block_seq(float *psi, double *psi64, const float *img, const float *w, const int b[3],
                   const float *k1, const int k1d[3], const float *k2, const int k2d[3],
                   double lambda, float minI, float maxI, int fp64, double *stats)
{
    block_seq_impl(psi, psi64, img, w, b, k1, k1d, k2, k2d, NULL, lambda, minI, maxI, fp64, stats);
}

/* One multiplicative block iteration: ComputeBlockMulThreadCPU.runIteration 87-188
 * (V x conv1, V x quotient, V x conv2, one computeFinalValuesMul, DM 187-306);
 * maxIntensity = (float) mean of the views' maxima in double (147-149). */
static void block_mul_impl(float *psi, double *psi64, int nv, const float *const *img,
                           const float *const *w, const int b[3], const float *const *k1,
                           const int (*k1d)[3], const float *const *k2, const int (*k2d)[3],
                           const orc_view_cache *caches, double lambda, float minI,
                           const float *maxI, int fp64, double *stats)
{
    const long n = (long)b[0] * b[1] * b[2];
    double *t = (double *)malloc(sizeof(double) * (size_t)n);
    double *u = (double *)malloc(sizeof(double) * (size_t)n);
    double *conv2 = (double *)malloc(sizeof(double) * (size_t)n * nv);
    double *p0 = (double *)malloc(sizeof(double) * (size_t)n);
    if (fp64) memcpy(p0, psi64, sizeof(double) * (size_t)n);
    else for (long i = 0; i < n; ++i) p0[i] = psi[i];
    for (int v = 0; v < nv; ++v) {
        convolve_ext(p0, b, ORC_EXT_MIRROR_SINGLE, 0.0, k1[v], k1d[v], caches ? caches[v].k1hat : NULL, u);
        for (long i = 0; i < n; ++i) {
            if (fp64) u[i] = img[v][i] > 0 ? (double)img[v][i] / u[i] : 1.0;
            else {
                const float blurred = (float)u[i];
                u[i] = img[v][i] > 0 ? (double)(img[v][i] / blurred) : 1.0;
            }
        }
        convolve_ext(u, b, ORC_EXT_VALUE, 1.0, k2[v], k2d[v], caches ? caches[v].k2hat : NULL, conv2 + (long)v * n);
    }
    double miv = 0;
    for (int v = 0; v < nv; ++v) miv += maxI[v];
    miv /= (double)nv;
    const float mivf = (float)miv;
    double sum = 0, mx = -1;
    float *ivf = (float *)malloc(sizeof(float) * (size_t)nv);
    float *wvf = (float *)malloc(sizeof(float) * (size_t)nv);
    double *ivd = (double *)malloc(sizeof(double) * (size_t)nv);
    double *wvd = (double *)malloc(sizeof(double) * (size_t)nv);
    for (long i = 0; i < n; ++i) {
        for (int v = 0; v < nv; ++v) {
            ivf[v] = (float)conv2[(long)v * n + i];
            wvf[v] = w[v][i];
            ivd[v] = conv2[(long)v * n + i];
            wvd[v] = w[v][i];
        }
        if (fp64) {
            const double last = psi64[i];
            const double next = next_value_mul_f64(last, ivd, wvd, nv, lambda, minI, miv);
            psi64[i] = next;
            const double ch = next - last;
            sum += ch;
            if (ch > mx) mx = ch;
        } else {
            const float last = psi[i];
            const float next = next_value_mul_f32(last, ivf, wvf, nv, lambda, minI, mivf);
            psi[i] = next;
            const float ch = next - last;
            sum += ch;
            if ((double)ch > mx) mx = ch;
        }
    }
    stats[0] = sum;
    stats[1] = mx;
    free(ivf); free(wvf); free(ivd); free(wvd);
    free(t); free(u); free(conv2); free(p0);
}

void orc_block_mul(float *psi, double *psi64, int nv, const float *const *img,
                   const float *const *w, const int b[3], const float *const *k1,
                   const int *k1d_flat, const float *const *k2, const int *k2d_flat,
                   double lambda, float minI, const float *maxI, int fp64, double *stats)
{
    block_mul_impl(psi, psi64, nv, img, w, b, k1, (const int(*)[3])k1d_flat, k2,
                   (const int(*)[3])k2d_flat, NULL, lambda, minI, maxI, fp64, stats);
}

/* ------------------------------------------------------------------------- */
/* PSF preparation (DeconViewPSF.init 119-254)                                */
/* ------------------------------------------------------------------------- */

/* FusionTools.divideIntoPortions 1287-1329: first portion length for T threads. */
static long first_portion_len(long size, int T)
{
    if (size == 0) return 0;
    long np = size <= T ? size : (T > size / (64L * 64L * 64L) ? T : size / (64L * 64L * 64L));
    long chunk = size / np;
    while (chunk == 0) { --np; chunk = size / np; }
    return np == 1 ? size : chunk;
}

/* AdjustInput.normToSum1 52-58 with sumImg 65-122: the sum over all voxels plus the
 * first thread portion's partial sum a second time (sumImg 115-119).  T <= 0 gives
 * the plain sum. */
void orc_norm_to_sum1(float *k, long size, int T)
{
    double s = 0;
    for (long i = 0; i < size; ++i) s += (double)k[i];
    if (T > 0) {
        const long f = first_portion_len(size, T);
        double s0 = 0;
        for (long i = 0; i < f; ++i) s0 += (double)k[i];
        s += s0;
    }
    for (long i = 0; i < size; ++i) k[i] = (float)((double)k[i] / s);
}

/* Mirror.mirror 55-132 applied to every axis (computeInvertedKernel 266-274):
 * positions p <= n/2 are swapped with n-1-p, so for even n the middle pair is
 * swapped twice (left unmirrored).  Odd n is an exact index reversal. */
void orc_invert_kernel(const float *k, const int kd[3], float *out)
{
    const long n = (long)kd[0] * kd[1] * kd[2];
    memcpy(out, k, sizeof(float) * (size_t)n);
    for (int ax = 0; ax < 3; ++ax) {
        const long dimA = kd[ax];
        const long half = dimA / 2, maxm = dimA - 1;
        for (long z = 0; z < kd[2]; ++z)
            for (long y = 0; y < kd[1]; ++y)
                for (long x = 0; x < kd[0]; ++x) {
                    long c[3] = {x, y, z};
                    if (c[ax] <= half) {
                        long o[3] = {x, y, z};
                        o[ax] = maxm - c[ax];
                        const long i1 = (c[2] * kd[1] + c[1]) * kd[0] + c[0];
                        const long i2 = (o[2] * kd[1] + o[1]) * kd[0] + o[0];
                        float tmp = out[i1];
                        out[i1] = out[i2];
                        out[i2] = tmp;
                    }
                }
    }
}

/* conv with zero extension, output cropped to the input's size, rounded to float
 * (FFTConvolution(extendZero(input), input, extendZero(kernel), kernel, output)). */
static void conv_zero_f32(const float *in, const int id[3], const float *k, const int kd[3], float *out)
{
    const long n = (long)id[0] * id[1] * id[2];
    double *d = (double *)malloc(sizeof(double) * (size_t)n);
    double *o = (double *)malloc(sizeof(double) * (size_t)n);
    for (long i = 0; i < n; ++i) d[i] = in[i];
    convolve_ext(d, id, ORC_EXT_ZERO, 0.0, k, kd, NULL, o);
    for (long i = 0; i < n; ++i) out[i] = (float)o[i];
    free(d);
    free(o);
}

enum { ORC_PSF_OPTIMIZATION_II = 0, ORC_PSF_OPTIMIZATION_I = 1, ORC_PSF_EFFICIENT_BAYESIAN = 2,
       ORC_PSF_INDEPENDENT = 3 };

/* DeconViewPSF.init 119-254 for all views in order (DeconViews 68-70).
 * kernels[v] (k1, in/out: normalised in place) and k2[v] (out, same dims as k1).
 * As in the reference, view v's compound kernel sees the other views' kernel1 in
 * their state at that time: normalised for w < v, raw for w > v. */
void orc_psf_init(int nv, float *const *k1, const int *kd_flat, int psf_type, int T, float *const *k2)
{
    const int(*kd)[3] = (const int(*)[3])kd_flat;
    for (int v = 0; v < nv; ++v) {
        const long n = (long)kd[v][0] * kd[v][1] * kd[v][2];
        orc_norm_to_sum1(k1[v], n, T);
        if (nv == 1 || psf_type == ORC_PSF_INDEPENDENT) {
            orc_invert_kernel(k1[v], kd[v], k2[v]);
        } else if (psf_type == ORC_PSF_EFFICIENT_BAYESIAN) {
            float *tmp = (float *)malloc(sizeof(float) * (size_t)n);
            float *inv = (float *)malloc(sizeof(float) * (size_t)n);
            float *o1 = (float *)malloc(sizeof(float) * (size_t)n);
            float *o2 = (float *)malloc(sizeof(float) * (size_t)n);
            orc_invert_kernel(k1[v], kd[v], tmp);
            for (int w = 0; w < nv; ++w) {
                if (w == v) continue;
                const long nw = (long)kd[w][0] * kd[w][1] * kd[w][2];
                float *invw = (float *)malloc(sizeof(float) * (size_t)nw);
                orc_invert_kernel(k1[v], kd[v], inv);
                conv_zero_f32(inv, kd[v], k1[w], kd[w], o1);
                orc_invert_kernel(k1[w], kd[w], invw);
                conv_zero_f32(o1, kd[v], invw, kd[w], o2);
                for (long i = 0; i < n; ++i) tmp[i] = o2[i] * tmp[i];
                free(invw);
            }
            orc_norm_to_sum1(tmp, n, T);
            memcpy(k2[v], tmp, sizeof(float) * (size_t)n);
            free(tmp); free(inv); free(o1); free(o2);
        } else if (psf_type == ORC_PSF_OPTIMIZATION_I) {
            float *tmp = (float *)malloc(sizeof(float) * (size_t)n);
            float *o = (float *)malloc(sizeof(float) * (size_t)n);
            memcpy(tmp, k1[v], sizeof(float) * (size_t)n);
            for (int w = 0; w < nv; ++w) {
                if (w == v) continue;
                const long nw = (long)kd[w][0] * kd[w][1] * kd[w][2];
                float *invw = (float *)malloc(sizeof(float) * (size_t)nw);
                orc_invert_kernel(k1[w], kd[w], invw);
                conv_zero_f32(k1[v], kd[v], invw, kd[w], o);
                for (long i = 0; i < n; ++i) tmp[i] = o[i] * tmp[i];
                free(invw);
            }
            orc_norm_to_sum1(tmp, n, T);
            orc_invert_kernel(tmp, kd[v], k2[v]);
            free(tmp); free(o);
        } else { /* OPTIMIZATION_II: computeExponentialKernel 256-264, pow 276-284 */
            float *e = (float *)malloc(sizeof(float) * (size_t)n);
            for (long i = 0; i < n; ++i) {
                float r = k1[v][i];
                for (int j = 1; j < nv; ++j) r *= k1[v][i];
                e[i] = r;
            }
            orc_norm_to_sum1(e, n, T);
            orc_invert_kernel(e, kd[v], k2[v]);
            free(e);
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Block geometry                                                             */
/* ------------------------------------------------------------------------- */

/* One block: BlockGeneratorFixedSizePrecise.divideIntoBlocks 59-131. */
typedef struct {
    long offset[3];
    long eff_offset[3];
    long eff_size[3];
    long eff_local[3];
} orc_block;

/* Returns the number of blocks (<= max_blocks written), or -1 if the block is
 * smaller than the kernel (divideIntoBlocks 70-77).  kernel2 is the doubled kernel
 * size 2k-1 (DeconView 155-157). */
int orc_divide_into_blocks(const long img[3], const long kernel2[3], const long bsize[3],
                           long *out /* 12 longs per block */, int max_blocks)
{
    long eff[3], loc[3], nb[3];
    for (int d = 0; d < 3; ++d) {
        eff[d] = bsize[d] - kernel2[d] + 1;
        if (eff[d] <= 0) return -1;
        loc[d] = kernel2[d] / 2;
        nb[d] = img[d] / eff[d] + (img[d] % eff[d] != 0);
    }
    int cnt = 0;
    for (long bz = 0; bz < nb[2]; ++bz)
        for (long by = 0; by < nb[1]; ++by)
            for (long bx = 0; bx < nb[0]; ++bx) {
                const long cb[3] = {bx, by, bz};
                if (cnt < max_blocks) {
                    long *o = out + 12L * cnt;
                    for (int d = 0; d < 3; ++d) {
                        long es = eff[d];
                        const long eo = cb[d] * eff[d];
                        if (eo + es > img[d]) es = img[d] - eo;
                        o[d] = eo - kernel2[d] / 2;
                        o[3 + d] = eo;
                        o[6 + d] = es;
                        o[9 + d] = loc[d];
                    }
                }
                ++cnt;
            }
    return cnt;
}

/* BlockSorter.sortBlocksBySmallestFootprint 55-143: returns the slab dimension and
 * writes batch[i] = slab index of block i (blocks grouped by min along that dim).
 * The HashMap keyed by the product of the other dims' block counts keeps the LAST
 * dimension for equal products (76-89), and ties sort by that key only. */
int orc_sort_blocks(const long nb[3], int min_required)
{
    long sz[3];
    int key_dim[3];
    for (int d = 0; d < 3; ++d) {
        sz[d] = 1;
        for (int e = 0; e < 3; ++e) if (e != d) sz[d] *= nb[e];
    }
    for (int d = 0; d < 3; ++d) { /* map value: last d with this size */
        key_dim[d] = d;
        for (int e = 0; e < 3; ++e) if (sz[e] == sz[d]) key_dim[d] = e;
    }
    long sorted[3] = {sz[0], sz[1], sz[2]};
    for (int i = 0; i < 3; ++i)
        for (int j = i + 1; j < 3; ++j)
            if (sorted[j] < sorted[i]) { long t = sorted[i]; sorted[i] = sorted[j]; sorted[j] = t; }
    for (int i = 0; i < 3; ++i) {
        if (sorted[i] >= min_required || i == 2) {
            for (int d = 0; d < 3; ++d) if (sz[d] == sorted[i]) return key_dim[d];
        }
    }
    return 2;
}

/* ------------------------------------------------------------------------- */
/* Weights and psi initialisation                                             */
/* ------------------------------------------------------------------------- */

/* NormalizingRandomAccess.get 76-109 with hardWeights 211-214 / smoothWeights
 * 183-200, evaluated for every voxel of every view. */
void orc_normalize_weights(int nv, const float *const *raw, long n, double osem, int smooth,
                           float maxDiffRange, float scalingRange, float *const *out)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        double sumW = 0;
        for (int v = 0; v < nv; ++v) {
            const double val = raw[v][i] < 1.0 ? raw[v][i] : 1.0;
            sumW += val;
        }
        for (int v = 0; v < nv; ++v) {
            const double val = raw[v][i] < 1.0 ? raw[v][i] : 1.0;
            const float my = (float)val;
            double r;
            if (smooth) {
                float s;
                if (sumW <= 0) s = 0;
                else {
                    const float ideal = (float)(my / sumW);
                    const float diff = my - ideal;
                    float y = (maxDiffRange - fabsf(diff)) * (1.0f / maxDiffRange);
                    y = y > 0 ? y : 0;
                    const float scale = y * my * scalingRange;
                    s = (my < ideal ? my : ideal) - (float)scale;
                }
                r = s;
            } else if (sumW > 1) r = (float)(my / sumW);
            else r = my;
            const double m = r * osem;
            out[v][i] = (float)(m < 1 ? m : 1);
        }
    }
}

/* PsiInitAvgPrecise.runInitialization 52-110 / PsiInitAvgPreciseThread 127-160:
 * mean over views with img > 0 averaged over voxels covered by >= 1 view; psi set
 * to that average; max[v] = maximum of view v. Returns the average. */
double orc_psi_init_avg(int nv, const float *const *img, long n, float *psi, float *maxv)
{
    double s = 0;
    long cnt = 0;
    for (int v = 0; v < nv; ++v) maxv[v] = 0;
    for (long i = 0; i < n; ++i) {
        double sum = 0;
        int c = 0;
        for (int v = 0; v < nv; ++v) {
            const float x = img[v][i];
            if (x > 0) {
                if (x > maxv[v]) maxv[v] = x;
                sum += x;
                ++c;
            }
        }
        if (c > 0) { s += sum / c; ++cnt; }
    }
    double avg = s / (double)cnt;
    if (isnan(avg)) avg = 1.0;
    if (psi) for (long i = 0; i < n; ++i) psi[i] = (float)avg;
    return avg;
}

/* ------------------------------------------------------------------------- */
/* Whole-volume iterations with the reference's block order                   */
/* ------------------------------------------------------------------------- */

static void extract_block(const float *vol, const double *vol64, const long D[3], const long off[3],
                          const int b[3], int mirror, float *out, double *out64)
{
#pragma omp parallel for schedule(static)
    for (long z = 0; z < b[2]; ++z)
        for (long y = 0; y < b[1]; ++y)
            for (long x = 0; x < b[0]; ++x) {
                long g[3] = {off[0] + x, off[1] + y, off[2] + z};
                int inside = 1;
                for (int d = 0; d < 3; ++d) {
                    if (g[d] < 0 || g[d] >= D[d]) inside = 0;
                    if (mirror) g[d] = orc_mirror_single(g[d], D[d]);
                }
                const long o = (z * b[1] + y) * b[0] + x;
                const long gi = (g[2] * D[1] + g[1]) * D[0] + g[0];
                if (!mirror && !inside) {
                    if (out) out[o] = 0;
                    if (out64) out64[o] = 0;
                } else {
                    if (out) out[o] = vol ? vol[gi] : (float)vol64[gi];
                    if (out64) out64[o] = vol64 ? vol64[gi] : (double)vol[gi];
                }
            }
}

static void paste_block(float *vol, double *vol64, const long D[3], const orc_block *bl, const int b[3],
                        const float *blk, const double *blk64)
{
    for (long z = 0; z < bl->eff_size[2]; ++z)
        for (long y = 0; y < bl->eff_size[1]; ++y)
            for (long x = 0; x < bl->eff_size[0]; ++x) {
                const long bi = ((z + bl->eff_local[2]) * b[1] + y + bl->eff_local[1]) * b[0] + x + bl->eff_local[0];
                const long gi = ((z + bl->eff_offset[2]) * D[1] + y + bl->eff_offset[1]) * D[0] + x + bl->eff_offset[0];
                if (vol) vol[gi] = blk[bi];
                if (vol64) vol64[gi] = blk64[bi];
            }
}

/* MultiViewDeconvolutionSeq.runNextIteration 57-180 and
 * MultiViewDeconvolutionMul.runNextIteration 116-245 for `iters` iterations:
 *  - blocks from divideIntoBlocks with the doubled kernel (per view in Seq mode),
 *    slab batches from sortBlocksBySmallestFootprint(min_required = 1, one block
 *    thread), blocks whose zero-extended weight is all zero dropped (DeconView
 *    filterBlocksForContent 204-274; Mul keeps all blocks of view 0's grid);
 *  - every block of batch j reads psi with batches < j-1 written back; batch j-1 is
 *    pasted after batch j is computed, the last batch after the loop;
 *  - a single block is pasted at once.
 * psi (float) or psi64 (double) hold the volume.  k1/k2 are the prepared kernels
 * (after DeconViewPSF.init).  stats_out (optional): per iteration and view (Seq) or
 * per iteration (Mul) {sumChange, maxChange}. */
int orc_decon_run(int nv, const long D[3], const float *const *img, const float *const *w,
                  const float *const *k1, const int *k1d_flat, const float *const *k2,
                  const int *k2d_flat, const int bsize[3], int iters, int mul, double lambda,
                  float minI, const float *maxv, int filter_blocks, int fp64, float *psi,
                  double *psi64, double *stats_out)
{
    const int(*k1d)[3] = (const int(*)[3])k1d_flat;
    const int(*k2d)[3] = (const int(*)[3])k2d_flat;
    const long nvox = D[0] * D[1] * D[2];
    const long bn = (long)bsize[0] * bsize[1] * bsize[2];
    int nsteps = mul ? 1 : nv;
    /* block grids per view-step */
    orc_block **blocks = (orc_block **)calloc((size_t)nsteps, sizeof(orc_block *));
    int *nblk = (int *)calloc((size_t)nsteps, sizeof(int));
    int **batch = (int **)calloc((size_t)nsteps, sizeof(int *));
    int *nbatch = (int *)calloc((size_t)nsteps, sizeof(int));
    for (int s = 0; s < nsteps; ++s) {
        long kk[3], bs[3];
        for (int d = 0; d < 3; ++d) { kk[d] = 2L * k1d[s][d] - 1; bs[d] = bsize[d]; }
        int cnt = orc_divide_into_blocks(D, kk, bs, NULL, 0);
        if (cnt < 0) return -1;
        long *raw = (long *)malloc(sizeof(long) * 12 * (size_t)cnt);
        orc_divide_into_blocks(D, kk, bs, raw, cnt);
        blocks[s] = (orc_block *)malloc(sizeof(orc_block) * (size_t)cnt);
        long nb[3];
        for (int d = 0; d < 3; ++d) {
            long eff = bs[d] - kk[d] + 1;
            nb[d] = D[d] / eff + (D[d] % eff != 0);
        }
        const int sd = orc_sort_blocks(nb, 1);
        batch[s] = (int *)malloc(sizeof(int) * (size_t)cnt);
        int keep = 0;
        for (int i = 0; i < cnt; ++i) {
            orc_block bl;
            for (int d = 0; d < 3; ++d) {
                bl.offset[d] = raw[12L * i + d];
                bl.eff_offset[d] = raw[12L * i + 3 + d];
                bl.eff_size[d] = raw[12L * i + 6 + d];
                bl.eff_local[d] = raw[12L * i + 9 + d];
            }
            int has = 1;
            if (filter_blocks) { /* weight of view s (Mul: view 0's grid), zero-extended over the block */
                has = 0;
                for (long z = 0; z < bsize[2] && !has; ++z)
                    for (long y = 0; y < bsize[1] && !has; ++y)
                        for (long x = 0; x < bsize[0]; ++x) {
                            long g[3] = {bl.offset[0] + x, bl.offset[1] + y, bl.offset[2] + z};
                            if (g[0] < 0 || g[1] < 0 || g[2] < 0 || g[0] >= D[0] || g[1] >= D[1] || g[2] >= D[2]) continue;
                            if (w[s][(g[2] * D[1] + g[1]) * D[0] + g[0]] != 0.0f) { has = 1; break; } /* s == 0 in Mul */
                        }
            }
            if (!has) continue;
            const long eff = bs[sd] - kk[sd] + 1;
            batch[s][keep] = (int)((bl.offset[sd] - (-(kk[sd] / 2))) / eff);
            blocks[s][keep++] = bl;
        }
        nblk[s] = keep;
        free(raw);
        int mb = 0;
        for (int i = 0; i < keep; ++i) if (batch[s][i] + 1 > mb) mb = batch[s][i] + 1;
        nbatch[s] = mb;
    }
    orc_view_cache *caches = (orc_view_cache *)calloc((size_t)nv, sizeof(orc_view_cache));
    for (int v = 0; v < nv; ++v) cache_build(&caches[v], bsize, k1[v], k1d[v], k2[v], k2d[v]);

    float *blk = fp64 ? NULL : (float *)malloc(sizeof(float) * (size_t)bn);
    double *blk64 = fp64 ? (double *)malloc(sizeof(double) * (size_t)bn) : NULL;
    float **imgb = (float **)malloc(sizeof(float *) * (size_t)nv);
    float **wb = (float **)malloc(sizeof(float *) * (size_t)nv);
    for (int v = 0; v < nv; ++v) {
        imgb[v] = (float *)malloc(sizeof(float) * (size_t)bn);
        wb[v] = (float *)malloc(sizeof(float) * (size_t)bn);
    }
    int maxb = 0;
    for (int s = 0; s < nsteps; ++s) if (nblk[s] > maxb) maxb = nblk[s];
    float **q = (float **)calloc((size_t)maxb, sizeof(float *));
    double **q64 = (double **)calloc((size_t)maxb, sizeof(double *));
    for (int i = 0; i < maxb; ++i) {
        if (fp64) q64[i] = (double *)malloc(sizeof(double) * (size_t)bn);
        else q[i] = (float *)malloc(sizeof(float) * (size_t)bn);
    }
    int *prev = (int *)malloc(sizeof(int) * (size_t)(maxb > 0 ? maxb : 1));
    int nprev;
    int sidx = 0;
    for (int it = 0; it < iters; ++it) {
        for (int s = 0; s < nsteps; ++s) {
            double ssum = 0, smax = -1;
            nprev = 0;
            const int single = nblk[s] == 1;
            for (int bt = 0; bt < nbatch[s]; ++bt) {
                int cur[4096];
                int ncur = 0;
                for (int i = 0; i < nblk[s]; ++i) if (batch[s][i] == bt) cur[ncur++] = i;
                for (int c = 0; c < ncur; ++c) {
                    const orc_block *bl = &blocks[s][cur[c]];
                    extract_block(fp64 ? NULL : psi, fp64 ? psi64 : NULL, D, bl->offset, bsize, 1,
                                  blk, blk64);
                    double st[2];
                    if (!mul) {
                        extract_block(img[s], NULL, D, bl->offset, bsize, 0, imgb[0], NULL);
                        extract_block(w[s], NULL, D, bl->offset, bsize, 0, wb[0], NULL);
                        block_seq_impl(blk, blk64, imgb[0], wb[0], bsize, k1[s], k1d[s], k2[s], k2d[s],
                                       &caches[s], lambda, minI, maxv[s], fp64, st);
                    } else {
                        for (int v = 0; v < nv; ++v) {
                            extract_block(img[v], NULL, D, bl->offset, bsize, 0, imgb[v], NULL);
                            extract_block(w[v], NULL, D, bl->offset, bsize, 0, wb[v], NULL);
                        }
                        block_mul_impl(blk, blk64, nv, (const float *const *)imgb, (const float *const *)wb,
                                       bsize, k1, k1d, k2, k2d, caches, lambda, minI, maxv, fp64, st);
                    }
                    ssum += st[0];
                    if (st[1] > smax) smax = st[1];
                    if (single) {
                        paste_block(fp64 ? NULL : psi, fp64 ? psi64 : NULL, D, bl, bsize, blk, blk64);
                    } else {
                        if (fp64) memcpy(q64[cur[c]], blk64, sizeof(double) * (size_t)bn);
                        else memcpy(q[cur[c]], blk, sizeof(float) * (size_t)bn);
                    }
                }
                if (!single) {
                    for (int c = 0; c < nprev; ++c)
                        paste_block(fp64 ? NULL : psi, fp64 ? psi64 : NULL, D, &blocks[s][prev[c]], bsize,
                                    q[prev[c]], q64[prev[c]]);
                    for (int c = 0; c < ncur; ++c) prev[c] = cur[c];
                    nprev = ncur;
                }
            }
            if (!single)
                for (int c = 0; c < nprev; ++c)
                    paste_block(fp64 ? NULL : psi, fp64 ? psi64 : NULL, D, &blocks[s][prev[c]], bsize,
                                q[prev[c]], q64[prev[c]]);
            if (stats_out) { stats_out[2 * sidx] = ssum; stats_out[2 * sidx + 1] = smax; }
            ++sidx;
        }
    }
    (void)nvox;
    for (int i = 0; i < maxb; ++i) { free(q[i]); free(q64[i]); }
    free(q); free(q64); free(prev);
    for (int v = 0; v < nv; ++v) { free(imgb[v]); free(wb[v]); cache_free(&caches[v]); }
    free(imgb); free(wb); free(caches); free(blk); free(blk64);
    for (int s = 0; s < nsteps; ++s) { free(blocks[s]); free(batch[s]); }
    free(blocks); free(batch); free(nblk); free(nbatch);
    return 0;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
