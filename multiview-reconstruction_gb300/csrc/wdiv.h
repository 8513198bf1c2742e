// The weight normalisation of NormalizingRandomAccess (NormalizingRandomAccess.java:76-109,
// 183-200, 211-214: each view's weight over the double sum of all views' weights, rounded to
// float) from float operations, bit for bit the reference's double formulas, with double
// operations kept only where a float rounding boundary is within a hair.
//
// The division (float)((double)my / s): with s = sh + sl + t (|t| <= 2^-40 s: the double sum
// itself, split into two floats, or the float pair below standing in for it), a float
// candidate q and r = my - q s evaluated as a float-float residual (p + e = q sh exactly by an
// FMA), the true quotient Q = my / s lies strictly between the midpoints q - a and q + b
// around q (a, b half the gaps to q's neighbours) exactly when -a s < r < b s.  The evaluation
// error of r, t's share included, is below 2^-16.9 u s (u the gap above q; q < 2^24 u).  When r
// clears both bounds by B = 2^-14 u s, RN_f(Q) = q, and RN_f(RN_d(Q)) = q as well: the double
// rounding can only change the result when RN_d(Q) is a float midpoint, i.e. |Q - midpoint| <=
// 2^-53 Q, inside the excluded band.  Everything else (the band, my below 2^-60 but not 0,
// sums outside [2^-20, 2^16], sums next to 1, negative weights) takes the double operations.
//
// The sum: the weights' float two-sums into hi, their rounding errors into lo; for up to 16
// weights in [0, 1], |hi + lo - sum| <= 2^-41 of the sum, and the reference's sequential double
// sum is within 2^-49 of it.
// Plain C so that the same source is checked on the host against the double formulas.
#pragma once
#ifdef __CUDACC__
#define MVR_WD_FN __host__ __device__ __forceinline__
#else
#include <math.h>
#include <string.h>
#define MVR_WD_FN static inline
#endif

MVR_WD_FN float mvr_wd_bits_to_float(unsigned int b)
{
    float f;
    memcpy(&f, &b, sizeof f);
    return f;
}

MVR_WD_FN unsigned int mvr_wd_float_to_bits(float f)
{
    unsigned int b;
    memcpy(&b, &f, sizeof b);
    return b;
}

// my - q s with s = sh + sl, q sh = p + e exactly
MVR_WD_FN float mvr_wd_resid(float my, float q, float sh, float sl)
{
    const float p = q * sh;
    const float e = fmaf(q, sh, -p);
    return ((my - p) - e) - q * sl;
}

// Per-voxel part: s split into sh + sl and the reciprocal of sh (shared by every view); s itself
// only for mvr_weight_div's double fallback (not set from a float pair)
typedef struct {
    double s;
    float sh, sl, rs;
} MvrWdSum;

MVR_WD_FN MvrWdSum mvr_wd_sum(double s)
{
    MvrWdSum w;
    w.s = s;
    w.sh = (float)s;
    w.sl = (float)(s - (double)w.sh);
    w.rs = 1.0f / w.sh;
    return w;
}

// 1: the fast path decided (*out = q); 0: the caller divides in double
MVR_WD_FN int mvr_wd_fast(float my, const MvrWdSum *w, float *out)
{
    if (!(w->sh >= 9.5367431640625e-07f) || !(w->sh <= 65536.0f)) return 0;  // s in [2^-20, 2^16]
    if (my == 0.0f) {  // +-0 / s
        *out = my;
        return 1;
    }
    if (!(my >= 8.673617379884035e-19f) || !(my <= 1.0f)) return 0;  // below 2^-60, above 1, NaN
    const float sh = w->sh, sl = w->sl;
    const float q0 = my * w->rs;
    const float q = fmaf(mvr_wd_resid(my, q0, sh, sl), w->rs, q0);  // within about half a gap of Q
    if (!(q > 0.0f)) return 0;
    const unsigned int qb = mvr_wd_float_to_bits(q);
    if ((qb >> 23) == 0u || (qb >> 23) >= 254u) return 0;  // denormal or near the top: not here
    const float up = mvr_wd_bits_to_float(qb + 1u), dn = mvr_wd_bits_to_float(qb - 1u);
    const float b = (up - q) * 0.5f, a = (q - dn) * 0.5f, u = up - q;  // exact (powers of two)
    const float r = mvr_wd_resid(my, q, sh, sl);
    const float bound = u * sh * 6.103515625e-05f;  // 2^-14 u s
    if (r < b * sh - bound && r > -(a * sh) + bound) {
        *out = q;
        return 1;
    }
    return 0;
}

// (float)((double)my / s)
MVR_WD_FN float mvr_weight_div(float my, const MvrWdSum *w)
{
    float q;
    if (mvr_wd_fast(my, w, &q)) return q;
    return (float)((double)my / w->s);
}

// hi + lo += w: a float two-sum into hi, its error into lo
MVR_WD_FN void mvr_wd_pair_add(float *hi, float *lo, float w)
{
    const float s = *hi + w;
    const float bb = s - *hi;
    *lo += (*hi - (s - bb)) + (w - bb);
    *hi = s;
}

// The per-voxel part from the float pair of a sum of non-negative weights (no double s:
// the caller's fallback forms the reference's double sum itself)
MVR_WD_FN MvrWdSum mvr_wd_sum_pair(float hi, float lo)
{
    MvrWdSum w;
    w.sh = hi + lo;
    w.sl = lo - (w.sh - hi);
    w.s = 0.0;
    w.rs = 1.0f / w.sh;
    return w;
}

#ifdef __CUDA_ARCH__
// the reference's float operations, kept apart from contraction into FMAs
#define MVR_WD_SUB(a, b) __fsub_rn(a, b)
#define MVR_WD_MUL(a, b) __fmul_rn(a, b)
#define MVR_WD_DIV(a, b) __fdiv_rn(a, b)
#else
#define MVR_WD_SUB(a, b) ((a) - (b))
#define MVR_WD_MUL(a, b) ((a) * (b))
#define MVR_WD_DIV(a, b) ((a) / (b))
#endif
#define MVR_WD_MAX_VIEWS 16

// One voxel: w[v] = min(1, raw weight of view v) for v < nv (nv <= 16), out[v] the
// normalised weight (hard: w / sum where the sum exceeds 1; smooth: the blended form), times
// the OSEM factor (osem_one: the factor is 1) and capped at 1 -- as the reference computes it
// in double.  Ordinary voxels take no double operation.  maxv (>= nv, at most 16): the length
// of w and out, a constant in the caller so that the loops unroll onto registers.
MVR_WD_FN void mvr_wd_normalize(const float *w, int nv, int maxv, int osem_one, double osem, int smooth,
                                float maxDiffRange, float scalingRange, float *out)
{
    float hi = 0.0f, lo = 0.0f;
    int neg = 0;
#ifdef __CUDACC__
#pragma unroll
#endif
    for (int v = 0; v < maxv; ++v)
        if (v < nv) {
            neg |= !(w[v] >= 0.0f);
            mvr_wd_pair_add(&hi, &lo, w[v]);
        }
    MvrWdSum ws = mvr_wd_sum_pair(hi, lo);
    double sd = 0.0;  // the reference's sequential double sum, where the pair cannot stand in
    int have_sd = 0;
    if (neg || !(ws.sh < 0.99999904632568359f || ws.sh > 1.0000009536743164f)) {  // 1 -+ 2^-20
#ifdef __CUDACC__
#pragma unroll
#endif
        for (int v = 0; v < maxv; ++v)
            if (v < nv) sd += (double)w[v];
        have_sd = 1;
        ws = mvr_wd_sum(sd);
    }
    int gt1, le0;
    if (have_sd) {
        gt1 = sd > 1.0;
        le0 = sd <= 0.0;
    } else {
        gt1 = ws.sh > 1.0f;
        le0 = !(ws.sh > 0.0f);  // non-negative weights: 0 only when all are
    }
#ifdef __CUDACC__
#pragma unroll
#endif
    for (int v = 0; v < maxv; ++v) {
        if (v >= nv) continue;
        const float my = w[v];
        float q = 0.0f;
        const int need_q = smooth ? !le0 : gt1;
        if (need_q && !mvr_wd_fast(my, &ws, &q)) {
            if (!have_sd) {
                sd = 0.0;
                for (int u = 0; u < nv; ++u) sd += (double)w[u];
                have_sd = 1;
            }
            q = (float)((double)my / sd);
        }
        if (!smooth && osem_one) {
            out[v] = gt1 ? q : my;
            continue;
        }
        double r;
        if (smooth) {
            float s;
            if (le0) s = 0.0f;
            else {
                const float ideal = q;
                const float diff = MVR_WD_SUB(my, ideal);
                float y = MVR_WD_MUL(MVR_WD_SUB(maxDiffRange, fabsf(diff)), MVR_WD_DIV(1.0f, maxDiffRange));
                y = y > 0.0f ? y : 0.0f;
                const float scale = MVR_WD_MUL(MVR_WD_MUL(y, my), scalingRange);
                s = MVR_WD_SUB(fminf(my, ideal), scale);
            }
            r = s;
        } else if (gt1) r = q;
        else r = my;
        const double m = r * osem;
        out[v] = (float)(m < 1.0 ? m : 1.0);
    }
}
