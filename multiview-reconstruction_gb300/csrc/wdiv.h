// (float)((double)my / s) for a float my and a double s > 0 -- the weight normalisation's
// division (NormalizingRandomAccess.java:183-200: the view's weight over the double sum of all
// views' weights, rounded to float) -- from float operations, with the double division kept
// only where the quotient lies within a hair of a float rounding boundary (and outside the
// ranges the fast path covers: s in [2^-20, 2^16], my in [2^-60, 1] or 0).
//
// With sh = RN_f(s), sl = RN_f(s - sh) (s = sh + sl to 2^-48 relative), a float candidate q
// and r = my - q s evaluated as a float-float residual (p + e = q sh exactly by an FMA), the
// true quotient Q = my / s lies strictly between the midpoints q - a and q + b around q
// (a, b half the gaps to q's neighbours) exactly when -a s < r < b s.  When r clears both
// bounds by more than B = 2^-18 u s (u the gap above q; the evaluation error of r is below
// 2^-21 u s), RN_f(Q) = q, and RN_f(RN_d(Q)) = q as well: the double rounding can only
// change the result when RN_d(Q) is a float midpoint, i.e. |Q - midpoint| <= 2^-53 Q, inside
// the excluded band.  Everything else (the band, my <= 2^-60, my non-finite) takes the double
// division itself, so the function returns exactly the reference's value for every input.
// Plain C so that the same source is checked on the host against the double formula.
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

// Per-voxel part: s split into sh + sl and the reciprocal of sh (shared by every view)
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
    if (!(w->s >= 9.5367431640625e-07) || !(w->s <= 65536.0)) return 0;  // s in [2^-20, 2^16]
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
    const float bound = u * sh * 3.814697265625e-06f;  // 2^-18 u s
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
