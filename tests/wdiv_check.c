/* Host check of the weight normalisation's division (multiview-reconstruction_gb300/csrc/wdiv.h)
 * against the double formula it replaces, (float)((double)my / s): random weights and sums, and
 * quotients placed next to float rounding boundaries, whole voxels through mvr_wd_normalize
 * against the reference's double formulas, and the fast path with a perturbed sum.  Prints:
 * cases, mismatches, double fallbacks, cases with a weight of at least 1e-6, their fallbacks;
 * voxel weights, their mismatches; perturbed cases, their mismatches. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include "../multiview-reconstruction_gb300/csrc/wdiv.h"

static uint64_t st = 0x9E3779B97F4A7C15ull;
static uint64_t next_u64(void)
{
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return st;
}
static double unit(void) { return (double)(next_u64() >> 11) * (1.0 / 9007199254740992.0); }

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    long bad = 0, fall = 0, cases = 0, reg = 0, reg_fall = 0;
    for (long i = 0; i < n; ++i) {
        /* a voxel: nv weights in [0, 1] (some exactly 0 or 1, some tiny), their double sum */
        const int nv = 2 + (int)(next_u64() % 7);
        float w[8];
        double s = 0.0;
        for (int v = 0; v < nv; ++v) {
            const uint64_t k = next_u64() % 16;
            float x = (float)unit();
            if (k == 0) x = 0.0f;
            else if (k == 1) x = 1.0f;
            else if (k == 2) x = (float)(unit() * 1e-12);
            else if (k == 3) x = (float)(unit() * 1e-30);
            w[v] = x;
            s += (double)x;
        }
        if (!(s > 0.0)) continue;
        if (next_u64() % 4 == 0) s *= 0.001 + unit();  /* sums below 1 (the smooth blending divides those too) */
        const MvrWdSum ws = mvr_wd_sum(s);
        for (int v = 0; v < nv; ++v) {
            float q;
            const int f = !mvr_wd_fast(w[v], &ws, &q);
            fall += f;
            if (w[v] >= 1e-6f) {
                ++reg;
                reg_fall += f;
            }
            const float got = mvr_weight_div(w[v], &ws), ref = (float)((double)w[v] / s);
            bad += mvr_wd_float_to_bits(got) != mvr_wd_float_to_bits(ref);
            ++cases;
        }
        /* a quotient at a float midpoint m = c + u/2 (and a double ulp either side): my = RN_f(m s') */
        {
            const double sp = 1.0 + unit() * 7.0;
            const float c = (float)(0.01 + unit() * 0.9);
            const unsigned int cb = mvr_wd_float_to_bits(c);
            const double m = ((double)c + (double)mvr_wd_bits_to_float(cb + 1u)) * 0.5;
            const float my = (float)(m * sp);
            if (my <= 1.0f) {
                for (int j = -1; j <= 1; ++j) {
                    /* the sum that puts my / s exactly on (or a double ulp off) the midpoint */
                    double s2 = (double)my / m;
                    s2 = j < 0 ? nextafter(s2, 0.0) : (j > 0 ? nextafter(s2, 2.0 * s2) : s2);
                    if (!(s2 > 1.0)) continue;
                    const MvrWdSum w2 = mvr_wd_sum(s2);
                    float q;
                    fall += !mvr_wd_fast(my, &w2, &q);
                    const float got = mvr_weight_div(my, &w2), ref = (float)((double)my / s2);
                    bad += mvr_wd_float_to_bits(got) != mvr_wd_float_to_bits(ref);
                    ++cases;
                }
            }
        }
    }
    /* whole voxels: mvr_wd_normalize against the reference's formulas in double
     * (NormalizingRandomAccess: the sequential double sum, hard / smooth, OSEM factor) */
    long vbad = 0, vcases = 0;
    for (long i = 0; i < n / 2; ++i) {
        const int nv = 1 + (int)(next_u64() % 16);
        float w[16], out[16];
        for (int v = 0; v < nv; ++v) {
            const uint64_t k = next_u64() % 24;
            float x = (float)unit();
            if (k == 0) x = 0.0f;
            else if (k == 1) x = 1.0f;
            else if (k == 2) x = (float)(unit() * 1e-12);
            else if (k == 3) x = (float)(unit() * 1e-30);
            else if (k == 4) x = -(float)unit() * 0.01f;    /* a negative weight */
            else if (k == 5) x = (float)(1.0 / nv);         /* sums at 1 */
            w[v] = x;
        }
        const int smooth = (int)(next_u64() % 2);
        const double osem = (next_u64() % 3 == 0) ? 2.5 : 1.0;
        const float maxDiff = 0.1f, scaling = 0.05f;
        mvr_wd_normalize(w, nv, 16, osem == 1.0, osem, smooth, maxDiff, scaling, out);
        double sumW = 0.0;
        for (int v = 0; v < nv; ++v) sumW += (double)w[v];
        for (int v = 0; v < nv; ++v) {
            const float my = w[v];
            double r;
            if (smooth) {
                float sm;
                if (sumW <= 0) sm = 0.0f;
                else {
                    const float ideal = (float)((double)my / sumW);
                    const float diff = my - ideal;
                    float y = (maxDiff - fabsf(diff)) * (1.0f / maxDiff);
                    y = y > 0.0f ? y : 0.0f;
                    const float scale = (y * my) * scaling;
                    sm = fminf(my, ideal) - scale;
                }
                r = sm;
            } else if (sumW > 1) r = (float)((double)my / sumW);
            else r = my;
            const double m = r * osem;
            const float ref = (float)(m < 1.0 ? m : 1.0);
            vbad += mvr_wd_float_to_bits(out[v]) != mvr_wd_float_to_bits(ref);
            ++vcases;
        }
    }
    /* the fast path with the sum off by up to 2^-40 of itself (the float pair's deviation)
     * and quotients on float midpoints: never a wrong rounding */
    long pbad = 0, pcases = 0;
    for (long i = 0; i < n / 2; ++i) {
        const double sp = 1.0 + unit() * 7.0;
        const float c = (float)(0.01 + unit() * 0.9);
        const unsigned int cb = mvr_wd_float_to_bits(c);
        const double m = ((double)c + (double)mvr_wd_bits_to_float(cb + 1u)) * 0.5;
        const float my = (float)(m * sp);
        if (!(my <= 1.0f)) continue;
        double s2 = (double)my / m;
        const int j = (int)(next_u64() % 3) - 1;
        s2 = j < 0 ? nextafter(s2, 0.0) : (j > 0 ? nextafter(s2, 2.0 * s2) : s2);
        const double dev = (unit() * 2.0 - 1.0) * 9.094947017729282e-13 * s2; /* 2^-40 */
        MvrWdSum w2 = mvr_wd_sum(s2 + dev);
        w2.s = s2 + dev;
        float q;
        if (mvr_wd_fast(my, &w2, &q)) pbad += mvr_wd_float_to_bits(q) != mvr_wd_float_to_bits((float)((double)my / s2));
        ++pcases;
    }
    printf("%ld %ld %ld %ld %ld %ld %ld %ld %ld\n", cases, bad, fall, reg, reg_fall, vcases, vbad, pcases, pbad);
    return bad != 0 || vbad != 0 || pbad != 0;
}
