/* Host check of the weight normalisation's division (multiview-reconstruction_gb300/csrc/wdiv.h)
 * against the double formula it replaces, (float)((double)my / s): random weights and sums, and
 * quotients placed next to float rounding boundaries.  Prints: cases, mismatches, double
 * fallbacks, cases with a weight of at least 1e-6, their fallbacks. */
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
    printf("%ld %ld %ld %ld %ld\n", cases, bad, fall, reg, reg_fall);
    return bad != 0;
}
