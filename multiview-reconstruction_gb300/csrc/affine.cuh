// 3D affine transforms (row-packed 3 x 4: x' = m[0] x + m[1] y + m[2] z + m[3], ...) and the
// linear interpolation of the image utilities (imglib2 AffineTransform3D, NLinearInterpolator3D).
#pragma once
#include <cuda_runtime.h>

#include <cmath>

namespace mvr {

// Inverse of an affine transform by the adjugate of its 3 x 3 part; false when singular.
inline bool invert_affine(const double *m, double *inv)
{
    const double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], k = m[10];
    const double det = a * (e * k - f * h) - b * (d * k - f * g) + c * (d * h - e * g);
    if (det == 0.0 || !std::isfinite(det)) return false;
    const double r = 1.0 / det;
    const double i00 = (e * k - f * h) * r, i01 = (c * h - b * k) * r, i02 = (b * f - c * e) * r;
    const double i10 = (f * g - d * k) * r, i11 = (a * k - c * g) * r, i12 = (c * d - a * f) * r;
    const double i20 = (d * h - e * g) * r, i21 = (b * g - a * h) * r, i22 = (a * e - b * d) * r;
    inv[0] = i00, inv[1] = i01, inv[2] = i02;
    inv[4] = i10, inv[5] = i11, inv[6] = i12;
    inv[8] = i20, inv[9] = i21, inv[10] = i22;
    inv[3] = -(i00 * m[3] + i01 * m[7] + i02 * m[11]);
    inv[7] = -(i10 * m[3] + i11 * m[7] + i12 * m[11]);
    inv[11] = -(i20 * m[3] + i21 * m[7] + i22 * m[11]);
    return true;
}

// AffineTransform3D.apply: each coordinate s0 m0 + s1 m1 + s2 m2 + m3 summed left to right,
// every operation rounded (no contraction into fused multiply-adds).
__host__ __device__ __forceinline__ void apply_affine(const double *m, const double *s, double *t)
{
#ifdef __CUDA_ARCH__
#pragma unroll
    for (int r = 0; r < 3; ++r)
        t[r] = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(s[0], m[4 * r]), __dmul_rn(s[1], m[4 * r + 1])),
                                   __dmul_rn(s[2], m[4 * r + 2])),
                         m[4 * r + 3]);
#else
    for (int r = 0; r < 3; ++r) {
        volatile double p0 = s[0] * m[4 * r], p1 = s[1] * m[4 * r + 1], p2 = s[2] * m[4 * r + 2];
        t[r] = ((p0 + p1) + p2) + m[4 * r + 3];
    }
#endif
}

// Linear interpolation from the corner values at floor(t) + (dx, dy, dz): weights in double
// (w = t - floor t), every corner's value times its weight rounded to float, the corners
// summed in float in the order 000, 100, 110, 010, 011, 111, 101, 001 (the Gray-code walk
// of imglib2's NLinearInterpolator3D.get).  get(dx, dy, dz) returns the corner value.
template <class Get>
__device__ __forceinline__ float nlinear3(const double w[3], Get get)
{
    const double u0 = __dsub_rn(1.0, w[0]), u1 = __dsub_rn(1.0, w[1]), u2 = __dsub_rn(1.0, w[2]);
    const int order[8] = {0, 1, 3, 2, 6, 7, 5, 4};  // dx + 2 dy + 4 dz
    float acc = 0.0f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int c = order[k], dx = c & 1, dy = (c >> 1) & 1, dz = c >> 2;
        const double wk = __dmul_rn(__dmul_rn(dx ? w[0] : u0, dy ? w[1] : u1), dz ? w[2] : u2);
        const float term = __double2float_rn(__dmul_rn((double)get(dx, dy, dz), wk));
        acc = k == 0 ? term : __fadd_rn(acc, term);
    }
    return acc;
}

}  // namespace mvr
