// Compensated float sums.
#pragma once
#include <cuda_runtime.h>

namespace mvr {

// Sum of two float-pair values (hi + lo) without losing the low part (Knuth's TwoSum on
// the high parts, the low parts and the rounding error added, then renormalised).  The
// pair carries about 48 significant bits, which is what the CTA reduction needs: the
// GPU's double rate is so low that a few double additions per thread at the end of every
// CTA cost a large part of the kernel.
__device__ __forceinline__ void pair_add(float &hi, float &lo, float bhi, float blo)
{
    const float s = hi + bhi;
    const float v = s - hi;
    float e = (hi - (s - v)) + (bhi - v);
    e += lo + blo;
    hi = s + e;
    lo = e - (hi - s);
}

}  // namespace mvr
