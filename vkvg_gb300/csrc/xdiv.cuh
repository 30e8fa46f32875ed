/* Exact integer division helpers for the crossing computations (device). */
#ifndef VKVG_GB300_XDIV_CUH
#define VKVG_GB300_XDIV_CUH

#include <cuda_runtime.h>

/* ceil(num / den) for den > 0, exact.  An fp32 quotient estimate is within
   0.75 of the true value when |q| < 2^22 (three roundings of relative error
   2^-24 each), so one exact product test fixes it; larger quotients use an
   exact 64-bit division. */
__device__ __forceinline__ long long gb_ceil_div(long long num, int den) {
    float qf = __ll2float_rn(num) / (float)den;
    if (fabsf(qf) < 4194304.0f) {
        long long c = (long long)ceilf(qf);
        long long p = c * (long long)den;
        if (p < num)
            c++;
        else if (p - den >= num)
            c--;
        return c;
    }
    long long q = num / den, r = num % den;
    return r > 0 ? q + 1 : q;
}
__device__ __forceinline__ long long gb_floor_div(long long num, int den) { return -gb_ceil_div(-num, den); }

#endif
