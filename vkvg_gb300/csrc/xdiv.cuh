/* Exact integer division helper for the crossing computations (device). */
#ifndef VKVG_GB300_XDIV_CUH
#define VKVG_GB300_XDIV_CUH

#include <cuda_runtime.h>
#include <stdint.h>

/* exact int -> float for |a| < 2^22: the integer added to the bits of
   1.5 * 2^23 moves the value by a units of its last place (1.0) */
__device__ __forceinline__ float gb_small_i2f(int32_t a) { return __int_as_float(0x4B400000 + a) - 12582912.0f; }

/* ceil(a * b / den) for den > 0 and |b| <= den, exact.
 *
 * Fast path (|a| < 2^20, den < 2^22, so |quotient| <= |a| < 2^20): the three
 * operands convert exactly; the fp32 product (one rounding, 2^-24 relative)
 * divided by __fdividef (at most 2 ulp) is within |q| * 2^-21.6 < 0.35 of the
 * true quotient q, so its nearest integer c lies within 1 of ceil(q).  The
 * remainder r = a*b - c*den has |r| < 2 * den < 2^31, so it is exact in
 * wrapping 32-bit arithmetic, and one step on its sign gives ceil(q).
 * Otherwise an exact 64-bit division. */
__device__ __forceinline__ long long gb_ceil_muldiv(int32_t a, int32_t b, int32_t den) {
    const uint32_t aa = a < 0 ? 0u - (uint32_t)a : (uint32_t)a;
    if (aa < (1u << 20) && den < (1 << 22)) {
        const float qf = __fdividef(gb_small_i2f(a) * gb_small_i2f(b), gb_small_i2f(den));
        int32_t     c  = __float_as_int(qf + 12582912.0f) - 0x4B400000; /* nearest integer, |qf| < 2^21 */
        const int32_t r = (int32_t)((uint32_t)a * (uint32_t)b - (uint32_t)c * (uint32_t)den);
        if (r > 0)
            c++;
        else if (r <= -den)
            c--;
        return c;
    }
    const long long num = (long long)a * (long long)b;
    long long       q = num / den, r = num % den;
    return r > 0 ? q + 1 : q;
}

#endif
