/*
 * Oracle (test infrastructure) copy of the portable single-precision
 * transcendental functions that the GPU geometry kernels use.
 *
 * The oracle runs in one of two math modes (vko_set_math_mode):
 *   portable - these functions, bit-identical to the device kernels, so the
 *              oracle and the GPU take the same Bezier subdivision and join
 *              decisions and produce the same vertices;
 *   libm     - the host C library's atan2f/acosf/cosf/sinf, i.e. vkvg's own
 *              code as it runs on a Linux host; used to measure how often the
 *              platform libm changes a flattening decision.
 * Method: Cephes single precision (S. L. Moshier) sinf/cosf/asinf/acosf/atanf
 * with C99 Annex F special cases for atan2f.  Only IEEE +,-,*,/,sqrt in a fixed
 * order; the oracle is compiled with -ffp-contract=off.
 */
#ifndef VKO_PMATH_H
#define VKO_PMATH_H

#ifdef __CUDACC__
#define VKO_PM_FN __host__ __device__ static inline
#else
#define VKO_PM_FN static inline
#endif

#include <math.h>

#define VKO_PM_PIF   3.14159265358979323846f
#define VKO_PM_PIO2F 1.57079632679489661923f
#define VKO_PM_PIO4F 0.785398163397448309616f
#define VKO_PM_FOPI  1.27323954473516268615f /* 4/pi */

VKO_PM_FN unsigned vko_pm__bits(float x) {
    union { float f; unsigned u; } c;
    c.f = x;
    return c.u;
}
VKO_PM_FN float vko_pm__from_bits(unsigned u) {
    union { float f; unsigned u; } c;
    c.u = u;
    return c.f;
}
VKO_PM_FN float vko_pm_nanf(void) { return vko_pm__from_bits(0x7fc00000u); }
VKO_PM_FN int vko_pm_isnan(float x) { return (vko_pm__bits(x) & 0x7fffffffu) > 0x7f800000u; }
VKO_PM_FN int vko_pm_isinf(float x) { return (vko_pm__bits(x) & 0x7fffffffu) == 0x7f800000u; }
VKO_PM_FN int vko_pm_signbit(float x) { return (int)(vko_pm__bits(x) >> 31); }

/* sin(x) for |x| <= pi/4, z = x*x */
VKO_PM_FN float vko_pm__sin_poly(float x, float z) {
    float p = -1.9515295891e-4f * z;
    p = p + 8.3321608736e-3f;
    p = p * z;
    p = p - 1.6666654611e-1f;
    p = p * z;
    p = p * x;
    return p + x;
}
/* cos(x) for |x| <= pi/4, z = x*x */
VKO_PM_FN float vko_pm__cos_poly(float z) {
    float p = 2.443315711809948e-5f * z;
    p = p - 1.388731625493765e-3f;
    p = p * z;
    p = p + 4.166664568298827e-2f;
    p = p * z;
    p = p * z;
    p = p - 0.5f * z;
    return p + 1.0f;
}
/* Reduce |x| (x >= 0) to r in [-pi/4, pi/4]; returns the octant j in 0..7 (even). */
VKO_PM_FN int vko_pm__reduce(float x, float *r) {
    if (x > 65536.0f) /* far outside the geometry's range: deterministic fold */
        x = fmodf(x, 6.28318548202514648f);
    int j   = (int)(VKO_PM_FOPI * x);
    float y = (float)j;
    if (j & 1) {
        j += 1;
        y += 1.0f;
    }
    float t = x - y * 0.78515625f;
    t       = t - y * 2.4187564849853515625e-4f;
    t       = t - y * 3.77489497744594108e-8f;
    *r      = t;
    return j & 7;
}
VKO_PM_FN float vko_pm_sinf(float xx) {
    if (vko_pm_isnan(xx))
        return xx;
    if (vko_pm_isinf(xx))
        return vko_pm_nanf();
    int sign = 0;
    float x  = xx;
    if (x < 0.0f) {
        sign = 1;
        x    = -x;
    }
    float r;
    int j = vko_pm__reduce(x, &r);
    if (j > 3) {
        sign ^= 1;
        j -= 4;
    }
    float z = r * r;
    float v = (j == 1 || j == 2) ? vko_pm__cos_poly(z) : vko_pm__sin_poly(r, z);
    return sign ? -v : v;
}
VKO_PM_FN float vko_pm_cosf(float xx) {
    if (vko_pm_isnan(xx))
        return xx;
    if (vko_pm_isinf(xx))
        return vko_pm_nanf();
    float x = xx < 0.0f ? -xx : xx;
    float r;
    int j    = vko_pm__reduce(x, &r);
    int sign = 0;
    if (j > 3) {
        j -= 4;
        sign = 1;
    }
    if (j > 1)
        sign ^= 1;
    float z = r * r;
    float v = (j == 1 || j == 2) ? vko_pm__sin_poly(r, z) : vko_pm__cos_poly(z);
    return sign ? -v : v;
}
VKO_PM_FN float vko_pm_asinf(float xx) {
    float a = xx < 0.0f ? -xx : xx;
    if (!(a <= 1.0f))
        return vko_pm_nanf();
    float x, z;
    int flag;
    if (a > 0.5f) {
        z    = 0.5f * (1.0f - a);
        x    = sqrtf(z);
        flag = 1;
    } else {
        if (a < 1.0e-4f)
            return xx;
        x    = a;
        z    = x * x;
        flag = 0;
    }
    float p = 4.2163199048e-2f * z;
    p       = p + 2.4181311049e-2f;
    p       = p * z;
    p       = p + 4.5470025998e-2f;
    p       = p * z;
    p       = p + 7.4953002686e-2f;
    p       = p * z;
    p       = p + 1.6666752422e-1f;
    p       = p * z;
    p       = p * x;
    p       = p + x;
    if (flag) {
        p = p + p;
        p = VKO_PM_PIO2F - p;
    }
    return xx < 0.0f ? -p : p;
}
VKO_PM_FN float vko_pm_acosf(float x) {
    float a = x < 0.0f ? -x : x;
    if (!(a <= 1.0f))
        return vko_pm_nanf();
    if (x < -0.5f)
        return VKO_PM_PIF - 2.0f * vko_pm_asinf(sqrtf(0.5f * (1.0f + x)));
    if (x > 0.5f)
        return 2.0f * vko_pm_asinf(sqrtf(0.5f * (1.0f - x)));
    return VKO_PM_PIO2F - vko_pm_asinf(x);
}
VKO_PM_FN float vko_pm_atanf(float xx) {
    float x = xx < 0.0f ? -xx : xx;
    float y;
    if (x > 2.414213562373095f) {
        y = VKO_PM_PIO2F;
        x = -(1.0f / x);
    } else if (x > 0.4142135623730950f) {
        y = VKO_PM_PIO4F;
        x = (x - 1.0f) / (x + 1.0f);
    } else {
        y = 0.0f;
    }
    float z = x * x;
    float p = 8.05374449538e-2f * z;
    p       = p - 1.38776856032e-1f;
    p       = p * z;
    p       = p + 1.99777106478e-1f;
    p       = p * z;
    p       = p - 3.33329491539e-1f;
    p       = p * z;
    p       = p * x;
    p       = p + x;
    y       = y + p;
    return xx < 0.0f ? -y : y;
}
VKO_PM_FN float vko_pm_atan2f(float y, float x) {
    if (vko_pm_isnan(x) || vko_pm_isnan(y))
        return x + y;
    if (y == 0.0f) {
        if (vko_pm_signbit(x))
            return vko_pm_signbit(y) ? -VKO_PM_PIF : VKO_PM_PIF;
        return y;
    }
    if (x == 0.0f)
        return y > 0.0f ? VKO_PM_PIO2F : -VKO_PM_PIO2F;
    if (vko_pm_isinf(x)) {
        if (vko_pm_isinf(y)) {
            float r = x > 0.0f ? VKO_PM_PIO4F : 3.0f * VKO_PM_PIO4F;
            return y > 0.0f ? r : -r;
        }
        if (x > 0.0f)
            return y > 0.0f ? 0.0f : -0.0f;
        return y > 0.0f ? VKO_PM_PIF : -VKO_PM_PIF;
    }
    if (vko_pm_isinf(y))
        return y > 0.0f ? VKO_PM_PIO2F : -VKO_PM_PIO2F;
    float w = 0.0f;
    if (x < 0.0f)
        w = y < 0.0f ? -VKO_PM_PIF : VKO_PM_PIF;
    float z = vko_pm_atanf(y / x);
    return w + z;
}

#endif
