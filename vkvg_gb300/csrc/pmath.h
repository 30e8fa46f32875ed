/*
 * Portable single-precision transcendental functions shared by the host
 * recorder and the sm_103a geometry kernels.
 *
 * Why: the path geometry branches on atan2f differences (Bezier subdivision,
 * src/vkvg_context_internal.c:1360-1385 of vkvg) and places round-join / arc
 * vertices with cosf/sinf/acosf.  glibc's and CUDA's implementations of these
 * functions differ by an ulp or two, which would make the host and the GPU
 * take different subdivision decisions.  Every function here uses only IEEE
 * +, -, *, / and sqrt on float, in a fixed order, so the host build
 * (-ffp-contract=off) and the device build (-fmad=false, IEEE div/sqrt) give
 * identical bits.
 *
 * Method: the single-precision algorithms of S. L. Moshier's Cephes library
 * (sinf.c / cosf.c: Cody-Waite reduction by pi/4 in three parts plus degree-7
 * odd / degree-8 even minimax polynomials; asinf.c / acosf.c: half-angle
 * reduction at |x| > 0.5 plus a degree-11 odd polynomial; atanf.c: reduction
 * at tan(pi/8) and tan(3pi/8) plus a degree-9 odd polynomial), with C99 Annex F
 * handling of zeros, infinities and NaN added to atan2f.  Accuracy is a few
 * ulp; what matters here is that both sides compute the same value.
 */
#ifndef VKVG_GB300_PMATH_H
#define VKVG_GB300_PMATH_H

#ifdef __CUDACC__
#define PM_FN __host__ __device__ static inline
#else
#define PM_FN static inline
#endif

#include <math.h>

#define PM_PIF   3.14159265358979323846f
#define PM_PIO2F 1.57079632679489661923f
#define PM_PIO4F 0.785398163397448309616f
#define PM_FOPI  1.27323954473516268615f /* 4/pi */

PM_FN unsigned pm__bits(float x) {
    union { float f; unsigned u; } c;
    c.f = x;
    return c.u;
}
PM_FN float pm__from_bits(unsigned u) {
    union { float f; unsigned u; } c;
    c.u = u;
    return c.f;
}
PM_FN float pm_nanf(void) { return pm__from_bits(0x7fc00000u); }
PM_FN int pm_isnan(float x) { return (pm__bits(x) & 0x7fffffffu) > 0x7f800000u; }
PM_FN int pm_isinf(float x) { return (pm__bits(x) & 0x7fffffffu) == 0x7f800000u; }
PM_FN int pm_signbit(float x) { return (int)(pm__bits(x) >> 31); }

/* sin(x) for |x| <= pi/4, z = x*x */
PM_FN float pm__sin_poly(float x, float z) {
    float p = -1.9515295891e-4f * z;
    p = p + 8.3321608736e-3f;
    p = p * z;
    p = p - 1.6666654611e-1f;
    p = p * z;
    p = p * x;
    return p + x;
}
/* cos(x) for |x| <= pi/4, z = x*x */
PM_FN float pm__cos_poly(float z) {
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
PM_FN int pm__reduce(float x, float *r) {
    if (x > 65536.0f) /* far outside the geometry's range: deterministic fold */
        x = fmodf(x, 6.28318548202514648f);
    int j   = (int)(PM_FOPI * x);
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
PM_FN float pm_sinf(float xx) {
    if (pm_isnan(xx))
        return xx;
    if (pm_isinf(xx))
        return pm_nanf();
    int sign = 0;
    float x  = xx;
    if (x < 0.0f) {
        sign = 1;
        x    = -x;
    }
    float r;
    int j = pm__reduce(x, &r);
    if (j > 3) {
        sign ^= 1;
        j -= 4;
    }
    float z = r * r;
    float v = (j == 1 || j == 2) ? pm__cos_poly(z) : pm__sin_poly(r, z);
    return sign ? -v : v;
}
PM_FN float pm_cosf(float xx) {
    if (pm_isnan(xx))
        return xx;
    if (pm_isinf(xx))
        return pm_nanf();
    float x = xx < 0.0f ? -xx : xx;
    float r;
    int j    = pm__reduce(x, &r);
    int sign = 0;
    if (j > 3) {
        j -= 4;
        sign = 1;
    }
    if (j > 1)
        sign ^= 1;
    float z = r * r;
    float v = (j == 1 || j == 2) ? pm__sin_poly(r, z) : pm__cos_poly(z);
    return sign ? -v : v;
}
PM_FN float pm_asinf(float xx) {
    float a = xx < 0.0f ? -xx : xx;
    if (!(a <= 1.0f))
        return pm_nanf();
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
        p = PM_PIO2F - p;
    }
    return xx < 0.0f ? -p : p;
}
PM_FN float pm_acosf(float x) {
    float a = x < 0.0f ? -x : x;
    if (!(a <= 1.0f))
        return pm_nanf();
    if (x < -0.5f)
        return PM_PIF - 2.0f * pm_asinf(sqrtf(0.5f * (1.0f + x)));
    if (x > 0.5f)
        return 2.0f * pm_asinf(sqrtf(0.5f * (1.0f - x)));
    return PM_PIO2F - pm_asinf(x);
}
PM_FN float pm_atanf(float xx) {
    float x = xx < 0.0f ? -xx : xx;
    float y;
    if (x > 2.414213562373095f) {
        y = PM_PIO2F;
        x = -(1.0f / x);
    } else if (x > 0.4142135623730950f) {
        y = PM_PIO4F;
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
PM_FN float pm_atan2f(float y, float x) {
    if (pm_isnan(x) || pm_isnan(y))
        return x + y;
    if (y == 0.0f) {
        if (pm_signbit(x))
            return pm_signbit(y) ? -PM_PIF : PM_PIF;
        return y;
    }
    if (x == 0.0f)
        return y > 0.0f ? PM_PIO2F : -PM_PIO2F;
    if (pm_isinf(x)) {
        if (pm_isinf(y)) {
            float r = x > 0.0f ? PM_PIO4F : 3.0f * PM_PIO4F;
            return y > 0.0f ? r : -r;
        }
        if (x > 0.0f)
            return y > 0.0f ? 0.0f : -0.0f;
        return y > 0.0f ? PM_PIF : -PM_PIF;
    }
    if (pm_isinf(y))
        return y > 0.0f ? PM_PIO2F : -PM_PIO2F;
    float w = 0.0f;
    if (x < 0.0f)
        w = y < 0.0f ? -PM_PIF : PM_PIF;
    float z = pm_atanf(y / x);
    return w + z;
}

#endif
