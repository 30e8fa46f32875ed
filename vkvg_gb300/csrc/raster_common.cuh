/*
 * Pieces shared by the raster kernels: vkvg's source-over blend on
 * premultiplied UNORM8 words, and the bulk-copy staging primitives
 * (cp.async.bulk into shared memory completing mbarrier transactions).
 */
#ifndef VKVG_GB300_RASTER_COMMON_CUH
#define VKVG_GB300_RASTER_COMMON_CUH

#include "gb_types.h"

#include <cuda_runtime.h>
#include <stdint.h>

#define WAIT_LIMIT WAIT_LIMIT_POLLS

#define BM_ADD  0 /* valid premultiplied source: exact on the FMA pipe */
#define BM_SADD 1 /* saturating add */
#define BM_SSUB 2 /* DIFFERENCE: saturating subtract */

struct blend_k {
    uint32_t src, inv;          /* integer modes */
    float    k, c0, c1, c2, c3; /* BM_ADD */
};

/* t = floor((d * inv + 127) / 255) per channel, two channels per 32-bit
   lane: floor(x / 255) = (x + (x >> 8) + 1) >> 8 for x <= 65152 */
__device__ __forceinline__ uint32_t scaled_dst(uint32_t d, uint32_t inv) {
    uint32_t rb = (d & 0x00FF00FFu) * inv + 0x007F007Fu;
    uint32_t ag = ((d >> 8) & 0x00FF00FFu) * inv + 0x007F007Fu;
    rb          = rb + ((rb >> 8) & 0x00FF00FFu) + 0x00010001u;
    ag          = ag + ((ag >> 8) & 0x00FF00FFu) + 0x00010001u;
    return ((rb >> 8) & 0x00FF00FFu) | (ag & 0xFF00FF00u);
}
template <int M> __device__ __forceinline__ uint32_t blend(uint32_t d, const blend_k &B) {
    if (M == BM_ADD) {
        /* byte c of d as the float 2^23 + d_c, then one fmaf per channel */
        const float    z0 = fmaf(__uint_as_float(__byte_perm(d, 0x4B000000u, 0x7440)), B.k, B.c0);
        const float    z1 = fmaf(__uint_as_float(__byte_perm(d, 0x4B000000u, 0x7441)), B.k, B.c1);
        const float    z2 = fmaf(__uint_as_float(__byte_perm(d, 0x4B000000u, 0x7442)), B.k, B.c2);
        const float    z3 = fmaf(__uint_as_float(__byte_perm(d, 0x4B000000u, 0x7443)), B.k, B.c3);
        const uint32_t lo = __byte_perm(__float_as_uint(z0), __float_as_uint(z1), 0x0040);
        const uint32_t hi = __byte_perm(__float_as_uint(z2), __float_as_uint(z3), 0x0040);
        return __byte_perm(lo, hi, 0x5410);
    }
    const uint32_t t = scaled_dst(d, B.inv);
    if (M == BM_SADD)
        return __vaddus4(B.src, t);
    return __vsubus4(B.src, t);
}

__device__ __forceinline__ blend_k make_blend(uint32_t src, uint32_t op, int *mode) {
    blend_k B;
    if (op == GB_OP_CLEAR)
        src = 0u;
    const uint32_t sa  = src >> 24;
    const uint32_t inv = op == GB_OP_CLEAR ? 0u : 255u - sa;
    B.src              = src;
    B.inv              = inv;
    const uint32_t kq  = ((inv << 23) + 127u) / 255u; /* round(inv * 2^23 / 255) <= 2^23 */
    B.k                = (float)kq * (1.0f / 8388608.0f);
    B.c0               = (float)(12582912 + (int32_t)(src & 0xFFu) - (int32_t)kq);
    B.c1               = (float)(12582912 + (int32_t)((src >> 8) & 0xFFu) - (int32_t)kq);
    B.c2               = (float)(12582912 + (int32_t)((src >> 16) & 0xFFu) - (int32_t)kq);
    B.c3               = (float)(12582912 + (int32_t)sa - (int32_t)kq);
    const bool pm      = (src & 0xFFu) <= sa && ((src >> 8) & 0xFFu) <= sa && ((src >> 16) & 0xFFu) <= sa;
    *mode              = op == GB_OP_DIFFERENCE ? BM_SSUB : pm ? BM_ADD : BM_SADD;
    return B;
}

/* gradient draws: every sample has its own premultiplied source word s
   (from the draw's source image), blended with the same exact formula */
__device__ __forceinline__ uint32_t blend_src(uint32_t d, uint32_t s) { return s + scaled_dst(d, 255u - (s >> 24)); }
/* ---- bulk-copy staging (cp.async.bulk + mbarrier transaction counts) */
__device__ __forceinline__ void mbar_init(uint32_t bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_init_n(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
/* one arrival (release: this thread's earlier shared-memory writes are
   visible to a thread whose wait observes the phase complete) */
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
/* thread-level: one copy of `bytes` (multiple of 16, both ends 16-byte
   aligned) from global memory into this CTA's shared memory, completing one
   phase of the mbarrier at bar */
__device__ __forceinline__ void stage_copy(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
/* wait for the phase with the given parity to complete; false after limit polls */
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t limit = WAIT_LIMIT) {
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(bar), "r"(parity)
                     : "memory");
        if (ok)
            return true;
    }
    return false;
}


#endif
