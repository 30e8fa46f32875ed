/*
 * K1 - path flattening on sm_103a.
 *
 * One thread per recorded segment.  A count pass sizes every segment's
 * output, an exclusive scan turns counts into offsets, and an emit pass
 * writes the points (float2) and their per-point flags in path order.
 *
 * Cubic segments follow vkvg's _recursive_bezier
 * (src/vkvg_context_internal.c:1313-1461) through the explicit-stack walk of
 * bezier.cuh, so points come out in exactly the order of the recursive host
 * code.  The translation unit is built with -fmad=false and IEEE division,
 * and the trigonometry comes from pmath.h, so every decision and every
 * coordinate matches the CPU restatement bit for bit.
 */
#include "gb_types.h"
#include "pmath.h"

#include <cuda_runtime.h>

#include "bezier.cuh"

struct gb_count_emit {
    uint32_t n;
    __device__ void operator()(float x, float y, int = 0, float = 0.f, float = 0.f) {
        if (!(x != x || y != y))
            n++;
    }
};
struct gb_write_emit {
    float2  *pts;
    uint8_t *flg;
    uint32_t o, end;
    uint8_t  flag;
    __device__ void operator()(float x, float y, int = 0, float = 0.f, float = 0.f) {
        if (x != x || y != y)
            return;
        if (o < end) {
            pts[o] = make_float2(x, y);
            flg[o] = flag;
        }
        o++;
    }
};

/* the subdivision work cap per cubic (a test hook can lower it) */
__device__ uint32_t g_flatten_node_cap = GB_CURVE_NODE_CAP;

__device__ __forceinline__ bool gb_finite(float v) { return (__float_as_uint(v) & 0x7f800000u) != 0x7f800000u; }

/* Visit every point one segment adds, in order. */
template <class Emit>
__device__ __forceinline__ bool gb_segment_points(uint32_t info, float4 a, float4 b, float4 c, uint32_t n, uint32_t aux,
                                                  const float *__restrict__ thetas, Emit &emit) {
    bool     ok   = true;
    uint32_t kind = GB_SEG_KIND(info);
    if (kind == GB_SEG_POINT) {
        emit(a.x, a.y);
    } else if (kind == GB_SEG_CUBIC) {
        bool fin = gb_finite(a.x) && gb_finite(a.y) && gb_finite(a.z) && gb_finite(a.w) && gb_finite(b.x) &&
                   gb_finite(b.y) && gb_finite(b.z) && gb_finite(b.w);
        if (fin)
            ok = gb_bezier_walk<false>(c.x, a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, emit, g_flatten_node_cap);
        emit(b.z, b.w);
    } else if (kind == GB_SEG_ARC) {
        /* vkvg_arc / vkvg_arc_negative loop, src/vkvg_context.c:424-430 */
        float ang = a.w, step = c.x;
        for (uint32_t k = 0; k < n; k++) {
            emit(pm_cosf(ang) * a.z + a.x, pm_sinf(ang) * a.z + a.y);
            ang = ang + step;
        }
    } else if (kind == GB_SEG_ELLIPSE) {
        /* _elliptic_arc point evaluation, src/vkvg_context_internal.c:1558-1566 */
        for (uint32_t k = 0; k < n; k++) {
            float t  = thetas[aux + k];
            float px = a.z * pm_cosf(t);
            float py = a.w * pm_sinf(t);
            emit((b.x * px + b.y * py) + a.x, (b.z * px + b.w * py) + a.y);
        }
    }
    return ok;
}

/* pass 1: points per segment */
__global__ void gb_flatten_count(uint32_t nseg, const uint32_t *__restrict__ seg_info, const float4 *__restrict__ seg_a,
                                 const float4 *__restrict__ seg_b, const float4 *__restrict__ seg_c,
                                 const uint32_t *__restrict__ seg_n, const uint32_t *__restrict__ seg_aux,
                                 const float *__restrict__ thetas, uint32_t *__restrict__ counts,
                                 uint32_t *__restrict__ status) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nseg)
        return;
    uint32_t      info = seg_info[i];
    gb_count_emit e{0};
    bool ok = gb_segment_points(info, seg_a[i], seg_b[i], seg_c[i], seg_n[i], seg_aux[i], thetas, e);
    if (!ok) {
        atomicOr(status, GB_ERR_CURVE_LIMIT);
        e.n = 0;
    }
    uint32_t cnt = e.n;
    if ((info & GB_SEG_DROP_LAST) && cnt > 0)
        cnt--;
    counts[i] = cnt;
}

/* pass 2: write points at the scanned offsets */
__global__ void gb_flatten_emit(uint32_t nseg, const uint32_t *__restrict__ seg_info, const float4 *__restrict__ seg_a,
                                const float4 *__restrict__ seg_b, const float4 *__restrict__ seg_c,
                                const uint32_t *__restrict__ seg_n, const uint32_t *__restrict__ seg_aux,
                                const float *__restrict__ thetas, const uint32_t *__restrict__ offsets,
                                float2 *__restrict__ pts, uint8_t *__restrict__ pflag) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nseg)
        return;
    uint32_t      info = seg_info[i];
    gb_write_emit e{pts, pflag, offsets[i], offsets[i + 1], (uint8_t)((info & GB_SEG_CURVED) ? 1 : 0)};
    gb_segment_points(info, seg_a[i], seg_b[i], seg_c[i], seg_n[i], seg_aux[i], thetas, e);
}

/* subpath point ranges from the segment offsets */
__global__ void gb_subpath_ranges(uint32_t nsub, const uint32_t *__restrict__ sub_seg0,
                                  const uint32_t *__restrict__ sub_nseg, const uint32_t *__restrict__ seg_off,
                                  uint32_t *__restrict__ sub_pt0, uint32_t *__restrict__ sub_npts) {
    uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nsub)
        return;
    uint32_t a = seg_off[sub_seg0[s]];
    uint32_t b = seg_off[sub_seg0[s] + sub_nseg[s]];
    sub_pt0[s]  = a;
    sub_npts[s] = b - a;
}

/* device evaluation of the portable math, for the host/device identity test */
__global__ void gb_pmath_eval(int fn, const float *__restrict__ a, const float *__restrict__ b, float *__restrict__ out,
                              uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    float r;
    switch (fn) {
    case 0: r = pm_atan2f(a[i], b[i]); break;
    case 1: r = pm_acosf(a[i]); break;
    case 2: r = pm_cosf(a[i]); break;
    case 3: r = pm_sinf(a[i]); break;
    case 4: r = pm_asinf(a[i]); break;
    default: r = pm_atanf(a[i]); break;
    }
    out[i] = r;
}

extern "C" {
/* set the flattening kernels' work cap per cubic (0: the default) */
cudaError_t gb_set_flatten_node_cap(uint32_t cap) {
    const uint32_t v = cap ? cap : GB_CURVE_NODE_CAP;
    return cudaMemcpyToSymbol(g_flatten_node_cap, &v, sizeof(v));
}
cudaError_t gb_launch_pmath_eval(cudaStream_t st, int fn, const float *a, const float *b, float *out, uint64_t n) {
    if (!n)
        return cudaSuccess;
    gb_pmath_eval<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(fn, a, b, out, n);
    return cudaGetLastError();
}
cudaError_t gb_launch_flatten_count(cudaStream_t st, uint32_t nseg, const uint32_t *info, const float4 *a,
                                    const float4 *b, const float4 *c, const uint32_t *n, const uint32_t *aux,
                                    const float *thetas, uint32_t *counts, uint32_t *status) {
    if (!nseg)
        return cudaSuccess;
    gb_flatten_count<<<(nseg + 127) / 128, 128, 0, st>>>(nseg, info, a, b, c, n, aux, thetas, counts, status);
    return cudaGetLastError();
}
cudaError_t gb_launch_flatten_emit(cudaStream_t st, uint32_t nseg, const uint32_t *info, const float4 *a,
                                   const float4 *b, const float4 *c, const uint32_t *n, const uint32_t *aux,
                                   const float *thetas, const uint32_t *offsets, float2 *pts, uint8_t *pflag) {
    if (!nseg)
        return cudaSuccess;
    gb_flatten_emit<<<(nseg + 127) / 128, 128, 0, st>>>(nseg, info, a, b, c, n, aux, thetas, offsets, pts, pflag);
    return cudaGetLastError();
}
cudaError_t gb_launch_subpath_ranges(cudaStream_t st, uint32_t nsub, const uint32_t *sub_seg0,
                                     const uint32_t *sub_nseg, const uint32_t *seg_off, uint32_t *sub_pt0,
                                     uint32_t *sub_npts) {
    if (!nsub)
        return cudaSuccess;
    gb_subpath_ranges<<<(nsub + 255) / 256, 256, 0, st>>>(nsub, sub_seg0, sub_nseg, seg_off, sub_pt0, sub_npts);
    return cudaGetLastError();
}
}
