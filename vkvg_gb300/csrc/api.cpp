/*
 * C ABI of the GB300 vkvg library: devices, surfaces, contexts, the path
 * recorder and state setters.
 *
 * Path commands never flatten on the host.  The recorder keeps vkvg's path
 * semantics (src/vkvg_context.c:341-639, src/vkvg_context_internal.c:132-252)
 * with symbolic point counts: a finite cubic is known to add at least three
 * points (two subdivision halves plus its end point), which decides every
 * count test vkvg makes (< 2 in _finish_path, < 3 and < 4 in close_path).  The
 * cheap, sequential parts that vkvg runs at record time and that later
 * commands depend on - arc step counts, arc and ellipse end points, the
 * elliptic-arc angle walk in double precision, quadratic-to-cubic control
 * points in double - run here with the same portable math the kernels use.
 */
#include "host.h"
#include "launch.h"
#include "pmath.h"

#include <float.h>
#include <math.h>
#include <new>
#include <stdio.h>
#include <stdlib.h>

#define PIF    3.14159265358979323846f
#define PIF_2  1.57079632679489661923f
#define EQUF(a, b) (fabsf((a) - (b)) <= FLT_EPSILON)

/* status sentinels returned instead of NULL on creation failure
   (src/vkvg_internal.h:104-109) */
static vkvg_status_t s_no_memory      = VKVG_STATUS_NO_MEMORY;
static vkvg_status_t s_null_pattern   = VKVG_STATUS_NULL_POINTER;
static vkvg_status_t s_invalid_surf   = VKVG_STATUS_INVALID_SURFACE;
static vkvg_status_t s_device_error   = VKVG_STATUS_DEVICE_ERROR;
static vkvg_status_t s_invalid_dev_ci = VKVG_STATUS_INVALID_DEVICE_CREATE_INFO;

/* ================================================================ matrices */
/* src/vkvg_matrix.c (cairo-derived) */
/* Unpremultiply of vkvg_surface_write_to_memory (src/vkvg_surface.c:393-467,
   the same loop as write_to_png :372-382): p = (uchar)(p / (a / 255.f)),
   evaluated in double.  The result depends only on (a, p), so all 65,536
   cases are evaluated once here with that exact expression and the device
   applies the table.  Where vkvg's conversion is undefined (a == 0, or
   p > a so that the quotient exceeds 255) the table holds 0 / 255. */
const uint8_t *gb_unpremul_table() {
    static uint8_t        t[65536];
    static std::once_flag once;
    std::call_once(once, [] {
        for (uint32_t a = 0; a < 256; a++)
            for (uint32_t p = 0; p < 256; p++) {
                uint8_t r = 0;
                if (a) {
                    double alpha = (double)a / 255.f;
                    double v     = (double)p / alpha;
                    r            = v >= 255.0 ? 255 : (uint8_t)v;
                }
                t[a * 256 + p] = r;
            }
    });
    return t;
}
extern "C" {
void vkvg_matrix_init(vkvg_matrix_t *m, float xx, float yx, float xy, float yy, float x0, float y0) {
    m->xx = xx;
    m->yx = yx;
    m->xy = xy;
    m->yy = yy;
    m->x0 = x0;
    m->y0 = y0;
}
void vkvg_matrix_init_identity(vkvg_matrix_t *m) { vkvg_matrix_init(m, 1, 0, 0, 1, 0, 0); }
void vkvg_matrix_init_translate(vkvg_matrix_t *m, float tx, float ty) { vkvg_matrix_init(m, 1, 0, 0, 1, tx, ty); }
void vkvg_matrix_init_scale(vkvg_matrix_t *m, float sx, float sy) { vkvg_matrix_init(m, sx, 0, 0, sy, 0, 0); }
void vkvg_matrix_init_rotate(vkvg_matrix_t *m, float radians) {
    float s = pm_sinf(radians), c = pm_cosf(radians);
    vkvg_matrix_init(m, c, s, -s, c, 0, 0);
}
void vkvg_matrix_multiply(vkvg_matrix_t *result, const vkvg_matrix_t *a, const vkvg_matrix_t *b) {
    vkvg_matrix_t r;
    r.xx    = a->xx * b->xx + a->yx * b->xy;
    r.yx    = a->xx * b->yx + a->yx * b->yy;
    r.xy    = a->xy * b->xx + a->yy * b->xy;
    r.yy    = a->xy * b->yx + a->yy * b->yy;
    r.x0    = a->x0 * b->xx + a->y0 * b->xy + b->x0;
    r.y0    = a->x0 * b->yx + a->y0 * b->yy + b->y0;
    *result = r;
}
void vkvg_matrix_translate(vkvg_matrix_t *m, float tx, float ty) {
    vkvg_matrix_t t;
    vkvg_matrix_init_translate(&t, tx, ty);
    vkvg_matrix_multiply(m, &t, m);
}
void vkvg_matrix_scale(vkvg_matrix_t *m, float sx, float sy) {
    vkvg_matrix_t t;
    vkvg_matrix_init_scale(&t, sx, sy);
    vkvg_matrix_multiply(m, &t, m);
}
void vkvg_matrix_rotate(vkvg_matrix_t *m, float radians) {
    vkvg_matrix_t t;
    vkvg_matrix_init_rotate(&t, radians);
    vkvg_matrix_multiply(m, &t, m);
}
void vkvg_matrix_transform_distance(const vkvg_matrix_t *m, float *dx, float *dy) {
    float nx = (m->xx * *dx + m->xy * *dy);
    float ny = (m->yx * *dx + m->yy * *dy);
    *dx      = nx;
    *dy      = ny;
}
void vkvg_matrix_transform_point(const vkvg_matrix_t *m, float *x, float *y) {
    vkvg_matrix_transform_distance(m, x, y);
    *x += m->x0;
    *y += m->y0;
}
vkvg_status_t vkvg_matrix_invert(vkvg_matrix_t *m) {
    if (m->xy == 0. && m->yx == 0.) {
        m->x0 = -m->x0;
        m->y0 = -m->y0;
        if (m->xx != 1.f) {
            if (m->xx == 0.)
                return VKVG_STATUS_INVALID_MATRIX;
            m->xx = 1.f / m->xx;
            m->x0 *= m->xx;
        }
        if (m->yy != 1.f) {
            if (m->yy == 0.)
                return VKVG_STATUS_INVALID_MATRIX;
            m->yy = 1.f / m->yy;
            m->y0 *= m->yy;
        }
        return VKVG_STATUS_SUCCESS;
    }
    float det = m->xx * m->yy - m->yx * m->xy;
    if (!(det * det >= 0.))
        return VKVG_STATUS_INVALID_MATRIX;
    if (det == 0)
        return VKVG_STATUS_INVALID_MATRIX;
    float a = m->xx, b = m->yx, c = m->xy, d = m->yy, tx = m->x0, ty = m->y0;
    vkvg_matrix_init(m, d, -b, -c, a, c * ty - d * tx, b * tx - a * ty);
    float s = 1 / det;
    m->xx *= s;
    m->yx *= s;
    m->xy *= s;
    m->yy *= s;
    m->x0 *= s;
    m->y0 *= s;
    return VKVG_STATUS_SUCCESS;
}
void vkvg_matrix_get_scale(const vkvg_matrix_t *m, float *sx, float *sy) {
    *sx = (float)sqrt(m->xx * m->xx + m->xy * m->xy);
    *sy = (float)sqrt(m->yx * m->yx + m->yy * m->yy);
}

/* ================================================================= device */
VkvgDevice vkvg_device_create(vkvg_device_create_info_t *info) {
    if (!info)
        return (VkvgDevice)&s_invalid_dev_ci;
    uint32_t samples = info->samples ? (uint32_t)info->samples : 1u;
    if (samples != 1 && samples != 4)
        return (VkvgDevice)&s_invalid_dev_ci;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) {
        fprintf(stderr, "vkvg_gb300: no CUDA device available\n");
        return (VkvgDevice)&s_device_error;
    }
    _vkvg_device_t *dev = new (std::nothrow) _vkvg_device_t();
    if (!dev)
        return (VkvgDevice)&s_no_memory;
    dev->status = VKVG_STATUS_SUCCESS;
    dev->refs   = 1;
    dev->samples = samples;
    cudaGetDevice(&dev->cuda_dev);
    dev->thread_aware = info->threadAware;
    dev->hdpi = dev->vdpi = 72; /* _device_init, src/vkvg_device.c:71-72 */
    const uint8_t *lut = gb_unpremul_table();
    if (cudaMalloc(&dev->d_unpremul, 65536) != cudaSuccess ||
        cudaMemcpy(dev->d_unpremul, lut, 65536, cudaMemcpyHostToDevice) != cudaSuccess) {
        if (dev->d_unpremul)
            cudaFree(dev->d_unpremul);
        delete dev;
        return (VkvgDevice)&s_no_memory;
    }
    return dev;
}
vkvg_status_t vkvg_device_status(VkvgDevice dev) { return dev ? dev->status : VKVG_STATUS_NULL_POINTER; }
void          vkvg_device_destroy(VkvgDevice dev) {
    if (vkvg_device_status(dev))
        return;
    if (--dev->refs > 0)
        return;
    cudaFree(dev->d_unpremul);
    delete dev;
}
VkvgDevice vkvg_device_reference(VkvgDevice dev) {
    if (!vkvg_device_status(dev))
        dev->refs++;
    return dev;
}
uint32_t vkvg_device_get_reference_count(VkvgDevice dev) { return vkvg_device_status(dev) ? 0 : dev->refs; }
void     vkvg_device_set_dpy(VkvgDevice dev, int h, int v) {
    if (vkvg_device_status(dev))
        return;
    dev->hdpi = h;
    dev->vdpi = v;
}
void vkvg_device_get_dpy(VkvgDevice dev, int *h, int *v) {
    if (vkvg_device_status(dev) || !h || !v)
        return;
    *h = dev->hdpi;
    *v = dev->vdpi;
}
void vkvg_device_set_context_cache_size(VkvgDevice, uint32_t) {}

/* ================================================================ surface */
static VkvgSurface surface_alloc(VkvgDevice dev, uint32_t width, uint32_t height) {
    if (vkvg_device_status(dev))
        return (VkvgSurface)&s_device_error;
    _vkvg_surface_t *s = new (std::nothrow) _vkvg_surface_t();
    if (!s)
        return (VkvgSurface)&s_no_memory;
    s->status  = VKVG_STATUS_SUCCESS;
    s->refs    = 1;
    s->dev     = dev;
    s->width   = width < 1 ? 1 : width;
    s->height  = height < 1 ? 1 : height;
    s->samples = dev->samples;
    s->wpad    = (s->width + 15) & ~15u;
    s->nrows   = s->height * (s->samples == 4 ? 4 : 1);
    s->nbands  = (s->nrows + GB_BAND_ROWS - 1) / GB_BAND_ROWS;
    size_t sb  = (size_t)s->nbands * GB_BAND_ROWS * s->wpad * 4;
    size_t rb  = (size_t)s->width * s->height * 4;
    s->clip_wpr = (s->wpad + 31) / 32;
    s->plane_words = (size_t)s->nbands * GB_BAND_ROWS * s->clip_wpr;
    size_t cb      = s->plane_words * 4;
    if (gb_inject_alloc_fail() || cudaMalloc(&s->d_samples, sb) != cudaSuccess ||
        cudaMalloc(&s->d_rgba, rb) != cudaSuccess ||
        cudaMalloc(&s->d_out, rb) != cudaSuccess || cudaMalloc(&s->d_clip, cb) != cudaSuccess) {
        if (s->d_samples)
            cudaFree(s->d_samples);
        if (s->d_rgba)
            cudaFree(s->d_rgba);
        if (s->d_out)
            cudaFree(s->d_out);
        delete s;
        return (VkvgSurface)&s_no_memory;
    }
    cudaMemset(s->d_samples, 0, sb);
    cudaMemset(s->d_rgba, 0, rb);
    cudaDeviceSynchronize();
    vkvg_device_reference(dev);
    return s;
}
/* vkvg_surface_create, src/vkvg_surface.c:38-52: new surfaces start cleared */
VkvgSurface vkvg_surface_create(VkvgDevice dev, uint32_t width, uint32_t height) {
    return surface_alloc(dev, width, height);
}
/* vkvg_surface_create_from_bitmap, src/vkvg_surface.c:83-152: the RGBA8
   bitmap becomes the surface content (every sample) */
VkvgSurface vkvg_surface_create_from_bitmap(VkvgDevice dev, unsigned char *img, uint32_t width, uint32_t height) {
    if (!img || width == 0 || height == 0)
        return (VkvgSurface)&s_no_memory;
    VkvgSurface s = surface_alloc(dev, width, height);
    if (vkvg_surface_status(s))
        return s;
    size_t                sb = (size_t)s->nbands * GB_BAND_ROWS * s->wpad;
    std::vector<uint32_t> h(sb, 0u);
    uint32_t              rpp = s->samples == 4 ? 4 : 1;
    for (uint32_t y = 0; y < height; y++)
        for (uint32_t x = 0; x < width; x++) {
            uint32_t v;
            memcpy(&v, img + ((size_t)y * width + x) * 4, 4);
            for (uint32_t k = 0; k < rpp; k++)
                h[(size_t)(y * rpp + k) * s->wpad + x] = v;
        }
    cudaMemcpy(s->d_samples, h.data(), sb * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(s->d_rgba, img, (size_t)width * height * 4, cudaMemcpyHostToDevice);
    return s;
}
vkvg_status_t vkvg_surface_status(VkvgSurface s) { return s ? s->status : VKVG_STATUS_NULL_POINTER; }
VkvgSurface   vkvg_surface_reference(VkvgSurface s) {
    if (!vkvg_surface_status(s))
        s->refs++;
    return s;
}
uint32_t vkvg_surface_get_reference_count(VkvgSurface s) { return vkvg_surface_status(s) ? 0 : s->refs; }
void     vkvg_surface_destroy(VkvgSurface s) {
    if (vkvg_surface_status(s))
        return;
    if (--s->refs > 0)
        return;
    cudaFree(s->d_samples);
    cudaFree(s->d_rgba);
    cudaFree(s->d_out);
    cudaFree(s->d_clip);
    s->clip_planes.release();
    VkvgDevice dev = s->dev;
    delete s;
    vkvg_device_destroy(dev);
}
void vkvg_surface_clear(VkvgSurface s) {
    if (vkvg_surface_status(s))
        return;
    std::lock_guard<std::mutex> lk(s->mtx);
    cudaMemset(s->d_samples, 0, (size_t)s->nbands * GB_BAND_ROWS * s->wpad * 4);
    cudaMemset(s->d_rgba, 0, (size_t)s->width * s->height * 4);
    cudaDeviceSynchronize();
}
uint32_t vkvg_surface_get_width(VkvgSurface s) { return vkvg_surface_status(s) ? 0 : s->width; }
uint32_t vkvg_surface_get_height(VkvgSurface s) { return vkvg_surface_status(s) ? 0 : s->height; }
uint32_t vkvg_surface_get_samples(VkvgSurface s) { return vkvg_surface_status(s) ? 0 : s->samples; }
void    *vkvg_surface_get_device_ptr(VkvgSurface s) { return vkvg_surface_status(s) ? nullptr : s->d_rgba; }
void     vkvg_surface_resolve(VkvgSurface) {}

vkvg_status_t vkvg_gb300_surface_read_premult(VkvgSurface s, uint8_t *out) {
    if (vkvg_surface_status(s))
        return VKVG_STATUS_INVALID_STATUS;
    if (!out)
        return VKVG_STATUS_WRITE_ERROR;
    std::lock_guard<std::mutex> lk(s->mtx);
    if (cudaMemcpy(out, s->d_rgba, (size_t)s->width * s->height * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return VKVG_STATUS_DEVICE_ERROR;
    return VKVG_STATUS_SUCCESS;
}
vkvg_status_t vkvg_gb300_surface_read_samples(VkvgSurface s, uint8_t *out) {
    if (vkvg_surface_status(s))
        return VKVG_STATUS_INVALID_STATUS;
    if (!out)
        return VKVG_STATUS_WRITE_ERROR;
    std::lock_guard<std::mutex> lk(s->mtx);
    size_t                sb = (size_t)s->nbands * GB_BAND_ROWS * s->wpad;
    std::vector<uint32_t> h(sb);
    if (cudaMemcpy(h.data(), s->d_samples, sb * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return VKVG_STATUS_DEVICE_ERROR;
    uint32_t rpp = s->samples == 4 ? 4 : 1;
    for (uint32_t y = 0; y < s->height; y++)
        for (uint32_t x = 0; x < s->width; x++)
            for (uint32_t k = 0; k < rpp; k++)
                memcpy(out + (((size_t)y * s->width + x) * rpp + k) * 4, &h[(size_t)(y * rpp + k) * s->wpad + x], 4);
    return VKVG_STATUS_SUCCESS;
}
vkvg_status_t vkvg_surface_write_to_memory(VkvgSurface s, unsigned char *const bitmap) {
    if (vkvg_surface_status(s))
        return VKVG_STATUS_INVALID_STATUS;
    if (!bitmap)
        return VKVG_STATUS_WRITE_ERROR;
    std::lock_guard<std::mutex> lk(s->mtx);
    size_t                      n = (size_t)s->width * s->height;
    if (gb_launch_unpremultiply(0, s->d_rgba, n, s->dev->d_unpremul, s->d_out) != cudaSuccess)
        return VKVG_STATUS_DEVICE_ERROR;
    gb_count_launch(1);
    if (cudaMemcpy(bitmap, s->d_out, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return VKVG_STATUS_DEVICE_ERROR;
    return VKVG_STATUS_SUCCESS;
}
vkvg_status_t vkvg_surface_write_to_png(VkvgSurface s, const char *path) {
    if (vkvg_surface_status(s))
        return VKVG_STATUS_INVALID_STATUS;
    if (!path)
        return VKVG_STATUS_WRITE_ERROR;
    std::vector<uint8_t> img((size_t)s->width * s->height * 4);
    vkvg_status_t        r = vkvg_surface_write_to_memory(s, img.data());
    if (r)
        return r;
    return gb_png_write(path, s->width, s->height, img.data()) ? VKVG_STATUS_WRITE_ERROR : VKVG_STATUS_SUCCESS;
}

/* ================================================================ context */
static void plane_op(VkvgContext ctx, uint32_t kind, uint32_t param);
VkvgContext vkvg_create(VkvgSurface surf) {
    if (vkvg_surface_status(surf))
        return (VkvgContext)&s_invalid_surf;
    if (vkvg_device_status(surf->dev))
        return (VkvgContext)&s_device_error;
    _vkvg_context_t *ctx = new (std::nothrow) _vkvg_context_t();
    if (!ctx)
        return (VkvgContext)&s_no_memory;
    ctx->status = VKVG_STATUS_SUCCESS;
    ctx->refs   = 1;
    ctx->surf   = surf;
    ctx->dev    = surf->dev;
    if (!ctx->pl.init()) {
        const bool oom = ctx->pl.init_oom;
        ctx->pl.destroy();
        delete ctx;
        return (VkvgContext)(oom ? &s_no_memory : &s_device_error);
    }
    vkvg_surface_reference(surf);
    /* a context's first render pass clears the stencil (renderPass_ClearStencil,
       src/vkvg_context.c:43-49) */
    if (surf->clip_active || surf->save_nz)
        plane_op(ctx, GB_DRAW_CLIP_RESET, 0);
    return ctx;
}
vkvg_status_t vkvg_status(VkvgContext ctx) { return !ctx ? VKVG_STATUS_NULL_POINTER : ctx->status; }
VkvgContext   vkvg_reference(VkvgContext ctx) {
    if (!vkvg_status(ctx))
        ctx->refs++;
    return ctx;
}
uint32_t vkvg_get_reference_count(VkvgContext ctx) { return vkvg_status(ctx) ? 0 : ctx->refs; }
}

/* ------------------------------------------------------------- recorder */

static float ctx_arc_step(const VkvgContext ctx, float radius) {
    /* _get_arc_step, src/vkvg_context_internal.c:245-252 */
    float sx, sy;
    vkvg_matrix_get_scale(&ctx->mat, &sx, &sy);
    float r = radius * fabsf(fmaxf(sx, sy));
    if (r < 30.0f)
        return fminf(PIF / 3.f, PIF / r);
    return fminf(PIF / 3.f, PIF / (r * 0.4f));
}
static bool ps_empty(const VkvgContext ctx) { return !ctx->ps.open; }
static bool ps_count_lt(const VkvgContext ctx, uint32_t k) { return ctx->ps.ncubic == 0 && ctx->ps.exact < k; }
static void ps_begin_point(VkvgContext ctx, float x, float y) {
    PathState &p = ctx->ps;
    if (!p.open) {
        p.open  = true;
        p.seg0  = (uint32_t)ctx->frame.seg_info.size();
        p.fx    = x;
        p.fy    = y;
        p.exact = 0;
        p.ncubic = 0;
    }
    p.lx = x;
    p.ly = y;
}
static void push_seg(VkvgContext ctx, uint32_t info, f4 a, f4 b, f4 c, uint32_t n, uint32_t aux) {
    FrameHost &f = ctx->frame;
    f.seg_info.push_back(info);
    f.seg_a.push_back(a);
    f.seg_b.push_back(b);
    f.seg_c.push_back(c);
    f.seg_n.push_back(n);
    f.seg_aux.push_back(aux);
}
/* _add_point (NaN points are dropped) */
static void add_point(VkvgContext ctx, float x, float y) {
    if (isnan(x) || isnan(y))
        return;
    ps_begin_point(ctx, x, y);
    push_seg(ctx, GB_SEG_POINT, f4{x, y, 0, 0}, f4{0, 0, 0, 0}, f4{0, 0, 0, 0}, 1, 0);
    ctx->ps.exact++;
}
/* _set_curve_start / _set_curve_end: points recorded in between belong to a
   curve segment (curve joins in strokes) */
static void curve_start(VkvgContext ctx) {
    ctx->ps.pending      = true;
    ctx->ps.pending_from = (uint32_t)ctx->frame.seg_info.size();
}
static void curve_end(VkvgContext ctx) {
    FrameHost &f = ctx->frame;
    if (ctx->ps.pending)
        for (size_t i = ctx->ps.pending_from; i < f.seg_info.size(); i++)
            f.seg_info[i] |= GB_SEG_CURVED;
    ctx->ps.pending = false;
}
static void ps_reset(VkvgContext ctx) {
    PathState &p = ctx->ps;
    p.open       = false;
    p.closed     = false;
    p.pending    = false;
    p.exact = p.ncubic = 0;
}
/* _finish_path, src/vkvg_context_internal.c:163-197 */
static void finish_path(VkvgContext ctx) {
    PathState &p = ctx->ps;
    if (!p.open)
        return;
    FrameHost &f = ctx->frame;
    if (ps_count_lt(ctx, 2)) {
        size_t n = p.seg0;
        f.seg_info.resize(n);
        f.seg_a.resize(n);
        f.seg_b.resize(n);
        f.seg_c.resize(n);
        f.seg_n.resize(n);
        f.seg_aux.resize(n);
        ps_reset(ctx);
        return;
    }
    f.sub_seg0.push_back(p.seg0);
    f.sub_nseg.push_back((uint32_t)f.seg_info.size() - p.seg0);
    f.sub_flags.push_back(p.closed ? GB_SUB_CLOSED : 0u);
    ps_reset(ctx);
}
/* _clear_path */
static void clear_path(VkvgContext ctx) {
    PathState &p = ctx->ps;
    if (p.open) {
        FrameHost &f = ctx->frame;
        size_t     n = p.seg0;
        f.seg_info.resize(n);
        f.seg_a.resize(n);
        f.seg_b.resize(n);
        f.seg_c.resize(n);
        f.seg_n.resize(n);
        f.seg_aux.resize(n);
    }
    ps_reset(ctx);
    p.path_sub0 = (uint32_t)ctx->frame.sub_seg0.size();
}
/* _line_to, src/vkvg_context_internal.c:1463-1472 */
static void line_to_i(VkvgContext ctx, float x, float y) {
    if (!ps_empty(ctx)) {
        if (EQUF(ctx->ps.lx, x) && EQUF(ctx->ps.ly, y))
            return;
    }
    add_point(ctx, x, y);
}
static bool finite8(float a, float b, float c, float d, float e, float f, float g, float h) {
    return isfinite(a) && isfinite(b) && isfinite(c) && isfinite(d) && isfinite(e) && isfinite(f) && isfinite(g) &&
           isfinite(h);
}
/* _curve_to, src/vkvg_context.c:541-566 */
static void curve_to_i(VkvgContext ctx, float x1, float y1, float x2, float y2, float x3, float y3) {
    if (EQUF(x1, x2) && EQUF(x2, x3) && EQUF(y1, y2) && EQUF(y2, y3)) {
        if (ps_empty(ctx) || (EQUF(ctx->ps.lx, x1) && EQUF(ctx->ps.ly, y1)))
            return;
    }
    curve_start(ctx);
    if (ps_empty(ctx))
        add_point(ctx, x1, y1);
    if (ps_empty(ctx)) { /* x1 or y1 NaN: vkvg would read a stale point */
        curve_end(ctx);
        return;
    }
    float cx = ctx->ps.lx, cy = ctx->ps.ly;
    float sx = 1, sy = 1;
    vkvg_matrix_get_scale(&ctx->mat, &sx, &sy);
    float tol = (float)fabs(0.25f / fmaxf(sx, sy));
    bool  fin = finite8(cx, cy, x1, y1, x2, y2, x3, y3);
    bool  end = !(isnan(x3) || isnan(y3));
    if (fin || end) {
        push_seg(ctx, GB_SEG_CUBIC, f4{cx, cy, x1, y1}, f4{x2, y2, x3, y3}, f4{tol, 0, 0, 0}, 0, 0);
        if (fin)
            ctx->ps.ncubic++;
        else
            ctx->ps.exact++;
        if (end) {
            ctx->ps.lx = x3;
            ctx->ps.ly = y3;
        }
    }
    curve_end(ctx);
}
static void quadratic_to_i(VkvgContext ctx, float x1, float y1, float x2, float y2) {
    static const double qf = 2.0 / 3.0; /* src/vkvg_context.c:567 */
    float               x0, y0;
    if (ps_empty(ctx)) {
        x0 = x1;
        y0 = y1;
    } else {
        x0 = ctx->ps.lx;
        y0 = ctx->ps.ly;
    }
    curve_to_i(ctx, (float)(x0 + (x1 - x0) * qf), (float)(y0 + (y1 - y0) * qf), (float)(x2 + (x1 - x2) * qf),
               (float)(y2 + (y1 - y2) * qf), x2, y2);
}

/* vkvg_close_path, src/vkvg_context.c:350-373 */
static void close_path_i(VkvgContext ctx) {
    PathState &p = ctx->ps;
    if (!p.open || ps_count_lt(ctx, 3))
        return;
    if (EQUF(p.lx, p.fx) && EQUF(p.ly, p.fy)) {
        if (ps_count_lt(ctx, 4))
            return;
        /* _remove_last_point: the last recorded segment drops its last point */
        ctx->frame.seg_info.back() |= GB_SEG_DROP_LAST;
    }
    p.closed = true;
    finish_path(ctx);
}

static const uint32_t ARC_LOOP_CAP = 1u << 24;

/* vkvg_arc (src/vkvg_context.c:394-449) and vkvg_arc_negative (:450-503) */
static void arc_i(VkvgContext ctx, float xc, float yc, float radius, float a1, float a2, bool neg) {
    if (!neg) {
        while (a2 < a1)
            a2 += 2.f * PIF;
        if (a2 - a1 > 2.f * PIF)
            a2 = a1 + 2.f * PIF;
    } else {
        while (a2 > a1)
            a2 -= 2.f * PIF;
        if (a1 - a2 > a1 + 2.f * PIF) /* kept as written in vkvg */
            a2 = a1 - 2.f * PIF;
    }
    float vx   = pm_cosf(a1) * radius + xc;
    float vy   = pm_sinf(a1) * radius + yc;
    float step = ctx_arc_step(ctx, radius);
    float a    = a1;
    if (ps_empty(ctx)) {
        curve_start(ctx);
        add_point(ctx, vx, vy);
    } else {
        line_to_i(ctx, vx, vy);
        curve_start(ctx);
    }
    float sstep = neg ? -step : step;
    a           = a + sstep;
    if (EQUF(a2, a1))
        return; /* vkvg leaves the curve segment open here */
    float    a0 = a, alast = a;
    uint32_t n = 0;
    while (neg ? (a > a2) : (a < a2)) {
        if (++n > ARC_LOOP_CAP) {
            ctx->status = VKVG_STATUS_INVALID_STATUS;
            return;
        }
        alast = a;
        a     = a + sstep;
    }
    if (n) {
        float lx = pm_cosf(alast) * radius + xc, ly = pm_sinf(alast) * radius + yc;
        bool  nanv = isnan(lx) || isnan(ly);
        if (!nanv) {
            ps_begin_point(ctx, lx, ly);
            push_seg(ctx, GB_SEG_ARC, f4{xc, yc, radius, a0}, f4{0, 0, 0, 0}, f4{sstep, 0, 0, 0}, n, 0);
            ctx->ps.exact += n;
        }
    }
    if (neg ? EQUF(a1 - a2, PIF * 2.f) : EQUF(a2 - a1, PIF * 2.f)) {
        curve_end(ctx);
        close_path_i(ctx);
        return;
    }
    add_point(ctx, pm_cosf(a2) * radius + xc, pm_sinf(a2) * radius + yc);
    curve_end(ctx);
}

/* _elliptic_arc, src/vkvg_context_internal.c:1473-1580.  The angle walk runs
   in double exactly as in vkvg; the kernels evaluate the points. */
static void elliptic_arc_i(VkvgContext ctx, float x1, float y1, float x2, float y2, bool largeArc,
                           bool counterClockWise, float _rx, float _ry, float phi) {
    if (ctx->status)
        return;
    if (_rx == 0 || _ry == 0) {
        if (ps_empty(ctx)) {
            finish_path(ctx);
            add_point(ctx, x1, y1);
        }
        line_to_i(ctx, x2, y2);
        return;
    }
    float rx = fabsf(_rx), ry = fabsf(_ry);
    float cph = pm_cosf(phi), sph = pm_sinf(phi);
    float p1x = (cph * ((x1 - x2) / 2)) + (sph * ((y1 - y2) / 2));
    float p1y = (-sph * ((x1 - x2) / 2)) + (cph * ((y1 - y2) / 2));
    double lambda = (p1x * p1x) / (rx * rx) + (p1y * p1y) / (ry * ry);
    if (lambda > 1) {
        lambda = sqrtf((float)lambda);
        rx     = (float)(rx * lambda);
        ry     = (float)(ry * lambda);
    }
    float px = rx * p1y / ry, py = -ry * p1x / rx;
    float rx2 = rx * rx, ry2 = ry * ry, p1x2 = p1x * p1x, p1y2 = p1y * p1y;
    float k   = sqrtf(fabsf((rx2 * ry2 - rx2 * p1y2 - ry2 * p1x2) / (rx2 * p1y2 + ry2 * p1x2)));
    float cpx = px * k, cpy = py * k;
    if (largeArc == counterClockWise) {
        cpx = -cpx;
        cpy = -cpy;
    }
    /* m = {{cos, -sin}, {sin, cos}} */
    float m00 = cph, m01 = -sph, m10 = sph, m11 = cph;
    float cx = ((m00 * cpx) + (m01 * cpy)) + (x1 + x2) / 2;
    float cy = ((m10 * cpx) + (m11 * cpy)) + (y1 + y2) / 2;
    float ux = 1.f, uy = 0;
    float vx = (p1x - cpx) / rx, vy = (p1y - cpy) / ry;
    auto  len = [](float a, float b) { return sqrtf(a * a + b * b); };
    double sa = pm_acosf(((ux * vx) + (uy * vy)) / (fabsf(len(vx, vy)) * fabsf(len(ux, uy))));
    if (isnan(sa))
        sa = PIF;
    if (ux * vy - uy * vx < 0)
        sa = -sa;
    ux = vx;
    uy = vy;
    vx = (-p1x - cpx) / rx;
    vy = (-p1y - cpy) / ry;
    double dt = pm_acosf(((ux * vx) + (uy * vy)) / (fabsf(len(vx, vy)) * fabsf(len(ux, uy))));
    if (isnan(dt))
        dt = PIF;
    if (ux * vy - uy * vx < 0)
        dt = -dt;
    if (counterClockWise) {
        if (dt < 0)
            dt += PIF * 2.0;
    } else if (dt > 0)
        dt -= PIF * 2.0;
    double theta = sa, ea = sa + dt;
    float  step = fmaxf(0.001f, fminf(PIF, ctx_arc_step(ctx, fminf(rx, ry)) * 0.1f));
    auto   pt   = [&](float t, float *ox, float *oy) {
        float qx = rx * pm_cosf(t), qy = ry * pm_sinf(t);
        *ox      = (m00 * qx + m01 * qy) + cx;
        *oy      = (m10 * qx + m11 * qy) + cy;
    };
    float fx, fy;
    pt((float)theta, &fx, &fy);
    if (ps_empty(ctx)) {
        curve_start(ctx);
        add_point(ctx, fx, fy);
    } else {
        line_to_i(ctx, fx, fy);
        curve_start(ctx);
    }
    curve_start(ctx); /* vkvg calls _set_curve_start twice */
    FrameHost &f    = ctx->frame;
    uint32_t   aux  = (uint32_t)f.thetas.size();
    uint32_t   n    = 0;
    if (sa < ea) {
        theta += step;
        while (theta < ea) {
            f.thetas.push_back((float)theta);
            n++;
            theta += step;
        }
    } else {
        theta -= step;
        while (theta > ea) {
            f.thetas.push_back((float)theta);
            n++;
            theta -= step;
        }
    }
    if (n) {
        float lx, ly;
        pt(f.thetas.back(), &lx, &ly);
        if (!(isnan(lx) || isnan(ly))) {
            ps_begin_point(ctx, lx, ly);
            push_seg(ctx, GB_SEG_ELLIPSE, f4{cx, cy, rx, ry}, f4{m00, m01, m10, m11}, f4{0, 0, 0, 0}, n, aux);
            ctx->ps.exact += n;
        }
    }
    float ex, ey;
    pt((float)ea, &ex, &ey);
    add_point(ctx, ex, ey);
    curve_end(ctx);
}

/* premultiplied source word: vertex colour (byte 0 = R) times opacity,
   rounded to UNORM8 as the fragment output */
uint32_t gb_source_word(uint32_t color, float opacity) {
    uint32_t out = 0;
    for (int c = 0; c < 4; c++) {
        uint32_t b = (color >> (8 * c)) & 0xFF;
        float    v = (((float)b / 255.0f) * opacity) * 255.0f;
        if (!(v > 0.0f))
            v = 0.0f;
        if (v > 255.0f)
            v = 255.0f;
        out |= ((uint32_t)lrintf(v) & 0xFF) << (8 * c);
    }
    return out;
}

static void flush_i(VkvgContext ctx);
/* the frame's source image for the context's gradient at the current
   opacity, added if new; a frame holding GB_MAX_GRAD_SOURCES of them is
   flushed first (the current path carries over) */
static uint32_t grad_source(VkvgContext ctx) {
    gb_grad g = ctx->grad_snap;
    g.opacity = ctx->opacity;
    VkvgSurface src = nullptr;
    if (g.type == GB_SRC_SURFACE) {
        /* the push constants as this draw pushes them */
        const vkvg_matrix_t &m = ctx->mat_inv;
        const float          mv[6] = {m.xx, m.yx, m.xy, m.yy, m.x0, m.y0};
        memcpy(g.m, mv, sizeof(mv));
        g.ox = ctx->src_x;
        g.oy = ctx->src_y;
        src  = ctx->pattern->surf;
    }
    std::vector<gb_grad> &v = ctx->frame.grads;
    for (size_t i = 0; i < v.size(); i++)
        if (memcmp(&v[i], &g, sizeof(g)) == 0)
            return (uint32_t)i + 1;
    if (v.size() >= GB_MAX_GRAD_SOURCES)
        flush_i(ctx);
    ctx->frame.grads.push_back(g);
    if (src)
        ctx->frame.sources.emplace_back(src);
    return (uint32_t)ctx->frame.grads.size();
}
static gb_draw make_draw(VkvgContext ctx, uint32_t kind) {
    const bool     paints = kind <= GB_DRAW_PAINT; /* clip draws and clears have no source */
    const uint32_t gsrc   = paints && ctx->grad_on ? grad_source(ctx) : 0u;
    gb_draw        d;
    memset(&d, 0, sizeof(d));
    d.gsrc      = gsrc;
    d.kind      = kind;
    d.op        = (uint32_t)ctx->op;
    d.join      = (uint32_t)ctx->line_join;
    d.cap       = (uint32_t)ctx->line_cap;
    d.src       = gb_source_word(ctx->cur_color, ctx->opacity);
    d.sub_first = ctx->ps.path_sub0;
    d.sub_count = (uint32_t)ctx->frame.sub_seg0.size() - ctx->ps.path_sub0;
    d.hw        = ctx->line_width * 0.5f;
    d.lh_max    = ctx->miter_limit * ctx->line_width;
    d.arc_step  = ctx_arc_step(ctx, d.hw);
    d.mat[0]    = ctx->mat.xx;
    d.mat[1]    = ctx->mat.yx;
    d.mat[2]    = ctx->mat.xy;
    d.mat[3]    = ctx->mat.yy;
    d.mat[4]    = ctx->mat.x0;
    d.mat[5]    = ctx->mat.y0;
    return d;
}
/* _fill_preserve, src/vkvg_context.c:796-821 */
static void fill_preserve_i(VkvgContext ctx) {
    finish_path(ctx);
    FrameHost &f = ctx->frame;
    if (f.sub_seg0.size() == ctx->ps.path_sub0)
        return;
    gb_draw  d  = make_draw(ctx, ctx->fill_rule == VKVG_FILL_RULE_EVEN_ODD ? GB_DRAW_FILL_EO : GB_DRAW_FILL_NZ);
    uint32_t di = (uint32_t)f.draws.size();
    f.draws.push_back(d);
    for (uint32_t s = d.sub_first; s < d.sub_first + d.sub_count; s++) {
        f.fpair_draw.push_back(di);
        f.fpair_sub.push_back(s);
    }
    f.paths++;
}
/* the fill geometry of _clip_preserve (src/vkvg_context.c:754-795): the
   current path as an even-odd or non-zero region that the clip keeps */
static bool clip_preserve_i(VkvgContext ctx) {
    finish_path(ctx);
    FrameHost &f = ctx->frame;
    if (f.sub_seg0.size() == ctx->ps.path_sub0)
        return false;
    gb_draw  d  = make_draw(ctx, ctx->fill_rule == VKVG_FILL_RULE_EVEN_ODD ? GB_DRAW_CLIP_EO : GB_DRAW_CLIP_NZ);
    uint32_t di = (uint32_t)f.draws.size();
    f.draws.push_back(d);
    for (uint32_t s = d.sub_first; s < d.sub_first + d.sub_count; s++) {
        f.fpair_draw.push_back(di);
        f.fpair_sub.push_back(s);
    }
    return true;
}
/* a stencil plane operation (GB_DRAW_CLIP_RESET ... GB_DRAW_CLIP_LOAD) */
static void plane_op(VkvgContext ctx, uint32_t kind, uint32_t param) {
    gb_draw d;
    memset(&d, 0, sizeof(d));
    d.kind      = kind;
    d.src       = param;
    d.sub_first = (uint32_t)ctx->frame.sub_seg0.size();
    ctx->frame.draws.push_back(d);
}
/* _stroke_preserve, src/vkvg_context.c:822-948 */
static void stroke_preserve_i(VkvgContext ctx) {
    finish_path(ctx);
    FrameHost &f = ctx->frame;
    if (f.sub_seg0.size() == ctx->ps.path_sub0)
        return;
    gb_draw d = make_draw(ctx, GB_DRAW_STROKE);
    if (!ctx->dashes.empty()) {
        float tot = 0;
        for (float v : ctx->dashes)
            tot += v;
        if (tot == 0) {
            ctx->status = VKVG_STATUS_INVALID_DASH;
            return;
        }
        d.dash_first  = (uint32_t)f.dashes.size();
        d.dash_count  = (uint32_t)ctx->dashes.size();
        d.dash_offset = ctx->dash_offset;
        f.dashes.insert(f.dashes.end(), ctx->dashes.begin(), ctx->dashes.end());
        f.any_dash = true;
        if (d.sub_first < f.dash_sub_hi)
            f.dash_shared = true; /* e.g. stroke_preserve then stroke, both dashed */
        f.dash_sub_hi = std::max(f.dash_sub_hi, d.sub_first + d.sub_count);
    }
    uint32_t di = (uint32_t)f.draws.size();
    f.draws.push_back(d);
    if (f.sdraw_pair0.empty())
        f.sdraw_pair0.push_back(0);
    uint32_t p0 = (uint32_t)f.spair_draw.size();
    for (uint32_t s = d.sub_first; s < d.sub_first + d.sub_count; s++) {
        f.spair_draw.push_back(di);
        f.spair_sub.push_back(s);
        f.spair_dfirst.push_back(p0);
    }
    f.sdraw_id.push_back(di);
    f.sdraw_pair0.back() = p0;
    f.sdraw_pair0.push_back((uint32_t)f.spair_draw.size());
    f.paths++;
}

static void flush_i(VkvgContext ctx) {
    if (ctx->frame.empty())
        return;
    vkvg_status_t r = gb_run_frame(ctx->pl, ctx->frame, ctx->surf, true, false);
    ctx->have_run   = true;
    if (r)
        ctx->status = r;
    /* subpaths of the current path survive a flush (vkvg keeps its path) */
    FrameHost keep;
    PathState &p = ctx->ps;
    uint32_t   s0 = p.path_sub0, s1 = (uint32_t)ctx->frame.sub_seg0.size();
    FrameHost &f  = ctx->frame;
    uint32_t   segA = s0 < s1 ? f.sub_seg0[s0] : (p.open ? p.seg0 : (uint32_t)f.seg_info.size());
    uint32_t   segB = (uint32_t)f.seg_info.size();
    for (uint32_t i = segA; i < segB; i++) {
        keep.seg_info.push_back(f.seg_info[i]);
        keep.seg_a.push_back(f.seg_a[i]);
        keep.seg_b.push_back(f.seg_b[i]);
        keep.seg_c.push_back(f.seg_c[i]);
        keep.seg_n.push_back(f.seg_n[i]);
        uint32_t aux = f.seg_aux[i];
        if (GB_SEG_KIND(f.seg_info[i]) == GB_SEG_ELLIPSE) {
            uint32_t na = (uint32_t)keep.thetas.size();
            keep.thetas.insert(keep.thetas.end(), f.thetas.begin() + aux, f.thetas.begin() + aux + f.seg_n[i]);
            aux = na;
        }
        keep.seg_aux.push_back(aux);
    }
    for (uint32_t s = s0; s < s1; s++) {
        keep.sub_seg0.push_back(f.sub_seg0[s] - segA);
        keep.sub_nseg.push_back(f.sub_nseg[s]);
        keep.sub_flags.push_back(f.sub_flags[s]);
    }
    ctx->frame.clear();
    FrameHost &n = ctx->frame;
    n.seg_info   = std::move(keep.seg_info);
    n.seg_a      = std::move(keep.seg_a);
    n.seg_b      = std::move(keep.seg_b);
    n.seg_c      = std::move(keep.seg_c);
    n.seg_n      = std::move(keep.seg_n);
    n.seg_aux    = std::move(keep.seg_aux);
    n.thetas     = std::move(keep.thetas);
    n.sub_seg0   = std::move(keep.sub_seg0);
    n.sub_nseg   = std::move(keep.sub_nseg);
    n.sub_flags  = std::move(keep.sub_flags);
    if (p.open)
        p.seg0 -= segA;
    if (p.pending)
        p.pending_from = p.pending_from >= segA ? p.pending_from - segA : 0;
    p.path_sub0 = 0;
}

extern "C" {
/* vkvg_flush, src/vkvg_context.c:180-184 (blocking) */
void vkvg_flush(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    flush_i(ctx);
}
static void set_solid(VkvgContext ctx);
void        vkvg_destroy(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    if (--ctx->refs > 0)
        return;
    flush_i(ctx);
    set_solid(ctx);
    for (gb_saved_state &sv : ctx->saved)
        if (sv.pattern)
            vkvg_pattern_destroy(sv.pattern);
    ctx->pl.destroy();
    VkvgSurface s = ctx->surf;
    delete ctx;
    vkvg_surface_destroy(s);
}
const char *vkvg_status_to_string(vkvg_status_t status) {
    switch (status) {
    case VKVG_STATUS_SUCCESS: return "no error has occurred";
    case VKVG_STATUS_NO_MEMORY: return "out of memory";
    case VKVG_STATUS_NULL_POINTER: return "NULL pointer";
    case VKVG_STATUS_INVALID_RESTORE: return "vkvg_restore() without matching vkvg_save()";
    case VKVG_STATUS_NO_CURRENT_POINT: return "no current point defined";
    case VKVG_STATUS_INVALID_MATRIX: return "invalid matrix (not invertible)";
    case VKVG_STATUS_INVALID_STATUS: return "invalid value for an input vkvg_status_t";
    case VKVG_STATUS_INVALID_INDEX: return "invalid index passed to getter";
    case VKVG_STATUS_WRITE_ERROR: return "error while writing to output stream";
    case VKVG_STATUS_PATTERN_TYPE_MISMATCH: return "the pattern type is not appropriate for the operation";
    case VKVG_STATUS_PATTERN_INVALID_GRADIENT: return "the stops count is zero";
    case VKVG_STATUS_INVALID_FORMAT: return "invalid value for an input vkvg_format_t";
    case VKVG_STATUS_FILE_NOT_FOUND: return "file not found";
    case VKVG_STATUS_INVALID_DASH: return "invalid value for a dash setting";
    case VKVG_STATUS_INVALID_RECT: return "a rectangle has the height or width equal to 0";
    case VKVG_STATUS_TIMEOUT: return "waiting for a GPU operation to finish timed out";
    case VKVG_STATUS_DEVICE_ERROR: return "a CUDA device operation failed";
    case VKVG_STATUS_INVALID_IMAGE: return "invalid image";
    case VKVG_STATUS_INVALID_SURFACE: return "invalid surface";
    case VKVG_STATUS_INVALID_FONT: return "unresolved font name";
    default: return "<unknown error status>";
    }
}

void vkvg_new_path(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    clear_path(ctx);
}
void vkvg_new_sub_path(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    finish_path(ctx);
}
void vkvg_close_path(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    close_path_i(ctx);
}
void vkvg_rel_line_to(VkvgContext ctx, float dx, float dy) {
    if (vkvg_status(ctx))
        return;
    if (ps_empty(ctx))
        add_point(ctx, 0, 0);
    line_to_i(ctx, ctx->ps.lx + dx, ctx->ps.ly + dy);
}
void vkvg_line_to(VkvgContext ctx, float x, float y) {
    if (vkvg_status(ctx))
        return;
    line_to_i(ctx, x, y);
}
void vkvg_arc(VkvgContext ctx, float xc, float yc, float radius, float a1, float a2) {
    if (vkvg_status(ctx))
        return;
    arc_i(ctx, xc, yc, radius, a1, a2, false);
}
void vkvg_arc_negative(VkvgContext ctx, float xc, float yc, float radius, float a1, float a2) {
    if (vkvg_status(ctx))
        return;
    arc_i(ctx, xc, yc, radius, a1, a2, true);
}
void vkvg_rel_move_to(VkvgContext ctx, float x, float y) {
    if (vkvg_status(ctx))
        return;
    if (ps_empty(ctx))
        add_point(ctx, 0, 0);
    float cx = ctx->ps.lx, cy = ctx->ps.ly;
    finish_path(ctx);
    add_point(ctx, cx + x, cy + y);
}
void vkvg_move_to(VkvgContext ctx, float x, float y) {
    if (vkvg_status(ctx))
        return;
    finish_path(ctx);
    add_point(ctx, x, y);
}
bool vkvg_has_current_point(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return false;
    return !ps_empty(ctx);
}
void vkvg_get_current_point(VkvgContext ctx, float *x, float *y) {
    if (vkvg_status(ctx) || !x || !y)
        return;
    if (ps_empty(ctx)) {
        *x = *y = 0;
        return;
    }
    *x = ctx->ps.lx;
    *y = ctx->ps.ly;
}
void vkvg_curve_to(VkvgContext ctx, float x1, float y1, float x2, float y2, float x3, float y3) {
    if (vkvg_status(ctx))
        return;
    curve_to_i(ctx, x1, y1, x2, y2, x3, y3);
}
void vkvg_rel_curve_to(VkvgContext ctx, float x1, float y1, float x2, float y2, float x3, float y3) {
    if (vkvg_status(ctx))
        return;
    if (ps_empty(ctx)) {
        ctx->status = VKVG_STATUS_NO_CURRENT_POINT;
        return;
    }
    float cx = ctx->ps.lx, cy = ctx->ps.ly;
    curve_to_i(ctx, cx + x1, cy + y1, cx + x2, cy + y2, cx + x3, cy + y3);
}
void vkvg_quadratic_to(VkvgContext ctx, float x1, float y1, float x2, float y2) {
    if (vkvg_status(ctx))
        return;
    quadratic_to_i(ctx, x1, y1, x2, y2);
}
/* vkvg reads a stale point here without a current point; this library
   reports VKVG_STATUS_NO_CURRENT_POINT as vkvg_rel_curve_to does */
void vkvg_rel_quadratic_to(VkvgContext ctx, float x1, float y1, float x2, float y2) {
    if (vkvg_status(ctx))
        return;
    if (ps_empty(ctx)) {
        ctx->status = VKVG_STATUS_NO_CURRENT_POINT;
        return;
    }
    float cx = ctx->ps.lx, cy = ctx->ps.ly;
    quadratic_to_i(ctx, cx + x1, cy + y1, cx + x2, cy + y2);
}
vkvg_status_t vkvg_rectangle(VkvgContext ctx, float x, float y, float w, float h) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    finish_path(ctx);
    if (w <= 0 || h <= 0)
        return VKVG_STATUS_INVALID_RECT;
    add_point(ctx, x, y);
    add_point(ctx, x + w, y);
    add_point(ctx, x + w, y + h);
    add_point(ctx, x, y + h);
    if (ctx->ps.open) /* vkvg would flag an empty subpath here (NaN corners) */
        ctx->ps.closed = true;
    finish_path(ctx);
    return VKVG_STATUS_SUCCESS;
}
vkvg_status_t vkvg_rounded_rectangle(VkvgContext ctx, float x, float y, float w, float h, float radius) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    finish_path(ctx);
    if (w <= 0 || h <= 0)
        return VKVG_STATUS_INVALID_RECT;
    if ((radius > w / 2.0f) || (radius > h / 2.0f))
        radius = (float)fmin(w / 2.0f, h / 2.0f);
    vkvg_move_to(ctx, x, y + radius);
    vkvg_arc(ctx, x + radius, y + radius, radius, PIF, -PIF_2);
    vkvg_line_to(ctx, x + w - radius, y);
    vkvg_arc(ctx, x + w - radius, y + radius, radius, -PIF_2, 0);
    vkvg_line_to(ctx, x + w, y + h - radius);
    vkvg_arc(ctx, x + w - radius, y + h - radius, radius, 0, PIF_2);
    vkvg_line_to(ctx, x + radius, y + h);
    vkvg_arc(ctx, x + radius, y + h - radius, radius, PIF_2, PIF);
    vkvg_line_to(ctx, x, y + radius);
    vkvg_close_path(ctx);
    return VKVG_STATUS_SUCCESS;
}
void vkvg_rounded_rectangle2(VkvgContext ctx, float x, float y, float w, float h, float rx, float ry) {
    if (vkvg_status(ctx))
        return;
    vkvg_move_to(ctx, x + rx, y);
    vkvg_line_to(ctx, x + w - rx, y);
    vkvg_elliptic_arc_to(ctx, x + w, y + ry, false, true, rx, ry, 0);
    vkvg_line_to(ctx, x + w, y + h - ry);
    vkvg_elliptic_arc_to(ctx, x + w - rx, y + h, false, true, rx, ry, 0);
    vkvg_line_to(ctx, x + rx, y + h);
    vkvg_elliptic_arc_to(ctx, x, y + h - ry, false, true, rx, ry, 0);
    vkvg_line_to(ctx, x, y + ry);
    vkvg_elliptic_arc_to(ctx, x + rx, y, false, true, rx, ry, 0);
    vkvg_close_path(ctx);
}
void vkvg_elliptic_arc_to(VkvgContext ctx, float x2, float y2, bool large, bool sweep, float rx, float ry,
                          float phi) {
    if (vkvg_status(ctx))
        return;
    float x1, y1;
    vkvg_get_current_point(ctx, &x1, &y1);
    elliptic_arc_i(ctx, x1, y1, x2, y2, large, sweep, rx, ry, phi);
}
void vkvg_rel_elliptic_arc_to(VkvgContext ctx, float x2, float y2, bool large, bool sweep, float rx, float ry,
                              float phi) {
    if (vkvg_status(ctx))
        return;
    float x1, y1;
    vkvg_get_current_point(ctx, &x1, &y1);
    elliptic_arc_i(ctx, x1, y1, x2 + x1, y2 + y1, large, sweep, rx, ry, phi);
}
/* vkvg_ellipse, src/vkvg_context.c:1605-1639 */
void vkvg_ellipse(VkvgContext ctx, float radiusX, float radiusY, float x, float y, float rotationAngle) {
    if (vkvg_status(ctx))
        return;
    float w23 = radiusX * 4 / 3;
    float dx1 = pm_sinf(rotationAngle) * radiusY;
    float dy1 = pm_cosf(rotationAngle) * radiusY;
    float dx2 = pm_cosf(rotationAngle) * w23;
    float dy2 = pm_sinf(rotationAngle) * w23;
    float tcx = x - dx1, tcy = y + dy1;
    float trx = tcx + dx2, try_ = tcy + dy2;
    float tlx = tcx - dx2, tly = tcy - dy2;
    float bcx = x + dx1, bcy = y - dy1;
    float brx = bcx + dx2, bry = bcy + dy2;
    float blx = bcx - dx2, bly = bcy - dy2;
    finish_path(ctx);
    add_point(ctx, bcx, bcy);
    curve_to_i(ctx, brx, bry, trx, try_, tcx, tcy);
    curve_to_i(ctx, tlx, tly, blx, bly, bcx, bcy);
    if (ctx->ps.open)
        ctx->ps.closed = true;
    finish_path(ctx);
}
void vkvg_fill(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    fill_preserve_i(ctx);
    clear_path(ctx);
}
void vkvg_fill_preserve(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    fill_preserve_i(ctx);
}
void vkvg_stroke(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    stroke_preserve_i(ctx);
    clear_path(ctx);
}
void vkvg_stroke_preserve(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    stroke_preserve_i(ctx);
}
/* vkvg_paint, src/vkvg_context.c:990-1003 */
void vkvg_paint(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    finish_path(ctx);
    if (ctx->frame.sub_seg0.size() > ctx->ps.path_sub0) {
        vkvg_fill(ctx);
        return;
    }
    ctx->frame.draws.push_back(make_draw(ctx, GB_DRAW_PAINT));
}
/* vkvg_clear, src/vkvg_context.c:734-753: colour and the whole stencil */
static uint8_t prev_clip_state(VkvgContext ctx) {
    /* _get_previous_clip_state, src/vkvg_context.c:698-702 */
    return ctx->saved.empty() ? (uint8_t)GB_CLIP_CLEAR : ctx->saved.back().clip_state;
}
void vkvg_clear(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    ctx->clip_state = prev_clip_state(ctx) == GB_CLIP_CLEAR ? GB_CLIP_NONE : GB_CLIP_CLEAR;
    ctx->frame.draws.push_back(make_draw(ctx, GB_DRAW_CLEAR));
}

/* ---- clip, save and restore (src/vkvg_context.c:719-795, 950-976, 1251-1512).
   The stencil's bits become the surface's clip planes: the clip bit is the
   inverse of the visibility plane, save bit 2 + p is save plane p, and each
   extra stencil image of vkvg_save is a seven-plane image. */
void vkvg_reset_clip(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    if (ctx->clip_state == GB_CLIP_CLEAR)
        return;
    ctx->clip_state = prev_clip_state(ctx) == GB_CLIP_CLEAR ? GB_CLIP_NONE : GB_CLIP_CLEAR;
    plane_op(ctx, GB_DRAW_CLIP_RESET, 0);
}
void vkvg_clip_preserve(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    if (clip_preserve_i(ctx))
        ctx->clip_state = GB_CLIP_CLIP;
}
void vkvg_clip(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    if (clip_preserve_i(ctx))
        ctx->clip_state = GB_CLIP_CLIP;
    clear_path(ctx);
}
void vkvg_save(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    gb_saved_state sv;
    if (ctx->clip_state == GB_CLIP_CLIP) {
        sv.clip_state = GB_CLIP_SAVED;
        /* a seventh save first copies the whole stencil to a new image */
        if (ctx->sav_bit > 0 && ctx->sav_bit % GB_CLIP_SAVE_PLANES == 0)
            plane_op(ctx, GB_DRAW_CLIP_STORE, ctx->sav_bit / GB_CLIP_SAVE_PLANES - 1u);
        plane_op(ctx, GB_DRAW_CLIP_SAVE, ctx->sav_bit % GB_CLIP_SAVE_PLANES);
        ctx->sav_bit++;
    } else if (ctx->clip_state == GB_CLIP_NONE) {
        sv.clip_state = (uint8_t)(prev_clip_state(ctx) & 0x03u);
    } else {
        sv.clip_state = GB_CLIP_CLEAR;
    }
    sv.line_width  = ctx->line_width;
    sv.miter_limit = ctx->miter_limit;
    sv.dash_offset = ctx->dash_offset;
    sv.dashes      = ctx->dashes;
    sv.opacity     = ctx->opacity;
    sv.line_cap    = ctx->line_cap;
    sv.fill_rule   = ctx->fill_rule;
    sv.op          = ctx->op;
    sv.mat         = ctx->mat;
    sv.mat_inv     = ctx->mat_inv;
    sv.src_x       = ctx->src_x;
    sv.src_y       = ctx->src_y;
    sv.cur_color   = ctx->cur_color;
    sv.pattern     = ctx->pattern;
    if (sv.pattern)
        vkvg_pattern_reference(sv.pattern);
    ctx->saved.push_back(std::move(sv));
}
static void snap_gradient(VkvgContext ctx, VkvgPattern pat);
void        vkvg_restore(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    if (ctx->saved.empty()) {
        ctx->status = VKVG_STATUS_INVALID_RESTORE;
        return;
    }
    gb_saved_state sv = std::move(ctx->saved.back());
    ctx->saved.pop_back();
    if (ctx->clip_state != GB_CLIP_NONE) {
        if (ctx->clip_state == GB_CLIP_CLIP && sv.clip_state == GB_CLIP_CLEAR) {
            plane_op(ctx, GB_DRAW_CLIP_RESET, 0);
        } else {
            /* the clip bit from save bit (curSavBit - 1) % 6 + 2; with no
               save bit in use that expression names the clip bit itself */
            const int j = (int)ctx->sav_bit - 1;
            if (j >= 0)
                plane_op(ctx, GB_DRAW_CLIP_RESTORE, (uint32_t)(j % (int)GB_CLIP_SAVE_PLANES));
        }
    }
    if (sv.clip_state == GB_CLIP_SAVED) {
        ctx->sav_bit--;
        if (ctx->sav_bit > 0 && ctx->sav_bit % GB_CLIP_SAVE_PLANES == 0)
            plane_op(ctx, GB_DRAW_CLIP_LOAD, ctx->sav_bit / GB_CLIP_SAVE_PLANES - 1u);
    }
    ctx->clip_state  = GB_CLIP_NONE;
    ctx->dash_offset = sv.dash_offset;
    ctx->dashes      = sv.dashes;
    ctx->line_width  = sv.line_width;
    ctx->miter_limit = sv.miter_limit;
    ctx->op          = sv.op;
    ctx->line_cap    = sv.line_cap;
    ctx->line_join   = VKVG_LINE_JOIN_MITER; /* the unsaved lineJoint field */
    ctx->fill_rule   = sv.fill_rule;
    ctx->mat         = sv.mat; /* the push constants: matrices, source.xy, opacity */
    ctx->mat_inv     = sv.mat_inv;
    ctx->src_x       = sv.src_x;
    ctx->src_y       = sv.src_y;
    ctx->opacity     = sv.opacity;
    if (sv.pattern) {
        if (sv.pattern != ctx->pattern) {
            /* _update_cur_pattern: the gradient again, with the restored matrix */
            VkvgPattern last = ctx->pattern;
            ctx->pattern     = sv.pattern; /* takes the saved reference */
            ctx->grad_on     = false;
            snap_gradient(ctx, sv.pattern);
            if (last)
                vkvg_pattern_destroy(last);
        } else {
            vkvg_pattern_destroy(sv.pattern);
        }
    } else {
        ctx->cur_color = sv.cur_color;
        set_solid(ctx);
    }
}

/* ---- state (src/vkvg_context.c:1004-1140) */
static uint32_t clamp_byte(float v) {
    if (!(v > 0.0f))
        return 0;
    if (v > 255.0f)
        return 255;
    return (uint32_t)v;
}
/* CreateRgbaf, src/vkvg_context_internal.h:59-62: premultiplied, truncating */
static uint32_t create_rgbaf(float r, float g, float b, float a) {
    return (clamp_byte(a * 255.0f) << 24) | (clamp_byte(b * a * 255.0f) << 16) | (clamp_byte(g * a * 255.0f) << 8) |
           clamp_byte(r * a * 255.0f);
}
/* ================================================================ patterns */
/* src/vkvg_pattern.c, linear gradients */
static void set_solid(VkvgContext ctx) {
    if (ctx->pattern)
        vkvg_pattern_destroy(ctx->pattern);
    ctx->pattern = nullptr;
    ctx->grad_on = false;
}
VkvgPattern vkvg_pattern_create_linear(float x0, float y0, float x1, float y1) {
    _vkvg_pattern_t *p = new (std::nothrow) _vkvg_pattern_t();
    if (!p)
        return (VkvgPattern)&s_no_memory;
    p->status     = VKVG_STATUS_SUCCESS;
    p->refs       = 1;
    p->type       = VKVG_PATTERN_TYPE_LINEAR;
    p->extend     = VKVG_EXTEND_NONE;
    p->filter     = VKVG_FILTER_FAST;
    p->cp[0]      = x0;
    p->cp[1]      = y0;
    p->cp[2]      = x1;
    p->cp[3]      = y1;
    p->count      = 0;
    p->matrix     = VKVG_IDENTITY_MATRIX;
    p->has_matrix = false;
    return p;
}
/* vkvg_pattern_edit_radial, src/vkvg_pattern.c:95-119: radius0 is kept
   below radius1 - 1 and the focus circle is moved inside circle 1 */
vkvg_status_t vkvg_pattern_edit_radial(VkvgPattern pat, float cx0, float cy0, float radius0, float cx1, float cy1,
                                       float radius1) {
    if (vkvg_pattern_status(pat))
        return vkvg_pattern_status(pat);
    if (pat->type != VKVG_PATTERN_TYPE_RADIAL)
        return VKVG_STATUS_PATTERN_TYPE_MISMATCH;
    if (radius0 > radius1 - 1.0f)
        radius0 = radius1 - 1.0f;
    const float ux = cx0 - cx1, uy = cy0 - cy1;
    const float l = sqrtf(ux * ux + uy * uy);
    if (l + radius0 + 1.0f >= radius1) {
        const float vx = ux / l, vy = uy / l, k = radius1 - radius0 - 1.0f;
        cx0 = cx1 + vx * k;
        cy0 = cy1 + vy * k;
    }
    const float cp[8] = {cx0, cy0, radius0, 0.0f, cx1, cy1, radius1, 0.0f};
    memcpy(pat->cp, cp, sizeof(cp));
    return VKVG_STATUS_SUCCESS;
}
VkvgPattern vkvg_pattern_create_radial(float cx0, float cy0, float radius0, float cx1, float cy1, float radius1) {
    _vkvg_pattern_t *p = new (std::nothrow) _vkvg_pattern_t();
    if (!p)
        return (VkvgPattern)&s_no_memory;
    p->status     = VKVG_STATUS_SUCCESS;
    p->refs       = 1;
    p->type       = VKVG_PATTERN_TYPE_RADIAL;
    p->extend     = VKVG_EXTEND_NONE;
    p->filter     = VKVG_FILTER_FAST;
    p->count      = 0;
    p->matrix     = VKVG_IDENTITY_MATRIX;
    p->has_matrix = false;
    vkvg_pattern_edit_radial(p, cx0, cy0, radius0, cx1, cy1, radius1);
    return p;
}
vkvg_status_t vkvg_pattern_status(VkvgPattern pat) { return pat ? pat->status : VKVG_STATUS_NULL_POINTER; }
VkvgPattern   vkvg_pattern_reference(VkvgPattern pat) {
    if (!vkvg_pattern_status(pat))
        pat->refs++;
    return pat;
}
uint32_t vkvg_pattern_get_reference_count(VkvgPattern pat) { return vkvg_pattern_status(pat) ? 0 : pat->refs; }
void     vkvg_pattern_destroy(VkvgPattern pat) {
    if (vkvg_pattern_status(pat))
        return;
    if (--pat->refs > 0)
        return;
    if (pat->surf)
        vkvg_surface_destroy(pat->surf);
    delete pat;
}
/* vkvg_pattern_create_for_surface, src/vkvg_pattern.c:28-48: the pattern
   references the surface */
VkvgPattern vkvg_pattern_create_for_surface(VkvgSurface surf) {
    if (!surf)
        return (VkvgPattern)&s_null_pattern;
    _vkvg_pattern_t *p = new (std::nothrow) _vkvg_pattern_t();
    if (!p)
        return (VkvgPattern)&s_null_pattern;
    p->status     = VKVG_STATUS_SUCCESS;
    p->refs       = 1;
    p->type       = VKVG_PATTERN_TYPE_SURFACE;
    p->extend     = VKVG_EXTEND_NONE;
    p->filter     = VKVG_FILTER_FAST;
    p->count      = 0;
    p->matrix     = VKVG_IDENTITY_MATRIX;
    p->has_matrix = false;
    p->surf       = surf;
    vkvg_surface_reference(surf);
    if (vkvg_surface_status(surf))
        p->status = VKVG_STATUS_INVALID_SURFACE;
    return p;
}
vkvg_status_t vkvg_pattern_edit_linear(VkvgPattern pat, float x0, float y0, float x1, float y1) {
    if (vkvg_pattern_status(pat))
        return vkvg_pattern_status(pat);
    if (pat->type != VKVG_PATTERN_TYPE_LINEAR)
        return VKVG_STATUS_PATTERN_TYPE_MISMATCH;
    pat->cp[0] = x0;
    pat->cp[1] = y0;
    pat->cp[2] = x1;
    pat->cp[3] = y1;
    return VKVG_STATUS_SUCCESS;
}
vkvg_status_t vkvg_pattern_get_linear_points(VkvgPattern pat, float *x0, float *y0, float *x1, float *y1) {
    if (vkvg_pattern_status(pat))
        return vkvg_pattern_status(pat);
    if (pat->type != VKVG_PATTERN_TYPE_LINEAR)
        return VKVG_STATUS_PATTERN_TYPE_MISMATCH;
    if (!x0 || !y0 || !x1 || !y1)
        return VKVG_STATUS_NULL_POINTER;
    *x0 = pat->cp[0];
    *y0 = pat->cp[1];
    *x1 = pat->cp[2];
    *y1 = pat->cp[3];
    return VKVG_STATUS_SUCCESS;
}
/* vkvg_pattern_add_color_stop, src/vkvg_pattern.c:149-168: stops keep their
   premultiplied colour (a*r, a*g, a*b, a) */
vkvg_status_t vkvg_pattern_add_color_stop(VkvgPattern pat, float offset, float r, float g, float b, float a) {
    if (vkvg_pattern_status(pat))
        return vkvg_pattern_status(pat);
    if (pat->type == VKVG_PATTERN_TYPE_SURFACE || pat->type == VKVG_PATTERN_TYPE_SOLID)
        return VKVG_STATUS_PATTERN_TYPE_MISMATCH;
    if (pat->count >= GB_GRAD_STOPS)
        return VKVG_STATUS_INVALID_INDEX;
    float *c            = pat->colors + 4 * pat->count;
    c[0]                = a * r;
    c[1]                = a * g;
    c[2]                = a * b;
    c[3]                = a;
    pat->stops[pat->count++] = offset;
    return VKVG_STATUS_SUCCESS;
}
vkvg_status_t vkvg_pattern_get_color_stop_count(VkvgPattern pat, uint32_t *count) {
    if (vkvg_pattern_status(pat))
        return vkvg_pattern_status(pat);
    if (pat->type == VKVG_PATTERN_TYPE_SURFACE || pat->type == VKVG_PATTERN_TYPE_SOLID)
        return VKVG_STATUS_PATTERN_TYPE_MISMATCH;
    if (!count)
        return VKVG_STATUS_NULL_POINTER;
    *count = pat->count;
    return VKVG_STATUS_SUCCESS;
}
vkvg_status_t vkvg_pattern_get_color_stop_rgba(VkvgPattern pat, uint32_t index, float *offset, float *r, float *g,
                                               float *b, float *a) {
    if (vkvg_pattern_status(pat))
        return vkvg_pattern_status(pat);
    if (pat->type == VKVG_PATTERN_TYPE_SURFACE || pat->type == VKVG_PATTERN_TYPE_SOLID)
        return VKVG_STATUS_PATTERN_TYPE_MISMATCH;
    if (index >= pat->count)
        return VKVG_STATUS_INVALID_INDEX;
    if (!offset || !r || !g || !b || !a)
        return VKVG_STATUS_NULL_POINTER;
    *offset = pat->stops[index];
    *r      = pat->colors[4 * index];
    *g      = pat->colors[4 * index + 1];
    *b      = pat->colors[4 * index + 2];
    *a      = pat->colors[4 * index + 3];
    return VKVG_STATUS_SUCCESS;
}
void vkvg_pattern_set_extend(VkvgPattern pat, vkvg_extend_t extend) {
    if (!vkvg_pattern_status(pat))
        pat->extend = extend;
}
vkvg_extend_t vkvg_pattern_get_extend(VkvgPattern pat) {
    return vkvg_pattern_status(pat) ? (vkvg_extend_t)0 : pat->extend;
}
void vkvg_pattern_set_filter(VkvgPattern pat, vkvg_filter_t filter) {
    if (!vkvg_pattern_status(pat))
        pat->filter = filter;
}
vkvg_filter_t vkvg_pattern_get_filter(VkvgPattern pat) {
    return vkvg_pattern_status(pat) ? (vkvg_filter_t)0 : pat->filter;
}
vkvg_pattern_type_t vkvg_pattern_get_type(VkvgPattern pat) {
    return vkvg_pattern_status(pat) ? (vkvg_pattern_type_t)0 : pat->type;
}
void vkvg_pattern_set_matrix(VkvgPattern pat, const vkvg_matrix_t *matrix) {
    if (vkvg_pattern_status(pat) || !matrix)
        return;
    pat->matrix     = *matrix;
    pat->has_matrix = true;
}
void vkvg_pattern_get_matrix(VkvgPattern pat, vkvg_matrix_t *matrix) {
    if (vkvg_pattern_status(pat) || !matrix)
        return;
    *matrix = pat->has_matrix ? pat->matrix : VKVG_IDENTITY_MATRIX;
}
/* vkvg_set_source + _update_cur_pattern (src/vkvg_context.c:1034-1040,
   src/vkvg_context_internal.c:774-826): the gradient is captured now, its
   control points through the inverse pattern matrix (identity if singular)
   and the current CTM, with the target surface's size */
void vkvg_set_source(VkvgContext ctx, VkvgPattern pat) {
    if (vkvg_status(ctx) || vkvg_pattern_status(pat))
        return;
    vkvg_pattern_reference(pat);
    set_solid(ctx);
    ctx->pattern = pat;
    snap_gradient(ctx, pat);
}
/* vkvg_set_source_surface, src/vkvg_context.c:1025-1033: the offset goes to
   the push constants, the new pattern's only reference to the context */
void vkvg_set_source_surface(VkvgContext ctx, VkvgSurface surf, float x, float y) {
    if (vkvg_status(ctx) || vkvg_surface_status(surf))
        return;
    ctx->src_x      = x;
    ctx->src_y      = y;
    VkvgPattern pat = vkvg_pattern_create_for_surface(surf);
    if (vkvg_pattern_status(pat)) {
        ctx->status = vkvg_pattern_status(pat);
        return;
    }
    set_solid(ctx);
    ctx->pattern = pat;
    snap_gradient(ctx, pat);
}
/* _update_cur_pattern (src/vkvg_context_internal.c:682-831) for a pattern
   source: a surface samples through the push constants of each draw, with
   the pattern matrix multiplied into the inverse matrix now; a gradient is
   captured now and sets source.xy to the surface size */
static void snap_gradient(VkvgContext ctx, VkvgPattern pat) {
    if (pat->type == VKVG_PATTERN_TYPE_SURFACE) {
        VkvgSurface s = pat->surf;
        gb_grad    &g = ctx->grad_snap;
        memset(&g, 0, sizeof(g));
        g.type   = GB_SRC_SURFACE;
        g.w      = (float)ctx->surf->width;
        g.h      = (float)ctx->surf->height;
        g.sw     = s->width;
        g.sh     = s->height;
        g.extend = (uint32_t)pat->extend;
        g.filter = (pat->filter == VKVG_FILTER_BILINEAR || pat->filter == VKVG_FILTER_BEST) ? 1u : 0u;
        g.texels = s->d_rgba;
        if (pat->has_matrix) {
            vkvg_matrix_t r;
            vkvg_matrix_multiply(&r, &ctx->mat_inv, &pat->matrix);
            ctx->mat_inv = r;
        }
        ctx->grad_on = true;
        return;
    }
    if (pat->type != VKVG_PATTERN_TYPE_LINEAR && pat->type != VKVG_PATTERN_TYPE_RADIAL) {
        ctx->status = VKVG_STATUS_PATTERN_TYPE_MISMATCH;
        return;
    }
    ctx->src_x = (float)ctx->surf->width;
    ctx->src_y = (float)ctx->surf->height;
    if (pat->count < 2) {
        ctx->status = VKVG_STATUS_PATTERN_INVALID_GRADIENT;
        return;
    }
    gb_grad &g = ctx->grad_snap;
    memset(&g, 0, sizeof(g));
    float *cp = g.cp; /* vkvg's grad.cp[0] = cp[0..3], grad.cp[1] = cp[4..7] */
    memcpy(cp, pat->cp, sizeof(g.cp));
    vkvg_matrix_t m = VKVG_IDENTITY_MATRIX;
    if (pat->has_matrix) {
        m = pat->matrix;
        if (vkvg_matrix_invert(&m) != VKVG_STATUS_SUCCESS)
            m = VKVG_IDENTITY_MATRIX;
        vkvg_matrix_transform_point(&m, &cp[0], &cp[1]);
    }
    vkvg_matrix_transform_point(&ctx->mat, &cp[0], &cp[1]);
    if (pat->type == VKVG_PATTERN_TYPE_LINEAR) {
        if (pat->has_matrix)
            vkvg_matrix_transform_point(&m, &cp[2], &cp[3]);
        vkvg_matrix_transform_point(&ctx->mat, &cp[2], &cp[3]);
    } else {
        if (pat->has_matrix)
            vkvg_matrix_transform_point(&m, &cp[4], &cp[5]);
        vkvg_matrix_transform_point(&ctx->mat, &cp[4], &cp[5]);
        /* both radii go through transform_distance with cp[0].w as their y
           (src/vkvg_context_internal.c:815-821) */
        if (pat->has_matrix) {
            vkvg_matrix_transform_distance(&m, &cp[2], &cp[3]);
            vkvg_matrix_transform_distance(&m, &cp[6], &cp[3]);
        }
        vkvg_matrix_transform_distance(&ctx->mat, &cp[2], &cp[3]);
        vkvg_matrix_transform_distance(&ctx->mat, &cp[6], &cp[3]);
    }
    g.type  = (uint32_t)pat->type;
    g.w     = (float)ctx->surf->width;
    g.h     = (float)ctx->surf->height;
    g.count = pat->count;
    memcpy(g.stops, pat->stops, sizeof(g.stops));
    memcpy(g.colors, pat->colors, sizeof(g.colors));
    ctx->grad_on = true;
}
/* vkvg_get_source, src/vkvg_context.c:1141-1146: referenced for the caller */
VkvgPattern vkvg_get_source(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return nullptr;
    vkvg_pattern_reference(ctx->pattern);
    return ctx->pattern;
}
void vkvg_set_source_color(VkvgContext ctx, uint32_t c) {
    if (vkvg_status(ctx))
        return;
    set_solid(ctx);
    ctx->cur_color = c;
}
void vkvg_set_source_rgba(VkvgContext ctx, float r, float g, float b, float a) {
    if (vkvg_status(ctx))
        return;
    set_solid(ctx);
    ctx->cur_color = create_rgbaf(r, g, b, a);
}
void vkvg_set_source_rgb(VkvgContext ctx, float r, float g, float b) {
    if (vkvg_status(ctx))
        return;
    set_solid(ctx);
    ctx->cur_color = create_rgbaf(r, g, b, 1);
}
void vkvg_set_opacity(VkvgContext ctx, float opacity) {
    if (vkvg_status(ctx))
        return;
    ctx->opacity = opacity;
}
float vkvg_get_opacity(VkvgContext ctx) { return vkvg_status(ctx) ? 0 : ctx->opacity; }
void  vkvg_set_line_width(VkvgContext ctx, float w) {
    if (!vkvg_status(ctx))
        ctx->line_width = w;
}
void vkvg_set_miter_limit(VkvgContext ctx, float l) {
    if (!vkvg_status(ctx))
        ctx->miter_limit = l;
}
float vkvg_get_miter_limit(VkvgContext ctx) { return vkvg_status(ctx) ? 0 : ctx->miter_limit; }
void  vkvg_set_line_cap(VkvgContext ctx, vkvg_line_cap_t cap) {
    if (!vkvg_status(ctx))
        ctx->line_cap = cap;
}
void vkvg_set_line_join(VkvgContext ctx, vkvg_line_join_t join) {
    if (!vkvg_status(ctx))
        ctx->line_join = join;
}
void vkvg_set_operator(VkvgContext ctx, vkvg_operator_t op) {
    if (!vkvg_status(ctx))
        ctx->op = op;
}
void vkvg_set_fill_rule(VkvgContext ctx, vkvg_fill_rule_t fr) {
    if (!vkvg_status(ctx))
        ctx->fill_rule = fr;
}
void vkvg_set_dash(VkvgContext ctx, const float *dashes, uint32_t num_dashes, float offset) {
    if (vkvg_status(ctx))
        return;
    ctx->dash_offset = offset;
    ctx->dashes.assign(dashes ? dashes : (const float *)nullptr, dashes ? dashes + num_dashes : nullptr);
}
void vkvg_get_dash(VkvgContext ctx, const float *dashes, uint32_t *num_dashes, float *offset) {
    if (vkvg_status(ctx) || !num_dashes || !offset)
        return;
    *num_dashes = (uint32_t)ctx->dashes.size();
    *offset     = ctx->dash_offset;
    if (ctx->dashes.empty() || dashes == NULL)
        return;
    memcpy((float *)dashes, ctx->dashes.data(), sizeof(float) * ctx->dashes.size());
}
float            vkvg_get_line_width(VkvgContext ctx) { return vkvg_status(ctx) ? 0 : ctx->line_width; }
vkvg_line_cap_t  vkvg_get_line_cap(VkvgContext ctx) { return vkvg_status(ctx) ? VKVG_LINE_CAP_BUTT : ctx->line_cap; }
vkvg_line_join_t vkvg_get_line_join(VkvgContext ctx) {
    return vkvg_status(ctx) ? VKVG_LINE_JOIN_MITER : ctx->line_join;
}
vkvg_operator_t  vkvg_get_operator(VkvgContext ctx) { return vkvg_status(ctx) ? VKVG_OPERATOR_OVER : ctx->op; }
vkvg_fill_rule_t vkvg_get_fill_rule(VkvgContext ctx) {
    return vkvg_status(ctx) ? VKVG_FILL_RULE_NON_ZERO : ctx->fill_rule;
}
VkvgSurface vkvg_get_target(VkvgContext ctx) { return vkvg_status(ctx) ? nullptr : ctx->surf; }
/* _set_mat_inv_and_vkCmdPush, src/vkvg_context_internal.c:672-676: every
   matrix change recomputes the pushed inverse (a failed inversion leaves
   vkvg_matrix_invert's partial result) */
static void mat_changed(VkvgContext ctx) {
    ctx->mat_inv = ctx->mat;
    vkvg_matrix_invert(&ctx->mat_inv);
}
void vkvg_translate(VkvgContext ctx, float dx, float dy) {
    if (vkvg_status(ctx))
        return;
    vkvg_matrix_translate(&ctx->mat, dx, dy);
    mat_changed(ctx);
}
void vkvg_scale(VkvgContext ctx, float sx, float sy) {
    if (vkvg_status(ctx))
        return;
    vkvg_matrix_scale(&ctx->mat, sx, sy);
    mat_changed(ctx);
}
void vkvg_rotate(VkvgContext ctx, float radians) {
    if (vkvg_status(ctx))
        return;
    vkvg_matrix_rotate(&ctx->mat, radians);
    mat_changed(ctx);
}
void vkvg_transform(VkvgContext ctx, const vkvg_matrix_t *m) {
    if (vkvg_status(ctx) || !m)
        return;
    vkvg_matrix_t r;
    vkvg_matrix_multiply(&r, &ctx->mat, m);
    ctx->mat = r;
    mat_changed(ctx);
}
void vkvg_set_matrix(VkvgContext ctx, const vkvg_matrix_t *m) {
    if (vkvg_status(ctx) || !m)
        return;
    ctx->mat = *m;
    mat_changed(ctx);
}
void vkvg_get_matrix(VkvgContext ctx, vkvg_matrix_t *const m) {
    if (vkvg_status(ctx) || !m)
        return;
    *m = ctx->mat;
}
void vkvg_identity_matrix(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return;
    vkvg_matrix_init_identity(&ctx->mat);
    mat_changed(ctx);
}
} /* extern "C" */
