/*
 * Entry points of vkvg_gb300.h: parity hooks over a context's last flush,
 * captured frames (device-resident command buffers executed on demand) and
 * portable-math evaluation.
 */
#include "host.h"
#include "launch.h"
#include "pmath.h"

#include <float.h>
#include <new>

extern "C" {

void vkvg_gb300_debug_capture(VkvgContext ctx, int enable) {
    if (!vkvg_status(ctx))
        ctx->debug = enable != 0;
}

vkvg_status_t vkvg_gb300_debug_counts(VkvgContext ctx, uint32_t out[8]) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    if (!out)
        return VKVG_STATUS_NULL_POINTER;
    const Pipeline &p = ctx->pl;
    out[0]            = p.nsub;
    out[1]            = p.npts;
    out[2]            = p.ndraw;
    out[3]            = p.nverts;
    out[4]            = p.ninds;
    out[5]            = p.dev_status;
    out[6]            = p.nedges;
    out[7]            = p.nunits;
    return VKVG_STATUS_SUCCESS;
}

static vkvg_status_t d2h(void *dst, const void *src, size_t bytes) {
    if (!bytes)
        return VKVG_STATUS_SUCCESS;
    return cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost) == cudaSuccess ? VKVG_STATUS_SUCCESS
                                                                             : VKVG_STATUS_DEVICE_ERROR;
}

vkvg_status_t vkvg_gb300_debug_points(VkvgContext ctx, float *xy, uint8_t *flags) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    const Pipeline &p = ctx->pl;
    vkvg_status_t   r = VKVG_STATUS_SUCCESS;
    if (xy)
        r = d2h(xy, p.pts.p, (size_t)p.npts * 8);
    if (!r && flags)
        r = d2h(flags, p.pflag.p, p.npts);
    return r;
}

vkvg_status_t vkvg_gb300_debug_subpaths(VkvgContext ctx, uint32_t *first, uint32_t *count, uint32_t *flags) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    const Pipeline &p = ctx->pl;
    vkvg_status_t   r = VKVG_STATUS_SUCCESS;
    if (first)
        r = d2h(first, p.sub_pt0.p, (size_t)p.nsub * 4);
    if (!r && count)
        r = d2h(count, p.sub_npts.p, (size_t)p.nsub * 4);
    if (!r && flags)
        r = d2h(flags, (const uint8_t *)p.in.p + p.o_sub_flags, (size_t)p.nsub * 4);
    return r;
}

static vkvg_status_t stroke_range(const Pipeline &p, uint32_t i, uint32_t *k_out, uint32_t *v0, uint32_t *nv,
                                  uint32_t *i0, uint32_t *ni) {
    /* find the stroke-draw ordinal of draw i */
    std::vector<uint32_t> sid(p.nsdraw);
    if (d2h(sid.data(), (const uint8_t *)p.in.p + p.o_sdid, (size_t)p.nsdraw * 4))
        return VKVG_STATUS_DEVICE_ERROR;
    uint32_t k = UINT32_MAX;
    for (uint32_t j = 0; j < p.nsdraw; j++)
        if (sid[j] == i)
            k = j;
    if (k == UINT32_MAX)
        return VKVG_STATUS_INVALID_INDEX;
    uint32_t tri[2], vb[2];
    if (d2h(tri, p.sdraw_tri0.as<uint32_t>() + k, 8) || d2h(vb, p.sdraw_vbase.as<uint32_t>() + k, 8))
        return VKVG_STATUS_DEVICE_ERROR;
    *k_out = k;
    *v0    = vb[0];
    *nv    = vb[1] - vb[0];
    *i0    = tri[0] * 3;
    *ni    = (tri[1] - tri[0]) * 3;
    return VKVG_STATUS_SUCCESS;
}

vkvg_status_t vkvg_gb300_debug_draw(VkvgContext ctx, uint32_t i, uint32_t info[8]) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    const Pipeline &p = ctx->pl;
    if (i >= p.ndraw || !info)
        return VKVG_STATUS_INVALID_INDEX;
    gb_draw d;
    if (d2h(&d, (const uint8_t *)p.in.p + p.o_draws + (size_t)i * sizeof(gb_draw), sizeof(gb_draw)))
        return VKVG_STATUS_DEVICE_ERROR;
    memset(info, 0, 8 * sizeof(uint32_t));
    info[0] = d.kind;
    info[1] = d.sub_first;
    info[2] = d.sub_count;
    info[5] = d.src;
    if (d.kind == GB_DRAW_STROKE) {
        uint32_t k, v0, nv, i0, ni;
        if (!stroke_range(p, i, &k, &v0, &nv, &i0, &ni)) {
            info[3] = nv;
            info[4] = ni;
        }
    }
    return VKVG_STATUS_SUCCESS;
}

vkvg_status_t vkvg_gb300_debug_stroke(VkvgContext ctx, uint32_t i, float *xy, uint32_t *inds) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    uint32_t      k, v0, nv, i0, ni;
    vkvg_status_t r = stroke_range(ctx->pl, i, &k, &v0, &nv, &i0, &ni);
    if (r)
        return r;
    if (xy)
        r = d2h(xy, ctx->pl.verts.as<float2>() + v0, (size_t)nv * 8);
    if (!r && inds)
        r = d2h(inds, ctx->pl.inds.as<uint32_t>() + i0, (size_t)ni * 4);
    return r;
}

void vkvg_gb300_debug_set_raster_form(int form) { gb_form_override.store(form >= 0 && form <= 5 ? form : -1); }
int  vkvg_gb300_debug_raster_form(VkvgContext ctx) { return vkvg_status(ctx) ? -1 : ctx->pl.form_run; }
void vkvg_gb300_debug_inject(int what, uint32_t value) {
    if (what == 0)
        gb_fail_alloc.store(value);
    else if (what == 1)
        gb_wait_limit.store(value);
    else if (what == 2)
        gb_set_flatten_node_cap(value);
}

vkvg_status_t vkvg_gb300_debug_coverage(VkvgContext ctx, uint32_t i, int32_t *out) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    Pipeline   &p = ctx->pl;
    VkvgSurface s = ctx->surf;
    if (i >= p.ndraw || !out)
        return VKVG_STATUS_INVALID_INDEX;
    size_t n = (size_t)s->width * s->height * s->samples;
    if (!p.dbg.grow(n * 4))
        return VKVG_STATUS_NO_MEMORY;
    cudaMemsetAsync(p.dbg.p, 0, n * 4, p.st);
    gb_raster_args A;
    memset(&A, 0, sizeof(A));
    A.W        = s->width;
    A.H        = s->height;
    A.S        = s->samples;
    A.Wpad     = s->wpad;
    A.nrows    = s->nrows;
    A.nbands   = s->nbands;
    A.ndraws   = p.ndraw;
    A.draws    = (const gb_draw *)((const uint8_t *)p.in.p + p.o_draws);
    A.cell_off = p.cells.as<uint32_t>();
    A.apos     = p.apos.as<uint32_t>();
    A.alist    = p.alist.as<uint32_t>();
    A.dbox     = p.dbox.as<int2>();
    A.cell0    = 0;
    A.recs     = p.recs.as<int4>();
    A.nunits   = p.nunits;
    A.status   = p.status.as<uint32_t>();
    A.samples  = s->d_samples;
    A.rgba     = s->d_rgba;
    A.cov_out  = p.dbg.as<int32_t>();
    A.cov_draw = i;
    A.wait_limit = WAIT_LIMIT_POLLS;
    gb_clip_args CA;
    memset(&CA, 0, sizeof(CA));
    /* the form the frame itself ran (the register tile after a clipping frame) */
    const cudaError_t e =
        p.form_run == 3 || p.form_run == 4 ? gb_launch_raster_rows(p.st, &A, 0, p.form_half)
                                           : gb_launch_raster(p.st, &A, &CA, 0, 0, 0);
    if (e != cudaSuccess)
        return VKVG_STATUS_DEVICE_ERROR;
    gb_count_launch(1);
    if (cudaStreamSynchronize(p.st) != cudaSuccess)
        return VKVG_STATUS_DEVICE_ERROR;
    return d2h(out, p.dbg.p, n * 4);
}

/* vkvg_path_extents, src/vkvg_context.c:688-699 with _vkvg_path_extents
   (src/vkvg_context_internal.c:1878-1917): bounds of the flattened points of
   the current path, untransformed (vkvg starts the maxima at FLT_MIN).  The
   points come from the flatten kernels. */
void vkvg_path_extents(VkvgContext ctx, float *const x1, float *const y1, float *const x2, float *const y2) {
    if (vkvg_status(ctx))
        return;
    vkvg_new_sub_path(ctx); /* _finish_path */
    FrameHost     &f  = ctx->frame;
    const uint32_t s0 = ctx->ps.path_sub0, s1 = (uint32_t)f.sub_seg0.size();
    if (s0 == s1) {
        if (x1 && y1 && x2 && y2)
            *x1 = *x2 = *y1 = *y2 = 0;
        return;
    }
    Pipeline tmp;
    if (!tmp.init() || tmp.upload(f) != cudaSuccess || tmp.flatten_only() != cudaSuccess) {
        tmp.destroy();
        ctx->status = VKVG_STATUS_DEVICE_ERROR;
        return;
    }
    std::vector<uint32_t> first(s1), count(s1);
    std::vector<float>    xy((size_t)tmp.npts * 2 + 2);
    d2h(first.data(), tmp.sub_pt0.p, (size_t)s1 * 4);
    d2h(count.data(), tmp.sub_npts.p, (size_t)s1 * 4);
    d2h(xy.data(), tmp.pts.p, (size_t)tmp.npts * 8);
    tmp.destroy();
    float xMin = FLT_MAX, yMin = FLT_MAX, xMax = FLT_MIN, yMax = FLT_MIN;
    for (uint32_t s = s0; s < s1; s++)
        for (uint32_t i = first[s]; i < first[s] + count[s]; i++) {
            float x = xy[2 * i], y = xy[2 * i + 1];
            if (x < xMin)
                xMin = x;
            if (x > xMax)
                xMax = x;
            if (y < yMin)
                yMin = y;
            if (y > yMax)
                yMax = y;
        }
    if (x1 && y1 && x2 && y2) {
        *x1 = xMin;
        *x2 = xMax;
        *y1 = yMin;
        *y2 = yMax;
    }
}

/* ------------------------------------------------------------- frames */

VkvgFrame vkvg_gb300_frame_capture(VkvgContext ctx) {
    if (vkvg_status(ctx))
        return nullptr;
    _vkvg_gb300_frame_t *fr = new (std::nothrow) _vkvg_gb300_frame_t();
    if (!fr)
        return nullptr;
    if (!fr->pl.init()) {
        delete fr;
        return nullptr;
    }
    fr->frame = ctx->frame;
    fr->width   = ctx->surf->width;
    fr->height  = ctx->surf->height;
    fr->samples = ctx->surf->samples;
    /* the context keeps its current path, as after a flush */
    ctx->frame.draws.clear();
    ctx->frame.spair_draw.clear();
    ctx->frame.spair_sub.clear();
    ctx->frame.spair_dfirst.clear();
    ctx->frame.sdraw_id.clear();
    ctx->frame.sdraw_pair0.clear();
    ctx->frame.fpair_draw.clear();
    ctx->frame.fpair_sub.clear();
    ctx->frame.dashes.clear();
    ctx->frame.paths    = 0;
    ctx->frame.any_dash = false;
    if (fr->pl.upload(fr->frame) != cudaSuccess || cudaStreamSynchronize(fr->pl.st) != cudaSuccess) {
        fr->pl.destroy();
        delete fr;
        return nullptr;
    }
    return fr;
}

vkvg_status_t vkvg_gb300_frame_execute(VkvgFrame fr, VkvgSurface surf) {
    if (!fr)
        return VKVG_STATUS_NULL_POINTER;
    if (vkvg_surface_status(surf))
        return VKVG_STATUS_INVALID_SURFACE;
    if (surf->width != fr->width || surf->height != fr->height || surf->samples != fr->samples)
        return VKVG_STATUS_INVALID_SURFACE;
    uint64_t      l0 = vkvg_gb300_kernel_launches();
    vkvg_status_t r  = gb_run_frame(fr->pl, fr->frame, surf, false, true);
    fr->pl.launches  = vkvg_gb300_kernel_launches() - l0;
    return r;
}

vkvg_status_t vkvg_gb300_frame_stats(VkvgFrame fr, uint64_t out[16]) {
    if (!fr || !out)
        return VKVG_STATUS_NULL_POINTER;
    memset(out, 0, 16 * sizeof(uint64_t));
    const Pipeline &p = fr->pl;
    out[0]            = fr->frame.paths;
    out[1]            = p.npts;
    out[2]            = p.nverts;
    out[3]            = p.ninds;
    out[4]            = p.nedges;
    out[5]            = p.nunits;
    out[6]            = p.nseg;
    out[7]            = p.ndraw;
    out[8]            = p.launches;
    out[9]            = p.nsub;
    out[10]           = p.ntris;
    out[11]           = p.dev_status;
    out[12]           = p.upload_bytes;
    return VKVG_STATUS_SUCCESS;
}

vkvg_status_t vkvg_gb300_frame_timing(VkvgFrame fr, float out[8]) {
    if (!fr || !out)
        return VKVG_STATUS_NULL_POINTER;
    for (int i = 0; i < 8; i++)
        out[i] = i < 5 ? fr->pl.ms[i] : 0.f;
    return VKVG_STATUS_SUCCESS;
}

void vkvg_gb300_frame_destroy(VkvgFrame fr) {
    if (!fr)
        return;
    fr->pl.destroy();
    delete fr;
}

/* ------------------------------------------------------- command replay */

vkvg_status_t vkvg_gb300_replay_stream(VkvgContext ctx, const uint32_t *cmds, uint32_t ncmds, const float *args,
                                       uint64_t nargs) {
    if (vkvg_status(ctx))
        return vkvg_status(ctx);
    if ((!cmds && ncmds) || (!args && nargs))
        return VKVG_STATUS_NULL_POINTER;
    uint64_t a = 0;
#define NEED(k)                                                                                                            do {                                                                                                                       if (a + (k) > nargs)                                                                                                       return VKVG_STATUS_INVALID_INDEX;                                                                              } while (0)
    const float *A = args;
    for (uint32_t i = 0; i < ncmds; i++) {
        switch (cmds[i]) {
        case VKVG_CMD_NEW_PATH: vkvg_new_path(ctx); break;
        case VKVG_CMD_NEW_SUB_PATH: vkvg_new_sub_path(ctx); break;
        case VKVG_CMD_CLOSE_PATH: vkvg_close_path(ctx); break;
        case VKVG_CMD_MOVE_TO: NEED(2); vkvg_move_to(ctx, A[a], A[a + 1]); a += 2; break;
        case VKVG_CMD_LINE_TO: NEED(2); vkvg_line_to(ctx, A[a], A[a + 1]); a += 2; break;
        case VKVG_CMD_REL_MOVE_TO: NEED(2); vkvg_rel_move_to(ctx, A[a], A[a + 1]); a += 2; break;
        case VKVG_CMD_REL_LINE_TO: NEED(2); vkvg_rel_line_to(ctx, A[a], A[a + 1]); a += 2; break;
        case VKVG_CMD_RECTANGLE: NEED(4); vkvg_rectangle(ctx, A[a], A[a + 1], A[a + 2], A[a + 3]); a += 4; break;
        case VKVG_CMD_ARC: NEED(5); vkvg_arc(ctx, A[a], A[a + 1], A[a + 2], A[a + 3], A[a + 4]); a += 5; break;
        case VKVG_CMD_ARC_NEG:
            NEED(5);
            vkvg_arc_negative(ctx, A[a], A[a + 1], A[a + 2], A[a + 3], A[a + 4]);
            a += 5;
            break;
        case VKVG_CMD_CURVE_TO:
            NEED(6);
            vkvg_curve_to(ctx, A[a], A[a + 1], A[a + 2], A[a + 3], A[a + 4], A[a + 5]);
            a += 6;
            break;
        case VKVG_CMD_REL_CURVE_TO:
            NEED(6);
            vkvg_rel_curve_to(ctx, A[a], A[a + 1], A[a + 2], A[a + 3], A[a + 4], A[a + 5]);
            a += 6;
            break;
        case VKVG_CMD_QUADRATIC_TO:
            NEED(4);
            vkvg_quadratic_to(ctx, A[a], A[a + 1], A[a + 2], A[a + 3]);
            a += 4;
            break;
        case VKVG_CMD_REL_QUADRATIC_TO:
            NEED(4);
            vkvg_rel_quadratic_to(ctx, A[a], A[a + 1], A[a + 2], A[a + 3]);
            a += 4;
            break;
        case VKVG_CMD_ELLIPTICAL_ARC_TO: /* x, y, large, sweep, rx, ry, phi */
            NEED(7);
            vkvg_elliptic_arc_to(ctx, A[a], A[a + 1], A[a + 2] != 0, A[a + 3] != 0, A[a + 4], A[a + 5], A[a + 6]);
            a += 7;
            break;
        case VKVG_CMD_SET_LINE_WIDTH: NEED(1); vkvg_set_line_width(ctx, A[a++]); break;
        case VKVG_CMD_SET_MITER_LIMIT: NEED(1); vkvg_set_miter_limit(ctx, A[a++]); break;
        case VKVG_CMD_SET_LINE_JOIN: NEED(1); vkvg_set_line_join(ctx, (vkvg_line_join_t)(int)A[a++]); break;
        case VKVG_CMD_SET_LINE_CAP: NEED(1); vkvg_set_line_cap(ctx, (vkvg_line_cap_t)(int)A[a++]); break;
        case VKVG_CMD_SET_OPERATOR: NEED(1); vkvg_set_operator(ctx, (vkvg_operator_t)(int)A[a++]); break;
        case VKVG_CMD_SET_FILL_RULE: NEED(1); vkvg_set_fill_rule(ctx, (vkvg_fill_rule_t)(int)A[a++]); break;
        case VKVG_CMD_SET_DASH: {
            NEED(2);
            uint32_t n   = (uint32_t)A[a];
            float    off = A[a + 1];
            a += 2;
            NEED(n);
            vkvg_set_dash(ctx, n ? A + a : nullptr, n, off);
            a += n;
            break;
        }
        case VKVG_CMD_TRANSLATE: NEED(2); vkvg_translate(ctx, A[a], A[a + 1]); a += 2; break;
        case VKVG_CMD_SCALE: NEED(2); vkvg_scale(ctx, A[a], A[a + 1]); a += 2; break;
        case VKVG_CMD_ROTATE: NEED(1); vkvg_rotate(ctx, A[a++]); break;
        case VKVG_CMD_IDENTITY_MATRIX: vkvg_identity_matrix(ctx); break;
        case VKVG_CMD_SET_MATRIX: {
            NEED(6);
            vkvg_matrix_t m = {A[a], A[a + 1], A[a + 2], A[a + 3], A[a + 4], A[a + 5]};
            vkvg_set_matrix(ctx, &m);
            a += 6;
            break;
        }
        case VKVG_CMD_PAINT: vkvg_paint(ctx); break;
        case VKVG_CMD_FILL: vkvg_fill(ctx); break;
        case VKVG_CMD_STROKE: vkvg_stroke(ctx); break;
        case VKVG_CMD_CLEAR: vkvg_clear(ctx); break;
        case VKVG_CMD_CLIP: vkvg_clip(ctx); break;
        case VKVG_CMD_CLIP_PRESERVE: vkvg_clip_preserve(ctx); break;
        case VKVG_CMD_RESET_CLIP: vkvg_reset_clip(ctx); break;
        case VKVG_CMD_SAVE: vkvg_save(ctx); break;
        case VKVG_CMD_RESTORE: vkvg_restore(ctx); break;
        case VKVG_CMD_FILL_PRESERVE: vkvg_fill_preserve(ctx); break;
        case VKVG_CMD_STROKE_PRESERVE: vkvg_stroke_preserve(ctx); break;
        case VKVG_CMD_SET_SOURCE_RGB: NEED(3); vkvg_set_source_rgb(ctx, A[a], A[a + 1], A[a + 2]); a += 3; break;
        case VKVG_CMD_SET_SOURCE_RGBA:
            NEED(4);
            vkvg_set_source_rgba(ctx, A[a], A[a + 1], A[a + 2], A[a + 3]);
            a += 4;
            break;
        case VKVG_CMD_SET_SOURCE_COLOR: {
            NEED(1);
            uint32_t c;
            memcpy(&c, &A[a++], 4);
            vkvg_set_source_color(ctx, c);
            break;
        }
        default: return VKVG_STATUS_INVALID_INDEX;
        }
        if (vkvg_status(ctx))
            return vkvg_status(ctx);
    }
#undef NEED
    return VKVG_STATUS_SUCCESS;
}

/* ------------------------------------------------------- portable math */

vkvg_status_t vkvg_gb300_pmath_eval(int fn, const float *a, const float *b, float *out, uint64_t n, int device) {
    if (!a || !b || !out)
        return VKVG_STATUS_NULL_POINTER;
    if (!device) {
        for (uint64_t i = 0; i < n; i++) {
            switch (fn) {
            case 0: out[i] = pm_atan2f(a[i], b[i]); break;
            case 1: out[i] = pm_acosf(a[i]); break;
            case 2: out[i] = pm_cosf(a[i]); break;
            case 3: out[i] = pm_sinf(a[i]); break;
            case 4: out[i] = pm_asinf(a[i]); break;
            default: out[i] = pm_atanf(a[i]); break;
            }
        }
        return VKVG_STATUS_SUCCESS;
    }
    float *d = nullptr;
    if (cudaMalloc(&d, n * 12 + 16) != cudaSuccess)
        return VKVG_STATUS_NO_MEMORY;
    vkvg_status_t r = VKVG_STATUS_SUCCESS;
    if (cudaMemcpy(d, a, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(d + n, b, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        gb_launch_pmath_eval(0, fn, d, d + n, d + 2 * n, n) != cudaSuccess ||
        cudaMemcpy(out, d + 2 * n, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        r = VKVG_STATUS_DEVICE_ERROR;
    gb_count_launch(1);
    cudaFree(d);
    return r;
}

} /* extern "C" */
