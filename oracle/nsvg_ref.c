/*
 * nsvg_ref.c - TEST INFRASTRUCTURE ONLY.  A dump interface over vkvg's own
 * vendored SVG parser (nanoSVG, src/nsvg/nanosvg.h of vkvg, included from the
 * reference tree by oracle/build_ref.py, with the configuration vkvg builds it
 * in: NANOSVG_IMPLEMENTATION, no NANOSVG_ALL_COLOR_KEYWORDS).  The parity
 * tests read what vkvg's SVG walk (src/nsvg/vkvg_nsvg.c:82-136) reads from
 * nanoSVG's image through these functions.  Only this driver is written here;
 * the parser is the reference's.
 */
#include <stdint.h>
#include <stdio.h> /* nanosvg.h expects its includer to provide it (vkvg's headers do) */
#include <stdlib.h>
#include <string.h>

#define NANOSVG_IMPLEMENTATION
#include "nanosvg.h"

#if defined(__GNUC__)
#define NREF_API __attribute__((visibility("default")))
#else
#define NREF_API
#endif

/* nsvgParse(copy of text, units, dpi) */
NREF_API void *nref_parse(const char *text, const char *units, float dpi) {
    size_t n   = strlen(text);
    char  *buf = (char *)malloc(n + 1);
    if (!buf)
        return NULL;
    memcpy(buf, text, n + 1);
    NSVGimage *img = nsvgParse(buf, units, dpi);
    free(buf);
    return img;
}
NREF_API void nref_free(void *img) { nsvgDelete((NSVGimage *)img); }
NREF_API void nref_dims(void *img, float *w, float *h) {
    *w = ((NSVGimage *)img)->width;
    *h = ((NSVGimage *)img)->height;
}
static NSVGshape *shape_at(void *img, uint32_t i) {
    NSVGshape *s = ((NSVGimage *)img)->shapes;
    while (s && i--)
        s = s->next;
    return s;
}
NREF_API uint32_t nref_shape_count(void *img) {
    uint32_t n = 0;
    for (NSVGshape *s = ((NSVGimage *)img)->shapes; s; s = s->next)
        n++;
    return n;
}
/* the paint as vkvg's walk sees it: type, and the colour (a gradient's first stop) */
static void paint(const NSVGpaint *p, uint32_t *type, uint32_t *color) {
    *type  = (uint32_t)p->type;
    *color = 0;
    if (p->type == NSVG_PAINT_COLOR)
        *color = p->color;
    else if (p->type == NSVG_PAINT_LINEAR_GRADIENT || p->type == NSVG_PAINT_RADIAL_GRADIENT)
        *color = p->gradient->stops[0].color;
}
/* u: fill type, fill colour, stroke type, stroke colour, visible, paths;
   f: opacity, stroke width, bounds[4] */
NREF_API int nref_shape(void *img, uint32_t i, char id[64], uint32_t u[6], float f[6]) {
    NSVGshape *s = shape_at(img, i);
    if (!s)
        return -1;
    memcpy(id, s->id, 64);
    paint(&s->fill, &u[0], &u[1]);
    paint(&s->stroke, &u[2], &u[3]);
    u[4] = (s->flags & NSVG_FLAGS_VISIBLE) ? 1u : 0u;
    u[5] = 0;
    for (NSVGpath *p = s->paths; p; p = p->next)
        u[5]++;
    f[0] = s->opacity;
    f[1] = s->strokeWidth;
    memcpy(f + 2, s->bounds, 4 * sizeof(float));
    return 0;
}
NREF_API int nref_path(void *img, uint32_t shape, uint32_t path, float *pts, uint32_t cap, uint32_t *npts,
                       uint32_t *closed) {
    NSVGshape *s = shape_at(img, shape);
    if (!s)
        return -1;
    NSVGpath *p = s->paths;
    while (p && path--)
        p = p->next;
    if (!p)
        return -1;
    *npts   = (uint32_t)p->npts;
    *closed = (uint32_t)p->closed;
    if (pts && cap)
        memcpy(pts, p->pts, (size_t)((uint32_t)p->npts < cap ? (uint32_t)p->npts : cap) * 2 * sizeof(float));
    return 0;
}
