/* vkvg_gb300: vkvg's SVG entry points, with the names, signatures and
 * behaviour of vkvg's include/vkvg-svg.h:22-108 (implemented by its nanoSVG
 * adapter, src/nsvg/vkvg_nsvg.c:28-136).  The parser is this library's own
 * (vkvg_gb300/csrc/svg.cpp); documents load in px at 96 dpi, surfaces from
 * SVG at the device's horizontal dpi (vkvg_device_set_dpy). */
#ifndef VKVG_SVG_H
#define VKVG_SVG_H

#include "vkvg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct _vkvg_svg_t *VkvgSvg;

/* a new surface of the document's size with the document drawn on it; the
   width and height arguments are accepted and not used, as in vkvg; null if
   the file cannot be read */
vkvg_public VkvgSurface vkvg_surface_create_from_svg(VkvgDevice dev, uint32_t width, uint32_t height,
                                                     const char *svgFilePath);
vkvg_public VkvgSurface vkvg_surface_create_from_svg_fragment(VkvgDevice dev, uint32_t width, uint32_t height,
                                                              char *svgFragment);
vkvg_public void        vkvg_svg_get_dimensions(VkvgSvg svg, uint32_t *width, uint32_t *height);
/* parse a file / a string (the string is not modified); null if the file
   cannot be read */
vkvg_public VkvgSvg vkvg_svg_load(const char *svgFilePath);
vkvg_public VkvgSvg vkvg_svg_load_fragment(char *svgFragment);
/* draw the document (or the shapes whose id, or whose group's id, is id) on
   the context, inside a save / restore */
vkvg_public void vkvg_svg_render(VkvgSvg svg, VkvgContext ctx, const char *id);
vkvg_public void vkvg_svg_destroy(VkvgSvg svg);

#ifdef __cplusplus
}
#endif
#endif
