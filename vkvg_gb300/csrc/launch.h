/* Kernel launch entry points (defined in the .cu units). */
#ifndef VKVG_GB300_LAUNCH_H
#define VKVG_GB300_LAUNCH_H

#include "gb_types.h"

#include <cuda_runtime.h>
#include <stddef.h>

struct gb_raster_args {
    uint32_t        W, H, S, Wpad, nrows, nbands, ndraws, draw_first;
    uint32_t        init_mode, init_color;
    const gb_draw  *draws;
    const uint32_t *cell_off; /* band-major (band * ndraws + draw) offsets, nbands*ndraws + 1 */
    const uint32_t *apos;     /* per cell: position of its entry in alist (exclusive scan of active cells) */
    const uint32_t *alist;    /* active cells (global cell indices), band-major and in draw order */
    const int2     *dbox;     /* per draw: (min x, -max x) of its edges, 24.8 fixed point */
    uint32_t        cell0;    /* global index of this surface's first cell */
    const int4     *recs;   /* per-cell primitive records: an edge is one 16-byte unit, a triangle two */
    uint32_t        nunits; /* record units in recs */
    uint32_t       *status; /* device status word (GB_ERR_*) */
    uint32_t       *samples; /* [nrows][Wpad] */
    uint32_t       *rgba;    /* [H][W] */
    int32_t        *cov_out; /* debug coverage output [H][W][S] or null */
    uint32_t        cov_draw;
    const uint32_t *gsrc;   /* gradient source images [n][H][W], premultiplied RGBA8 */
    uint32_t        stage_min; /* cells of fewer record units are read from global memory, not staged */
    uint32_t        gc_src;    /* row form, 4x MSAA: source image (index + 1) whose band rows are staged, or 0 */
    uint32_t        wait_limit; /* row form: mbarrier polls before a slot counts as lost */
};
/* the clip planes, a kernel parameter of their own (read by the clipping
   variant only; kept out of gb_raster_args, whose size the register
   allocation of the other variants is sensitive to) */
struct gb_clip_args {
    uint32_t *clip;        /* visibility plane [band rows][clip_wpr] */
    uint32_t *clip_planes; /* save planes, then stencil images, plane_words apart */
    size_t    plane_words;
    uint32_t  clip_wpr;
    uint32_t  clip_load; /* at frame start: 0 all visible, 1 load the plane,
                            2 all visible and save planes zeroed */
};

extern "C" {
/* one gradient source image: out[y * W + x] = premultiplied RGBA8 of g at pixel (x, y) */
cudaError_t gb_launch_gradient_fill(cudaStream_t st, uint32_t W, uint32_t H, const gb_grad *g, uint32_t *out);
/* out[i] = table-unpremultiplied in[i] (RGBA8, alpha in the top byte) */
cudaError_t gb_launch_unpremultiply(cudaStream_t st, const uint32_t *in, size_t n, const uint8_t *table,
                                    uint32_t *out);
size_t      gb_scan_scratch_words(uint32_t n);
cudaError_t gb_exclusive_scan(cudaStream_t st, const uint32_t *in, uint32_t n, uint32_t *out, uint32_t *scratch);

cudaError_t gb_launch_flatten_count(cudaStream_t st, uint32_t nseg, const uint32_t *info, const float4 *a,
                                    const float4 *b, const float4 *c, const uint32_t *n, const uint32_t *aux,
                                    const float *thetas, uint32_t *counts, uint32_t *status);
cudaError_t gb_launch_flatten_emit(cudaStream_t st, uint32_t nseg, const uint32_t *info, const float4 *a,
                                   const float4 *b, const float4 *c, const uint32_t *n, const uint32_t *aux,
                                   const float *thetas, const uint32_t *offsets, float2 *pts, uint8_t *pflag);
cudaError_t gb_launch_subpath_ranges(cudaStream_t st, uint32_t nsub, const uint32_t *sub_seg0,
                                     const uint32_t *sub_nseg, const uint32_t *seg_off, uint32_t *sub_pt0,
                                     uint32_t *sub_npts);

cudaError_t gb_launch_stroke_pair_events(cudaStream_t st, uint32_t npairs, const uint32_t *pair_draw,
                                         const uint32_t *pair_sub, const gb_draw *draws, const uint32_t *sub_pt0,
                                         const uint32_t *sub_npts, const uint32_t *sub_flags, const float2 *pts,
                                         const uint8_t *pflag, const float *dashes, uint32_t *counts,
                                         int walk_dashes);
/* dashed subpaths in parallel: segment lengths + sequential dash state (counts
   of dashed pairs), then the events; see stroke.cu */
cudaError_t gb_launch_dash_count(cudaStream_t st, uint32_t npairs, const uint32_t *pair_draw, const uint32_t *pair_sub,
                                 const gb_draw *draws, const uint32_t *sub_pt0, const uint32_t *sub_npts,
                                 const uint32_t *sub_flags, const float2 *pts, const float *dashes, float *seglen,
                                 uint4 *dseg, uint4 *dfin, uint32_t *counts);
cudaError_t gb_launch_dash_emit(cudaStream_t st, uint32_t npairs, const uint32_t *pair_draw, const uint32_t *pair_sub,
                                const gb_draw *draws, const uint32_t *sub_pt0, const uint32_t *sub_npts,
                                const uint32_t *sub_flags, const float2 *pts, const uint8_t *pflag,
                                const float *dashes, const uint4 *dseg, const uint4 *dfin, const uint32_t *ev_off,
                                gb_event *events);
cudaError_t gb_launch_stroke_dash_events(cudaStream_t st, uint32_t npairs, const uint32_t *pair_draw,
                                         const uint32_t *pair_sub, const gb_draw *draws, const uint32_t *sub_pt0,
                                         const uint32_t *sub_npts, const uint32_t *sub_flags, const float2 *pts,
                                         const uint8_t *pflag, const float *dashes, const uint32_t *ev_off,
                                         gb_event *events);
cudaError_t gb_launch_stroke_event_count(cudaStream_t st, uint32_t nev, uint32_t npairs, const uint32_t *ev_off,
                                         const uint32_t *pair_draw, const uint32_t *pair_sub, const gb_draw *draws,
                                         const uint32_t *sub_pt0, const uint32_t *sub_npts, const uint32_t *sub_flags,
                                         const float2 *pts, const uint8_t *pflag, const gb_event *events,
                                         uint32_t *cnt_v, uint32_t *cnt_i);
cudaError_t gb_launch_stroke_event_emit(cudaStream_t st, uint32_t nev, uint32_t npairs, const uint32_t *ev_off,
                                        const uint32_t *pair_draw, const uint32_t *pair_sub, const gb_draw *draws,
                                        const uint32_t *sub_pt0, const uint32_t *sub_npts, const uint32_t *sub_flags,
                                        const float2 *pts, const uint8_t *pflag, const gb_event *events,
                                        const uint32_t *off_v, const uint32_t *off_i, const uint32_t *pair_dfirst,
                                        float2 *verts, uint32_t *inds, uint8_t *ev_ret);
cudaError_t gb_launch_stroke_close_patch(cudaStream_t st, uint32_t ndraw_s, const uint32_t *draw_pair0,
                                         const uint32_t *pair_sub, const gb_draw *draws, const uint32_t *pair_draw,
                                         const uint32_t *sub_npts, const uint32_t *sub_flags, const uint32_t *ev_off,
                                         const uint32_t *off_v, const uint32_t *off_i, const uint8_t *ev_ret,
                                         uint32_t *inds);
cudaError_t gb_launch_stroke_draw_bases(cudaStream_t st, uint32_t ndraw_s, const uint32_t *draw_pair0,
                                        const uint32_t *ev_off, const uint32_t *off_v, const uint32_t *off_i,
                                        uint32_t *draw_tri0, uint32_t *draw_vbase);

cudaError_t gb_launch_fill_pair_edges(cudaStream_t st, uint32_t npairs, const uint32_t *pair_sub,
                                      const uint32_t *sub_npts, uint32_t *counts);
cudaError_t gb_launch_fill_edges(cudaStream_t st, uint32_t nedges, uint32_t npairs, const uint32_t *e_off,
                                 const uint32_t *pair_draw, const uint32_t *pair_sub, const gb_draw *draws,
                                 const uint32_t *sub_pt0, const uint32_t *sub_npts, const float2 *pts,
                                 const gb_surf *surfs, int4 *edges, uint32_t *edge_draw);
cudaError_t gb_launch_stroke_tris(cudaStream_t st, uint32_t ntris, uint32_t ndraw_s, const uint32_t *draw_tri0,
                                  const uint32_t *sdraw_id, const uint32_t *draw_vbase, const gb_draw *draws,
                                  const float2 *verts, const uint32_t *inds, const gb_surf *surfs, int4 *tri_a,
                                  int4 *tri_b, uint32_t *tri_draw, uint4 *tri_idx, int4 *edges, uint32_t *edge_draw);
/* scatter 0: count each edge into its (band, draw) cells (and, where given,
   fold the draws' x extents into dbox/dcnt, the record total into the 32
   partial sums of total); scatter 1: write the records at the cells'
   advancing offsets */
cudaError_t gb_launch_bin(cudaStream_t st, int scatter, uint32_t nedges, const int4 *edges, const uint32_t *edge_draw,
                          const gb_draw *draws, const gb_surf *surfs, uint32_t samples, uint32_t *cell, int4 *recs,
                          uint32_t nunits, int2 *dbox, uint32_t *dcnt, unsigned long long *total);
/* counts[c] |= GB_CELL_EVERY in every band's cell of the draws that act on
   all bands (kinds after STROKE): with the cells' record counts, the cells
   the raster visits are then the nonzero entries */
cudaError_t gb_launch_cell_flags(cudaStream_t st, uint32_t ndraws, const gb_draw *draws, const gb_surf *surfs,
                                 uint32_t *counts);
/* stats[0] += clipped pixel width x edges of each fill and stroke draw, stats[1] += its edges */
cudaError_t gb_launch_draw_width_stats(cudaStream_t st, uint32_t ndraws, const gb_draw *draws, const int2 *dbox,
                                       const uint32_t *dcnt, uint32_t W, unsigned long long *stats);
/* From the cells' counts (bit 31: GB_CELL_EVERY), in two launchers over the
   same scratch (gb_cells_scratch_words(ncells)): _reduce sums each tile of
   cells (records, active cells) and folds the heaviest cell into *mx where
   given; _lists then writes off[c] = the exclusive sum of the record counts
   before cell c, off[ncells] the total; alist = the active cells (nonzero
   counts) in cell order; apos[c] = the number of active cells before c, at
   every band's first cell of each of the nsurf surfaces and at ncells. */
size_t      gb_cells_scratch_words(uint64_t ncells);
cudaError_t gb_launch_cells_reduce(cudaStream_t st, uint64_t ncells, const uint32_t *counts, uint32_t *scratch,
                                   uint32_t *mx);
cudaError_t gb_launch_cells_lists(cudaStream_t st, uint64_t ncells, const uint32_t *counts, uint32_t *scratch,
                                  uint32_t *off, uint32_t *alist, uint32_t *apos, const gb_surf *surfs, uint32_t nsurf);

/* narrow: 1 the 256-pixel raster form (4 warps, 4 CTAs per SM), 2 the
   128-pixel one (2 warps, 8 CTAs per SM), 5 the 64-pixel one (one warp, 16
   CTAs per SM), 0 the 1024-pixel one (16 warps, one CTA per SM); clipping
   frames run the last */
cudaError_t gb_launch_raster(cudaStream_t st, const gb_raster_args *a, const gb_clip_args *c, int gradients,
                             int clipping, int narrow);
/* pixels per raster tile of a form: 0 wide (1024), 1 narrow (256), 2 middle (512), 3 tiny (128), 4 micro (64) */
uint32_t gb_raster_tile_width(int form);
/* out[i] = src[idx[i]] */
cudaError_t gb_launch_gather_u32(cudaStream_t st, uint32_t n, const uint64_t *idx, const uint32_t *src,
                                 uint32_t *out);
/* the persistent batch raster over a work list of (surface, band, tile, -)
   items (queue: a zeroed counter), nctas SMs' worth of CTAs, tiles of the
   given form (as gb_raster_tile_width) */
cudaError_t gb_launch_raster_batch(cudaStream_t st, const gb_raster_args *a, const gb_surf *surfs, const uint4 *items,
                                   uint32_t nitems, uint32_t *queue, uint32_t nctas, int form, int gradients);
/* the row form of the raster (one warp per sample row, samples in shared
   memory, a producer warp staging each draw's records through a ring of
   slots): one CTA per (1024-pixel tile, band), or with half per (tile, half
   band) with 16-bit counters, three CTAs per SM (every cell under 2^15
   record units); frames without clipping */
cudaError_t gb_launch_raster_rows(cudaStream_t st, const gb_raster_args *a, int gradients, int half);
/* the row form as the persistent batch raster (one CTA per SM, nctas CTAs) */
cudaError_t gb_launch_raster_rows_batch(cudaStream_t st, const gb_raster_args *a, const gb_surf *surfs,
                                        const uint4 *items, uint32_t nitems, uint32_t *queue, uint32_t nctas);
uint32_t    gb_raster_rows_tile_width(void);
/* the flattening kernels' subdivision work cap per cubic, in nodes (0: 2^22) */
cudaError_t gb_set_flatten_node_cap(uint32_t cap);
cudaError_t gb_launch_pmath_eval(cudaStream_t st, int fn, const float *a, const float *b, float *out, uint64_t n);
}

#endif
