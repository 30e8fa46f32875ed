/*
 * Device-side description of an analytic-coverage scene and the launchers of
 * its kernels (analytic_flat.cu: flattening and its adjoint; analytic.cu:
 * coverage, compositing, their adjoints, reductions, Adam).
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define AK_SEG_LINE  1 /* segment kinds = the control points a segment consumes */
#define AK_SEG_CUBIC 3
#define AK_FILL      1u
#define AK_STROKE    2u

#define AK_ERR_POINTS 1u /* flattened points exceeded the point buffer */
#define AK_ERR_WALK   2u /* an edge walk hit its iteration bound */

/* pixel rows per coverage block: 32 where a band of 32 rows fits the blocks'
   shared memory (canvases up to AK_BAND_WIDE_MAX wide), else 16 */
#define AK_BAND_WIDE_MAX 1024
#define AK_CHUNK 16 /* layers per compositing checkpoint */

/* a tile of a tiled scene: its first (tile, layer) pair, the number of its
   layers, and the offset (in elements) of its checkpoints */
struct ak_tile_info {
    uint32_t           first, count;
    unsigned long long ckpt;
};

struct ak_scene {
    uint32_t        W, H, npaths, ncontours, nseg, ncp, nlayers, nbands, band;
    float4          bg;
    /* CW x CH: the canvas.  One window (tiles == 0): the kernels cover the
       canvas, W x H = CW x CH, over its nlayers layers.  Tiled (tiles: the
       tile side): every launch covers all tiles at once; W = H = tiles, nbands
       the bands of a tile, nlayers the number of (tile, layer) pairs (tile
       by tile, each tile's layers in scene order), layer_map[j] the scene
       layer of pair j, pair_tile[j] its tile, pair_box[j] the layer's box
       inside the tile (x0 | y0 << 16, w | h << 16: its area plane covers
       only that box, the layer's area being zero outside it), pair_off[j]
       the plane's first element, tinfo[t] tile t's pairs and checkpoints,
       ntx the tiles across, ntiles the tiles in all */
    uint32_t            CW, CH, tiles, ntx, ntiles;
    const uint32_t     *layer_map;
    const uint32_t     *pair_tile;
    const uint2        *pair_box;
    const uint32_t     *pair_off;
    const ak_tile_info *tinfo;
    const uint8_t  *seg_kind;     /* nseg */
    const uint32_t *seg_cp;       /* nseg: first control point */
    const uint32_t *seg_end;      /* nseg: control point the segment ends at */
    const uint32_t *seg_contour;  /* nseg */
    const uint32_t *cont_s0;      /* ncontours+1: first segment */
    const uint32_t *path_s0;      /* npaths+1: first segment */
    const uint32_t *layer_path;   /* nlayers */
    const uint8_t  *layer_stroke; /* nlayers */
};

/* per-evaluation buffers */
struct ak_bufs {
    const uint32_t *off;     /* nseg+1 point offsets of the segments */
    const float2   *pts;     /* flattened points */
    const uint2    *pt_nb;   /* each point's previous and next point in its contour */
    uint32_t        cap;     /* capacity of pts */
    float          *area;    /* nlayers * W * H: signed areas, then their gradients */
    float4         *ckpt;    /* ceil(nlayers / AK_CHUNK) * W * H: colour under every chunk */
    float4         *canvas;  /* W * H */
    uint32_t       *status;
    uint32_t       *blk_na;  /* tiled scenes: per compositing block, how many layers reach its rows */
    uint32_t       *blist;   /* tiled scenes: those layers (tile-local, in order); block b of tile t
                                from (first pair of t) * blocks per tile + b * (pairs of t) */
};

/* lanes: one lane per segment (scenes of small curves) instead of a warp */
cudaError_t ak_launch_flat_count(cudaStream_t st, const ak_scene &S, const float2 *ctrl, uint32_t *cnt, bool lanes);
cudaError_t ak_launch_flat_emit(cudaStream_t st, const ak_scene &S, const float2 *ctrl, const uint32_t *off,
                                float2 *pts, uint2 *pt_nb, uint32_t cap, uint32_t *status, bool lanes);
cudaError_t ak_launch_flat_bwd(cudaStream_t st, const ak_scene &S, const float2 *ctrl, const uint32_t *off,
                               uint32_t cap, const float2 *gpts, float2 *gctrl, bool lanes);

uint32_t    ak_band_rows(uint32_t W);
size_t      ak_cover_smem(uint32_t W);
cudaError_t ak_launch_cover(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float *widths);
cudaError_t ak_launch_composite(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float4 *colors,
                                const float4 *target, float *loss_part);
cudaError_t ak_launch_composite_bwd(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float4 *colors,
                                    const float4 *target, const float4 *d_canvas, float4 *color_part);
cudaError_t ak_launch_cover_bwd(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float *widths,
                                float2 *gpts, float *gwidth);
cudaError_t ak_launch_reduce(cudaStream_t st, const ak_scene &S, uint32_t nblocks, const float4 *color_part,
                             float4 *d_colors, const float *loss_part, float *loss);
/* tiled scenes: per scene layer its box in pixels (x0, y0, x1, y1
   inclusive, clipped to the canvas; x0 > x1 when empty), from its flattened
   points (strokes widened by half their width plus a pixel, fills by a
   pixel), the boxes' pixel total added to *total */
cudaError_t ak_launch_layer_boxes(cudaStream_t st, const ak_scene &S, const ak_bufs &B, const float *widths, int4 *box,
                                  unsigned long long *total);
/* The (tile, layer) pairs (layer l's box meets tile t), tile by tile in
   layer order, in two sweeps that test the boxes as they go: a run is one
   tile and AK_TP_LAYERS consecutive layers (run r = t * chunks + c,
   chunks = ceil(nlayers / AK_TP_LAYERS)); _count sums every run's pairs
   into bsum[r] and every tile's into tcount[t] (zeroed by the caller);
   after an exclusive scan of bsum into bpos, _lists writes every pair at
   its run's position plus its rank: its layer, its tile, the layer's box
   inside the tile (x0 | y0 << 16, w | h << 16) and its pixel count.  Runs:
   ak_tile_runs(ntiles, nlayers). */
#define AK_TP_LAYERS 8192
uint32_t    ak_tile_runs(uint32_t ntiles, uint32_t nlayers);
cudaError_t ak_launch_tile_count(cudaStream_t st, uint32_t ntiles, uint32_t nlayers, uint32_t ntx, uint32_t tile,
                                 const int4 *box, uint32_t *bsum, uint32_t *tcount);
cudaError_t ak_launch_tile_lists(cudaStream_t st, uint32_t ntiles, uint32_t nlayers, uint32_t ntx, uint32_t tile,
                                 const int4 *box, const uint32_t *bpos, uint32_t *list, uint32_t *ptile, uint2 *pbox,
                                 uint32_t *psize);
cudaError_t ak_launch_adam(cudaStream_t st, float *param, const float *grad, float *m, float *v, uint32_t n, float lr,
                           float beta1, float beta2, float eps, uint32_t step, float lo, float hi);
/* pixel blocks of ak_composite (loss partials) and of ak_composite_bwd per
   window (the canvas, or one tile), and in all */
uint32_t    ak_pixel_blocks(const ak_scene &S);
uint32_t    ak_composite_bwd_blocks(const ak_scene &S);
uint32_t    ak_pixel_blocks_all(const ak_scene &S);
size_t      ak_color_partials(const ak_scene &S); /* float4 colour partials of ak_composite_bwd */
