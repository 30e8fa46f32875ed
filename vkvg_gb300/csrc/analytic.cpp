/* Differentiable analytic coverage: the scene object and its C ABI
 * (include/vkvg_gb300.h).  No vkvg counterpart.
 *
 * create() uploads the scene's topology once.  forward() queues: per-segment
 * point counts of the flattening, their exclusive scan, the points, the
 * per-(band, layer) signed areas, the compositing (canvas, chunk checkpoints,
 * loss).  backward() queues the compositing adjoint (dL/dA in place of A,
 * colour partials), the colour reduction, the coverage adjoint (dL/dpoint,
 * dL/dwidth) and the flattening adjoint, which walks the subdivision again
 * (dL/dcontrol).  Nothing is read back in steady state: the point total is
 * copied to pinned memory after each forward and checked when it has landed;
 * only the first forward waits for it, to size the point buffer.
 *
 * A tiled scene (create_tiled) keeps the same kernels and runs each of them
 * once over every square tile of the canvas.  After the flattening, every
 * layer's box in pixels (from its points, strokes widened by half their
 * width; a layer's area is exactly zero outside it), two sweeps over every
 * (tile, layer) entry, testing the boxes as they go (counts per run of
 * entries and per tile, then a scan of the runs and the compaction), give
 * the (tile, layer) pairs, tile by tile in scene order, each with the
 * layer's box inside the tile; a pair's area plane covers only that box
 * (planes placed by a scan of their sizes).  The per-tile counts and the box total are read back
 * (the one synchronisation of a tiled forward) to size the planes and every
 * tile's checkpoints, all kept resident for the backward.  A coverage block
 * covers its pair's box; a compositing thread one pixel of a tile, reading a
 * layer's plane where the pixel lies in its box and zero elsewhere.
 */
#include "analytic.h"
#include "host.h"
#include "launch.h"

#include <algorithm>
#include <new>
#include <string.h>

struct _vkvg_gb300_analytic_t {
    vkvg_status_t status = VKVG_STATUS_SUCCESS;
    uint32_t      W = 0, H = 0, npaths = 0, ncontours = 0, nseg = 0, ncp = 0, nlayers = 0;
    float         bg[4]  = {1, 1, 1, 1};
    cudaStream_t  stream = nullptr;
    bool          own_stream = false;
    /* topology */
    DevBuf d_seg_kind, d_seg_cp, d_seg_end, d_seg_contour, d_cont_s0, d_path_s0, d_layer_path, d_layer_stroke;
    ak_scene S{};
    /* per evaluation */
    DevBuf    d_cnt, d_off, d_scan, d_pts, d_pt_nb, d_area, d_ckpt, d_canvas, d_loss_part, d_loss, d_color_part,
              d_gpts, d_status;
    PinnedBuf h_mon; /* [0] status word, [1] point total of the last forward */
    cudaEvent_t ev_mon = nullptr;
    bool        mon_pending = false;
    uint32_t    cap = 0;
    vkvg_status_t pending = VKVG_STATUS_SUCCESS; /* first error since the last sync */
    /* phase timing (set_timing): events around flatten, cover, composite of
       the forward and composite, cover, flatten adjoints of the backward */
    bool        timing = false;
    cudaEvent_t ev[8]  = {};
    /* tiled scenes: tile side (0: one window, the whole canvas), tiles
       across and down, per-layer boxes, per run of (tile, layer) entries
       its pair count (d_flags) and their scan (d_fpos), per tile its pair
       count, the pairs' scene layers and tiles, per tile its pairs and
       plane offsets (pinned, then on the device), and the scene the tiled
       launches take (TS: every tile at once) */
    uint32_t  tile = 0, ntx = 1, nty = 1;
    DevBuf    d_box, d_tot, d_flags, d_fpos, d_fscan, d_list, d_ptile, d_pbox, d_psize, d_poff, d_pscan, d_tinfo,
              d_blkna, d_blist, d_tcount;
    PinnedBuf h_tiles, h_tinfo;
    ak_scene  TS{};
    /* the last forward */
    bool         have_fwd = false, sized = false, lane_flat = false;
    const float *f_ctrl = nullptr, *f_colors = nullptr, *f_widths = nullptr, *f_target = nullptr;
};

namespace {

template <class T> bool upload(DevBuf &b, const std::vector<T> &v) {
    size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(T);
    if (!b.grow(bytes))
        return false;
    return cudaMemcpy(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) == cudaSuccess;
}

vkvg_status_t fail(VkvgAnalytic a, cudaError_t e) {
    if (e == cudaSuccess)
        return VKVG_STATUS_SUCCESS;
    /* an allocation that failed (or a tiled scene whose pairs or planes
       outgrow 32-bit offsets) is NO_MEMORY; anything else a device error */
    const vkvg_status_t st = e == cudaErrorMemoryAllocation ? VKVG_STATUS_NO_MEMORY : VKVG_STATUS_DEVICE_ERROR;
    if (a->pending == VKVG_STATUS_SUCCESS)
        a->pending = st;
    return st;
}

bool size_points(VkvgAnalytic a, uint32_t need) {
    if (need <= a->cap)
        return true;
    uint32_t cap = std::max<uint32_t>(need + need / 4, 1024);
    if (!a->d_pts.grow((size_t)cap * sizeof(float2)) || !a->d_pt_nb.grow((size_t)cap * 8) ||
        !a->d_gpts.grow((size_t)cap * sizeof(float2)))
        return false;
    a->cap = cap;
    return true;
}

ak_bufs bufs(VkvgAnalytic a) {
    ak_bufs B;
    B.off     = a->d_off.as<uint32_t>();
    B.pts     = a->d_pts.as<float2>();
    B.pt_nb   = a->d_pt_nb.as<uint2>();
    B.cap     = a->cap;
    B.area    = a->d_area.as<float>();
    B.ckpt    = a->d_ckpt.as<float4>();
    B.canvas  = a->d_canvas.as<float4>();
    B.status  = a->d_status.as<uint32_t>();
    B.blk_na  = a->d_blkna.as<uint32_t>();
    B.blist   = a->d_blist.as<uint32_t>();
    return B;
}

/* fold the last forward's landed point total and status into pending */
void poll(VkvgAnalytic a, bool wait) {
    if (!a->mon_pending)
        return;
    cudaError_t e = wait ? cudaEventSynchronize(a->ev_mon) : cudaEventQuery(a->ev_mon);
    if (e == cudaErrorNotReady)
        return;
    a->mon_pending = false;
    if (e != cudaSuccess) {
        fail(a, e);
        return;
    }
    const uint32_t *m = (const uint32_t *)a->h_mon.p;
    if (m[1] > a->cap) {
        if (a->pending == VKVG_STATUS_SUCCESS)
            a->pending = VKVG_STATUS_NO_MEMORY;
        size_points(a, m[1]);
    } else if (m[0] && a->pending == VKVG_STATUS_SUCCESS) {
        a->pending = VKVG_STATUS_DEVICE_ERROR;
    }
}

} /* namespace */

extern "C" {

} /* extern "C" */

namespace {
VkvgAnalytic create_scene(uint32_t width, uint32_t height, uint32_t tile, const float background[4], uint32_t npaths,
                          const uint32_t *path_ncontours, const uint32_t *path_flags, uint32_t ncontours,
                          const uint32_t *contour_nseg, uint32_t nseg, const uint8_t *seg_kind) {
    /* a band of a window (the canvas, or a tile) must fit in one block's
       shared memory */
    const uint32_t win = tile ? std::min(tile, width) : width;
    if (!width || !height || !npaths || !path_ncontours || !path_flags || !contour_nseg || !seg_kind ||
        ak_cover_smem(win) > 227 * 1024 || height > 65536 || (tile && (tile < 16 || tile > 4096)))
        return nullptr;
    std::vector<uint8_t>  kind(nseg), lstroke;
    std::vector<uint32_t> seg_cp(nseg), seg_end(nseg), seg_cont(nseg), cont_s0(ncontours + 1), path_s0(npaths + 1),
        lpath;
    uint32_t c = 0, s = 0, cp = 0;
    for (uint32_t p = 0; p < npaths; p++) {
        path_s0[p] = s;
        for (uint32_t k = 0; k < path_ncontours[p]; k++, c++) {
            if (c >= ncontours)
                return nullptr;
            cont_s0[c]   = s;
            uint32_t s0 = s, cp0 = cp;
            for (uint32_t q = 0; q < contour_nseg[c]; q++, s++) {
                if (s >= nseg || (seg_kind[s] != AK_SEG_LINE && seg_kind[s] != AK_SEG_CUBIC))
                    return nullptr;
                kind[s] = seg_kind[s], seg_cp[s] = cp, seg_cont[s] = c;
                cp += seg_kind[s];
            }
            for (uint32_t q = s0; q < s; q++)
                seg_end[q] = q + 1 < s ? seg_cp[q + 1] : cp0;
        }
        if (path_flags[p] & AK_FILL)
            lpath.push_back(p), lstroke.push_back(0);
        if (path_flags[p] & AK_STROKE)
            lpath.push_back(p), lstroke.push_back(1);
    }
    if (c != ncontours || s != nseg)
        return nullptr;
    cont_s0[c] = s, path_s0[npaths] = s;
    VkvgAnalytic a = new (std::nothrow) _vkvg_gb300_analytic_t;
    if (!a)
        return nullptr;
    a->W = width, a->H = height, a->npaths = npaths, a->ncontours = ncontours, a->nseg = nseg, a->ncp = cp;
    a->nlayers = (uint32_t)lpath.size();
    a->tile    = tile;
    a->ntx     = tile ? (width + tile - 1) / tile : 1;
    a->nty     = tile ? (height + tile - 1) / tile : 1;
    if (background)
        memcpy(a->bg, background, sizeof a->bg);
    size_t np    = (size_t)width * height;
    size_t nchk  = (a->nlayers + AK_CHUNK - 1) / AK_CHUNK;
    uint32_t nbk = (uint32_t)((np + 255) / 256);
    bool ok = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking) == cudaSuccess;
    a->own_stream = ok;
    ok = ok && cudaEventCreateWithFlags(&a->ev_mon, cudaEventDisableTiming) == cudaSuccess;
    ok = ok && upload(a->d_seg_kind, kind) && upload(a->d_seg_cp, seg_cp) && upload(a->d_seg_end, seg_end) &&
         upload(a->d_seg_contour, seg_cont) && upload(a->d_cont_s0, cont_s0) && upload(a->d_path_s0, path_s0) &&
         upload(a->d_layer_path, lpath) && upload(a->d_layer_stroke, lstroke);
    ok = ok && a->d_cnt.grow(4 * ((size_t)nseg + 1)) && a->d_off.grow(4 * ((size_t)nseg + 1)) &&
         a->d_scan.grow(4 * gb_scan_scratch_words(nseg + 1)) && a->d_canvas.grow(sizeof(float4) * np) &&
         a->d_loss.grow(sizeof(float)) && a->d_status.grow(4) && a->h_mon.grow(8) &&
         size_points(a, 65536) /* the first forward sizes it */;
    if (!tile) /* one window: its planes are sized now */
        ok = ok && a->d_area.grow(sizeof(float) * np * std::max<uint32_t>(a->nlayers, 1)) &&
             a->d_ckpt.grow(sizeof(float4) * np * std::max<size_t>(nchk, 1)) && a->d_loss_part.grow(sizeof(float) * nbk) &&
             a->d_color_part.grow(sizeof(float4) * (size_t)(np + 127) / 128 * std::max<uint32_t>(a->nlayers, 1));
    else
        ok = ok && a->d_box.grow(sizeof(int4) * std::max<uint32_t>(a->nlayers, 1)) && a->d_tot.grow(8);
    ok = ok && cudaMemset(a->d_status.p, 0, 4) == cudaSuccess;
    if (!ok) {
        vkvg_gb300_analytic_destroy(a);
        return nullptr;
    }
    ak_scene &S    = a->S;
    S.W = width, S.H = height, S.npaths = npaths, S.ncontours = ncontours, S.nseg = nseg, S.ncp = cp;
    S.CW = width, S.CH = height, S.tiles = 0, S.ntx = 1, S.ntiles = 1;
    S.layer_map = nullptr, S.pair_tile = nullptr, S.tinfo = nullptr;
    S.nlayers      = a->nlayers;
    S.band         = ak_band_rows(width);
    S.nbands       = (height + S.band - 1) / S.band;
    S.bg           = make_float4(a->bg[0], a->bg[1], a->bg[2], a->bg[3]);
    S.seg_kind     = a->d_seg_kind.as<uint8_t>();
    S.seg_cp       = a->d_seg_cp.as<uint32_t>();
    S.seg_end      = a->d_seg_end.as<uint32_t>();
    S.seg_contour  = a->d_seg_contour.as<uint32_t>();
    S.cont_s0      = a->d_cont_s0.as<uint32_t>();
    S.path_s0      = a->d_path_s0.as<uint32_t>();
    S.layer_path   = a->d_layer_path.as<uint32_t>();
    S.layer_stroke = a->d_layer_stroke.as<uint8_t>();
    return a;
}
} /* namespace */

extern "C" {
VkvgAnalytic vkvg_gb300_analytic_create(uint32_t width, uint32_t height, const float background[4], uint32_t npaths,
                                        const uint32_t *path_ncontours, const uint32_t *path_flags,
                                        uint32_t ncontours, const uint32_t *contour_nseg, uint32_t nseg,
                                        const uint8_t *seg_kind) {
    return create_scene(width, height, 0, background, npaths, path_ncontours, path_flags, ncontours, contour_nseg,
                        nseg, seg_kind);
}
VkvgAnalytic vkvg_gb300_analytic_create_tiled(uint32_t width, uint32_t height, uint32_t tile, const float background[4],
                                              uint32_t npaths, const uint32_t *path_ncontours,
                                              const uint32_t *path_flags, uint32_t ncontours,
                                              const uint32_t *contour_nseg, uint32_t nseg, const uint8_t *seg_kind) {
    if (!tile)
        return nullptr;
    return create_scene(width, height, tile, background, npaths, path_ncontours, path_flags, ncontours, contour_nseg,
                        nseg, seg_kind);
}

void vkvg_gb300_analytic_destroy(VkvgAnalytic a) {
    if (!a)
        return;
    if (a->stream)
        cudaStreamSynchronize(a->stream);
    DevBuf *bs[] = {&a->d_seg_kind, &a->d_seg_cp,  &a->d_seg_end, &a->d_seg_contour, &a->d_cont_s0,
                    &a->d_path_s0,  &a->d_layer_path, &a->d_layer_stroke, &a->d_cnt, &a->d_off, &a->d_scan,
                    &a->d_pts, &a->d_pt_nb, &a->d_area, &a->d_ckpt, &a->d_canvas, &a->d_loss_part, &a->d_loss,
                    &a->d_color_part, &a->d_gpts, &a->d_status, &a->d_box, &a->d_flags, &a->d_fpos, &a->d_fscan,
                    &a->d_list, &a->d_ptile, &a->d_tinfo, &a->d_tot, &a->d_pbox, &a->d_psize, &a->d_poff,
                    &a->d_pscan, &a->d_blkna, &a->d_blist, &a->d_tcount};
    for (DevBuf *b : bs)
        b->release();
    a->h_mon.release();
    a->h_tiles.release();
    a->h_tinfo.release();
    if (a->ev_mon)
        cudaEventDestroy(a->ev_mon);
    for (cudaEvent_t ev : a->ev)
        if (ev)
            cudaEventDestroy(ev);
    if (a->own_stream)
        cudaStreamDestroy(a->stream);
    delete a;
}

vkvg_status_t vkvg_gb300_analytic_status(VkvgAnalytic a) { return a ? a->status : VKVG_STATUS_NULL_POINTER; }
uint32_t vkvg_gb300_analytic_control_point_count(VkvgAnalytic a) { return a ? a->ncp : 0; }
uint32_t vkvg_gb300_analytic_layer_count(VkvgAnalytic a) { return a ? a->nlayers : 0; }

vkvg_status_t vkvg_gb300_analytic_set_stream(VkvgAnalytic a, void *stream) {
    if (!a)
        return VKVG_STATUS_NULL_POINTER;
    cudaStreamSynchronize(a->stream);
    if (a->own_stream)
        cudaStreamDestroy(a->stream);
    a->own_stream = false;
    a->stream     = (cudaStream_t)stream;
    return VKVG_STATUS_SUCCESS;
}

} /* extern "C" */

namespace {
/* tiled scenes: the (tile, layer) pairs with each layer's box inside each
   tile, their area planes (one per pair, covering only its box), every
   tile's pairs and checkpoints, the buffers sized for them and the scene of
   the tiled launches (after the flattening of this forward) */
cudaError_t tile_setup(VkvgAnalytic a, const float *widths) {
    cudaStream_t   st = a->stream;
    const uint32_t nt = a->ntx * a->nty, nl = a->nlayers;
    const uint64_t nr64 = (uint64_t)nt * ((nl + AK_TP_LAYERS - 1) / AK_TP_LAYERS);
    if (nr64 >= 0xFFFFFFFFull || (uint64_t)(nt + 7) / 8 > 65535u)
        return cudaErrorMemoryAllocation; /* runs and the launch grid's tile groups */
    const uint32_t nr = ak_tile_runs(nt, nl);
    if (!a->d_flags.grow(4 * ((size_t)nr + 1)) || !a->d_fpos.grow(4 * ((size_t)nr + 1)) ||
        !a->d_fscan.grow(4 * gb_scan_scratch_words(nr) + 64) || !a->d_tcount.grow(4 * (size_t)nt) ||
        !a->h_tiles.grow(4 * ((size_t)nt + 4)) || !a->h_tinfo.grow(sizeof(ak_tile_info) * nt) ||
        !a->d_tinfo.grow(sizeof(ak_tile_info) * nt))
        return cudaErrorMemoryAllocation;
    ak_bufs     B = bufs(a);
    cudaError_t e = cudaMemsetAsync(a->d_tot.p, 0, 8, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(a->d_tcount.p, 0, 4 * (size_t)nt, st);
    if (e == cudaSuccess)
        e = ak_launch_layer_boxes(st, a->S, B, widths, a->d_box.as<int4>(), a->d_tot.as<unsigned long long>());
    /* every tile's pair count and every run's, the boxes tested as the
       entries go by (no flag per entry is stored) */
    if (e == cudaSuccess)
        e = ak_launch_tile_count(st, nt, nl, a->ntx, a->tile, a->d_box.as<int4>(), a->d_flags.as<uint32_t>(),
                                 a->d_tcount.as<uint32_t>());
    uint32_t *h = (uint32_t *)a->h_tiles.p;
    if (e == cudaSuccess) /* the tiles' pair counts, the box pixel total */
        e = cudaMemcpyAsync(h, a->d_tcount.p, 4 * (size_t)nt, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(h + nt + 2, a->d_tot.p, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    gb_count_launch(2);
    if (e != cudaSuccess)
        return e;
    uint64_t total64 = 0;
    for (uint32_t t = 0; t < nt; t++)
        total64 += h[t];
    unsigned long long area;
    memcpy(&area, h + nt + 2, sizeof area);
    /* pair positions and plane offsets are 32-bit */
    if (total64 >= 0xFFFFFFFFull || area >= 0xFFFFFFFFull)
        return cudaErrorMemoryAllocation;
    const uint32_t total = (uint32_t)total64;
    const size_t   np1   = (size_t)std::max<uint32_t>(total, 1);
    if (!a->d_list.grow(4 * np1) || !a->d_ptile.grow(4 * np1) || !a->d_pbox.grow(8 * np1) ||
        !a->d_psize.grow(4 * np1) || !a->d_poff.grow(4 * (np1 + 1)) ||
        !a->d_pscan.grow(4 * gb_scan_scratch_words(total) + 64))
        return cudaErrorMemoryAllocation;
    /* the runs' first pairs, then the pairs in (tile, layer) order */
    e = gb_exclusive_scan(st, a->d_flags.as<uint32_t>(), nr, a->d_fpos.as<uint32_t>(), a->d_fscan.as<uint32_t>());
    if (e == cudaSuccess)
        e = ak_launch_tile_lists(st, nt, nl, a->ntx, a->tile, a->d_box.as<int4>(), a->d_fpos.as<uint32_t>(),
                                 a->d_list.as<uint32_t>(), a->d_ptile.as<uint32_t>(), a->d_pbox.as<uint2>(),
                                 a->d_psize.as<uint32_t>());
    if (e == cudaSuccess) /* every pair's plane: the running sum of the box sizes */
        e = gb_exclusive_scan(st, a->d_psize.as<uint32_t>(), total, a->d_poff.as<uint32_t>(),
                              a->d_pscan.as<uint32_t>());
    gb_count_launch((nr ? 4 : 0) + (total ? 3 : 0));
    /* every tile's first pair and checkpoints: a tile of tw x th pixels and
       c layers holds ceil(c / AK_CHUNK) planes of tw x th */
    ak_tile_info *ti    = (ak_tile_info *)a->h_tinfo.p;
    size_t        ckpt  = 0;
    uint32_t      first = 0;
    for (uint32_t t = 0; t < nt; t++) {
        const uint32_t tw = std::min(a->tile, a->W - (t % a->ntx) * a->tile);
        const uint32_t th = std::min(a->tile, a->H - (t / a->ntx) * a->tile);
        const size_t   px = (size_t)tw * th, cnt = h[t];
        ti[t].first = first, ti[t].count = (uint32_t)cnt, ti[t].ckpt = ckpt;
        first += (uint32_t)cnt;
        ckpt += px * ((cnt + AK_CHUNK - 1) / AK_CHUNK);
    }
    ak_scene &T = a->TS;
    T           = a->S;
    T.tiles = a->tile, T.ntx = a->ntx, T.ntiles = nt;
    T.W = T.H    = a->tile;
    T.band       = std::min(16u, ak_band_rows(a->tile)); /* the pairs' accumulators: a small box fits one band */
    T.nbands     = (a->tile + T.band - 1) / T.band;
    T.nlayers    = total;
    T.layer_map  = a->d_list.as<uint32_t>();
    T.pair_tile  = a->d_ptile.as<uint32_t>();
    T.pair_box   = a->d_pbox.as<uint2>();
    T.pair_off   = a->d_poff.as<uint32_t>();
    T.tinfo      = a->d_tinfo.as<ak_tile_info>();
    if (!a->d_area.grow(sizeof(float) * std::max<size_t>(area, 1)) ||
        !a->d_ckpt.grow(sizeof(float4) * std::max<size_t>(ckpt, 1)) ||
        !a->d_loss_part.grow(sizeof(float) * ak_pixel_blocks_all(T)) ||
        !a->d_blkna.grow(sizeof(uint32_t) * ak_pixel_blocks_all(T)) ||
        !a->d_blist.grow(sizeof(uint32_t) * std::max<size_t>((size_t)total * ak_pixel_blocks(T), 1)) ||
        !a->d_color_part.grow(sizeof(float4) * std::max<size_t>(ak_color_partials(T), 1)))
        return cudaErrorMemoryAllocation;
    if (e == cudaSuccess) /* pinned, copied in stream order before the launches that read it */
        e = cudaMemcpyAsync(a->d_tinfo.p, ti, sizeof(ak_tile_info) * nt, cudaMemcpyHostToDevice, st);
    return e;
}
} /* namespace */

extern "C" {
vkvg_status_t vkvg_gb300_analytic_forward(VkvgAnalytic a, const float *ctrl, const float *colors,
                                          const float *widths, const float *target, float *canvas, float *loss) {
    if (!a)
        return VKVG_STATUS_NULL_POINTER;
    if (a->status)
        return a->status;
    if (!ctrl || !colors || !widths || (loss && !target))
        return VKVG_STATUS_NULL_POINTER;
    poll(a, false);
    cudaStream_t st = a->stream;
    const float2 *c2 = (const float2 *)ctrl;
    if (a->timing)
        cudaEventRecord(a->ev[0], st);
    cudaError_t e = ak_launch_flat_count(st, a->S, c2, a->d_cnt.as<uint32_t>(), a->lane_flat);
    if (e == cudaSuccess)
        e = gb_exclusive_scan(st, a->d_cnt.as<uint32_t>(), a->nseg, a->d_off.as<uint32_t>(), a->d_scan.as<uint32_t>());
    gb_count_launch(4);
    if (e != cudaSuccess)
        return fail(a, e);
    uint32_t *mon = (uint32_t *)a->h_mon.p;
    if (!a->sized) { /* the first evaluation sizes the point buffer */
        if (cudaMemcpyAsync(&mon[1], a->d_off.as<uint32_t>() + a->nseg, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess)
            return fail(a, cudaGetLastError());
        if (!size_points(a, mon[1]))
            return a->pending = VKVG_STATUS_NO_MEMORY;
        a->sized = true;
        /* small curves (at most 8 points per segment on average): a lane per
           segment walks them with fewer idle lanes than a warp per segment */
        a->lane_flat = (uint64_t)mon[1] <= 8ull * a->nseg;
    }
    ak_bufs B = bufs(a);
    e         = ak_launch_flat_emit(st, a->S, c2, B.off, a->d_pts.as<float2>(), a->d_pt_nb.as<uint2>(), a->cap,
                                    B.status, a->lane_flat);
    if (a->tile && e == cudaSuccess) { /* tiled: the (tile, layer) pairs, then one launch for all tiles */
        e = tile_setup(a, widths);
        B = bufs(a); /* the planes were sized (and may have moved) for this forward's pairs */
    }
    {
        const ak_scene &S = a->tile ? a->TS : a->S;
        if (a->timing)
            cudaEventRecord(a->ev[1], st);
        if (e == cudaSuccess)
            e = ak_launch_cover(st, S, B, widths);
        if (a->timing)
            cudaEventRecord(a->ev[2], st);
        if (e == cudaSuccess)
            e = ak_launch_composite(st, S, B, (const float4 *)colors, (const float4 *)target,
                                    target ? a->d_loss_part.as<float>() : nullptr);
        gb_count_launch(3);
        if (e == cudaSuccess && loss) {
            e = ak_launch_reduce(st, S, ak_pixel_blocks_all(S), nullptr, nullptr, a->d_loss_part.as<float>(), loss);
            gb_count_launch(1);
        }
        if (a->timing)
            cudaEventRecord(a->ev[3], st);
    }
    if (e == cudaSuccess && canvas)
        e = cudaMemcpyAsync(canvas, a->d_canvas.p, sizeof(float4) * a->W * a->H, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && !a->mon_pending) {
        e = cudaMemcpyAsync(&mon[0], a->d_status.p, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(&mon[1], a->d_off.as<uint32_t>() + a->nseg, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess)
            e = cudaEventRecord(a->ev_mon, st);
        a->mon_pending = e == cudaSuccess;
    }
    if (e != cudaSuccess)
        return fail(a, e);
    a->have_fwd = true;
    a->f_ctrl = ctrl, a->f_colors = colors, a->f_widths = widths, a->f_target = target;
    return VKVG_STATUS_SUCCESS;
}

vkvg_status_t vkvg_gb300_analytic_backward(VkvgAnalytic a, const float *d_canvas, float *d_ctrl, float *d_colors,
                                           float *d_widths) {
    if (!a)
        return VKVG_STATUS_NULL_POINTER;
    if (a->status)
        return a->status;
    if (!a->have_fwd || (!d_canvas && !a->f_target))
        return VKVG_STATUS_INVALID_STATUS;
    if (!d_ctrl || !d_colors || !d_widths)
        return VKVG_STATUS_NULL_POINTER;
    cudaStream_t st = a->stream;
    ak_bufs      B  = bufs(a);
    uint32_t     nb = ak_composite_bwd_blocks(a->S);
    cudaError_t  e  = cudaMemsetAsync(d_ctrl, 0, sizeof(float) * 2 * a->ncp, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d_colors, 0, sizeof(float) * 4 * a->npaths, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(d_widths, 0, sizeof(float) * a->npaths, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(a->d_gpts.p, 0, sizeof(float2) * a->cap, st);
    if (a->timing)
        cudaEventRecord(a->ev[4], st);
    {
        const ak_scene &S = a->tile ? a->TS : a->S; /* tiled: every tile in one launch */
        if (e == cudaSuccess)
            e = ak_launch_composite_bwd(st, S, B, (const float4 *)a->f_colors, (const float4 *)a->f_target,
                                        (const float4 *)d_canvas, a->d_color_part.as<float4>());
        if (e == cudaSuccess)
            e = ak_launch_reduce(st, S, a->tile ? ak_composite_bwd_blocks(S) : nb, a->d_color_part.as<float4>(),
                                 (float4 *)d_colors, nullptr, nullptr);
        if (a->timing)
            cudaEventRecord(a->ev[5], st);
        if (e == cudaSuccess)
            e = ak_launch_cover_bwd(st, S, B, a->f_widths, a->d_gpts.as<float2>(), d_widths);
        if (a->timing)
            cudaEventRecord(a->ev[6], st);
    }
    if (e == cudaSuccess)
        e = ak_launch_flat_bwd(st, a->S, (const float2 *)a->f_ctrl, B.off, a->cap, a->d_gpts.as<float2>(),
                               (float2 *)d_ctrl, a->lane_flat);
    if (a->timing)
        cudaEventRecord(a->ev[7], st);
    gb_count_launch(4);
    a->have_fwd = false; /* the areas now hold their gradients */
    return fail(a, e);
}

vkvg_status_t vkvg_gb300_analytic_adam(VkvgAnalytic a, float *param, const float *grad, float *m, float *v,
                                       uint32_t n, float lr, float beta1, float beta2, float eps, uint32_t step,
                                       float lo, float hi) {
    if (!a)
        return VKVG_STATUS_NULL_POINTER;
    if (a->status)
        return a->status;
    if (!param || !grad || !m || !v || !step)
        return VKVG_STATUS_NULL_POINTER;
    gb_count_launch(n ? 1 : 0);
    return fail(a, ak_launch_adam(a->stream, param, grad, m, v, n, lr, beta1, beta2, eps, step, lo, hi));
}

vkvg_status_t vkvg_gb300_analytic_sync(VkvgAnalytic a) {
    if (!a)
        return VKVG_STATUS_NULL_POINTER;
    if (a->status)
        return a->status;
    cudaError_t e = cudaStreamSynchronize(a->stream);
    if (e != cudaSuccess)
        fail(a, e);
    poll(a, true);
    vkvg_status_t s = a->pending;
    a->pending      = VKVG_STATUS_SUCCESS;
    if (s != VKVG_STATUS_SUCCESS)
        cudaMemsetAsync(a->d_status.p, 0, 4, a->stream);
    return s;
}

uint32_t vkvg_gb300_analytic_points(VkvgAnalytic a, float *pts, uint32_t cap, uint32_t *seg_offsets) {
    if (!a || a->status || cudaStreamSynchronize(a->stream) != cudaSuccess)
        return 0;
    std::vector<uint32_t> off(a->nseg + 1);
    if (cudaMemcpy(off.data(), a->d_off.p, 4 * off.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
        return 0;
    uint32_t n = off[a->nseg];
    if (n > a->cap)
        return 0;
    if (pts && cap)
        cudaMemcpy(pts, a->d_pts.p, sizeof(float2) * std::min(n, cap), cudaMemcpyDeviceToHost);
    if (seg_offsets)
        memcpy(seg_offsets, off.data(), 4 * off.size());
    return n;
}

vkvg_status_t vkvg_gb300_analytic_set_timing(VkvgAnalytic a, int on) {
    if (!a)
        return VKVG_STATUS_NULL_POINTER;
    if (on && !a->ev[0])
        for (cudaEvent_t &ev : a->ev)
            if (cudaEventCreate(&ev) != cudaSuccess)
                return VKVG_STATUS_DEVICE_ERROR;
    a->timing = on != 0;
    return VKVG_STATUS_SUCCESS;
}

vkvg_status_t vkvg_gb300_analytic_timing(VkvgAnalytic a, float out[6]) {
    if (!a || !out)
        return VKVG_STATUS_NULL_POINTER;
    if (!a->timing || cudaStreamSynchronize(a->stream) != cudaSuccess)
        return VKVG_STATUS_INVALID_STATUS;
    for (int k = 0; k < 6; k++) {
        int i0 = k < 3 ? k : k + 1;
        if (cudaEventElapsedTime(&out[k], a->ev[i0], a->ev[i0 + 1]) != cudaSuccess)
            out[k] = -1.f;
    }
    return VKVG_STATUS_SUCCESS;
}

uint32_t vkvg_gb300_analytic_point_grads(VkvgAnalytic a, float *grads, uint32_t cap) {
    if (!a || a->status || cudaStreamSynchronize(a->stream) != cudaSuccess)
        return 0;
    uint32_t n = 0;
    if (cudaMemcpy(&n, a->d_off.as<uint32_t>() + a->nseg, 4, cudaMemcpyDeviceToHost) != cudaSuccess || n > a->cap)
        return 0;
    if (grads && cap)
        cudaMemcpy(grads, a->d_gpts.p, sizeof(float2) * std::min(n, cap), cudaMemcpyDeviceToHost);
    return n;
}

} /* extern "C" */
