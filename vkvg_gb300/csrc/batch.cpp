/* Batches: many recorded frames, each for its own surface, rendered as one
 * job (no vkvg counterpart: vkvg renders a surface per command buffer).
 *
 * The frames' command arrays are merged into one device-resident frame whose
 * draws carry their surface's index; one pass of the flatten, stroke, set-up
 * and binning kernels covers every surface (each surface's cells are its own
 * block of the bins), and one launch of the persistent batch raster renders
 * every (surface, band, tile) item, heaviest first.  The first execution
 * establishes the sizes; the next few compare raster settings (the stage
 * threshold and the work-list order) and keep the fastest for this class of
 * scene; from then on the whole job is one CUDA graph launch.
 */
#include "host.h"
#include "launch.h"

#include <algorithm>
#include <map>
#include <new>
#include <stdio.h>
#include <tuple>

namespace {

/* raster settings the tuner chooses between */
struct RasterParams {
    uint32_t stage_min;  /* cells of fewer record units skip the shared-memory stage */
    bool     cost_order; /* work list heaviest first (else surface, band, tile order) */
    int      form;       /* tiles: 0 1024 pixels (one CTA per SM), 1 256 (four), 2 512 (two), 3 128 (eight),
                            4 64 (sixteen) */
};
const RasterParams CANDIDATES[] = {{0, true, 0},  {8, true, 0}, {32, true, 0}, {0, false, 0}, {0, true, 2},
                                   {8, true, 2},  {32, true, 2}, {0, true, 1}, {8, true, 1},  {32, true, 1},
                                   {0, true, 3},  {32, true, 3}, {64, true, 3}, {64, true, 4}};
constexpr int NFORMS = 5;
constexpr int      NCAND        = sizeof(CANDIDATES) / sizeof(CANDIDATES[0]);

/* the tuner's choice per class of scene: surfaces, draws and record units,
   each by power of two */
std::mutex                                          g_tune_mtx;
std::map<std::tuple<int, int, int>, RasterParams> g_tuned;
int log2i(uint64_t v) {
    int k = 0;
    while (v > 1) {
        v >>= 1;
        k++;
    }
    return k;
}

} /* namespace */

struct _vkvg_gb300_batch_t {
    std::vector<SurfRef> targets;
    FrameHost            merged;
    Pipeline             pl;
    std::vector<gb_surf> tab;
    DevBuf               d_tab, d_items, d_queue, d_idx, d_units;
    PinnedBuf            h_stage;
    std::vector<uint4>   items_cost[NFORMS], items_plain[NFORMS]; /* the work lists (per tile form) in both orders */
    /* pattern source images: per surface, its frame's images [n][H][W] in
       one buffer; the merged frame's gradient records in the same order */
    DevBuf                d_grad;
    std::vector<uint32_t> grad_surf; /* per merged gradient record: its surface */
    std::vector<size_t>   grad_off;  /* per merged gradient record: its image's offset in d_grad, words */
    uint64_t             ncells  = 0;
    uint64_t             every   = 0; /* cells of the draws that act on every band */
    uint32_t             samples = 0;
    uint32_t             nctas   = 1; /* persistent raster CTAs: one per SM */
    int                  runs    = 0; /* executions so far */
    RasterParams         params  = CANDIDATES[0];
    bool                 tuned   = false;
    float                cand_ms[NCAND];
    cudaGraphExec_t      exec       = nullptr;
    uint64_t             graph_kern = 0; /* kernels in the graph */
    float                last_ms    = 0;
    bool                 last_graph = false;
    cudaEvent_t          ev0 = nullptr, ev1 = nullptr;
};

namespace {

/* append frame k's arrays to the merged frame, indices rebased */
bool merge_frame(FrameHost &m, const FrameHost &f, uint32_t k) {
    const uint32_t seg0 = (uint32_t)m.seg_info.size(), sub0 = (uint32_t)m.sub_seg0.size();
    const uint32_t draw0 = (uint32_t)m.draws.size(), sp0 = (uint32_t)m.spair_draw.size();
    const uint32_t dash0 = (uint32_t)m.dashes.size(), th0 = (uint32_t)m.thetas.size();
    for (const gb_draw &d : f.draws)
        if (d.kind >= GB_DRAW_CLIP_EO)
            return false; /* clip is not batched */
    /* pattern sources: a draw's gsrc stays an index into its own frame's
       images, which its surface's table entry points at */
    m.grads.insert(m.grads.end(), f.grads.begin(), f.grads.end());
    m.sources.insert(m.sources.end(), f.sources.begin(), f.sources.end());
    for (size_t i = 0; i < f.seg_info.size(); i++) {
        m.seg_info.push_back(f.seg_info[i]);
        m.seg_n.push_back(f.seg_n[i]);
        m.seg_aux.push_back(GB_SEG_KIND(f.seg_info[i]) == GB_SEG_ELLIPSE ? f.seg_aux[i] + th0 : f.seg_aux[i]);
        m.seg_a.push_back(f.seg_a[i]);
        m.seg_b.push_back(f.seg_b[i]);
        m.seg_c.push_back(f.seg_c[i]);
    }
    for (size_t i = 0; i < f.sub_seg0.size(); i++) {
        m.sub_seg0.push_back(f.sub_seg0[i] + seg0);
        m.sub_nseg.push_back(f.sub_nseg[i]);
        m.sub_flags.push_back(f.sub_flags[i]);
    }
    for (gb_draw d : f.draws) {
        d.sub_first += sub0;
        d.dash_first += dash0;
        d.surf = k;
        m.draws.push_back(d);
    }
    for (size_t i = 0; i < f.spair_draw.size(); i++) {
        m.spair_draw.push_back(f.spair_draw[i] + draw0);
        m.spair_sub.push_back(f.spair_sub[i] + sub0);
        m.spair_dfirst.push_back(f.spair_dfirst[i] + sp0);
    }
    for (uint32_t id : f.sdraw_id)
        m.sdraw_id.push_back(id + draw0);
    /* per stroke draw its first pair; one sentinel at the end of the merge */
    for (size_t i = 0; i + 1 < f.sdraw_pair0.size(); i++)
        m.sdraw_pair0.push_back(f.sdraw_pair0[i] + sp0);
    for (size_t i = 0; i < f.fpair_draw.size(); i++) {
        m.fpair_draw.push_back(f.fpair_draw[i] + draw0);
        m.fpair_sub.push_back(f.fpair_sub[i] + sub0);
    }
    m.dashes.insert(m.dashes.end(), f.dashes.begin(), f.dashes.end());
    m.thetas.insert(m.thetas.end(), f.thetas.begin(), f.thetas.end());
    m.paths += f.paths;
    m.any_dash    = m.any_dash || f.any_dash;
    m.dash_shared = m.dash_shared || f.dash_shared;
    if (f.any_dash)
        m.dash_sub_hi = std::max(m.dash_sub_hi, f.dash_sub_hi + sub0);
    return true;
}

/* a first draw the raster applies while loading the tile (as for a single
   frame): a clear, or an opaque solid paint with OVER or SOURCE */
void first_draw_init(const gb_draw *d, uint32_t n, gb_surf &s) {
    s.init_mode = s.init_color = s.draw_first = 0;
    if (!n)
        return;
    if (d[0].kind == GB_DRAW_CLEAR) {
        s.init_mode  = 1;
        s.init_color = 0;
        s.draw_first = 1;
    } else if (d[0].kind == GB_DRAW_PAINT && (d[0].op == GB_OP_OVER || d[0].op == GB_OP_SOURCE) &&
               (d[0].src >> 24) == 255u && d[0].gsrc == 0) {
        s.init_mode  = 1;
        s.init_color = d[0].src;
        s.draw_first = 1;
    }
}

} /* namespace */

#define BCK(x)                                                                                                         \
    do {                                                                                                               \
        cudaError_t _e = (x);                                                                                          \
        if (_e != cudaSuccess)                                                                                         \
            return _e;                                                                                                 \
    } while (0)

namespace {

/* the work lists: every (surface, band, tile) for each tile form, in
   surface order and sorted by the band's record units (heaviest first); all
   six kept on the device, one after another */
cudaError_t build_items(VkvgBatch b) {
    Pipeline            &pl = b->pl;
    std::vector<uint64_t> idx;
    for (const gb_surf &s : b->tab)
        for (uint32_t k = 0; k <= s.nbands; k++)
            idx.push_back(s.cell0 + (uint64_t)k * s.ndraws);
    const uint32_t n = (uint32_t)idx.size();
    if (!b->d_idx.grow(n * 8) || !b->d_units.grow(n * 4) || !b->h_stage.grow(std::max<size_t>(n * 8, 64)))
        return cudaErrorMemoryAllocation;
    memcpy(b->h_stage.p, idx.data(), n * 8);
    BCK(cudaMemcpyAsync(b->d_idx.p, b->h_stage.p, n * 8, cudaMemcpyHostToDevice, pl.st));
    BCK(gb_launch_gather_u32(pl.st, n, b->d_idx.as<uint64_t>(), pl.cells.as<uint32_t>(), b->d_units.as<uint32_t>()));
    gb_count_launch(1);
    std::vector<uint32_t> off(n);
    BCK(cudaMemcpyAsync(b->h_stage.p, b->d_units.p, n * 4, cudaMemcpyDeviceToHost, pl.st));
    BCK(cudaStreamSynchronize(pl.st));
    memcpy(off.data(), b->h_stage.p, n * 4);
    size_t tot = 0;
    for (int nw = 0; nw < NFORMS; nw++) {
        const uint32_t                          tw = gb_raster_tile_width(nw);
        std::vector<std::pair<uint32_t, uint4>> costed;
        b->items_plain[nw].clear();
        size_t j = 0;
        for (uint32_t si = 0; si < b->tab.size(); si++) {
            const gb_surf &s     = b->tab[si];
            const uint32_t tiles = (s.W + tw - 1) / tw;
            for (uint32_t band = 0; band < s.nbands; band++, j++) {
                const uint32_t units = off[j + 1] - off[j];
                for (uint32_t t = 0; t < tiles; t++) {
                    const uint4 it = make_uint4(si, band, t, units);
                    b->items_plain[nw].push_back(it);
                    costed.push_back({units, it});
                }
            }
            j++; /* the surface's end boundary */
        }
        std::stable_sort(costed.begin(), costed.end(),
                         [](const std::pair<uint32_t, uint4> &x, const std::pair<uint32_t, uint4> &y) {
                             return x.first > y.first;
                         });
        b->items_cost[nw].clear();
        for (auto &c : costed)
            b->items_cost[nw].push_back(c.second);
        tot += 2 * b->items_plain[nw].size();
    }
    if (!b->d_items.grow(std::max<size_t>(tot * 16, 16)) || !b->h_stage.grow(std::max<size_t>(tot * 16, 64)))
        return cudaErrorMemoryAllocation;
    uint8_t *h = (uint8_t *)b->h_stage.p;
    for (int nw = 0; nw < NFORMS; nw++) {
        memcpy(h, b->items_plain[nw].data(), b->items_plain[nw].size() * 16);
        h += b->items_plain[nw].size() * 16;
        memcpy(h, b->items_cost[nw].data(), b->items_cost[nw].size() * 16);
        h += b->items_cost[nw].size() * 16;
    }
    BCK(cudaMemcpyAsync(b->d_items.p, b->h_stage.p, tot * 16, cudaMemcpyHostToDevice, pl.st));
    return cudaStreamSynchronize(pl.st);
}

/* one execution on the batch's stream: geometry (with the sizes read back
   unless sized), the batch raster with settings p, the status read back */
cudaError_t run_batch(VkvgBatch b, bool sized, const RasterParams &p) {
    Pipeline &pl = b->pl;
    bool wide = false; /* the draws' x extents, for every tile width a candidate uses (down to 128 pixels) */
    for (const gb_surf &s : b->tab)
        wide |= s.W > gb_raster_tile_width(4);
    BCK(pl.geometry(b->merged, b->d_tab.as<gb_surf>(), (uint32_t)b->tab.size(), b->ncells, b->every, wide,
                    b->samples, false, sized));
    if (!sized)
        BCK(build_items(b));
    const int      nw   = p.form;
    const uint32_t ni   = (uint32_t)b->items_plain[nw].size();
    size_t         base = 0; /* this form's lists on the device */
    for (int k = 0; k < nw; k++)
        base += 2 * b->items_plain[k].size();
    gb_raster_args A0;
    memset(&A0, 0, sizeof(A0));
    A0.S         = b->samples;
    A0.draws     = (const gb_draw *)((const uint8_t *)pl.in.p + pl.o_draws);
    A0.cell_off  = pl.cells.as<uint32_t>();
    A0.apos      = pl.apos.as<uint32_t>();
    A0.alist     = pl.alist.as<uint32_t>();
    A0.dbox      = pl.dbox.as<int2>();
    A0.recs      = pl.recs.as<int4>();
    A0.nunits    = pl.nunits;
    A0.status    = pl.status.as<uint32_t>();
    A0.stage_min = p.stage_min;
    /* every surface's pattern source images (its frame's gradients and surface sources) */
    const gb_grad *g = (const gb_grad *)((const uint8_t *)pl.in.p + pl.o_grads);
    for (size_t i = 0; i < b->grad_surf.size(); i++) {
        const gb_surf &s = b->tab[b->grad_surf[i]];
        BCK(gb_launch_gradient_fill(pl.st, s.W, s.H, g + i, b->d_grad.as<uint32_t>() + b->grad_off[i]));
    }
    gb_count_launch(b->grad_surf.size());
    BCK(cudaMemsetAsync(b->d_queue.p, 0, 4, pl.st));
    BCK(gb_launch_raster_batch(pl.st, &A0, b->d_tab.as<gb_surf>(),
                               b->d_items.as<uint4>() + base + (p.cost_order ? ni : 0),
                               ni, b->d_queue.as<uint32_t>(), b->nctas, p.form, b->grad_surf.empty() ? 0 : 1));
    gb_count_launch(ni ? 1 : 0);
    return cudaMemcpyAsync(pl.rb.p, pl.status.p, 4, cudaMemcpyDeviceToHost, pl.st);
}

} /* namespace */

extern "C" {
VkvgBatch vkvg_gb300_batch_create(VkvgFrame *frames, VkvgSurface *targets, uint32_t count) {
    if (!frames || !targets || !count)
        return nullptr;
    _vkvg_gb300_batch_t *b = new (std::nothrow) _vkvg_gb300_batch_t();
    if (!b)
        return nullptr;
    int  nsm = 0, cur = 0;
    bool ok  = b->pl.init() && cudaEventCreate(&b->ev0) == cudaSuccess && cudaEventCreate(&b->ev1) == cudaSuccess &&
              b->d_queue.grow(16) && cudaGetDevice(&cur) == cudaSuccess &&
              cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, cur) == cudaSuccess;
    b->nctas = (uint32_t)std::max(nsm, 1);
    for (uint32_t k = 0; ok && k < count; k++) {
        VkvgFrame   fr = frames[k];
        VkvgSurface s  = targets[k];
        ok = fr && !vkvg_surface_status(s) && s->width == fr->width && s->height == fr->height &&
             s->samples == fr->samples && !s->clip_active && !s->save_nz && (k == 0 || s->samples == b->samples);
        for (uint32_t j = 0; ok && j < k; j++)
            ok = targets[j] != s; /* one frame per surface */
        if (!ok)
            break;
        b->samples          = s->samples;
        const uint32_t d0   = (uint32_t)b->merged.draws.size();
        const size_t   g0   = b->merged.grads.size();
        ok                  = merge_frame(b->merged, fr->frame, k);
        size_t gwords = 0; /* the images before this surface's */
        for (size_t gi = 0; gi < b->grad_off.size(); gi++)
            gwords = std::max(gwords, b->grad_off[gi] + (size_t)b->tab[b->grad_surf[gi]].W * b->tab[b->grad_surf[gi]].H);
        for (size_t gi = g0; ok && gi < b->merged.grads.size(); gi++) {
            b->grad_surf.push_back(k);
            b->grad_off.push_back(gwords + (gi - g0) * (size_t)s->width * s->height);
        }
        gb_surf e;
        memset(&e, 0, sizeof(e));
        e.W       = s->width;
        e.H       = s->height;
        e.nrows   = s->nrows;
        e.nbands  = s->nbands;
        e.wpad    = s->wpad;
        e.draw0   = d0;
        e.ndraws  = (uint32_t)b->merged.draws.size() - d0;
        e.cell0   = b->ncells;
        e.samples = s->d_samples;
        e.rgba    = s->d_rgba;
        first_draw_init(b->merged.draws.data() + d0, e.ndraws, e);
        b->ncells += (uint64_t)e.nbands * e.ndraws;
        for (uint32_t j = d0; j < d0 + e.ndraws; j++)
            b->every += b->merged.draws[j].kind > GB_DRAW_STROKE ? e.nbands : 0u;
        b->tab.push_back(e);
        b->targets.emplace_back(s);
    }
    if (ok && !b->merged.sdraw_id.empty())
        b->merged.sdraw_pair0.push_back((uint32_t)b->merged.spair_draw.size());
    if (ok && !b->grad_surf.empty()) {
        /* one buffer for every surface's source images; each surface's entry
           points at its first */
        size_t words = 0;
        for (size_t gi = 0; gi < b->grad_off.size(); gi++)
            words = std::max(words, b->grad_off[gi] + (size_t)b->tab[b->grad_surf[gi]].W * b->tab[b->grad_surf[gi]].H);
        ok = b->d_grad.grow(words * 4);
        for (size_t gi = b->grad_off.size(); ok && gi-- > 0;)
            b->tab[b->grad_surf[gi]].gsrc = b->d_grad.as<uint32_t>() + b->grad_off[gi];
    }
    const size_t tb = b->tab.size() * sizeof(gb_surf);
    ok = ok && b->pl.upload(b->merged) == cudaSuccess && b->d_tab.grow(tb) && b->h_stage.grow(tb);
    if (ok) {
        memcpy(b->h_stage.p, b->tab.data(), tb);
        ok = cudaMemcpyAsync(b->d_tab.p, b->h_stage.p, tb, cudaMemcpyHostToDevice, b->pl.st) == cudaSuccess &&
             cudaStreamSynchronize(b->pl.st) == cudaSuccess;
    }
    if (!ok) {
        vkvg_gb300_batch_destroy(b);
        return nullptr;
    }
    return b;
}

vkvg_status_t vkvg_gb300_batch_execute(VkvgBatch b) {
    if (!b)
        return VKVG_STATUS_NULL_POINTER;
    std::vector<std::unique_lock<std::mutex>> locks;
    for (SurfRef &t : b->targets)
        locks.emplace_back(t.s->mtx);
    Pipeline   &pl = b->pl;
    cudaError_t e  = cudaSuccess;
    b->last_graph  = false;
    if (b->runs == 0) {
        /* sizes, work list; a tuned class skips the comparison */
        e = cudaEventRecord(b->ev0, pl.st);
        if (e == cudaSuccess)
            e = run_batch(b, false, b->params);
        if (e == cudaSuccess) {
            std::lock_guard<std::mutex> lk(g_tune_mtx);
            auto it = g_tuned.find({log2i(b->tab.size()), log2i(pl.ndraw), log2i(pl.nunits)});
            if (it != g_tuned.end()) {
                b->params = it->second;
                b->tuned  = true;
            }
        }
    } else if (!b->tuned) {
        /* one execution per candidate setting, then keep the fastest */
        const int c = b->runs - 1;
        e           = cudaEventRecord(b->ev0, pl.st);
        if (e == cudaSuccess)
            e = run_batch(b, true, CANDIDATES[c]);
        if (e == cudaSuccess)
            e = cudaEventRecord(b->ev1, pl.st);
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(pl.st);
        if (e == cudaSuccess) {
            cudaEventElapsedTime(&b->cand_ms[c], b->ev0, b->ev1);
            if (c == NCAND - 1) {
                int best = 0;
                for (int k = 1; k < NCAND; k++)
                    if (b->cand_ms[k] < b->cand_ms[best])
                        best = k;
                b->params = CANDIDATES[best];
                b->tuned  = true;
                std::lock_guard<std::mutex> lk(g_tune_mtx);
                g_tuned[{log2i(b->tab.size()), log2i(pl.ndraw), log2i(pl.nunits)}] = b->params;
            }
        }
    } else {
        if (!b->exec) {
            /* the whole job as one graph, with the tuned settings */
            cudaGraph_t    g  = nullptr;
            const uint64_t l0 = vkvg_gb300_kernel_launches();
            e                 = cudaStreamBeginCapture(pl.st, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                cudaError_t e2 = run_batch(b, true, b->params);
                e              = cudaStreamEndCapture(pl.st, &g);
                if (e2 != cudaSuccess)
                    e = e2;
            }
            b->graph_kern = vkvg_gb300_kernel_launches() - l0;
            if (e == cudaSuccess)
                e = cudaGraphInstantiate(&b->exec, g, 0);
            if (g)
                cudaGraphDestroy(g);
        }
        if (e == cudaSuccess)
            e = cudaEventRecord(b->ev0, pl.st);
        if (e == cudaSuccess)
            e = cudaGraphLaunch(b->exec, pl.st);
        gb_count_launch(b->graph_kern);
        b->last_graph = true;
    }
    if (e == cudaSuccess)
        e = cudaEventRecord(b->ev1, pl.st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(pl.st);
    if (e == cudaSuccess)
        cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
    b->runs++;
    if (e == cudaErrorMemoryAllocation)
        return VKVG_STATUS_NO_MEMORY;
    if (e != cudaSuccess) {
        fprintf(stderr, "vkvg_gb300: batch: CUDA error %s\n", cudaGetErrorString(e));
        return VKVG_STATUS_DEVICE_ERROR;
    }
    const uint32_t st = *(const uint32_t *)pl.rb.p;
    if (st & (GB_ERR_RASTER_WAIT | GB_ERR_OVERFLOW)) {
        fprintf(stderr, "vkvg_gb300: batch: device status 0x%x\n", st);
        return VKVG_STATUS_DEVICE_ERROR;
    }
    return VKVG_STATUS_SUCCESS;
}

vkvg_status_t vkvg_gb300_batch_timing(VkvgBatch b, float out[9]) {
    if (!b || !out)
        return VKVG_STATUS_NULL_POINTER;
    out[0] = b->last_ms;
    out[1] = b->last_graph ? 1.f : 0.f;
    out[2] = (float)b->params.stage_min;
    out[3] = b->params.cost_order ? 1.f : 0.f;
    out[4] = (float)b->items_plain[b->params.form].size();
    out[5] = (float)b->tab.size();
    out[6] = b->tuned ? 1.f : 0.f;
    out[7] = (float)b->pl.nunits;
    out[8] = (float)gb_raster_tile_width(b->params.form);
    return VKVG_STATUS_SUCCESS;
}

void vkvg_gb300_batch_destroy(VkvgBatch b) {
    if (!b)
        return;
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    b->pl.destroy();
    DevBuf *bufs[] = {&b->d_tab, &b->d_items, &b->d_queue, &b->d_idx, &b->d_units, &b->d_grad};
    for (DevBuf *d : bufs)
        d->release();
    b->h_stage.release();
    if (b->ev0)
        cudaEventDestroy(b->ev0);
    if (b->ev1)
        cudaEventDestroy(b->ev1);
    delete b;
}
} /* extern "C" */
