/*
 * Frame pipeline: upload the recorded structure-of-arrays command buffers in
 * one copy, then run K1 flatten -> K2 stroke expansion -> K3 setup and band
 * binning -> K5 coverage/compositing on the context's stream.  Output sizes
 * are read back after each count+scan step (four small device->host reads
 * per frame); buffers only grow.
 */
#include "host.h"
#include "launch.h"

#include <algorithm>
#include <utility>
#include <cstdio>

static std::atomic<uint64_t> g_launches{0};
void                         gb_count_launch(uint64_t n) { g_launches += n; }
extern "C" uint64_t          vkvg_gb300_kernel_launches(void) { return g_launches.load(); }

void FrameHost::clear() {
    seg_info.clear();
    seg_n.clear();
    seg_aux.clear();
    seg_a.clear();
    seg_b.clear();
    seg_c.clear();
    sub_seg0.clear();
    sub_nseg.clear();
    sub_flags.clear();
    draws.clear();
    spair_draw.clear();
    spair_sub.clear();
    spair_dfirst.clear();
    sdraw_id.clear();
    sdraw_pair0.clear();
    fpair_draw.clear();
    fpair_sub.clear();
    dashes.clear();
    thetas.clear();
    grads.clear();
    sources.clear();
    paths       = 0;
    any_dash    = false;
    dash_shared = false;
    dash_sub_hi = 0;
}

std::atomic<int>      gb_form_override{-1};
std::atomic<uint32_t> gb_fail_alloc{0};
std::atomic<uint32_t> gb_wait_limit{0};

/* true when a test armed an allocation failure and this growth is the one */
static bool injected_alloc_failure() {
    uint32_t v = gb_fail_alloc.load();
    while (v) {
        if (gb_fail_alloc.compare_exchange_weak(v, v - 1))
            return v == 1;
    }
    return false;
}
bool gb_inject_alloc_fail() { return injected_alloc_failure(); }

bool DevBuf::grow(size_t bytes) {
    if (bytes <= cap)
        return true;
    if (injected_alloc_failure())
        return false;
    size_t nc = std::max(bytes + bytes / 4, (size_t)4096);
    if (p)
        cudaFree(p);
    p   = nullptr;
    cap = 0;
    if (cudaMalloc(&p, nc) != cudaSuccess) {
        p = nullptr;
        return false;
    }
    cap = nc;
    return true;
}
void DevBuf::release() {
    if (p)
        cudaFree(p);
    p   = nullptr;
    cap = 0;
}
bool PinnedBuf::grow(size_t bytes) {
    if (bytes <= cap)
        return true;
    size_t nc = std::max(bytes + bytes / 4, (size_t)4096);
    if (p)
        cudaFreeHost(p);
    p   = nullptr;
    cap = 0;
    if (cudaHostAlloc(&p, nc, cudaHostAllocDefault) != cudaSuccess) {
        p = nullptr;
        return false;
    }
    cap = nc;
    return true;
}
void PinnedBuf::release() {
    if (p)
        cudaFreeHost(p);
    p   = nullptr;
    cap = 0;
}

bool Pipeline::init() {
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        return false;
    for (auto &e : evs)
        if (cudaEventCreate(&e) != cudaSuccess)
            return false;
    init_oom = !(rb.grow(512) && status.grow(512));
    return !init_oom;
}
void Pipeline::destroy() {
    if (st)
        cudaStreamSynchronize(st);
    DevBuf *bufs[] = {&in,     &seg_cnt, &seg_off,   &scratch,    &pts,         &pflag,    &sub_pt0, &sub_npts,
                      &ev_cnt, &ev_off,  &events,    &cnt_v,      &cnt_i,       &off_v,    &off_i,   &verts,
                      &inds,   &ev_ret,  &fe_cnt,    &fe_off,     &edges,       &edge_draw, &sdraw_tri0,
                      &sdraw_vbase, &tri_a, &tri_b, &tri_draw, &cells,   &cursor,   &recs,    &status, &dbox, &apos, &alist, &dseglen, &dseg, &dfin, &tri_idx, &gsrc, &dbg, &surf_tab};
    for (DevBuf *b : bufs)
        b->release();
    staging.release();
    surf_stage.release();
    rb.release();
    for (auto &e : evs)
        if (e)
            cudaEventDestroy(e);
    if (st)
        cudaStreamDestroy(st);
    st = nullptr;
}

template <class T> static size_t put(uint8_t *base, size_t &o, const std::vector<T> &v) {
    o           = (o + 255) & ~(size_t)255;
    size_t here = o;
    if (!v.empty() && base)
        memcpy(base + o, v.data(), v.size() * sizeof(T));
    o += v.size() * sizeof(T) + sizeof(T); /* one spare element for sentinels */
    return here;
}

cudaError_t Pipeline::upload(const FrameHost &f) {
    size_t o = 0;
    /* sizing pass, then copy into pinned staging */
    for (int pass = 0; pass < 2; pass++) {
        uint8_t *b = pass ? (uint8_t *)staging.p : nullptr;
        o          = 0;
        o_seg_info = put(b, o, f.seg_info);
        o_seg_a    = put(b, o, f.seg_a);
        o_seg_b    = put(b, o, f.seg_b);
        o_seg_c    = put(b, o, f.seg_c);
        o_seg_n    = put(b, o, f.seg_n);
        o_seg_aux  = put(b, o, f.seg_aux);
        o_sub_seg0 = put(b, o, f.sub_seg0);
        o_sub_nseg = put(b, o, f.sub_nseg);
        o_sub_flags = put(b, o, f.sub_flags);
        o_draws    = put(b, o, f.draws);
        o_spd      = put(b, o, f.spair_draw);
        o_sps      = put(b, o, f.spair_sub);
        o_spf      = put(b, o, f.spair_dfirst);
        o_sdid     = put(b, o, f.sdraw_id);
        o_sdp0     = put(b, o, f.sdraw_pair0);
        o_fpd      = put(b, o, f.fpair_draw);
        o_fps      = put(b, o, f.fpair_sub);
        o_dashes   = put(b, o, f.dashes);
        o_thetas   = put(b, o, f.thetas);
        o_grads    = put(b, o, f.grads);
        if (pass == 0) {
            if (!staging.grow(o) || !in.grow(o))
                return cudaErrorMemoryAllocation;
        }
    }
    nseg   = (uint32_t)f.seg_info.size();
    nsub   = (uint32_t)f.sub_seg0.size();
    ndraw  = (uint32_t)f.draws.size();
    nspair = (uint32_t)f.spair_draw.size();
    nsdraw = (uint32_t)f.sdraw_id.size();
    nfpair = (uint32_t)f.fpair_draw.size();
    upload_bytes  = o;
    cudaError_t e = cudaMemcpyAsync(in.p, staging.p, o, cudaMemcpyHostToDevice, st);
    uploaded      = e == cudaSuccess;
    return e;
}

#define CK(x)                                                                                                          \
    do {                                                                                                               \
        cudaError_t _e = (x);                                                                                          \
        if (_e != cudaSuccess)                                                                                         \
            return _e;                                                                                                 \
    } while (0)

static cudaError_t readback_u32(Pipeline &pl, const uint32_t *dptr, uint32_t *out, int n) {
    CK(cudaMemcpyAsync(pl.rb.p, dptr, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, pl.st));
    CK(cudaStreamSynchronize(pl.st));
    memcpy(out, pl.rb.p, sizeof(uint32_t) * n);
    return cudaSuccess;
}
/* the current device's SM count (152 on a GB300 when the query fails) */
static int sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        n <= 0)
        return 152;
    return n;
}
static cudaError_t scan(Pipeline &pl, const uint32_t *in, uint32_t n, uint32_t *out) {
    if (!pl.scratch.grow(gb_scan_scratch_words(n) * 4 + 64))
        return cudaErrorMemoryAllocation;
    gb_count_launch(n ? 3 : 0);
    return gb_exclusive_scan(pl.st, in, n, out, pl.scratch.as<uint32_t>());
}
#define GROW(buf, bytes)                                                                                               \
    do {                                                                                                               \
        if (!(buf).grow(bytes))                                                                                        \
            return cudaErrorMemoryAllocation;                                                                          \
    } while (0)

/* flattening, stroke expansion, primitive set-up and binning of the uploaded
   frame into the cells of its surface table (ncells cells in all).  With
   sized, the sizes of a previous run of the same frame are reused and nothing
   is read back, so the sequence can be captured in a CUDA graph. */
cudaError_t Pipeline::geometry(const FrameHost &f, const gb_surf *surfs, uint32_t nsurf, uint64_t ncells,
                               uint64_t every_cells, bool wide, uint32_t S, bool timing, bool sized) {
    const uint8_t *I        = (const uint8_t *)in.p;
    auto           U        = [&](size_t o) { return (const uint32_t *)(I + o); };
    const uint32_t *seg_inf = U(o_seg_info);
    const float4   *sa = (const float4 *)(I + o_seg_a), *sb = (const float4 *)(I + o_seg_b),
                 *sc = (const float4 *)(I + o_seg_c);
    const gb_draw *draws = (const gb_draw *)(I + o_draws);
    const float   *dsh   = (const float *)(I + o_dashes);
    const float   *th    = (const float *)(I + o_thetas);
    uint32_t       hv[4];
    /* cell indices, their scans and the active-cell lists are 32-bit */
    if (ncells + every_cells + 2 >= (1ull << 32))
        return cudaErrorMemoryAllocation;

    CK(cudaMemsetAsync(status.p, 0, 16, st));
    if (timing)
        CK(cudaEventRecord(evs[0], st));

    /* ---------------- K1 flatten */
    GROW(seg_cnt, (size_t)(nseg + 1) * 4);
    GROW(seg_off, (size_t)(nseg + 1) * 4);
    CK(gb_launch_flatten_count(st, nseg, seg_inf, sa, sb, sc, U(o_seg_n), U(o_seg_aux), th, seg_cnt.as<uint32_t>(),
                               status.as<uint32_t>()));
    gb_count_launch(nseg ? 1 : 0);
    CK(scan(*this, seg_cnt.as<uint32_t>(), nseg, seg_off.as<uint32_t>()));
    if (!sized) {
        CK(readback_u32(*this, seg_off.as<uint32_t>() + nseg, hv, 1));
        npts = hv[0];
    }
    GROW(pts, (size_t)(npts + 1) * 8);
    GROW(pflag, (size_t)(npts + 1));
    GROW(sub_pt0, (size_t)(nsub + 1) * 4);
    GROW(sub_npts, (size_t)(nsub + 1) * 4);
    CK(gb_launch_flatten_emit(st, nseg, seg_inf, sa, sb, sc, U(o_seg_n), U(o_seg_aux), th, seg_off.as<uint32_t>(),
                              pts.as<float2>(), pflag.as<uint8_t>()));
    CK(gb_launch_subpath_ranges(st, nsub, U(o_sub_seg0), U(o_sub_nseg), seg_off.as<uint32_t>(),
                                sub_pt0.as<uint32_t>(), sub_npts.as<uint32_t>()));
    gb_count_launch((nseg ? 1 : 0) + (nsub ? 1 : 0));
    if (timing)
        CK(cudaEventRecord(evs[1], st));

    /* ---------------- K2 stroke expansion; fill edge counts alongside */
    GROW(ev_cnt, (size_t)(nspair + 1) * 4);
    GROW(ev_off, (size_t)(nspair + 1) * 4);
    GROW(fe_cnt, (size_t)(nfpair + 1) * 4);
    GROW(fe_off, (size_t)(nfpair + 1) * 4);
    /* dashed pairs: parallel walk unless a subpath is shared by two dashed pairs */
    const bool fast_dash = f.any_dash && !f.dash_shared;
    CK(gb_launch_stroke_pair_events(st, nspair, U(o_spd), U(o_sps), draws, sub_pt0.as<uint32_t>(),
                                    sub_npts.as<uint32_t>(), U(o_sub_flags), pts.as<float2>(), pflag.as<uint8_t>(),
                                    dsh, ev_cnt.as<uint32_t>(), fast_dash ? 0 : 1));
    if (fast_dash) {
        GROW(dseglen, (size_t)(npts + 1) * 4);
        GROW(dseg, (size_t)(npts + 1) * 16);
        GROW(dfin, (size_t)(nspair + 1) * 16);
        CK(gb_launch_dash_count(st, nspair, U(o_spd), U(o_sps), draws, sub_pt0.as<uint32_t>(), sub_npts.as<uint32_t>(),
                                U(o_sub_flags), pts.as<float2>(), dsh, dseglen.as<float>(), dseg.as<uint4>(),
                                dfin.as<uint4>(), ev_cnt.as<uint32_t>()));
        gb_count_launch(2);
    }
    CK(gb_launch_fill_pair_edges(st, nfpair, U(o_fps), sub_npts.as<uint32_t>(), fe_cnt.as<uint32_t>()));
    gb_count_launch((nspair ? 1 : 0) + (nfpair ? 1 : 0));
    CK(scan(*this, ev_cnt.as<uint32_t>(), nspair, ev_off.as<uint32_t>()));
    CK(scan(*this, fe_cnt.as<uint32_t>(), nfpair, fe_off.as<uint32_t>()));
    if (!sized) {
        CK(cudaMemcpyAsync(rb.p, ev_off.as<uint32_t>() + nspair, 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync((uint8_t *)rb.p + 4, fe_off.as<uint32_t>() + nfpair, 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        memcpy(hv, rb.p, 8);
        nev    = hv[0];
        nedges = hv[1];
    }
    GROW(events, (size_t)(f.any_dash ? nev + 1 : 1) * sizeof(gb_event));
    if (fast_dash) {
        CK(gb_launch_dash_emit(st, nspair, U(o_spd), U(o_sps), draws, sub_pt0.as<uint32_t>(), sub_npts.as<uint32_t>(),
                               U(o_sub_flags), pts.as<float2>(), pflag.as<uint8_t>(), dsh, dseg.as<uint4>(),
                               dfin.as<uint4>(), ev_off.as<uint32_t>(), events.as<gb_event>()));
        gb_count_launch(1);
    } else if (f.any_dash) {
        CK(gb_launch_stroke_dash_events(st, nspair, U(o_spd), U(o_sps), draws, sub_pt0.as<uint32_t>(),
                                        sub_npts.as<uint32_t>(), U(o_sub_flags), pts.as<float2>(),
                                        pflag.as<uint8_t>(), dsh, ev_off.as<uint32_t>(), events.as<gb_event>()));
        gb_count_launch(1);
    }
    GROW(cnt_v, (size_t)(nev + 1) * 4);
    GROW(cnt_i, (size_t)(nev + 1) * 4);
    GROW(off_v, (size_t)(nev + 1) * 4);
    GROW(off_i, (size_t)(nev + 1) * 4);
    CK(gb_launch_stroke_event_count(st, nev, nspair, ev_off.as<uint32_t>(), U(o_spd), U(o_sps), draws,
                                    sub_pt0.as<uint32_t>(), sub_npts.as<uint32_t>(), U(o_sub_flags), pts.as<float2>(),
                                    pflag.as<uint8_t>(), events.as<gb_event>(), cnt_v.as<uint32_t>(),
                                    cnt_i.as<uint32_t>()));
    gb_count_launch(nev ? 1 : 0);
    CK(scan(*this, cnt_v.as<uint32_t>(), nev, off_v.as<uint32_t>()));
    CK(scan(*this, cnt_i.as<uint32_t>(), nev, off_i.as<uint32_t>()));
    if (!sized) {
        CK(cudaMemcpyAsync(rb.p, off_v.as<uint32_t>() + nev, 4, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync((uint8_t *)rb.p + 4, off_i.as<uint32_t>() + nev, 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        memcpy(hv, rb.p, 8);
        nverts = hv[0];
        ninds  = hv[1];
        ntris  = ninds / 3;
    }
    GROW(verts, (size_t)(nverts + 1) * 8);
    GROW(inds, (size_t)(ninds + 1) * 4);
    GROW(ev_ret, (size_t)(nev + 1));
    CK(gb_launch_stroke_event_emit(st, nev, nspair, ev_off.as<uint32_t>(), U(o_spd), U(o_sps), draws,
                                   sub_pt0.as<uint32_t>(), sub_npts.as<uint32_t>(), U(o_sub_flags), pts.as<float2>(),
                                   pflag.as<uint8_t>(), events.as<gb_event>(), off_v.as<uint32_t>(),
                                   off_i.as<uint32_t>(), U(o_spf), verts.as<float2>(), inds.as<uint32_t>(),
                                   ev_ret.as<uint8_t>()));
    CK(gb_launch_stroke_close_patch(st, nsdraw, U(o_sdp0), U(o_sps), draws, U(o_spd), sub_npts.as<uint32_t>(),
                                    U(o_sub_flags), ev_off.as<uint32_t>(), off_v.as<uint32_t>(), off_i.as<uint32_t>(),
                                    ev_ret.as<uint8_t>(), inds.as<uint32_t>()));
    GROW(sdraw_tri0, (size_t)(nsdraw + 1) * 4);
    GROW(sdraw_vbase, (size_t)(nsdraw + 1) * 4);
    if (nsdraw)
        CK(gb_launch_stroke_draw_bases(st, nsdraw, U(o_sdp0), ev_off.as<uint32_t>(), off_v.as<uint32_t>(),
                                       off_i.as<uint32_t>(), sdraw_tri0.as<uint32_t>(), sdraw_vbase.as<uint32_t>()));
    gb_count_launch((nev ? 1 : 0) + (nsdraw ? 2 : 0));
    if (timing)
        CK(cudaEventRecord(evs[2], st));

    /* ---------------- K3 primitive setup + binning */
    /* edges: fill edges, then three slots per stroke triangle */
    const uint32_t nedge_all = nedges + 3 * ntris;
    GROW(edges, (size_t)(nedge_all + 1) * 16);
    GROW(edge_draw, (size_t)(nedge_all + 1) * 4);
    GROW(tri_a, (size_t)(ntris + 1) * 16);
    GROW(tri_b, (size_t)(ntris + 1) * 16);
    GROW(tri_draw, (size_t)(ntris + 1) * 4);
    GROW(tri_idx, (size_t)(ntris + 1) * 16);
    CK(gb_launch_fill_edges(st, nedges, nfpair, fe_off.as<uint32_t>(), U(o_fpd), U(o_fps), draws,
                            sub_pt0.as<uint32_t>(), sub_npts.as<uint32_t>(), pts.as<float2>(), surfs, edges.as<int4>(),
                            edge_draw.as<uint32_t>()));
    CK(gb_launch_stroke_tris(st, ntris, nsdraw, sdraw_tri0.as<uint32_t>(), U(o_sdid), sdraw_vbase.as<uint32_t>(),
                             draws, verts.as<float2>(), inds.as<uint32_t>(), surfs, tri_a.as<int4>(), tri_b.as<int4>(),
                             tri_draw.as<uint32_t>(), tri_idx.as<uint4>(), edges.as<int4>() + nedges,
                             edge_draw.as<uint32_t>() + nedges));
    gb_count_launch((nedges ? 1 : 0) + (ntris ? 2 : 0));
    /* cells: the counts; cursor: one zero, then their exclusive scan, which
       the scatter pass advances in place, so that afterwards cursor[c] is
       the first record of cell c (the scatter leaves slot c + 1 at the end
       of cell c); the two buffers then swap names */
    GROW(cells, (ncells + 2) * 4);
    GROW(cursor, (ncells + 2) * 4);
    CK(cudaMemsetAsync(cells.p, 0, (ncells + 1) * 4, st));
    CK(cudaMemsetAsync(cursor.p, 0, 4, st));
    /* per draw: (min x, -max x) from 0x7F7F7F7F, then its edge count from 0 */
    uint32_t *dcnt = nullptr;
    if (wide) {
        GROW(dbox, (size_t)(ndraw + 1) * 12);
        dcnt = (uint32_t *)(dbox.as<int2>() + ndraw + 1);
        CK(cudaMemsetAsync(dbox.p, 0x7F, (size_t)(ndraw + 1) * 8, st));
        CK(cudaMemsetAsync(dcnt, 0, (size_t)(ndraw + 1) * 4, st));
    }
    /* status bytes 256-511: the record total in 64 bits, as 32 partial
       sums; a one-surface frame's edge-weighted mean draw width (status
       words 4..7) and heaviest cell (word 8) pick the raster form */
    unsigned long long *total64 = (unsigned long long *)(status.as<uint8_t>() + 256);
    const bool          stats   = stats_w && !sized;
    if (!sized)
        CK(cudaMemsetAsync(total64, 0, 256, st));
    if (stats)
        CK(cudaMemsetAsync(status.as<uint32_t>() + 4, 0, 20, st));
    CK(gb_launch_bin(st, 0, nedge_all, edges.as<int4>(), edge_draw.as<uint32_t>(), draws, surfs, S,
                     cells.as<uint32_t>(), nullptr, 0u, wide ? dbox.as<int2>() : nullptr, dcnt,
                     sized ? nullptr : total64));
    gb_count_launch(nedge_all ? 1 : 0);
    if (stats && wide) {
        CK(gb_launch_draw_width_stats(st, ndraw, draws, dbox.as<int2>(), dcnt, stats_w,
                                      (unsigned long long *)(status.as<uint32_t>() + 4)));
        gb_count_launch(ndraw ? 1 : 0);
    }
    /* the every-band draws' marks, then the cells' tile sums (an active cell
       holds a record unit or belongs to an every-band draw) */
    GROW(scratch, gb_cells_scratch_words(ncells) * 4 + 64);
    CK(gb_launch_cell_flags(st, ndraw, draws, surfs, cells.as<uint32_t>()));
    CK(gb_launch_cells_reduce(st, ncells, cells.as<uint32_t>(), scratch.as<uint32_t>(),
                              stats ? status.as<uint32_t>() + 8 : nullptr));
    gb_count_launch((ndraw ? 1 : 0) + (ncells ? 1 : 0));
    if (!sized) {
        CK(cudaMemcpyAsync((uint8_t *)rb.p + 256, total64, 256, cudaMemcpyDeviceToHost, st));
        if (stats)
            CK(cudaMemcpyAsync((uint8_t *)rb.p + 8, status.as<uint32_t>() + 4, 20, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        uint64_t ws[2] = {0, 0};
        uint32_t mxc   = 0;
        memcpy(ws, (uint8_t *)rb.p + 8, 16);
        memcpy(&mxc, (uint8_t *)rb.p + 24, 4);
        uint64_t tot = 0, part[32];
        memcpy(part, (uint8_t *)rb.p + 256, 256);
        for (uint64_t v : part)
            tot += v;
        /* record offsets are 32-bit and a cell's count keeps bit 31 for its
           every-band mark */
        if (tot >= (uint64_t)GB_CELL_EVERY)
            return cudaErrorMemoryAllocation;
        nunits   = (uint32_t)tot;
        max_cell = stats ? mxc : 0xFFFFFFFFu;
        /* narrow tiles (256 pixels; 128 when every cell fits 128 units) when
           every cell fits the narrow form's staging buffer (480 units)
           (a heavy cell is one CTA's serial work: the wide form's 512 threads
           finish it sooner) and the draws that carry the edges are small next
           to a wide tile, or the surface is no wider than a narrow one */
        const bool small = !wide || (ws[1] && ws[0] <= 384u * ws[1]);
        narrow           = !(stats && small) ? 0 : mxc <= 128u ? 5 : mxc <= 480u ? 1 : 0;
        /* candidates for the row form: draws that span most of a tile (mean
           width over 640 pixels, weighted by edges), or a surface whose
           1024-pixel tiles give fewer CTAs than SMs (the row form's half
           bands double them); the raster launch then checks how thinly
           their crossings spread */
        const uint64_t tile_ctas = (uint64_t)nbands * ((stats_w + 1023u) / 1024u);
        row_draws = stats && wide && ws[1] && (ws[0] > 640u * ws[1] || tile_ctas < (uint64_t)sm_count());
        mean_width = ws[1] ? (double)ws[0] / (double)ws[1] : 0.0;
    }
    /* the cells' record offsets and the raster's per-band draw lists in one
       more pass over the counts, then the records */
    GROW(recs, (size_t)(nunits + 1) * 16);
    GROW(apos, (ncells + 1) * 4);
    GROW(alist, (size_t)(nunits + every_cells + 1) * 4);
    CK(gb_launch_cells_lists(st, ncells, cells.as<uint32_t>(), scratch.as<uint32_t>(), cursor.as<uint32_t>() + 1,
                             alist.as<uint32_t>(), apos.as<uint32_t>(), surfs, nsurf));
    gb_count_launch(ncells ? 2 : 0);
    CK(gb_launch_bin(st, 1, nedge_all, edges.as<int4>(), edge_draw.as<uint32_t>(), draws, surfs, S,
                     cursor.as<uint32_t>() + 1, recs.as<int4>(), nunits, nullptr, nullptr, nullptr));
    gb_count_launch(nedge_all ? 1 : 0);
    std::swap(cells, cursor); /* cells <- the offsets (kept for the raster); cursor is free */
    if (timing)
        CK(cudaEventRecord(evs[3], st));
    return cudaSuccess;
}

/* The row form spends per crossing in a lane's run of 32 samples (a walk
   over the run's flagged positions), the register tiles per sample: the
   row form wins (the curve-heavy scene) when a draw's records per band,
   spread over its width in runs, stay near one per run, and loses two- to
   fourfold on denser geometry (the uneven batch's surfaces: hundreds of
   segments in one bounding box).  Records per active cell over the mean
   draw width in runs below 3 picks it. */
bool Pipeline::sparse_crossings(uint64_t ncells_run) {
    uint32_t active = 0;
    if (readback_u32(*this, apos.as<uint32_t>() + ncells_run, &active, 1) != cudaSuccess || !active)
        return false;
    const double runs = mean_width / 32.0;
    return runs > 0.0 && (double)nunits / (double)active < 3.0 * runs;
}

cudaError_t Pipeline::run(const FrameHost &f, _vkvg_surface_t *surf, bool timing) {
    const uint8_t  *I     = (const uint8_t *)in.p;
    const gb_draw  *draws = (const gb_draw *)(I + o_draws);
    const uint32_t  W = surf->width, H = surf->height, S = surf->samples;
    nbands                = surf->nbands;
    /* the frame's surface table: its one target */
    gb_surf sd;
    memset(&sd, 0, sizeof(sd));
    sd.W       = W;
    sd.H       = H;
    sd.nrows   = surf->nrows;
    sd.nbands  = nbands;
    sd.wpad    = surf->wpad;
    sd.ndraws  = ndraw;
    sd.samples = surf->d_samples;
    sd.rgba    = surf->d_rgba;
    if (!surf_stage.grow(sizeof(gb_surf)))
        return cudaErrorMemoryAllocation;
    GROW(surf_tab, sizeof(gb_surf));
    memcpy(surf_stage.p, &sd, sizeof(sd));
    CK(cudaMemcpyAsync(surf_tab.p, surf_stage.p, sizeof(sd), cudaMemcpyHostToDevice, st));
    uint64_t every = 0;
    for (const gb_draw &d : f.draws)
        every += d.kind > GB_DRAW_STROKE ? nbands : 0u;
    stats_w = W;
    CK(geometry(f, surf_tab.as<gb_surf>(), 1u, (uint64_t)nbands * ndraw, every, W > gb_raster_tile_width(4), S, timing,
                false));
    stats_w = 0;

    /* ---------------- K5 coverage + compositing */
    gb_raster_args A;
    memset(&A, 0, sizeof(A));
    A.W = W;
    A.H = H;
    A.S = S;
    A.Wpad       = surf->wpad;
    A.nrows      = surf->nrows;
    A.nbands     = nbands;
    A.ndraws     = ndraw;
    A.draw_first = 0;
    A.init_mode  = 0;
    /* clip planes: follow which of them may hold anything but their reset
       value through the frame's draws; a frame that touches a nontrivial
       plane, or has any clip draw, runs the clipping variant */
    bool     clip_use = surf->clip_active, act = surf->clip_active;
    uint8_t  snz      = surf->save_nz;
    uint32_t nimg     = (uint32_t)surf->clip_images.size();
    for (const gb_draw &d : f.draws) {
        switch (d.kind) {
        case GB_DRAW_CLIP_EO:
        case GB_DRAW_CLIP_NZ: act = true; clip_use = true; break;
        case GB_DRAW_CLEAR:
            clip_use |= act || snz;
            act = false;
            snz = 0;
            break;
        case GB_DRAW_CLIP_RESET:
            clip_use = true;
            act      = false;
            snz      = 0;
            break;
        case GB_DRAW_CLIP_SAVE:
            clip_use = true;
            snz      = (uint8_t)(act ? snz | (1u << d.src) : snz & ~(1u << d.src));
            break;
        case GB_DRAW_CLIP_RESTORE:
            clip_use = true;
            act      = (snz >> d.src) & 1u;
            break;
        case GB_DRAW_CLIP_STORE:
            clip_use = true;
            if (d.src >= surf->clip_images.size())
                surf->clip_images.resize(d.src + 1, 0);
            surf->clip_images[d.src] = (uint8_t)(snz | (act ? 0x80u : 0u));
            nimg                     = std::max(nimg, d.src + 1);
            break;
        case GB_DRAW_CLIP_LOAD: {
            clip_use          = true;
            const uint8_t img = d.src < surf->clip_images.size() ? surf->clip_images[d.src] : 0;
            act               = (img & 0x80u) != 0;
            snz               = (uint8_t)(img & 0x3Fu);
            break;
        }
        default: break;
        }
    }
    const bool reset0 = ndraw > 0 && f.draws[0].kind == GB_DRAW_CLEAR && surf->save_nz;
    if (clip_use) {
        /* planes keep their contents when the store grows */
        const size_t need = (GB_CLIP_SAVE_PLANES + (size_t)GB_CLIP_IMAGE_PLANES * nimg) * surf->plane_words * 4;
        DevBuf      &cp   = surf->clip_planes;
        if (need > cp.cap) {
            void *np = nullptr;
            if (cudaMalloc(&np, need) != cudaSuccess)
                return cudaErrorMemoryAllocation;
            CK(cudaMemsetAsync(np, 0, need, st));
            if (cp.p)
                CK(cudaMemcpyAsync(np, cp.p, cp.cap, cudaMemcpyDeviceToDevice, st));
            CK(cudaStreamSynchronize(st));
            cp.release();
            cp.p   = np;
            cp.cap = need;
        }
    }
    gb_clip_args CA;
    CA.clip        = surf->d_clip;
    CA.clip_planes = surf->clip_planes.as<uint32_t>();
    CA.plane_words = surf->plane_words;
    CA.clip_wpr    = surf->clip_wpr;
    CA.clip_load   = surf->clip_active ? 1u : 0u;
    if (ndraw > 0) {
        const gb_draw &d0 = f.draws[0];
        if (d0.kind == GB_DRAW_CLEAR) {
            A.init_mode  = 1;
            A.init_color = 0;
            A.draw_first = 1;
            CA.clip_load = reset0 ? 2u : 0u; /* a clear also resets the stencil */
        } else if (d0.kind == GB_DRAW_PAINT && (d0.op == GB_OP_OVER || d0.op == GB_OP_SOURCE) &&
                   (d0.src >> 24) == 255u && d0.gsrc == 0 && !surf->clip_active) {
            A.init_mode  = 1;
            A.init_color = d0.src;
            A.draw_first = 1;
        }
    }
    A.draws    = draws;
    A.cell_off = cells.as<uint32_t>();
    A.apos     = apos.as<uint32_t>();
    A.alist    = alist.as<uint32_t>();
    A.dbox     = dbox.as<int2>();
    A.cell0    = 0;
    A.recs     = recs.as<int4>();
    A.nunits   = nunits;
    A.status   = status.as<uint32_t>();
    A.samples  = surf->d_samples;
    A.rgba     = surf->d_rgba;
    /* gradient source images: one per distinct (gradient, opacity) of the frame */
    const uint32_t ngrad = (uint32_t)f.grads.size();
    if (ngrad) {
        GROW(gsrc, (size_t)ngrad * W * H * 4);
        const gb_grad *g = (const gb_grad *)(I + o_grads);
        for (uint32_t i = 0; i < ngrad; i++)
            CK(gb_launch_gradient_fill(st, W, H, g + i, gsrc.as<uint32_t>() + (size_t)i * W * H));
        gb_count_launch(ngrad);
        A.gsrc = gsrc.as<uint32_t>();
    }
    /* the band rows of a frame's only source image are staged by the row form */
    A.gc_src     = ngrad == 1 && S == 4 ? 1u : 0u;
    A.wait_limit = gb_wait_limit.load() ? gb_wait_limit.load() : WAIT_LIMIT_POLLS;
    int form     = gb_form_override.load();
    if (clip_use)
        form = 0; /* only the register tile carries the clip planes */
    else if (form < 0 || form > 5)
        form = narrow ? narrow : row_draws && sparse_crossings((uint64_t)nbands * ndraw) ? 3 : 0;
    if (form == 3 && max_cell >= 32768u)
        form = 4; /* 16-bit counters would not hold a cell's crossings: whole bands */
    form_run  = form;
    form_half = form == 3 ? 1 : 0;
    /* the small-draw forms read their smallest cells from L2 instead of
       staging them (a bulk copy and a wait per draw): the tiny form cells
       under 64 record units (glyph raster 11.23 -> 10.87 ms, no change
       above 64), the micro form cells under 16 (10.31 ms at 64, 10.23 ms
       staging every cell, 10.16 ms at 16) */
    A.stage_min = form == 2 ? 64u : form == 5 ? 16u : 0u;
    if (form == 3 || form == 4)
        CK(gb_launch_raster_rows(st, &A, ngrad > 0, form_half));
    else
        CK(gb_launch_raster(st, &A, &CA, ngrad > 0, clip_use, form));
    surf->clip_active = act;
    surf->save_nz     = snz;
    gb_count_launch(1);
    if (timing)
        CK(cudaEventRecord(evs[4], st));
    CK(cudaMemcpyAsync(rb.p, status.p, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    dev_status = *(uint32_t *)rb.p;
    if (timing) {
        for (int i = 0; i < 4; i++)
            cudaEventElapsedTime(&ms[i], evs[i], evs[i + 1]);
        cudaEventElapsedTime(&ms[4], evs[0], evs[4]);
    }
    return cudaGetLastError();
}

cudaError_t Pipeline::flatten_only() {
    const uint8_t  *I = (const uint8_t *)in.p;
    auto            U = [&](size_t o) { return (const uint32_t *)(I + o); };
    const float4   *sa = (const float4 *)(I + o_seg_a), *sb = (const float4 *)(I + o_seg_b),
                 *sc = (const float4 *)(I + o_seg_c);
    const float    *th = (const float *)(I + o_thetas);
    uint32_t        hv[1];
    CK(cudaMemsetAsync(status.p, 0, 16, st));
    GROW(seg_cnt, (size_t)(nseg + 1) * 4);
    GROW(seg_off, (size_t)(nseg + 1) * 4);
    CK(gb_launch_flatten_count(st, nseg, U(o_seg_info), sa, sb, sc, U(o_seg_n), U(o_seg_aux), th,
                               seg_cnt.as<uint32_t>(), status.as<uint32_t>()));
    CK(scan(*this, seg_cnt.as<uint32_t>(), nseg, seg_off.as<uint32_t>()));
    CK(readback_u32(*this, seg_off.as<uint32_t>() + nseg, hv, 1));
    npts = hv[0];
    GROW(pts, (size_t)(npts + 1) * 8);
    GROW(pflag, (size_t)(npts + 1));
    GROW(sub_pt0, (size_t)(nsub + 1) * 4);
    GROW(sub_npts, (size_t)(nsub + 1) * 4);
    CK(gb_launch_flatten_emit(st, nseg, U(o_seg_info), sa, sb, sc, U(o_seg_n), U(o_seg_aux), th,
                              seg_off.as<uint32_t>(), pts.as<float2>(), pflag.as<uint8_t>()));
    CK(gb_launch_subpath_ranges(st, nsub, U(o_sub_seg0), U(o_sub_nseg), seg_off.as<uint32_t>(),
                                sub_pt0.as<uint32_t>(), sub_npts.as<uint32_t>()));
    gb_count_launch((nseg ? 2 : 0) + (nsub ? 1 : 0));
    return cudaStreamSynchronize(st);
}

vkvg_status_t gb_run_frame(Pipeline &pl, const FrameHost &f, VkvgSurface surf, bool do_upload, bool timing) {
    if (f.empty())
        return VKVG_STATUS_SUCCESS;
    std::lock_guard<std::mutex> lk(surf->mtx);
    if (do_upload || !pl.uploaded) {
        const cudaError_t ue = pl.upload(f);
        if (ue == cudaErrorMemoryAllocation)
            return VKVG_STATUS_NO_MEMORY;
        if (ue != cudaSuccess)
            return VKVG_STATUS_DEVICE_ERROR;
    }
    cudaError_t e = pl.run(f, surf, timing);
    if (e == cudaErrorMemoryAllocation)
        return VKVG_STATUS_NO_MEMORY;
    if (e != cudaSuccess) {
        fprintf(stderr, "vkvg_gb300: CUDA error %s\n", cudaGetErrorString(e));
        return VKVG_STATUS_DEVICE_ERROR;
    }
    if (pl.dev_status & GB_ERR_RASTER_WAIT) {
        fprintf(stderr, "vkvg_gb300: raster staging wait exceeded its limit\n");
        return VKVG_STATUS_DEVICE_ERROR;
    }
    if (pl.dev_status & GB_ERR_OVERFLOW) {
        fprintf(stderr, "vkvg_gb300: a raster cell's records lay beyond the binned total\n");
        return VKVG_STATUS_DEVICE_ERROR;
    }
    if (pl.dev_status & GB_ERR_CURVE_LIMIT) {
        fprintf(stderr, "vkvg_gb300: a curve exceeded the subdivision work cap and was cut short\n");
        return VKVG_STATUS_DEVICE_ERROR;
    }
    return VKVG_STATUS_SUCCESS;
}
