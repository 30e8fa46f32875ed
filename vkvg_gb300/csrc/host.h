/*
 * Host-side structures of the GB300 vkvg library: device, surface, context,
 * the per-context path recorder and the kernel pipeline.
 */
#ifndef VKVG_GB300_HOST_H
#define VKVG_GB300_HOST_H

#include "../../include/vkvg.h"
#include "../../include/vkvg_gb300.h"
#include "gb_types.h"

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <stdint.h>
#include <string.h>
#include <utility>
#include <vector>

struct f4 {
    float x, y, z, w;
};

/* one frame of recorded work, as host structure-of-arrays */
/* a counted reference to a surface (a frame's surface sources stay alive
   until the frame has run) */
struct SurfRef {
    VkvgSurface s = nullptr;
    SurfRef()     = default;
    explicit SurfRef(VkvgSurface x) : s(x) { vkvg_surface_reference(s); }
    SurfRef(const SurfRef &o) : s(o.s) {
        if (s)
            vkvg_surface_reference(s);
    }
    SurfRef &operator=(const SurfRef &o) {
        if (this != &o) {
            SurfRef t(o);
            std::swap(s, t.s);
        }
        return *this;
    }
    ~SurfRef() {
        if (s)
            vkvg_surface_destroy(s);
    }
};

struct FrameHost {
    std::vector<uint32_t> seg_info, seg_n, seg_aux;
    std::vector<f4>       seg_a, seg_b, seg_c;
    std::vector<uint32_t> sub_seg0, sub_nseg, sub_flags;
    std::vector<gb_draw>  draws;
    std::vector<uint32_t> spair_draw, spair_sub, spair_dfirst;
    std::vector<uint32_t> sdraw_id, sdraw_pair0; /* per stroke draw (+ sentinel in pair0) */
    std::vector<uint32_t> fpair_draw, fpair_sub;
    std::vector<float>    dashes, thetas;
    std::vector<gb_grad>  grads;   /* pattern source images of the frame */
    std::vector<SurfRef>  sources; /* surfaces that surface sources read */
    uint32_t              paths = 0; /* fill + stroke draws */
    bool                  any_dash = false;
    bool                  dash_shared = false; /* a subpath belongs to two dashed stroke pairs */
    uint32_t              dash_sub_hi = 0;     /* end of the subpath ranges dashed strokes used */
    void                  clear();
    bool                  empty() const { return draws.empty(); }
};

/* grow-only device buffer */
struct DevBuf {
    void  *p   = nullptr;
    size_t cap = 0;
    bool   grow(size_t bytes);
    void   release();
    template <class T> T *as() const { return (T *)p; }
};
struct PinnedBuf {
    void  *p   = nullptr;
    size_t cap = 0;
    bool   grow(size_t bytes);
    void   release();
};

struct Pipeline {
    cudaStream_t st = nullptr;
    DevBuf       in;
    DevBuf       seg_cnt, seg_off, scratch, pts, pflag, sub_pt0, sub_npts;
    DevBuf       ev_cnt, ev_off, events, cnt_v, cnt_i, off_v, off_i, verts, inds, ev_ret;
    DevBuf       fe_cnt, fe_off, edges, edge_draw;
    DevBuf       sdraw_tri0, sdraw_vbase, tri_a, tri_b, tri_draw;
    DevBuf       cells, cursor, recs, status, dbg;
    DevBuf       dbox;        /* per draw: x extent of its binned edges (min x, -max x) */
    DevBuf       apos, alist; /* the raster's per-band draw lists: cell -> list position, active cells */
    DevBuf       dseglen, dseg, dfin;
    DevBuf       tri_idx; /* oriented vertex indices of stroke triangles (edge cancellation) */
    DevBuf       gsrc;    /* gradient source images of the frame, [n][H][W] */
    DevBuf       surf_tab; /* the frame's surface table (gb_surf) */
    PinnedBuf    surf_stage; /* parallel dash walk: per-point lengths / states, per-pair final state */
    PinnedBuf    staging, rb;
    cudaEvent_t  evs[8] = {};
    /* offsets of the uploaded arrays inside `in` */
    size_t o_seg_info, o_seg_a, o_seg_b, o_seg_c, o_seg_n, o_seg_aux, o_sub_seg0, o_sub_nseg, o_sub_flags, o_draws,
        o_spd, o_sps, o_spf, o_sdid, o_sdp0, o_fpd, o_fps, o_dashes, o_thetas, o_grads;
    bool     uploaded = false;
    /* sizes of the last run */
    uint32_t nseg = 0, nsub = 0, ndraw = 0, nspair = 0, nsdraw = 0, nfpair = 0;
    uint32_t npts = 0, nev = 0, nverts = 0, ninds = 0, nedges = 0, ntris = 0, nunits = 0, nbands = 0;
    uint32_t dev_status = 0;
    uint32_t stats_w    = 0;     /* surface width of a one-surface frame: geometry measures its draws' widths */
    int      narrow     = 0; /* the register-tile form geometry picked: 0 1024-pixel, 1 256-pixel, 5 64-pixel tiles */
    int      form_run   = -1; /* the raster form the last frame ran (as vkvg_gb300_debug_set_raster_form) */
    int      form_half  = 0;  /* the row form ran in half bands with 16-bit counters */
    bool     row_draws  = false; /* the row form's candidates: draws spanning most of a 1024-pixel tile, or few tiles */
    double   mean_width = 0.0;   /* edge-weighted mean draw width of a one-surface frame, pixels */
    bool     sparse_crossings(uint64_t ncells_run); /* records per active cell thin enough for the row form */
    uint32_t max_cell   = 0xFFFFFFFFu; /* record units of the heaviest cell (one-surface frames; else unknown) */
    uint64_t launches   = 0;
    uint64_t upload_bytes = 0;
    bool     init_oom     = false; /* init failed growing a buffer */
    float    ms[5]      = {0, 0, 0, 0, 0};

    bool init();
    void destroy();
    /* upload a frame's host arrays (one copy) */
    cudaError_t upload(const FrameHost &f);
    /* run the uploaded frame on a surface */
    cudaError_t run(const FrameHost &f, struct _vkvg_surface_t *surf, bool timing);
    /* every_cells: the cells of the draws that act on every band of their
       surface (kinds after STROKE), a bound the draw lists are sized by;
       wide: a surface is wider than one raster tile (the raster then reads
       the draws' x extents); surfs: the nsurf surfaces' table on the device */
    cudaError_t geometry(const FrameHost &f, const gb_surf *surfs, uint32_t nsurf, uint64_t ncells,
                         uint64_t every_cells, bool wide, uint32_t S, bool timing, bool sized);
    /* K1 only: flatten the uploaded segments (for vkvg_path_extents) */
    cudaError_t flatten_only();
};

/* process-wide test settings (vkvg_gb300_debug_set_raster_form, _inject) */
extern std::atomic<int>      gb_form_override; /* -1 automatic */
extern std::atomic<uint32_t> gb_fail_alloc;    /* growths until one fails, 0 off */
extern std::atomic<uint32_t> gb_wait_limit;    /* row-form staging wait polls, 0 default */
/* true when an armed allocation failure falls on this allocation */
bool gb_inject_alloc_fail();

struct _vkvg_device_t {
    vkvg_status_t status;
    uint32_t      refs;
    uint32_t      samples;
    int           cuda_dev;
    bool          thread_aware;
    int           hdpi, vdpi;
    uint8_t      *d_unpremul; /* [alpha][channel] -> write_to_memory's unpremultiplied byte */
    std::mutex    mtx;
};

/* a linear gradient pattern (src/vkvg_pattern.c: vkvg_gradient_t) */
struct _vkvg_pattern_t {
    vkvg_status_t       status;
    uint32_t            refs;
    vkvg_pattern_type_t type;
    vkvg_extend_t       extend;
    vkvg_filter_t       filter;
    float               cp[8]; /* vkvg_gradient_t.cp: two vec4 */
    VkvgSurface         surf = nullptr; /* surface patterns: referenced */
    uint32_t            count;
    float               stops[GB_GRAD_STOPS];
    float               colors[GB_GRAD_STOPS * 4]; /* premultiplied */
    vkvg_matrix_t       matrix;
    bool                has_matrix;
};

struct _vkvg_surface_t {
    vkvg_status_t status;
    uint32_t      refs;
    VkvgDevice    dev;
    uint32_t      width, height, samples, wpad, nrows, nbands;
    uint32_t     *d_samples; /* [nrows][wpad] premultiplied RGBA8 */
    uint32_t     *d_rgba;    /* [height][width] resolved */
    uint32_t     *d_out;     /* [height][width] unpremultiplied, staged for write_to_memory */
    /* the stencil as bit planes, one bit per sample, [band rows][clip_wpr]
       words each: d_clip is the visibility plane; clip_planes holds the six
       save planes, then seven planes per stencil image */
    uint32_t     *d_clip;
    uint32_t      clip_wpr;               /* words per sample row */
    size_t        plane_words;            /* words per plane */
    DevBuf        clip_planes;
    bool          clip_active = false;    /* visibility may not be all ones */
    uint8_t       save_nz     = 0;        /* bit p: save plane p may be nonzero */
    std::vector<uint8_t> clip_images;     /* per image: save_nz bits, 0x80 = visibility not all ones */
    std::mutex    mtx;
};

/* reference path state of the open subpath (vkvg's points/pathes arrays,
   src/vkvg_context_internal.c:132-238, with flattened counts kept symbolic) */
struct PathState {
    uint32_t path_sub0 = 0; /* first subpath of the current path */
    bool     open      = false;
    uint32_t seg0      = 0;
    uint32_t exact     = 0; /* points of non-cubic segments */
    uint32_t ncubic    = 0; /* finite cubics: each adds >= 3 points */
    float    fx = 0, fy = 0, lx = 0, ly = 0;
    bool     closed       = false;
    bool     pending      = false; /* a curve segment is open */
    uint32_t pending_from = 0;
};

/* clip states, vkvg_clip_state_t (src/vkvg_context_internal.h:95-99) */
#define GB_CLIP_NONE  0x00u
#define GB_CLIP_CLEAR 0x01u
#define GB_CLIP_CLIP  0x02u
#define GB_CLIP_SAVED 0x06u
/* one vkvg_save level, vkvg_context_save_t (src/vkvg_context_internal.h:101-124):
   the line join is not kept (vkvg_restore sets the field it never saved) */
struct gb_saved_state {
    float              line_width, miter_limit, dash_offset, opacity;
    vkvg_line_cap_t    line_cap;
    vkvg_fill_rule_t   fill_rule;
    vkvg_operator_t    op;
    vkvg_matrix_t      mat, mat_inv;
    float              src_x, src_y;
    std::vector<float> dashes;
    uint32_t           cur_color;
    VkvgPattern        pattern; /* referenced while saved */
    uint8_t            clip_state;
};

struct _vkvg_context_t {
    vkvg_status_t status;
    uint32_t      refs;
    VkvgSurface   surf;
    VkvgDevice    dev;

    /* drawing state (vkvg _init_ctx defaults, src/vkvg_context.c:24-70) */
    float              line_width  = 1.f;
    float              miter_limit = 10.f;
    vkvg_line_cap_t    line_cap    = VKVG_LINE_CAP_BUTT;
    vkvg_line_join_t   line_join   = VKVG_LINE_JOIN_MITER;
    vkvg_fill_rule_t   fill_rule   = VKVG_FILL_RULE_NON_ZERO;
    vkvg_operator_t    op          = VKVG_OPERATOR_OVER;
    uint32_t           cur_color   = 0xff000000u;
    float              opacity     = 1.0f;
    vkvg_matrix_t      mat         = {1, 0, 0, 1, 0, 0};
    std::vector<float> dashes;
    float              dash_offset = 0;
    VkvgPattern        pattern     = nullptr; /* source pattern, null for the solid colour */
    bool               grad_on     = false;   /* the source is a pattern (gradient snapshot or surface) */
    gb_grad            grad_snap;             /* gradients: as of vkvg_set_source (opacity filled per draw) */
    /* push constants the fragment stage reads for surface sources: source.xy
       and the inverse matrix (src/vkvg_context_internal.h:74-81) */
    float              src_x = 0, src_y = 0;
    vkvg_matrix_t      mat_inv     = {1, 0, 0, 1, 0, 0};

    /* clip and save/restore (vkvg's curClipState, curSavBit, pSavedCtxs) */
    uint8_t                     clip_state = GB_CLIP_NONE;
    uint8_t                     sav_bit    = 0;
    std::vector<gb_saved_state> saved;

    PathState ps;
    FrameHost frame;
    Pipeline  pl;
    bool      debug    = false;
    bool      have_run = false;
};

struct _vkvg_gb300_frame_t {
    FrameHost frame;
    Pipeline  pl;
    uint32_t  width, height, samples;
};

/* pipeline entry used by flush and frame execution */
vkvg_status_t gb_run_frame(Pipeline &pl, const FrameHost &f, VkvgSurface surf, bool upload, bool timing);
void          gb_count_launch(uint64_t n);
/* premultiplied source word after opacity (fragment stage + UNORM8 output) */
uint32_t gb_source_word(uint32_t color, float opacity);
/* write_to_memory's unpremultiply for every (alpha, channel) pair, [a * 256 + p] */
const uint8_t *gb_unpremul_table();
int      gb_png_write(const char *path, uint32_t w, uint32_t h, const uint8_t *rgba);

#endif
