/*
 * K5, row form - per-band coverage and compositing with one warp per sample
 * row and the band's samples in shared memory.
 *
 * A CTA owns a tile of 16 sample rows (one band: 4 pixel rows at 4x MSAA) by
 * up to 1024 pixels.  Sixteen consumer warps each own one sample row; a
 * seventeenth, the producer, walks the band's draws in submission order and
 * hands them over through a ring of shared-memory slots: per draw a header
 * (kind, record range, blend constants) and, for geometry, the cell's edge
 * records brought in by one cp.async.bulk completing the slot's "full"
 * mbarrier.  A consumer warp waits for the slot, accumulates its row's
 * crossings from the staged records, arrives on the slot's "empty" mbarrier
 * (sixteen arrivals free it for the producer) and then resolves and blends
 * its row on its own: no block-wide barrier per draw, so rows with little
 * work run ahead by up to the ring's depth.
 *
 * Coverage is the same exact integer arithmetic as the register-tile form:
 * an edge crossing the row's sample y at x_c adds its direction (+1 down,
 * -1 up) to every sample with x < x_c (top-left rule), so the suffix sum at a
 * sample is its winding number (fills) or its covering-triangle count
 * (strokes).  A crossing is recorded at the last sample left of it.  Even-odd
 * fills only need the parity: each crossing toggles that sample's bit of a
 * per-row bit plane, and the coverage of lane l's run of samples
 * [32 l, 32 l + 32) is the suffix XOR of its word (five shift-XORs) flipped
 * by the parity of the runs to its right (one ballot) - the stencil INVERT of
 * _poly_fill.  Non-zero fills and strokes add the direction to a per-sample
 * counter and flag the position in the bit plane; the lane sums the counters
 * at its flagged positions, a warp suffix scan gives the winding entering
 * each run from the right, and one walk over the flagged positions (a few per
 * run) turns the piecewise-constant winding into coverage masks: non-zero
 * w != 0 (glutess' NONZERO), strokes w > k for the k-th blend pass (each
 * covering triangle blends once under pipe_OVER; the first four passes'
 * masks come out of the same walk).
 *
 * The blend touches covered samples only.  The 32 run masks are transposed
 * across the warp (a 32 x 32 bit matrix), after which lane l holds the
 * coverage of samples {32 k + l}: covered spans spread evenly over the lanes,
 * each lane walks its set bits two at a time, and the 32 lanes of one step
 * address 32 distinct banks.  The blend is vkvg's source-over on
 * premultiplied UNORM8, exact (the FMA-pipe form for solid premultiplied
 * sources, two-channel integer arithmetic otherwise, per-sample source words
 * for gradient and surface sources).  At the end the tile's samples are
 * written back and resolved ((sum + S/2) / S) with 128-bit stores.
 */
#include "launch.h"
#include "raster_common.cuh"
#include "xdiv.cuh"

#include <cuda_runtime.h>

#include <atomic>

namespace rw {
constexpr int TW  = 1024; /* tile width in pixels (samples per row) */
constexpr int HDR = 16;   /* header words per slot */
/* header words (read as four 16-byte vectors) */
enum { H_KIND, H_OP, H_SRC, H_GS, H_LO, H_UNITS, H_STAGED, H_MODE, H_K, H_C0, H_C1, H_C2, H_C3, H_INV };
constexpr uint32_t KIND_END = 0xFFFFFFFFu;
/* misc words */
enum { M_ABORT, M_IEND, M_DLO, M_DHI, M_TILES, M_DENSE, M_I0 };
} // namespace rw

/* A row-form configuration: ROWS consumer warps (sample rows per CTA, 16 or
   8: a CTA then covers a half band), the ring's depth and slot capacity,
   and 32- or 16-bit crossing counters.  16-bit counters are kept biased by
   2^15 (an empty counter holds 0x8000), two to a word, so that a word-wide
   atomic add of +-1 or +-2^16 never carries between the halves and each
   half reads back with one 16-bit load; they hold a position's net crossings
   exactly while the draw's cell has fewer than 2^15 records (the host checks
   the heaviest cell). */
template <int ROWS_, int NSLOT_, int CAP_, bool C16_> struct RWT {
    static constexpr int  ROWS    = ROWS_;
    static constexpr int  NSLOT   = NSLOT_;
    static constexpr int  CAP     = CAP_;
    static constexpr bool C16     = C16_;
    static constexpr int  TW      = rw::TW;
    static constexpr int  HDR     = rw::HDR;
    static constexpr int  THREADS = (ROWS + 1) * 32;
    static constexpr int  PROD    = ROWS;            /* the producer's warp index */
    static constexpr int  CW      = C16 ? TW / 2 : TW; /* counter words per row */
    static constexpr int  GCR     = ROWS / 4;        /* pixel rows of the CTA at 4x MSAA */
    /* shared memory, in 32-bit words */
    static constexpr int S_SMP  = 0;                    /* samples [ROWS][TW] */
    static constexpr int S_CNT  = S_SMP + ROWS * TW;    /* crossing counters [ROWS][CW] */
    static constexpr int S_OCC  = S_CNT + ROWS * CW;    /* bit planes [ROWS][TW / 32] */
    static constexpr int S_GC   = S_OCC + ROWS * 32;    /* the CTA's pixel rows of one source image (4x MSAA) */
    static constexpr int S_HDR  = S_GC + GCR * TW;      /* slot headers */
    static constexpr int S_BAR  = S_HDR + NSLOT * HDR;  /* full[NSLOT], empty[NSLOT] mbarriers (8 bytes each) */
    static constexpr int S_MISC = S_BAR + 4 * NSLOT;    /* abort flag, walk bounds */
    static constexpr int S_STG  = (S_MISC + 16 + 3) / 4 * 4;
    static constexpr int SMEM   = (S_STG + NSLOT * CAP * 4) * 4;
    static constexpr int MINB   = SMEM + 1024 <= 233472 / 3 ? 3 : SMEM + 1024 <= 233472 / 2 ? 2 : 1; /* CTAs per SM */
    static_assert(S_HDR % 4 == 0 && S_BAR % 2 == 0 && S_STG % 4 == 0, "headers and staging 16-byte aligned");
    static_assert(SMEM <= 232448, "shared memory of one CTA");
};
/* the band-sized configuration (also the batch's) and the half-band one
   that fits three CTAs per SM */
using RW16 = RWT<16, 4, 1024, false>;
using RW8  = RWT<8, 4, 256, true>;

/* the bits [a, b] of a word, a <= b <= 31 */
__device__ __forceinline__ uint32_t bit_range(uint32_t a, uint32_t b) { return ((0xFFFFFFFFu >> (31u - b)) >> a) << a; }

/* 32 x 32 bit transpose across the warp: lane l holds row l on entry
   (bit c = column c) and column l on return (bit k = row k) */
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x, uint32_t lane) {
    const uint32_t lo[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int s = 0; s < 5; s++) {
        const uint32_t j = 16u >> s;
        const uint32_t y = __shfl_xor_sync(0xFFFFFFFFu, x, j);
        x = (lane & j) ? ((x & ~lo[s]) | ((y >> j) & lo[s])) : ((x & lo[s]) | ((y & lo[s]) << j));
    }
    return x;
}

/* source word of sample column c for a pattern draw */
struct rw_src {
    const uint32_t *row; /* global row of the source image, from the tile's first column */
    const uint32_t *gc;  /* the staged copy of that row, or null */
    __device__ __forceinline__ uint32_t at(uint32_t c) const { return gc ? gc[c] : __ldg(row + c); }
};

/* blend the samples of row smp whose bits are set in t (lane l: samples
   32 k + l), vkvg's source-over per sample */
template <int M, bool G>
__device__ __forceinline__ void blend_bits(uint32_t *smp, uint32_t t, uint32_t l, const blend_k &B, const rw_src &src) {
    if (__all_sync(0xFFFFFFFFu, t == 0xFFFFFFFFu)) {
#pragma unroll 8
        for (uint32_t k = 0; k < 32; k++) {
            const uint32_t i = (k << 5) | l;
            smp[i]           = G ? blend_src(smp[i], src.at(i)) : blend<M>(smp[i], B);
        }
        return;
    }
    /* two samples per step; with one bit left the second is the first again
       (the same value stored twice) */
    while (t) {
        const uint32_t k0 = __ffs(t) - 1;
        t &= t - 1;
        const uint32_t k1 = t ? __ffs(t) - 1 : k0;
        t &= t - 1;
        const uint32_t i0 = (k0 << 5) | l, i1 = (k1 << 5) | l;
        const uint32_t d0 = smp[i0], d1 = smp[i1];
        const uint32_t n0 = G ? blend_src(d0, src.at(i0)) : blend<M>(d0, B);
        const uint32_t n1 = G ? blend_src(d1, src.at(i1)) : blend<M>(d1, B);
        smp[i1]           = n1;
        smp[i0]           = n0;
    }
}
template <bool G>
__device__ __forceinline__ void blend_any(uint32_t *smp, uint32_t t, uint32_t l, int mode, const blend_k &B,
                                          const rw_src &src) {
    if (G)
        blend_bits<BM_ADD, true>(smp, t, l, B, src);
    else if (mode == BM_ADD)
        blend_bits<BM_ADD, false>(smp, t, l, B, src);
    else if (mode == BM_SADD)
        blend_bits<BM_SADD, false>(smp, t, l, B, src);
    else
        blend_bits<BM_SSUB, false>(smp, t, l, B, src);
}

/* One tile: sample rows [16 band, 16 band + 16) and columns
   [1024 tile, 1024 tile + 1024) of A's surface through every draw of the
   surface in order, then the resolve of its pixels.  seq is the CTA's running
   slot sequence number (identical in every thread), carried across the items
   of a persistent CTA so that the mbarrier phases stay in step.  DBG: the
   coverage read-back variant, which writes one draw's per-sample counts to
   A.cov_out and leaves the surface alone.  Returns false when a staging wait
   ran out (the tile keeps its previous samples). */
template <class T, bool GRAD, bool DBG>
__device__ __forceinline__ bool rows_item(const gb_raster_args &A, int32_t *smem, uint32_t band, uint32_t part,
                                          uint32_t tile, uint32_t &seq) {
    using namespace rw;
    constexpr int ROWS = T::ROWS, NSLOT = T::NSLOT, CAP = T::CAP, THREADS = T::THREADS, PROD = T::PROD;
    constexpr int S_SMP = T::S_SMP, S_CNT = T::S_CNT, S_OCC = T::S_OCC, S_GC = T::S_GC, S_HDR = T::S_HDR;
    constexpr int S_BAR = T::S_BAR, S_MISC = T::S_MISC, S_STG = T::S_STG, CW = T::CW;
    const uint32_t t = threadIdx.x, wi = t >> 5, l = t & 31;
    const int32_t  X0  = (int32_t)(tile * TW);
    const int32_t  TWr = min(TW, (int32_t)A.W - X0);
    const uint32_t nd  = A.ndraws;
    const size_t   cb  = (size_t)band * nd;
    const bool     dbg = DBG;
    const uint32_t rpp = A.S == 4 ? 4 : 1;
    const int32_t  tx_lo = X0 * 256 + 32, tx_hi = (X0 + TWr - 1) * 256 + 224;
    const uint32_t sm_base = (uint32_t)__cvta_generic_to_shared(smem);
    const uint32_t full0 = sm_base + S_BAR * 4, empty0 = full0 + NSLOT * 8;
    uint32_t      *misc = reinterpret_cast<uint32_t *>(smem + S_MISC);

    /* ---- load the tile's samples (or the first draw's uniform colour), the
       staged source rows and the walk bounds */
    const uint32_t band_r0 = band * GB_BAND_ROWS + part * ROWS; /* the CTA's first sample row */
    for (uint32_t i = t; i < (uint32_t)(ROWS * TW / 4); i += THREADS) {
        const uint32_t r = i / (TW / 4), c4 = (i % (TW / 4)) * 4;
        uint4          v = make_uint4(0, 0, 0, 0);
        if (band_r0 + r < A.nrows && (int32_t)c4 < TWr) {
            if (A.init_mode == 1) {
                v = make_uint4(A.init_color, A.init_color, A.init_color, A.init_color);
            } else {
                const uint32_t *src = A.samples + (size_t)(band_r0 + r) * A.Wpad + X0 + c4;
                v                   = *reinterpret_cast<const uint4 *>(src); /* Wpad: whole 16-byte runs */
            }
        }
        *reinterpret_cast<uint4 *>(smem + S_SMP + r * TW + c4) = v;
    }
    constexpr int32_t CZERO = T::C16 ? (int32_t)0x80008000u : 0; /* an empty counter word */
    for (uint32_t i = t; i < (uint32_t)(ROWS * CW) / 4; i += THREADS)
        reinterpret_cast<int4 *>(smem + S_CNT)[i] = make_int4(CZERO, CZERO, CZERO, CZERO);
    for (uint32_t i = t; i < (uint32_t)(ROWS * 32) / 4; i += THREADS)
        reinterpret_cast<int4 *>(smem + S_OCC)[i] = make_int4(0, 0, 0, 0);
    const uint32_t gc_gs = GRAD && A.S == 4 && !dbg ? A.gc_src : 0u;
    if (gc_gs) {
        for (uint32_t i = t; i < (uint32_t)(T::GCR * TW); i += THREADS) {
            const uint32_t pr = i / TW, px = i % TW, py = band_r0 / 4 + pr;
            smem[S_GC + i]    = ((int32_t)px < TWr && py < A.H)
                                    ? A.gsrc[((size_t)(gc_gs - 1) * A.H + py) * A.W + X0 + px]
                                    : 0u;
        }
    }
    if (t == 0) {
        const uint32_t ib = A.apos[cb], ie = A.apos[cb + nd];
        const uint32_t dlo = dbg ? A.cov_draw : A.draw_first, dhi = dbg ? A.cov_draw + 1 : nd;
        const uint32_t dense = 2u * (ie - ib) > nd ? 1u : 0u;
        misc[M_ABORT] = 0;
        misc[M_IEND]  = dense ? dhi : ie;
        misc[M_DLO]   = dlo;
        misc[M_DHI]   = dhi;
        misc[M_TILES] = A.W > (uint32_t)TW ? 1u : 0u;
        misc[M_DENSE] = dense;
        misc[M_I0]    = dense ? dlo : ib;
    }
    __syncthreads();

    if (wi == PROD) {
        /* ---- producer: the band's active draws in order, one slot each */
        const uint32_t iend = misc[M_IEND], dlo = misc[M_DLO], dhi = misc[M_DHI];
        const bool     tiles = misc[M_TILES] != 0, dense = misc[M_DENSE] != 0;
        bool           ok    = true;
        auto           put   = [&](uint32_t kind, uint32_t op, uint32_t src, uint32_t gs, uint32_t lo,
                                   uint32_t hi) -> bool {
            const uint32_t slot = seq % NSLOT, use = seq / NSLOT;
            bool           got  = true;
            if (l == 0 && use > 0)
                got = mbar_wait(empty0 + 8 * slot, (use - 1) & 1u, A.wait_limit);
            got = __shfl_sync(0xFFFFFFFFu, got, 0);
            /* the abort flag, read by every lane, decided for the warp */
            if (!got || __any_sync(0xFFFFFFFFu, *(volatile uint32_t *)&misc[M_ABORT] != 0)) {
                if (l == 0) {
                    atomicOr(A.status, GB_ERR_RASTER_WAIT);
                    atomicExch(&misc[M_ABORT], 1u);
                }
                return false;
            }
            if (l == 0) {
                uint32_t     *h = reinterpret_cast<uint32_t *>(smem + S_HDR + slot * HDR);
                int           mode;
                const blend_k B      = make_blend(src, op, &mode);
                const uint32_t units = hi - lo, staged = min(units, (uint32_t)CAP);
                h[H_KIND]   = kind;
                h[H_OP]     = op;
                h[H_SRC]    = B.src;
                h[H_GS]     = gs;
                h[H_LO]     = lo;
                h[H_UNITS]  = units;
                h[H_STAGED] = staged;
                h[H_MODE]   = (uint32_t)mode;
                h[H_K]      = __float_as_uint(B.k);
                h[H_C0]     = __float_as_uint(B.c0);
                h[H_C1]     = __float_as_uint(B.c1);
                h[H_C2]     = __float_as_uint(B.c2);
                h[H_C3]     = __float_as_uint(B.c3);
                h[H_INV]    = B.inv;
                if (staged)
                    stage_copy(sm_base + (S_STG + slot * CAP * 4) * 4, A.recs + lo, staged * 16u, full0 + 8 * slot);
                else
                    mbar_arrive(full0 + 8 * slot);
            }
            __syncwarp();
            seq++;
            return true;
        };
        for (uint32_t i0 = misc[M_I0]; ok && i0 < iend; i0 += 32) {
            const uint32_t il   = i0 + l;
            bool           act  = false;
            uint32_t       kind = 0, lo = 0, hi = 0, src = 0, op = 0, gs = 0;
            if (il < iend) {
                const uint32_t dl = dense ? il : A.alist[il] - A.cell0 - (uint32_t)cb;
                if (dl >= dlo && dl < dhi) {
                    const gb_draw &D = A.draws[dl];
                    kind             = D.kind;
                    src              = D.src;
                    op               = D.op;
                    gs               = D.gsrc;
                    lo               = A.cell_off[cb + dl];
                    hi               = A.cell_off[cb + dl + 1];
                    act              = kind == GB_DRAW_PAINT || kind == GB_DRAW_CLEAR || lo != hi;
                    if (hi > A.nunits || lo > hi) { /* inconsistent bins: report, skip */
                        atomicOr(A.status, GB_ERR_OVERFLOW);
                        act = false;
                    }
                    if (tiles && act && kind <= GB_DRAW_STROKE && A.dbox) {
                        const int2 bx = A.dbox[dl];
                        act           = bx.x <= tx_hi && -bx.y >= tx_lo;
                    }
                }
            }
            uint32_t amask = __ballot_sync(0xFFFFFFFFu, act);
            while (ok && amask) {
                const int j = __ffs(amask) - 1;
                amask &= amask - 1;
                ok = put(__shfl_sync(0xFFFFFFFFu, kind, j), __shfl_sync(0xFFFFFFFFu, op, j),
                         __shfl_sync(0xFFFFFFFFu, src, j), __shfl_sync(0xFFFFFFFFu, gs, j),
                         __shfl_sync(0xFFFFFFFFu, lo, j), __shfl_sync(0xFFFFFFFFu, hi, j));
            }
        }
        if (ok)
            ok = put(KIND_END, 0, 0, 0, 0, 0);
        if (l == 0) {
            /* every copy issued has landed before the tile ends (at once when
               the consumers saw them; after a consumer gave up, a copy may
               still be in flight): wait for each slot's last phase, with the
               normal limit, before the shared memory is reused or released */
            for (uint32_t s = 0; s < (uint32_t)NSLOT; s++) {
                if (seq > s) {
                    const uint32_t last = (seq - 1 - s) / NSLOT * NSLOT + s; /* the slot's last use */
                    mbar_wait(full0 + 8 * s, (last / NSLOT) & 1u);
                }
            }
        }
    } else {
        /* ---- consumer warp wi: sample row R */
        const uint32_t rr     = wi;
        const int32_t  R      = (int32_t)(band_r0 + rr);
        const bool     row_ok = R < (int32_t)A.nrows;
        const int32_t  sy     = A.S == 4 ? 32 + 64 * R : 128 + 256 * R;
        const int32_t  ox     = A.S == 4 ? ((R & 3) == 0 ? 96 : (R & 3) == 1 ? 224 : (R & 3) == 2 ? 32 : 160) : 128;
        uint32_t      *smp    = reinterpret_cast<uint32_t *>(smem + S_SMP + rr * TW);
        int32_t       *cnt    = smem + S_CNT + rr * CW;
        uint32_t      *occ    = reinterpret_cast<uint32_t *>(smem + S_OCC + rr * 32);
        /* the crossing counter of position p (16-bit ones: half p & 1 of
           word p >> 1, biased by 2^15) */
        auto cadd = [&](uint32_t p, int32_t dir) {
            if (T::C16)
                atomicAdd(&cnt[p >> 1], (int32_t)((uint32_t)dir << (16u * (p & 1u))));
            else
                atomicAdd(&cnt[p], dir);
        };
        auto cget = [&](uint32_t p) -> int32_t {
            if (!T::C16)
                return cnt[p];
            return (int32_t)reinterpret_cast<const uint16_t *>(cnt)[p] - 32768;
        };
        /* lane l's run of counters back to empty (16-byte stores) */
        auto cclear = [&]() {
            int4 *q = reinterpret_cast<int4 *>(cnt + (T::C16 ? 16u : 32u) * l);
#pragma unroll
            for (int i = 0; i < (T::C16 ? 4 : 8); i++)
                q[i] = make_int4(CZERO, CZERO, CZERO, CZERO);
        };
        /* this lane's run of the row [32 l, 32 l + 32): the samples inside the tile */
        const int32_t  nrun  = TWr - 32 * (int32_t)l;
        const uint32_t vmask = !row_ok || nrun <= 0 ? 0u : nrun >= 32 ? 0xFFFFFFFFu : (1u << nrun) - 1u;
        /* after the transpose lane l holds samples 32 k + l: valid for k with 32 k + l < TWr */
        const uint32_t  tvalid    = warp_transpose32(vmask, l);
        const uint32_t *grow_base = GRAD ? A.gsrc + (size_t)(row_ok ? R / rpp : 0) * A.W + X0 : nullptr;
        const uint32_t *gc_row    = reinterpret_cast<const uint32_t *>(smem + S_GC) + (rr / 4) * TW;
        for (;;) {
            const uint32_t slot = seq % NSLOT, use = seq / NSLOT;
            /* every lane observes the phase (the header and the staged records
               become visible to it); the warp decides together */
            const bool got = __all_sync(0xFFFFFFFFu, mbar_wait(full0 + 8 * slot, use & 1u, A.wait_limit));
            if (!got || __any_sync(0xFFFFFFFFu, *(volatile uint32_t *)&misc[M_ABORT] != 0)) {
                if (l == 0) {
                    atomicOr(A.status, GB_ERR_RASTER_WAIT);
                    atomicExch(&misc[M_ABORT], 1u);
                }
                break;
            }
            seq++;
            const uint32_t *h    = reinterpret_cast<const uint32_t *>(smem + S_HDR + slot * HDR);
            const uint32_t  kind = h[H_KIND];
            if (kind == KIND_END) {
                __syncwarp();
                if (l == 0)
                    mbar_arrive(empty0 + 8 * slot);
                break;
            }
            const uint4    h0 = reinterpret_cast<const uint4 *>(h)[0], h1 = reinterpret_cast<const uint4 *>(h)[1];
            const uint4    h2 = reinterpret_cast<const uint4 *>(h)[2], h3 = reinterpret_cast<const uint4 *>(h)[3];
            const uint32_t gs = h0.w, lo = h1.x, units = h1.y, staged = h1.z;
            const int      mode = (int)h1.w;
            blend_k        B;
            B.src = h0.z;
            B.k   = __uint_as_float(h2.x);
            B.c0  = __uint_as_float(h2.y);
            B.c1  = __uint_as_float(h2.z);
            B.c2  = __uint_as_float(h2.w);
            B.c3  = __uint_as_float(h3.x);
            B.inv = h3.y;
            /* even-odd fills keep only the parity of each position's crossings
               (a bit toggled per crossing); non-zero fills and strokes keep
               counts, with the occupied positions flagged */
            const bool eo = !dbg && kind == GB_DRAW_FILL_EO;
            /* ---- accumulate this row's crossings of the draw's edges */
            if (row_ok && kind <= GB_DRAW_STROKE) {
                const int4 *sg = reinterpret_cast<const int4 *>(smem + S_STG) + slot * CAP;
                for (uint32_t u = l; u < units; u += 32) {
                    const int4    ed  = u < staged ? sg[u] : A.recs[lo + u];
                    const int32_t ylo = min(ed.y, ed.w), yhi = max(ed.y, ed.w);
                    if (sy < ylo || sy >= yhi || max(ed.x, ed.z) < tx_lo)
                        continue; /* no crossing of this row, or left of every tile sample */
                    int32_t k;
                    if (min(ed.x, ed.z) > tx_hi) {
                        k = TWr;
                    } else {
                        const int32_t   dy  = ed.w - ed.y;
                        const int32_t   den = dy < 0 ? -dy : dy;
                        const int32_t   dxn = dy < 0 ? ed.x - ed.z : ed.z - ed.x;
                        const long long c   = gb_ceil_muldiv(dxn, sy - ed.y, den);
                        const long long kt  = (((long long)ed.x + c - 1 - ox) >> 8) + 1 - X0;
                        if (kt <= 0)
                            continue;
                        k = kt > TWr ? TWr : (int32_t)kt;
                    }
                    const uint32_t p = (uint32_t)(k - 1);
                    if (eo) {
                        atomicXor(&occ[p >> 5], 1u << (p & 31u));
                    } else {
                        cadd(p, ed.y < ed.w ? 1 : -1);
                        atomicOr(&occ[p >> 5], 1u << (p & 31u));
                    }
                }
            }
            __syncwarp();
            if (l == 0)
                mbar_arrive(empty0 + 8 * slot); /* this warp is done with the slot */
            if (!row_ok)
                continue;
            const rw_src S{grow_base, gc_gs && gs == gc_gs ? gc_row : nullptr};
            if (kind == GB_DRAW_PAINT || kind == GB_DRAW_CLEAR) {
                if (dbg) { /* a paint covers every sample; a clear reports nothing */
                    for (uint32_t k = 0; k < 32 && kind == GB_DRAW_PAINT; k++) {
                        const uint32_t c = (k << 5) | l;
                        if ((tvalid >> k) & 1u)
                            A.cov_out[((size_t)(R / rpp) * A.W + X0 + c) * A.S + R % rpp] = 1;
                    }
                    continue;
                }
                if (kind == GB_DRAW_CLEAR) {
                    for (uint32_t k = 0; k < 32; k++)
                        if ((tvalid >> k) & 1u)
                            smp[(k << 5) | l] = 0u;
                    continue;
                }
                if (GRAD && gs) {
                    const rw_src SG{grow_base + (size_t)(gs - 1) * A.H * A.W, S.gc};
                    blend_any<true>(smp, tvalid, l, mode, B, SG);
                } else {
                    blend_any<false>(smp, tvalid, l, mode, B, S);
                }
                continue;
            }
            const rw_src   SG{GRAD && gs ? grow_base + (size_t)(gs - 1) * A.H * A.W : grow_base, S.gc};
            const uint32_t m = occ[l];
            /* a row no crossing reached: winding zero everywhere, nothing to draw */
            if (__ballot_sync(0xFFFFFFFFu, m != 0) == 0) {
                __syncwarp();
                continue;
            }
            occ[l] = 0;
            if (eo) {
                /* bit j of the suffix XOR: parity of the crossings at or right
                   of sample j in this run; the runs to the right add theirs */
                uint32_t y = m;
                y ^= y >> 1;
                y ^= y >> 2;
                y ^= y >> 4;
                y ^= y >> 8;
                y ^= y >> 16;
                const uint32_t par = __ballot_sync(0xFFFFFFFFu, __popc(m) & 1);
                if (__popc(par >> l >> 1) & 1) /* l + 1 may be 32: shifted in two steps */
                    y = ~y;
                const uint32_t tb = warp_transpose32(y & vmask, l);
                if (GRAD && gs)
                    blend_any<true>(smp, tb, l, mode, B, SG);
                else
                    blend_any<false>(smp, tb, l, mode, B, S);
                __syncwarp();
                continue;
            }
            /* ---- resolve: the counts at the run's occupied positions, and the
               winding entering the run from the right */
            int32_t rs = 0;
            for (uint32_t b = m; b; b &= b - 1)
                rs += cget((l << 5) + __ffs(b) - 1);
            int32_t incl = rs; /* sum over this lane's run and the runs right of it */
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int32_t v = __shfl_down_sync(0xFFFFFFFFu, incl, o);
                if (l + o < 32)
                    incl += v;
            }
            if (dbg) {
                int32_t w = incl - rs;
                for (int j = 31; j >= 0; j--) {
                    w += cget((l << 5) + j);
                    if ((vmask >> j) & 1u)
                        A.cov_out[((size_t)(R / rpp) * A.W + X0 + 32 * l + j) * A.S + R % rpp] = w;
                }
            }
            /* walk the occupied positions left to right (the winding left of
               position p includes its count): non-zero fills cover w != 0;
               strokes blend once per covering triangle, so pass k covers
               w > k, the first two passes' masks in this walk */
            const bool stroke = kind == GB_DRAW_STROKE;
            uint32_t   c1 = 0, c2 = 0, start = 0;
            int32_t    w = incl, kmax = 0;
            if (!stroke) {
                for (uint32_t b = m; b; b &= b - 1) {
                    const uint32_t p = __ffs(b) - 1;
                    c1 |= w != 0 ? bit_range(start, p) : 0u;
                    w -= cget((l << 5) + p);
                    start = p + 1;
                }
                if (start < 32 && w != 0)
                    c1 |= bit_range(start, 31);
            } else {
                for (uint32_t b = m; b; b &= b - 1) {
                    const uint32_t p = __ffs(b) - 1;
                    const uint32_t r = bit_range(start, p);
                    c1 |= w > 0 ? r : 0u;
                    c2 |= w > 1 ? r : 0u;
                    kmax = max(kmax, w);
                    w -= cget((l << 5) + p);
                    start = p + 1;
                }
                if (start < 32) {
                    const uint32_t r = bit_range(start, 31);
                    c1 |= w > 0 ? r : 0u;
                    c2 |= w > 1 ? r : 0u;
                    kmax = max(kmax, w);
                }
            }
            if (!dbg) {
                const int32_t kw = stroke ? __reduce_max_sync(0xFFFFFFFFu, kmax) : 1;
                for (int32_t rep = 0; rep < kw; rep++) {
                    uint32_t cv = rep == 0 ? c1 : c2;
                    if (rep >= 2) { /* three or more covering triangles: walk again */
                        int32_t  ww = incl;
                        uint32_t st = 0;
                        cv          = 0;
                        for (uint32_t b = m; b; b &= b - 1) {
                            const uint32_t p = __ffs(b) - 1;
                            cv |= ww > rep ? bit_range(st, p) : 0u;
                            ww -= cget((l << 5) + p);
                            st = p + 1;
                        }
                        cv |= st < 32 && ww > rep ? bit_range(st, 31) : 0u;
                    }
                    const uint32_t tb = warp_transpose32(cv & vmask, l);
                    if (GRAD && gs)
                        blend_any<true>(smp, tb, l, mode, B, SG);
                    else
                        blend_any<false>(smp, tb, l, mode, B, S);
                }
            }
            if (m)
                cclear();
            __syncwarp();
        }
    }
    __syncthreads();
    if (misc[M_ABORT])
        return false; /* the tile keeps its previous samples; the status word says why */
    if (dbg)
        return true;
    /* ---- write back the samples, then resolve the tile's pixels */
    for (uint32_t i = t; i < (uint32_t)(ROWS * TW / 4); i += THREADS) {
        const uint32_t r = i / (TW / 4), c4 = (i % (TW / 4)) * 4;
        if (band_r0 + r < A.nrows && (int32_t)c4 < TWr)
            *reinterpret_cast<uint4 *>(A.samples + (size_t)(band_r0 + r) * A.Wpad + X0 + c4) =
                *reinterpret_cast<const uint4 *>(smem + S_SMP + r * TW + c4);
    }
    const uint32_t *stage = reinterpret_cast<const uint32_t *>(smem + S_SMP);
    const uint32_t  prows = ROWS / rpp;
    for (uint32_t q = t * 4; q < prows * TW; q += THREADS * 4) {
        const uint32_t pr = q / TW, px = q % TW, py = band_r0 / rpp + pr;
        if (py >= A.H || (int32_t)px >= TWr)
            continue;
        uint32_t outp[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t s0 = 0, s1 = 0, s2 = 0, s3 = 0;
            for (uint32_t s = 0; s < rpp; s++) {
                const uint32_t v = stage[(pr * rpp + s) * TW + px + k];
                s0 += v & 0xFFu;
                s1 += (v >> 8) & 0xFFu;
                s2 += (v >> 16) & 0xFFu;
                s3 += v >> 24;
            }
            const uint32_t hh = rpp / 2;
            outp[k] = ((s0 + hh) / rpp) | (((s1 + hh) / rpp) << 8) | (((s2 + hh) / rpp) << 16) |
                      (((s3 + hh) / rpp) << 24);
        }
        uint32_t *dst = A.rgba + (size_t)py * A.W + X0 + px;
        if ((int32_t)px + 4 <= TWr && ((((uintptr_t)dst) & 15u) == 0)) {
            *reinterpret_cast<uint4 *>(dst) = make_uint4(outp[0], outp[1], outp[2], outp[3]);
        } else {
            for (int k = 0; k < 4; k++)
                if ((int32_t)(px + k) < TWr)
                    dst[k] = outp[k];
        }
    }
    __syncthreads(); /* the next item of a persistent CTA reuses the shared memory */
    return true;
}

template <class T> __device__ __forceinline__ void rows_init_barriers(int32_t *smem) {
    if (threadIdx.x == 0) {
        const uint32_t full0 = (uint32_t)__cvta_generic_to_shared(smem) + T::S_BAR * 4, empty0 = full0 + T::NSLOT * 8;
        for (uint32_t s = 0; s < (uint32_t)T::NSLOT; s++) {
            mbar_init_n(full0 + 8 * s, 1);
            mbar_init_n(empty0 + 8 * s, T::ROWS);
        }
        mbar_init_fence();
    }
    __syncthreads();
}

/* grid: x tiles, y bands times the parts of a band (16 / ROWS).  The
   register file's four partitions hold whole warps: 17 warps leave 96
   registers a thread, three CTAs of 9 warps 72 */
template <class T, bool GRAD, bool DBG>
__global__ void __launch_bounds__(T::THREADS, T::MINB) gb_raster_rows(gb_raster_args A) {
    extern __shared__ __align__(16) int32_t smem[];
    rows_init_barriers<T>(smem);
    uint32_t           seq   = 0;
    constexpr uint32_t parts = GB_BAND_ROWS / T::ROWS;
    rows_item<T, GRAD, DBG>(A, smem, blockIdx.y / parts, blockIdx.y % parts, blockIdx.x, seq);
}

/* The batch raster in the row form: a persistent grid (one CTA per SM)
   takes (surface, band, tile) items from the work list until it is
   exhausted; no CTA waits on another. */
__global__ void __launch_bounds__(RW16::THREADS, 1)
    gb_raster_rows_batch(gb_raster_args A0, const gb_surf *__restrict__ surfs, const uint4 *__restrict__ items,
                         uint32_t nitems, uint32_t *__restrict__ queue) {
    extern __shared__ __align__(16) int32_t smem[];
    __shared__ gb_raster_args Ai;
    __shared__ uint32_t       cur_item, cur_band, cur_tile;
    rows_init_barriers<RW16>(smem);
    uint32_t seq = 0;
    for (uint32_t iter = 0; iter < nitems; iter++) {
        if (threadIdx.x == 0) {
            const uint32_t it = atomicAdd(queue, 1u);
            cur_item          = it;
            if (it < nitems) {
                const uint4    w  = items[it];
                const gb_surf &sf = surfs[w.x];
                gb_raster_args a  = A0;
                a.W               = sf.W;
                a.H               = sf.H;
                a.Wpad            = sf.wpad;
                a.nrows           = sf.nrows;
                a.nbands          = sf.nbands;
                a.ndraws          = sf.ndraws;
                a.draw_first      = sf.draw_first;
                a.init_mode       = sf.init_mode;
                a.init_color      = sf.init_color;
                a.draws           = A0.draws + sf.draw0;
                a.cell_off        = A0.cell_off + sf.cell0;
                a.apos            = A0.apos + sf.cell0;
                a.cell0           = (uint32_t)sf.cell0;
                a.dbox            = A0.dbox ? A0.dbox + sf.draw0 : nullptr;
                a.samples         = sf.samples;
                a.rgba            = sf.rgba;
                Ai                = a;
                cur_band          = w.y;
                cur_tile          = w.z;
            }
        }
        __syncthreads();
        if (cur_item >= nitems)
            break;
        if (!rows_item<RW16, false, false>(Ai, smem, cur_band, 0, cur_tile, seq))
            break; /* mbarrier phases no longer in step: stop this CTA */
    }
}

extern "C" uint32_t gb_raster_rows_tile_width() { return rw::TW; }

template <class T, bool GRAD, bool DBG> static cudaError_t rows_launch(cudaStream_t st, const gb_raster_args *a) {
    static std::atomic<bool> configured{false}; /* set once; a second setter is harmless */
    if (!configured.load(std::memory_order_acquire)) {
        const cudaError_t e =
            cudaFuncSetAttribute(gb_raster_rows<T, GRAD, DBG>, cudaFuncAttributeMaxDynamicSharedMemorySize, T::SMEM);
        if (e != cudaSuccess)
            return e;
        configured.store(true, std::memory_order_release);
    }
    const dim3 grid((a->W + rw::TW - 1) / rw::TW, a->nbands * (GB_BAND_ROWS / T::ROWS));
    gb_raster_rows<T, GRAD, DBG><<<grid, T::THREADS, T::SMEM, st>>>(*a);
    return cudaGetLastError();
}
template <class T> static cudaError_t rows_pick(cudaStream_t st, const gb_raster_args *a, int gradients) {
    if (a->cov_out)
        return gradients ? rows_launch<T, true, true>(st, a) : rows_launch<T, false, true>(st, a);
    return gradients ? rows_launch<T, true, false>(st, a) : rows_launch<T, false, false>(st, a);
}
extern "C" cudaError_t gb_launch_raster_rows(cudaStream_t st, const gb_raster_args *a, int gradients, int half) {
    if (a->nbands == 0)
        return cudaSuccess;
    return half ? rows_pick<RW8>(st, a, gradients) : rows_pick<RW16>(st, a, gradients);
}

extern "C" cudaError_t gb_launch_raster_rows_batch(cudaStream_t st, const gb_raster_args *a, const gb_surf *surfs,
                                                  const uint4 *items, uint32_t nitems, uint32_t *queue,
                                                  uint32_t nctas) {
    static std::atomic<bool> configured{false}; /* set once; a second setter is harmless */
    if (!nitems)
        return cudaSuccess;
    if (!configured.load(std::memory_order_acquire)) {
        cudaError_t e =
            cudaFuncSetAttribute(gb_raster_rows_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, RW16::SMEM);
        if (e != cudaSuccess)
            return e;
        configured.store(true, std::memory_order_release);
    }
    gb_raster_rows_batch<<<nctas, RW16::THREADS, RW16::SMEM, st>>>(*a, surfs, items, nitems, queue);
    return cudaGetLastError();
}
