/*
 * Exclusive prefix sums over uint32 counts, used to turn per-item output
 * counts into output offsets.  out has n+1 entries; out[n] is the total.
 * Three phases: per-block sums, one-block scan of the block sums, per-block
 * scan plus block prefix.  4096 items per 1024-thread block.
 */
#include "vkvg_gb300.h"

#include <cuda.h>
#include <cuda_runtime.h>
#include <mutex>
#include <stdint.h>
#include <stdio.h>

#define SCAN_THREADS 1024
#define SCAN_ITEMS   4
#define SCAN_TILE    (SCAN_THREADS * SCAN_ITEMS)

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t v) {
    uint32_t lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= (uint32_t)o)
            v += t;
    }
    return v;
}
/* block-wide exclusive scan of one value per thread; returns the total */
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *excl) {
    __shared__ uint32_t wsum[SCAN_THREADS / 32];
    uint32_t            lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t            inc  = warp_incl_scan(v);
    if (lane == 31)
        wsum[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (blockDim.x >> 5) ? wsum[lane] : 0;
        w          = warp_incl_scan(w);
        wsum[lane] = w;
    }
    __syncthreads();
    uint32_t prefix = warp ? wsum[warp - 1] : 0;
    *excl           = prefix + inc - v;
    uint32_t total  = wsum[(blockDim.x >> 5) - 1];
    __syncthreads();
    return total;
}

__global__ void scan_block_sums(const uint32_t *__restrict__ in, uint32_t n, uint32_t *__restrict__ bsum) {
    uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    uint32_t s    = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++)
        if (base + k < n)
            s += in[base + k];
    uint32_t excl;
    uint32_t tot = block_excl_scan(s, &excl);
    if (threadIdx.x == 0)
        bsum[blockIdx.x] = tot;
}
/* single block: exclusive scan of nb block sums in place, writes total to bsum[nb] */
__global__ void scan_block_prefix(uint32_t *__restrict__ bsum, uint32_t nb) {
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += SCAN_THREADS) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < nb ? bsum[i] : 0;
        uint32_t excl;
        uint32_t tot = block_excl_scan(v, &excl);
        if (i < nb)
            bsum[i] = carry + excl;
        carry += tot;
    }
    if (threadIdx.x == 0)
        bsum[nb] = carry;
}
__global__ void scan_apply(const uint32_t *__restrict__ in, uint32_t n, const uint32_t *__restrict__ bsum,
                           uint32_t *__restrict__ out) {
    uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    uint32_t v[SCAN_ITEMS], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
    }
    uint32_t excl;
    block_excl_scan(s, &excl);
    uint32_t run = bsum[blockIdx.x] + excl;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n)
            out[base + k] = run;
        run += v[k];
    }
    uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (blockIdx.x == nb - 1 && threadIdx.x == 0)
        out[n] = bsum[nb];
}

extern "C" {
/* scratch must hold (n + SCAN_TILE - 1) / SCAN_TILE + 1 words */
size_t gb_scan_scratch_words(uint32_t n) { return (size_t)(n + SCAN_TILE - 1) / SCAN_TILE + 1; }
cudaError_t gb_exclusive_scan(cudaStream_t st, const uint32_t *in, uint32_t n, uint32_t *out, uint32_t *scratch) {
    if (n == 0)
        return cudaMemsetAsync(out, 0, sizeof(uint32_t), st);
    uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    scan_block_sums<<<nb, SCAN_THREADS, 0, st>>>(in, n, scratch);
    scan_block_prefix<<<1, SCAN_THREADS, 0, st>>>(scratch, nb);
    scan_apply<<<nb, SCAN_THREADS, 0, st>>>(in, n, scratch, out);
    return cudaGetLastError();
}
}

/* ---- exclusive scan without allocation.
 *
 * The same three kernels, with the block sums kept in a fixed array that is
 * part of the module's device image instead of a buffer allocated by the
 * pipeline.  Block sums are fully written by the first kernel before the
 * others read them, so the array needs no initial contents.  Its device
 * address is looked up once per device context, by the first call made with
 * that device current: the cache is keyed by the context's unique id, so a
 * context created anew after cudaDeviceReset (which reloads the module,
 * possibly elsewhere) gets a fresh lookup instead of a stale address.  All
 * calls on one device share the array. */
#define SCAN_NOALLOC_WORDS ((VKVG_GB300_SCAN_NOALLOC_MAX + SCAN_TILE - 1) / SCAN_TILE + 1)
#define SCAN_NOALLOC_DEVS  64

static __device__ __align__(256) uint32_t g_scan_noalloc_scratch[SCAN_NOALLOC_WORDS];

void gb_count_launch(uint64_t n);

/* the current context's unique id through the driver entry points the
   runtime hands out (nothing linked against libcuda); 0 when unavailable */
typedef CUresult (*pfn_ctx_current)(CUcontext *);
typedef CUresult (*pfn_ctx_id)(CUcontext, unsigned long long *);
static unsigned long long current_ctx_id() {
    static pfn_ctx_current get_cur = nullptr;
    static pfn_ctx_id      get_id  = nullptr;
    static std::once_flag  once;
    std::call_once(once, [] {
        void *f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, nullptr) ==
                cudaSuccess)
            get_cur = (pfn_ctx_current)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, nullptr) == cudaSuccess)
            get_id = (pfn_ctx_id)f;
    });
    CUcontext          c  = nullptr;
    unsigned long long id = 0;
    if (!get_cur || !get_id || get_cur(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

extern "C" vkvg_status_t vkvg_gb300_exclusive_scan_noalloc(void *stream, const uint32_t *counts, uint32_t n,
                                                            uint32_t *offsets) {
    static std::mutex         lock;
    static uint32_t          *scratch[SCAN_NOALLOC_DEVS];
    static unsigned long long scratch_ctx[SCAN_NOALLOC_DEVS];
    if (!offsets || (n && !counts))
        return VKVG_STATUS_NULL_POINTER;
    if (n > VKVG_GB300_SCAN_NOALLOC_MAX) {
        fprintf(stderr, "vkvg_gb300_exclusive_scan_noalloc: %u items exceed its fixed limit of %u\n", n,
                (unsigned)VKVG_GB300_SCAN_NOALLOC_MAX);
        return VKVG_STATUS_NO_MEMORY;
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= SCAN_NOALLOC_DEVS)
        return VKVG_STATUS_DEVICE_ERROR;
    uint32_t *sp;
    {
        std::lock_guard<std::mutex> g(lock);
        const unsigned long long    id = current_ctx_id();
        if (!scratch[dev] || !id || scratch_ctx[dev] != id) {
            /* the lookup also makes the device's primary context current */
            void       *p = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&p, g_scan_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                fprintf(stderr, "vkvg_gb300_exclusive_scan_noalloc: scratch lookup failed: %s\n",
                        cudaGetErrorString(e));
                return VKVG_STATUS_DEVICE_ERROR;
            }
            scratch[dev]     = (uint32_t *)p;
            scratch_ctx[dev] = current_ctx_id();
        }
        sp = scratch[dev];
    }
    cudaError_t e = gb_exclusive_scan((cudaStream_t)stream, counts, n, offsets, sp);
    if (e != cudaSuccess)
        return VKVG_STATUS_DEVICE_ERROR;
    gb_count_launch(n ? 3 : 0);
    return VKVG_STATUS_SUCCESS;
}
