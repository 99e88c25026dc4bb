/*
 * rsc_sort.cuh -- spatial order of the background scatterers.
 *
 * Scatterers are independent: where one sits in the attribute arrays changes
 * nothing in its evolution.  The worker may therefore keep the background
 * range in spatial order (range shells, then Morton order of direction),
 * which makes a warp's 32 scatterers neighbours in space: their range-gate candidates
 * coincide (the pulse kernel then sums each gate across the warp instead of
 * with per-lane atomics) and their LES texels overlap (the advance kernel's
 * gathers hit L1).  The order is restored by a counting sort every few
 * hundred steps; perm[slot] is the scatterer's index in the caller's order
 * and inv[index] its slot, used by upload and download.
 *
 * Sort of [origin, origin + count), H <= 2^22 cells:
 *   k_sort_key      cell of each scatterer, histogram (atomics)
 *   k_scan_*        exclusive scan of the histogram (three launches)
 *   k_sort_scatter  slot of each scatterer (atomics: the order inside a cell
 *                   is arbitrary, which no result depends on)
 *   k_sort_permute  every array and perm into the second buffer set (slots
 *                   outside the range copied through)
 *   k_sort_inverse  inv from the new perm
 */
#ifndef SIMRADAR_GB300_RSC_SORT_CUH
#define SIMRADAR_GB300_RSC_SORT_CUH

#include <cuda_runtime.h>
#include <stdint.h>

namespace rsc {

constexpr unsigned kSortThreads = 256;
constexpr unsigned kScanThreads = 1024;
constexpr unsigned kScanPerThread = 4;
constexpr unsigned kScanBlock = kScanThreads * kScanPerThread;   /* histogram entries per scan block */
constexpr unsigned kMaxSortCells = 1u << 22;                     /* histogram entries */

/* the 16 low bits of v spread to every second bit (2-D Morton order) */
__device__ __forceinline__ unsigned morton_spread(unsigned v) {
    v &= 0xffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

/* cell of x among `cells` equal cells covering [o, o + 1 / inv_len) */
__device__ __forceinline__ unsigned cell_axis(float x, float o, float inv_size, float cells) {
    float f = (x - o) * inv_size * cells;
    f = fminf(fmaxf(f, 0.0f), cells - 1.0f);   /* NaN -> 0 */
    return (unsigned)f;
}

/* Cells are range-major: shells of a quarter gate in range, each divided
 * in 2^bits x 2^bits direction cells (the direction cosines x / r and z / r
 * over the box) in Morton order.  A warp's scatterers then share a range
 * shell (so they reach the same few gates) and a small patch of directions
 * (so their LES texels are neighbours). */
struct SortArgs {
    const float4 *pos;
    unsigned long long origin, count;
    float r0, ir;          /* range covered by the shells: start, 1 / length */
    float u0, iu, v0, iv;  /* x / r and z / r covered by the cells: start, 1 / length */
    unsigned shells, bits;
    unsigned *key;
    unsigned *hist;
};

__global__ void __launch_bounds__(kSortThreads) k_sort_key(const SortArgs a) {
    const unsigned long long i = (unsigned long long)blockIdx.x * kSortThreads + threadIdx.x;
    if (i >= a.count) return;
    const float4 p = a.pos[a.origin + i];
    const float r = sqrtf(p.x * p.x + p.y * p.y + p.z * p.z);
    const float ri = r > 0.0f ? 1.0f / r : 0.0f;
    const unsigned sh = cell_axis(r, a.r0, a.ir, (float)a.shells);
    const float cells = (float)(1u << a.bits);
    const unsigned cu = cell_axis(p.x * ri, a.u0, a.iu, cells);
    const unsigned cv = cell_axis(p.z * ri, a.v0, a.iv, cells);
    const unsigned code = (sh << (2 * a.bits)) | morton_spread(cu) | (morton_spread(cv) << 1);
    a.key[i] = code;
    atomicAdd(a.hist + code, 1u);
}

/* exclusive scan of 4 per thread over a block: returns the thread's offset
 * within the block and the block total */
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned *total) {
    __shared__ unsigned warp_sums[kScanThreads / 32];
    const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    unsigned incl = v;
#pragma unroll
    for (unsigned o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned s = warp_sums[lane];
#pragma unroll
        for (unsigned o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        warp_sums[lane] = s;   /* inclusive over warps */
    }
    __syncthreads();
    const unsigned before = warp ? warp_sums[warp - 1] : 0u;
    *total = warp_sums[kScanThreads / 32 - 1];
    return before + incl - v;
}

/* per block: exclusive scan of kScanBlock entries in place, block total out */
__global__ void __launch_bounds__(kScanThreads) k_scan_blocks(unsigned *data, unsigned n, unsigned *block_sums) {
    const unsigned base = blockIdx.x * kScanBlock + threadIdx.x * kScanPerThread;
    unsigned v[kScanPerThread];
    unsigned sum = 0;
#pragma unroll
    for (unsigned k = 0; k < kScanPerThread; k++) {
        v[k] = (base + k < n) ? data[base + k] : 0u;
        sum += v[k];
    }
    unsigned total;
    unsigned off = block_exclusive_scan(sum, &total);
#pragma unroll
    for (unsigned k = 0; k < kScanPerThread; k++) {
        if (base + k < n) data[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

/* one block: exclusive scan of the block totals (n <= kScanBlock) */
__global__ void __launch_bounds__(kScanThreads) k_scan_top(unsigned *block_sums, unsigned n) {
    const unsigned base = threadIdx.x * kScanPerThread;
    unsigned v[kScanPerThread];
    unsigned sum = 0;
#pragma unroll
    for (unsigned k = 0; k < kScanPerThread; k++) {
        v[k] = (base + k < n) ? block_sums[base + k] : 0u;
        sum += v[k];
    }
    unsigned total;
    unsigned off = block_exclusive_scan(sum, &total);
#pragma unroll
    for (unsigned k = 0; k < kScanPerThread; k++) {
        if (base + k < n) block_sums[base + k] = off;
        off += v[k];
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(unsigned *data, unsigned n, const unsigned *block_sums) {
    const unsigned add = block_sums[blockIdx.x];
    const unsigned base = blockIdx.x * kScanBlock + threadIdx.x * kScanPerThread;
#pragma unroll
    for (unsigned k = 0; k < kScanPerThread; k++) {
        if (base + k < n) data[base + k] += add;
    }
}

__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const unsigned *key, unsigned long long count,
                                                               unsigned *offsets, unsigned *order) {
    const unsigned long long i = (unsigned long long)blockIdx.x * kSortThreads + threadIdx.x;
    if (i >= count) return;
    const unsigned slot = atomicAdd(offsets + key[i], 1u);
    order[slot] = (unsigned)i;
}

struct PermuteArgs {
    const uint4 *src[8];
    uint4 *dst[8];
    const unsigned *perm_src;
    unsigned *perm_dst;
    unsigned long long origin, count, numel;
    const unsigned *order;   /* slot - origin -> source index - origin, inside the range */
};

__global__ void __launch_bounds__(kSortThreads) k_sort_permute(const PermuteArgs a) {
    const unsigned long long s = (unsigned long long)blockIdx.x * kSortThreads + threadIdx.x;
    if (s >= a.numel) return;
    unsigned long long from = s;
    if (s >= a.origin && s - a.origin < a.count) from = a.origin + a.order[s - a.origin];
#pragma unroll
    for (int k = 0; k < 8; k++) a.dst[k][s] = a.src[k][from];
    a.perm_dst[s] = a.perm_src[from];
}

__global__ void __launch_bounds__(kSortThreads) k_sort_inverse(const unsigned *perm, unsigned *inv,
                                                               unsigned long long numel) {
    const unsigned long long s = (unsigned long long)blockIdx.x * kSortThreads + threadIdx.x;
    if (s >= numel) return;
    inv[perm[s]] = (unsigned)s;
}

__global__ void __launch_bounds__(kSortThreads) k_iota(unsigned *a, unsigned long long n) {
    const unsigned long long s = (unsigned long long)blockIdx.x * kSortThreads + threadIdx.x;
    if (s < n) a[s] = (unsigned)s;
}

/* caller order <-> slot order for upload and download */
__global__ void __launch_bounds__(kSortThreads) k_gather16(uint4 *dst, const uint4 *src, const unsigned *inv,
                                                           unsigned long long offset, unsigned long long count) {
    const unsigned long long j = (unsigned long long)blockIdx.x * kSortThreads + threadIdx.x;
    if (j < count) dst[j] = src[inv[offset + j]];
}

__global__ void __launch_bounds__(kSortThreads) k_scatter16(uint4 *dst, const uint4 *src, const unsigned *inv,
                                                            unsigned long long offset, unsigned long long count) {
    const unsigned long long j = (unsigned long long)blockIdx.x * kSortThreads + threadIdx.x;
    if (j < count) dst[inv[offset + j]] = src[j];
}

}  // namespace rsc

#endif
