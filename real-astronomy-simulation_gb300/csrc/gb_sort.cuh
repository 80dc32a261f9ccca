// Stable LSD radix sort of (key, 32-bit value) pairs, 8-bit digits, shared by
// the tree build (Morton keys) and the neighbour grid (cell keys).  One pass
// is an upsweep (per-tile digit counts), a row scan (per-digit offsets over
// tiles) and a stable downsweep (ranking within a tile in index order).
#pragma once

#include "gb_common.cuh"

namespace gb {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;  // 4096 keys per CTA
constexpr int RS_BINS = 256;

// Histogram entries the sort of up to n keys needs.
inline int64_t radix_hist_size(int64_t n) { return (int64_t)RS_BINS * ((n + RS_TILE - 1) / RS_TILE); }

// ------------------------------------------------------------ radix sort
template <typename KeyT>
__global__ void __launch_bounds__(RS_THREADS)
rs_upsweep_kernel(const KeyT *__restrict__ keys, int64_t n, int shift, uint32_t *__restrict__ hist, int nb) {
    __shared__ uint32_t h[RS_BINS];
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) h[d] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_TILE;
    for (int k = threadIdx.x; k < RS_TILE; k += RS_THREADS) {
        const int64_t i = base + k;
        if (i < n) atomicAdd(&h[(uint32_t)(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) hist[(int64_t)d * nb + blockIdx.x] = h[d];
}

// Exclusive scan of 256 values held one per thread of a 256-thread CTA.
__device__ __forceinline__ uint32_t cta256_exclusive_scan(uint32_t v, uint32_t *wsum) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const uint32_t w = lane < RS_WARPS ? wsum[lane] : 0u;
        uint32_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < RS_WARPS) wsum[lane] = wi - w;
    }
    __syncthreads();
    return wsum[wid] + inc - v;
}

// Row scan: CTA d turns row d of the digit-major histogram (one count per
// tile) into exclusive offsets within the digit and stores the digit total.
static __global__ void __launch_bounds__(RS_THREADS) rs_rowscan_kernel(uint32_t *hist, int nb, uint32_t *totals) {
    __shared__ uint32_t wsum[RS_WARPS];
    uint32_t *row = hist + (int64_t)blockIdx.x * nb;
    const int per = (nb + RS_THREADS - 1) / RS_THREADS;
    const int b0 = min(nb, (int)threadIdx.x * per), b1 = min(nb, b0 + per);
    uint32_t v = 0;
    for (int b = b0; b < b1; ++b) v += row[b];
    const uint32_t excl = cta256_exclusive_scan(v, wsum);
    uint32_t run = excl;
    for (int b = b0; b < b1; ++b) {
        const uint32_t t = row[b];
        row[b] = run;
        run += t;
    }
    if (threadIdx.x == RS_THREADS - 1) totals[blockIdx.x] = excl + v;
}

// Stable scatter: elements of a tile are ranked in index order (warp, round,
// lane) among equal digits with match/ballot, then written to the scanned
// global offset of (digit, tile).
template <typename KeyT>
__global__ void __launch_bounds__(RS_THREADS)
rs_downsweep_kernel(const KeyT *__restrict__ kin, const uint32_t *__restrict__ vin, KeyT *__restrict__ kout,
                    uint32_t *__restrict__ vout, int64_t n, int shift, const uint32_t *__restrict__ hist, int nb,
                    const uint32_t *__restrict__ totals, unsigned long long *diag) {
    static_assert(RS_THREADS == RS_BINS, "one thread per digit");
    __shared__ uint32_t whist[RS_WARPS][RS_BINS];
    __shared__ uint32_t boff[RS_BINS];
    __shared__ uint32_t wsum[RS_WARPS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    {
        const int d = threadIdx.x;
        const uint32_t base = cta256_exclusive_scan(totals[d], wsum);
        boff[d] = base + hist[(int64_t)d * nb + blockIdx.x];
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) whist[w][d] = 0;
    }
    __syncthreads();
    const int64_t wbase = (int64_t)blockIdx.x * RS_TILE + (int64_t)wid * (RS_ITEMS * 32);
    const uint32_t lt_mask = (1u << lane) - 1u;
    KeyT key[RS_ITEMS];
    uint32_t val[RS_ITEMS];
    uint32_t rank[RS_ITEMS];
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int64_t i = wbase + r * 32 + lane;
        const bool ok = i < n;
        key[r] = ok ? kin[i] : (KeyT)0;
        val[r] = ok ? vin[i] : 0u;
        const uint32_t dig = (uint32_t)(key[r] >> shift) & 0xFFu;
        const uint32_t tag = ok ? dig : (0x100u | (uint32_t)lane);
        const uint32_t peers = __match_any_sync(0xffffffffu, tag);
        const uint32_t before = ok ? whist[wid][dig] : 0u;
        rank[r] = before + __popc(peers & lt_mask);
        __syncwarp();
        if (ok && (peers & lt_mask) == 0) whist[wid][dig] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) {
            const uint32_t t = whist[w][d];
            whist[w][d] = run;
            run += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int64_t i = wbase + r * 32 + lane;
        if (i < n) {
            const uint32_t dig = (uint32_t)(key[r] >> shift) & 0xFFu;
            const uint32_t dst = boff[dig] + whist[wid][dig] + rank[r];
            if (dst < n) {
                kout[dst] = key[r];
                vout[dst] = val[r];
            } else {
                atomicAdd(diag + DIAG_BAD_TREE, 1ull);
            }
        }
    }
}

// Sorts (k[0], v[0]) by the low 8 * passes bits of the keys, ping-ponging
// with (k[1], v[1]); returns the index of the pair holding the result.
// hist holds radix_hist_size(n) entries, totals RS_BINS.
template <typename KeyT>
static int radix_sort_pairs(KeyT *k[2], uint32_t *v[2], int64_t n, int passes, uint32_t *hist, uint32_t *totals,
                            unsigned long long *diag, cudaStream_t s) {
    const int nb = (int)((n + RS_TILE - 1) / RS_TILE);
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        rs_upsweep_kernel<KeyT><<<nb, RS_THREADS, 0, s>>>(k[cur], n, 8 * p, hist, nb);
        rs_rowscan_kernel<<<RS_BINS, RS_THREADS, 0, s>>>(hist, nb, totals);
        rs_downsweep_kernel<KeyT><<<nb, RS_THREADS, 0, s>>>(k[cur], v[cur], k[cur ^ 1], v[cur ^ 1], n, 8 * p, hist,
                                                            nb, totals, diag);
        cur ^= 1;
    }
    return cur;
}

}  // namespace gb
