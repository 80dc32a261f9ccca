// Stable LSD radix sort of (key, 32-bit value) pairs, 8-bit digits, shared by
// the tree build (Morton keys) and the neighbour grid (cell keys).
//
// One histogram kernel counts the digits of every pass in a single read of
// the keys.  Each pass is then one kernel: a CTA takes the next tile of 2048
// keys from a counter, ranks them stably in index order (digit ballots within
// a warp, warp offsets within the tile), stages the tile in shared memory in
// digit order (so that global writes run in contiguous digit runs),
// publishes the tile's per-digit counts and finds the counts of all earlier
// tiles by decoupled look-back
// (Merrill and Garland, "Single-pass Parallel Prefix Scan with Decoupled
// Look-back", 2016): each digit's status word of a tile holds either the
// tile's own count (flag AGG) or its inclusive prefix over tiles 0..t (flag
// PRE), and a CTA walks back until it meets a prefix.  Tiles are handed out
// in counter order, so every tile a CTA waits for belongs to a CTA that is
// already running and publishes its count without waiting itself.  Each wait
// is bounded: after RS_SPIN_LIMIT polls the CTA counts DIAG_WAIT_TIMEOUT and
// goes on with the prefix it has (its scatter still stays inside [0, n)).
#pragma once

#include <algorithm>

#include "gb_common.cuh"

namespace gb {

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;  // 2048 keys per CTA
constexpr int RS_BINS = 256;
constexpr int RS_MAX_PASSES = 8;                // 64-bit keys
constexpr int RS_COUNTERS = 32;                 // tile counters, one per pass
constexpr uint32_t RS_AGG = 1u << 30;           // status: the tile's own count
constexpr uint32_t RS_PRE = 2u << 30;           // status: inclusive prefix over tiles 0..t
constexpr uint32_t RS_VAL = RS_AGG - 1u;        // count bits (n < 2^30)
constexpr int RS_SPIN_LIMIT = 1 << 20;          // polls of one status word before a wait gives up
constexpr int RS_LOOKBACK = 8;                  // status words a look-back step reads at once

inline int64_t radix_tiles(int64_t n) { return (n + RS_TILE - 1) / RS_TILE; }

// 32-bit scratch words a sort of up to n keys needs: digit counts of every
// pass, the per-pass tile counters and two status arrays (tiles x digits),
// used by alternate passes.
inline int64_t radix_scratch_size(int64_t n) {
    return (int64_t)RS_MAX_PASSES * RS_BINS + RS_COUNTERS + 2 * (int64_t)RS_BINS * std::max<int64_t>(radix_tiles(n), 1);
}

// Keys a sort accepts (status words hold counts below 2^30).
constexpr int64_t RS_MAX_N = (int64_t)RS_VAL;

__device__ __forceinline__ uint32_t ld_relaxed_gpu(const uint32_t *p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_gpu(uint32_t *p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Decoupled look-back for digit d of tile t with count c: publishes c,
// sums the counts of tiles t-1, t-2, ... until one has published its
// inclusive prefix, publishes its own inclusive prefix and returns the
// exclusive one.  Each step reads the words of RS_LOOKBACK earlier tiles at
// once and adds them down to the first prefix or unpublished tile.  A tile
// that has not published yet is polled at most spin_limit times; then the
// wait counts DIAG_WAIT_TIMEOUT and ends with the sum it has.
__device__ __forceinline__ uint32_t rs_lookback(uint32_t *status, int t, int d, uint32_t c, int spin_limit,
                                                unsigned long long *diag) {
    uint32_t *mine = status + (int64_t)t * RS_BINS + d;
    if (t == 0) {
        st_relaxed_gpu(mine, RS_PRE | c);
        return 0u;
    }
    st_relaxed_gpu(mine, RS_AGG | c);
    uint32_t excl = 0;
    int j = t - 1;  // the next tile to add
    int spins = 0;
    while (true) {
        // RS_LOOKBACK words per round trip: tiles j, j-1, ...; below tile 0
        // reads as an empty prefix (tile 0 always publishes its prefix).
        uint32_t w[RS_LOOKBACK];
#pragma unroll
        for (int q = 0; q < RS_LOOKBACK; ++q)
            w[q] = j - q >= 0 ? ld_relaxed_gpu(status + (int64_t)(j - q) * RS_BINS + d) : RS_PRE;
        int used = 0;
        bool done = false;
#pragma unroll
        for (int q = 0; q < RS_LOOKBACK; ++q) {
            if (done || used < q || (w[q] & ~RS_VAL) == 0u) continue;  // stop at an unpublished tile
            excl += w[q] & RS_VAL;
            used = q + 1;
            done = (w[q] & RS_PRE) != 0u;
        }
        if (done) break;
        j -= used;
        if (used < RS_LOOKBACK && ++spins > spin_limit) {  // tile j has not published yet
            atomicAdd(diag + DIAG_WAIT_TIMEOUT, 1ull);
            break;
        }
    }
    st_relaxed_gpu(mine, RS_PRE | ((excl + c) & RS_VAL));
    return excl;
}

// Lanes of the warp holding the same 8-bit digit as this lane (among the
// lanes with ok set; a lane without ok matches only itself): eight ballots,
// one per digit bit.
__device__ __forceinline__ uint32_t warp_digit_peers(uint32_t dig, bool ok, int lane) {
    uint32_t m = __ballot_sync(0xffffffffu, ok);
#pragma unroll
    for (int b = 0; b < 8; ++b) {
        const bool bit = (dig >> b) & 1u;
        const uint32_t bal = __ballot_sync(0xffffffffu, bit);
        m &= bit ? bal : ~bal;
    }
    return ok ? m : (1u << lane);
}

// Digit counts of all passes: counts[p * 256 + digit] += keys with that
// digit p (bits 8p .. 8p + 7).  Warp-aggregated shared-memory counts, then
// one global add per non-zero bin and CTA.
template <typename KeyT>
__global__ void __launch_bounds__(RS_THREADS)
rs_histogram_kernel(const KeyT *__restrict__ keys, int64_t n, int passes, uint32_t *__restrict__ counts) {
    __shared__ uint32_t h[RS_MAX_PASSES * RS_BINS];
    for (int i = threadIdx.x; i < passes * RS_BINS; i += RS_THREADS) h[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const int64_t stride = (int64_t)gridDim.x * RS_THREADS;
    // Every lane of a warp runs the same number of rounds (the ballots need them all).
    for (int64_t i0 = (int64_t)blockIdx.x * RS_THREADS + (threadIdx.x & ~31); i0 < n; i0 += stride) {
        const int64_t i = i0 + lane;
        const bool ok = i < n;
        const KeyT k = ok ? keys[i] : (KeyT)0;
        for (int p = 0; p < passes; ++p) {
            const uint32_t dig = (uint32_t)(k >> (8 * p)) & 0xFFu;
            const uint32_t peers = warp_digit_peers(dig, ok, lane);
            if (ok && (peers & lt_mask) == 0) atomicAdd(&h[p * RS_BINS + dig], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * RS_BINS; i += RS_THREADS) {
        const uint32_t c = h[i];
        if (c) atomicAdd(counts + i, c);
    }
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

// One pass: stable scatter of the tile the CTA takes from *counter.  Keys
// of a tile are ranked in index order (warp, round, lane) among equal
// digits; the destination is the digit's global start (scan of this pass's
// counts) + the digit's count in earlier tiles (look-back) + the rank within
// the tile.  status holds this pass's tile words (zeroed); status_next, when
// given, is zeroed here for the next pass.
template <typename KeyT>
__global__ void __launch_bounds__(RS_THREADS, 4)
rs_onesweep_kernel(const KeyT *__restrict__ kin, const uint32_t *__restrict__ vin, KeyT *__restrict__ kout,
                   uint32_t *__restrict__ vout, int64_t n, int shift, const uint32_t *__restrict__ counts,
                   uint32_t *counter, uint32_t *status, uint32_t *status_next, int nb,
                   unsigned long long *diag) {
    static_assert(RS_THREADS == RS_BINS, "one thread per digit");
    __shared__ uint32_t whist[RS_WARPS][RS_BINS];
    __shared__ uint32_t boff[RS_BINS];
    __shared__ uint32_t wsum[RS_WARPS];
    __shared__ int tile_s;
    __shared__ uint32_t wsum2[RS_WARPS];
    __shared__ uint32_t tst[RS_BINS];
    __shared__ KeyT skey[RS_TILE];  // the tile in digit order
    __shared__ uint32_t sval[RS_TILE];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, d = threadIdx.x;
    if (status_next) {
        for (int64_t i = (int64_t)blockIdx.x * RS_THREADS + threadIdx.x; i < (int64_t)nb * RS_BINS;
             i += (int64_t)gridDim.x * RS_THREADS)
            status_next[i] = 0u;
    }
    if (threadIdx.x == 0) tile_s = (int)atomicAdd(counter, 1u);
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) whist[w][d] = 0;
    __syncthreads();
    const int t = tile_s;
    const int64_t wbase = (int64_t)t * RS_TILE + (int64_t)wid * (RS_ITEMS * 32);
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
        const uint32_t peers = warp_digit_peers(dig, ok, lane);
        const uint32_t before = ok ? whist[wid][dig] : 0u;
        rank[r] = before + __popc(peers & lt_mask);
        __syncwarp();
        if (ok && (peers & lt_mask) == 0) whist[wid][dig] = before + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // Thread d: warp offsets of digit d within the tile, and its tile count.
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
        const uint32_t x = whist[w][d];
        whist[w][d] = c;
        c += x;
    }
    const uint32_t excl = rs_lookback(status, t, d, c, RS_SPIN_LIMIT, diag);
    // Digit d's first position in the tile; the tile's keys are staged in
    // shared memory in digit order, and position p of the staged tile goes
    // to boff[digit] + p (mod 2^32), so consecutive threads write
    // consecutive addresses within each digit's run.
    const uint32_t tstart = cta256_exclusive_scan(c, wsum2);
    tst[d] = tstart;
    boff[d] = cta256_exclusive_scan(counts[d], wsum) + excl - tstart;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int64_t i = wbase + r * 32 + lane;
        if (i < n) {
            const uint32_t dig = (uint32_t)(key[r] >> shift) & 0xFFu;
            const uint32_t q = tst[dig] + whist[wid][dig] + rank[r];  // < RS_TILE for a consistent count
            if (q < (uint32_t)RS_TILE) {
                skey[q] = key[r];
                sval[q] = val[r];
            }
        }
    }
    __syncthreads();
    const int64_t left = n - (int64_t)t * RS_TILE;
    const int cnt = left < (int64_t)RS_TILE ? (int)left : RS_TILE;
    for (int q = threadIdx.x; q < cnt; q += RS_THREADS) {
        const KeyT k = skey[q];
        const uint32_t dst = boff[(uint32_t)(k >> shift) & 0xFFu] + (uint32_t)q;
        if (dst < n) {
            kout[dst] = k;
            vout[dst] = sval[q];
        } else {
            atomicAdd(diag + DIAG_BAD_TREE, 1ull);
        }
    }
}

// Sorts (k[0], v[0]) by the low 8 * passes bits of the keys (n < 2^30,
// passes <= 8), ping-ponging with (k[1], v[1]); returns the index of the
// pair holding the result.  scratch holds radix_scratch_size(n) words.
// Launches: one memset, the histogram kernel and one kernel per pass.
template <typename KeyT>
static int radix_sort_pairs(KeyT *k[2], uint32_t *v[2], int64_t n, int passes, uint32_t *scratch,
                            unsigned long long *diag, cudaStream_t s) {
    if (n <= 0 || passes <= 0) return 0;
    const int nb = (int)radix_tiles(n);
    uint32_t *counts = scratch;
    uint32_t *counters = counts + RS_MAX_PASSES * RS_BINS;
    uint32_t *status[2] = {counters + RS_COUNTERS, counters + RS_COUNTERS + (int64_t)nb * RS_BINS};
    cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * ((int64_t)RS_MAX_PASSES * RS_BINS + RS_COUNTERS + (int64_t)nb * RS_BINS),
                    s);
    const int hb = (int)std::min<int64_t>((n + RS_THREADS - 1) / RS_THREADS, 4 * (int64_t)num_sms());
    rs_histogram_kernel<KeyT><<<hb, RS_THREADS, 0, s>>>(k[0], n, passes, counts);
    int cur = 0;
    for (int p = 0; p < passes; ++p) {
        uint32_t *next = p + 1 < passes ? status[(p + 1) & 1] : nullptr;
        rs_onesweep_kernel<KeyT><<<nb, RS_THREADS, 0, s>>>(k[cur], v[cur], k[cur ^ 1], v[cur ^ 1], n, 8 * p,
                                                           counts + p * RS_BINS, counters + p, status[p & 1], next,
                                                           nb, diag);
        cur ^= 1;
    }
    return cur;
}

}  // namespace gb
