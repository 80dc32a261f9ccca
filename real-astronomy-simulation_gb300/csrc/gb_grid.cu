// Uniform neighbour grid over the gas particles, rebuilt on the device:
// NeighborGrid.rebuild / rebuild_all (core/solvers/neighbor_grid.py:49-136),
// which the reference runs in host numpy before uploading gsort and
// cell_start.  Same outputs, bit for bit:
//   cell   = max(2 h_max, min_radius) (1 if not > 1e-9), grown by 1.3 while
//            the grid has more than max_cells = max(64, 4n) cells;
//   dims   = max(floor((max - min) / cell) + 1, 1) per axis;
//   ijk    = clip(trunc((x - min) / cell), 0, dims - 1), all in FP64;
//   flat   = (i dims_y + j) dims_z + k;
//   gsort  = gas indices in stable order of flat, zero-padded to n;
//   cell_start[c] = number of gas particles with flat < c for c <= n_cells,
//            zero above.
// Stages (one stream, no host round trip):
//   1 grid_reduce_kernel  gas count, bounding box and h_max (block partials,
//                         merged by the last CTA, which also derives the
//                         geometry in FP64);
//   2 grid_key_kernel     cell key per particle; stars (and every particle
//                         when there is no gas) get a key that sorts last;
//   3 radix sort          stable, 8-bit digits, enough passes for max_cells;
//   4 grid_gsort_kernel / grid_start_kernel: outputs (skipped when there is
//                         no gas, which leaves them as the reference does).
#include <algorithm>
#include <climits>
#include <cmath>

#include "gb_common.cuh"
#include "gb_sort.cuh"

namespace gb {

constexpr int GRID_THREADS = 256;
constexpr int GRID_MAX_GROW = 4096;  // bound on the cell-growth loop

// Geometry of the last rebuild (device-resident; copied to gb_grid_info_t).
struct GridGeom {
    long long ngas, n_cells;
    int nx, ny, nz, status;  // status: 0 ok, 1 non-finite input, 2 growth loop did not converge
    double lo[3], cell, inv_cell;
    int active;              // this rebuild writes the outputs (ngas > 0)
};

struct GridPart {
    float mn[3], mx[3], hmax;
    unsigned long long count, nonfinite;
};

// numpy's float64 -> int64 cast on x86-64: truncation, and the "integer
// indefinite" value INT64_MIN for NaN and out-of-range inputs.
__device__ __forceinline__ long long np_trunc_i64(double t) {
    if (!(t < 9.2233720368547758e18 && t > -9.2233720368547758e18)) return (long long)(-9223372036854775807ll - 1);
    return __double2ll_rz(t);
}

__global__ void __launch_bounds__(GRID_THREADS)
grid_reduce_kernel(const float4 *__restrict__ xm, const float *__restrict__ hsml, const int *__restrict__ is_star,
                   int64_t n, double min_radius, long long max_cells, GridPart *part, unsigned *ticket,
                   GridGeom *geom) {
    float mn0 = INFINITY, mn1 = INFINITY, mn2 = INFINITY, mx0 = -INFINITY, mx1 = -INFINITY, mx2 = -INFINITY;
    float hm = -INFINITY;
    unsigned long long cnt = 0, bad = 0;
    for (int64_t i = (int64_t)blockIdx.x * GRID_THREADS + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * GRID_THREADS) {
        if (is_star && __ldg(is_star + i) != 0) continue;
        const float4 p = __ldg(xm + i);
        const float hv = __ldg(hsml + i);
        if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z) && isfinite(hv))) ++bad;
        mn0 = fminf(mn0, p.x); mn1 = fminf(mn1, p.y); mn2 = fminf(mn2, p.z);
        mx0 = fmaxf(mx0, p.x); mx1 = fmaxf(mx1, p.y); mx2 = fmaxf(mx2, p.z);
        hm = fmaxf(hm, hv);
        ++cnt;
    }
    __shared__ float sm[7][GRID_THREADS / 32];
    __shared__ unsigned long long sc[2][GRID_THREADS / 32];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn0 = fminf(mn0, __shfl_xor_sync(0xffffffffu, mn0, o));
        mn1 = fminf(mn1, __shfl_xor_sync(0xffffffffu, mn1, o));
        mn2 = fminf(mn2, __shfl_xor_sync(0xffffffffu, mn2, o));
        mx0 = fmaxf(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
        mx1 = fmaxf(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
        mx2 = fmaxf(mx2, __shfl_xor_sync(0xffffffffu, mx2, o));
        hm = fmaxf(hm, __shfl_xor_sync(0xffffffffu, hm, o));
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    if (lane == 0) {
        sm[0][wid] = mn0; sm[1][wid] = mn1; sm[2][wid] = mn2;
        sm[3][wid] = mx0; sm[4][wid] = mx1; sm[5][wid] = mx2; sm[6][wid] = hm;
        sc[0][wid] = cnt; sc[1][wid] = bad;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        GridPart bp;
        for (int a = 0; a < 3; ++a) {
            bp.mn[a] = INFINITY;
            bp.mx[a] = -INFINITY;
        }
        bp.hmax = -INFINITY;
        bp.count = bp.nonfinite = 0;
        for (int w = 0; w < GRID_THREADS / 32; ++w) {
            for (int a = 0; a < 3; ++a) {
                bp.mn[a] = fminf(bp.mn[a], sm[a][w]);
                bp.mx[a] = fmaxf(bp.mx[a], sm[3 + a][w]);
            }
            bp.hmax = fmaxf(bp.hmax, sm[6][w]);
            bp.count += sc[0][w];
            bp.nonfinite += sc[1][w];
        }
        part[blockIdx.x] = bp;
        __threadfence();
        const unsigned t = atomicAdd(ticket, 1u);
        last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!last || threadIdx.x != 0) return;
    // Last CTA: merge the block partials in block order and derive the grid.
    __threadfence();
    *ticket = 0;  // ready for the next rebuild (stream-ordered)
    float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY}, hmax = -INFINITY;
    unsigned long long count = 0, nonfinite = 0;
    for (unsigned b = 0; b < gridDim.x; ++b) {
        const GridPart *q = part + b;  // written by other CTAs: read past L1
        for (int a = 0; a < 3; ++a) {
            mn[a] = fminf(mn[a], __ldcg(q->mn + a));
            mx[a] = fmaxf(mx[a], __ldcg(q->mx + a));
        }
        hmax = fmaxf(hmax, __ldcg(&q->hmax));
        count += __ldcg(&q->count);
        nonfinite += __ldcg(&q->nonfinite);
    }
    GridGeom g = *geom;  // a rebuild without gas keeps the previous geometry
    g.ngas = (long long)count;
    g.active = count > 0 ? 1 : 0;
    g.status = nonfinite ? 1 : 0;
    if (count > 0) {
        double cell = fmax(__dmul_rn(2.0, (double)hmax), min_radius);
        cell = cell > 1e-9 ? cell : 1.0;
        double lo[3], span[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = (double)mn[a];
            span[a] = __dsub_rn((double)mx[a], lo[a]);
        }
        long long dims[3];
        auto set_dims = [&]() {
            for (int a = 0; a < 3; ++a) {
                const long long f = np_trunc_i64(floor(__ddiv_rn(span[a], cell)));
                dims[a] = (f != LLONG_MIN && f + 1 > 1) ? f + 1 : 1;
            }
        };
        set_dims();
        int grow = 0;
        // Products past 2^53 are inexact in FP64 but far above max_cells.
        while ((double)dims[0] * (double)dims[1] * (double)dims[2] > (double)max_cells) {
            if (++grow > GRID_MAX_GROW) {
                g.status = 2;
                break;
            }
            cell = __dmul_rn(cell, 1.3);
            set_dims();
        }
        if (g.status == 2) {
            g.active = 0;
        } else {
            g.nx = (int)dims[0];
            g.ny = (int)dims[1];
            g.nz = (int)dims[2];
            g.n_cells = dims[0] * dims[1] * dims[2];
            for (int a = 0; a < 3; ++a) g.lo[a] = lo[a];
            g.cell = cell;
            g.inv_cell = __ddiv_rn(1.0, cell);
        }
    }
    *geom = g;
}

// Cell key of every particle; stars and inactive rebuilds get n_cells (or
// 0), which sorts after every gas key.
__global__ void grid_key_kernel(const float4 *__restrict__ xm, const int *__restrict__ is_star, int64_t n,
                                const GridGeom *__restrict__ geom, uint32_t *keys, uint32_t *vals) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GridGeom &g = *geom;
    uint32_t key = 0;
    if (g.active) {
        key = (uint32_t)g.n_cells;
        if (!(is_star && __ldg(is_star + i) != 0)) {
            const float4 p = __ldg(xm + i);
            const float c[3] = {p.x, p.y, p.z};
            const long long dm[3] = {g.nx, g.ny, g.nz};
            long long q[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const double t = __ddiv_rn(__dsub_rn((double)c[a], g.lo[a]), g.cell);
                long long v = np_trunc_i64(t);
                v = v < 0 ? 0 : (v > dm[a] - 1 ? dm[a] - 1 : v);
                q[a] = v;
            }
            key = (uint32_t)((q[0] * dm[1] + q[1]) * dm[2] + q[2]);
        }
    }
    keys[i] = key;
    vals[i] = (uint32_t)i;
}

__global__ void grid_gsort_kernel(const uint32_t *__restrict__ vals, int64_t n, const GridGeom *__restrict__ geom,
                                  int *gsort) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n || !geom->active) return;
    gsort[p] = p < geom->ngas ? (int)vals[p] : 0;
}

// cell_start[c] = lower bound of c in the sorted gas keys (c <= n_cells);
// 0 above n_cells, as the reference re-zeroes its field each rebuild.
__global__ void grid_start_kernel(const uint32_t *__restrict__ keys, const GridGeom *__restrict__ geom,
                                  long long max_cells, int *cell_start) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c > max_cells || !geom->active) return;
    const long long nc = geom->n_cells, ng = geom->ngas;
    int out = 0;
    if (c <= nc) {
        long long lo = 0, hi = ng;  // first index in [0, ngas) with key >= c
        while (lo < hi) {
            const long long mid = (lo + hi) >> 1;
            if ((long long)__ldg(keys + mid) < c) lo = mid + 1;
            else hi = mid;
        }
        out = (int)lo;
    }
    cell_start[c] = out;
}

}  // namespace gb

using namespace gb;

struct gb_grid {
    int device;
    int64_t n;
    long long max_cells;
    double min_radius;
    int passes, red_blocks;
    uint32_t *keys[2], *vals[2], *sort_scratch;
    unsigned long long timeouts_seen;  // DIAG_WAIT_TIMEOUT at the last rebuild with info
    GridPart *part;
    unsigned *ticket;
    GridGeom *geom;
    unsigned long long *diag;
    uint64_t launches;
};

extern "C" int gb_grid_destroy(gb_grid_t *h) {
    if (!h) return GB_OK;
    void *ptrs[] = {h->keys[0], h->keys[1], h->vals[0], h->vals[1], h->sort_scratch, h->part, h->ticket,
                    h->geom, h->diag};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    delete h;
    return GB_OK;
}

extern "C" int gb_grid_create(gb_grid_t **out, int64_t n, double min_radius) {
    if (!out) return fail(GB_EINVAL, "out is NULL");
    *out = nullptr;
    if (n < 0 || n > ((int64_t)1 << 29)) return fail(GB_EINVAL, "n=%lld out of range", (long long)n);
    if (!(min_radius >= 0.0) || !std::isfinite(min_radius)) return fail(GB_EINVAL, "min_radius must be finite and >= 0");
    gb_grid_t *h = new gb_grid();
    GB_CUDA_TRY(cudaGetDevice(&h->device));
    h->n = n;
    h->max_cells = std::max<long long>(64, 4 * (long long)n);
    h->min_radius = min_radius;
    int bits = 1;
    while (bits < 32 && (1ll << bits) <= h->max_cells) ++bits;  // keys <= max_cells
    h->passes = (bits + 7) / 8;
    const int64_t nn = std::max<int64_t>(n, 1);
    h->red_blocks = std::max(1, std::min(num_sms() * 4, (int)((nn + GRID_THREADS - 1) / GRID_THREADS)));
    bool ok = true;
    auto A = [&](void **p, size_t bytes) {
        if (ok && cudaMalloc(p, bytes) != cudaSuccess) ok = false;
    };
    A((void **)&h->keys[0], sizeof(uint32_t) * nn);
    A((void **)&h->keys[1], sizeof(uint32_t) * nn);
    A((void **)&h->vals[0], sizeof(uint32_t) * nn);
    A((void **)&h->vals[1], sizeof(uint32_t) * nn);
    A((void **)&h->sort_scratch, sizeof(uint32_t) * radix_scratch_size(nn));
    A((void **)&h->part, sizeof(GridPart) * h->red_blocks);
    A((void **)&h->ticket, sizeof(unsigned));
    A((void **)&h->geom, sizeof(GridGeom));
    A((void **)&h->diag, sizeof(unsigned long long) * DIAG_COUNT);
    if (!ok) {
        gb_grid_destroy(h);
        return fail(GB_ENOMEM, "gb_grid_create: device allocation failed for n=%lld", (long long)n);
    }
    GridGeom g0 = {};
    g0.nx = g0.ny = g0.nz = 1;
    g0.cell = g0.inv_cell = 1.0;
    if (cudaMemset(h->ticket, 0, sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(h->diag, 0, sizeof(unsigned long long) * DIAG_COUNT) != cudaSuccess ||
        cudaMemcpy(h->geom, &g0, sizeof(GridGeom), cudaMemcpyHostToDevice) != cudaSuccess) {
        gb_grid_destroy(h);
        return fail(GB_ECUDA, "gb_grid_create: initialisation failed");
    }
    *out = h;
    return GB_OK;
}

extern "C" int64_t gb_grid_max_cells(gb_grid_t *h) { return h ? (int64_t)h->max_cells : -1; }

extern "C" int gb_grid_rebuild(gb_grid_t *h, const float *xm, const float *hsml, const int32_t *is_star,
                               int32_t *gsort, int32_t *cell_start, gb_grid_info_t *info, void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n = h->n;
    if (n > 0) {
        if (!xm || !aligned16(xm)) return fail(GB_EINVAL, "xm is NULL or not 16-byte aligned");
        if (!hsml) return fail(GB_EINVAL, "hsml is NULL");
        if (!gsort || !cell_start) return fail(GB_EINVAL, "gsort and cell_start must not be NULL");
        const int nblk = std::max(1, std::min(h->red_blocks, (int)((n + GRID_THREADS - 1) / GRID_THREADS)));
        grid_reduce_kernel<<<nblk, GRID_THREADS, 0, s>>>((const float4 *)xm, hsml, is_star, n, h->min_radius,
                                                        h->max_cells, h->part, h->ticket, h->geom);
        const unsigned g = (unsigned)((n + GRID_THREADS - 1) / GRID_THREADS);
        grid_key_kernel<<<g, GRID_THREADS, 0, s>>>((const float4 *)xm, is_star, n, h->geom, h->keys[0],
                                                   h->vals[0]);
        const int cur = radix_sort_pairs<uint32_t>(h->keys, h->vals, n, h->passes, h->sort_scratch, h->diag, s);
        grid_gsort_kernel<<<g, GRID_THREADS, 0, s>>>(h->vals[cur], n, h->geom, gsort);
        const unsigned gc = (unsigned)((h->max_cells + 1 + GRID_THREADS - 1) / GRID_THREADS);
        grid_start_kernel<<<gc, GRID_THREADS, 0, s>>>(h->keys[cur], h->geom, h->max_cells, cell_start);
        GB_CUDA_TRY(cudaGetLastError());
        h->launches += 4 + 1 + h->passes;
    }
    if (info) {
        GridGeom g;
        GB_CUDA_TRY(cudaMemcpyAsync(&g, h->geom, sizeof(GridGeom), cudaMemcpyDeviceToHost, s));
        GB_CUDA_TRY(cudaStreamSynchronize(s));
        if (n == 0) g.ngas = 0;
        info->ngas = g.ngas;
        info->n_cells = g.n_cells;
        info->nx = g.nx;
        info->ny = g.ny;
        info->nz = g.nz;
        info->status = g.status;
        for (int a = 0; a < 3; ++a) info->lo[a] = g.lo[a];
        info->cell = g.cell;
        info->inv_cell = g.inv_cell;
        if (g.status == 1) return fail(GB_EINVAL, "gb_grid_rebuild: non-finite gas position or smoothing length");
        if (g.status == 2) return fail(GB_EINVAL, "gb_grid_rebuild: cell growth did not converge");
        unsigned long long to = 0;
        GB_CUDA_TRY(cudaMemcpy(&to, h->diag + DIAG_WAIT_TIMEOUT, sizeof(to), cudaMemcpyDeviceToHost));
        const unsigned long long inc = to - h->timeouts_seen;
        h->timeouts_seen = to;
        if (inc) return fail(GB_ETIMEOUT, "gb_grid_rebuild: %llu bounded device waits expired (radix sort)", inc);
    }
    return GB_OK;
}

extern "C" uint64_t gb_grid_launch_count(gb_grid_t *h) { return h ? h->launches : 0; }
