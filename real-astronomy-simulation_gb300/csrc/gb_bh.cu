// LBVH Barnes-Hut on the GB300 (sm_103a): every stage on the device.
//
// Replaces BarnesHut.compute (core/solvers/barnes_hut.py:242-259), which runs
// Morton keys and the stable sort on the host in numpy and the tree kernels
// in Taichi.  Stages (one CUDA graph per step when driven by gb_bh_kdk):
//   0 bbox      per-axis min/max (optionally after the fused kick+drift),
//               last-CTA-done combine -> FP64 quantisation parameters
//   1 morton    keys bit-identical to morton_codes (:27-46): FP64
//               (x - lo) * scale with separate roundings, clip, truncate,
//               interleave x,y,z into bits 3b, 3b+1, 3b+2
//   2 sort      stable LSD radix sort (8-bit digits) of (key, index): the
//               permutation of np.argsort(kind="stable") (:247)
//   3 gather    particles into key order (leaf records)
//   4 karras    binary radix tree, identical to _build_radix (:84-121)
//   5 bottom-up node mass, first moment and AABB (FP32); a node is
//               summarised by the second of its two children to finish
//               (integer arrival ticket with acquire-release ordering, L2
//               reads): no floating-point atomics, and the result is
//               independent of scheduling (:124-177 use FP64 atomics on
//               every ancestor instead)
//   6 traverse  warp-coherent walk: 32 key-consecutive targets share one
//               shared-memory stack of (node, lane mask); every lane applies
//               the reference's own acceptance test size^2 < theta^2 (r^2 +
//               eps^2) (:204-210), so each particle accepts exactly the node
//               set of _traverse (:180-217); a per-lane count reproduces the
//               max_stack rule (:212) and the skipped pushes are counted
//               instead of being lost silently.  Closing kick fused in the
//               epilogue for KDK steps.
#include <algorithm>
#include <cstdio>

#include "gb_common.cuh"
#include "gb_sort.cuh"

namespace gb {

struct BHParams {
    double lo[3];
    double scale;
};



constexpr int BBOX_THREADS = 256;
constexpr int BU_THREADS = 64;   // bottom-up CTA (a CTA retires with its longest ancestor chain)
constexpr int MAX_DEPTH = 128;

// ------------------------------------------------------------------ bbox
template <bool KDK>
__global__ void __launch_bounds__(BBOX_THREADS)
bh_bbox_kernel(float4 *xm, float4 *vel, const float4 *acc, int64_t n, float h, float dt, float4 *part,
               unsigned *ticket, BHParams *prm, int bits, unsigned long long *diag) {
    float mn0 = INFINITY, mn1 = INFINITY, mn2 = INFINITY;
    float mx0 = -INFINITY, mx1 = -INFINITY, mx2 = -INFINITY;
    unsigned long long bad = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float4 x = xm[i];
        if (KDK) {
            const float4 v = vel[i], a = acc[i];
            const float vx = kick(v.x, a.x, h), vy = kick(v.y, a.y, h), vz = kick(v.z, a.z, h);
            x = make_float4(drift(x.x, vx, dt), drift(x.y, vy, dt), drift(x.z, vz, dt), x.w);
            xm[i] = x;
            vel[i] = make_float4(vx, vy, vz, v.w);
        }
        if (isfinite(x.x) && isfinite(x.y) && isfinite(x.z)) {
            mn0 = fminf(mn0, x.x); mn1 = fminf(mn1, x.y); mn2 = fminf(mn2, x.z);
            mx0 = fmaxf(mx0, x.x); mx1 = fmaxf(mx1, x.y); mx2 = fmaxf(mx2, x.z);
        } else {
            ++bad;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mn0 = fminf(mn0, __shfl_xor_sync(0xffffffffu, mn0, o));
        mn1 = fminf(mn1, __shfl_xor_sync(0xffffffffu, mn1, o));
        mn2 = fminf(mn2, __shfl_xor_sync(0xffffffffu, mn2, o));
        mx0 = fmaxf(mx0, __shfl_xor_sync(0xffffffffu, mx0, o));
        mx1 = fmaxf(mx1, __shfl_xor_sync(0xffffffffu, mx1, o));
        mx2 = fmaxf(mx2, __shfl_xor_sync(0xffffffffu, mx2, o));
        bad += __shfl_xor_sync(0xffffffffu, bad, o);
    }
    __shared__ float4 smn[BBOX_THREADS / 32], smx[BBOX_THREADS / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        smn[wid] = make_float4(mn0, mn1, mn2, 0.f);
        smx[wid] = make_float4(mx0, mx1, mx2, 0.f);
        if (bad) atomicAdd(diag + DIAG_NONFINITE, bad);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float4 a = smn[0], b = smx[0];
        for (int w = 1; w < BBOX_THREADS / 32; ++w) {
            a.x = fminf(a.x, smn[w].x); a.y = fminf(a.y, smn[w].y); a.z = fminf(a.z, smn[w].z);
            b.x = fmaxf(b.x, smx[w].x); b.y = fmaxf(b.y, smx[w].y); b.z = fmaxf(b.z, smx[w].z);
        }
        part[2 * blockIdx.x] = a;
        part[2 * blockIdx.x + 1] = b;
        __threadfence();
        is_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!is_last) return;
    // Last CTA: merge every CTA's partial with all its threads (strided L2
    // reads, then the same warp/CTA reduction).
    __threadfence();
    float4 a = make_float4(INFINITY, INFINITY, INFINITY, 0.f), b = make_float4(-INFINITY, -INFINITY, -INFINITY, 0.f);
    for (unsigned k = threadIdx.x; k < gridDim.x; k += BBOX_THREADS) {
        const float4 c = __ldcg(part + 2 * k), d = __ldcg(part + 2 * k + 1);
        a.x = fminf(a.x, c.x); a.y = fminf(a.y, c.y); a.z = fminf(a.z, c.z);
        b.x = fmaxf(b.x, d.x); b.y = fmaxf(b.y, d.y); b.z = fmaxf(b.z, d.z);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a.x = fminf(a.x, __shfl_xor_sync(0xffffffffu, a.x, o));
        a.y = fminf(a.y, __shfl_xor_sync(0xffffffffu, a.y, o));
        a.z = fminf(a.z, __shfl_xor_sync(0xffffffffu, a.z, o));
        b.x = fmaxf(b.x, __shfl_xor_sync(0xffffffffu, b.x, o));
        b.y = fmaxf(b.y, __shfl_xor_sync(0xffffffffu, b.y, o));
        b.z = fmaxf(b.z, __shfl_xor_sync(0xffffffffu, b.z, o));
    }
    __syncthreads();  // smn/smx reused
    if (lane == 0) {
        smn[wid] = a;
        smx[wid] = b;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    a = smn[0];
    b = smx[0];
    for (int w = 1; w < BBOX_THREADS / 32; ++w) {
        a.x = fminf(a.x, smn[w].x); a.y = fminf(a.y, smn[w].y); a.z = fminf(a.z, smn[w].z);
        b.x = fmaxf(b.x, smx[w].x); b.y = fmaxf(b.y, smx[w].y); b.z = fmaxf(b.z, smx[w].z);
    }
    // span = largest per-axis extent (:41); 1.0 when not > 0 (:42).
    const double lo0 = a.x, lo1 = a.y, lo2 = a.z;
    double span = __dsub_rn((double)b.x, lo0);
    span = fmax(span, __dsub_rn((double)b.y, lo1));
    span = fmax(span, __dsub_rn((double)b.z, lo2));
    if (!(span > 0.0)) span = 1.0;
    const double qmax = (double)((1ull << bits) - 1ull);
    prm->lo[0] = lo0;
    prm->lo[1] = lo1;
    prm->lo[2] = lo2;
    prm->scale = __ddiv_rn(qmax, __dmul_rn(span, 1.0000001));
    *ticket = 0u;
}

// ---------------------------------------------------------------- morton
template <int BITS>
__device__ __forceinline__ uint64_t interleave3(uint32_t x, uint32_t y, uint32_t z) {
    uint64_t r = 0;
#pragma unroll
    for (int b = 0; b < BITS; ++b) {
        const uint64_t t = ((x >> b) & 1u) | (((y >> b) & 1u) << 1) | (((z >> b) & 1u) << 2);
        r |= t << (3 * b);
    }
    return r;
}

__device__ __forceinline__ uint32_t quantise(float x, double lo, double scale, double qmax) {
    double t = __dmul_rn(__dsub_rn((double)x, lo), scale);
    t = t > qmax ? qmax : t;
    t = t >= 0.0 ? t : 0.0;  // also maps NaN to 0 (counted in the bbox pass)
    return __double2uint_rz(t);
}

template <typename KeyT, int BITS>
__global__ void bh_morton_kernel(const float4 *__restrict__ xm, int64_t n, const BHParams *__restrict__ prm,
                                 KeyT *__restrict__ keys, uint32_t *__restrict__ vals) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double qmax = (double)((1ull << BITS) - 1ull);
    const double sc = prm->scale;
    const float4 x = xm[i];
    const uint32_t qx = quantise(x.x, prm->lo[0], sc, qmax);
    const uint32_t qy = quantise(x.y, prm->lo[1], sc, qmax);
    const uint32_t qz = quantise(x.z, prm->lo[2], sc, qmax);
    keys[i] = (KeyT)interleave3<BITS>(qx, qy, qz);
    vals[i] = (uint32_t)i;
}

// ----------------------------------------------------------------- gather
__global__ void bh_gather_kernel(const float4 *__restrict__ xm, const uint32_t *__restrict__ order, int64_t n,
                                 float4 *__restrict__ leaf, unsigned long long *diag) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = order[i];
    if (o < n) {
        leaf[i] = __ldg(xm + o);
    } else {
        leaf[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        atomicAdd(diag + DIAG_BAD_TREE, 1ull);
    }
}

// ----------------------------------------------------------------- karras
// Common-prefix length of keys i and j over bits 62..0; equal keys continue
// with the index bits 30..0 (63 + prefix); -1 outside [0, n) (:71-81).
__device__ __forceinline__ int clz63(uint64_t x) { return __clzll(x) - 1; }
__device__ __forceinline__ int clz63(uint32_t x) { return __clz(x) + 31; }

template <typename KeyT>
__device__ __forceinline__ int kdelta(const KeyT *__restrict__ k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    const KeyT x = __ldg(k + i) ^ __ldg(k + j);
    if (x == 0) return 63 + (__clz(i ^ j) - 1);
    return clz63(x);
}

// Leaves per group of the group walk (traversal shape 3).
constexpr int GW_GROUP = 32;

// gsize (when not NULL, zeroed before the launch): the group walk's groups,
// the maximal subtrees with at most GW_GROUP leaves; gsize[first leaf] =
// its leaf count.  They partition the leaves into key-order ranges, each
// inside one node's box (32 key-consecutive leaves can straddle a jump of
// the Morton curve and span most of the system).
template <typename KeyT>
__global__ void bh_karras_kernel(const KeyT *__restrict__ k, int n, int2 *__restrict__ child,
                                 int *__restrict__ parent, int *__restrict__ gsize) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) parent[n] = -1;  // the root (internal node 0 = id n)
    if (i >= n - 1) return;
    const int d = kdelta(k, n, i, i + 1) > kdelta(k, n, i, i - 1) ? 1 : -1;
    const int d_min = kdelta(k, n, i, i - d);
    int l_max = 2;
    while (kdelta(k, n, i, i + l_max * d) > d_min) l_max *= 2;
    int l = 0;
    for (int t = l_max / 2; t >= 1; t /= 2)
        if (kdelta(k, n, i, i + (l + t) * d) > d_min) l += t;
    const int j = i + l * d;
    const int d_node = kdelta(k, n, i, j);
    int s = 0;
    int t2 = (l + 1) / 2;
    while (t2 >= 1) {
        if (kdelta(k, n, i, i + (s + t2) * d) > d_node) s += t2;
        t2 = t2 > 1 ? (t2 + 1) / 2 : 0;
    }
    const int gamma = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int lc = (lo == gamma) ? gamma : gamma + n;
    const int rc = (hi == gamma + 1) ? gamma + 1 : gamma + 1 + n;
    child[i] = make_int2(lc, rc);
    parent[lc] = i + n;
    parent[rc] = i + n;
    if (gsize) {
        const int cnt = hi - lo + 1, cl = gamma - lo + 1, cr = hi - gamma;
        if (cnt > GW_GROUP) {
            if (cl <= GW_GROUP) gsize[lo] = cl;
            if (cr <= GW_GROUP) gsize[gamma + 1] = cr;
        } else if (i == 0) {
            gsize[0] = cnt;  // the whole system is one group
        }
    }
}

// -------------------------------------------------------------- bottom-up
// Node summary in FP32: mass, first moment about the node's AABB minimum
// corner, and the AABB.  Moments about the corner keep the centre of mass
// accurate to rounding of the node size (a cluster of coincident particles
// gets its exact position); the reference keeps FP64 moments about the
// origin (core/solvers/barnes_hut.py:143-177).
struct NodeSum {
    float m, sx, sy, sz;    // mass, moment about (lx, ly, lz)
    float lx, ly, lz, hx, hy, hz;
};

__device__ __forceinline__ NodeSum child_sum(int c, int n, const float4 *__restrict__ leaf,
                                             const float4 *__restrict__ sums, const float4 *__restrict__ bmin,
                                             const float4 *__restrict__ bmax) {
    NodeSum s;
    if (c < n) {
        const float4 p = __ldg(leaf + c);
        s.m = p.w;
        s.sx = s.sy = s.sz = 0.f;
        s.lx = s.hx = p.x;
        s.ly = s.hy = p.y;
        s.lz = s.hz = p.z;
    } else {
        const int k = c - n;
        const float4 q = __ldcg(sums + k), a = __ldcg(bmin + k), b = __ldcg(bmax + k);
        s.m = q.x; s.sx = q.y; s.sy = q.z; s.sz = q.w;
        s.lx = a.x; s.ly = a.y; s.lz = a.z;
        s.hx = b.x; s.hy = b.y; s.hz = b.z;
    }
    return s;
}

// Centre of mass and mass; a node without mass keeps a zero centre, like the
// freshly allocated com field of the reference.
__device__ __forceinline__ float4 trav_com(const NodeSum &s) {
    if (!(s.m > 0.f)) return make_float4(0.f, 0.f, 0.f, 0.f);
    return make_float4(s.lx + __fdiv_rn(s.sx, s.m), s.ly + __fdiv_rn(s.sy, s.m), s.lz + __fdiv_rn(s.sz, s.m), s.m);
}

// Squared largest AABB extent (:207).
__device__ __forceinline__ float size2_of(const NodeSum &s) {
    const float e = fmaxf(fmaxf(s.hx - s.lx, s.hy - s.ly), s.hz - s.lz);
    return e * e;
}

// Arrival ticket with acquire-release ordering at GPU scope: the first child
// to finish publishes its summary; the second observes it.
__device__ __forceinline__ unsigned arrive(unsigned *p) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(p) : "memory");
    return old;
}

// True for the second child to arrive.  A sibling that already arrived is
// seen by an acquire load, which synchronises with its release and needs no
// fence of the caller's own stores: those are released by the atomic at the
// first node where the caller arrives first, the only place it stops.
__device__ __forceinline__ bool second_arrival(unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v != 0u || arrive(p) != 0u;
}

// Summarises every internal node k once both children are done and writes
// the traversal record of its two children as (left, right) pairs:
//   inode[3k] = {x_L, x_R, y_L, y_R}, inode[3k+1] = {z_L, z_R, m_L, m_R},
//   inode[3k+2] = {size2_L, size2_R, id_L, id_R} (ids as bits; size2 = -1
//   marks a leaf child), so the traversal loads both children pre-packed for
//   .f32x2 arithmetic.
// Bounded for 20 resident CTAs per SM: 48 registers (a 20-byte spill)
// against 56 registers and 18 CTAs without the bound (1M disk: 181 against
// 184 us; 4M: 542 against 567 us).
__global__ void __launch_bounds__(BU_THREADS, 20) bh_bottomup_kernel(const float4 *__restrict__ leaf, const int2 *__restrict__ child,
                                   const int *__restrict__ parent, int n, unsigned *__restrict__ arrivals,
                                   float4 *__restrict__ sums, float4 *__restrict__ bmin, float4 *__restrict__ bmax,
                                   float4 *__restrict__ inode, float4 *__restrict__ root, unsigned long long *diag) {
    const int li = blockIdx.x * blockDim.x + threadIdx.x;
    if (li >= n) return;
    int node = __ldg(parent + li);
    for (int depth = 0; node >= 0; ++depth) {
        if (depth >= MAX_DEPTH || node < n || node >= 2 * n - 1) {
            atomicAdd(diag + DIAG_BAD_TREE, 1ull);
            return;
        }
        const int k = node - n;
        if (!second_arrival(arrivals + k)) return;  // the sibling subtree is still running
        const int2 c = __ldg(child + k);
        if ((unsigned)c.x >= (unsigned)(2 * n - 1) || (unsigned)c.y >= (unsigned)(2 * n - 1)) {
            atomicAdd(diag + DIAG_BAD_TREE, 1ull);
            return;
        }
        const NodeSum a = child_sum(c.x, n, leaf, sums, bmin, bmax);
        const NodeSum b = child_sum(c.y, n, leaf, sums, bmin, bmax);
        NodeSum s;
        s.lx = fminf(a.lx, b.lx); s.ly = fminf(a.ly, b.ly); s.lz = fminf(a.lz, b.lz);
        s.hx = fmaxf(a.hx, b.hx); s.hy = fmaxf(a.hy, b.hy); s.hz = fmaxf(a.hz, b.hz);
        s.m = a.m + b.m;
        s.sx = __fmaf_rn(b.m, b.lx - s.lx, __fmaf_rn(a.m, a.lx - s.lx, a.sx + b.sx));
        s.sy = __fmaf_rn(b.m, b.ly - s.ly, __fmaf_rn(a.m, a.ly - s.ly, a.sy + b.sy));
        s.sz = __fmaf_rn(b.m, b.lz - s.lz, __fmaf_rn(a.m, a.lz - s.lz, a.sz + b.sz));
        sums[k] = make_float4(s.m, s.sx, s.sy, s.sz);
        bmin[k] = make_float4(s.lx, s.ly, s.lz, 0.f);
        bmax[k] = make_float4(s.hx, s.hy, s.hz, 0.f);
        const float4 ca = trav_com(a), cb = trav_com(b);
        inode[3 * k] = make_float4(ca.x, cb.x, ca.y, cb.y);
        inode[3 * k + 1] = make_float4(ca.z, cb.z, ca.w, cb.w);
        inode[3 * k + 2] = make_float4(c.x < n ? -1.f : size2_of(a), c.y < n ? -1.f : size2_of(b),
                                       __int_as_float(c.x), __int_as_float(c.y));
        const int up = __ldg(parent + node);
        if (up < 0) {
            root[0] = trav_com(s);
            root[1] = make_float4(size2_of(s), 0.f, 0.f, 0.f);
        }
        node = up;
    }
}

}  // namespace gb

#include "gb_bh_traverse.cuh"

namespace gb {

// ----------------------------------------------------------------- export
// Tree arrays in the reference's layout for parity checks.
enum ExportWhat {
    EXP_CODES = 0,   // uint64[n]  keys in sorted order
    EXP_ORDER = 1,   // int32[n]
    EXP_LEFT = 2,    // int32[n-1]
    EXP_RIGHT = 3,   // int32[n-1]
    EXP_PARENT = 4,  // int32[2n-1]
    EXP_MASS = 5,    // double[2n-1]
    EXP_COM = 6,     // double[2n-1][3]
    EXP_MIN = 7,     // double[2n-1][3]
    EXP_MAX = 8      // double[2n-1][3]
};

template <typename KeyT>
__global__ void bh_export_kernel(int what, int n, const KeyT *keys, const uint32_t *order, const int2 *child,
                                 const int *parent, const float4 *leaf, const float4 *sums, const float4 *bmin,
                                 const float4 *bmax, void *dst) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nodes = 2 * (int64_t)n - 1;
    switch (what) {
        case EXP_CODES:
            if (i < n) ((uint64_t *)dst)[i] = (uint64_t)keys[i];
            break;
        case EXP_ORDER:
            if (i < n) ((int *)dst)[i] = (int)order[i];
            break;
        case EXP_LEFT:
            if (i < n - 1) ((int *)dst)[i] = child[i].x;
            break;
        case EXP_RIGHT:
            if (i < n - 1) ((int *)dst)[i] = child[i].y;
            break;
        case EXP_PARENT:
            if (i < nodes) ((int *)dst)[i] = i < n ? parent[i] : parent[i];
            break;
        default: {
            if (i >= nodes) break;
            double m, c[3], lo[3], hi[3];
            if (i < n) {
                const float4 p = leaf[i];
                m = p.w;
                c[0] = lo[0] = hi[0] = p.x;
                c[1] = lo[1] = hi[1] = p.y;
                c[2] = lo[2] = hi[2] = p.z;
            } else {
                const int k = (int)(i - n);
                const float4 q = sums[k];
                m = q.x;
                lo[0] = bmin[k].x; lo[1] = bmin[k].y; lo[2] = bmin[k].z;
                c[0] = m > 0.0 ? lo[0] + q.y / m : 0.0;
                c[1] = m > 0.0 ? lo[1] + q.z / m : 0.0;
                c[2] = m > 0.0 ? lo[2] + q.w / m : 0.0;
                hi[0] = bmax[k].x; hi[1] = bmax[k].y; hi[2] = bmax[k].z;
            }
            double *o = (double *)dst;
            if (what == EXP_MASS) o[i] = m;
            else {
                const double *src = what == EXP_COM ? c : (what == EXP_MIN ? lo : hi);
                o[3 * i] = src[0];
                o[3 * i + 1] = src[1];
                o[3 * i + 2] = src[2];
            }
        }
    }
}

}  // namespace gb

// ================================================================ C ABI
using namespace gb;

struct gb_bh {
    int device, sms;
    int64_t n_max;
    int key_bits;
    int64_t n;  // n of the last build (-1: none)
    void *keys[2];
    uint32_t *vals[2];
    int cur;  // which buffer holds the sorted result
    uint32_t *sort_scratch;  // radix_scratch_size(n_max) words
    float4 *bbox_part;
    int bbox_blocks;
    unsigned *ticket;
    BHParams *prm;
    float4 *leaf;
    int2 *child;
    int *parent;
    unsigned *arrivals;
    float4 *sums;
    float4 *bmin, *bmax;
    float4 *inode;
    float4 *root;
    unsigned long long *diag;
    // Stage timing (gb_bh_timing): events recorded on the launch stream at
    // stage boundaries, GB_BH_STAGES + 1 per step, reused cyclically.
    int timing;
    int ev_used;
    cudaEvent_t ev[GB_BH_TIMING_STEPS * (GB_BH_STAGES + 1)];
    uint64_t launches;  // kernels launched by this handle (host count)
    int pending_slot;   // timing slot of the last gb_bh_build
    int tpl;            // traversal shape: -1 by n (default), 0 per lane, 1 or 2 targets per lane
    // One KDK step captured as a CUDA graph (gb_bh_kdk), replayed per step
    // on the handle's own stream and joined to the caller's by events.
    // gexec[0]: a plain step; gexec[1]: a step that also writes the tree
    // potential (gb_bh_kdk_phi); each captured again when its key changes.
    int use_graph;
    cudaStream_t gstream;
    cudaEvent_t gev_in, gev_out;
    cudaGraphExec_t gexec[2];
    struct Key {
        const void *xm, *vel, *acc, *phi;
        int64_t n;
        float theta, eps2, G, dt;
        int max_stack, tpl;
        bool operator==(const Key &o) const {
            return xm == o.xm && vel == o.vel && acc == o.acc && phi == o.phi && n == o.n && theta == o.theta &&
                   eps2 == o.eps2 && G == o.G && dt == o.dt && max_stack == o.max_stack && tpl == o.tpl;
        }
    } gkey[2];
    uint64_t graph_launches[2];  // kernels in each captured step
    double2 *epart;              // energy block partials (gb_bh_energy)
    int epart_cap;
    int *gsize;                  // group-walk groups of the last build (mode 3)
    int64_t groups_n;            // n of the build that marked them (-1: none)
    // Failure checks (GB_CHECK, gb_bh_set_check): the failure counters as
    // read by the last checked call (or zero after a diag reset).
    int check;
    unsigned long long seen[DIAG_COUNT];  // failure counters at the last checked call
};

static void mark(gb_bh_t *h, int step_slot, int stage, cudaStream_t s) {
    if (!h->timing) return;
    cudaEventRecord(h->ev[step_slot * (GB_BH_STAGES + 1) + stage], s);
}

static size_t key_size(int bits) { return bits <= 10 ? sizeof(uint32_t) : sizeof(uint64_t); }

extern "C" int gb_bh_destroy(gb_bh_t *h) {
    if (!h) return GB_OK;
    void *ptrs[] = {h->keys[0], h->keys[1], h->vals[0], h->vals[1], h->sort_scratch, h->bbox_part, h->ticket,
                    h->prm, h->leaf, h->child, h->parent, h->arrivals, h->sums, h->bmin, h->bmax,
                    h->inode, h->root, h->diag, h->epart, h->gsize};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (auto &g : h->gexec)
        if (g) cudaGraphExecDestroy(g);
    if (h->gev_in) cudaEventDestroy(h->gev_in);
    if (h->gev_out) cudaEventDestroy(h->gev_out);
    if (h->gstream) cudaStreamDestroy(h->gstream);
    for (auto &e : h->ev)
        if (e) cudaEventDestroy(e);
    delete h;
    return GB_OK;
}

extern "C" int gb_bh_create(gb_bh_t **out, int64_t n_max, int key_bits) {
    if (!out) return fail(GB_EINVAL, "out is NULL");
    *out = nullptr;
    if (n_max < 1 || n_max > RS_MAX_N) return fail(GB_EINVAL, "n_max=%lld out of range", (long long)n_max);
    if (key_bits != 10 && key_bits != 21) return fail(GB_EINVAL, "key_bits must be 10 or 21 (got %d)", key_bits);
    gb_bh_t *h = new gb_bh();
    GB_CUDA_TRY(cudaGetDevice(&h->device));
    h->sms = num_sms();
    h->n_max = n_max;
    h->key_bits = key_bits;
    h->tpl = -1;
    h->use_graph = 1;
    {
        const int smem_max = (int)sizeof(int) * LANE_MAX_STACK * LANE_THREADS;
        const void *lk[] = {(const void *)bh_traverse_lane_kernel<false, false, false>,
                            (const void *)bh_traverse_lane_kernel<false, true, false>,
                            (const void *)bh_traverse_lane_kernel<true, false, false>,
                            (const void *)bh_traverse_lane_kernel<true, true, false>,
                            (const void *)bh_traverse_lane_kernel<false, false, true>,
                            (const void *)bh_traverse_lane_kernel<false, true, true>,
                            (const void *)bh_traverse_lane_kernel<true, false, true>,
                            (const void *)bh_traverse_lane_kernel<true, true, true>};
        for (const void *f : lk) {
            if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max) != cudaSuccess) {
                delete h;
                return fail(GB_ECUDA, "gb_bh_create: cannot enable %d bytes of shared memory", smem_max);
            }
        }
    }
    h->n = -1;
    h->cur = 0;
    const int64_t nn = n_max, ni = std::max<int64_t>(n_max - 1, 1), nodes = 2 * n_max;
    h->bbox_blocks = std::max(1, std::min(h->sms * 4, (int)((n_max + BBOX_THREADS - 1) / BBOX_THREADS)));
    bool ok = true;
    auto A = [&](void **p, size_t bytes) {
        if (ok && cudaMalloc(p, bytes) != cudaSuccess) ok = false;
    };
    A(&h->keys[0], key_size(key_bits) * nn);
    A(&h->keys[1], key_size(key_bits) * nn);
    A((void **)&h->vals[0], sizeof(uint32_t) * nn);
    A((void **)&h->vals[1], sizeof(uint32_t) * nn);
    A((void **)&h->sort_scratch, sizeof(uint32_t) * radix_scratch_size(n_max));
    A((void **)&h->bbox_part, sizeof(float4) * 2 * h->bbox_blocks);
    A((void **)&h->ticket, sizeof(unsigned));
    A((void **)&h->prm, sizeof(BHParams));
    A((void **)&h->leaf, sizeof(float4) * nn);
    A((void **)&h->child, sizeof(int2) * ni);
    A((void **)&h->parent, sizeof(int) * nodes);
    A((void **)&h->arrivals, sizeof(unsigned) * ni);
    A((void **)&h->sums, sizeof(float4) * ni);
    A((void **)&h->bmin, sizeof(float4) * ni);
    A((void **)&h->bmax, sizeof(float4) * ni);
    A((void **)&h->inode, sizeof(float4) * 3 * ni);
    A((void **)&h->root, sizeof(float4) * 2);
    A((void **)&h->diag, sizeof(unsigned long long) * DIAG_COUNT);
    h->epart_cap = 4 * h->sms;
    A((void **)&h->epart, sizeof(double2) * (h->epart_cap + ENERGY_EXTRA));
    A((void **)&h->gsize, sizeof(int) * nn);
    h->groups_n = -1;
    if (!ok) {
        gb_bh_destroy(h);
        return fail(GB_ENOMEM, "gb_bh_create: device allocation failed for n_max=%lld", (long long)n_max);
    }
    if (cudaMemset(h->ticket, 0, sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(h->diag, 0, sizeof(unsigned long long) * DIAG_COUNT) != cudaSuccess ||
        cudaMemset(h->epart, 0, sizeof(double2) * (h->epart_cap + ENERGY_EXTRA)) != cudaSuccess) {
        gb_bh_destroy(h);
        return fail(GB_ECUDA, "gb_bh_create: memset failed");
    }
    *out = h;
    return GB_OK;
}

template <typename KeyT, int BITS>
static int build_impl(gb_bh_t *h, float4 *xm, float4 *vel, const float4 *acc, int64_t n, float dt, bool kdk,
                      cudaStream_t s, int slot) {
    mark(h, slot, 0, s);
    const int nblk = std::max(1, std::min(h->bbox_blocks, (int)((n + BBOX_THREADS - 1) / BBOX_THREADS)));
    if (kdk)
        bh_bbox_kernel<true><<<nblk, BBOX_THREADS, 0, s>>>(xm, vel, acc, n, 0.5f * dt, dt, h->bbox_part, h->ticket,
                                                           h->prm, BITS, h->diag);
    else
        bh_bbox_kernel<false><<<nblk, BBOX_THREADS, 0, s>>>(xm, nullptr, nullptr, n, 0.f, 0.f, h->bbox_part,
                                                            h->ticket, h->prm, BITS, h->diag);
    const unsigned g256 = (unsigned)((n + 255) / 256);
    KeyT *k0 = (KeyT *)h->keys[0], *k1 = (KeyT *)h->keys[1];
    uint32_t *v0 = h->vals[0], *v1 = h->vals[1];
    bh_morton_kernel<KeyT, BITS><<<g256, 256, 0, s>>>(xm, n, h->prm, k0, v0);
    mark(h, slot, 1, s);
    const int passes = (3 * BITS + 7) / 8;
    KeyT *kk[2] = {k0, k1};
    uint32_t *vv[2] = {v0, v1};
    h->cur = radix_sort_pairs<KeyT>(kk, vv, n, passes, h->sort_scratch, h->diag, s);
    k0 = kk[h->cur];
    v0 = vv[h->cur];
    mark(h, slot, 2, s);
    bh_gather_kernel<<<g256, 256, 0, s>>>(xm, v0, n, h->leaf, h->diag);
    const int ni = (int)std::max<int64_t>(n - 1, 1);
    // The group walk's groups are marked when the handle walks groups.
    int *gsize = h->tpl == 3 ? h->gsize : nullptr;
    if (gsize) GB_CUDA_TRY(cudaMemsetAsync(gsize, 0, sizeof(int) * n, s));
    bh_karras_kernel<KeyT><<<(ni + 255) / 256, 256, 0, s>>>(k0, (int)n, h->child, h->parent, gsize);
    h->groups_n = gsize ? n : -1;
    mark(h, slot, 3, s);
    if (n >= 2) {
        GB_CUDA_TRY(cudaMemsetAsync(h->arrivals, 0, sizeof(unsigned) * (n - 1), s));
        bh_bottomup_kernel<<<(unsigned)((n + BU_THREADS - 1) / BU_THREADS), BU_THREADS, 0, s>>>(
            h->leaf, h->child, h->parent, (int)n, h->arrivals, h->sums, h->bmin, h->bmax, h->inode, h->root, h->diag);
    }
    GB_CUDA_TRY(cudaGetLastError());
    mark(h, slot, 4, s);
    h->launches += 5 + 1 + passes - (n >= 2 ? 0 : 1);
    h->n = n;
    return GB_OK;
}

static int next_slot(gb_bh_t *h) {
    if (!h->timing) return 0;
    const int slot = h->ev_used % GB_BH_TIMING_STEPS;
    ++h->ev_used;
    return slot;
}

static int build_any(gb_bh_t *h, float4 *xm, float4 *vel, const float4 *acc, int64_t n, float dt, bool kdk,
                     cudaStream_t s, int slot) {
    if (h->key_bits == 10) return build_impl<uint32_t, 10>(h, xm, vel, acc, n, dt, kdk, s, slot);
    return build_impl<uint64_t, 21>(h, xm, vel, acc, n, dt, kdk, s, slot);
}

static int check_bh(gb_bh_t *h, int64_t n) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (n < 0 || n > h->n_max) return fail(GB_EINVAL, "n=%lld outside [0, n_max=%lld]", (long long)n, (long long)h->n_max);
    return GB_OK;
}

static int check_ptr(const void *p, const char *name) {
    if (!p) return fail(GB_EINVAL, "%s is NULL", name);
    if (!aligned16(p)) return fail(GB_EINVAL, "%s is not 16-byte aligned", name);
    return GB_OK;
}

template <bool KDK, bool COUNT, bool PHI>
static void launch_lane(unsigned grid, size_t smem, const TravArgs &a, float *phi, const int *parent, int2 r,
                        cudaStream_t s) {
    bh_traverse_lane_kernel<KDK, COUNT, PHI><<<grid, LANE_THREADS, smem, s>>>(a, phi, parent, r.x, r.y);
}

template <bool KDK, bool COUNT, bool PHI>
static void launch_warp(int tpl, unsigned grid, const TravArgs &a, float *phi, const int *parent, int2 r,
                        cudaStream_t s) {
    if (tpl == 2) bh_traverse_kernel<KDK, COUNT, 2, PHI><<<grid, TRAV_WARPS * 32, 0, s>>>(a, phi, parent, r.x, r.y);
    else bh_traverse_kernel<KDK, COUNT, 1, PHI><<<grid, TRAV_WARPS * 32, 0, s>>>(a, phi, parent, r.x, r.y);
}

// Dispatches L<KDK, COUNT, PHI>::go(args...) on run-time flags.
template <template <bool, bool, bool> class L, typename... Args>
static void dispatch3(bool kdk, bool count, bool phi, Args... args) {
    const int sel = (kdk ? 4 : 0) + (count ? 2 : 0) + (phi ? 1 : 0);
    switch (sel) {
        case 0: L<false, false, false>::go(args...); break;
        case 1: L<false, false, true>::go(args...); break;
        case 2: L<false, true, false>::go(args...); break;
        case 3: L<false, true, true>::go(args...); break;
        case 4: L<true, false, false>::go(args...); break;
        case 5: L<true, false, true>::go(args...); break;
        case 6: L<true, true, false>::go(args...); break;
        default: L<true, true, true>::go(args...); break;
    }
}
template <bool KDK, bool COUNT, bool PHI>
struct LaneLaunch {
    static void go(unsigned grid, size_t smem, const TravArgs *a, float *phi, const int *parent, int2 r,
                   cudaStream_t s) {
        launch_lane<KDK, COUNT, PHI>(grid, smem, *a, phi, parent, r, s);
    }
};
template <bool KDK, bool COUNT, bool PHI>
struct GroupLaunch {
    static void go(unsigned grid, const TravArgs *a, const int *gsize, float *phi, int2 r, cudaStream_t s) {
        bh_group_kernel<KDK, COUNT, PHI><<<grid, GW_WARPS * 32, 0, s>>>(*a, gsize, phi, r.x, r.y);
    }
};
template <bool KDK, bool COUNT, bool PHI>
struct WarpLaunch {
    static void go(int tpl, unsigned grid, const TravArgs *a, float *phi, const int *parent, int2 r,
                   cudaStream_t s) {
        launch_warp<KDK, COUNT, PHI>(tpl, grid, *a, phi, parent, r, s);
    }
};

// The traversal of the last build: accelerations into acc (KDK: the
// closing kick into vel too) and, when phi is not NULL, the tree potential
// sums into phi.
// Targets: key-order indices [s0, s1) (s1 < 0: all n).
static int traverse(gb_bh_t *h, float4 *acc, float4 *vel, float *phi, float theta, float eps2, float G, float dt,
                    int max_stack, int flags, bool kdk, cudaStream_t s, int slot, const ExtPot &pot = ExtPot{},
                    int64_t s0 = 0, int64_t s1 = -1) {
    const int64_t n = h->n;
    if (n <= 0) return GB_OK;
    if (s1 < 0) s1 = n;
    if (s1 <= s0) return GB_OK;
    const int64_t nt = s1 - s0;
    const int2 range = make_int2((int)s0, (int)s1);  // key-order targets [s0, s1)
    TravArgs a;
    a.leaf = h->leaf;
    a.inode = h->inode;
    a.root = h->root;
    a.order = h->vals[h->cur];
    a.acc = acc;
    a.vel = vel;
    a.n = (int)n;
    a.theta2 = theta * theta;
    a.eps2 = eps2;
    a.G = G;
    a.h = 0.5f * dt;
    a.max_stack = max_stack;
    a.accumulate = (flags & GB_ACCUMULATE) ? 1 : 0;
    a.diag = h->diag;
    a.pot = pot;
    const bool count = (flags & GB_COUNT_WORK) != 0;
    // By n: per-lane walks below LANE_AUTO_N, where a warp-coherent launch
    // has too few warps to hide each step's latency (1M disk: 3.44 ms
    // warp-coherent against 5.84 ms per lane; 10k: 0.24 against 0.18 ms).
    const int shape = h->tpl >= 0 ? h->tpl : (n < LANE_AUTO_N ? 0 : 1);
    if (shape == 3) {
        const int64_t warps = (nt + 31) / 32;
        const unsigned grid = (unsigned)((warps + GW_WARPS - 1) / GW_WARPS);
        if (h->groups_n != n) {
            // Built in another traversal mode: mark the groups from the
            // sorted keys of the same build (the topology is rewritten with
            // identical values).
            int *gsize = h->gsize;
            GB_CUDA_TRY(cudaMemsetAsync(gsize, 0, sizeof(int) * n, s));
            const int ni = (int)std::max<int64_t>(n - 1, 1);
            if (h->key_bits == 10)
                bh_karras_kernel<uint32_t><<<(ni + 255) / 256, 256, 0, s>>>(
                    (const uint32_t *)h->keys[h->cur], (int)n, h->child, h->parent, gsize);
            else
                bh_karras_kernel<uint64_t><<<(ni + 255) / 256, 256, 0, s>>>(
                    (const uint64_t *)h->keys[h->cur], (int)n, h->child, h->parent, gsize);
            GB_CUDA_TRY(cudaGetLastError());
            h->launches += 1;
            h->groups_n = n;
        }
        dispatch3<GroupLaunch>(kdk, count, phi != nullptr, grid, &a, (const int *)h->gsize, phi, range, s);
    } else if (shape == 0 && max_stack <= LANE_MAX_STACK && n - 1 <= ((int64_t)1 << LANE_KBITS)) {
        const unsigned grid = (unsigned)((nt + LANE_THREADS - 1) / LANE_THREADS);
        const size_t smem = sizeof(int) * (size_t)std::max(max_stack, 1) * LANE_THREADS;
        dispatch3<LaneLaunch>(kdk, count, phi != nullptr, grid, smem, &a, phi, (const int *)h->parent, range, s);
    } else {
        const int tpl = shape == 2 ? 2 : 1;
        const int64_t warps = (nt + 32 * tpl - 1) / (32 * tpl);
        const unsigned grid = (unsigned)((warps + TRAV_WARPS - 1) / TRAV_WARPS);
        dispatch3<WarpLaunch>(kdk, count, phi != nullptr, tpl, grid, &a, phi, (const int *)h->parent, range, s);
    }
    GB_CUDA_TRY(cudaGetLastError());
    mark(h, slot, 5, s);
    h->launches += 1;
    return GB_OK;
}

// Synchronises `s` and compares the failure counters (stack drops, stack
// overflow, non-finite positions, bad tree, expired waits) with the values
// the last check saw: anything counted since then fails the call.
// Non-finite positions and index guards give GB_EINVAL, an expired wait
// GB_ETIMEOUT, dropped or overflowed pushes GB_ESTACK.
static int check_failures(gb_bh_t *h, cudaStream_t s, const char *call) {
    unsigned long long d[DIAG_COUNT];
    GB_CUDA_TRY(cudaMemcpyAsync(d, h->diag, sizeof(d), cudaMemcpyDeviceToHost, s));
    GB_CUDA_TRY(cudaStreamSynchronize(s));
    unsigned long long inc[DIAG_COUNT];
    for (int k = 0; k < DIAG_COUNT; ++k) {
        inc[k] = d[k] - h->seen[k];
        h->seen[k] = d[k];
    }
    if (inc[DIAG_NONFINITE])
        return fail(GB_EINVAL, "%s: %llu non-finite particle positions", call, inc[DIAG_NONFINITE]);
    if (inc[DIAG_BAD_TREE])
        return fail(GB_EINVAL, "%s: inconsistent tree (%llu index guards taken)", call, inc[DIAG_BAD_TREE]);
    if (inc[DIAG_WAIT_TIMEOUT])
        return fail(GB_ETIMEOUT, "%s: %llu bounded device waits expired (radix sort look-back)", call,
                    inc[DIAG_WAIT_TIMEOUT]);
    if (inc[DIAG_STACK_DROPS] || inc[DIAG_STACK_OVERFLOW])
        return fail(GB_ESTACK, "%s: the max_stack rule dropped %llu pushes; %llu overflowed the traversal stack",
                    call, inc[DIAG_STACK_DROPS], inc[DIAG_STACK_OVERFLOW]);
    return GB_OK;
}

static int check_params(float theta, float eps2, int max_stack) {
    if (!(theta >= 0.f)) return fail(GB_EINVAL, "theta must be >= 0");
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    if (max_stack < 1) return fail(GB_EINVAL, "max_stack must be >= 1");
    return GB_OK;
}

extern "C" int gb_bh_build(gb_bh_t *h, const float *xm, int64_t n, void *stream) {
    GB_TRY(check_bh(h, n));
    if (n == 0) {
        h->n = 0;
        return GB_OK;
    }
    GB_TRY(check_ptr(xm, "xm"));
    h->pending_slot = next_slot(h);
    return build_any(h, (float4 *)xm, nullptr, nullptr, n, 0.f, false, (cudaStream_t)stream, h->pending_slot);
}

extern "C" int gb_bh_accel(gb_bh_t *h, float *acc, float theta, float eps2, float G, int max_stack, int flags,
                           void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (h->n < 0) return fail(GB_ENOTREADY, "gb_bh_accel before gb_bh_build");
    if (h->n == 0) return GB_OK;
    GB_TRY(check_ptr(acc, "acc"));
    GB_TRY(check_params(theta, eps2, max_stack));
    GB_TRY(traverse(h, (float4 *)acc, nullptr, nullptr, theta, eps2, G, 0.f, max_stack, flags, false,
                    (cudaStream_t)stream, h->pending_slot));
    if ((flags & GB_CHECK) || h->check) return check_failures(h, (cudaStream_t)stream, "gb_bh_accel");
    return GB_OK;
}

extern "C" int gb_bh_accel_range(gb_bh_t *h, float *acc, float *phi, int64_t s0, int64_t ns, float theta,
                                 float eps2, float G, int max_stack, int flags, void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (h->n < 0) return fail(GB_ENOTREADY, "gb_bh_accel_range before gb_bh_build");
    if (s0 < 0 || ns < 0 || s0 > h->n || ns > h->n - s0)
        return fail(GB_EINVAL, "target range [%lld, %lld) outside the %lld particles of the last build",
                    (long long)s0, (long long)(s0 + ns), (long long)h->n);
    if (flags & ~(GB_ACCUMULATE | GB_CHECK))
        return fail(GB_EINVAL, "gb_bh_accel_range: flags 0x%x: only GB_ACCUMULATE and GB_CHECK apply", flags);
    if (ns == 0) return GB_OK;
    GB_TRY(check_ptr(acc, "acc"));
    GB_TRY(check_params(theta, eps2, max_stack));
    GB_TRY(traverse(h, (float4 *)acc, nullptr, phi, theta, eps2, G, 0.f, max_stack, flags, false,
                    (cudaStream_t)stream, h->pending_slot, ExtPot{}, s0, s0 + ns));
    if ((flags & GB_CHECK) || h->check) return check_failures(h, (cudaStream_t)stream, "gb_bh_accel_range");
    return GB_OK;
}

extern "C" int gb_bh_accel_phi(gb_bh_t *h, float *acc, float *phi, float theta, float eps2, float G, int max_stack,
                               int flags, void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (h->n < 0) return fail(GB_ENOTREADY, "gb_bh_accel_phi before gb_bh_build");
    if (h->n == 0) return GB_OK;
    GB_TRY(check_ptr(acc, "acc"));
    if (!phi) return fail(GB_EINVAL, "phi is NULL");
    GB_TRY(check_params(theta, eps2, max_stack));
    GB_TRY(traverse(h, (float4 *)acc, nullptr, phi, theta, eps2, G, 0.f, max_stack, flags, false,
                    (cudaStream_t)stream, h->pending_slot));
    if ((flags & GB_CHECK) || h->check) return check_failures(h, (cudaStream_t)stream, "gb_bh_accel_phi");
    return GB_OK;
}

extern "C" int gb_bh_accel_ext(gb_bh_t *h, float *acc, float theta, float eps2, float G, int max_stack,
                               const gb_potential_t *pot, int flags, void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    ExtPot ep;
    GB_TRY(make_extpot(pot, G, &ep));
    if (h->n < 0) return fail(GB_ENOTREADY, "gb_bh_accel_ext before gb_bh_build");
    if (h->n == 0) return GB_OK;
    GB_TRY(check_ptr(acc, "acc"));
    GB_TRY(check_params(theta, eps2, max_stack));
    GB_TRY(traverse(h, (float4 *)acc, nullptr, nullptr, theta, eps2, G, 0.f, max_stack, flags, false,
                    (cudaStream_t)stream, h->pending_slot, ep));
    if ((flags & GB_CHECK) || h->check) return check_failures(h, (cudaStream_t)stream, "gb_bh_accel_ext");
    return GB_OK;
}

extern "C" int gb_bh_compute(gb_bh_t *h, const float *xm, float *acc, int64_t n, float theta, float eps2, float G,
                             int max_stack, int flags, void *stream) {
    GB_TRY(check_bh(h, n));
    if (n > 0) {
        GB_TRY(check_ptr(acc, "acc"));
        GB_TRY(check_params(theta, eps2, max_stack));
    }
    GB_TRY(gb_bh_build(h, xm, n, stream));
    return gb_bh_accel(h, acc, theta, eps2, G, max_stack, flags, stream);
}

// One KDK step: tree build with the fused kick and drift, then the traversal
// with the closing kick (and the tree potential of the new positions when
// phi is not NULL).
static int kdk_step(gb_bh_t *h, float4 *xm, float4 *vel, float4 *acc, float *phi, int64_t n, float theta,
                    float eps2, float G, float dt, int max_stack, cudaStream_t s) {
    const int slot = next_slot(h);
    GB_TRY(build_any(h, xm, vel, acc, n, dt, true, s, slot));
    return traverse(h, acc, vel, phi, theta, eps2, G, dt, max_stack, 0, true, s, slot);
}

// Graph slot g (0 plain, 1 with the potential) holds one captured step with
// this key, captured again when the key changed.
static int ensure_graph(gb_bh_t *h, int g, const gb_bh::Key &key, float4 *x, float4 *v, float4 *a, float *phi,
                        int64_t n, float theta, float eps2, float G, float dt, int max_stack) {
    if (h->gexec[g] && h->gkey[g] == key) return GB_OK;
    if (h->gexec[g]) cudaGraphExecDestroy(h->gexec[g]);
    h->gexec[g] = nullptr;
    GB_CUDA_TRY(cudaStreamBeginCapture(h->gstream, cudaStreamCaptureModeThreadLocal));
    const uint64_t l0 = h->launches;
    const int st = kdk_step(h, x, v, a, phi, n, theta, eps2, G, dt, max_stack, h->gstream);
    h->graph_launches[g] = h->launches - l0;
    h->launches = l0;
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->gstream, &graph);
    if (st != GB_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess) return fail(GB_ECUDA, "graph capture: %s", cudaGetErrorString(e));
    const cudaError_t ei = cudaGraphInstantiate(&h->gexec[g], graph, 0);
    cudaGraphDestroy(graph);
    if (ei != cudaSuccess) {
        h->gexec[g] = nullptr;
        return fail(GB_ECUDA, "graph instantiate: %s", cudaGetErrorString(ei));
    }
    h->gkey[g] = key;
    return GB_OK;
}

// nsteps KDK steps; with phi, the last step also writes the tree potential.
static int bh_kdk_impl(gb_bh_t *h, float *xm, float *vel, float *acc, float *phi, int64_t n, float theta, float eps2,
                       float G, float dt, int64_t nsteps, int max_stack, void *stream, const char *call) {
    GB_TRY(check_bh(h, n));
    if (nsteps < 0) return fail(GB_EINVAL, "nsteps < 0");
    if (n == 0 || nsteps == 0) return GB_OK;
    GB_TRY(check_ptr(xm, "xm"));
    GB_TRY(check_ptr(vel, "vel"));
    GB_TRY(check_ptr(acc, "acc"));
    GB_TRY(check_params(theta, eps2, max_stack));
    cudaStream_t s = (cudaStream_t)stream;
    float4 *x = (float4 *)xm, *v = (float4 *)vel, *a = (float4 *)acc;
    if (!h->use_graph || h->timing) {
        for (int64_t k = 0; k < nsteps; ++k)
            GB_TRY(kdk_step(h, x, v, a, k == nsteps - 1 ? phi : nullptr, n, theta, eps2, G, dt, max_stack, s));
        return h->check ? check_failures(h, s, call) : GB_OK;
    }
    if (!h->gstream) {
        GB_CUDA_TRY(cudaStreamCreateWithFlags(&h->gstream, cudaStreamNonBlocking));
        GB_CUDA_TRY(cudaEventCreateWithFlags(&h->gev_in, cudaEventDisableTiming));
        GB_CUDA_TRY(cudaEventCreateWithFlags(&h->gev_out, cudaEventDisableTiming));
    }
    const int64_t plain_steps = phi ? nsteps - 1 : nsteps;
    gb_bh::Key key{xm, vel, acc, nullptr, n, theta, eps2, G, dt, max_stack, h->tpl};
    if (plain_steps) GB_TRY(ensure_graph(h, 0, key, x, v, a, nullptr, n, theta, eps2, G, dt, max_stack));
    if (phi) {
        key.phi = phi;
        GB_TRY(ensure_graph(h, 1, key, x, v, a, phi, n, theta, eps2, G, dt, max_stack));
    }
    GB_CUDA_TRY(cudaEventRecord(h->gev_in, s));
    GB_CUDA_TRY(cudaStreamWaitEvent(h->gstream, h->gev_in, 0));
    for (int64_t k = 0; k < plain_steps; ++k) GB_CUDA_TRY(cudaGraphLaunch(h->gexec[0], h->gstream));
    if (phi) GB_CUDA_TRY(cudaGraphLaunch(h->gexec[1], h->gstream));
    GB_CUDA_TRY(cudaEventRecord(h->gev_out, h->gstream));
    GB_CUDA_TRY(cudaStreamWaitEvent(s, h->gev_out, 0));
    h->launches += h->graph_launches[0] * (uint64_t)plain_steps + (phi ? h->graph_launches[1] : 0);
    h->n = n;
    return h->check ? check_failures(h, s, call) : GB_OK;
}

extern "C" int gb_bh_kdk(gb_bh_t *h, float *xm, float *vel, float *acc, int64_t n, float theta, float eps2, float G,
                         float dt, int64_t nsteps, int max_stack, void *stream) {
    return bh_kdk_impl(h, xm, vel, acc, nullptr, n, theta, eps2, G, dt, nsteps, max_stack, stream, "gb_bh_kdk");
}

extern "C" int gb_bh_kdk_phi(gb_bh_t *h, float *xm, float *vel, float *acc, float *phi, int64_t n, float theta,
                             float eps2, float G, float dt, int64_t nsteps, int max_stack, void *stream) {
    if (!phi && n > 0 && nsteps > 0) return fail(GB_EINVAL, "phi is NULL");
    return bh_kdk_impl(h, xm, vel, acc, phi, n, theta, eps2, G, dt, nsteps, max_stack, stream, "gb_bh_kdk_phi");
}

extern "C" int gb_bh_energy(gb_bh_t *h, const float *xm, const float *vel, const float *phi, int64_t n, float G,
                            double *out3, void *stream) {
    GB_TRY(check_bh(h, n));
    if (n > 0) {
        GB_TRY(check_ptr(xm, "xm"));
        GB_TRY(check_ptr(vel, "vel"));
        if (!phi) return fail(GB_EINVAL, "phi is NULL");
    }
    if (!out3) return fail(GB_EINVAL, "out3 is NULL");
    GB_TRY(launch_energy((const float4 *)xm, (const float4 *)vel, phi, n, G, h->epart, h->epart_cap, out3,
                         (cudaStream_t)stream));
    h->launches += 1;
    return GB_OK;
}

// One CTA runs the radix sort's look-back for tile 1 of a two-tile status
// array.  publish_first = 1: each thread first publishes tile 0's prefix
// (its digit d as the count), so the look-back returns d; 0: tile 0 never
// publishes and every wait runs out after spin_limit polls.
__global__ void sort_wait_probe_kernel(uint32_t *status, int spin_limit, int publish_first, uint32_t *excl,
                                       unsigned long long *diag) {
    const int d = threadIdx.x;
    if (publish_first) st_relaxed_gpu(status + d, RS_PRE | (uint32_t)d);
    excl[d] = rs_lookback(status, 1, d, 1u, spin_limit, diag);
}

extern "C" int gb_sort_wait_probe(int spin_limit, int publish_first, uint32_t *excl_out, uint64_t *timeouts_out) {
    if (spin_limit < 1 || spin_limit > RS_SPIN_LIMIT)
        return fail(GB_EINVAL, "spin_limit must be in [1, %d] (got %d)", RS_SPIN_LIMIT, spin_limit);
    if (!excl_out || !timeouts_out) return fail(GB_EINVAL, "NULL argument");
    uint32_t *status = nullptr, *excl = nullptr;
    unsigned long long *diag = nullptr;
    int rc = GB_OK;
    if (cudaMalloc(&status, sizeof(uint32_t) * 2 * RS_BINS) != cudaSuccess ||
        cudaMalloc(&excl, sizeof(uint32_t) * RS_BINS) != cudaSuccess ||
        cudaMalloc(&diag, sizeof(unsigned long long) * DIAG_COUNT) != cudaSuccess) {
        rc = fail(GB_ENOMEM, "gb_sort_wait_probe: device allocation failed");
    }
    if (rc == GB_OK && (cudaMemset(status, 0, sizeof(uint32_t) * 2 * RS_BINS) != cudaSuccess ||
                        cudaMemset(diag, 0, sizeof(unsigned long long) * DIAG_COUNT) != cudaSuccess))
        rc = fail(GB_ECUDA, "gb_sort_wait_probe: memset failed");
    if (rc == GB_OK) {
        sort_wait_probe_kernel<<<1, RS_BINS>>>(status, spin_limit, publish_first ? 1 : 0, excl, diag);
        unsigned long long d[DIAG_COUNT];
        if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(excl_out, excl, sizeof(uint32_t) * RS_BINS, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(d, diag, sizeof(d), cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = fail(GB_ECUDA, "gb_sort_wait_probe: %s", cudaGetErrorString(cudaGetLastError()));
        } else {
            *timeouts_out = (uint64_t)d[DIAG_WAIT_TIMEOUT];
            if (d[DIAG_WAIT_TIMEOUT])
                rc = fail(GB_ETIMEOUT, "gb_sort_wait_probe: %llu waits expired", d[DIAG_WAIT_TIMEOUT]);
        }
    }
    if (status) cudaFree(status);
    if (excl) cudaFree(excl);
    if (diag) cudaFree(diag);
    return rc;
}

extern "C" int gb_bh_set_check(gb_bh_t *h, int on) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    h->check = on ? 1 : 0;
    return GB_OK;
}

extern "C" int gb_bh_set_graph(gb_bh_t *h, int on) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    h->use_graph = on ? 1 : 0;
    return GB_OK;
}

extern "C" int gb_bh_export(gb_bh_t *h, int what, void *dst, void *stream) {
    if (!h || !dst) return fail(GB_EINVAL, "NULL argument");
    if (h->n < 1) return fail(GB_ENOTREADY, "no tree built");
    if (what < EXP_CODES || what > EXP_MAX) return fail(GB_EINVAL, "unknown export %d", what);
    const int n = (int)h->n;
    const int64_t count = 2 * (int64_t)n;
    const unsigned grid = (unsigned)((count + 255) / 256);
    cudaStream_t s = (cudaStream_t)stream;
    if (h->key_bits == 10)
        bh_export_kernel<uint32_t><<<grid, 256, 0, s>>>(what, n, (const uint32_t *)h->keys[h->cur], h->vals[h->cur],
                                                        h->child, h->parent, h->leaf, h->sums, h->bmin, h->bmax, dst);
    else
        bh_export_kernel<uint64_t><<<grid, 256, 0, s>>>(what, n, (const uint64_t *)h->keys[h->cur], h->vals[h->cur],
                                                        h->child, h->parent, h->leaf, h->sums, h->bmin, h->bmax, dst);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

extern "C" int gb_bh_diag(gb_bh_t *h, gb_diag_t *out, int reset) {
    if (!h || !out) return fail(GB_EINVAL, "NULL argument");
    GB_TRY(read_diag(h->diag, out, reset));
    if (reset)
        for (auto &v : h->seen) v = 0;
    return GB_OK;
}

extern "C" int gb_bh_timing(gb_bh_t *h, int enable) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (enable && !h->ev[0]) {
        for (auto &e : h->ev) GB_CUDA_TRY(cudaEventCreate(&e));
    }
    h->timing = enable ? 1 : 0;
    h->ev_used = 0;
    return GB_OK;
}

extern "C" int gb_bh_stage_times(gb_bh_t *h, float *ms, int *steps) {
    if (!h || !ms || !steps) return fail(GB_EINVAL, "NULL argument");
    for (int k = 0; k < GB_BH_STAGES; ++k) ms[k] = 0.f;
    const int used = std::min(h->ev_used, GB_BH_TIMING_STEPS);
    GB_CUDA_TRY(cudaDeviceSynchronize());
    for (int st = 0; st < used; ++st)
        for (int k = 0; k < GB_BH_STAGES; ++k) {
            float t = 0.f;
            GB_CUDA_TRY(cudaEventElapsedTime(&t, h->ev[st * (GB_BH_STAGES + 1) + k],
                                             h->ev[st * (GB_BH_STAGES + 1) + k + 1]));
            ms[k] += t;
        }
    *steps = used;
    h->ev_used = 0;
    return GB_OK;
}

extern "C" uint64_t gb_bh_launch_count(gb_bh_t *h) { return h ? h->launches : 0; }

extern "C" int gb_bh_set_traversal(gb_bh_t *h, int targets_per_lane) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (targets_per_lane < -1 || targets_per_lane > 3)
        return fail(GB_EINVAL, "traversal mode must be -1, 0, 1, 2 or 3 (got %d)", targets_per_lane);
    h->tpl = targets_per_lane;
    return GB_OK;
}
