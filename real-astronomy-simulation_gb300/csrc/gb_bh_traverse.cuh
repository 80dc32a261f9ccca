// Tree traversal kernels of the LBVH Barnes-Hut path (included by gb_bh.cu,
// which builds the tree they walk):
//   bh_traverse_kernel       warp-coherent walk: 32 (or 64) key-consecutive
//                            targets share one shared-memory stack of (node,
//                            lane mask); every lane applies the reference's
//                            own acceptance test (core/solvers/barnes_hut.py:
//                            204-210), so each particle accepts exactly the
//                            node set of _traverse (:180-217)
//   bh_traverse_lane_kernel  the same walk with one stack per lane
//   bh_group_kernel          the opt-in group walk (a refinement of each
//                            target's node set, one walk per leaf group)
// Node records: inode[3k .. 3k+2] = the two children of internal node k as
// (left, right) pairs {x, y, z, m, size^2, id}; root[0..1] = the root's.
#pragma once

#include "gb_common.cuh"

namespace gb {

constexpr int TRAV_WARPS = 4;
constexpr int TRAV_STACK = 128;  // > maximum Karras depth (63 + 31 levels)

// --------------------------------------------------------------- traverse
struct TravArgs {
    const float4 *__restrict__ leaf;
    const float4 *__restrict__ inode;
    const float4 *__restrict__ root;
    const uint32_t *__restrict__ order;
    float4 *acc;
    float4 *vel;
    int n;
    float theta2, eps2, G, h;
    int max_stack;
    int accumulate;
    unsigned long long *diag;
    ExtPot pot;  // analytic potential added in the epilogue (pot.on)
};

struct Lane {
    float px, py, pz, ax, ay, az;
    f2 PX, PY, PZ;  // (p, p) pairs
    f2 AX, AY, AZ;  // accumulators for (left, right) children
    unsigned n_int, n_test, drops;
};

// Tree-potential sums of a lane (PHI kernels only): pw for the root, PW for
// the (left, right) children.  The children's terms are added as sc * r2
// (= m / |d| up to rsqrt rounding) from the masked force factor, the lane's
// own leaf included; self records whether the walk reached it (its parent,
// internal node kp, was expanded for the lane), and the epilogue then
// removes its term m rsqrt(eps^2)^3 eps^2.
struct LanePhi {
    float pw, pm;
    f2 PW;
    int kp;
    bool self;
};

// The lane's potential sum without its own leaf's term.
__device__ __forceinline__ float lane_phi(const LanePhi &W, float eps2) {
    float wl, wr;
    unpack2(W.PW, wl, wr);
    const float pw = W.pw + (wl + wr);
    if (!W.self) return pw;
    const float inv = rsqrt_approx(eps2);
    return __fmaf_rn(-((W.pm * inv) * (inv * inv)), eps2, pw);
}

// One child for one lane of the expanding mask (branch-free).  Leaves carry
// size2 = -1 in the record, so the one comparison size2 < theta^2 (|d|^2 +
// eps^2) accepts every leaf and applies the reference's test (:208) to
// internal nodes.  An accepted child adds its monopole; the lane's own leaf
// (which the reference skips, :198) sits exactly at the lane's position, so
// its term is d * (...) = +0 and needs no test.  A rejected (internal) child
// is opened.  Returns "open".  PHI: an accepted child other than the lane's
// own leaf also adds its monopole potential m / |d| (|d|^2 = d.d + eps^2),
// the tree form of the potential_energy sum (core/solvers/gravity.py:47-55).
template <bool COUNT, bool PHI>
__device__ __forceinline__ bool visit_child(Lane &L, LanePhi &W, const TravArgs &a, float4 q, float size2, int id,
                                            int s, bool in) {
    const float dx = q.x - L.px, dy = q.y - L.py, dz = q.z - L.pz;
    const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, a.eps2)));
    const bool accept = size2 < a.theta2 * r2;
    const bool add = in && accept;
    const float inv = rsqrt_approx(r2);
    const float sc = add ? q.w * inv * inv * inv : 0.f;
    L.ax = __fmaf_rn(sc, dx, L.ax);
    L.ay = __fmaf_rn(sc, dy, L.ay);
    L.az = __fmaf_rn(sc, dz, L.az);
    if (PHI) W.pw += (add && id != s) ? q.w * inv : 0.f;  // the root: never the own leaf
    if (COUNT) {
        L.n_int += (add && id != s) ? 1u : 0u;
        L.n_test += (in && size2 >= 0.f) ? 1u : 0u;
    }
    return in && !accept;
}

// Both children of an expanded node for one lane, on packed (left, right)
// pairs: the same test and monopole as visit_child, two children per
// instruction.  Sets openL / openR.  PHI as in visit_child.
template <bool COUNT, bool PHI>
__device__ __forceinline__ void visit_pair(Lane &L, LanePhi &W, const TravArgs &a, ulonglong2 A, ulonglong2 B,
                                           float4 C, int s, bool in, f2 E2, f2 TH2, bool &openL, bool &openR) {
    const f2 dx = sub2(A.x, L.PX), dy = sub2(A.y, L.PY), dz = sub2(B.x, L.PZ);
    f2 r2 = fma2(dx, dx, E2);
    r2 = fma2(dy, dy, r2);
    r2 = fma2(dz, dz, r2);
    const f2 t = mul2(TH2, r2);
    float r2L, r2R, tL, tR;
    unpack2(r2, r2L, r2R);
    unpack2(t, tL, tR);
    const bool accL = C.x < tL, accR = C.y < tR;
    const f2 inv = pack2(rsqrt_approx(r2L), rsqrt_approx(r2R));
    const f2 sc = mul2(mul2(B.y, inv), mul2(inv, inv));
    float scL, scR;
    unpack2(sc, scL, scR);
    const f2 scm = pack2((in && accL) ? scL : 0.f, (in && accR) ? scR : 0.f);
    L.AX = fma2(scm, dx, L.AX);
    L.AY = fma2(scm, dy, L.AY);
    L.AZ = fma2(scm, dz, L.AZ);
    if (PHI) W.PW = fma2(scm, r2, W.PW);
    if (COUNT) {
        L.n_int += (in && accL && __float_as_int(C.z) != s) ? 1u : 0u;
        L.n_int += (in && accR && __float_as_int(C.w) != s) ? 1u : 0u;
        L.n_test += (in && C.x >= 0.f) ? 1u : 0u;
        L.n_test += (in && C.y >= 0.f) ? 1u : 0u;
    }
    openL = in && !accL;
    openR = in && !accR;
}

// The reference's push rule (:212): a lane that opens a node popped at stack
// depth sp pushes its children only if sp + 2 <= max_stack.  sp is uniform
// over the warp, so the (rare) drop path is a uniform branch.
__device__ __forceinline__ bool apply_room(Lane &L, bool open, int sp, int max_stack) {
    if (sp + 2 <= max_stack) return open;
    L.drops += open ? 1u : 0u;
    return false;
}

// Warp-coherent traversal: TPL x 32 key-consecutive targets per warp walk the
// tree together (TPL targets per lane: slot q of lane l is target wbase +
// 32 q + l).  The warp expands one internal node per iteration: it loads the
// node's two-children record (48 B) and every lane visits both children for
// each of its slots in the node's masks (right first, as the reference pops
// it first).  The right child, if any slot opened it, is expanded next
// straight from registers; an opened left child waits on a shared-memory
// stack of {node, mask slot 0, mask slot 1, sp}.  sp, the depth of the
// reference's per-particle stack when a node is popped, depends only on the
// node's path (one pending left sibling per right turn), so it travels with
// the node.
// PHI: phi receives the tree potential sum of every particle (no G).  It is
// a kernel argument of its own: inside TravArgs it changed the register
// allocation of the kernels without it (46 against 48 registers, 13% more
// instructions per node expansion, measured).
template <bool KDK, bool COUNT, int TPL, bool PHI>
__global__ void __launch_bounds__(TRAV_WARPS * 32)
bh_traverse_kernel(TravArgs a, float *__restrict__ phi, const int *__restrict__ parent, int s0, int s1) {
    __shared__ int4 stk[TRAV_WARPS][TRAV_STACK];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int wbase = s0 + (blockIdx.x * TRAV_WARPS + wid) * (32 * TPL);
    if (wbase >= s1) return;  // whole warp out of range
    const int n = a.n;
    int s[TPL];
    bool valid[TPL];
    Lane L[TPL];
    LanePhi W[TPL];
#pragma unroll
    for (int q = 0; q < TPL; ++q) {
        s[q] = wbase + 32 * q + lane;
        valid[q] = s[q] < s1;
        L[q].px = L[q].py = L[q].pz = 0.f;
        W[q].pm = 0.f;
        if (valid[q]) {
            const float4 p = __ldg(a.leaf + s[q]);
            L[q].px = p.x; L[q].py = p.y; L[q].pz = p.z;
            W[q].pm = p.w;
        }
        L[q].ax = L[q].ay = L[q].az = 0.f;
        L[q].PX = pack2(L[q].px, L[q].px);
        L[q].PY = pack2(L[q].py, L[q].py);
        L[q].PZ = pack2(L[q].pz, L[q].pz);
        L[q].AX = L[q].AY = L[q].AZ = 0ull;
        W[q].pw = 0.f;
        W[q].PW = 0ull;
        W[q].self = false;
        W[q].kp = (PHI && valid[q] && n >= 2) ? __ldg(parent + s[q]) - n : -1;
        L[q].n_int = L[q].n_test = L[q].drops = 0;
    }
    const f2 E2 = pack2(a.eps2, a.eps2), TH2 = pack2(a.theta2, a.theta2);
    unsigned overflow = 0, bad = 0, iters = 0;
    int top = 0;
    int k = 0, sp = 0;
    unsigned m[TPL];
    unsigned any = 0;
#pragma unroll
    for (int q = 0; q < TPL; ++q) m[q] = 0;
    if (n >= 2) {
        // The root is popped first, with an empty stack (sp = 0).
        const float4 R0 = __ldg(a.root), R1 = __ldg(a.root + 1);
#pragma unroll
        for (int q = 0; q < TPL; ++q) {
            const bool want = apply_room(L[q], visit_child<COUNT, PHI>(L[q], W[q], a, R0, R1.x, n, s[q], valid[q]),
                                         0, a.max_stack);
            m[q] = __ballot_sync(0xffffffffu, want);
            any |= m[q];
        }
    }
    while (any) {
        if ((unsigned)k >= (unsigned)(n - 1)) {  // never for a consistent tree
#pragma unroll
            for (int q = 0; q < TPL; ++q) bad += ((m[q] >> lane) & 1u);
            any = 0;
        } else {
            const ulonglong2 A = __ldg(reinterpret_cast<const ulonglong2 *>(a.inode + 3 * k));
            const ulonglong2 B = __ldg(reinterpret_cast<const ulonglong2 *>(a.inode + 3 * k + 1));
            const float4 C = __ldg(a.inode + 3 * k + 2);
            const int idL = __float_as_int(C.z), idR = __float_as_int(C.w);
            if (COUNT) ++iters;
            unsigned omL[TPL], omR[TPL], anyL = 0, anyR = 0;
            // Room for both children's pushes (the right child is popped at
            // depth sp + 1): one warp-uniform test; the per-child rule only
            // runs near max_stack.
            const bool room2 = sp + 3 <= a.max_stack;
#pragma unroll
            for (int q = 0; q < TPL; ++q) {
                const bool in = (m[q] >> lane) & 1u;
                bool wantR, wantL;
                visit_pair<COUNT, PHI>(L[q], W[q], a, A, B, C, s[q], in, E2, TH2, wantL, wantR);
                if (PHI) W[q].self |= in && k == W[q].kp;
                if (!room2) {
                    wantR = apply_room(L[q], wantR, sp + 1, a.max_stack);
                    wantL = apply_room(L[q], wantL, sp, a.max_stack);
                }
                omL[q] = __ballot_sync(0xffffffffu, wantL);
                omR[q] = __ballot_sync(0xffffffffu, wantR);
                anyL |= omL[q];
                anyR |= omR[q];
            }
            if (anyR) {  // expand the right child next; a left child waits on the stack
                if (anyL) {
                    if (top < TRAV_STACK) {
                        // Every lane stores the same entry (no lane predicate).
                        stk[wid][top] = make_int4(idL - n, (int)omL[0], TPL > 1 ? (int)omL[TPL - 1] : 0, sp);
                        ++top;
                    } else {
#pragma unroll
                        for (int q = 0; q < TPL; ++q) overflow += ((omL[q] >> lane) & 1u);
                    }
                }
                k = idR - n;
#pragma unroll
                for (int q = 0; q < TPL; ++q) m[q] = omR[q];
                sp = sp + 1;
                continue;
            }
            if (anyL) {  // only the left child was opened: expand it next directly
                k = idL - n;
#pragma unroll
                for (int q = 0; q < TPL; ++q) m[q] = omL[q];
                continue;
            }
            any = 0;
        }
        if (top > 0) {
            __syncwarp();
            const int4 e = stk[wid][--top];
            k = e.x;
            m[0] = (unsigned)e.y;
            if (TPL > 1) m[TPL - 1] = (unsigned)e.z;
            sp = e.w;
            any = m[0] | m[TPL - 1];
            __syncwarp();
        }
    }
    // Counters: one atomic per warp and counter.
    unsigned dsum = 0, osum = overflow, bsum = bad;
#pragma unroll
    for (int q = 0; q < TPL; ++q) dsum += L[q].drops;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        osum += __shfl_xor_sync(0xffffffffu, osum, o);
        bsum += __shfl_xor_sync(0xffffffffu, bsum, o);
    }
    if (COUNT) {
        unsigned isum = 0, tsum = 0;
#pragma unroll
        for (int q = 0; q < TPL; ++q) {
            isum += L[q].n_int;
            tsum += L[q].n_test;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            isum += __shfl_xor_sync(0xffffffffu, isum, o);
            tsum += __shfl_xor_sync(0xffffffffu, tsum, o);
        }
        if (lane == 0) {
            atomicAdd(a.diag + DIAG_NODE_READS, (unsigned long long)iters);
            atomicAdd(a.diag + DIAG_ROOT_READS, 1ull);
            atomicAdd(a.diag + DIAG_INTERACTIONS, (unsigned long long)isum);
            atomicAdd(a.diag + DIAG_TESTS, (unsigned long long)tsum);
        }
    }
    if (lane == 0) {
        if (dsum) atomicAdd(a.diag + DIAG_STACK_DROPS, (unsigned long long)dsum);
        if (osum) atomicAdd(a.diag + DIAG_STACK_OVERFLOW, (unsigned long long)osum);
        if (bsum) atomicAdd(a.diag + DIAG_BAD_TREE, (unsigned long long)bsum);
    }
    // Epilogue: scatter to the original particle index.
#pragma unroll
    for (int q = 0; q < TPL; ++q) {
        if (!valid[q]) continue;
        const uint32_t p = __ldg(a.order + s[q]);
        if (p >= (uint32_t)n) continue;
        float xl, xr, yl, yr, zl, zr;
        unpack2(L[q].AX, xl, xr);
        unpack2(L[q].AY, yl, yr);
        unpack2(L[q].AZ, zl, zr);
        float gx = a.G * (L[q].ax + (xl + xr)), gy = a.G * (L[q].ay + (yl + yr)),
              gz = a.G * (L[q].az + (zl + zr));
        if (a.pot.on) ext_acc_add(a.pot, L[q].px, L[q].py, L[q].pz, gx, gy, gz);
        if (PHI) phi[p] = lane_phi(W[q], a.eps2);
        if (KDK) {
            const float4 vh = a.vel[p];
            a.vel[p] = make_float4(kick(vh.x, gx, a.h), kick(vh.y, gy, a.h), kick(vh.z, gz, a.h), vh.w);
            a.acc[p] = make_float4(gx, gy, gz, 0.f);
        } else if (a.accumulate) {
            float4 o = a.acc[p];
            o.x += gx; o.y += gy; o.z += gz;
            a.acc[p] = o;
        } else {
            a.acc[p] = make_float4(gx, gy, gz, 0.f);
        }
    }
}

// Per-lane traversal: each lane walks the tree for its own target, exactly
// the reference's per-particle loop (:185-217) on the two-children records:
// expanding node k tests both children (the reference pushes both and then
// tests each when popped; the decisions do not depend on when a child is
// tested), continues into an opened right child directly (the reference pops
// the right child first) and keeps an opened left child on the lane's own
// shared-memory stack.  Lanes of a warp are at different nodes, so a warp
// runs as many iterations as its busiest lane, instead of the union of all
// its lanes' nodes as the warp-coherent kernel does.  Stack entries hold
// the internal index (25 bits) and the reference's stack depth d when the
// node is popped (7 bits): a right child is popped at d + 1 and a left child
// at d, which gives the max_stack rule exactly.  Layout [depth][thread]:
// every lane hits its own bank whatever its depth.
constexpr int LANE_THREADS = 128;
constexpr int LANE_KBITS = 25;
constexpr int LANE_MAX_STACK = 127;
// Below this n the traversal runs per lane by default (measured crossover
// between 100k and 300k particles on a disk).
constexpr int64_t LANE_AUTO_N = 131072;

template <bool KDK, bool COUNT, bool PHI>
__global__ void __launch_bounds__(LANE_THREADS)
bh_traverse_lane_kernel(TravArgs a, float *__restrict__ phi, const int *__restrict__ parent, int s0, int s1) {
    extern __shared__ int lstk[];  // [max_stack][LANE_THREADS]
    const int tid = threadIdx.x;
    const int n = a.n;
    const int s = s0 + blockIdx.x * LANE_THREADS + tid;
    const bool valid = s < s1;
    Lane L;
    LanePhi W;
    W.pw = 0.f;
    W.PW = 0ull;
    W.pm = 0.f;
    W.self = false;
    W.kp = (PHI && valid && n >= 2) ? __ldg(parent + s) - n : -1;
    L.px = L.py = L.pz = 0.f;
    if (valid) {
        const float4 p = __ldg(a.leaf + s);
        L.px = p.x; L.py = p.y; L.pz = p.z;
        W.pm = p.w;
    }
    L.ax = L.ay = L.az = 0.f;
    L.PX = pack2(L.px, L.px);
    L.PY = pack2(L.py, L.py);
    L.PZ = pack2(L.pz, L.pz);
    L.AX = L.AY = L.AZ = 0ull;
    L.n_int = L.n_test = L.drops = 0;
    const f2 E2 = pack2(a.eps2, a.eps2), TH2 = pack2(a.theta2, a.theta2);
    unsigned overflow = 0, bad = 0, reads = 0;
    int k = 0, d = 0, top = 0;
    bool active = false;
    if (valid && n >= 2) {
        // The root is popped first, with an empty stack (d = 0).
        const float4 R0 = __ldg(a.root), R1 = __ldg(a.root + 1);
        active = apply_room(L, visit_child<COUNT, PHI>(L, W, a, R0, R1.x, n, s, true), 0, a.max_stack);
    }
    for (;;) {
        if (!active) {
            if (top == 0) break;
            const unsigned e = (unsigned)lstk[(--top) * LANE_THREADS + tid];
            k = (int)(e & ((1u << LANE_KBITS) - 1u));
            d = (int)(e >> LANE_KBITS);
            active = true;
        }
        if ((unsigned)k >= (unsigned)(n - 1)) {  // never for a consistent tree
            ++bad;
            break;
        }
        const ulonglong2 A = __ldg(reinterpret_cast<const ulonglong2 *>(a.inode + 3 * k));
        const ulonglong2 B = __ldg(reinterpret_cast<const ulonglong2 *>(a.inode + 3 * k + 1));
        const float4 C = __ldg(a.inode + 3 * k + 2);
        if (COUNT) ++reads;
        bool wantL, wantR;
        visit_pair<COUNT, PHI>(L, W, a, A, B, C, s, true, E2, TH2, wantL, wantR);
        if (PHI) W.self |= k == W.kp;
        if (d + 3 > a.max_stack) {  // the rule only bites near max_stack
            wantR = apply_room(L, wantR, d + 1, a.max_stack);
            wantL = apply_room(L, wantL, d, a.max_stack);
        }
        if (wantR) {
            if (wantL) {
                if (top < a.max_stack) {
                    lstk[(top++) * LANE_THREADS + tid] =
                        (int)((unsigned)(__float_as_int(C.z) - n) | ((unsigned)d << LANE_KBITS));
                } else {
                    ++overflow;
                }
            }
            k = __float_as_int(C.w) - n;
            d = d + 1;
        } else if (wantL) {
            k = __float_as_int(C.z) - n;
        } else {
            active = false;
        }
    }
    // Counters: one atomic per warp and counter.
    unsigned dsum = L.drops, osum = overflow, bsum = bad;
    const int lane = tid & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        dsum += __shfl_xor_sync(0xffffffffu, dsum, o);
        osum += __shfl_xor_sync(0xffffffffu, osum, o);
        bsum += __shfl_xor_sync(0xffffffffu, bsum, o);
    }
    if (COUNT) {
        unsigned isum = L.n_int, tsum = L.n_test, rsum = reads, vsum = (valid && n >= 2) ? 1u : 0u;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            isum += __shfl_xor_sync(0xffffffffu, isum, o);
            tsum += __shfl_xor_sync(0xffffffffu, tsum, o);
            rsum += __shfl_xor_sync(0xffffffffu, rsum, o);
            vsum += __shfl_xor_sync(0xffffffffu, vsum, o);
        }
        if (lane == 0) {
            atomicAdd(a.diag + DIAG_NODE_READS, (unsigned long long)rsum);
            atomicAdd(a.diag + DIAG_ROOT_READS, (unsigned long long)vsum);
            atomicAdd(a.diag + DIAG_INTERACTIONS, (unsigned long long)isum);
            atomicAdd(a.diag + DIAG_TESTS, (unsigned long long)tsum);
        }
    }
    if (lane == 0) {
        if (dsum) atomicAdd(a.diag + DIAG_STACK_DROPS, (unsigned long long)dsum);
        if (osum) atomicAdd(a.diag + DIAG_STACK_OVERFLOW, (unsigned long long)osum);
        if (bsum) atomicAdd(a.diag + DIAG_BAD_TREE, (unsigned long long)bsum);
    }
    if (!valid) return;
    const uint32_t p = __ldg(a.order + s);
    if (p >= (uint32_t)n) return;
    float xl, xr, yl, yr, zl, zr;
    unpack2(L.AX, xl, xr);
    unpack2(L.AY, yl, yr);
    unpack2(L.AZ, zl, zr);
    float gx = a.G * (L.ax + (xl + xr)), gy = a.G * (L.ay + (yl + yr)), gz = a.G * (L.az + (zl + zr));
    if (a.pot.on) ext_acc_add(a.pot, L.px, L.py, L.pz, gx, gy, gz);
    if (PHI) phi[p] = lane_phi(W, a.eps2);
    if (KDK) {
        const float4 vh = a.vel[p];
        a.vel[p] = make_float4(kick(vh.x, gx, a.h), kick(vh.y, gy, a.h), kick(vh.z, gz, a.h), vh.w);
        a.acc[p] = make_float4(gx, gy, gz, 0.f);
    } else if (a.accumulate) {
        float4 o = a.acc[p];
        o.x += gx; o.y += gy; o.z += gz;
        a.acc[p] = o;
    } else {
        a.acc[p] = make_float4(gx, gy, gz, 0.f);
    }
}

// ------------------------------------------------------------- group walk
// Group walk (gb_bh_set_traversal 3): the warp's 32 key-consecutive targets
// share one walk and one interaction list.  A node is accepted for the whole
// group when size^2 < theta^2 (dmin^2 + eps^2), dmin the distance from its
// centre of mass to the group's bounding box; since every target is at
// least dmin away, each target then also passes the reference's own test
// (core/solvers/barnes_hut.py:204-210), so the group accepts a refinement of
// every target's node set: more, smaller nodes, never a coarser one.  Leaves
// are always accepted.  The walk keeps a stack of internal nodes in shared
// memory; each iteration pops up to 32 of them, one per lane, loads their
// two-children records and tests both children: accepted children go to the
// interaction list (compacted by ballots), opened ones are pushed.  The list
// is evaluated by every lane for its own target, two entries per packed
// .f32x2 instruction, whenever it fills and at the end.  Deterministic (no
// atomics); not the reference's per-particle node set, so its results are
// not bit-identical to the other shapes; the max_stack rule does not apply.
// A push that would overflow the warp's stack takes the child as a monopole
// instead and counts it in stack_overflow.
constexpr int GW_WARPS = 2;
constexpr int GW_STACK = 640;            // internal nodes per warp (the 1M disk peaks near 310)
constexpr int GW_LIST = 256;             // list entries per warp
constexpr int GW_FLUSH = GW_LIST - 64;   // an iteration appends at most 64

// The list holds entry pairs as {x0, x1, y0, y1} in la and {z0, z1, m0, m1}
// in lb (two arrays: the scalar stores of 32 consecutive entries meet 2-way
// bank conflicts, against 4-way with the two halves interleaved).
struct GwWarp {
    int stk[GW_STACK];
    float4 la[GW_LIST / 2];
    float4 lb[GW_LIST / 2];
};

__device__ __forceinline__ void gw_put(GwWarp &w, int j, float x, float y, float z, float m) {
    float *a = reinterpret_cast<float *>(&w.la[j >> 1]);
    float *b = reinterpret_cast<float *>(&w.lb[j >> 1]);
    const int h = j & 1;
    a[h] = x;
    a[2 + h] = y;
    b[h] = z;
    b[2 + h] = m;
}

// Squared distance from (x, y, z) to the box [lo, hi].
__device__ __forceinline__ float box_dist2(float x, float y, float z, float lx, float ly, float lz, float hx, float hy,
                                           float hz) {
    const float dx = fmaxf(fmaxf(lx - x, x - hx), 0.f);
    const float dy = fmaxf(fmaxf(ly - y, y - hy), 0.f);
    const float dz = fmaxf(fmaxf(lz - z, z - hz), 0.f);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, dx * dx));
}

// Adds entries [0, cnt) of the list (cnt even) to the lane's target.
template <bool PHI>
__device__ __forceinline__ void gw_eval(const GwWarp &w, int cnt, f2 PX, f2 PY, f2 PZ, f2 E2, f2 &AX, f2 &AY,
                                        f2 &AZ, f2 &PW) {
    const ulonglong2 *LA = reinterpret_cast<const ulonglong2 *>(w.la);
    const ulonglong2 *LB = reinterpret_cast<const ulonglong2 *>(w.lb);
#pragma unroll 4
    for (int q = 0; q < (cnt >> 1); ++q) {
        const ulonglong2 A = LA[q], B = LB[q];
        const f2 dx = sub2(A.x, PX), dy = sub2(A.y, PY), dz = sub2(B.x, PZ);
        f2 r2 = fma2(dx, dx, E2);
        r2 = fma2(dy, dy, r2);
        r2 = fma2(dz, dz, r2);
        const f2 inv = rsqrt2(r2);
        const f2 mi = mul2(B.y, inv);
        const f2 sc = mul2(mi, mul2(inv, inv));
        AX = fma2(sc, dx, AX);
        AY = fma2(sc, dy, AY);
        AZ = fma2(sc, dz, AZ);
        if (PHI) PW = add2(PW, mi);
    }
}

// One group: leaves [g0, g0 + size) (size <= 32), lane l walks with target
// g0 + l.
template <bool KDK, bool COUNT, bool PHI>
__device__ __forceinline__ void gw_group(GwWarp &w, const TravArgs &a, float *__restrict__ phi, int g0, int size,
                                         int lane, unsigned &reads, unsigned &evals, unsigned &overflow,
                                         unsigned &bad) {
    const int n = a.n;
    const int s = g0 + lane;
    const bool valid = lane < size;
    float px = 0.f, py = 0.f, pz = 0.f, pm = 0.f;
    if (valid) {
        const float4 p = __ldg(a.leaf + s);
        px = p.x; py = p.y; pz = p.z; pm = p.w;
    }
    // The group's bounding box.
    float lx = valid ? px : INFINITY, ly = valid ? py : INFINITY, lz = valid ? pz : INFINITY;
    float hx = valid ? px : -INFINITY, hy = valid ? py : -INFINITY, hz = valid ? pz : -INFINITY;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
        ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
        lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
        hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
        hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
    }
    const f2 PX = pack2(px, px), PY = pack2(py, py), PZ = pack2(pz, pz), E2 = pack2(a.eps2, a.eps2);
    f2 AX = 0ull, AY = 0ull, AZ = 0ull, PW = 0ull;
    const unsigned lt = (1u << lane) - 1u;
    unsigned selfbits = 0;
    int cnt = 0, top = 0;
    if (n >= 2) {
        // The root, tested for the whole group: a monopole, or its children.
        const float4 R0 = __ldg(a.root), R1 = __ldg(a.root + 1);
        const float d2 = box_dist2(R0.x, R0.y, R0.z, lx, ly, lz, hx, hy, hz);
        if (R1.x < a.theta2 * (d2 + a.eps2)) {
            if (lane == 0) gw_put(w, 0, R0.x, R0.y, R0.z, R0.w);
            cnt = 1;
        } else {
            if (lane == 0) w.stk[0] = 0;
            top = 1;
        }
        __syncwarp();
    }
    // A consistent tree expands each internal node at most once per group,
    // so more than n - 1 iterations means a corrupted tree: stop.
    for (int iter = 0; top > 0; ++iter) {
        if (iter >= n) {
            bad += lane == 0 ? 1u : 0u;
            break;
        }
        const int take = min(top, 32);
        top -= take;
        bool act = lane < take;
        const int k = act ? w.stk[top + lane] : 0;
        __syncwarp();  // the popped entries are read before pushes reuse them
        if (act && (unsigned)k >= (unsigned)(n - 1)) {  // never for a consistent tree
            ++bad;
            act = false;
        }
        float4 A = make_float4(0.f, 0.f, 0.f, 0.f), B = A, C = A;
        if (act) {
            A = __ldg(a.inode + 3 * k);      // {x_L, x_R, y_L, y_R}
            B = __ldg(a.inode + 3 * k + 1);  // {z_L, z_R, m_L, m_R}
            C = __ldg(a.inode + 3 * k + 2);  // {size2_L, size2_R, id_L, id_R}
        }
        if (COUNT) reads += __popc(__ballot_sync(0xffffffffu, act));
        // A leaf child carries size2 = -1 and is always accepted.
        const bool accL = act && C.x < a.theta2 * (box_dist2(A.x, A.z, B.x, lx, ly, lz, hx, hy, hz) + a.eps2);
        const bool accR = act && C.y < a.theta2 * (box_dist2(A.y, A.w, B.y, lx, ly, lz, hx, hy, hz) + a.eps2);
        const bool openL = act && !accL, openR = act && !accR;
        const int idL = __float_as_int(C.z), idR = __float_as_int(C.w);
        const unsigned bL = __ballot_sync(0xffffffffu, accL), bR = __ballot_sync(0xffffffffu, accR);
        if (accL) gw_put(w, cnt + __popc(bL & lt), A.x, A.z, B.x, B.z);
        if (accR) gw_put(w, cnt + __popc(bL) + __popc(bR & lt), A.y, A.w, B.y, B.w);
        cnt += __popc(bL) + __popc(bR);
        if (PHI) {
            // Own leaves of the group's targets in the list: their terms are
            // removed from the potential at the end.
            unsigned bit = 0;
            if (accL && (unsigned)(idL - g0) < (unsigned)size) bit |= 1u << (idL - g0);
            if (accR && (unsigned)(idR - g0) < (unsigned)size) bit |= 1u << (idR - g0);
            selfbits |= __reduce_or_sync(0xffffffffu, bit);
        }
        const unsigned cL = __ballot_sync(0xffffffffu, openL), cR = __ballot_sync(0xffffffffu, openR);
        const int np = __popc(cL) + __popc(cR);
        if (top + np <= GW_STACK) {
            if (openL) w.stk[top + __popc(cL & lt)] = idL - n;
            if (openR) w.stk[top + __popc(cL) + __popc(cR & lt)] = idR - n;
            top += np;
        } else {  // no room: the opened children enter the list as monopoles
            if (openL) gw_put(w, cnt + __popc(cL & lt), A.x, A.z, B.x, B.z);
            if (openR) gw_put(w, cnt + __popc(cL) + __popc(cR & lt), A.y, A.w, B.y, B.w);
            cnt += np;
            overflow += np;
        }
        __syncwarp();
        if (cnt > GW_FLUSH) {
            if ((cnt & 1) && lane == 0) gw_put(w, cnt, 0.f, 0.f, 0.f, 0.f);
            __syncwarp();
            gw_eval<PHI>(w, cnt + (cnt & 1), PX, PY, PZ, E2, AX, AY, AZ, PW);
            if (COUNT) evals += cnt * size;
            cnt = 0;
            __syncwarp();  // the list is read before the next appends
        }
    }
    if (cnt > 0) {
        if ((cnt & 1) && lane == 0) gw_put(w, cnt, 0.f, 0.f, 0.f, 0.f);
        __syncwarp();
        gw_eval<PHI>(w, cnt + (cnt & 1), PX, PY, PZ, E2, AX, AY, AZ, PW);
        if (COUNT) evals += cnt * size;
    }
    __syncwarp();  // the next group reuses the stack and the list
    if (!valid) return;
    const uint32_t p = __ldg(a.order + s);
    if (p >= (uint32_t)n) {
        ++bad;
        return;
    }
    float xl, xr, yl, yr, zl, zr;
    unpack2(AX, xl, xr);
    unpack2(AY, yl, yr);
    unpack2(AZ, zl, zr);
    float gx = a.G * (xl + xr), gy = a.G * (yl + yr), gz = a.G * (zl + zr);
    if (a.pot.on) ext_acc_add(a.pot, px, py, pz, gx, gy, gz);
    if (PHI) {
        float wl, wr;
        unpack2(PW, wl, wr);
        float pw = wl + wr;
        if ((selfbits >> lane) & 1u) pw -= pm * rsqrt_approx(a.eps2);  // the term the list added
        phi[p] = pw;
    }
    if (KDK) {
        const float4 vh = a.vel[p];
        a.vel[p] = make_float4(kick(vh.x, gx, a.h), kick(vh.y, gy, a.h), kick(vh.z, gz, a.h), vh.w);
        a.acc[p] = make_float4(gx, gy, gz, 0.f);
    } else if (a.accumulate) {
        float4 o = a.acc[p];
        o.x += gx; o.y += gy; o.z += gz;
        a.acc[p] = o;
    } else {
        a.acc[p] = make_float4(gx, gy, gz, 0.f);
    }
}

// Warp w walks the groups whose first leaf lies in [32 w, 32 w + 32) (gsize
// from the Karras kernel), one after the other.
// 32 resident warps per SM (64 registers, 13 KB of shared memory per CTA of
// 2 warps): 7.8% less time than 24 warps on the 1M disk; CTAs of 2 warps
// against 4: 1.3% less (a CTA retires when its slowest warp is done).
template <bool KDK, bool COUNT, bool PHI>
__global__ void __launch_bounds__(GW_WARPS * 32, 16)
bh_group_kernel(TravArgs a, const int *__restrict__ gsize, float *__restrict__ phi, int s0, int s1) {
    __shared__ GwWarp sw[GW_WARPS];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    GwWarp &w = sw[wid];
    // Groups whose first leaf lies in [s0, s1) (a group may end past s1).
    const int c0 = s0 + (blockIdx.x * GW_WARPS + wid) * 32;
    if (c0 >= s1) return;  // whole warp out of range
    const int n = a.n;
    int gs = (c0 + lane < s1) ? __ldg(gsize + c0 + lane) : 0;
    if (n == 1 && lane == 0) gs = 1;  // a single particle: no internal node, one group
    unsigned starts = __ballot_sync(0xffffffffu, gs > 0 && gs <= GW_GROUP);
    unsigned reads = 0, evals = 0, overflow = 0, bad = 0, ngroups = 0;
    while (starts) {
        const int j = __ffs(starts) - 1;
        starts &= starts - 1u;
        const int size = min(__shfl_sync(0xffffffffu, gs, j), n - (c0 + j));
        gw_group<KDK, COUNT, PHI>(w, a, phi, c0 + j, size, lane, reads, evals, overflow, bad);
        ++ngroups;
    }
    const unsigned bsum = __reduce_add_sync(0xffffffffu, bad);
    if (lane == 0) {
        if (overflow) atomicAdd(a.diag + DIAG_STACK_OVERFLOW, (unsigned long long)overflow);
        if (bsum) atomicAdd(a.diag + DIAG_BAD_TREE, (unsigned long long)bsum);
        if (COUNT) {
            atomicAdd(a.diag + DIAG_NODE_READS, (unsigned long long)reads);
            atomicAdd(a.diag + DIAG_ROOT_READS, (unsigned long long)ngroups);
            atomicAdd(a.diag + DIAG_INTERACTIONS, (unsigned long long)evals);
            atomicAdd(a.diag + DIAG_TESTS, 2ull * reads + ngroups);
        }
    }
}

}  // namespace gb
