// Building blocks shared by the single-system and batched direct-sum kernels.
#pragma once

#include <algorithm>
#include <vector>

#include "gb_common.cuh"

namespace gb {

// ------------------------------------------------------------ stream-K plan
// First unit of CTA c when U units are split into P equal contiguous runs.
__device__ __forceinline__ int64_t unit_begin(int64_t U, int64_t P, int64_t c) { return U * c / P; }
// CTA whose unit run contains unit u: the largest c with U*c/P <= u.
__device__ __forceinline__ int64_t unit_owner(int64_t U, int64_t P, int64_t u) {
    return ((u + 1) * P - 1) / U;
}

// Units are (target supertile of warps*32*2*np targets) x (source chunk of
// unit_src sources), supertile-major; smax bounds the supertiles one CTA run
// touches, so a CTA's partials fit smax slots.
// nt >= 0: only the targets of a range of nt particles (sources: all n).
struct DirectPlan {
    int np, warps;
    int64_t n, nt, st_size, num_st, num_ju, U, P;
    int smax;
};

static inline void make_plan(int64_t n, int np, int warps, int64_t P, DirectPlan *p, int unit_src = 0,
                             int64_t nt = -1) {
    p->np = np;
    p->warps = warps;
    p->n = n;
    p->nt = nt >= 0 ? nt : n;
    p->st_size = (int64_t)warps * 32 * 2 * np;
    p->num_st = (p->nt + p->st_size - 1) / p->st_size;
    const int64_t ju = unit_src > 0 ? unit_src : (int64_t)warps * 32;
    p->num_ju = (n + ju - 1) / ju;
    p->U = p->num_st * p->num_ju;
    p->P = P < 1 ? 1 : (P > p->U ? p->U : P);
    const int64_t per = (p->U + p->P - 1) / p->P;
    p->smax = (int)((per + p->num_ju - 1) / p->num_ju + 1);
}

// Scratch (float4 elements) a plan needs for its partials: (hi, lo) per
// target slot.
static inline int64_t plan_partials(const DirectPlan &p) { return 2 * p.P * p.smax * p.st_size; }

// Adds the accelerations of JU staged sources (src, {x, y, z, m}) on K
// targets per lane into AX/AY/AZ (FP32; G applied later):
//   d = x_j - x_i, r2 = d.d + eps2, a += m_j rsqrt(r2)^3 d
// (core/solvers/gravity.py:22-25).  Zero-mass padding sources add zero.
// PHI also adds the potential terms m_j rsqrt(r2) into PW (the product the
// force term starts from), the self pair included (the caller removes it).
template <int K, int JU, bool PHI = false>
__device__ __forceinline__ void interact_chunk(const float4 *src, const float (&X)[K], const float (&Y)[K],
                                               const float (&Z)[K], float (&AX)[K], float (&AY)[K],
                                               float (&AZ)[K], float (&PW)[K], float eps2) {
#pragma unroll 4
    for (int jj = 0; jj < JU; ++jj) {
        const float4 sj = src[jj];
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const float dx = sj.x - X[q], dy = sj.y - Y[q], dz = sj.z - Z[q];
            const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, eps2)));
            const float inv = rsqrt_approx(r2);
            const float mi = sj.w * inv;
            const float sc = mi * (inv * inv);
            AX[q] = __fmaf_rn(sc, dx, AX[q]);
            AY[q] = __fmaf_rn(sc, dy, AY[q]);
            AZ[q] = __fmaf_rn(sc, dz, AZ[q]);
            if (PHI) PW[q] += mi;
        }
    }
}

// The potential term a particle adds to its own sum in the per-target
// passes: d = 0 gives r2 = eps2 exactly, so the term is m * rsqrt(eps2)
// rounded as the pair loop rounds it.  The fix-up subtracts it, which gives
// the j != i sum of potential_energy (core/solvers/gravity.py:51-52).
__device__ __forceinline__ float self_phi_term(float m, float eps2) { return m * rsqrt_approx(eps2); }

// Sources per stream-K unit of the scalar force kernel: one warp-width
// sub-chunk, so CTA runs split the work evenly even at small N.
constexpr int SCALAR_UNIT = 32;

// ------------------------------------------------ unordered tile pairs
// Largest s in [0, nsys) with base[s] <= x (base is non-decreasing).
__device__ __forceinline__ int find_base(const int64_t *__restrict__ base, int nsys, int64_t x) {
    int lo = 0, hi = nsys - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(base + mid) <= x) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Tile pairs (I <= J) of nt tiles numbered row-major: row I starts at
// sym_base(I); sym_row(p) is the row of pair p.
__device__ __forceinline__ int64_t sym_base(int64_t I, int64_t nt) { return I * nt - I * (I - 1) / 2; }

__device__ __forceinline__ int64_t sym_row(int64_t p, int64_t nt) {
    int64_t lo = 0, hi = nt - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi + 1) >> 1;
        if (sym_base(mid, nt) <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Merges the (hi, lo) partials of one target written by CTAs c_lo..c_hi at
// slots slot_of(c) (Kahan, fixed CTA order) and returns the sum.
template <typename SlotFn>
__device__ __forceinline__ float3 merge_partials(const float4 *__restrict__ part, int64_t c_lo, int64_t c_hi,
                                                 SlotFn slot_of) {
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
    for (int64_t c = c_lo; c <= c_hi; ++c) {
        const int64_t slot = slot_of(c);
        const float4 hi = part[2 * slot];
        const float4 lo = part[2 * slot + 1];
        kahan_add(sx, cx, hi.x);
        kahan_add(sx, cx, lo.x);
        kahan_add(sy, cy, hi.y);
        kahan_add(sy, cy, lo.y);
        kahan_add(sz, cz, hi.z);
        kahan_add(sz, cz, lo.z);
    }
    return make_float3(sx - cx, sy - cy, sz - cz);
}

// Closing kick and in-place state write-back of one KDK step: the particle's
// predicted position and half-kicked velocity are recomputed exactly as the
// loaders computed them.
__device__ __forceinline__ void kdk_writeback(float4 *xm, float4 *vel, float4 *acc, int64_t i, float4 an, float h,
                                              float dt) {
    const float4 x = xm[i], v = vel[i], a0 = acc[i];
    const float vhx = kick(v.x, a0.x, h), vhy = kick(v.y, a0.y, h), vhz = kick(v.z, a0.z, h);
    xm[i] = make_float4(drift(x.x, vhx, dt), drift(x.y, vhy, dt), drift(x.z, vhz, dt), x.w);
    vel[i] = make_float4(kick(vhx, an.x, h), kick(vhy, an.y, h), kick(vhz, an.z, h), v.w);
    acc[i] = an;
}

// Bands of tile rows for the tile-pair passes: band b covers rows
// [rows[b], rows[b + 1]) and at most `budget` tile pairs (one row more when a
// single row exceeds it).  Returns the largest band's pair count.
static inline int64_t sym_bands(int64_t nt, int64_t budget, std::vector<int64_t> &rows) {
    rows.assign(1, 0);
    int64_t max_pairs = 0, pairs = 0;
    for (int64_t I = 0; I < nt; ++I) {
        if (pairs > 0 && pairs + (nt - I) > budget) {
            rows.push_back(I);
            max_pairs = std::max(max_pairs, pairs);
            pairs = 0;
        }
        pairs += nt - I;
    }
    rows.push_back(nt);
    return std::max(max_pairs, pairs);
}

static inline int64_t host_sym_base(int64_t I, int64_t nt) { return I * nt - I * (I - 1) / 2; }

// Symmetric (tile-pair) scratch above this size is not used: the callers
// fall back to their per-target forms.
constexpr int64_t SYM_MAX_BYTES = 3LL << 30;

}  // namespace gb

// Steps in the multi-step KDK graph of gb_direct_kdk.
constexpr int GRAPH_STEPS = 8;

// Direct-sum handle (opaque in the C ABI), shared by the direct-sum and
// adjoint translation units.
struct gb_direct {
    int device;
    int sms;
    int64_t n_max;
    int np, warps, ctas_per_sm;  // tile shape (ctas_per_sm 0 = occupancy max)
    int packed;                  // 2: symmetric .f32x2 pairs, 1: .f32x2 per target, 0: scalar FP32
    float4 *part;
    int64_t part_cap;            // float4 elements
    int *st0tab;                 // first supertile of each CTA of the last launch
    int st0_cap;
    float *phi;                  // n_max floats (energy scratch)
    double2 *epart;              // energy block partials
    int epart_cap;
    unsigned long long *diag;
    uint64_t launches;  // kernels launched by this handle (host count)
    float4 *sym;        // symmetric adjoint partials (allocated on first use)
    int64_t sym_cap;    // float4 elements
    int adj_variant;    // 2: symmetric packed, 1: symmetric scalar, 0: one pass per target
    int64_t sym_band;   // symmetric force pass: tile-pair slot bytes per band at most
    // KDK steps captured as CUDA graphs (gb_direct_kdk with GB_USE_GRAPH):
    // gexec[0] one step, gexec[1] GRAPH_STEPS steps, gexec[2] one step that
    // also writes the potential (gb_direct_kdk_phi), replayed on the
    // handle's own stream; glaunches[g] = kernels per replay of slot g; a
    // slot is captured again when its key changes.
    cudaStream_t gstream;
    cudaEvent_t gev_in, gev_out;
    cudaGraphExec_t gexec[3];
    uint64_t glaunches[3];
    struct Key {
        const void *xm, *vel, *acc, *sym, *phi;
        int64_t n, sym_band;
        float G, eps2, dt;
        int plain, np, warps, ctas_per_sm, packed;
        bool operator==(const Key &o) const {
            return xm == o.xm && vel == o.vel && acc == o.acc && sym == o.sym && phi == o.phi && n == o.n &&
                   sym_band == o.sym_band && G == o.G && eps2 == o.eps2 && dt == o.dt && plain == o.plain &&
                   np == o.np && warps == o.warps && ctas_per_sm == o.ctas_per_sm && packed == o.packed;
        }
    } gkey[3];
};

namespace gb {

// Grows the handle's tile-pair scratch (shared by the symmetric force pass
// and the symmetric adjoint, which run in stream order) to need float4s.
inline int ensure_sym(gb_direct *h, int64_t need) {
    if (need <= h->sym_cap) return GB_OK;
    if (h->sym) cudaFree(h->sym);
    h->sym = nullptr;
    h->sym_cap = 0;
    if (cudaMalloc(&h->sym, sizeof(float4) * need) != cudaSuccess)
        return fail(GB_ENOMEM, "tile-pair scratch (%lld bytes)", (long long)(need * 16));
    h->sym_cap = need;
    return GB_OK;
}

// Symmetric direct-sum pass (gb_direct_sym.cu): mode 0 acceleration, 1
// fused KDK, 2 the potential sums into phi.  Returns GB_OK with
// *done = false when the scratch it needs passes SYM_MAX_BYTES (the caller
// then runs the per-target pass).
int run_direct_sym(gb_direct *h, int mode, const float4 *xm, float4 *vel, float4 *acc, float *phi, int64_t n,
                   float G, float eps2, float dt, int flags, cudaStream_t s, const ExtPot &pot, bool *done);
// Sizes the tile-pair scratch run_direct_sym needs for n particles (nothing
// when that passes SYM_MAX_BYTES).
int reserve_direct_sym(gb_direct *h, int64_t n);

// The symmetric pass over many systems at once (gb_batch_set_variant 1).
// Device tables of nsys + 1 entries: particle offsets, unit bases (units of
// system s: its tile pairs x Q slices), column-slot bases (its tile pairs)
// and fix-up block bases (ceil(n_s / 32) blocks per system), and the system
// of every fix-up block.  scratch holds NU row slots and NPtot column slots
// of SYM_TILE float4s, then the unit counter.
constexpr int SYM_TILE = 512;
struct SymBatch {
    const int64_t *off, *ubase, *cbase, *fbase;
    const int *fsys;
    int nsys, Q;
    int64_t NU, NPtot, nfb, P;
    float4 *scratch;
};
// Source slices per tile pair (at most qmax) for a pass of the given
// tile-pair count over `slots` resident CTAs, and the symmetric force
// kernel's resident CTAs and slices for such a pass.
int direct_sym_slices(int64_t pairs, int64_t slots, int qmax);
struct SymShape {
    int Q;
    int64_t slots;
};
SymShape direct_sym_shape(int sms, int64_t pairs);
int run_batch_sym(const SymBatch &b, int mode, const float4 *xm, float4 *vel, float4 *acc, float G, float eps2,
                  float dt, int flags, cudaStream_t s);

}  // namespace gb
