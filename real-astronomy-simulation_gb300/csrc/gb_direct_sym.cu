// Symmetric direct-sum forces: every unordered pair {t, s} is evaluated
// once and applied to both particles (Newton's third law), in packed
// FP32x2 arithmetic.  The sum is that of compute_acc_direct
// (core/solvers/gravity.py:13-26):
//   d = x_s - x_t, r2 = d.d + eps2, c = rsqrt(r2)^3,
//   a_t += m_s c d,   a_s -= m_t c d,
// with the self pair (d = 0) adding nothing.  Per two pairs: 16 packed
// instructions and 2 rsqrt, against 24 FP32 instructions and 2 rsqrt for
// two ordered pairs of the per-target kernel.
//
// The schedule is that of adjoint_vjp_sym2_kernel with a wider CTA shape:
// tiles of 512 particles, 2 warps, 8 targets per lane as four packed pairs
// (targets q = 0 .. 7 of lane l in warp w: 256 w + 32 q + l); CTAs take
// units (tile pair I <= J, one of Q <= 8 source slices of tile J) from an
// atomic counter; in round r warp w takes source group (G/2 w + r) mod G of
// the slice (G = 16/Q groups of 32) and at step k lane l source
// 32 g + (l + k) mod 32, so the per-source shared-memory sums have one
// writer at a time.  Each unit writes its own
// row slot (tile I's sums over the slice) and its slice of the pair's column
// slot; the fix-up adds a particle's slots in a fixed order (Kahan unless
// GB_PLAIN_FP32), scales by G and writes the result (or, fused KDK, applies
// the closing kick and writes x', v', a').  In the fused KDK form both sides
// load the leapfrog prediction x' = x + (v + a dt/2) dt with the same FMAs as
// the per-target kernel, so the two forms see identical positions.
//
// A system whose slots pass the handle's band budget runs in bands of tile
// rows (one kernel and one fix-up per band, running sums in between); the
// BATCH form runs the tile pairs of many systems in one launch.  Rounds over
// a system's last-tile padding (zero-mass records) are skipped.
#include <algorithm>
#include <vector>

#include "gb_direct_core.cuh"

namespace gb {

constexpr int DS_T = SYM_TILE;
constexpr int DS_K_UNROLL = 4;  // steps of a round unrolled (1-4 measured within 3%)
constexpr int DS_ACC = 0, DS_KDK = 1, DS_PHI = 2;

// CTA shape for H packed target pairs per lane (2H targets): 8/H warps
// cover one tile of 512 targets.  The pass runs H = 4 (2 warps, 128
// registers at 8 resident CTAs per SM): against H = 2 (4 warps, 80
// registers at 6) it halves the per-source overhead per pair (staging, the
// shared-memory sum and its 6 scalar adds), and with up to 8 source slices
// per tile pair its units stay short enough for small systems too.
template <int H>
struct DsShape {
    static constexpr int WARPS = 8 / H, WT = 64 * H, MIN_CTAS = H == 4 ? 8 : 6;
    static constexpr int QMAX = 16 / WARPS;  // each warp of a round takes its own source group
    static_assert(WARPS * WT == DS_T, "a CTA's warps cover one tile");
};
constexpr int DS_H = 4;

struct DsArgs {
    const float4 *__restrict__ xm;
    const float4 *__restrict__ vel;  // fused KDK: v and a of the step start
    const float4 *__restrict__ acc;
    float4 *__restrict__ rowpart;  // NU x DS_T (one row slot per unit)
    float4 *__restrict__ colpart;  // tile pairs x DS_T
    unsigned long long *counter;   // zero at launch
    int64_t n, nt, NU;             // one system: particles, tiles; units in all
    int64_t p0;                    // one system: first tile pair of the band
    // Many systems (BATCH): nsys + 1 particle offsets, unit bases and
    // column-slot bases; units are numbered system after system.
    const int64_t *__restrict__ off;
    const int64_t *__restrict__ ubase;
    const int64_t *__restrict__ cbase;
    int nsys;
    float eps2, h, dt;
};

template <int MODE>
__device__ __forceinline__ float4 ds_load(const DsArgs &a, int64_t o, int64_t n_s, int64_t i) {
    if (i >= n_s) return make_float4(0.f, 0.f, 0.f, 0.f);
    float4 x = __ldg(a.xm + o + i);
    if (MODE == DS_KDK) x = predict_xm(x, __ldg(a.vel + o + i), __ldg(a.acc + o + i), a.h, a.dt);
    return x;
}

// One round: lane l at step k takes source jj = 32 g + (l + k) mod 32 of the
// staged tile against its 2H targets.  DIAG zeroes the pairs with target
// index >= source index (diagonal tile).  PHI also sums the pair's
// potential terms, phi_t += m_s / |d| into NW and phi_s += m_t / |d| into
// sacc.w (one packed FMA per side), the sums of potential_energy
// (core/solvers/gravity.py:47-55) taken from the same pass.
template <bool DIAG, int H, bool PHI>
__device__ __forceinline__ void ds_round(const float4 *__restrict__ sxm, float4 *sacc, int g, int lane, int wib,
                                         f2 EPS2, const f2 (&TX)[H], const f2 (&TY)[H], const f2 (&TZ)[H],
                                         const f2 (&TM)[H], f2 (&NX)[H], f2 (&NY)[H], f2 (&NZ)[H],
                                         f2 (&NW)[H]) {
#pragma unroll DS_K_UNROLL
    for (int k = 0; k < 32; ++k) {
        const int jj = g * 32 + ((lane + k) & 31);
        const float4 xs = sxm[jj];
        const f2 sx = pack2(xs.x, xs.x), sy = pack2(xs.y, xs.y), sz = pack2(xs.z, xs.z);
        const f2 sm = pack2(xs.w, xs.w);
        f2 PX = 0ull, PY = 0ull, PZ = 0ull, PW = 0ull;
#pragma unroll
        for (int h = 0; h < H; ++h) {
            const f2 dx = sub2(sx, TX[h]), dy = sub2(sy, TY[h]), dz = sub2(sz, TZ[h]);
            const f2 r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, EPS2)));
            f2 inv = rsqrt2(r2);
            if (DIAG) {  // a zero inv zeroes the pair's force and potential terms
                float c0, c1;
                unpack2(inv, c0, c1);
                const int t0 = DsShape<H>::WT * wib + 64 * h + lane;
                c0 = t0 < jj ? c0 : 0.f;
                c1 = t0 + 32 < jj ? c1 : 0.f;
                inv = pack2(c0, c1);
            }
            const f2 c = mul2(inv, mul2(inv, inv));
            const f2 ct = mul2(sm, c);     // m_s c: the targets' side
            const f2 cs = mul2(TM[h], c);  // m_t c: the source's side (subtracted)
            NX[h] = fma2(ct, dx, NX[h]);
            NY[h] = fma2(ct, dy, NY[h]);
            NZ[h] = fma2(ct, dz, NZ[h]);
            PX = fma2(cs, dx, PX);
            PY = fma2(cs, dy, PY);
            PZ = fma2(cs, dz, PZ);
            if (PHI) {
                NW[h] = fma2(sm, inv, NW[h]);
                PW = fma2(TM[h], inv, PW);
            }
        }
        float4 acc = sacc[jj];
        float lo, hi;
        unpack2(PX, lo, hi);
        acc.x -= lo + hi;
        unpack2(PY, lo, hi);
        acc.y -= lo + hi;
        unpack2(PZ, lo, hi);
        acc.z -= lo + hi;
        if (PHI) {
            unpack2(PW, lo, hi);
            acc.w += lo + hi;
        }
        sacc[jj] = acc;
        __syncwarp();
    }
}

// The potential form of a round: phi_t += m_s / |d|, phi_s += m_t / |d|
// (|d|^2 = d.d + eps2), the sum of potential_energy
// (core/solvers/gravity.py:47-55); the target sums live in NX, the source
// sums are added to sacc.x.  DIAG keeps the pairs t < s, so a particle
// never meets itself (the reference skips j == i).
template <bool DIAG, int H>
__device__ __forceinline__ void ds_round_phi(const float4 *__restrict__ sxm, float4 *sacc, int g, int lane, int wib,
                                             f2 EPS2, const f2 (&TX)[H], const f2 (&TY)[H], const f2 (&TZ)[H],
                                             const f2 (&TM)[H], f2 (&NX)[H]) {
#pragma unroll DS_K_UNROLL
    for (int k = 0; k < 32; ++k) {
        const int jj = g * 32 + ((lane + k) & 31);
        const float4 xs = sxm[jj];
        const f2 sx = pack2(xs.x, xs.x), sy = pack2(xs.y, xs.y), sz = pack2(xs.z, xs.z);
        const f2 sm = pack2(xs.w, xs.w);
        f2 PW = 0ull;
#pragma unroll
        for (int h = 0; h < H; ++h) {
            const f2 dx = sub2(sx, TX[h]), dy = sub2(sy, TY[h]), dz = sub2(sz, TZ[h]);
            const f2 r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, EPS2)));
            f2 inv = rsqrt2(r2);
            if (DIAG) {
                float c0, c1;
                unpack2(inv, c0, c1);
                const int t0 = DsShape<H>::WT * wib + 64 * h + lane;
                c0 = t0 < jj ? c0 : 0.f;
                c1 = t0 + 32 < jj ? c1 : 0.f;
                inv = pack2(c0, c1);
            }
            NX[h] = fma2(sm, inv, NX[h]);
            PW = fma2(TM[h], inv, PW);
        }
        float4 acc = sacc[jj];
        float lo, hi;
        unpack2(PW, lo, hi);
        acc.x += lo + hi;
        sacc[jj] = acc;
        __syncwarp();
    }
}

// PHI (one system, MODE DS_ACC or DS_KDK): the pass also returns the
// potential sums of its positions, in the slots' .w.
template <int Q, int MODE, bool BATCH, int H, bool PHI>
__global__ void __launch_bounds__(DsShape<H>::WARPS * 32, DsShape<H>::MIN_CTAS) direct_sym_kernel(DsArgs a) {
    constexpr int G = 16 / Q, SPAN = G * 32;
    constexpr int WARPS = DsShape<H>::WARPS, WT = DsShape<H>::WT;
    static_assert(G >= WARPS, "each warp of a round takes its own source group");
    __shared__ float4 sxm[DS_T], sacc[DS_T];
    // The unit and, for a batch, its system's offset, size, local unit and
    // column-slot base (decoded once by thread 0).
    __shared__ long long s_unit, s_off, s_n, s_local, s_cb;
    __shared__ int s_gend, s_ntgt;  // source groups and targets of the unit that hold particles
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, tid = threadIdx.x;
    const f2 EPS2 = pack2(a.eps2, a.eps2);
    for (;;) {
        __syncthreads();  // the previous unit is done with the shared state
        if (tid == 0) {
            const long long u = (long long)atomicAdd(a.counter, 1ull);
            s_unit = u;
            if (BATCH && u < a.NU) {
                const int sy = find_base(a.ubase, a.nsys, u);
                s_off = __ldg(a.off + sy);
                s_n = __ldg(a.off + sy + 1) - s_off;
                s_local = u - __ldg(a.ubase + sy);
                s_cb = __ldg(a.cbase + sy);
            }
        }
        __syncthreads();
        f2 TX[H], TY[H], TZ[H], TM[H], NX[H], NY[H], NZ[H], NW[H];
        bool diag;
        int gbase;
        {
            // Unit bookkeeping is re-read from shared memory after the pair
            // loop, so none of it stays in registers across the loop.
            const int64_t u = s_unit;
            if (u >= a.NU) break;
            const int64_t o = BATCH ? s_off : 0, n_s = BATCH ? s_n : a.n;
            const int64_t nt = BATCH ? (n_s + DS_T - 1) / DS_T : a.nt;
            const int64_t lu = BATCH ? s_local : u;
            const int64_t p = lu / Q;
            const int sl = (int)(lu - p * Q);
            const int64_t pg = BATCH ? p : a.p0 + p;  // pair index in the system's triangle
            const int64_t I = sym_row(pg, nt);
            const int64_t J = I + (pg - sym_base(I, nt));
            diag = J == I;
            gbase = sl * G;
            // Padding of the system's last tile: source groups past the last
            // particle, and warps whose 128 targets are all past it, hold
            // zero-mass records only; their rounds would add exact zeros.
            // The bounds live in shared memory, not in registers.
            if (tid == 0) {
                s_gend = (int)((min(n_s - J * DS_T, (int64_t)DS_T) + 31) / 32);
                s_ntgt = (int)min(n_s - I * DS_T, (int64_t)DS_T);
            }
#pragma unroll
            for (int h = 0; h < H; ++h) {
                const float4 x0 = ds_load<MODE>(a, o, n_s, I * DS_T + WT * wib + 64 * h + lane);
                const float4 x1 = ds_load<MODE>(a, o, n_s, I * DS_T + WT * wib + 64 * h + 32 + lane);
                TX[h] = pack2(x0.x, x1.x);
                TY[h] = pack2(x0.y, x1.y);
                TZ[h] = pack2(x0.z, x1.z);
                TM[h] = pack2(x0.w, x1.w);
                NX[h] = NY[h] = NZ[h] = NW[h] = 0ull;
            }
            for (int t = tid; t < SPAN; t += WARPS * 32) {
                const int tt = sl * SPAN + t;
                sxm[tt] = ds_load<MODE>(a, o, n_s, J * DS_T + tt);
                sacc[tt] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        __syncthreads();
        for (int r = 0; r < G; ++r) {
            const int g = gbase + (((G / WARPS) * wib + r) & (G - 1));
            // Diagonal tile: targets WT w .. WT w + WT - 1 against sources
            // 32 g .. 32 g + 31; no pair has t < s when (WT / 32) w > g.
            // (Taking the unmasked round where every pair of the group has
            // t < s measured 2.5% slower on the 512-system batch.)
            // Warp-uniform branches; every warp still reaches the barrier.
            if (WT * wib < s_ntgt && g < s_gend) {
                if constexpr (MODE == DS_PHI) {
                    if (!diag)
                        ds_round_phi<false, H>(sxm, sacc, g, lane, wib, EPS2, TX, TY, TZ, TM, NX);
                    else if ((WT / 32) * wib <= g)
                        ds_round_phi<true, H>(sxm, sacc, g, lane, wib, EPS2, TX, TY, TZ, TM, NX);
                } else {
                    if (!diag)
                        ds_round<false, H, PHI>(sxm, sacc, g, lane, wib, EPS2, TX, TY, TZ, TM, NX, NY, NZ, NW);
                    else if ((WT / 32) * wib <= g)
                        ds_round<true, H, PHI>(sxm, sacc, g, lane, wib, EPS2, TX, TY, TZ, TM, NX, NY, NZ, NW);
                }
            }
            __syncthreads();
        }
        const int64_t u = s_unit;
        const int64_t lu = BATCH ? s_local : u;
        const int64_t p = lu / Q;
        const int sl = (int)(lu - p * Q);
        const int64_t col = (BATCH ? s_cb : 0) + p;
        for (int t = tid; t < SPAN; t += WARPS * 32) {
            const int tt = sl * SPAN + t;
            a.colpart[col * DS_T + tt] = sacc[tt];
        }
#pragma unroll
        for (int h = 0; h < H; ++h) {
            float x0, x1, y0, y1, z0, z1, w0 = 0.f, w1 = 0.f;
            unpack2(NX[h], x0, x1);
            unpack2(NY[h], y0, y1);
            unpack2(NZ[h], z0, z1);
            if (PHI) unpack2(NW[h], w0, w1);
            float4 *row = a.rowpart + u * DS_T + WT * wib + 64 * h + lane;
            row[0] = make_float4(x0, y0, z0, w0);
            row[32] = make_float4(x1, y1, z1, w1);
        }
    }
}

struct DsFix {
    const float4 *__restrict__ rowpart;
    const float4 *__restrict__ colpart;
    float4 *xm, *vel, *acc;
    float *phi;  // DS_PHI: the potential sums (in the slots' x)
    int64_t n, nt;
    int Q;
    // One system, in bands of tile rows [Ib, Ie) whose pairs start at p0;
    // aux holds the running (sum, compensation) of particles in tiles >= Ie
    // between bands (two float4 per particle).
    int64_t Ib, Ie, p0;
    float4 *aux;
    // Many systems (BATCH): as in DsArgs, plus each system's first fix-up
    // block (blocks of 32 particles never straddle two systems) and the
    // system of every block.
    const int64_t *__restrict__ off;
    const int64_t *__restrict__ ubase;
    const int64_t *__restrict__ cbase;
    const int64_t *__restrict__ fbase;
    const int *__restrict__ fsys;  // system of each fix-up block
    int nsys;
    float G, h, dt;
    int accumulate;
    ExtPot pot;
};

// Particle i (in tile T) has, in a fixed order: the running sum left by
// earlier bands (columns of rows < Ib), its row units (T, J, slice) for
// J = T .. nt-1 when T is in the band, then its column slots (I', T) for the
// band's rows I' <= T.  A particle whose tile is in the band is complete
// (all rows I' <= T are done) and is written out; one past the band keeps
// its running sum in aux.  A single band (Ib = 0, Ie = nt) is the whole
// pass, as is a batch system.  A CTA of DS_FIX_WARPS warps takes 32
// consecutive particles (one tile); warp w adds slots w, w + DS_FIX_WARPS,
// ... (coalesced 512-byte rows), and warp 0 adds the warps' sums in warp
// order.
constexpr int DS_FIX_WARPS = 8;

// PHI: the slots also carry potential sums in .w (force pass with the
// potential); the particle's sum is written to phi (without G) beside its
// acceleration.
template <int MODE, bool KAHAN, bool BATCH, bool PHI>
__global__ void __launch_bounds__(DS_FIX_WARPS * 32) direct_sym_fixup_kernel(DsFix f) {
    __shared__ float4 part[DS_FIX_WARPS][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t o = 0, n_s = f.n, nt = f.nt, li0 = f.Ib * DS_T + (int64_t)blockIdx.x * 32, ub = 0, cb = 0;
    int64_t Ib = f.Ib, Ie = f.Ie, p0 = f.p0;
    if (BATCH) {
        const int sy = __ldg(f.fsys + blockIdx.x);
        o = __ldg(f.off + sy);
        n_s = __ldg(f.off + sy + 1) - o;
        nt = (n_s + DS_T - 1) / DS_T;
        li0 = ((int64_t)blockIdx.x - __ldg(f.fbase + sy)) * 32;
        ub = __ldg(f.ubase + sy);
        cb = __ldg(f.cbase + sy);
        Ib = 0;
        Ie = nt;
        p0 = 0;
    }
    const int64_t li = li0 + lane;
    const int64_t T = li0 / DS_T, r = li - T * DS_T;
    const bool in_band = T < Ie;
    const int64_t R = in_band ? (nt - T) * f.Q : 0;
    const int64_t C = (in_band ? T : Ie - 1) - Ib + 1;
    const int64_t rbase = ub + (sym_base(T, nt) - p0) * f.Q;
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, sw = 0.f, cw = 0.f;
    auto add = [&](float4 v) {
        if (KAHAN) {
            kahan_add(sx, cx, v.x);
            kahan_add(sy, cy, v.y);
            kahan_add(sz, cz, v.z);
            if (PHI) kahan_add(sw, cw, v.w);
        } else {
            sx += v.x; sy += v.y; sz += v.z;
            if (PHI) sw += v.w;
        }
    };
    // Rows of padded particles (li >= n_s) are zero-mass records: reading
    // them stays inside the scratch; their sums are dropped below.
    for (int64_t k = w; k < R; k += DS_FIX_WARPS) add(f.rowpart[(rbase + k) * DS_T + r]);
    for (int64_t k = (R + DS_FIX_WARPS - 1 - w) / DS_FIX_WARPS * DS_FIX_WARPS + w - R; k < C; k += DS_FIX_WARPS) {
        const int64_t I2 = Ib + k;
        add(f.colpart[(cb + sym_base(I2, nt) + (T - I2) - p0) * DS_T + r]);
    }
    part[w][lane] = make_float4(sx - cx, sy - cy, sz - cz, sw - cw);
    __syncthreads();
    if (w != 0 || li >= n_s) return;
    const int64_t i = o + li;
    sx = sy = sz = cx = cy = cz = sw = cw = 0.f;
    if (!BATCH && Ib > 0) {  // the running sum of the earlier bands
        const float4 s0 = f.aux[2 * i], c0 = f.aux[2 * i + 1];
        sx = s0.x; sy = s0.y; sz = s0.z; sw = s0.w;
        cx = c0.x; cy = c0.y; cz = c0.z; cw = c0.w;
    }
#pragma unroll
    for (int q = 0; q < DS_FIX_WARPS; ++q) add(part[q][lane]);
    if (!BATCH && !in_band) {
        f.aux[2 * i] = make_float4(sx, sy, sz, sw);
        f.aux[2 * i + 1] = make_float4(cx, cy, cz, cw);
        return;
    }
    if (PHI) f.phi[i] = sw - cw;
    float4 an = make_float4(f.G * (sx - cx), f.G * (sy - cy), f.G * (sz - cz), 0.f);
    if (MODE == DS_PHI) {
        f.phi[i] = an.x;
        return;
    }
    if (MODE == DS_ACC) {
        if (f.pot.on) {
            const float4 x = f.xm[i];
            ext_acc_add(f.pot, x.x, x.y, x.z, an.x, an.y, an.z);
        }
        if (f.accumulate) {
            float4 v = f.acc[i];
            v.x += an.x; v.y += an.y; v.z += an.z;
            f.acc[i] = v;
        } else {
            f.acc[i] = an;
        }
        return;
    }
    kdk_writeback(f.xm, f.vel, f.acc, i, an, f.h, f.dt);
}

template <int MODE, bool BATCH, int H, bool PHI>
static void launch_force(int Q, unsigned grid, const DsArgs &a, cudaStream_t s) {
    const unsigned b = DsShape<H>::WARPS * 32;
    if (Q == 1) direct_sym_kernel<1, MODE, BATCH, H, PHI><<<grid, b, 0, s>>>(a);
    else if (Q == 2) direct_sym_kernel<2, MODE, BATCH, H, PHI><<<grid, b, 0, s>>>(a);
    else if (Q == 4) direct_sym_kernel<4, MODE, BATCH, H, PHI><<<grid, b, 0, s>>>(a);
    else direct_sym_kernel<8, MODE, BATCH, H, PHI><<<grid, b, 0, s>>>(a);
}

template <int MODE, bool BATCH, bool PHI>
static void launch_mode(int Q, bool kahan, unsigned grid, unsigned fgrid, const DsArgs &a, const DsFix &f,
                        cudaStream_t s) {
    launch_force<MODE, BATCH, DS_H, PHI>(Q, grid, a, s);
    if (kahan) direct_sym_fixup_kernel<MODE, true, BATCH, PHI><<<fgrid, DS_FIX_WARPS * 32, 0, s>>>(f);
    else direct_sym_fixup_kernel<MODE, false, BATCH, PHI><<<fgrid, DS_FIX_WARPS * 32, 0, s>>>(f);
}

// mode: DS_ACC, DS_KDK or (one system) DS_PHI; phi (one system, DS_ACC or
// DS_KDK): the force pass also writes the potential sums.
template <bool BATCH>
static void launch_pass(int mode, bool phi, int Q, bool kahan, unsigned grid, unsigned fgrid, const DsArgs &a,
                        const DsFix &f, cudaStream_t s) {
    if constexpr (!BATCH) {
        if (phi && mode == DS_KDK) return launch_mode<DS_KDK, false, true>(Q, kahan, grid, fgrid, a, f, s);
        if (phi && mode == DS_ACC) return launch_mode<DS_ACC, false, true>(Q, kahan, grid, fgrid, a, f, s);
    }
    if (mode == DS_KDK) launch_mode<DS_KDK, BATCH, false>(Q, kahan, grid, fgrid, a, f, s);
    else if (mode == DS_ACC) launch_mode<DS_ACC, BATCH, false>(Q, kahan, grid, fgrid, a, f, s);
    else if constexpr (!BATCH) launch_mode<DS_PHI, BATCH, false>(Q, kahan, grid, fgrid, a, f, s);
}

SymShape direct_sym_shape(int sms, int64_t pairs) {
    SymShape sh;
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, direct_sym_kernel<1, DS_ACC, false, DS_H, false>,
                                                  DsShape<DS_H>::WARPS * 32, 0);
    sh.slots = (int64_t)sms * std::max(occ, 1);
    sh.Q = direct_sym_slices(pairs, sh.slots, DsShape<DS_H>::QMAX);
    return sh;
}

int direct_sym_slices(int64_t pairs, int64_t slots, int qmax) {
    // Source slices per tile pair: enough units that the last ones are a
    // small share of each CTA's work.
    int Q = 1;
    while (Q < qmax && pairs * Q < 16 * slots) Q *= 2;
    return Q;
}

struct DsPlan {
    int64_t nt, NP, slots, max_pairs, need;  // need: float4s of scratch
    int Q;
    std::vector<int64_t> rows;  // band b covers tile rows [rows[b], rows[b + 1])
};

static DsPlan ds_plan(const gb_direct *h, int64_t n) {
    DsPlan p;
    p.nt = (n + DS_T - 1) / DS_T;
    p.NP = p.nt * (p.nt + 1) / 2;
    const SymShape sh = direct_sym_shape(h->sms, p.NP);
    p.slots = sh.slots;
    p.Q = sh.Q;
    // Tile pairs per band: the handle's slot budget (larger systems run in
    // bands of tile rows, so the scratch stays bounded at any N).
    const int64_t budget = h->sym_band / ((int64_t)sizeof(float4) * DS_T * (p.Q + 1));
    p.max_pairs = sym_bands(p.nt, budget, p.rows);
    // Row slots, column slots, the running sums between bands, the counter.
    const int64_t aux = p.rows.size() > 2 ? 2 * n : 0;
    p.need = p.max_pairs * p.Q * DS_T + p.max_pairs * DS_T + aux + 1;
    return p;
}

int reserve_direct_sym(gb_direct *h, int64_t n) {
    const DsPlan p = ds_plan(h, n);
    if (p.need * (int64_t)sizeof(float4) > SYM_MAX_BYTES) return GB_OK;
    return ensure_sym(h, p.need);
}

int run_direct_sym(gb_direct *h, int mode, const float4 *xm, float4 *vel, float4 *acc, float *phi, int64_t n,
                   float G, float eps2, float dt, int flags, cudaStream_t s, const ExtPot &pot, bool *done) {
    *done = false;
    const DsPlan pl = ds_plan(h, n);
    if (pl.need * (int64_t)sizeof(float4) > SYM_MAX_BYTES) return GB_OK;
    GB_TRY(ensure_sym(h, pl.need));
    DsArgs a{};
    a.xm = xm;
    a.vel = vel;
    a.acc = acc;
    a.rowpart = h->sym;
    a.colpart = h->sym + pl.max_pairs * pl.Q * DS_T;
    a.counter = (unsigned long long *)(h->sym + pl.need - 1);
    a.n = n;
    a.nt = pl.nt;
    a.eps2 = eps2;
    a.h = 0.5f * dt;
    a.dt = dt;
    DsFix f{};
    f.rowpart = a.rowpart;
    f.colpart = a.colpart;
    f.aux = a.colpart + pl.max_pairs * DS_T;
    f.xm = const_cast<float4 *>(xm);
    f.vel = vel;
    f.acc = acc;
    f.n = n;
    f.nt = pl.nt;
    f.Q = pl.Q;
    f.G = G;
    f.h = 0.5f * dt;
    f.dt = dt;
    f.phi = phi;
    f.accumulate = (flags & GB_ACCUMULATE) ? 1 : 0;
    f.pot = pot;
    const bool kahan = !(flags & GB_PLAIN_FP32);
    for (size_t b = 0; b + 1 < pl.rows.size(); ++b) {
        const int64_t Ib = pl.rows[b], Ie = pl.rows[b + 1];
        a.p0 = host_sym_base(Ib, pl.nt);
        a.NU = (host_sym_base(Ie, pl.nt) - a.p0) * pl.Q;
        f.Ib = Ib;
        f.Ie = Ie;
        f.p0 = a.p0;
        GB_CUDA_TRY(cudaMemsetAsync(a.counter, 0, sizeof(unsigned long long), s));
        launch_pass<false>(mode, phi != nullptr && mode != DS_PHI, pl.Q, kahan,
                           (unsigned)std::min(pl.slots, a.NU), (unsigned)((n - Ib * DS_T + 31) / 32), a, f, s);
        GB_CUDA_TRY(cudaGetLastError());
        h->launches += 2;
    }
    *done = true;
    return GB_OK;
}

int run_batch_sym(const SymBatch &b, int mode, const float4 *xm, float4 *vel, float4 *acc, float G, float eps2,
                  float dt, int flags, cudaStream_t s) {
    DsArgs a{};
    a.xm = xm;
    a.vel = vel;
    a.acc = acc;
    a.rowpart = b.scratch;
    a.colpart = b.scratch + b.NU * DS_T;
    a.counter = (unsigned long long *)(b.scratch + (b.NU + b.NPtot) * DS_T);
    a.NU = b.NU;
    a.off = b.off;
    a.ubase = b.ubase;
    a.cbase = b.cbase;
    a.nsys = b.nsys;
    a.eps2 = eps2;
    a.h = 0.5f * dt;
    a.dt = dt;
    DsFix f{};
    f.rowpart = a.rowpart;
    f.colpart = a.colpart;
    f.xm = const_cast<float4 *>(xm);
    f.vel = vel;
    f.acc = acc;
    f.Q = b.Q;
    f.off = b.off;
    f.ubase = b.ubase;
    f.cbase = b.cbase;
    f.fbase = b.fbase;
    f.fsys = b.fsys;
    f.nsys = b.nsys;
    f.G = G;
    f.h = 0.5f * dt;
    f.dt = dt;
    f.accumulate = (flags & GB_ACCUMULATE) ? 1 : 0;
    GB_CUDA_TRY(cudaMemsetAsync(a.counter, 0, sizeof(unsigned long long), s));
    launch_pass<true>(mode, false, b.Q, !(flags & GB_PLAIN_FP32), (unsigned)b.P, (unsigned)b.nfb, a, f, s);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

}  // namespace gb
