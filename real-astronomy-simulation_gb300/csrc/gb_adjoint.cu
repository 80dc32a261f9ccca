// Hand-written adjoint (reverse mode) of the direct-sum KDK leapfrog.
//
// Forward step (core/engine.py:108-116, core/integrators/leapfrog.py:11-22):
//   vh = v + h a,  x' = x + dt vh,  a' = F(x'),  v' = vh + h a'   (h = dt/2)
// with F_j = G sum_i m_i (x_i - x_j) (|x_i - x_j|^2 + eps2)^{-3/2}
// (core/solvers/gravity.py:13-26).  Given the adjoints (lx', lv', la') of
// x', v', a', one backward step returns those of x, v, a and accumulates the
// mass gradient:
//   w   = la' + h lv'                       (adjoint of a')
//   gx  = J_x^T w,  gm = J_m^T w             (VJP of F at x')
//   lxt = lx' + gx
//   lvh = lv' + dt lxt
//   lx = lxt,  lv = lvh,  la = h lvh,  lm += gm
// and the priming evaluation a0 = F(x0) adds J^T la to (lx, lm) at the end.
//
// VJP of the pairwise force, for target j and source i, d = x_j - x_i,
// r2 = |d|^2 + eps2, s = r2^{-3/2}, t = r2^{-5/2}:
//   gx_j = G sum_i (s I - 3 t d d^T)(m_j w_i - m_i w_j)
//   gm_j = G sum_i s d.w_i
// With u = m_j w_i - m_i w_j the self pair contributes exactly zero.  The
// kernel uses the stream-K layout of the force kernel (equal unit runs per
// CTA, partials merged in CTA order by the fix-up, which also applies the
// elementwise part of the backward step).
#include <algorithm>

#include "gb_direct_core.cuh"

namespace gb {

struct VjpArgs {
    const float4 *__restrict__ xm;  // positions and masses at which F was evaluated
    const float4 *__restrict__ lv;  // adjoint of v' (ignored when prime)
    const float4 *__restrict__ la;  // adjoint of a'
    float4 *__restrict__ part;
    int64_t n, num_ju, U, P;
    int smax;
    float eps2, h;
    int prime;
};

__device__ __forceinline__ float4 load_w(const VjpArgs &a, int64_t i) {
    if (i >= a.n) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 la = __ldg(a.la + i);
    if (a.prime) return la;
    const float4 lv = __ldg(a.lv + i);
    return make_float4(__fmaf_rn(a.h, lv.x, la.x), __fmaf_rn(a.h, lv.y, la.y), __fmaf_rn(a.h, lv.z, la.z), 0.f);
}

__device__ __forceinline__ float4 load_x(const VjpArgs &a, int64_t i) {
    return i < a.n ? __ldg(a.xm + i) : make_float4(0.f, 0.f, 0.f, 0.f);
}

template <int K, int WARPS>
__global__ void __launch_bounds__(WARPS * 32, K == 2 ? 1024 / (WARPS * 32) : 1)
adjoint_vjp_kernel(VjpArgs a) {
    constexpr int TILE = 32 * K;
    constexpr int ST = WARPS * TILE;
    constexpr int JU = WARPS * 32;
    __shared__ float4 sx[JU], sw[JU];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t c = blockIdx.x;
    const int64_t u_begin = unit_begin(a.U, a.P, c), u_end = unit_begin(a.U, a.P, c + 1);
    if (u_begin >= u_end) return;
    const int64_t st0 = u_begin / a.num_ju;
    int64_t u = u_begin;
    while (u < u_end) {
        const int64_t st = u / a.num_ju;
        const int64_t run_end = min(u_end, (st + 1) * a.num_ju);
        const int64_t tbase = st * ST + wib * TILE + lane;
        float X[K], Y[K], Z[K], M[K], WX[K], WY[K], WZ[K];
        float SX[K], SY[K], SZ[K], SG[K];
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const float4 x = load_x(a, tbase + q * 32), w = load_w(a, tbase + q * 32);
            X[q] = x.x; Y[q] = x.y; Z[q] = x.z; M[q] = x.w;
            WX[q] = w.x; WY[q] = w.y; WZ[q] = w.z;
            SX[q] = SY[q] = SZ[q] = SG[q] = 0.f;
        }
        for (; u < run_end; ++u) {
            const int64_t j = (u - st * a.num_ju) * JU + threadIdx.x;
            const float4 xj = load_x(a, j), wj = load_w(a, j);
            __syncthreads();
            sx[threadIdx.x] = xj;
            sw[threadIdx.x] = wj;
            __syncthreads();
            float PX[K], PY[K], PZ[K], PG[K];
#pragma unroll
            for (int q = 0; q < K; ++q) PX[q] = PY[q] = PZ[q] = PG[q] = 0.f;
#pragma unroll 2
            for (int jj = 0; jj < JU; ++jj) {
                const float4 xs = sx[jj], ws = sw[jj];
#pragma unroll
                for (int q = 0; q < K; ++q) {
                    const float dx = X[q] - xs.x, dy = Y[q] - xs.y, dz = Z[q] - xs.z;
                    const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, a.eps2)));
                    const float inv = rsqrt_approx(r2);
                    const float inv2 = inv * inv;
                    const float s = inv * inv2;
                    const float t3 = s * (3.f * inv2);
                    const float ux = __fmaf_rn(-xs.w, WX[q], M[q] * ws.x);
                    const float uy = __fmaf_rn(-xs.w, WY[q], M[q] * ws.y);
                    const float uz = __fmaf_rn(-xs.w, WZ[q], M[q] * ws.z);
                    const float du = __fmaf_rn(dz, uz, __fmaf_rn(dy, uy, dx * ux));
                    const float cf = t3 * du;
                    PX[q] = __fmaf_rn(-cf, dx, __fmaf_rn(s, ux, PX[q]));
                    PY[q] = __fmaf_rn(-cf, dy, __fmaf_rn(s, uy, PY[q]));
                    PZ[q] = __fmaf_rn(-cf, dz, __fmaf_rn(s, uz, PZ[q]));
                    const float dw = __fmaf_rn(dz, ws.z, __fmaf_rn(dy, ws.y, dx * ws.x));
                    PG[q] = __fmaf_rn(s, dw, PG[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < K; ++q) {
                SX[q] += PX[q]; SY[q] += PY[q]; SZ[q] += PZ[q]; SG[q] += PG[q];
            }
        }
        const int64_t slot = (c * a.smax + (st - st0)) * ST + wib * TILE + lane;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const int64_t sq = slot + q * 32;
            a.part[2 * sq] = make_float4(SX[q], SY[q], SZ[q], SG[q]);  // (the lo half is unused)
        }
    }
}

struct VjpFix {
    const float4 *__restrict__ part;
    float4 *lx, *lv, *la;
    float *lm;
    int64_t n, num_ju, U, P, st_size;
    int smax;
    float G, h, dt;
    int prime;
};

__global__ void adjoint_fixup_kernel(VjpFix f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const int64_t st = i / f.st_size, off = i - st * f.st_size;
    const int64_t c_lo = unit_owner(f.U, f.P, st * f.num_ju);
    const int64_t c_hi = unit_owner(f.U, f.P, (st + 1) * f.num_ju - 1);
    float gx = 0.f, gy = 0.f, gz = 0.f, gm = 0.f;
    for (int64_t c = c_lo; c <= c_hi; ++c) {
        const int64_t st0c = unit_begin(f.U, f.P, c) / f.num_ju;
        const float4 p = f.part[2 * ((c * f.smax + (st - st0c)) * f.st_size + off)];
        gx += p.x; gy += p.y; gz += p.z; gm += p.w;
    }
    gx *= f.G; gy *= f.G; gz *= f.G; gm *= f.G;
    f.lm[i] += gm;
    const float4 lx = f.lx[i];
    const float tx = lx.x + gx, ty = lx.y + gy, tz = lx.z + gz;
    if (f.prime) {
        f.lx[i] = make_float4(tx, ty, tz, 0.f);
        return;
    }
    const float4 lv = f.lv[i];
    const float hx = __fmaf_rn(f.dt, tx, lv.x), hy = __fmaf_rn(f.dt, ty, lv.y), hz = __fmaf_rn(f.dt, tz, lv.z);
    f.lx[i] = make_float4(tx, ty, tz, 0.f);
    f.lv[i] = make_float4(hx, hy, hz, 0.f);
    f.la[i] = make_float4(f.h * hx, f.h * hy, f.h * hz, 0.f);
}

constexpr int VJP_K = 2;
constexpr int VJP_WARPS = 8;

// --------------------------------------------------- symmetric evaluation
// Every unordered pair {i, j} once (Newton's third law).  With d = x_j - x_i
// and P = K(d) (m_j w_i - m_i w_j) (K = s I - 3 t d d^T, symmetric in i, j):
//   gx_j += P,  gx_i -= P,  gm_j += s d.w_i,  gm_i -= s d.w_j.
// Tiles of ST_T = 256 particles; unordered tile pairs (I <= J) are numbered
// row-major and split into equal runs over a persistent grid.  A CTA (4 warps,
// 2 targets per lane) keeps tile I's sums in registers along its row; tile J
// sits in shared memory with per-source accumulators.  In round r warp w
// works on source group g = (2w + r) mod 8 and at step k lane l on source
// 32g + (l + k) mod 32: no two lanes touch one accumulator at once, so there
// are no atomics.  Row sums go to slot (I + CTA) and each tile pair's source
// sums to slot (pair); the fix-up merges them in a fixed order.
constexpr int SYM_T = 256;
constexpr int SYM_WARPS = 4;


struct SymArgs {
    const float4 *__restrict__ xm;
    const float4 *__restrict__ lv;
    const float4 *__restrict__ la;
    float4 *__restrict__ rowpart;  // (nt + P) x SYM_T
    float4 *__restrict__ colpart;  // NP x SYM_T
    int64_t n, nt, NP, P;
    float eps2, h;
    int prime;
};

__device__ __forceinline__ float4 sym_w(const SymArgs &a, int64_t i) {
    if (i >= a.n) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 la = __ldg(a.la + i);
    if (a.prime) return la;
    const float4 lv = __ldg(a.lv + i);
    return make_float4(__fmaf_rn(a.h, lv.x, la.x), __fmaf_rn(a.h, lv.y, la.y), __fmaf_rn(a.h, lv.z, la.z), 0.f);
}

__global__ void __launch_bounds__(SYM_WARPS * 32) adjoint_vjp_sym_kernel(SymArgs a) {
    __shared__ float4 sxm[SYM_T], sw[SYM_T], sacc[SYM_T];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, tid = threadIdx.x;
    const int64_t c = blockIdx.x;
    const int64_t p0 = a.NP * c / a.P, p1 = a.NP * (c + 1) / a.P;
    if (p0 >= p1) return;
    int64_t p = p0;
    int64_t I = sym_row(p, a.nt);
    int64_t rbase = sym_base(I, a.nt);
    float X[2], Y[2], Z[2], M[2], WX[2], WY[2], WZ[2], AX[2], AY[2], AZ[2], AG[2];
    auto load_row = [&]() {
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int64_t i = I * SYM_T + 64 * wib + 32 * q + lane;
            const float4 x = i < a.n ? __ldg(a.xm + i) : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 w = sym_w(a, i);
            X[q] = x.x; Y[q] = x.y; Z[q] = x.z; M[q] = x.w;
            WX[q] = w.x; WY[q] = w.y; WZ[q] = w.z;
            AX[q] = AY[q] = AZ[q] = AG[q] = 0.f;
        }
    };
    load_row();
    while (p < p1) {
        const int64_t J = I + (p - rbase);
        const bool diag = J == I;
        // Stage tile J.
        __syncthreads();
        for (int t = tid; t < SYM_T; t += SYM_WARPS * 32) {
            const int64_t j = J * SYM_T + t;
            sxm[t] = j < a.n ? __ldg(a.xm + j) : make_float4(0.f, 0.f, 0.f, 0.f);
            sw[t] = sym_w(a, j);
            sacc[t] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        __syncthreads();
        if (!diag) {
            // Off-diagonal tile pair: every (target, source) pair, no masks.
            for (int r = 0; r < 8; ++r) {
                const int g = (2 * wib + r) & 7;
                const float4 *bx = sxm + g * 32, *bw = sw + g * 32;
                float4 *bacc = sacc + g * 32;
#pragma unroll 4
                for (int k = 0; k < 32; ++k) {
                    const int jj = (lane + k) & 31;
                    const float4 xs = bx[jj], ws = bw[jj];
                    float px = 0.f, py = 0.f, pz = 0.f, pg = 0.f;
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const float dx = xs.x - X[q], dy = xs.y - Y[q], dz = xs.z - Z[q];
                        const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, a.eps2)));
                        const float inv = rsqrt_approx(r2);
                        const float inv2 = inv * inv;
                        const float sv = inv * inv2;
                        // P = sv (u - 3 inv2 (d.u) d), applied with opposite
                        // signs to both sides without forming P.
                        const float ux = __fmaf_rn(-M[q], ws.x, xs.w * WX[q]);
                        const float uy = __fmaf_rn(-M[q], ws.y, xs.w * WY[q]);
                        const float uz = __fmaf_rn(-M[q], ws.z, xs.w * WZ[q]);
                        const float du = __fmaf_rn(dz, uz, __fmaf_rn(dy, uy, dx * ux));
                        const float e = (3.f * inv2) * du;
                        const float vx = __fmaf_rn(-e, dx, ux), vy = __fmaf_rn(-e, dy, uy), vz = __fmaf_rn(-e, dz, uz);
                        const float dwi = __fmaf_rn(dz, WZ[q], __fmaf_rn(dy, WY[q], dx * WX[q]));
                        const float dwj = __fmaf_rn(dz, ws.z, __fmaf_rn(dy, ws.y, dx * ws.x));
                        AX[q] = __fmaf_rn(-sv, vx, AX[q]);
                        AY[q] = __fmaf_rn(-sv, vy, AY[q]);
                        AZ[q] = __fmaf_rn(-sv, vz, AZ[q]);
                        AG[q] = __fmaf_rn(-sv, dwj, AG[q]);
                        px = __fmaf_rn(sv, vx, px);
                        py = __fmaf_rn(sv, vy, py);
                        pz = __fmaf_rn(sv, vz, pz);
                        pg = __fmaf_rn(sv, dwi, pg);
                    }
                    float4 acc = bacc[jj];
                    acc.x += px; acc.y += py; acc.z += pz; acc.w += pg;
                    bacc[jj] = acc;
                    __syncwarp();
                }
                __syncthreads();
            }
        } else {
            for (int r = 0; r < 8; ++r) {
                const int g = (2 * wib + r) & 7;
                // Diagonal tile: slot group ga meets group g fully if ga < g, half
                // the in-group pairs if ga == g, and not at all if ga > g.
                int act[2];
    #pragma unroll
                for (int q = 0; q < 2; ++q) {
                    const int ga = 2 * wib + q;
                    act[q] = !diag ? 2 : (ga < g ? 2 : (ga == g ? 1 : 0));
                }
                // Warp-uniform skip; every warp still reaches the barrier below.
                const int nsteps = (act[0] == 0 && act[1] == 0) ? 0 : 32;
    #pragma unroll 2
                for (int k = 0; k < nsteps; ++k) {
                    const int jj = g * 32 + ((lane + k) & 31);
                    const float4 xs = sxm[jj], ws = sw[jj];
                    const bool half_on = (k >= 1 && k < 16) || (k == 16 && lane < 16);
                    float px = 0.f, py = 0.f, pz = 0.f, pg = 0.f;
    #pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const bool on = act[q] == 2 || (act[q] == 1 && half_on);
                        const float dx = xs.x - X[q], dy = xs.y - Y[q], dz = xs.z - Z[q];
                        const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, a.eps2)));
                        const float inv = rsqrt_approx(r2);
                        const float inv2 = inv * inv;
                        const float sv = on ? inv * inv2 : 0.f;
                        const float ux = __fmaf_rn(-M[q], ws.x, xs.w * WX[q]);
                        const float uy = __fmaf_rn(-M[q], ws.y, xs.w * WY[q]);
                        const float uz = __fmaf_rn(-M[q], ws.z, xs.w * WZ[q]);
                        const float du = __fmaf_rn(dz, uz, __fmaf_rn(dy, uy, dx * ux));
                        const float e = (3.f * inv2) * du;
                        const float vx = __fmaf_rn(-e, dx, ux), vy = __fmaf_rn(-e, dy, uy), vz = __fmaf_rn(-e, dz, uz);
                        const float dwi = __fmaf_rn(dz, WZ[q], __fmaf_rn(dy, WY[q], dx * WX[q]));
                        const float dwj = __fmaf_rn(dz, ws.z, __fmaf_rn(dy, ws.y, dx * ws.x));
                        AX[q] = __fmaf_rn(-sv, vx, AX[q]);
                        AY[q] = __fmaf_rn(-sv, vy, AY[q]);
                        AZ[q] = __fmaf_rn(-sv, vz, AZ[q]);
                        AG[q] = __fmaf_rn(-sv, dwj, AG[q]);
                        px = __fmaf_rn(sv, vx, px);
                        py = __fmaf_rn(sv, vy, py);
                        pz = __fmaf_rn(sv, vz, pz);
                        pg = __fmaf_rn(sv, dwi, pg);
                    }
                    float4 acc = sacc[jj];
                    acc.x += px; acc.y += py; acc.z += pz; acc.w += pg;
                    sacc[jj] = acc;
                    __syncwarp();
                }
                __syncthreads();
            }
        }
        // Source-side sums of this tile pair.
        for (int t = tid; t < SYM_T; t += SYM_WARPS * 32) a.colpart[p * SYM_T + t] = sacc[t];
        ++p;
        if (p == p1 || p == rbase + (a.nt - I)) {  // row (or run) ends: flush tile I's sums
#pragma unroll
            for (int q = 0; q < 2; ++q)
                a.rowpart[(I + c) * SYM_T + 64 * wib + 32 * q + lane] = make_float4(AX[q], AY[q], AZ[q], AG[q]);
            if (p < p1) {
                ++I;
                rbase = sym_base(I, a.nt);
                load_row();
            }
        }
    }
}

// ------------------------------------- symmetric evaluation, packed pairs
// The pair algebra of adjoint_vjp_sym_kernel in .f32x2 arithmetic, where one
// instruction serves two (target, source) pairs.  Tiles of SYM2_T = 512
// particles; 4 warps, 4 targets per lane held as two packed pairs (targets
// q = 0, 1 and q = 2, 3; lane l of warp w owns targets 128 w + 32 q + l).
// A unit is one unordered tile pair (I <= J) and one of Q source slices of
// tile J (512 / Q sources, G = 16 / Q groups of 32).  CTAs take units from
// an atomic counter, so CTAs that the schedulers favour take more units and
// all of them stay resident until the work runs out; each unit writes its
// own row slot (tile I's sums over the slice) and its slice of the pair's
// column slot, and the fix-up adds the slots in a fixed order, so results
// do not depend on which CTA did which unit.  In round r warp w takes group
// g = (G/4 w + r) mod G of the slice (distinct across the warps of a round)
// and at step k lane l source 32 g + (l + k) mod 32, so no two lanes update
// one source accumulator at once.  Target sums N = sum sv v (and sum sv
// d.w_source) stay in registers and are written negated.  On the diagonal
// tile a pair (t, s) counts when t < s; the self pair is exactly zero.
constexpr int SYM2_T = 512;
constexpr int SYM2_WARPS = 4;

struct Sym2Args {
    const float4 *__restrict__ xm;
    const float4 *__restrict__ lv;
    const float4 *__restrict__ la;
    float4 *__restrict__ rowpart;  // NU x SYM2_T (one row slot per unit)
    float4 *__restrict__ colpart;  // band pairs x SYM2_T
    unsigned long long *counter;   // zero at launch
    int64_t n, nt, NU, p0;         // units of the band, its first tile pair
    float eps2, h;
    int prime;
};

__device__ __forceinline__ float4 sym2_w(const Sym2Args &a, int64_t i) {
    if (i >= a.n) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 la = __ldg(a.la + i);
    if (a.prime) return la;
    const float4 lv = __ldg(a.lv + i);
    return make_float4(__fmaf_rn(a.h, lv.x, la.x), __fmaf_rn(a.h, lv.y, la.y), __fmaf_rn(a.h, lv.z, la.z), 0.f);
}

// One round of sym2 pair steps: lane l at step k takes source jj =
// 32 g + (l + k) mod 32 of the staged tile against its 4 targets.  DIAG
// masks the pairs with target index >= source index (diagonal tile).
template <bool DIAG>
__device__ __forceinline__ void sym2_round(const float4 *__restrict__ sxm, const float4 *__restrict__ sw,
                                           float4 *sacc, int g, int lane, int wib, f2 EPS2, f2 NEG3,
                                           const f2 (&TX)[2], const f2 (&TY)[2], const f2 (&TZ)[2],
                                           const f2 (&TNM)[2], const f2 (&TWX)[2], const f2 (&TWY)[2],
                                           const f2 (&TWZ)[2], f2 (&NX)[2], f2 (&NY)[2], f2 (&NZ)[2],
                                           f2 (&NG)[2]) {
    // 3 m_t for the lane's targets: d.u = m_s d.w_t - m_t d.w_s, so
    // -3 d.u = (-3 m_s) d.w_t + (3 m_t) d.w_s from the two dot products.
    const f2 TM3[2] = {mul2(TNM[0], NEG3), mul2(TNM[1], NEG3)};
#pragma unroll 2
    for (int k = 0; k < 32; ++k) {
        const int jj = g * 32 + ((lane + k) & 31);
        const float4 xs = sxm[jj], ws = sw[jj];
        const f2 sx = pack2(xs.x, xs.x), sy = pack2(xs.y, xs.y), sz = pack2(xs.z, xs.z);
        const f2 sm = pack2(xs.w, xs.w);
        const f2 sm3 = mul2(sm, NEG3);
        const f2 swx = pack2(ws.x, ws.x), swy = pack2(ws.y, ws.y), swz = pack2(ws.z, ws.z);
        f2 PX = 0ull, PY = 0ull, PZ = 0ull, PG = 0ull;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const f2 dx = sub2(sx, TX[h]), dy = sub2(sy, TY[h]), dz = sub2(sz, TZ[h]);
            const f2 r2 = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, EPS2)));
            const f2 inv = rsqrt2(r2);
            const f2 inv2 = mul2(inv, inv);
            f2 sv = mul2(inv, inv2);
            if (DIAG) {
                // Target index 128 w + 64 h + 32 e + lane < source index jj.
                float s0, s1;
                unpack2(sv, s0, s1);
                const int t0 = 128 * wib + 64 * h + lane;
                s0 = t0 < jj ? s0 : 0.f;
                s1 = t0 + 32 < jj ? s1 : 0.f;
                sv = pack2(s0, s1);
            }
            // u = m_s w_t - m_t w_s; v = u - 3 inv2 (d.u) d.
            const f2 ux = fma2(TNM[h], swx, mul2(sm, TWX[h]));
            const f2 uy = fma2(TNM[h], swy, mul2(sm, TWY[h]));
            const f2 uz = fma2(TNM[h], swz, mul2(sm, TWZ[h]));
            const f2 dwt = fma2(dz, TWZ[h], fma2(dy, TWY[h], mul2(dx, TWX[h])));
            const f2 dws = fma2(dz, swz, fma2(dy, swy, mul2(dx, swx)));
            const f2 ne = mul2(inv2, fma2(sm3, dwt, mul2(TM3[h], dws)));  // -3 inv2 d.u
            const f2 vx = fma2(ne, dx, ux), vy = fma2(ne, dy, uy), vz = fma2(ne, dz, uz);
            NX[h] = fma2(sv, vx, NX[h]);
            NY[h] = fma2(sv, vy, NY[h]);
            NZ[h] = fma2(sv, vz, NZ[h]);
            NG[h] = fma2(sv, dws, NG[h]);
            PX = fma2(sv, vx, PX);
            PY = fma2(sv, vy, PY);
            PZ = fma2(sv, vz, PZ);
            PG = fma2(sv, dwt, PG);
        }
        float4 acc = sacc[jj];
        float lo, hi;
        unpack2(PX, lo, hi);
        acc.x += lo + hi;
        unpack2(PY, lo, hi);
        acc.y += lo + hi;
        unpack2(PZ, lo, hi);
        acc.z += lo + hi;
        unpack2(PG, lo, hi);
        acc.w += lo + hi;
        sacc[jj] = acc;
        __syncwarp();
    }
}

template <int Q>
__global__ void __launch_bounds__(SYM2_WARPS * 32, 4) adjoint_vjp_sym2_kernel(Sym2Args a) {
    constexpr int G = 16 / Q, SPAN = G * 32;
    __shared__ float4 sxm[SYM2_T], sw[SYM2_T], sacc[SYM2_T];
    __shared__ long long s_unit;
    __shared__ int s_gend, s_ntgt;  // source groups and targets of the unit that hold particles
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, tid = threadIdx.x;
    const int64_t NU = a.NU;
    const f2 EPS2 = pack2(a.eps2, a.eps2), NEG3 = pack2(-3.f, -3.f);
    for (;;) {
        __syncthreads();  // the previous unit is done with s_unit and shared memory
        if (tid == 0) s_unit = (long long)atomicAdd(a.counter, 1ull);
        __syncthreads();
        f2 TX[2], TY[2], TZ[2], TNM[2], TWX[2], TWY[2], TWZ[2], NX[2], NY[2], NZ[2], NG[2];
        bool diag;
        int gbase;
        {
        // Unit bookkeeping is re-read from shared memory after the pair
        // loop, so none of it stays in registers across the loop.
        const int64_t u = s_unit;
        if (u >= NU) break;
        const int64_t p = u / Q;
        const int sl = (int)(u - p * Q);
        const int64_t pg = a.p0 + p;  // pair index in the triangle
        const int64_t I = sym_row(pg, a.nt);
        const int64_t J = I + (pg - sym_base(I, a.nt));
        diag = J == I;
        gbase = sl * G;
        // Padding of the last tile (zero mass and zero w) adds exact zeros:
        // its source groups and all-padding target warps are skipped.
        if (tid == 0) {
            s_gend = (int)((min(a.n - J * SYM2_T, (int64_t)SYM2_T) + 31) / 32);
            s_ntgt = (int)min(a.n - I * SYM2_T, (int64_t)SYM2_T);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float4 x[2], w[2];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int64_t i = I * SYM2_T + 128 * wib + 32 * (2 * h + e) + lane;
                x[e] = i < a.n ? __ldg(a.xm + i) : make_float4(0.f, 0.f, 0.f, 0.f);
                w[e] = sym2_w(a, i);
            }
            TX[h] = pack2(x[0].x, x[1].x);
            TY[h] = pack2(x[0].y, x[1].y);
            TZ[h] = pack2(x[0].z, x[1].z);
            TNM[h] = pack2(-x[0].w, -x[1].w);
            TWX[h] = pack2(w[0].x, w[1].x);
            TWY[h] = pack2(w[0].y, w[1].y);
            TWZ[h] = pack2(w[0].z, w[1].z);
            NX[h] = NY[h] = NZ[h] = NG[h] = 0ull;
        }
        // Stage the slice's sources (tile-local indices sl*SPAN .. +SPAN-1).
        for (int t = tid; t < SPAN; t += SYM2_WARPS * 32) {
            const int tt = sl * SPAN + t;
            const int64_t j = J * SYM2_T + tt;
            sxm[tt] = j < a.n ? __ldg(a.xm + j) : make_float4(0.f, 0.f, 0.f, 0.f);
            sw[tt] = sym2_w(a, j);
            sacc[tt] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        }
        __syncthreads();
        for (int r = 0; r < G; ++r) {
            const int g = gbase + (((G / 4) * wib + r) & (G - 1));
            // Diagonal tile: targets 128 w .. 128 w + 127 against sources
            // 32 g .. 32 g + 31; no pair has t < s when 4 w > g.
            // Warp-uniform branches; every warp still reaches the barrier.
            if (128 * wib < s_ntgt && g < s_gend) {
                if (!diag)
                    sym2_round<false>(sxm, sw, sacc, g, lane, wib, EPS2, NEG3, TX, TY, TZ, TNM, TWX, TWY, TWZ, NX,
                                      NY, NZ, NG);
                else if (4 * wib <= g)
                    sym2_round<true>(sxm, sw, sacc, g, lane, wib, EPS2, NEG3, TX, TY, TZ, TNM, TWX, TWY, TWZ, NX,
                                     NY, NZ, NG);
            }
            __syncthreads();
        }
        const int64_t u = s_unit;
        const int64_t p = u / Q;
        const int sl = (int)(u - p * Q);
        for (int t = tid; t < SPAN; t += SYM2_WARPS * 32) {
            const int tt = sl * SPAN + t;
            a.colpart[p * SYM2_T + tt] = sacc[tt];
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            float x0, x1, y0, y1, z0, z1, g0, g1;
            unpack2(NX[h], x0, x1);
            unpack2(NY[h], y0, y1);
            unpack2(NZ[h], z0, z1);
            unpack2(NG[h], g0, g1);
            float4 *row = a.rowpart + u * SYM2_T + 128 * wib + 64 * h + lane;
            row[0] = make_float4(-x0, -y0, -z0, -g0);
            row[32] = make_float4(-x1, -y1, -z1, -g1);
        }
    }
}

struct Sym2Fix {
    const float4 *__restrict__ rowpart;
    const float4 *__restrict__ colpart;
    float4 *lx, *lv, *la;
    float *lm;
    float4 *aux;  // running sums of particles past the band (one float4 each)
    int64_t n, nt, Ib, Ie, p0;
    int Q;
    float G, h, dt;
    int prime;
};

// Particle i (in tile T, at or after the band's first row Ib) adds, in a
// fixed order: the running sum left by earlier bands, its row units
// (T, J, slice) for J = T .. nt-1 when T is in the band, then its column
// slots (I', T) for the band's rows I' <= T.  A particle of the band is
// complete and gets the elementwise part of the backward step; one past the
// band keeps its running sum in aux.  Later bands never read a finished
// tile, so its adjoint state may change.  One band (Ib = 0, Ie = nt) is the
// whole pass.
__global__ void adjoint_sym2_fixup_kernel(Sym2Fix f) {
    const int64_t i = f.Ib * SYM2_T + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const int64_t T = i / SYM2_T, r = i - T * SYM2_T;
    const bool in_band = T < f.Ie;
    float gx = 0.f, gy = 0.f, gz = 0.f, gm = 0.f;
    if (f.Ib > 0) {
        const float4 v = f.aux[i];
        gx = v.x; gy = v.y; gz = v.z; gm = v.w;
    }
    if (in_band) {
        const int64_t u0 = (sym_base(T, f.nt) - f.p0) * f.Q, u1 = u0 + (f.nt - T) * f.Q;
        for (int64_t u = u0; u < u1; ++u) {
            const float4 v = f.rowpart[u * SYM2_T + r];
            gx += v.x; gy += v.y; gz += v.z; gm += v.w;
        }
    }
    const int64_t last = in_band ? T : f.Ie - 1;
    for (int64_t I2 = f.Ib; I2 <= last; ++I2) {
        const float4 v = f.colpart[(sym_base(I2, f.nt) + (T - I2) - f.p0) * SYM2_T + r];
        gx += v.x; gy += v.y; gz += v.z; gm += v.w;
    }
    if (!in_band) {
        f.aux[i] = make_float4(gx, gy, gz, gm);
        return;
    }
    gx *= f.G; gy *= f.G; gz *= f.G; gm *= f.G;
    f.lm[i] += gm;
    const float4 lx = f.lx[i];
    const float tx = lx.x + gx, ty = lx.y + gy, tz = lx.z + gz;
    if (f.prime) {
        f.lx[i] = make_float4(tx, ty, tz, 0.f);
        return;
    }
    const float4 lv = f.lv[i];
    const float hx = __fmaf_rn(f.dt, tx, lv.x), hy = __fmaf_rn(f.dt, ty, lv.y), hz = __fmaf_rn(f.dt, tz, lv.z);
    f.lx[i] = make_float4(tx, ty, tz, 0.f);
    f.lv[i] = make_float4(hx, hy, hz, 0.f);
    f.la[i] = make_float4(f.h * hx, f.h * hy, f.h * hz, 0.f);
}

struct SymFix {
    const float4 *__restrict__ rowpart;
    const float4 *__restrict__ colpart;
    float4 *lx, *lv, *la;
    float *lm;
    int64_t n, nt, NP, P;
    float G, h, dt;
    int prime;
};

__global__ void adjoint_sym_fixup_kernel(SymFix f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const int64_t I = i / SYM_T, r = i - I * SYM_T;
    const int64_t b0 = sym_base(I, f.nt), b1 = b0 + (f.nt - I) - 1;
    const int64_t c_lo = ((b0 + 1) * f.P - 1) / f.NP, c_hi = ((b1 + 1) * f.P - 1) / f.NP;
    float gx = 0.f, gy = 0.f, gz = 0.f, gm = 0.f;
    for (int64_t c = c_lo; c <= c_hi; ++c) {
        const float4 v = f.rowpart[(I + c) * SYM_T + r];
        gx += v.x; gy += v.y; gz += v.z; gm += v.w;
    }
    for (int64_t I2 = 0; I2 <= I; ++I2) {
        const float4 v = f.colpart[(sym_base(I2, f.nt) + (I - I2)) * SYM_T + r];
        gx += v.x; gy += v.y; gz += v.z; gm += v.w;
    }
    gx *= f.G; gy *= f.G; gz *= f.G; gm *= f.G;
    f.lm[i] += gm;
    const float4 lx = f.lx[i];
    const float tx = lx.x + gx, ty = lx.y + gy, tz = lx.z + gz;
    if (f.prime) {
        f.lx[i] = make_float4(tx, ty, tz, 0.f);
        return;
    }
    const float4 lv = f.lv[i];
    const float hx = __fmaf_rn(f.dt, tx, lv.x), hy = __fmaf_rn(f.dt, ty, lv.y), hz = __fmaf_rn(f.dt, tz, lv.z);
    f.lx[i] = make_float4(tx, ty, tz, 0.f);
    f.lv[i] = make_float4(hx, hy, hz, 0.f);
    f.la[i] = make_float4(f.h * hx, f.h * hy, f.h * hz, 0.f);
}


// Grows the handle's symmetric scratch to at least need float4 elements.

}  // namespace gb

using namespace gb;

extern "C" int gb_adjoint_step(gb_direct_t *h, const float *xm, float *lx, float *lv, float *la, float *lm,
                               int64_t n, float G, float eps2, float dt, int prime, void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (n < 0 || n > h->n_max) return fail(GB_EINVAL, "n=%lld outside [0, n_max=%lld]", (long long)n,
                                           (long long)h->n_max);
    if (n == 0) return GB_OK;
    const void *ptrs[] = {xm, lx, lv, la};
    const char *names[] = {"xm", "lx", "lv", "la"};
    for (int k = 0; k < 4; ++k) {
        if (!ptrs[k]) return fail(GB_EINVAL, "%s is NULL", names[k]);
        if (!aligned16(ptrs[k])) return fail(GB_EINVAL, "%s is not 16-byte aligned", names[k]);
    }
    if (!lm) return fail(GB_EINVAL, "lm is NULL");
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    cudaStream_t s = (cudaStream_t)stream;
    if (h->adj_variant == 2) {
        const int64_t nt = (n + SYM2_T - 1) / SYM2_T, NP = nt * (nt + 1) / 2;
        int occs = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occs, adjoint_vjp_sym2_kernel<1>, SYM2_WARPS * 32, 0);
        const int64_t slots = (int64_t)h->sms * std::max(occs, 1);
        const int Q = direct_sym_slices(NP, slots, 16 / SYM2_WARPS);
        // Bands of tile rows within the handle's slot budget, as for the
        // symmetric force pass.
        std::vector<int64_t> rows;
        const int64_t max_pairs =
            sym_bands(nt, h->sym_band / ((int64_t)sizeof(float4) * SYM2_T * (Q + 1)), rows);
        const int64_t aux = rows.size() > 2 ? n : 0;
        const int64_t need = max_pairs * Q * SYM2_T + max_pairs * SYM2_T + aux + 1;  // + the unit counter
        if (need * (int64_t)sizeof(float4) <= SYM_MAX_BYTES) {
            GB_TRY(ensure_sym(h, need));
            Sym2Args a;
            a.xm = (const float4 *)xm;
            a.lv = (const float4 *)lv;
            a.la = (const float4 *)la;
            a.rowpart = h->sym;
            a.colpart = h->sym + max_pairs * Q * SYM2_T;
            a.counter = (unsigned long long *)(h->sym + need - 1);
            a.n = n;
            a.nt = nt;
            a.eps2 = eps2;
            a.h = 0.5f * dt;
            a.prime = prime ? 1 : 0;
            Sym2Fix f;
            f.rowpart = a.rowpart;
            f.colpart = a.colpart;
            f.aux = a.colpart + max_pairs * SYM2_T;
            f.lx = (float4 *)lx;
            f.lv = (float4 *)lv;
            f.la = (float4 *)la;
            f.lm = lm;
            f.n = n;
            f.nt = nt;
            f.Q = Q;
            f.G = G;
            f.h = 0.5f * dt;
            f.dt = dt;
            f.prime = a.prime;
            for (size_t b = 0; b + 1 < rows.size(); ++b) {
                a.p0 = host_sym_base(rows[b], nt);
                a.NU = (host_sym_base(rows[b + 1], nt) - a.p0) * Q;
                f.Ib = rows[b];
                f.Ie = rows[b + 1];
                f.p0 = a.p0;
                const unsigned P = (unsigned)std::min(slots, a.NU);
                GB_CUDA_TRY(cudaMemsetAsync(a.counter, 0, sizeof(unsigned long long), s));
                if (Q == 1) adjoint_vjp_sym2_kernel<1><<<P, SYM2_WARPS * 32, 0, s>>>(a);
                else if (Q == 2) adjoint_vjp_sym2_kernel<2><<<P, SYM2_WARPS * 32, 0, s>>>(a);
                else adjoint_vjp_sym2_kernel<4><<<P, SYM2_WARPS * 32, 0, s>>>(a);
                GB_CUDA_TRY(cudaGetLastError());
                adjoint_sym2_fixup_kernel<<<(unsigned)((n - f.Ib * SYM2_T + 255) / 256), 256, 0, s>>>(f);
                GB_CUDA_TRY(cudaGetLastError());
                h->launches += 2;
            }
            return GB_OK;
        }
    }
    if (h->adj_variant == 1) {
        const int64_t nt = (n + SYM_T - 1) / SYM_T, NP = nt * (nt + 1) / 2;
        int occs = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occs, adjoint_vjp_sym_kernel, SYM_WARPS * 32, 0);
        const int64_t P = std::max<int64_t>(1, std::min<int64_t>((int64_t)h->sms * std::max(occs, 1), NP));
        const int64_t need = (nt + P) * SYM_T + NP * SYM_T;
        if (need * (int64_t)sizeof(float4) <= SYM_MAX_BYTES) {
            GB_TRY(ensure_sym(h, need));
            SymArgs a;
            a.xm = (const float4 *)xm;
            a.lv = (const float4 *)lv;
            a.la = (const float4 *)la;
            a.rowpart = h->sym;
            a.colpart = h->sym + (nt + P) * SYM_T;
            a.n = n;
            a.nt = nt;
            a.NP = NP;
            a.P = P;
            a.eps2 = eps2;
            a.h = 0.5f * dt;
            a.prime = prime ? 1 : 0;
            adjoint_vjp_sym_kernel<<<(unsigned)P, SYM_WARPS * 32, 0, s>>>(a);
            GB_CUDA_TRY(cudaGetLastError());
            SymFix f;
            f.rowpart = a.rowpart;
            f.colpart = a.colpart;
            f.lx = (float4 *)lx;
            f.lv = (float4 *)lv;
            f.la = (float4 *)la;
            f.lm = lm;
            f.n = n;
            f.nt = nt;
            f.NP = NP;
            f.P = P;
            f.G = G;
            f.h = 0.5f * dt;
            f.dt = dt;
            f.prime = a.prime;
            adjoint_sym_fixup_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f);
            GB_CUDA_TRY(cudaGetLastError());
            h->launches += 2;
            return GB_OK;
        }
    }
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, adjoint_vjp_kernel<VJP_K, VJP_WARPS>, VJP_WARPS * 32, 0);
    int64_t P = (int64_t)h->sms * std::max(occ, 1);
    DirectPlan pl;
    make_plan(n, VJP_K / 2, VJP_WARPS, P, &pl);
    while (plan_partials(pl) > h->part_cap && P > 1) {  // stay inside the handle's scratch
        P = P / 2;
        make_plan(n, VJP_K / 2, VJP_WARPS, P, &pl);
    }
    if (plan_partials(pl) > h->part_cap) return fail(GB_EINVAL, "adjoint scratch too small for n=%lld", (long long)n);
    VjpArgs a;
    a.xm = (const float4 *)xm;
    a.lv = (const float4 *)lv;
    a.la = (const float4 *)la;
    a.part = h->part;
    a.n = n;
    a.num_ju = pl.num_ju;
    a.U = pl.U;
    a.P = pl.P;
    a.smax = pl.smax;
    a.eps2 = eps2;
    a.h = 0.5f * dt;
    a.prime = prime ? 1 : 0;
    adjoint_vjp_kernel<VJP_K, VJP_WARPS><<<(unsigned)pl.P, VJP_WARPS * 32, 0, s>>>(a);
    GB_CUDA_TRY(cudaGetLastError());
    VjpFix f;
    f.part = h->part;
    f.lx = (float4 *)lx;
    f.lv = (float4 *)lv;
    f.la = (float4 *)la;
    f.lm = lm;
    f.n = n;
    f.num_ju = pl.num_ju;
    f.U = pl.U;
    f.P = pl.P;
    f.st_size = pl.st_size;
    f.smax = pl.smax;
    f.G = G;
    f.h = 0.5f * dt;
    f.dt = dt;
    f.prime = a.prime;
    adjoint_fixup_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f);
    GB_CUDA_TRY(cudaGetLastError());
    h->launches += 2;
    return GB_OK;
}

extern "C" int gb_adjoint_set_variant(gb_direct_t *h, int variant) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (variant < 0 || variant > 2) return fail(GB_EINVAL, "variant must be 0, 1 or 2 (got %d)", variant);
    h->adj_variant = variant;
    return GB_OK;
}
