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

// Symmetric scratch above this size falls back to the per-target kernel.
constexpr int64_t SYM_MAX_BYTES = 3LL << 30;

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
    if (h->adj_variant == 1) {
        const int64_t nt = (n + SYM_T - 1) / SYM_T, NP = nt * (nt + 1) / 2;
        int occs = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occs, adjoint_vjp_sym_kernel, SYM_WARPS * 32, 0);
        const int64_t P = std::max<int64_t>(1, std::min<int64_t>((int64_t)h->sms * std::max(occs, 1), NP));
        const int64_t need = (nt + P) * SYM_T + NP * SYM_T;
        if (need * (int64_t)sizeof(float4) <= SYM_MAX_BYTES) {
            if (need > h->sym_cap) {
                if (h->sym) cudaFree(h->sym);
                h->sym = nullptr;
                h->sym_cap = 0;
                if (cudaMalloc(&h->sym, sizeof(float4) * need) != cudaSuccess)
                    return fail(GB_ENOMEM, "symmetric adjoint scratch (%lld bytes)", (long long)(need * 16));
                h->sym_cap = need;
            }
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

extern "C" int gb_adjoint_set_variant(gb_direct_t *h, int symmetric) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (symmetric != 0 && symmetric != 1) return fail(GB_EINVAL, "symmetric must be 0 or 1");
    h->adj_variant = symmetric;
    return GB_OK;
}
