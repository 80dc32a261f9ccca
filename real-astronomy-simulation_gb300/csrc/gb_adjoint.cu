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
    cudaStream_t s = (cudaStream_t)stream;
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
