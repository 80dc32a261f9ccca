// Direct N^2 self-gravity on the FP32 CUDA cores (sm_103a).
//
// Replaces compute_acc_direct / potential_energy / kinetic_energy
// (core/solvers/gravity.py:13-57) and the KDK kernels
// (core/integrators/leapfrog.py:11-22) of the reference.
//
// Work decomposition ("stream-K"): the (targets x sources) plane is cut into
// units of one target supertile (WARPS*32*K targets, K per lane) by one
// source chunk (WARPS*32 sources).  A persistent grid of P CTAs takes equal
// contiguous runs of units in supertile-major order, so every SM gets the
// same number of interactions at any N.  A CTA stages each source chunk in
// shared memory as duplicated pairs {(x,x),(y,y)},{(z,z),(m,m)} so the inner
// loop runs on packed .f32x2 instructions (two targets per instruction);
// per-unit partial sums are Kahan-added into the running sum.  When a run
// leaves a supertile the CTA writes its compensated partial (hi, lo) to
// scratch; the fix-up kernel merges the partials of every target in a fixed
// CTA order (deterministic for a given grid) and applies the epilogue
// (store / accumulate / closing kick).
//
// KDK fusion: in KDK mode the source loader and the target loader both
// predict x' = x + (v + a dt/2) dt on the fly from the stored state, and the
// fix-up applies v' = v + a dt/2 + a' dt/2, writing x', v', a' in place.
#include <algorithm>
#include <atomic>
#include <cstdio>
#include <mutex>

#include "gb_direct_core.cuh"

namespace gb {

enum DirectMode { MODE_ACC = 0, MODE_KDK = 1, MODE_PHI = 2 };

// Targets are particles t0 .. t0 + nt - 1 (all n in every call but
// gb_direct_acc_range); sources are particles 0 .. n - 1.
struct DirectArgs {
    const float4 *__restrict__ xm;
    const float4 *__restrict__ vel;
    const float4 *__restrict__ acc;
    float4 *__restrict__ part;
    int *st0tab;  // per CTA: its first supertile (read by the fix-up)
    int64_t n, num_ju, U;
    int64_t P;
    int64_t t0, nt;
    int smax;
    float eps2, h, dt;
};


template <int MODE>
__device__ __forceinline__ float4 load_particle(const DirectArgs &a, int64_t i) {
    if (i >= a.n) return make_float4(0.f, 0.f, 0.f, 0.f);
    float4 x = ldg4(a.xm + i);
    if (MODE == MODE_KDK) x = predict_xm(x, ldg4(a.vel + i), ldg4(a.acc + i), a.h, a.dt);
    return x;
}

// Target i of the call's range (zeros past its end).
template <int MODE>
__device__ __forceinline__ float4 load_target(const DirectArgs &a, int64_t i) {
    if (i >= a.nt) return make_float4(0.f, 0.f, 0.f, 0.f);
    return load_particle<MODE>(a, a.t0 + i);
}

// Force kernel for MODE_ACC / MODE_KDK.  NP packed target pairs per lane.
// The inner loop takes two sources per iteration into two accumulator sets
// (independent dependency chains for the scheduler); the Kahan running sums
// stay in registers.  FINE: units of SCALAR_UNIT sources (up to WARPS of
// them staged per shared-memory batch) instead of WARPS * 32, so short CTA
// runs split the work evenly (as in the scalar kernel).
template <int NP, int WARPS, int MODE, bool KAHAN, bool FINE, bool PHI>
__global__ void __launch_bounds__(WARPS * 32, NP == 1 ? 1024 / (WARPS * 32) : 1)
direct_force_kernel(DirectArgs a) {
    constexpr int K = 2 * NP;
    constexpr int TILE = 32 * K;
    constexpr int ST = WARPS * TILE;
    constexpr int JU = WARPS * 32;
    __shared__ ulonglong2 src[2 * JU];  // per source {(x, x), (y, y)}, {(z, z), (m, m)}

    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t c = blockIdx.x;
    const int64_t u_begin = unit_begin(a.U, a.P, c);
    const int64_t u_end = unit_begin(a.U, a.P, c + 1);
    if (u_begin >= u_end) return;  // whole CTA idle (tiny n)
    const int64_t st0 = u_begin / a.num_ju;
    if (threadIdx.x == 0) a.st0tab[c] = (int)st0;
    const f2 E2 = pack2(a.eps2, a.eps2);

    int64_t u = u_begin;
    while (u < u_end) {
        const int64_t st = u / a.num_ju;
        const int64_t run_end = min(u_end, (st + 1) * a.num_ju);
        const int64_t tbase = st * ST + wib * TILE + lane;

        f2 X[NP], Y[NP], Z[NP];
        f2 SX[NP], SY[NP], SZ[NP], CX[NP], CY[NP], CZ[NP], SW[NP], CW[NP];
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            const float4 t0 = load_target<MODE>(a, tbase + (2 * p) * 32);
            const float4 t1 = load_target<MODE>(a, tbase + (2 * p + 1) * 32);
            X[p] = pack2(t0.x, t1.x);
            Y[p] = pack2(t0.y, t1.y);
            Z[p] = pack2(t0.z, t1.z);
            SX[p] = SY[p] = SZ[p] = CX[p] = CY[p] = CZ[p] = SW[p] = CW[p] = 0ull;
        }

        while (u < run_end) {
            const int64_t jc = u - st * a.num_ju;
            int cnt = 1;
            float4 s4;
            if (FINE) {
                // Stage up to WARPS units (SCALAR_UNIT sources each) at once.
                cnt = (int)min((int64_t)WARPS, run_end - u);
                s4 = (int)threadIdx.x < cnt * SCALAR_UNIT ? load_particle<MODE>(a, jc * SCALAR_UNIT + threadIdx.x)
                                                          : make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
                s4 = load_particle<MODE>(a, jc * JU + threadIdx.x);
            }
            __syncthreads();  // previous batch fully consumed
            src[2 * threadIdx.x] = make_ulonglong2(pack2(s4.x, s4.x), pack2(s4.y, s4.y));
            src[2 * threadIdx.x + 1] = make_ulonglong2(pack2(s4.z, s4.z), pack2(s4.w, s4.w));
            __syncthreads();
            u += cnt;
            const int nsrc = FINE ? cnt * SCALAR_UNIT : JU;

            f2 AX[2][NP], AY[2][NP], AZ[2][NP], AW[2][NP];
#pragma unroll
            for (int p = 0; p < NP; ++p)
                AX[0][p] = AY[0][p] = AZ[0][p] = AX[1][p] = AY[1][p] = AZ[1][p] = AW[0][p] = AW[1][p] = 0ull;
#pragma unroll 2
            for (int jj = 0; jj < nsrc; jj += 2) {
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const ulonglong2 A = src[2 * (jj + h)];
                    const ulonglong2 B = src[2 * (jj + h) + 1];
#pragma unroll
                    for (int p = 0; p < NP; ++p) {
                        const f2 dx = sub2(A.x, X[p]);
                        const f2 dy = sub2(A.y, Y[p]);
                        const f2 dz = sub2(B.x, Z[p]);
                        f2 r2 = fma2(dx, dx, E2);
                        r2 = fma2(dy, dy, r2);
                        r2 = fma2(dz, dz, r2);
                        const f2 inv = rsqrt2(r2);
                        const f2 inv2 = mul2(inv, inv);
                        const f2 mi = mul2(B.y, inv);
                        const f2 sc = mul2(mi, inv2);
                        AX[h][p] = fma2(sc, dx, AX[h][p]);
                        AY[h][p] = fma2(sc, dy, AY[h][p]);
                        AZ[h][p] = fma2(sc, dz, AZ[h][p]);
                        if (PHI) AW[h][p] = add2(AW[h][p], mi);
                    }
                }
            }
#pragma unroll
            for (int p = 0; p < NP; ++p) {
                const f2 ax = add2(AX[0][p], AX[1][p]);
                const f2 ay = add2(AY[0][p], AY[1][p]);
                const f2 az = add2(AZ[0][p], AZ[1][p]);
                if (KAHAN) {
                    kahan_add2(SX[p], CX[p], ax);
                    kahan_add2(SY[p], CY[p], ay);
                    kahan_add2(SZ[p], CZ[p], az);
                } else {
                    SX[p] = add2(SX[p], ax);
                    SY[p] = add2(SY[p], ay);
                    SZ[p] = add2(SZ[p], az);
                }
                if (PHI) {
                    const f2 aw = add2(AW[0][p], AW[1][p]);
                    if (KAHAN) kahan_add2(SW[p], CW[p], aw);
                    else SW[p] = add2(SW[p], aw);
                }
            }
        }
        // Flush the compensated partial: estimate = hi + lo with lo = -c.
        const int64_t slot = (c * a.smax + (st - st0)) * ST + wib * TILE + lane;
#pragma unroll
        for (int p = 0; p < NP; ++p) {
            float hx0, hx1, hy0, hy1, hz0, hz1, cx0, cx1, cy0, cy1, cz0, cz1, hw0, hw1, cw0, cw1;
            unpack2(SX[p], hx0, hx1);
            unpack2(SY[p], hy0, hy1);
            unpack2(SZ[p], hz0, hz1);
            unpack2(CX[p], cx0, cx1);
            unpack2(CY[p], cy0, cy1);
            unpack2(CZ[p], cz0, cz1);
            unpack2(SW[p], hw0, hw1);
            unpack2(CW[p], cw0, cw1);
            const int64_t s0 = slot + (2 * p) * 32, s1 = s0 + 32;
            a.part[2 * s0] = make_float4(hx0, hy0, hz0, hw0);
            a.part[2 * s0 + 1] = make_float4(-cx0, -cy0, -cz0, -cw0);
            a.part[2 * s1] = make_float4(hx1, hy1, hz1, hw1);
            a.part[2 * s1 + 1] = make_float4(-cx1, -cy1, -cz1, -cw1);
        }
    }
}

// Scalar variant of the force kernel (same decomposition and Kahan
// scheme): K = 2 * NP targets per lane in plain FP32 registers, one source
// broadcast per shared-memory load.  Selected with gb_direct_set_variant.
// FINE: units of SCALAR_UNIT sources (up to WARPS of them staged per
// shared-memory batch) instead of WARPS * 32, so short CTA runs split the
// work evenly; the host picks it when the coarse split leaves a tail.
template <int NP, int WARPS, int MODE, bool KAHAN, bool FINE, bool PHI>
__global__ void __launch_bounds__(WARPS * 32, NP == 1 ? 1024 / (WARPS * 32) : 1)
direct_force_scalar_kernel(DirectArgs a) {
    constexpr int K = 2 * NP;
    constexpr int TILE = 32 * K;
    constexpr int ST = WARPS * TILE;
    constexpr int JU = WARPS * 32;
    __shared__ float4 src[JU];

    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t c = blockIdx.x;
    const int64_t u_begin = unit_begin(a.U, a.P, c);
    const int64_t u_end = unit_begin(a.U, a.P, c + 1);
    if (u_begin >= u_end) return;
    const int64_t st0 = u_begin / a.num_ju;
    if (threadIdx.x == 0) a.st0tab[c] = (int)st0;

    int64_t u = u_begin;
    while (u < u_end) {
        const int64_t st = u / a.num_ju;
        const int64_t run_end = min(u_end, (st + 1) * a.num_ju);
        const int64_t tbase = st * ST + wib * TILE + lane;
        float X[K], Y[K], Z[K], SX[K], SY[K], SZ[K], CX[K], CY[K], CZ[K], SW[K], CW[K];
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const float4 t = load_target<MODE>(a, tbase + q * 32);
            X[q] = t.x; Y[q] = t.y; Z[q] = t.z;
            SX[q] = SY[q] = SZ[q] = CX[q] = CY[q] = CZ[q] = SW[q] = CW[q] = 0.f;
        }
        while (u < run_end) {
            const int64_t jc = u - st * a.num_ju;
            int cnt = 1;
            float4 s4;
            if (FINE) {
                // Stage up to WARPS units (SCALAR_UNIT sources each) at once.
                cnt = (int)min((int64_t)WARPS, run_end - u);
                s4 = (int)threadIdx.x < cnt * SCALAR_UNIT ? load_particle<MODE>(a, jc * SCALAR_UNIT + threadIdx.x)
                                                          : make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
                s4 = load_particle<MODE>(a, jc * JU + threadIdx.x);
            }
            __syncthreads();
            src[threadIdx.x] = s4;
            __syncthreads();
            u += cnt;
            float AX[K], AY[K], AZ[K], PW[K];
#pragma unroll
            for (int q = 0; q < K; ++q) AX[q] = AY[q] = AZ[q] = PW[q] = 0.f;
            if (FINE) {
                for (int b = 0; b < cnt; ++b)
                    interact_chunk<K, SCALAR_UNIT, PHI>(src + b * SCALAR_UNIT, X, Y, Z, AX, AY, AZ, PW, a.eps2);
            } else {
                interact_chunk<K, JU, PHI>(src, X, Y, Z, AX, AY, AZ, PW, a.eps2);
            }
#pragma unroll
            for (int q = 0; q < K; ++q) {
                if (KAHAN) {
                    kahan_add(SX[q], CX[q], AX[q]);
                    kahan_add(SY[q], CY[q], AY[q]);
                    kahan_add(SZ[q], CZ[q], AZ[q]);
                    if (PHI) kahan_add(SW[q], CW[q], PW[q]);
                } else {
                    SX[q] += AX[q]; SY[q] += AY[q]; SZ[q] += AZ[q];
                    if (PHI) SW[q] += PW[q];
                }
            }
        }
        const int64_t slot = (c * a.smax + (st - st0)) * ST + wib * TILE + lane;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const int64_t sq = slot + q * 32;
            a.part[2 * sq] = make_float4(SX[q], SY[q], SZ[q], SW[q]);
            a.part[2 * sq + 1] = make_float4(-CX[q], -CY[q], -CZ[q], -CW[q]);
        }
    }
}

// Potential kernel: phi_i = sum_{j != i} m_j / sqrt(r^2 + eps2), scalar FP32
// with the same stream-K layout (K = 2 targets per lane, partial in .x).
template <int WARPS, bool KAHAN>
__global__ void __launch_bounds__(WARPS * 32)
direct_phi_kernel(DirectArgs a) {
    constexpr int K = 2;
    constexpr int TILE = 32 * K;
    constexpr int ST = WARPS * TILE;
    constexpr int JU = WARPS * 32;
    __shared__ float4 src[JU];

    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int64_t c = blockIdx.x;
    const int64_t u_begin = unit_begin(a.U, a.P, c);
    const int64_t u_end = unit_begin(a.U, a.P, c + 1);
    if (u_begin >= u_end) return;
    const int64_t st0 = u_begin / a.num_ju;
    if (threadIdx.x == 0) a.st0tab[c] = (int)st0;

    int64_t u = u_begin;
    while (u < u_end) {
        const int64_t st = u / a.num_ju;
        const int64_t run_end = min(u_end, (st + 1) * a.num_ju);
        const int64_t tbase = st * ST + wib * TILE + lane;
        float tx[K], ty[K], tz[K], S[K], C[K];
        int64_t ti[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            ti[k] = tbase + k * 32;
            const float4 t = load_particle<MODE_ACC>(a, ti[k]);
            tx[k] = t.x; ty[k] = t.y; tz[k] = t.z;
            S[k] = C[k] = 0.f;
        }
        for (; u < run_end; ++u) {
            const int64_t ju = u - st * a.num_ju;
            const int64_t j0 = ju * JU;
            const float4 s4 = load_particle<MODE_ACC>(a, j0 + threadIdx.x);
            __syncthreads();
            src[threadIdx.x] = s4;
            __syncthreads();
            float A[K];
#pragma unroll
            for (int k = 0; k < K; ++k) A[k] = 0.f;
#pragma unroll 4
            for (int jj = 0; jj < JU; ++jj) {
                const float4 s = src[jj];
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const float dx = s.x - tx[k], dy = s.y - ty[k], dz = s.z - tz[k];
                    const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, a.eps2)));
                    const float t = s.w * rsqrt_approx(r2);
                    A[k] += (j0 + jj != ti[k]) ? t : 0.f;
                }
            }
#pragma unroll
            for (int k = 0; k < K; ++k) {
                if (KAHAN) kahan_add(S[k], C[k], A[k]);
                else S[k] += A[k];
            }
        }
        const int64_t slot = (c * a.smax + (st - st0)) * ST + wib * TILE + lane;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int64_t s = slot + k * 32;
            a.part[2 * s] = make_float4(S[k], 0.f, 0.f, 0.f);
            a.part[2 * s + 1] = make_float4(-C[k], 0.f, 0.f, 0.f);
        }
    }
}

struct FixArgs {
    const float4 *__restrict__ part;
    const int *__restrict__ st0tab;  // first supertile of each CTA
    float4 *xm;   // KDK: in/out positions
    float4 *vel;  // KDK: in/out velocities
    float4 *acc;  // ACC/KDK: output accelerations (KDK: in = previous)
    float *phi;   // MODE_PHI, or a force pass with the potential: output
    int64_t n;    // targets (the range's nt; outputs acc[i], phi[i], i < n)
    int64_t t0;   // first target's particle index (xm[t0 + i]; 0 but for ranges)
    int64_t num_ju, U, P, st_size;
    int smax;
    float G, h, dt, eps2;
    int accumulate;
    ExtPot pot;  // ACC: analytic potential added to the result (pot.on)
};

// MODE_ACC / MODE_KDK with PHI: the partials also carry the potential sums
// in .w, whose sum less the particle's own term is written to phi.
template <int MODE, bool PHI = false>
__global__ void direct_fixup_kernel(FixArgs f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const int64_t st = i / f.st_size;
    const int64_t off = i - st * f.st_size;
    const int64_t c_lo = unit_owner(f.U, f.P, st * f.num_ju);
    const int64_t c_hi = unit_owner(f.U, f.P, (st + 1) * f.num_ju - 1);
    float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, sw = 0.f, cw = 0.f;
    for (int64_t c = c_lo; c <= c_hi; ++c) {
        const int64_t st0c = __ldg(f.st0tab + c);
        const int64_t slot = (c * f.smax + (st - st0c)) * f.st_size + off;
        const float4 hi = f.part[2 * slot];
        const float4 lo = f.part[2 * slot + 1];
        kahan_add(sx, cx, hi.x);
        kahan_add(sx, cx, lo.x);
        if (MODE != MODE_PHI) {
            kahan_add(sy, cy, hi.y);
            kahan_add(sy, cy, lo.y);
            kahan_add(sz, cz, hi.z);
            kahan_add(sz, cz, lo.z);
        }
        if (PHI) {
            kahan_add(sw, cw, hi.w);
            kahan_add(sw, cw, lo.w);
        }
    }
    const float tx = sx - cx, ty = sy - cy, tz = sz - cz;
    if (MODE == MODE_PHI) {
        f.phi[i] = tx;
        return;
    }
    if (PHI) {
        kahan_add(sw, cw, -self_phi_term(f.xm[f.t0 + i].w, f.eps2));
        f.phi[i] = sw - cw;
    }
    float4 an = make_float4(f.G * tx, f.G * ty, f.G * tz, 0.f);
    if (MODE == MODE_ACC) {
        if (f.pot.on) {
            const float4 x = f.xm[f.t0 + i];
            ext_acc_add(f.pot, x.x, x.y, x.z, an.x, an.y, an.z);
        }
        if (f.accumulate) {
            float4 o = f.acc[i];
            o.x += an.x; o.y += an.y; o.z += an.z;
            f.acc[i] = o;
        } else {
            f.acc[i] = an;
        }
        return;
    }
    // MODE_KDK: closing kick and state write-back (in place).
    const float4 x = f.xm[i], v = f.vel[i], a0 = f.acc[i];
    const float vhx = kick(v.x, a0.x, f.h), vhy = kick(v.y, a0.y, f.h), vhz = kick(v.z, a0.z, f.h);
    f.xm[i] = make_float4(drift(x.x, vhx, f.dt), drift(x.y, vhy, f.dt), drift(x.z, vhz, f.dt), x.w);
    f.vel[i] = make_float4(kick(vhx, an.x, f.h), kick(vhy, an.y, f.h), kick(vhz, an.z, f.h), v.w);
    f.acc[i] = an;
}

// ------------------------------------------------------------- energies
// Per-block FP64 partial sums of KE = 1/2 m v.v and W = m phi, then a single
// block combines them in block order (deterministic).
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// One launch: every block writes its partial, the block that arrives last
// (ticket) adds the partials in block order; it leaves the ticket at zero.
__global__ void energy_kernel(const float4 *__restrict__ xm, const float4 *__restrict__ vel,
                              const float *__restrict__ phi, int64_t n, double2 *part, unsigned *ticket, double G,
                              double *out3) {
    double ke = 0.0, w = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float4 x = xm[i], v = vel[i];
        const double m = x.w;
        const double vv = (double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z;
        ke += 0.5 * m * vv;
        w += m * (double)phi[i];
    }
    __shared__ double sk[32], sw[32];
    __shared__ bool last;
    ke = warp_sum_d(ke);
    w = warp_sum_d(w);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sk[wid] = ke; sw[wid] = w; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        ke = lane < nw ? sk[lane] : 0.0;
        w = lane < nw ? sw[lane] : 0.0;
        ke = warp_sum_d(ke);
        w = warp_sum_d(w);
        if (lane == 0) {
            part[blockIdx.x] = make_double2(ke, w);
            __threadfence();  // the partial is visible before the ticket counts it
            last = atomicAdd(ticket, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (!last || wid != 0) return;
    __threadfence();
    ke = 0.0;
    w = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) {
        const double2 pb = __ldcg(part + b);
        ke += pb.x;
        w += pb.y;
    }
    ke = warp_sum_d(ke);
    w = warp_sum_d(w);
    if (lane == 0) {
        const double pe = -0.5 * G * w;
        out3[0] = ke;
        out3[1] = pe;
        out3[2] = ke + pe;
        *ticket = 0u;
    }
}

int launch_energy(const float4 *xm, const float4 *vel, const float *phi, int64_t n, float G, double2 *epart,
                  int epart_cap, double *out3, cudaStream_t s) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, out3) != cudaSuccess) {
        cudaGetLastError();
        return fail(GB_EINVAL, "out3 is not a valid pointer");
    }
    const bool host = at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeUnregistered;
    double *dst = host ? reinterpret_cast<double *>(epart + epart_cap + 1) : out3;
    unsigned *ticket = reinterpret_cast<unsigned *>(epart + epart_cap);
    const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(epart_cap, (n + 255) / 256));
    energy_kernel<<<nb, 256, 0, s>>>(xm, vel, phi, n, epart, ticket, (double)G, dst);
    GB_CUDA_TRY(cudaGetLastError());
    if (host) {
        GB_CUDA_TRY(cudaMemcpyAsync(out3, dst, 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
        GB_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return GB_OK;
}

// ------------------------------------------------- FP64 sampled oracle
// One CTA per sampled target; threads stride the sources; FP64 arithmetic in
// the order of core/solvers/gravity.py:22-25; fixed-order block reduction.
__global__ void direct_fp64_kernel(const float4 *__restrict__ xm, int64_t n,
                                   const int64_t *__restrict__ targets, double G, double eps2,
                                   double *__restrict__ out) {
    const int64_t i = targets[blockIdx.x];
    const float4 t = xm[i];
    const double px = t.x, py = t.y, pz = t.z;
    double ax = 0.0, ay = 0.0, az = 0.0;
    for (int64_t j = threadIdx.x; j < n; j += blockDim.x) {
        const float4 s = xm[j];
        const double dx = __dsub_rn((double)s.x, px);
        const double dy = __dsub_rn((double)s.y, py);
        const double dz = __dsub_rn((double)s.z, pz);
        const double r2 = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                              __dmul_rn(dz, dz)), eps2);
        const double inv = 1.0 / sqrt(r2);
        const double sc = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(G, (double)s.w), inv), inv), inv);
        ax = __dadd_rn(ax, __dmul_rn(sc, dx));
        ay = __dadd_rn(ay, __dmul_rn(sc, dy));
        az = __dadd_rn(az, __dmul_rn(sc, dz));
    }
    __shared__ double sx[32], sy[32], sz[32];
    ax = warp_sum_d(ax);
    ay = warp_sum_d(ay);
    az = warp_sum_d(az);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sx[wid] = ax; sy[wid] = ay; sz[wid] = az; }
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        ax = lane < nw ? sx[lane] : 0.0;
        ay = lane < nw ? sy[lane] : 0.0;
        az = lane < nw ? sz[lane] : 0.0;
        ax = warp_sum_d(ax);
        ay = warp_sum_d(ay);
        az = warp_sum_d(az);
        if (lane == 0) {
            out[3 * blockIdx.x] = ax;
            out[3 * blockIdx.x + 1] = ay;
            out[3 * blockIdx.x + 2] = az;
        }
    }
}

// ------------------------------------------------------------------ host

template <int NP, int WARPS, int MODE, bool FINE, bool PHI>
static void launch_scalar_m(bool kahan, dim3 grid, const DirectArgs &a, cudaStream_t s) {
    const dim3 block(WARPS * 32);
    if (kahan) direct_force_scalar_kernel<NP, WARPS, MODE, true, FINE, PHI><<<grid, block, 0, s>>>(a);
    else direct_force_scalar_kernel<NP, WARPS, MODE, false, FINE, PHI><<<grid, block, 0, s>>>(a);
}

template <int NP, int WARPS, bool FINE>
static void launch_scalar(int mode, bool kahan, bool phi, dim3 grid, const DirectArgs &a, cudaStream_t s) {
    if (mode == MODE_ACC) {
        if (phi) launch_scalar_m<NP, WARPS, MODE_ACC, FINE, true>(kahan, grid, a, s);
        else launch_scalar_m<NP, WARPS, MODE_ACC, FINE, false>(kahan, grid, a, s);
    } else {
        if (phi) launch_scalar_m<NP, WARPS, MODE_KDK, FINE, true>(kahan, grid, a, s);
        else launch_scalar_m<NP, WARPS, MODE_KDK, FINE, false>(kahan, grid, a, s);
    }
}

template <int NP, int WARPS, int MODE, bool FINE, bool PHI>
static void launch_packed_m(bool kahan, dim3 grid, const DirectArgs &a, cudaStream_t s) {
    const dim3 block(WARPS * 32);
    if (kahan) direct_force_kernel<NP, WARPS, MODE, true, FINE, PHI><<<grid, block, 0, s>>>(a);
    else direct_force_kernel<NP, WARPS, MODE, false, FINE, PHI><<<grid, block, 0, s>>>(a);
}

template <int NP, int WARPS, bool FINE>
static void launch_packed(int mode, bool kahan, bool phi, dim3 grid, const DirectArgs &a, cudaStream_t s) {
    if (mode == MODE_ACC) {
        if (phi) launch_packed_m<NP, WARPS, MODE_ACC, FINE, true>(kahan, grid, a, s);
        else launch_packed_m<NP, WARPS, MODE_ACC, FINE, false>(kahan, grid, a, s);
    } else {
        if (phi) launch_packed_m<NP, WARPS, MODE_KDK, FINE, true>(kahan, grid, a, s);
        else launch_packed_m<NP, WARPS, MODE_KDK, FINE, false>(kahan, grid, a, s);
    }
}

// phi: the pass also sums the potential (PHI kernels).
template <int NP, int WARPS>
static cudaError_t launch_force(int mode, bool kahan, bool phi, const DirectPlan &pl, const DirectArgs &a,
                                cudaStream_t s, int packed, bool fine) {
    const dim3 grid((unsigned)pl.P);
    if (!packed) {
        if (fine) launch_scalar<NP, WARPS, true>(mode, kahan, phi, grid, a, s);
        else launch_scalar<NP, WARPS, false>(mode, kahan, phi, grid, a, s);
        return cudaGetLastError();
    }
    if (fine) launch_packed<NP, WARPS, true>(mode, kahan, phi, grid, a, s);
    else launch_packed<NP, WARPS, false>(mode, kahan, phi, grid, a, s);
    return cudaGetLastError();
}

typedef const void *KernelPtr;

static KernelPtr force_kernel_ptr(int np, int warps, int packed) {
    if (!packed) {
        if (np == 1 && warps == 4) return (KernelPtr)direct_force_scalar_kernel<1, 4, MODE_KDK, true, false, false>;
        if (np == 1 && warps == 8) return (KernelPtr)direct_force_scalar_kernel<1, 8, MODE_KDK, true, false, false>;
        if (np == 2 && warps == 4) return (KernelPtr)direct_force_scalar_kernel<2, 4, MODE_KDK, true, false, false>;
        return (KernelPtr)direct_force_scalar_kernel<2, 8, MODE_KDK, true, false, false>;
    }
    if (np == 1 && warps == 4) return (KernelPtr)direct_force_kernel<1, 4, MODE_KDK, true, false, false>;
    if (np == 1 && warps == 8) return (KernelPtr)direct_force_kernel<1, 8, MODE_KDK, true, false, false>;
    if (np == 2 && warps == 4) return (KernelPtr)direct_force_kernel<2, 4, MODE_KDK, true, false, false>;
    return (KernelPtr)direct_force_kernel<2, 8, MODE_KDK, true, false, false>;
}

}  // namespace gb

// ================================================================ C ABI
using namespace gb;


static int64_t grid_ctas(gb_direct_t *h, int np, int warps, int packed) {
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, force_kernel_ptr(np, warps, packed), warps * 32, 0);
    if (occ < 1) occ = 1;
    const int per_sm = h->ctas_per_sm > 0 ? std::min(h->ctas_per_sm, occ) : occ;
    return (int64_t)h->sms * per_sm;
}

static int ensure_partials(gb_direct_t *h, int64_t need) {
    if (need <= h->part_cap) return GB_OK;
    if (h->part) cudaFree(h->part);
    h->part = nullptr;
    h->part_cap = 0;
    if (cudaMalloc(&h->part, sizeof(float4) * need) != cudaSuccess)
        return fail(GB_ENOMEM, "partials: cannot allocate %lld bytes", (long long)(sizeof(float4) * need));
    h->part_cap = need;
    return GB_OK;
}

// Whether the scalar force kernel should run on SCALAR_UNIT-source units:
// the longest CTA run over the mean run (the tail the last CTAs add) of the
// coarse split against that of the fine split, which costs about 1.6% more
// per interaction (measured at N = 65,536 and 262,144).
static bool use_fine_units(int64_t n, int np, int warps, int64_t P, int64_t nt = -1) {
    DirectPlan c, f;
    make_plan(n, np, warps, P, &c, 0, nt);
    make_plan(n, np, warps, P, &f, SCALAR_UNIT, nt);
    const double tail_c = (double)((c.U + c.P - 1) / c.P) * (double)c.P / (double)c.U;
    const double tail_f = (double)((f.U + f.P - 1) / f.P) * (double)f.P / (double)f.U * 1.016;
    return tail_f < tail_c;
}

// Scratch for every supported tile shape at n_max, so a call never allocates.
static int64_t max_partials(gb_direct_t *h, int64_t n) {
    int64_t need = 0;
    const int shapes[4][2] = {{1, 4}, {1, 8}, {2, 4}, {2, 8}};
    for (auto &s : shapes)
        for (int packed = 0; packed < 2; ++packed) {
            DirectPlan pl;
            make_plan(n, s[0], s[1], grid_ctas(h, s[0], s[1], packed), &pl);
            need = std::max(need, plan_partials(pl));
            make_plan(n, s[0], s[1], grid_ctas(h, s[0], s[1], packed), &pl, SCALAR_UNIT);
            need = std::max(need, plan_partials(pl));
            make_plan(n, 1, s[1], grid_ctas(h, s[0], s[1], packed), &pl);  // phi layout (K=2)
            need = std::max(need, plan_partials(pl));
        }
    return need;
}

static int check_xm(const void *p, const char *name) {
    if (!p) return fail(GB_EINVAL, "%s is NULL", name);
    if (!aligned16(p)) return fail(GB_EINVAL, "%s is not 16-byte aligned", name);
    return GB_OK;
}

extern "C" int gb_direct_create(gb_direct_t **out, int64_t n_max) {
    if (!out) return fail(GB_EINVAL, "out is NULL");
    *out = nullptr;
    if (n_max < 1 || n_max > (int64_t)1 << 31) return fail(GB_EINVAL, "n_max=%lld out of range", (long long)n_max);
    gb_direct_t *h = new gb_direct();
    GB_CUDA_TRY(cudaGetDevice(&h->device));
    h->sms = num_sms();
    h->n_max = n_max;
    h->np = 2;
    h->warps = 8;
    h->ctas_per_sm = 0;
    h->packed = 0;
    h->adj_variant = 2;
    h->sym_band = 1LL << 30;
    int st = ensure_partials(h, max_partials(h, n_max));
    h->st0_cap = h->sms * 64;  // above every plan's CTA count (ctas_per_sm <= 32)
    if (st == GB_OK && cudaMalloc(&h->st0tab, sizeof(int) * h->st0_cap) != cudaSuccess)
        st = fail(GB_ENOMEM, "CTA table");
    if (st == GB_OK && cudaMalloc(&h->phi, sizeof(float) * n_max) != cudaSuccess)
        st = fail(GB_ENOMEM, "phi scratch");
    h->epart_cap = 4 * h->sms;
    if (st == GB_OK && cudaMalloc(&h->epart, sizeof(double2) * (h->epart_cap + ENERGY_EXTRA)) != cudaSuccess)
        st = fail(GB_ENOMEM, "energy scratch");
    if (st == GB_OK && cudaMemset(h->epart, 0, sizeof(double2) * (h->epart_cap + ENERGY_EXTRA)) != cudaSuccess)
        st = fail(GB_ECUDA, "energy scratch memset");
    if (st == GB_OK && cudaMalloc(&h->diag, sizeof(unsigned long long) * DIAG_COUNT) != cudaSuccess)
        st = fail(GB_ENOMEM, "diag");
    if (st == GB_OK && cudaMemset(h->diag, 0, sizeof(unsigned long long) * DIAG_COUNT) != cudaSuccess)
        st = fail(GB_ECUDA, "diag memset");
    if (st != GB_OK) {
        gb_direct_destroy(h);
        return st;
    }
    *out = h;
    return GB_OK;
}

extern "C" int gb_direct_destroy(gb_direct_t *h) {
    if (!h) return GB_OK;
    for (auto &g : h->gexec)
        if (g) cudaGraphExecDestroy(g);
    if (h->gev_in) cudaEventDestroy(h->gev_in);
    if (h->gev_out) cudaEventDestroy(h->gev_out);
    if (h->gstream) cudaStreamDestroy(h->gstream);
    cudaFree(h->part);
    cudaFree(h->st0tab);
    cudaFree(h->phi);
    cudaFree(h->epart);
    cudaFree(h->diag);
    cudaFree(h->sym);
    delete h;
    return GB_OK;
}

extern "C" int gb_direct_set_tiles(gb_direct_t *h, int k, int warps, int ctas_per_sm) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (k != 2 && k != 4) return fail(GB_EINVAL, "k must be 2 or 4 (got %d)", k);
    if (warps != 4 && warps != 8) return fail(GB_EINVAL, "warps must be 4 or 8 (got %d)", warps);
    if (ctas_per_sm < 0 || ctas_per_sm > 32) return fail(GB_EINVAL, "ctas_per_sm=%d", ctas_per_sm);
    h->np = k / 2;
    h->warps = warps;
    h->ctas_per_sm = ctas_per_sm;
    return GB_OK;
}

// mode MODE_ACC / MODE_KDK: accelerations (or one KDK step), and, when phi
// is not NULL, the potential sums of the same positions in the same pass;
// MODE_PHI: the potential sums alone.  nt >= 0 (MODE_ACC only): the targets
// are particles t0 .. t0 + nt - 1, written to acc[0 .. nt) and phi[0 .. nt),
// on the per-target pass of the handle's variant (the scalar pass for 2).
static int run_direct(gb_direct_t *h, int mode, const float4 *xm, float4 *vel, float4 *acc, float *phi,
                      int64_t n, float G, float eps2, float dt, int flags, cudaStream_t s,
                      const ExtPot &pot = ExtPot{}, int64_t t0 = 0, int64_t nt = -1) {
    const bool range = nt >= 0;
    if (!range) nt = n;
    if (h->packed == 2 && !range) {
        bool done = false;
        GB_TRY(run_direct_sym(h, mode, xm, vel, acc, phi, n, G, eps2, dt, flags, s, pot, &done));
        if (done) return GB_OK;
    }
    // Variant 2 beyond the tile-pair scratch limit runs the scalar pass.
    const int packed = h->packed == 1 ? 1 : 0;
    DirectPlan pl;
    const int np = mode == MODE_PHI ? 1 : h->np;
    const int64_t ctas = grid_ctas(h, h->np, h->warps, packed);
    const bool fine = mode != MODE_PHI && use_fine_units(n, np, h->warps, ctas, nt);
    make_plan(n, np, h->warps, ctas, &pl, fine ? SCALAR_UNIT : 0, nt);
    if (plan_partials(pl) > h->part_cap) return fail(GB_EINVAL, "scratch too small for n=%lld", (long long)n);
    if (pl.P > h->st0_cap) return fail(GB_EINVAL, "%lld CTAs exceed the handle's table", (long long)pl.P);
    DirectArgs a;
    a.xm = xm;
    a.vel = vel;
    a.acc = acc;
    a.part = h->part;
    a.st0tab = h->st0tab;
    a.n = n;
    a.num_ju = pl.num_ju;
    a.U = pl.U;
    a.P = pl.P;
    a.t0 = t0;
    a.nt = nt;
    a.smax = pl.smax;
    a.eps2 = eps2;
    a.h = 0.5f * dt;
    a.dt = dt;
    const bool kahan = !(flags & GB_PLAIN_FP32);
    const bool with_phi = mode != MODE_PHI && phi != nullptr;
    cudaError_t e;
    if (mode == MODE_PHI) {
        const dim3 grid((unsigned)pl.P), block(h->warps * 32);
        if (h->warps == 4) {
            if (kahan) direct_phi_kernel<4, true><<<grid, block, 0, s>>>(a);
            else direct_phi_kernel<4, false><<<grid, block, 0, s>>>(a);
        } else {
            if (kahan) direct_phi_kernel<8, true><<<grid, block, 0, s>>>(a);
            else direct_phi_kernel<8, false><<<grid, block, 0, s>>>(a);
        }
        e = cudaGetLastError();
    } else if (pl.np == 1) {
        e = pl.warps == 4 ? launch_force<1, 4>(mode, kahan, with_phi, pl, a, s, packed, fine)
                          : launch_force<1, 8>(mode, kahan, with_phi, pl, a, s, packed, fine);
    } else {
        e = pl.warps == 4 ? launch_force<2, 4>(mode, kahan, with_phi, pl, a, s, packed, fine)
                          : launch_force<2, 8>(mode, kahan, with_phi, pl, a, s, packed, fine);
    }
    if (e != cudaSuccess) return fail(GB_ECUDA, "force launch: %s", cudaGetErrorString(e));
    FixArgs f;
    f.part = h->part;
    f.st0tab = h->st0tab;
    f.xm = const_cast<float4 *>(xm);
    f.vel = vel;
    f.acc = acc;
    f.phi = phi;
    f.n = nt;
    f.t0 = t0;
    f.num_ju = pl.num_ju;
    f.U = pl.U;
    f.P = pl.P;
    f.st_size = pl.st_size;
    f.smax = pl.smax;
    f.G = G;
    f.h = 0.5f * dt;
    f.dt = dt;
    f.eps2 = eps2;
    f.accumulate = (flags & GB_ACCUMULATE) ? 1 : 0;
    f.pot = pot;
    const unsigned fb = 256, fg = (unsigned)((nt + fb - 1) / fb);
    if (mode == MODE_ACC) {
        if (with_phi) direct_fixup_kernel<MODE_ACC, true><<<fg, fb, 0, s>>>(f);
        else direct_fixup_kernel<MODE_ACC><<<fg, fb, 0, s>>>(f);
    } else if (mode == MODE_KDK) {
        if (with_phi) direct_fixup_kernel<MODE_KDK, true><<<fg, fb, 0, s>>>(f);
        else direct_fixup_kernel<MODE_KDK><<<fg, fb, 0, s>>>(f);
    } else {
        direct_fixup_kernel<MODE_PHI><<<fg, fb, 0, s>>>(f);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return fail(GB_ECUDA, "fix-up launch: %s", cudaGetErrorString(e));
    h->launches += 2;
    return GB_OK;
}

static int check_n(gb_direct_t *h, int64_t n) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (n < 0 || n > h->n_max) return fail(GB_EINVAL, "n=%lld outside [0, n_max=%lld]", (long long)n, (long long)h->n_max);
    return GB_OK;
}

extern "C" int gb_direct_acc(gb_direct_t *h, const float *xm, float *acc, int64_t n, float G, float eps2,
                             int flags, void *stream) {
    GB_TRY(check_n(h, n));
    if (n == 0) return GB_OK;
    GB_TRY(check_xm(xm, "xm"));
    GB_TRY(check_xm(acc, "acc"));
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    return run_direct(h, MODE_ACC, (const float4 *)xm, nullptr, (float4 *)acc, nullptr, n, G, eps2, 0.f,
                      flags, (cudaStream_t)stream);
}

extern "C" int gb_direct_acc_ext(gb_direct_t *h, const float *xm, float *acc, int64_t n, float G, float eps2,
                                 const gb_potential_t *pot, int flags, void *stream) {
    GB_TRY(check_n(h, n));
    ExtPot ep;
    GB_TRY(make_extpot(pot, G, &ep));
    if (n == 0) return GB_OK;
    GB_TRY(check_xm(xm, "xm"));
    GB_TRY(check_xm(acc, "acc"));
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    return run_direct(h, MODE_ACC, (const float4 *)xm, nullptr, (float4 *)acc, nullptr, n, G, eps2, 0.f,
                      flags, (cudaStream_t)stream, ep);
}

// Graph slot g holds `steps` captured KDK steps (the last one also writing
// the potential into phi when phi is not NULL); captured again when the key
// of the slot changed.
static int ensure_graph(gb_direct_t *h, int g, int steps, const gb_direct::Key &key, float *xm, float *vel,
                        float *acc, float *phi, int64_t n, float G, float eps2, float dt, int plain) {
    if (h->gexec[g] && h->gkey[g] == key) return GB_OK;
    if (h->gexec[g]) cudaGraphExecDestroy(h->gexec[g]);
    h->gexec[g] = nullptr;
    GB_CUDA_TRY(cudaStreamBeginCapture(h->gstream, cudaStreamCaptureModeThreadLocal));
    const uint64_t l0 = h->launches;
    int st = GB_OK;
    for (int k = 0; k < steps && st == GB_OK; ++k)
        st = run_direct(h, MODE_KDK, (const float4 *)xm, (float4 *)vel, (float4 *)acc, k == steps - 1 ? phi : nullptr,
                        n, G, eps2, dt, plain, h->gstream);
    h->glaunches[g] = h->launches - l0;
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

// nsteps fused KDK steps; with phi, the last step's force pass also writes
// the potential sums of the final positions.
static int kdk_impl(gb_direct_t *h, float *xm, float *vel, float *acc, float *phi, int64_t n, float G, float eps2,
                    float dt, int64_t nsteps, int flags, void *stream) {
    GB_TRY(check_n(h, n));
    if (n == 0 || nsteps == 0) return GB_OK;
    if (nsteps < 0) return fail(GB_EINVAL, "nsteps < 0");
    GB_TRY(check_xm(xm, "xm"));
    GB_TRY(check_xm(vel, "vel"));
    GB_TRY(check_xm(acc, "acc"));
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    cudaStream_t s = (cudaStream_t)stream;
    const int plain = flags & GB_PLAIN_FP32;
    if (!(flags & GB_USE_GRAPH)) {
        for (int64_t k = 0; k < nsteps; ++k)
            GB_TRY(run_direct(h, MODE_KDK, (const float4 *)xm, (float4 *)vel, (float4 *)acc,
                              k == nsteps - 1 ? phi : nullptr, n, G, eps2, dt, plain, s));
        return GB_OK;
    }
    // Steps captured on the handle's stream and replayed: runs of
    // GRAPH_STEPS steps first, single steps for the rest (one graph launch
    // per GRAPH_STEPS steps keeps small systems off the host's launch rate),
    // and the potential step last.  Tile-pair scratch is sized before the
    // capture (no allocation inside it); its address is part of the key,
    // since the adjoint may regrow it.
    if (h->packed == 2) GB_TRY(reserve_direct_sym(h, n));
    gb_direct::Key key{xm, vel, acc, h->sym, nullptr, n, h->sym_band, G, eps2, dt, plain, h->np, h->warps,
                       h->ctas_per_sm, h->packed};
    if (!h->gstream) {
        GB_CUDA_TRY(cudaStreamCreateWithFlags(&h->gstream, cudaStreamNonBlocking));
        GB_CUDA_TRY(cudaEventCreateWithFlags(&h->gev_in, cudaEventDisableTiming));
        GB_CUDA_TRY(cudaEventCreateWithFlags(&h->gev_out, cudaEventDisableTiming));
    }
    const int64_t plain_steps = phi ? nsteps - 1 : nsteps;
    const int64_t runs = plain_steps / GRAPH_STEPS, rest = plain_steps - runs * GRAPH_STEPS;
    if (runs) GB_TRY(ensure_graph(h, 1, GRAPH_STEPS, key, xm, vel, acc, nullptr, n, G, eps2, dt, plain));
    if (rest) GB_TRY(ensure_graph(h, 0, 1, key, xm, vel, acc, nullptr, n, G, eps2, dt, plain));
    if (phi) {
        key.phi = phi;
        GB_TRY(ensure_graph(h, 2, 1, key, xm, vel, acc, phi, n, G, eps2, dt, plain));
    }
    GB_CUDA_TRY(cudaEventRecord(h->gev_in, s));
    GB_CUDA_TRY(cudaStreamWaitEvent(h->gstream, h->gev_in, 0));
    for (int64_t k = 0; k < runs; ++k) GB_CUDA_TRY(cudaGraphLaunch(h->gexec[1], h->gstream));
    for (int64_t k = 0; k < rest; ++k) GB_CUDA_TRY(cudaGraphLaunch(h->gexec[0], h->gstream));
    if (phi) GB_CUDA_TRY(cudaGraphLaunch(h->gexec[2], h->gstream));
    GB_CUDA_TRY(cudaEventRecord(h->gev_out, h->gstream));
    GB_CUDA_TRY(cudaStreamWaitEvent(s, h->gev_out, 0));
    h->launches += h->glaunches[1] * (uint64_t)runs + h->glaunches[0] * (uint64_t)rest + (phi ? h->glaunches[2] : 0);
    return GB_OK;
}

extern "C" int gb_direct_kdk(gb_direct_t *h, float *xm, float *vel, float *acc, int64_t n, float G, float eps2,
                             float dt, int64_t nsteps, int flags, void *stream) {
    return kdk_impl(h, xm, vel, acc, nullptr, n, G, eps2, dt, nsteps, flags, stream);
}

extern "C" int gb_direct_kdk_phi(gb_direct_t *h, float *xm, float *vel, float *acc, float *phi, int64_t n, float G,
                                 float eps2, float dt, int64_t nsteps, int flags, void *stream) {
    if (!phi && n > 0 && nsteps > 0) return fail(GB_EINVAL, "phi is NULL");
    return kdk_impl(h, xm, vel, acc, phi, n, G, eps2, dt, nsteps, flags, stream);
}

extern "C" int gb_direct_acc_phi(gb_direct_t *h, const float *xm, float *acc, float *phi, int64_t n, float G,
                                 float eps2, int flags, void *stream) {
    GB_TRY(check_n(h, n));
    if (n == 0) return GB_OK;
    GB_TRY(check_xm(xm, "xm"));
    GB_TRY(check_xm(acc, "acc"));
    if (!phi) return fail(GB_EINVAL, "phi is NULL");
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    return run_direct(h, MODE_ACC, (const float4 *)xm, nullptr, (float4 *)acc, phi, n, G, eps2, 0.f, flags,
                      (cudaStream_t)stream);
}

extern "C" int gb_direct_acc_range(gb_direct_t *h, const float *xm, int64_t n, int64_t t0, int64_t nt, float *acc,
                                   float *phi, float G, float eps2, int flags, void *stream) {
    GB_TRY(check_n(h, n));
    if (t0 < 0 || nt < 0 || t0 > n || nt > n - t0)
        return fail(GB_EINVAL, "target range [%lld, %lld) outside [0, n=%lld)", (long long)t0,
                    (long long)(t0 + nt), (long long)n);
    if (flags & ~(GB_ACCUMULATE | GB_PLAIN_FP32))
        return fail(GB_EINVAL, "gb_direct_acc_range: flags 0x%x: only GB_ACCUMULATE and GB_PLAIN_FP32 apply",
                    flags);
    if (nt == 0) return GB_OK;
    GB_TRY(check_xm(xm, "xm"));
    GB_TRY(check_xm(acc, "acc"));
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    return run_direct(h, MODE_ACC, (const float4 *)xm, nullptr, (float4 *)acc, phi, n, G, eps2, 0.f, flags,
                      (cudaStream_t)stream, ExtPot{}, t0, nt);
}

extern "C" int gb_direct_phi(gb_direct_t *h, const float *xm, float *phi, int64_t n, float eps2, int flags,
                             void *stream) {
    GB_TRY(check_n(h, n));
    if (n == 0) return GB_OK;
    GB_TRY(check_xm(xm, "xm"));
    if (!phi) return fail(GB_EINVAL, "phi is NULL");
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    return run_direct(h, MODE_PHI, (const float4 *)xm, nullptr, nullptr, phi, n, 1.f, eps2, 0.f, flags,
                      (cudaStream_t)stream);
}

extern "C" int gb_energy(gb_direct_t *h, const float *xm, const float *vel, int64_t n, float G, float eps2,
                         double *out3, void *stream) {
    GB_TRY(check_n(h, n));
    if (n > 0) {  // an empty system reads neither buffer and gets zeros
        GB_TRY(check_xm(xm, "xm"));
        GB_TRY(check_xm(vel, "vel"));
    }
    if (!out3) return fail(GB_EINVAL, "out3 is NULL");
    if (n > 0) GB_TRY(gb_direct_phi(h, xm, h->phi, n, eps2, 0, stream));
    GB_TRY(launch_energy((const float4 *)xm, (const float4 *)vel, h->phi, n, G, h->epart, h->epart_cap, out3,
                         (cudaStream_t)stream));
    h->launches += 1;
    return GB_OK;
}

extern "C" int gb_energy_phi(gb_direct_t *h, const float *xm, const float *vel, const float *phi, int64_t n,
                             float G, double *out3, void *stream) {
    GB_TRY(check_n(h, n));
    if (n > 0) {
        GB_TRY(check_xm(xm, "xm"));
        GB_TRY(check_xm(vel, "vel"));
        if (!phi) return fail(GB_EINVAL, "phi is NULL");
    }
    if (!out3) return fail(GB_EINVAL, "out3 is NULL");
    GB_TRY(launch_energy((const float4 *)xm, (const float4 *)vel, phi, n, G, h->epart, h->epart_cap, out3,
                         (cudaStream_t)stream));
    h->launches += 1;
    return GB_OK;
}

extern "C" int gb_direct_acc_fp64(const float *xm, int64_t n, const int64_t *targets, int64_t nt, double G,
                                  double eps2, double *acc_out, void *stream) {
    if (n < 0 || nt < 0) return fail(GB_EINVAL, "negative size");
    if (nt == 0) return GB_OK;
    GB_TRY(check_xm(xm, "xm"));
    if (!targets || !acc_out) return fail(GB_EINVAL, "targets/acc_out is NULL");
    if (nt > INT32_MAX) return fail(GB_EINVAL, "too many targets");
    direct_fp64_kernel<<<(unsigned)nt, 256, 0, (cudaStream_t)stream>>>((const float4 *)xm, n, targets, G, eps2,
                                                                       acc_out);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

extern "C" int gb_direct_diag(gb_direct_t *h, gb_diag_t *out, int reset) {
    if (!h || !out) return fail(GB_EINVAL, "NULL argument");
    return read_diag(h->diag, out, reset);
}

extern "C" int gb_direct_set_variant(gb_direct_t *h, int packed) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (packed < 0 || packed > 2) return fail(GB_EINVAL, "variant must be 0, 1 or 2");
    h->packed = packed;
    return GB_OK;
}

extern "C" int gb_direct_set_sym_band(gb_direct_t *h, int64_t bytes) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    // At least one tile pair with its four source slices per band.
    const int64_t min_bytes = (int64_t)sizeof(float4) * SYM_TILE * 5;
    if (bytes < min_bytes) return fail(GB_EINVAL, "band budget %lld below %lld bytes", (long long)bytes,
                                       (long long)min_bytes);
    h->sym_band = bytes;
    return GB_OK;
}

extern "C" uint64_t gb_direct_launch_count(gb_direct_t *h) { return h ? h->launches : 0; }

// ====================================================== allocation-free call
// gb_direct_acc_noalloc: the direct force sum for callers that must not
// allocate device memory (a host that hands its whole GPU memory to its own
// pool, a plug-in living inside another framework's memory arena, or a loop
// that must never stall: cudaMalloc and cudaFree can synchronise the device).
// The stream-K partial sums, which gb_direct_acc keeps in its handle's
// scratch, live here in one file-scope device array instead.  The launch
// shape is fixed (256 CTAs of 4 warps, 2 targets per lane, scalar FP32 with
// Kahan) so that the partials of any n up to GB_NOALLOC_MAX_N fit the array.
//
// The array is shared by every call in the process on a given device and
// keeps whatever the previous call left in it.  Nothing in it has to start
// at zero: each call writes every partial slot it later reads.  Two calls
// whose kernels overlap on the GPU (different streams, or different host
// threads) write the same slots and race; the caller must order them.
constexpr int NOALLOC_CTAS = 256;
constexpr int NOALLOC_NP = 1;     // 2 targets per lane
constexpr int NOALLOC_WARPS = 4;  // supertile of 256 targets
constexpr int64_t NOALLOC_PART = 2LL * NOALLOC_CTAS * 2 * (NOALLOC_WARPS * 32 * 2 * NOALLOC_NP);  // float4s

static __device__ __align__(256) float4 g_noalloc_part[NOALLOC_PART];
static __device__ int g_noalloc_tab[NOALLOC_CTAS];  // first supertile per CTA

// Device addresses of g_noalloc_part and g_noalloc_tab per device: in host
// code the symbol names are only host-side stand-ins, so the addresses are
// looked up once per device (with that device current) and cached.  The
// cache is read without a lock (acquire loads); the first lookup on a
// device runs under a mutex, so concurrent first calls from several host
// threads look it up once.  A cudaDeviceReset of that device unloads the
// module and moves the array: the cached address is then stale (as is every
// device buffer the caller held), so the entry point must not be used on a
// device after it was reset.
static std::atomic<void *> g_noalloc_addr[GB_NOALLOC_MAX_DEVICES];
static std::atomic<void *> g_noalloc_tab_addr[GB_NOALLOC_MAX_DEVICES];
static std::mutex g_noalloc_mu;

static int noalloc_addresses(int dev, void **part, void **tab) {
    *part = g_noalloc_addr[dev].load(std::memory_order_acquire);
    *tab = g_noalloc_tab_addr[dev].load(std::memory_order_acquire);
    if (*part && *tab) return GB_OK;
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    *part = g_noalloc_addr[dev].load(std::memory_order_acquire);
    *tab = g_noalloc_tab_addr[dev].load(std::memory_order_acquire);
    if (*part && *tab) return GB_OK;
    void *p = nullptr, *t = nullptr;
    GB_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_part));
    GB_CUDA_TRY(cudaGetSymbolAddress(&t, g_noalloc_tab));
    g_noalloc_tab_addr[dev].store(t, std::memory_order_release);
    g_noalloc_addr[dev].store(p, std::memory_order_release);
    *part = p;
    *tab = t;
    return GB_OK;
}

extern "C" int gb_direct_acc_noalloc(const float *xm, float *acc, int64_t n, float G, float eps2, int flags,
                                     void *stream) {
    if (n < 0 || n > GB_NOALLOC_MAX_N)
        return fail(GB_EINVAL, "gb_direct_acc_noalloc: n=%lld outside [0, %d]; use gb_direct_acc for larger systems",
                    (long long)n, GB_NOALLOC_MAX_N);
    if (flags & ~(GB_ACCUMULATE | GB_PLAIN_FP32))
        return fail(GB_EINVAL, "gb_direct_acc_noalloc: flags 0x%x: only GB_ACCUMULATE and GB_PLAIN_FP32 apply",
                    flags);
    if (n == 0) return GB_OK;
    GB_TRY(check_xm(xm, "xm"));
    GB_TRY(check_xm(acc, "acc"));
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    int dev = 0;
    GB_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= GB_NOALLOC_MAX_DEVICES) return fail(GB_EINVAL, "device index %d not supported", dev);
    void *part_addr = nullptr, *tab_addr = nullptr;
    GB_TRY(noalloc_addresses(dev, &part_addr, &tab_addr));
    DirectPlan pl;
    const bool fine = use_fine_units(n, NOALLOC_NP, NOALLOC_WARPS, NOALLOC_CTAS);
    make_plan(n, NOALLOC_NP, NOALLOC_WARPS, NOALLOC_CTAS, &pl, fine ? SCALAR_UNIT : 0);
    if (plan_partials(pl) > NOALLOC_PART)
        return fail(GB_EINVAL, "gb_direct_acc_noalloc: partials for n=%lld exceed the static scratch", (long long)n);
    DirectArgs a;
    a.xm = (const float4 *)xm;
    a.vel = nullptr;
    a.acc = nullptr;
    a.part = (float4 *)part_addr;
    a.st0tab = (int *)tab_addr;
    a.n = n;
    a.num_ju = pl.num_ju;
    a.U = pl.U;
    a.P = pl.P;
    a.t0 = 0;
    a.nt = n;
    a.smax = pl.smax;
    a.eps2 = eps2;
    a.h = 0.f;
    a.dt = 0.f;
    cudaStream_t s = (cudaStream_t)stream;
    const dim3 grid((unsigned)pl.P);
    const bool kahan = !(flags & GB_PLAIN_FP32);
    if (fine) launch_scalar<NOALLOC_NP, NOALLOC_WARPS, true>(MODE_ACC, kahan, false, grid, a, s);
    else launch_scalar<NOALLOC_NP, NOALLOC_WARPS, false>(MODE_ACC, kahan, false, grid, a, s);
    GB_CUDA_TRY(cudaGetLastError());
    FixArgs f;
    f.part = a.part;
    f.st0tab = a.st0tab;
    f.xm = const_cast<float4 *>(a.xm);
    f.vel = nullptr;
    f.acc = (float4 *)acc;
    f.phi = nullptr;
    f.n = n;
    f.t0 = 0;
    f.num_ju = pl.num_ju;
    f.U = pl.U;
    f.P = pl.P;
    f.st_size = pl.st_size;
    f.smax = pl.smax;
    f.G = G;
    f.h = 0.f;
    f.dt = 0.f;
    f.eps2 = eps2;
    f.accumulate = (flags & GB_ACCUMULATE) ? 1 : 0;
    f.pot = ExtPot{};
    direct_fixup_kernel<MODE_ACC><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}
