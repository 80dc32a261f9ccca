// Batched direct N^2 for many independent systems of uneven size (sm_103a).
//
// All systems live concatenated in one set of float4 arrays.  The work of
// every system is cut into units (system, target supertile, source chunk)
// that are numbered globally, system after system, supertile-major; one
// persistent launch of P CTAs gives each CTA an equal contiguous run of
// units, so a CTA may finish the tail of one system and start the next:
// small and large systems share the GPU evenly and no launch is spent per
// system.  A CTA writes one compensated partial per global supertile it
// touches, at slot (global supertile + CTA): consecutive CTAs overlap in at
// most one supertile, so the slots never collide and need no padding.  The
// fix-up kernel merges each target's partials in CTA order and applies the
// KDK epilogue.  gb_batch_kdk can capture the whole nsteps loop (two
// launches per step) as one CUDA graph and replay it.
//
// The reference runs one system per Engine (core/engine.py:108-116); the
// per-system loop (gb_batch_kdk_loop) is the plain alternative measured
// against the batched launch.
#include <algorithm>
#include <vector>

#include "gb_direct_core.cuh"

namespace gb {

enum BatchMode { BMODE_ACC = 0, BMODE_KDK = 1 };

struct BatchArgs {
    const float4 *__restrict__ xm;
    const float4 *__restrict__ vel;
    const float4 *__restrict__ acc;
    float4 *__restrict__ part;
    const int64_t *__restrict__ off;     // nsys + 1 particle offsets
    const int64_t *__restrict__ ubase;   // nsys + 1 global unit bases
    const int64_t *__restrict__ stbase;  // nsys + 1 global supertile bases
    int nsys;
    int64_t U, P;
    float eps2, h, dt;
};

template <int MODE>
__device__ __forceinline__ float4 load_b(const BatchArgs &a, int64_t o, int64_t n_s, int64_t li) {
    if (li >= n_s) return make_float4(0.f, 0.f, 0.f, 0.f);
    float4 x = __ldg(a.xm + o + li);
    if (MODE == BMODE_KDK) x = predict_xm(x, __ldg(a.vel + o + li), __ldg(a.acc + o + li), a.h, a.dt);
    return x;
}

template <int NP, int WARPS, int MODE, bool KAHAN>
__global__ void __launch_bounds__(WARPS * 32, NP == 1 ? 1024 / (WARPS * 32) : 1)
batch_force_kernel(BatchArgs a) {
    constexpr int K = 2 * NP;
    constexpr int TILE = 32 * K;
    constexpr int ST = WARPS * TILE;
    constexpr int JU = WARPS * 32;
    __shared__ float4 src[JU];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t c = blockIdx.x;
    const int64_t u_begin = a.U * c / a.P, u_end = a.U * (c + 1) / a.P;
    if (u_begin >= u_end) return;
    int s = find_base(a.ubase, a.nsys, u_begin);
    int64_t u = u_begin;
    while (u < u_end) {
        while (s + 1 < a.nsys && u >= __ldg(a.ubase + s + 1)) ++s;
        const int64_t o = __ldg(a.off + s), n_s = __ldg(a.off + s + 1) - o;
        const int64_t ub = __ldg(a.ubase + s);
        const int64_t nju = (n_s + JU - 1) / JU;
        const int64_t st = (u - ub) / nju;
        const int64_t run_end = min(u_end, ub + (st + 1) * nju);
        const int64_t gst = __ldg(a.stbase + s) + st;
        const int64_t tl = st * ST + wib * TILE + lane;
        float X[K], Y[K], Z[K], SX[K], SY[K], SZ[K], CX[K], CY[K], CZ[K];
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const float4 t = load_b<MODE>(a, o, n_s, tl + q * 32);
            X[q] = t.x; Y[q] = t.y; Z[q] = t.z;
            SX[q] = SY[q] = SZ[q] = CX[q] = CY[q] = CZ[q] = 0.f;
        }
        for (; u < run_end; ++u) {
            const int64_t ju = (u - ub) - st * nju;
            const float4 s4 = load_b<MODE>(a, o, n_s, ju * JU + threadIdx.x);
            __syncthreads();
            src[threadIdx.x] = s4;
            __syncthreads();
            float AX[K], AY[K], AZ[K], PW[K];
#pragma unroll
            for (int q = 0; q < K; ++q) AX[q] = AY[q] = AZ[q] = PW[q] = 0.f;
            interact_chunk<K, JU>(src, X, Y, Z, AX, AY, AZ, PW, a.eps2);
#pragma unroll
            for (int q = 0; q < K; ++q) {
                if (KAHAN) {
                    kahan_add(SX[q], CX[q], AX[q]);
                    kahan_add(SY[q], CY[q], AY[q]);
                    kahan_add(SZ[q], CZ[q], AZ[q]);
                } else {
                    SX[q] += AX[q]; SY[q] += AY[q]; SZ[q] += AZ[q];
                }
            }
        }
        const int64_t slot = (gst + c) * ST + wib * TILE + lane;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            const int64_t sq = slot + q * 32;
            a.part[2 * sq] = make_float4(SX[q], SY[q], SZ[q], 0.f);
            a.part[2 * sq + 1] = make_float4(-CX[q], -CY[q], -CZ[q], 0.f);
        }
    }
}

struct BatchFix {
    const float4 *__restrict__ part;
    float4 *xm, *vel, *acc;
    const int64_t *__restrict__ off;
    const int64_t *__restrict__ ubase;
    const int64_t *__restrict__ stbase;
    int nsys;
    int64_t ntot, U, P, st_size, ju;
    float G, h, dt;
    int accumulate;
};

template <int MODE>
__global__ void batch_fixup_kernel(BatchFix f) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.ntot) return;
    const int s = find_base(f.off, f.nsys, i);
    const int64_t o = __ldg(f.off + s), n_s = __ldg(f.off + s + 1) - o;
    const int64_t li = i - o;
    const int64_t nju = (n_s + f.ju - 1) / f.ju;
    const int64_t st = li / f.st_size, r = li - st * f.st_size;
    const int64_t g0 = __ldg(f.ubase + s) + st * nju;
    const int64_t c_lo = ((g0 + 1) * f.P - 1) / f.U;
    const int64_t c_hi = ((g0 + nju) * f.P - 1) / f.U;
    const int64_t gst = __ldg(f.stbase + s) + st;
    const float3 sum = merge_partials(f.part, c_lo, c_hi, [&](int64_t c) { return (gst + c) * f.st_size + r; });
    const float4 an = make_float4(f.G * sum.x, f.G * sum.y, f.G * sum.z, 0.f);
    if (MODE == BMODE_KDK) {
        kdk_writeback(f.xm, f.vel, f.acc, i, an, f.h, f.dt);
    } else if (f.accumulate) {
        float4 v = f.acc[i];
        v.x += an.x; v.y += an.y; v.z += an.z;
        f.acc[i] = v;
    } else {
        f.acc[i] = an;
    }
}

typedef const void *KPtr;

static KPtr batch_kernel_ptr(int np, int warps) {
    if (np == 1 && warps == 4) return (KPtr)batch_force_kernel<1, 4, BMODE_KDK, true>;
    if (np == 1 && warps == 8) return (KPtr)batch_force_kernel<1, 8, BMODE_KDK, true>;
    if (np == 2 && warps == 4) return (KPtr)batch_force_kernel<2, 4, BMODE_KDK, true>;
    return (KPtr)batch_force_kernel<2, 8, BMODE_KDK, true>;
}

template <int NP, int WARPS>
static void launch_batch(int mode, bool kahan, unsigned grid, const BatchArgs &a, cudaStream_t s) {
    if (mode == BMODE_ACC) {
        if (kahan) batch_force_kernel<NP, WARPS, BMODE_ACC, true><<<grid, WARPS * 32, 0, s>>>(a);
        else batch_force_kernel<NP, WARPS, BMODE_ACC, false><<<grid, WARPS * 32, 0, s>>>(a);
    } else {
        if (kahan) batch_force_kernel<NP, WARPS, BMODE_KDK, true><<<grid, WARPS * 32, 0, s>>>(a);
        else batch_force_kernel<NP, WARPS, BMODE_KDK, false><<<grid, WARPS * 32, 0, s>>>(a);
    }
}

}  // namespace gb

// ================================================================ C ABI
using namespace gb;

struct GraphKey {
    const void *xm, *vel, *acc;
    float G, eps2, dt;
    int64_t nsteps;
    int np, warps, ctas_per_sm, flags, variant;
    bool operator==(const GraphKey &o) const {
        return xm == o.xm && vel == o.vel && acc == o.acc && G == o.G && eps2 == o.eps2 && dt == o.dt &&
               nsteps == o.nsteps && np == o.np && warps == o.warps && ctas_per_sm == o.ctas_per_sm &&
               flags == o.flags && variant == o.variant;
    }
};

struct gb_batch {
    int device, sms;
    int nsys;
    std::vector<int64_t> off;  // host copy, nsys + 1
    int64_t ntot, nmax_sys;
    int np, warps, ctas_per_sm;
    int64_t *d_off, *d_ubase, *d_stbase;
    int64_t U, P, st_size, ju;
    float4 *part;
    int64_t part_cap;
    cudaStream_t cstream;
    cudaEvent_t ev_in, ev_out;
    cudaGraphExec_t graph;
    GraphKey gkey;
    bool has_graph;
    gb_direct_t *loop;  // per-system handle for gb_batch_kdk_loop (lazy)
    uint64_t launches;
    // Symmetric pass (variant 1): its tables (unit, column-slot and fix-up
    // block bases, nsys + 1 each) and scratch, allocated on first selection.
    int variant;
    int64_t *d_symtab;
    int *d_fsys;
    float4 *sym;
    SymBatch symb;
};

// Tables and scratch of the symmetric pass (tiles of SYM_TILE particles;
// units are system after system, tile pairs row-major, Q slices each).
static int batch_sym_plan(gb_batch_t *h) {
    if (h->sym) return GB_OK;
    const int ns = h->nsys;
    std::vector<int64_t> tab(3 * (ns + 1), 0);
    int64_t *ub = tab.data(), *cb = ub + ns + 1, *fb = cb + ns + 1;
    int64_t pairs = 0;
    for (int s = 0; s < ns; ++s) {
        const int64_t n = h->off[s + 1] - h->off[s], nt = (n + SYM_TILE - 1) / SYM_TILE;
        pairs += nt * (nt + 1) / 2;
    }
    const SymShape sh = direct_sym_shape(h->sms, pairs);
    const int64_t slots = sh.slots;
    const int Q = sh.Q;
    for (int s = 0; s < ns; ++s) {
        const int64_t n = h->off[s + 1] - h->off[s], nt = (n + SYM_TILE - 1) / SYM_TILE;
        ub[s + 1] = ub[s] + nt * (nt + 1) / 2 * Q;
        cb[s + 1] = cb[s] + nt * (nt + 1) / 2;
        fb[s + 1] = fb[s] + (n + 31) / 32;
    }
    const int64_t NU = ub[ns], need = (NU + pairs) * SYM_TILE + 1;
    if (need * (int64_t)sizeof(float4) > SYM_MAX_BYTES)
        return fail(GB_EINVAL, "symmetric batch pass needs %lld bytes of scratch (limit %lld)",
                    (long long)(need * 16), (long long)SYM_MAX_BYTES);
    if (fb[ns] > INT32_MAX) return fail(GB_EINVAL, "too many particles for the symmetric batch fix-up");
    std::vector<int> fsys(fb[ns]);
    for (int s = 0; s < ns; ++s)
        for (int64_t k = fb[s]; k < fb[s + 1]; ++k) fsys[k] = s;
    auto release = [&]() {
        cudaFree(h->d_symtab);
        cudaFree(h->d_fsys);
        cudaFree(h->sym);
        h->d_symtab = nullptr;
        h->d_fsys = nullptr;
        h->sym = nullptr;
    };
    if (cudaMalloc(&h->d_symtab, sizeof(int64_t) * tab.size()) != cudaSuccess ||
        cudaMalloc(&h->d_fsys, sizeof(int) * fsys.size()) != cudaSuccess ||
        cudaMalloc(&h->sym, sizeof(float4) * need) != cudaSuccess) {
        release();
        return fail(GB_ENOMEM, "symmetric batch tables and scratch (%lld bytes)", (long long)(need * 16));
    }
    if (cudaMemcpy(h->d_symtab, tab.data(), sizeof(int64_t) * tab.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(h->d_fsys, fsys.data(), sizeof(int) * fsys.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
        release();
        return fail(GB_ECUDA, "symmetric batch tables upload");
    }
    SymBatch &b = h->symb;
    b.off = h->d_off;
    b.ubase = h->d_symtab;
    b.cbase = h->d_symtab + ns + 1;
    b.fbase = h->d_symtab + 2 * (ns + 1);
    b.fsys = h->d_fsys;
    b.nsys = ns;
    b.Q = Q;
    b.NU = NU;
    b.NPtot = pairs;
    b.nfb = fb[ns];
    b.P = std::min<int64_t>(slots, NU);
    b.scratch = h->sym;
    return GB_OK;
}

// Unit and supertile tables for the current tile shape (host, uploaded).
static int batch_plan(gb_batch_t *h, int np, int warps, int ctas_per_sm, bool upload) {
    const int64_t st = (int64_t)warps * 32 * 2 * np, ju = (int64_t)warps * 32;
    std::vector<int64_t> ub(h->nsys + 1), sb(h->nsys + 1);
    ub[0] = sb[0] = 0;
    for (int s = 0; s < h->nsys; ++s) {
        const int64_t n = h->off[s + 1] - h->off[s];
        const int64_t nst = (n + st - 1) / st, nju = (n + ju - 1) / ju;
        ub[s + 1] = ub[s] + nst * nju;
        sb[s + 1] = sb[s] + nst;
    }
    int occ = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel_ptr(np, warps), warps * 32, 0);
    occ = std::max(occ, 1);
    const int per_sm = ctas_per_sm > 0 ? std::min(ctas_per_sm, occ) : occ;
    const int64_t U = ub[h->nsys];
    const int64_t P = std::max<int64_t>(1, std::min<int64_t>((int64_t)h->sms * per_sm, U));
    const int64_t need = 2 * (sb[h->nsys] + P) * st;
    if (!upload) {
        h->part_cap = std::max(h->part_cap, need);
        return GB_OK;
    }
    if (need > h->part_cap) return fail(GB_EINVAL, "batch partial scratch too small");
    GB_CUDA_TRY(cudaMemcpy(h->d_ubase, ub.data(), sizeof(int64_t) * (h->nsys + 1), cudaMemcpyHostToDevice));
    GB_CUDA_TRY(cudaMemcpy(h->d_stbase, sb.data(), sizeof(int64_t) * (h->nsys + 1), cudaMemcpyHostToDevice));
    h->np = np;
    h->warps = warps;
    h->ctas_per_sm = ctas_per_sm;
    h->U = U;
    h->P = P;
    h->st_size = st;
    h->ju = ju;
    return GB_OK;
}

extern "C" int gb_batch_destroy(gb_batch_t *h) {
    if (!h) return GB_OK;
    if (h->has_graph) cudaGraphExecDestroy(h->graph);
    if (h->cstream) cudaStreamDestroy(h->cstream);
    if (h->ev_in) cudaEventDestroy(h->ev_in);
    if (h->ev_out) cudaEventDestroy(h->ev_out);
    cudaFree(h->d_off);
    cudaFree(h->d_ubase);
    cudaFree(h->d_stbase);
    cudaFree(h->part);
    cudaFree(h->d_symtab);
    cudaFree(h->d_fsys);
    cudaFree(h->sym);
    if (h->loop) gb_direct_destroy(h->loop);
    delete h;
    return GB_OK;
}

extern "C" int gb_batch_create(gb_batch_t **out, const int64_t *sizes, int nsys) {
    if (!out) return fail(GB_EINVAL, "out is NULL");
    *out = nullptr;
    if (!sizes || nsys < 1) return fail(GB_EINVAL, "need at least one system");
    gb_batch_t *h = new gb_batch();
    h->nsys = nsys;
    h->off.assign(nsys + 1, 0);
    h->nmax_sys = 0;
    for (int s = 0; s < nsys; ++s) {
        if (sizes[s] < 1 || sizes[s] > ((int64_t)1 << 30)) {
            delete h;
            return fail(GB_EINVAL, "system %d has size %lld", s, (long long)sizes[s]);
        }
        h->off[s + 1] = h->off[s] + sizes[s];
        h->nmax_sys = std::max(h->nmax_sys, sizes[s]);
    }
    h->ntot = h->off[nsys];
    int st = GB_OK;
    if (cudaGetDevice(&h->device) != cudaSuccess) st = fail(GB_ECUDA, "cudaGetDevice");
    h->sms = num_sms();
    const int shapes[4][2] = {{1, 4}, {1, 8}, {2, 4}, {2, 8}};
    for (auto &sh : shapes) batch_plan(h, sh[0], sh[1], 0, false);
    const size_t tb = sizeof(int64_t) * (nsys + 1);
    if (st == GB_OK && (cudaMalloc(&h->d_off, tb) != cudaSuccess || cudaMalloc(&h->d_ubase, tb) != cudaSuccess ||
                        cudaMalloc(&h->d_stbase, tb) != cudaSuccess ||
                        cudaMalloc(&h->part, sizeof(float4) * h->part_cap) != cudaSuccess))
        st = fail(GB_ENOMEM, "gb_batch_create: device allocation failed");
    if (st == GB_OK && cudaMemcpy(h->d_off, h->off.data(), tb, cudaMemcpyHostToDevice) != cudaSuccess)
        st = fail(GB_ECUDA, "gb_batch_create: copy of offsets failed");
    if (st == GB_OK && (cudaStreamCreateWithFlags(&h->cstream, cudaStreamNonBlocking) != cudaSuccess ||
                        cudaEventCreateWithFlags(&h->ev_in, cudaEventDisableTiming) != cudaSuccess ||
                        cudaEventCreateWithFlags(&h->ev_out, cudaEventDisableTiming) != cudaSuccess))
        st = fail(GB_ECUDA, "gb_batch_create: stream/event creation failed");
    if (st == GB_OK) st = batch_plan(h, 2, 8, 0, true);
    if (st != GB_OK) {
        gb_batch_destroy(h);
        return st;
    }
    *out = h;
    return GB_OK;
}

extern "C" int gb_batch_set_tiles(gb_batch_t *h, int k, int warps, int ctas_per_sm) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (k != 2 && k != 4) return fail(GB_EINVAL, "k must be 2 or 4 (got %d)", k);
    if (warps != 4 && warps != 8) return fail(GB_EINVAL, "warps must be 4 or 8 (got %d)", warps);
    if (ctas_per_sm < 0 || ctas_per_sm > 32) return fail(GB_EINVAL, "ctas_per_sm=%d", ctas_per_sm);
    return batch_plan(h, k / 2, warps, ctas_per_sm, true);
}

extern "C" int gb_batch_set_variant(gb_batch_t *h, int variant) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (variant != 0 && variant != 1) return fail(GB_EINVAL, "variant must be 0 or 1 (got %d)", variant);
    if (variant == 1) GB_TRY(batch_sym_plan(h));
    h->variant = variant;
    return GB_OK;
}

extern "C" int64_t gb_batch_total(gb_batch_t *h) { return h ? h->ntot : -1; }

static int batch_step(gb_batch_t *h, int mode, const float4 *xm, float4 *vel, float4 *acc, float G, float eps2,
                      float dt, int flags, cudaStream_t s) {
    if (h->variant == 1) {
        GB_TRY(run_batch_sym(h->symb, mode, xm, vel, acc, G, eps2, dt, flags, s));
        h->launches += 2;
        return GB_OK;
    }
    BatchArgs a;
    a.xm = xm;
    a.vel = vel;
    a.acc = acc;
    a.part = h->part;
    a.off = h->d_off;
    a.ubase = h->d_ubase;
    a.stbase = h->d_stbase;
    a.nsys = h->nsys;
    a.U = h->U;
    a.P = h->P;
    a.eps2 = eps2;
    a.h = 0.5f * dt;
    a.dt = dt;
    const bool kahan = !(flags & GB_PLAIN_FP32);
    const unsigned grid = (unsigned)h->P;
    if (h->np == 1) {
        if (h->warps == 4) launch_batch<1, 4>(mode, kahan, grid, a, s);
        else launch_batch<1, 8>(mode, kahan, grid, a, s);
    } else {
        if (h->warps == 4) launch_batch<2, 4>(mode, kahan, grid, a, s);
        else launch_batch<2, 8>(mode, kahan, grid, a, s);
    }
    GB_CUDA_TRY(cudaGetLastError());
    BatchFix f;
    f.part = h->part;
    f.xm = const_cast<float4 *>(xm);
    f.vel = vel;
    f.acc = acc;
    f.off = h->d_off;
    f.ubase = h->d_ubase;
    f.stbase = h->d_stbase;
    f.nsys = h->nsys;
    f.ntot = h->ntot;
    f.U = h->U;
    f.P = h->P;
    f.st_size = h->st_size;
    f.ju = h->ju;
    f.G = G;
    f.h = 0.5f * dt;
    f.dt = dt;
    f.accumulate = (flags & GB_ACCUMULATE) ? 1 : 0;
    const unsigned fg = (unsigned)((h->ntot + 255) / 256);
    if (mode == BMODE_KDK) batch_fixup_kernel<BMODE_KDK><<<fg, 256, 0, s>>>(f);
    else batch_fixup_kernel<BMODE_ACC><<<fg, 256, 0, s>>>(f);
    GB_CUDA_TRY(cudaGetLastError());
    h->launches += 2;
    return GB_OK;
}

static int check_buf(const void *p, const char *name) {
    if (!p) return fail(GB_EINVAL, "%s is NULL", name);
    if (!aligned16(p)) return fail(GB_EINVAL, "%s is not 16-byte aligned", name);
    return GB_OK;
}

extern "C" int gb_batch_acc(gb_batch_t *h, const float *xm, float *acc, float G, float eps2, int flags,
                            void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    GB_TRY(check_buf(xm, "xm"));
    GB_TRY(check_buf(acc, "acc"));
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    return batch_step(h, BMODE_ACC, (const float4 *)xm, nullptr, (float4 *)acc, G, eps2, 0.f, flags,
                      (cudaStream_t)stream);
}

extern "C" int gb_batch_kdk(gb_batch_t *h, float *xm, float *vel, float *acc, float G, float eps2, float dt,
                            int64_t nsteps, int flags, void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (nsteps < 0) return fail(GB_EINVAL, "nsteps < 0");
    if (nsteps == 0) return GB_OK;
    GB_TRY(check_buf(xm, "xm"));
    GB_TRY(check_buf(vel, "vel"));
    GB_TRY(check_buf(acc, "acc"));
    if (!(eps2 > 0.f)) return fail(GB_EINVAL, "eps2 must be > 0");
    cudaStream_t s = (cudaStream_t)stream;
    if (!(flags & GB_USE_GRAPH)) {
        for (int64_t k = 0; k < nsteps; ++k)
            GB_TRY(batch_step(h, BMODE_KDK, (const float4 *)xm, (float4 *)vel, (float4 *)acc, G, eps2, dt, flags, s));
        return GB_OK;
    }
    const GraphKey key{xm, vel, acc, G, eps2, dt, nsteps, h->np, h->warps, h->ctas_per_sm, flags, h->variant};
    if (!h->has_graph || !(h->gkey == key)) {
        if (h->has_graph) {
            cudaGraphExecDestroy(h->graph);
            h->has_graph = false;
        }
        // Capture the whole step loop on the handle's own stream.
        GB_CUDA_TRY(cudaStreamBeginCapture(h->cstream, cudaStreamCaptureModeThreadLocal));
        const uint64_t l0 = h->launches;
        int st = GB_OK;
        for (int64_t k = 0; k < nsteps && st == GB_OK; ++k)
            st = batch_step(h, BMODE_KDK, (const float4 *)xm, (float4 *)vel, (float4 *)acc, G, eps2, dt, flags,
                            h->cstream);
        h->launches = l0;
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->cstream, &graph);
        if (st != GB_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (e != cudaSuccess) return fail(GB_ECUDA, "graph capture: %s", cudaGetErrorString(e));
        const cudaError_t ei = cudaGraphInstantiate(&h->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (ei != cudaSuccess) return fail(GB_ECUDA, "graph instantiate: %s", cudaGetErrorString(ei));
        h->has_graph = true;
        h->gkey = key;
    }
    GB_CUDA_TRY(cudaEventRecord(h->ev_in, s));
    GB_CUDA_TRY(cudaStreamWaitEvent(h->cstream, h->ev_in, 0));
    GB_CUDA_TRY(cudaGraphLaunch(h->graph, h->cstream));
    GB_CUDA_TRY(cudaEventRecord(h->ev_out, h->cstream));
    GB_CUDA_TRY(cudaStreamWaitEvent(s, h->ev_out, 0));
    h->launches += 2 * (uint64_t)nsteps;
    return GB_OK;
}

extern "C" int gb_batch_kdk_loop(gb_batch_t *h, float *xm, float *vel, float *acc, float G, float eps2, float dt,
                                 int64_t nsteps, int flags, void *stream) {
    if (!h) return fail(GB_EINVAL, "handle is NULL");
    if (!h->loop) GB_TRY(gb_direct_create(&h->loop, h->nmax_sys));
    float4 *x = (float4 *)xm, *v = (float4 *)vel, *a = (float4 *)acc;
    const uint64_t l0 = gb_direct_launch_count(h->loop);
    for (int64_t k = 0; k < nsteps; ++k)
        for (int s = 0; s < h->nsys; ++s) {
            const int64_t o = h->off[s], n = h->off[s + 1] - o;
            GB_TRY(gb_direct_kdk(h->loop, (float *)(x + o), (float *)(v + o), (float *)(a + o), n, G, eps2, dt, 1,
                                 flags & GB_PLAIN_FP32, stream));
        }
    h->launches += gb_direct_launch_count(h->loop) - l0;
    return GB_OK;
}

extern "C" uint64_t gb_batch_launch_count(gb_batch_t *h) { return h ? h->launches : 0; }
