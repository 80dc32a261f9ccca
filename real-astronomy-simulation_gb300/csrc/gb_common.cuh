// Shared device/host helpers for the GB300 self-gravity engine (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/gbgrav.h"

namespace gb {

// ---------------------------------------------------------------- status
// Per-thread last error text, returned by gb_last_error_string().
void set_error(const char *fmt, ...);
int fail(int code, const char *fmt, ...);

#define GB_CUDA_TRY(expr)                                                    \
    do {                                                                     \
        cudaError_t e_ = (expr);                                             \
        if (e_ != cudaSuccess)                                               \
            return ::gb::fail(GB_ECUDA, "%s failed: %s (%s:%d)", #expr,      \
                              cudaGetErrorString(e_), __FILE__, __LINE__);   \
    } while (0)

#define GB_TRY(expr)                                                         \
    do {                                                                     \
        int s_ = (expr);                                                     \
        if (s_ != GB_OK) return s_;                                          \
    } while (0)

inline bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Device-side diagnostic counters (one block per context, zeroed at create).
// Index meaning is fixed by the C-ABI (gb_diag_t field order).
enum DiagIndex {
    DIAG_STACK_DROPS = 0,     // pushes skipped by the max_stack rule
    DIAG_STACK_OVERFLOW = 1,  // warp stack capacity hit (never expected)
    DIAG_NONFINITE = 2,       // non-finite key-quantisation inputs
    DIAG_BAD_TREE = 3,        // inconsistent index met (never for a valid tree)
    DIAG_NODE_READS = 4,      // traversal work counters (see gb_diag_t)
    DIAG_ROOT_READS = 5,
    DIAG_INTERACTIONS = 6,
    DIAG_TESTS = 7,
    DIAG_WAIT_TIMEOUT = 8,    // bounded device waits that gave up (never expected)
    DIAG_COUNT = 9
};

int num_sms();

// Copies the device counters into the C-ABI struct (synchronising).
int read_diag(unsigned long long *dev, gb_diag_t *out, int reset);

// FP64 energies into out3 (KE, PE = -1/2 G sum m phi, total) from n float4
// records and the potential sums phi, in one launch: per-block partials into
// epart (at most epart_cap blocks), and the last block to finish adds them
// in block order.  epart holds epart_cap + ENERGY_EXTRA double2: the partials,
// then an arrival ticket (zero between calls; set to zero at allocation),
// then a device copy of out3.  out3 in host memory (pinned or pageable):
// the kernel writes the device copy, which is copied to out3, and the call
// waits for stream s.
constexpr int ENERGY_EXTRA = 3;
int launch_energy(const float4 *xm, const float4 *vel, const float *phi, int64_t n, float G, double2 *epart,
                  int epart_cap, double *out3, cudaStream_t s);

// ------------------------------------------------------- packed FP32 pairs
// Blackwell executes two FP32 operations per lane per instruction with the
// .f32x2 forms; a pair lives in one 64-bit register.
typedef unsigned long long f2;

__device__ __forceinline__ f2 pack2(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void unpack2(f2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}

// Hardware reciprocal square root (MUFU), flush-to-zero: the argument is
// always >= eps^2 > 0 on the gravity paths.
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ f2 rsqrt2(f2 v) {
    float a, b;
    unpack2(v, a, b);
    return pack2(rsqrt_approx(a), rsqrt_approx(b));
}

// Kahan-compensated add of x into (s, c); s - c is the running estimate.
__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}
__device__ __forceinline__ void kahan_add2(f2 &s, f2 &c, f2 x) {
    const f2 y = sub2(x, c);
    const f2 t = add2(s, y);
    c = sub2(sub2(t, s), y);
    s = t;
}

// Leapfrog predictor used identically for targets and sources so that a
// particle's own source copy sits exactly on its target position:
// v_half = v + a*dt/2 (kick), x' = x + v_half*dt (drift).
__device__ __forceinline__ float kick(float v, float a, float h) { return __fmaf_rn(a, h, v); }
__device__ __forceinline__ float drift(float x, float vh, float dt) { return __fmaf_rn(vh, dt, x); }

__device__ __forceinline__ float4 predict_xm(float4 xm, float4 v, float4 a, float h, float dt) {
    return make_float4(drift(xm.x, kick(v.x, a.x, h), dt), drift(xm.y, kick(v.y, a.y, h), dt),
                       drift(xm.z, kick(v.z, a.z, h), dt), xm.w);
}

__device__ __forceinline__ float4 ldg4(const float4 *p) { return __ldg(p); }

// ------------------------------------------------ analytic external potential
// The analytic galaxy potential that grav_analytic
// (core/living_galaxy_engine.py:124-151), add_analytic
// (core/gas_disk_engine.py:54-81) and add_grav_ext (:20-51) add after
// self-gravity, in FP32 with G folded into the masses: a Miyamoto-Nagai disk
// (gmd, a, b), a Hernquist (hernquist = 1) or Plummer halo (gmh, ah) and a
// softened central point mass (gmbh, when smbh = 1).
struct ExtPot {
    float gmd, a, b, gmh, ah, gmbh;
    int hernquist, smbh, on;
};

// Host: checks *pot (NULL gives on = 0) and folds G into the masses.
int make_extpot(const gb_potential_t *pot, float G, ExtPot *out);

// Adds the potential's acceleration at (x, y, z) to (ax, ay, az).  Same terms
// and guards as the reference: r clamped to 1e-6 in the Hernquist term,
// r + 1e-6 in the point-mass term.
__device__ __forceinline__ void ext_acc_add(const ExtPot &p, float x, float y, float z, float &ax, float &ay,
                                            float &az) {
    const float R2 = x * x + y * y;
    const float S = sqrtf(z * z + p.b * p.b);
    const float aS = p.a + S;
    const float invD = rsqrtf(R2 + aS * aS);
    const float cd = -p.gmd * (invD * invD * invD);
    float ex = cd * x, ey = cd * y, ez = cd * z * aS / S;
    const float r = sqrtf(R2 + z * z);
    float ch;
    if (p.hernquist) {
        const float rs = fmaxf(r, 1e-6f);
        const float q = rs + p.ah;
        ch = -p.gmh / (q * q * rs);
    } else {
        const float invH = rsqrtf(R2 + z * z + p.ah * p.ah);
        ch = -p.gmh * (invH * invH * invH);
    }
    ex += ch * x;
    ey += ch * y;
    ez += ch * z;
    if (p.smbh) {
        const float rs = r + 1e-6f;
        const float cb = -p.gmbh / (rs * rs * rs);
        ex += cb * x;
        ey += cb * y;
        ez += cb * z;
    }
    ax += ex;
    ay += ey;
    az += ez;
}

}  // namespace gb
