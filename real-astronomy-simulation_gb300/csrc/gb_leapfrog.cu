// Standalone leapfrog kernels: kick and drift of core/integrators/
// leapfrog.py:11-22, for callers that step outside the fused KDK path.  They
// use the same FMA forms as the fused step (kick: fma(a, dt/2, v); drift:
// fma(v, dt, x)), so kick -> drift -> forces -> kick through these calls
// gives the fused gb_direct_kdk step bit for bit.
#include "gb_common.cuh"

namespace gb {

__global__ void kick_kernel(float4 *vel, const float4 *__restrict__ acc, int64_t n, float h) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 v = vel[i];
    const float4 a = __ldg(acc + i);
    v.x = kick(v.x, a.x, h);
    v.y = kick(v.y, a.y, h);
    v.z = kick(v.z, a.z, h);
    vel[i] = v;
}

__global__ void drift_kernel(float4 *xm, const float4 *__restrict__ vel, int64_t n, float dt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 x = xm[i];
    const float4 v = __ldg(vel + i);
    x.x = drift(x.x, v.x, dt);
    x.y = drift(x.y, v.y, dt);
    x.z = drift(x.z, v.z, dt);
    xm[i] = x;
}

static int check_pair(const void *a, const void *b, int64_t n) {
    if (n < 0) return fail(GB_EINVAL, "n < 0");
    if (n > 0 && (!a || !b)) return fail(GB_EINVAL, "NULL buffer");
    if (n > 0 && (!aligned16(a) || !aligned16(b))) return fail(GB_EINVAL, "buffers must be 16-byte aligned");
    return GB_OK;
}

}  // namespace gb

using namespace gb;

extern "C" int gb_kick(float *vel, const float *acc, int64_t n, float dt_half, void *stream) {
    GB_TRY(check_pair(vel, acc, n));
    if (n == 0) return GB_OK;
    kick_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>((float4 *)vel, (const float4 *)acc,
                                                                              n, dt_half);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}

extern "C" int gb_drift(float *xm, const float *vel, int64_t n, float dt, void *stream) {
    GB_TRY(check_pair(xm, vel, n));
    if (n == 0) return GB_OK;
    drift_kernel<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>((float4 *)xm, (const float4 *)vel, n,
                                                                               dt);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}
