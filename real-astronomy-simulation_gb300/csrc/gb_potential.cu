// Standalone analytic galaxy potential: grav_analytic
// (core/living_galaxy_engine.py:124-151) and add_analytic
// (core/gas_disk_engine.py:54-81) as one elementwise pass, for callers whose
// self-gravity comes from elsewhere.  The direct and tree paths add the same
// terms in their own result-writing pass (gb_direct_acc_ext,
// gb_bh_accel_ext).
#include "gb_common.cuh"

namespace gb {

__global__ void analytic_acc_kernel(const float4 *__restrict__ xm, float4 *acc, int64_t n, ExtPot pot,
                                    int accumulate) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 x = __ldg(xm + i);
    float ax = 0.f, ay = 0.f, az = 0.f;
    ext_acc_add(pot, x.x, x.y, x.z, ax, ay, az);
    if (accumulate) {
        float4 o = acc[i];
        o.x += ax;
        o.y += ay;
        o.z += az;
        acc[i] = o;
    } else {
        acc[i] = make_float4(ax, ay, az, 0.f);
    }
}

}  // namespace gb

using namespace gb;

extern "C" int gb_analytic_acc(const float *xm, float *acc, int64_t n, float G, const gb_potential_t *pot,
                               int flags, void *stream) {
    if (!pot) return fail(GB_EINVAL, "pot is NULL");
    ExtPot ep;
    GB_TRY(make_extpot(pot, G, &ep));
    if (n < 0) return fail(GB_EINVAL, "n < 0");
    if (n == 0) return GB_OK;
    if (!xm || !acc) return fail(GB_EINVAL, "xm and acc must not be NULL");
    if (!aligned16(xm) || !aligned16(acc)) return fail(GB_EINVAL, "xm and acc must be 16-byte aligned");
    const unsigned block = 256, grid = (unsigned)((n + block - 1) / block);
    analytic_acc_kernel<<<grid, block, 0, (cudaStream_t)stream>>>((const float4 *)xm, (float4 *)acc, n, ep,
                                                                   (flags & GB_ACCUMULATE) ? 1 : 0);
    GB_CUDA_TRY(cudaGetLastError());
    return GB_OK;
}
