// FP32 CUDA-core throughput calibration: the measured denominator for the
// direct-sum roofline (the reported peak is FP32 FLOP/s, FMA = 2 FLOP).
// Each thread runs 8 independent FMA chains (scalar) or 4 packed .f32x2
// chains, long enough that launch overhead is negligible.
#include "gb_common.cuh"

namespace gb {

__global__ void calib_ffma_kernel(float *out, int iters, float a, float b) {
    float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1e-7f, x2 = x0 + 2e-7f, x3 = x0 + 3e-7f;
    float x4 = x0 + 4e-7f, x5 = x0 + 5e-7f, x6 = x0 + 6e-7f, x7 = x0 + 7e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            x0 = __fmaf_rn(x0, a, b); x1 = __fmaf_rn(x1, a, b);
            x2 = __fmaf_rn(x2, a, b); x3 = __fmaf_rn(x3, a, b);
            x4 = __fmaf_rn(x4, a, b); x5 = __fmaf_rn(x5, a, b);
            x6 = __fmaf_rn(x6, a, b); x7 = __fmaf_rn(x7, a, b);
        }
    }
    const float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live
}

__global__ void calib_ffma2_kernel(float *out, int iters, float a, float b) {
    const float t = threadIdx.x * 1e-7f;
    f2 x0 = pack2(t, t + 1e-7f), x1 = pack2(t + 2e-7f, t + 3e-7f);
    f2 x2 = pack2(t + 4e-7f, t + 5e-7f), x3 = pack2(t + 6e-7f, t + 7e-7f);
    const f2 A = pack2(a, a), B = pack2(b, b);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int r = 0; r < 16; ++r) {
            x0 = fma2(x0, A, B); x1 = fma2(x1, A, B);
            x2 = fma2(x2, A, B); x3 = fma2(x3, A, B);
        }
    }
    float p, q, r, s, u, v, w, z;
    unpack2(x0, p, q); unpack2(x1, r, s); unpack2(x2, u, v); unpack2(x3, w, z);
    const float tot = p + q + r + s + u + v + w + z;
    if (tot == 12345.678f) out[blockIdx.x] = tot;
}

}  // namespace gb

// Runs the calibration kernel on `stream` and returns the FP32 FLOP count of
// one launch in *flops (the caller times the launch with events).
extern "C" int gb_calib_fp32(float *scratch, int iters, int packed, double *flops, void *stream) {
    if (!scratch || !flops || iters <= 0) return gb::fail(GB_EINVAL, "bad calibration arguments");
    const int sms = gb::num_sms();
    const int blocks = sms * 8, threads = 256;
    cudaStream_t s = (cudaStream_t)stream;
    if (packed) gb::calib_ffma2_kernel<<<blocks, threads, 0, s>>>(scratch, iters, 0.9999f, 1e-6f);
    else gb::calib_ffma_kernel<<<blocks, threads, 0, s>>>(scratch, iters, 0.9999f, 1e-6f);
    GB_CUDA_TRY(cudaGetLastError());
    *flops = 2.0 * 8.0 * 16.0 * (double)iters * blocks * threads;
    return GB_OK;
}
