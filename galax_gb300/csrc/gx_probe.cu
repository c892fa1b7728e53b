// gx_probe.cu -- measures this GPU's FP32 FMA throughput, the roofline ceiling of
// the FP32 P2P pass (the measured-peak file of the pool holds only HBM copy and
// bf16 tensor figures).  Every thread runs independent FMA chains; the result is
// written so the compiler keeps the work.
#include "gx_internal.cuh"

namespace {
constexpr int CHAINS = 8;
constexpr int ITERS = 4096;

__global__ void __launch_bounds__(256) k_fma_peak(float *out, float seed) {
    float a[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; c++) a[c] = seed + (float)(threadIdx.x + c);
    const float b = 0.999999f, d = 1e-7f;
    for (int it = 0; it < ITERS; it++) {
#pragma unroll
        for (int c = 0; c < CHAINS; c++) a[c] = fmaf(a[c], b, d);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < CHAINS; c++) s += a[c];
    if (s == 12345.678f) out[blockIdx.x] = s;  // practically never taken
}
}  // namespace

extern "C" int gx_probe_fp32_tflops(gx_ctx *ctx, double *tflops) {
    if (!ctx || !tflops) return GX_ERR_INVALID_ARG;
    GX_TRY(gx_ensure(ctx, ctx->scratch_f, 4096 * sizeof(float)));
    int blocks = ctx->sm_count * 8;
    float *out = dptr<float>(ctx->scratch_f);
    k_fma_peak<<<blocks, 256, 0, ctx->stream>>>(out, 1.0f);  // warm-up
    double best = 0.0;
    for (int r = 0; r < 5; r++) {
        GX_CUDA(ctx, cudaEventRecord(ctx->ev[8], ctx->stream));
        k_fma_peak<<<blocks, 256, 0, ctx->stream>>>(out, 1.0f + r);
        GX_CUDA(ctx, cudaEventRecord(ctx->ev[9], ctx->stream));
        GX_CUDA(ctx, cudaEventSynchronize(ctx->ev[9]));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev[8], ctx->ev[9]);
        double flops = 2.0 * CHAINS * ITERS * (double)blocks * 256.0;
        best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    GX_CUDA(ctx, cudaGetLastError());
    *tflops = best;
    return GX_OK;
}
