// k_probe.cu -- FP64 and FP32 peak probes (register-only DMMA / DFMA / FFMA loops) used to state
// the FP64 and FP32 rooflines of this GPU, which the HBM/BF16 peak table does not cover.
#include "qk_internal.cuh"

namespace {

constexpr int PROBE_ITERS = 4096;

__global__ void k_probe_dmma(double* out) {
  double d[8][2];
  double a = 1.0 + 1e-9 * threadIdx.x, b = 1.0 - 1e-9 * threadIdx.x;
#pragma unroll
  for (int i = 0; i < 8; ++i) d[i][0] = d[i][1] = 0.0;
  for (int it = 0; it < PROBE_ITERS; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(d[i][0]), "+d"(d[i][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += d[i][0] + d[i][1];
  if (s == 12345.678) out[0] = s;  // keep the work alive
}

__global__ void k_probe_dfma(double* out) {
  double x[8];
  const double a = 1.0 + 1e-12 * threadIdx.x, b = 1e-12;
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = i;
  for (int it = 0; it < PROBE_ITERS; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) s += x[i];
  if (s == 12345.678) out[0] = s;
}

__global__ void k_probe_ffma(float* out) {
  float x[16];
  const float a = 1.0f + 1e-7f * threadIdx.x, b = 1e-7f;
#pragma unroll
  for (int i = 0; i < 16; ++i) x[i] = (float)i;
  for (int it = 0; it < PROBE_ITERS; ++it) {
#pragma unroll
    for (int i = 0; i < 16; ++i) x[i] = fmaf(x[i], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 16; ++i) s += x[i];
  if (s == 12345.678f) out[0] = s;
}

}  // namespace

extern "C" {

void* qk_stream(const qk_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int qk_probe_fp64_peak(qk_ctx* ctx, double* tflops_dmma, double* tflops_dfma) {
  if (!ctx) return QK_ERR_ARG;
  cudaSetDevice(ctx->device);
  double* dummy = nullptr;
  QK_TRY(qk_wst(ctx, W_MISC, 16, &dummy));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = ctx->num_sms * 8, threads = 256;
  float ms = 0.f;
  // DMMA: 8 MMAs of 8x8x4 (256 FMA = 512 flop) per warp per iteration
  k_probe_dmma<<<blocks, threads, 0, ctx->stream>>>(dummy);
  cudaEventRecord(e0, ctx->stream);
  k_probe_dmma<<<blocks, threads, 0, ctx->stream>>>(dummy);
  cudaEventRecord(e1, ctx->stream);
  QK_CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1);
  const double warps = (double)blocks * threads / 32.0;
  if (tflops_dmma) *tflops_dmma = warps * PROBE_ITERS * 8 * 512.0 / (ms * 1e-3) / 1e12;
  k_probe_dfma<<<blocks, threads, 0, ctx->stream>>>(dummy);
  cudaEventRecord(e0, ctx->stream);
  k_probe_dfma<<<blocks, threads, 0, ctx->stream>>>(dummy);
  cudaEventRecord(e1, ctx->stream);
  QK_CK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(&ms, e0, e1);
  if (tflops_dfma) *tflops_dfma = (double)blocks * threads * PROBE_ITERS * 8 * 2.0 / (ms * 1e-3) / 1e12;
  ctx->launches += 4;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return QK_OK;
}

int qk_probe_fp32_peak(qk_ctx* ctx, double* tflops_ffma) {
  if (!ctx || !tflops_ffma) return QK_ERR_ARG;
  cudaSetDevice(ctx->device);
  double* dummy = nullptr;
  QK_TRY(qk_wst(ctx, W_MISC, 16, &dummy));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = ctx->num_sms * 8, threads = 256;
  float ms = 0.f;
  k_probe_ffma<<<blocks, threads, 0, ctx->stream>>>((float*)dummy);
  cudaEventRecord(e0, ctx->stream);
  k_probe_ffma<<<blocks, threads, 0, ctx->stream>>>((float*)dummy);
  cudaEventRecord(e1, ctx->stream);
  const cudaError_t st = cudaEventSynchronize(e1);
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  QK_CK(st);
  *tflops_ffma = (double)blocks * threads * PROBE_ITERS * 16 * 2.0 / (ms * 1e-3) / 1e12;
  ctx->launches += 2;
  return QK_OK;
}

}  // extern "C"
