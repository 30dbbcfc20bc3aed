// qk_ctx.cu -- context lifetime, workspace, error strings, stage timers.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <nvtx3/nvToolsExt.h>
#include "qk_internal.cuh"

static const char* k_timing_names[T_NUM] = {"casida_build", "tridiag", "bisect",  "stein",
                                            "back_transform", "slab",    "rho",     "sigma",
                                            "qp",             "casida2", "misc"};

int qk_fail(qk_ctx* ctx, int code, const char* fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return code;
}

int qk_cuda_fail(qk_ctx* ctx, cudaError_t e, const char* what, const char* file, int line) {
  int code = (e == cudaErrorMemoryAllocation) ? QK_ERR_NOMEM : QK_ERR_CUDA;
  return qk_fail(ctx, code, "%s failed at %s:%d: %s", what, file, line, cudaGetErrorString(e));
}

int qk_ws(qk_ctx* ctx, int slot, size_t bytes, void** out) {
  DevBuf& b = ctx->buf[slot];
  if (bytes == 0) bytes = 16;
  if (b.bytes < bytes) {
    // failure-path hook: the armed n-th growing allocation fails as cudaMalloc would
    if (ctx->fail_alloc_in > 0 && --ctx->fail_alloc_in == 0)
      return qk_fail(ctx, QK_ERR_NOMEM, "cudaMalloc(workspace) failed (simulated by the "
                                        "fail_alloc hook)");
    if (b.p) {
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) return qk_cuda_fail(ctx, e, "cudaStreamSynchronize", __FILE__, __LINE__);
      cudaFree(b.p);
      b.p = nullptr;
      b.bytes = 0;
    }
    size_t want = (bytes + 255) & ~(size_t)255;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
      b.p = nullptr;
      return qk_cuda_fail(ctx, e, "cudaMalloc(workspace)", __FILE__, __LINE__);
    }
    b.bytes = want;
  }
  *out = b.p;
  return QK_OK;
}

int qk_status_reset(qk_ctx* ctx) {
  QK_CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->stream));
  return QK_OK;
}

int qk_status_check(qk_ctx* ctx, int fatal_mask) {
  int h = 0;
  QK_CK(cudaMemcpyAsync(&h, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  ctx->last_dev_status = h;
  if (h & fatal_mask)
    return qk_fail(ctx, QK_ERR_DEVICE, "device-side check failed (status bits 0x%x)", h);
  return QK_OK;
}

int qk_order_after_default(qk_ctx* ctx) {
  QK_CK(cudaEventRecord(ctx->ev_in, cudaStreamLegacy));
  QK_CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_in, 0));
  return QK_OK;
}

// Each stage is also an NVTX range (host-side span of the enqueueing, named like the timer), so
// that a profiler timeline shows the library's stages; start/end pairs by id, not a stack, so
// nested stages (the eigensolver inside the second Casida) stay well formed.
void qk_tic(qk_ctx* ctx, int stage) {
  ctx->nvtx[stage] = nvtxRangeStartA(k_timing_names[stage]);
  if (ctx->timing && !ctx->capturing) cudaEventRecord(ctx->ev[2 * stage], ctx->stream);
}
void qk_toc(qk_ctx* ctx, int stage) {
  if (ctx->nvtx[stage]) {
    nvtxRangeEnd(ctx->nvtx[stage]);
    ctx->nvtx[stage] = 0;
  }
  if (!ctx->timing || ctx->capturing) return;
  cudaEventRecord(ctx->ev[2 * stage + 1], ctx->stream);
  ctx->timings[stage] = -1.0;  // mark pending
}
void qk_timings_clear(qk_ctx* ctx) {
  for (int i = 0; i < T_NUM; ++i) ctx->timings[i] = 0.0;
}
void qk_timings_collect(qk_ctx* ctx) {
  for (int i = 0; i < T_NUM; ++i) {
    if (ctx->timings[i] < 0.0) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, ctx->ev[2 * i], ctx->ev[2 * i + 1]) == cudaSuccess)
        ctx->timings[i] = ms;
      else
        ctx->timings[i] = 0.0;
    }
  }
}

extern "C" {

int qk_init(int device, qk_ctx** out) {
  if (!out) return QK_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return QK_ERR_NO_DEVICE;
  if (device < 0 || device >= ndev) return QK_ERR_ARG;
  qk_ctx* ctx = new qk_ctx();
  ctx->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) { delete ctx; return QK_ERR_CUDA; }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, device);
  if (prop.major < 10) { delete ctx; return QK_ERR_NO_DEVICE; }
  ctx->num_sms = prop.multiProcessorCount;
  if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return QK_ERR_CUDA;
  }
  for (auto& ev : ctx->ev) cudaEventCreate(&ev);
  cudaEventCreateWithFlags(&ctx->ev_in, cudaEventDisableTiming);
  if (cudaMalloc(&ctx->d_status, 256) != cudaSuccess ||
      cudaMalloc(&ctx->d_bar, 256 * sizeof(unsigned)) != cudaSuccess) {
    qk_finalize(ctx);
    return QK_ERR_NOMEM;
  }
  cudaMemset(ctx->d_status, 0, 256);
  cudaMemset(ctx->d_bar, 0, 256 * sizeof(unsigned));
  cudaDeviceSynchronize();
  *out = ctx;
  return QK_OK;
}

int qk_finalize(qk_ctx* ctx) {
  if (!ctx) return QK_OK;
  for (auto* w : ctx->workers) qk_finalize(w);
  ctx->workers.clear();
  if (ctx->evgw_exec) cudaGraphExecDestroy(ctx->evgw_exec);
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& b : ctx->buf)
    if (b.p) cudaFree(b.p);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->d_bar) cudaFree(ctx->d_bar);
  for (auto& ev : ctx->ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->ev_in) cudaEventDestroy(ctx->ev_in);
  if (ctx->ev_tri) cudaEventDestroy(ctx->ev_tri);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  if (ctx->ev_copy) cudaEventDestroy(ctx->ev_copy);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return QK_OK;
}

int qk_trim(qk_ctx* ctx) {
  if (!ctx) return QK_ERR_ARG;
  cudaStreamSynchronize(ctx->stream);
  for (auto& b : ctx->buf) {
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
  }
  return QK_OK;
}

const char* qk_last_error_string(const qk_ctx* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

int qk_get_timings(const qk_ctx* ctx, double* ms, int n) {
  if (!ctx || !ms) return QK_ERR_ARG;
  for (int i = 0; i < n && i < T_NUM; ++i) ms[i] = ctx->timings[i];
  return QK_OK;
}

int qk_last_device_status(const qk_ctx* ctx) { return ctx ? ctx->last_dev_status : 0; }
int qk_batch_group_stats(const qk_ctx* ctx, long long* launches, long long* matrices) {
  if (!ctx) return QK_ERR_ARG;
  if (launches) *launches = ctx->tri_groups;
  if (matrices) *matrices = ctx->tri_grouped;
  return QK_OK;
}
const char* qk_timing_name(int i) { return (i >= 0 && i < T_NUM) ? k_timing_names[i] : ""; }
int qk_num_timings(void) { return T_NUM; }
long long qk_launch_count(const qk_ctx* ctx) { return ctx ? ctx->launches : 0; }

long long qk_qp_evals(const qk_ctx* ctx) { return ctx ? ctx->qp_evals : 0; }

int qk_set_graph_mode(qk_ctx* ctx, int on) {
  if (!ctx) return QK_ERR_ARG;
  ctx->graph_mode = on != 0;
  return QK_OK;
}

int qk_get_qp_iters(const qk_ctx* ctx, int* iters, int n) {
  if (!ctx || !iters) return QK_ERR_ARG;
  const int m = (int)ctx->qp_iters.size();
  for (int i = 0; i < n; ++i) iters[i] = i < m ? ctx->qp_iters[i] : 0;
  return QK_OK;
}

}  // extern "C"
