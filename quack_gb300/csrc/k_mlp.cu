// k_mlp.cu -- the learned quasiparticle guess: a 16 -> 64 -> 64 -> 1 SiLU perceptron trained
// and evaluated on the GPU with hand-written kernels.
//
//   forward   Z1 = X W1^T + b1, A1 = silu(Z1), Z2 = A1 W2^T + b2, A2 = silu(Z2), Y = A2 W3^T + b3
//   loss      mean squared error against the QP shift targets
//   backward  the chain rule layer by layer (small FP32 GEMMs), then Adam (FP32)
//   inference BF16 weights and inputs, FP32 accumulation
// Parameters are one flat FP32 vector [W1 (64x16) | b1 | W2 (64x64) | b2 | W3 (1x64) | b3],
// row-major weight matrices (row = output unit).  Per-orbital features (16 per orbital) are
// built from the quantities of the linearised G0W0 stage (k_features).
#include <cuda_bf16.h>
#include <cmath>
#include "qk_internal.cuh"

namespace {

constexpr int NIN = QK_MLP_NIN, NH = QK_MLP_NH;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NH * NIN, OFF_W2 = OFF_B1 + NH,
              OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH,
              NPARAM = OFF_B3 + 1;
static_assert(NPARAM == QK_MLP_NPARAM, "parameter layout");

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

// one thread per sample: forward pass keeping Z1, Z2 (for backward) and Y
__global__ void k_mlp_forward(int B, const float* __restrict__ X, const float* __restrict__ P,
                              float* __restrict__ Z1, float* __restrict__ Z2, float* __restrict__ Y) {
  __shared__ float w[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) w[i] = P[i];
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  float x[NIN], a1[NH];
  for (int k = 0; k < NIN; ++k) x[k] = X[(size_t)b * NIN + k];
  for (int h = 0; h < NH; ++h) {
    float z = w[OFF_B1 + h];
    for (int k = 0; k < NIN; ++k) z = fmaf(w[OFF_W1 + h * NIN + k], x[k], z);
    if (Z1) Z1[(size_t)b * NH + h] = z;
    a1[h] = silu(z);
  }
  float y = w[OFF_B3];
  for (int h = 0; h < NH; ++h) {
    float z = w[OFF_B2 + h];
    for (int k = 0; k < NH; ++k) z = fmaf(w[OFF_W2 + h * NH + k], a1[k], z);
    if (Z2) Z2[(size_t)b * NH + h] = z;
    y = fmaf(w[OFF_W3 + h], silu(z), y);
  }
  Y[b] = y;
}

// per-sample backward: dY, dZ2, dZ1 (B x 64 each) from the saved pre-activations
__global__ void k_mlp_backward_deltas(int B, const float* __restrict__ P, const float* __restrict__ Z1,
                                      const float* __restrict__ Z2, const float* __restrict__ Y,
                                      const float* __restrict__ T, float* __restrict__ dY,
                                      float* __restrict__ D2, float* __restrict__ D1) {
  __shared__ float w[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) w[i] = P[i];
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const float dy = 2.0f * (Y[b] - T[b]) / (float)B;
  dY[b] = dy;
  float d2[NH];
  for (int h = 0; h < NH; ++h) {
    d2[h] = dy * w[OFF_W3 + h] * dsilu(Z2[(size_t)b * NH + h]);
    D2[(size_t)b * NH + h] = d2[h];
  }
  for (int k = 0; k < NH; ++k) {
    float s = 0.0f;
    for (int h = 0; h < NH; ++h) s = fmaf(d2[h], w[OFF_W2 + h * NH + k], s);
    D1[(size_t)b * NH + k] = s * dsilu(Z1[(size_t)b * NH + k]);
  }
}

// parameter gradients: one thread per parameter, reduction over the batch
//   dW1[h,k] = sum_b D1[b,h] X[b,k]      db1[h] = sum_b D1[b,h]
//   dW2[h,k] = sum_b D2[b,h] A1[b,k]     db2[h] = sum_b D2[b,h]
//   dW3[h]   = sum_b dY[b] A2[b,h]       db3    = sum_b dY[b]
__global__ void k_mlp_param_grads(int B, const float* __restrict__ X, const float* __restrict__ Z1,
                                  const float* __restrict__ Z2, const float* __restrict__ dY,
                                  const float* __restrict__ D2, const float* __restrict__ D1,
                                  float* __restrict__ G) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  float s = 0.0f;
  if (i < OFF_B1) {
    const int h = i / NIN, k = i % NIN;
    for (int b = 0; b < B; ++b) s = fmaf(D1[(size_t)b * NH + h], X[(size_t)b * NIN + k], s);
  } else if (i < OFF_W2) {
    const int h = i - OFF_B1;
    for (int b = 0; b < B; ++b) s += D1[(size_t)b * NH + h];
  } else if (i < OFF_B2) {
    const int h = (i - OFF_W2) / NH, k = (i - OFF_W2) % NH;
    for (int b = 0; b < B; ++b) s = fmaf(D2[(size_t)b * NH + h], silu(Z1[(size_t)b * NH + k]), s);
  } else if (i < OFF_W3) {
    const int h = i - OFF_B2;
    for (int b = 0; b < B; ++b) s += D2[(size_t)b * NH + h];
  } else if (i < OFF_B3) {
    const int h = i - OFF_W3;
    for (int b = 0; b < B; ++b) s = fmaf(dY[b], silu(Z2[(size_t)b * NH + h]), s);
  } else {
    for (int b = 0; b < B; ++b) s += dY[b];
  }
  G[i] = s;
}

__global__ void k_adam(int n, float* __restrict__ P, const float* __restrict__ G,
                       float* __restrict__ M, float* __restrict__ V, float lr, float b1, float b2,
                       float eps, int t) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = G[i];
  const float m = b1 * M[i] + (1.0f - b1) * g;
  const float v = b2 * V[i] + (1.0f - b2) * g * g;
  M[i] = m;
  V[i] = v;
  const float mh = m / (1.0f - powf(b1, (float)t));
  const float vh = v / (1.0f - powf(b2, (float)t));
  P[i] -= lr * mh / (sqrtf(vh) + eps);
}

__global__ void k_mse(int B, const float* __restrict__ Y, const float* __restrict__ T,
                      float* __restrict__ out) {
  __shared__ float red[32];
  float s = 0.0f;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    const float d = Y[b] - T[b];
    s += d * d;
  }
  s = qk_block_sum(s, red);
  if (threadIdx.x == 0) *out = s / (float)(B > 0 ? B : 1);
}

// BF16 inference: weights and inputs rounded to BF16, FP32 accumulation
__global__ void k_mlp_infer_bf16(int B, const float* __restrict__ X, const float* __restrict__ P,
                                 float* __restrict__ Y) {
  __shared__ __nv_bfloat16 w[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) w[i] = __float2bfloat16(P[i]);
  __syncthreads();
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  float x[NIN], a1[NH];
  for (int k = 0; k < NIN; ++k) x[k] = __bfloat162float(__float2bfloat16(X[(size_t)b * NIN + k]));
  for (int h = 0; h < NH; ++h) {
    float z = __bfloat162float(w[OFF_B1 + h]);
    for (int k = 0; k < NIN; ++k) z = fmaf(__bfloat162float(w[OFF_W1 + h * NIN + k]), x[k], z);
    a1[h] = __bfloat162float(__float2bfloat16(silu(z)));
  }
  float y = __bfloat162float(w[OFF_B3]);
  for (int h = 0; h < NH; ++h) {
    float z = __bfloat162float(w[OFF_B2 + h]);
    for (int k = 0; k < NH; ++k) z = fmaf(__bfloat162float(w[OFF_W2 + h * NH + k]), a1[k], z);
    y = fmaf(__bfloat162float(w[OFF_W3 + h]), silu(z), y);
  }
  Y[b] = y;
}

// deterministic initialisation (uniform +-sqrt(6/(fan_in+fan_out)) weights, zero biases)
__global__ void k_mlp_init(float* __restrict__ P, unsigned long long seed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NPARAM) return;
  unsigned long long z = (i + 1) * 0x9E3779B97F4A7C15ull ^ seed;
  z ^= z >> 30; z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27; z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  const float u = (float)((z >> 40) * (1.0 / 16777216.0)) * 2.0f - 1.0f;
  float lim = 0.0f;
  if (i < OFF_B1) lim = sqrtf(6.0f / (NIN + NH));
  else if (i >= OFF_W2 && i < OFF_B2) lim = sqrtf(6.0f / (NH + NH));
  else if (i >= OFF_W3 && i < OFF_B3) lim = sqrtf(6.0f / (NH + 1));
  P[i] = lim * u;
}

// x_norm = (F - mean) / std for n orbitals
__global__ void k_normalise(int n, const float* __restrict__ F, const float* __restrict__ mean,
                            const float* __restrict__ stdv, float* __restrict__ X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * NIN) return;
  const int k = i % NIN;
  X[i] = (F[i] - mean[k]) / stdv[k];
}

// w0 = e + (y * ystd + ymean)
// The network predicts the nonlinear correction y = eGW - eGWlin.  The Halley step h of the QP
// equation from eGWlin (FP64, from the feature sweep) is exact to far below the network's
// resolution where the search is regular; where the two agree to QK_GUESS_AGREE the search starts
// at eGWlin + h, elsewhere it starts at the reference start and follows the reference trajectory.
// Gate 1 (the context setting "guess_gate" = 1) starts every search at eGWlin + y instead, and
// gate 2 at eGWlin + h wherever h exists; the root certificate keeps the results either way.
constexpr double QK_GUESS_AGREE = 3e-3;  // Ha
__global__ void k_guess(int n, const float* __restrict__ Y, float ymean, float ystd,
                        const double* __restrict__ base, const double* __restrict__ hal,
                        double* __restrict__ w0, int* __restrict__ fromref, int gate) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double y = (double)(Y[i] * ystd + ymean);
  const double h = hal[i];
  bool use = (h == h) && fabs(y - h) <= QK_GUESS_AGREE;
  double start = base[i] + h;
  if (gate == 1) {
    use = y == y;
    start = base[i] + y;
  } else if (gate == 2) {
    use = h == h;
  }
  w0[i] = use ? start : base[i];
  fromref[i] = use ? 0 : 1;
}

}  // namespace

// ---------------------------------------------------------------------------------------------
struct qk_mlp {
  float* P = nullptr;   // parameters
  float* M = nullptr;   // Adam first moment
  float* V = nullptr;   // Adam second moment
  float* G = nullptr;   // gradient
  int t = 0;            // Adam step
  float* work = nullptr;
  size_t work_n = 0;
  float xmean[QK_MLP_NIN], xstd[QK_MLP_NIN];  // feature normalisation (host copy)
  float ymean = 0.f, ystd = 1.f;
};

static int mlp_work(qk_ctx* ctx, qk_mlp* m, int B) {
  const size_t need = (size_t)B * (2 * NH + 2 * NH + 2) + 16;  // Z1 Z2 D1 D2 Y dY
  if (m->work_n < need) {
    if (m->work) cudaFree(m->work);
    m->work = nullptr;
    QK_CK(cudaMalloc(&m->work, need * sizeof(float)));
    m->work_n = need;
  }
  return QK_OK;
}

int qk_guess_from_model(qk_ctx* ctx, int N, const float* F, const double* base, const double* hal,
                        double* w0, int* fromref) {
  qk_mlp* m = ctx->mlp;
  if (!m) return qk_fail(ctx, QK_ERR_ARG, "qp_guess requested but no model attached");
  float* buf = nullptr;
  QK_TRY(qk_wst(ctx, W_MLPIO, (size_t)N * (NIN + 1) + 2 * NIN + 16, &buf));
  float* X = buf;
  float* Y = X + (size_t)N * NIN;
  float* ms = Y + N;
  QK_CK(cudaMemcpyAsync(ms, m->xmean, NIN * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  QK_CK(cudaMemcpyAsync(ms + NIN, m->xstd, NIN * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  k_normalise<<<(N * NIN + 255) / 256, 256, 0, ctx->stream>>>(N, F, ms, ms + NIN, X);
  QK_LAUNCHED();
  k_mlp_infer_bf16<<<(N + 127) / 128, 128, 0, ctx->stream>>>(N, X, m->P, Y);
  QK_LAUNCHED();
  k_guess<<<(N + 127) / 128, 128, 0, ctx->stream>>>(N, Y, m->ymean, m->ystd, base, hal, w0,
                                                   fromref,
                                                   ctx->guess_gate);
  QK_LAUNCHED();
  return QK_OK;
}

extern "C" {

int qk_set_qp_model(qk_ctx* ctx, qk_mlp* mlp) {
  if (!ctx) return QK_ERR_ARG;
  ctx->mlp = mlp;
  return QK_OK;
}

int qk_set_feature_capture(qk_ctx* ctx, int on) {
  if (!ctx) return QK_ERR_ARG;
  ctx->capture_features = on != 0;
  return QK_OK;
}

int qk_get_features(const qk_ctx* ctx, float* host, int n) {
  if (!ctx || !host) return QK_ERR_ARG;
  const int m = (int)ctx->features.size();
  for (int i = 0; i < n; ++i) host[i] = i < m ? ctx->features[i] : 0.f;
  return QK_OK;
}

int qk_mlp_create(qk_ctx* ctx, unsigned long long seed, qk_mlp** out) {
  if (!ctx || !out) return QK_ERR_ARG;
  cudaSetDevice(ctx->device);
  qk_mlp* m = new qk_mlp();
  if (cudaMalloc(&m->P, 4 * NPARAM * sizeof(float)) != cudaSuccess) {
    delete m;
    return QK_ERR_NOMEM;
  }
  m->M = m->P + NPARAM;
  m->V = m->M + NPARAM;
  m->G = m->V + NPARAM;
  cudaMemsetAsync(m->M, 0, 3 * NPARAM * sizeof(float), ctx->stream);
  k_mlp_init<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(m->P, seed);
  ctx->launches++;
  for (int k = 0; k < NIN; ++k) { m->xmean[k] = 0.f; m->xstd[k] = 1.f; }
  if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) { delete m; return QK_ERR_CUDA; }
  *out = m;
  return QK_OK;
}

int qk_mlp_free(qk_mlp* m) {
  if (!m) return QK_OK;
  if (m->P) cudaFree(m->P);
  if (m->work) cudaFree(m->work);
  delete m;
  return QK_OK;
}

int qk_mlp_params(qk_ctx* ctx, qk_mlp* m, float* host, int set) {
  if (!ctx || !m || !host) return QK_ERR_ARG;
  if (set) QK_CK(cudaMemcpyAsync(m->P, host, NPARAM * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  else QK_CK(cudaMemcpyAsync(host, m->P, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  return QK_OK;
}

int qk_mlp_set_scaling(qk_mlp* m, const float* xmean, const float* xstd, float ymean, float ystd) {
  if (!m || !xmean || !xstd || !(ystd > 0.f)) return QK_ERR_ARG;
  for (int k = 0; k < NIN; ++k) {
    m->xmean[k] = xmean[k];
    m->xstd[k] = xstd[k] > 0.f ? xstd[k] : 1.f;
  }
  m->ymean = ymean;
  m->ystd = ystd;
  return QK_OK;
}

// gradient of the mean squared error over (X, T) (normalised inputs/targets), device buffers
int qk_mlp_grad_dev(qk_ctx* ctx, qk_mlp* m, int B, const float* d_X, const float* d_T,
                    float* d_grad, float* loss) {
  if (!ctx || !m || B <= 0) return QK_ERR_ARG;
  QK_TRY(qk_order_after_default(ctx));
  QK_TRY(mlp_work(ctx, m, B));
  float* Z1 = m->work;
  float* Z2 = Z1 + (size_t)B * NH;
  float* D1 = Z2 + (size_t)B * NH;
  float* D2 = D1 + (size_t)B * NH;
  float* Y = D2 + (size_t)B * NH;
  float* dY = Y + B;
  float* L = dY + B;
  const int tb = 128, nb = (B + tb - 1) / tb;
  k_mlp_forward<<<nb, tb, 0, ctx->stream>>>(B, d_X, m->P, Z1, Z2, Y);
  QK_LAUNCHED();
  k_mlp_backward_deltas<<<nb, tb, 0, ctx->stream>>>(B, m->P, Z1, Z2, Y, d_T, dY, D2, D1);
  QK_LAUNCHED();
  k_mlp_param_grads<<<(NPARAM + 127) / 128, 128, 0, ctx->stream>>>(B, d_X, Z1, Z2, dY, D2, D1,
                                                                   d_grad ? d_grad : m->G);
  QK_LAUNCHED();
  if (loss) {
    k_mse<<<1, 256, 0, ctx->stream>>>(B, Y, d_T, L);
    QK_LAUNCHED();
    QK_CK(cudaMemcpyAsync(loss, L, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  }
  QK_CK(cudaStreamSynchronize(ctx->stream));
  return QK_OK;
}

// Adam training on (X, T) (normalised), mini-batches taken in order with a fixed rotation
int qk_mlp_train_dev(qk_ctx* ctx, qk_mlp* m, int n, const float* d_X, const float* d_T, int epochs,
                     int batch, float lr, float* final_loss) {
  if (!ctx || !m || n <= 0 || batch <= 0 || epochs < 0) return QK_ERR_ARG;
  QK_TRY(qk_order_after_default(ctx));
  if (batch > n) batch = n;
  QK_TRY(mlp_work(ctx, m, batch));
  float* Z1 = m->work;
  float* Z2 = Z1 + (size_t)batch * NH;
  float* D1 = Z2 + (size_t)batch * NH;
  float* D2 = D1 + (size_t)batch * NH;
  float* Y = D2 + (size_t)batch * NH;
  float* dY = Y + batch;
  const int tb = 128, nb = (batch + tb - 1) / tb;
  const int steps_per_epoch = n / batch;
  for (int ep = 0; ep < epochs; ++ep) {
    for (int s = 0; s < steps_per_epoch; ++s) {
      const int off = ((s + ep * 7) % steps_per_epoch) * batch;
      const float* X = d_X + (size_t)off * NIN;
      const float* T = d_T + off;
      k_mlp_forward<<<nb, tb, 0, ctx->stream>>>(batch, X, m->P, Z1, Z2, Y);
      k_mlp_backward_deltas<<<nb, tb, 0, ctx->stream>>>(batch, m->P, Z1, Z2, Y, T, dY, D2, D1);
      k_mlp_param_grads<<<(NPARAM + 127) / 128, 128, 0, ctx->stream>>>(batch, X, Z1, Z2, dY, D2, D1,
                                                                       m->G);
      m->t++;
      k_adam<<<(NPARAM + 255) / 256, 256, 0, ctx->stream>>>(NPARAM, m->P, m->G, m->M, m->V, lr,
                                                            0.9f, 0.999f, 1e-8f, m->t);
      ctx->launches += 4;
    }
    QK_CK(cudaGetLastError());
  }
  if (final_loss) {
    float* Yall = nullptr;
    QK_CK(cudaMalloc(&Yall, ((size_t)n + 1) * sizeof(float)));
    k_mlp_forward<<<(n + 127) / 128, 128, 0, ctx->stream>>>(n, d_X, m->P, nullptr, nullptr, Yall);
    k_mse<<<1, 256, 0, ctx->stream>>>(n, Yall, d_T, Yall + n);
    ctx->launches += 2;
    QK_CK(cudaMemcpyAsync(final_loss, Yall + n, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    QK_CK(cudaStreamSynchronize(ctx->stream));
    cudaFree(Yall);
  }
  QK_CK(cudaStreamSynchronize(ctx->stream));
  return QK_OK;
}

// predictions for n samples (normalised inputs) in FP32 or BF16
int qk_mlp_predict_dev(qk_ctx* ctx, qk_mlp* m, int n, const float* d_X, float* d_Y, int bf16) {
  if (!ctx || !m || n < 0) return QK_ERR_ARG;
  QK_TRY(qk_order_after_default(ctx));
  if (n == 0) return QK_OK;
  if (bf16)
    k_mlp_infer_bf16<<<(n + 127) / 128, 128, 0, ctx->stream>>>(n, d_X, m->P, d_Y);
  else
    k_mlp_forward<<<(n + 127) / 128, 128, 0, ctx->stream>>>(n, d_X, m->P, nullptr, nullptr, d_Y);
  QK_LAUNCHED();
  QK_CK(cudaStreamSynchronize(ctx->stream));
  return QK_OK;
}

}  // extern "C"
