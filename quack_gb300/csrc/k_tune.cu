// k_tune.cu -- the library's autotuner.
//
// Tunable launch parameters (all runtime-selectable, looked up per size bucket
// floor(log2(size)) by the kernels' host launchers):
//   bf16x3_chunk  k blocks per TMEM accumulation chunk of the BF16x3 GEMM {1,2,4}   (size = K)
//   splitk_mult   target CTAs per SM below which FP64 GEMMs split K {1,2,4}       (size = K)
//   sigma_chunks  m chunks per p tile of the pole sweeps, in units of SMs {2,4,8}   (size = nS)
//   sytrd_grid    CTAs of the cooperative tridiagonalisation, quarters of the SMs {2,3,4}
//                 (size = n)
//   dgemm_path    FP64 GEMM on DFMA (1) or on the DMMA tensor path (2)           (size = m*n)
//   stebz_k       lanes per eigenvalue of the k-section bisection {2,4,8}        (size = n)
// qk_autotune times every candidate on buffers of the caller's problem sizes (CUDA events on the
// context stream, best of two runs) and records the fastest; qk_tune_save / qk_tune_load keep
// the table as JSON so that a later process starts tuned.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "qk_internal.cuh"

static const char* k_tune_names[TUNE_NUM] = {"bf16x3_chunk", "splitk_mult", "sigma_chunks",
                                             "sytrd_grid", "dgemm_path", "stebz_k",
                                             "qp_persist"};

static int bucket_of(long long size) {
  int b = 0;
  while (size > 1 && b < TUNE_BUCKETS - 1) {
    size >>= 1;
    ++b;
  }
  return b;
}

int qk_tune_get(const qk_ctx* ctx, int param, long long size, int dflt) {
  if (!ctx || param < 0 || param >= TUNE_NUM) return dflt;
  const int v = ctx->tune[param][bucket_of(size)];
  return v > 0 ? v : dflt;
}

namespace {

__global__ void k_fill(long long n, double* x, double scale, unsigned long long seed) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    unsigned long long z = (i + 1) * 0x9E3779B97F4A7C15ull ^ seed;
    z ^= z >> 31;
    z *= 0xBF58476D1CE4E5B9ull;
    z ^= z >> 29;
    x[i] = scale * (((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 0.5);
  }
}

__global__ void k_symmetrise(int n, double* A) {
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < (long long)n * n;
       idx += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(idx % n), c = (int)(idx / n);
    if (r > c) A[idx] = A[c + (long long)n * r];
  }
}

template <class F>
float time_best(qk_ctx* ctx, F&& fn, int reps = 2) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  float best = 1e30f;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(a, ctx->stream);
    const int st = fn();
    cudaEventRecord(b, ctx->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    if (st == QK_OK && ms < best) best = ms;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return best;
}

}  // namespace

extern "C" {

int qk_tune_set(qk_ctx* ctx, const char* name, long long size, int value) {
  if (!ctx || !name) return QK_ERR_ARG;
  // context-wide settings (size ignored)
  if (!strcmp(name, "newton_maxit")) {
    if (value < 1 || value > 4096) return QK_ERR_ARG;
    ctx->newton_maxit = value;
    return QK_OK;
  }
  if (!strcmp(name, "guess_gate")) {
    if (value < 0 || value > 2) return QK_ERR_ARG;
    ctx->guess_gate = value;
    return QK_OK;
  }
  if (!strcmp(name, "fail_alloc")) {
    if (value < 0) return QK_ERR_ARG;
    ctx->fail_alloc_in = value;
    return QK_OK;
  }
  if (!strcmp(name, "dsyev_df")) {
    if (value < 0 || value > 1) return QK_ERR_ARG;
    ctx->dsyev_df = value;
    return QK_OK;
  }
  if (!strcmp(name, "spin_limit")) {
    if (value < 0) return QK_ERR_ARG;
    cudaSetDevice(ctx->device);
    QK_CK(cudaMemcpyAsync(ctx->d_status + 1, &value, sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
    QK_CK(cudaStreamSynchronize(ctx->stream));
    return QK_OK;
  }
  for (int p = 0; p < TUNE_NUM; ++p)
    if (!strcmp(name, k_tune_names[p])) {
      ctx->tune[p][bucket_of(size)] = value;
      return QK_OK;
    }
  return QK_ERR_ARG;
}

int qk_tune_query(const qk_ctx* ctx, const char* name, long long size) {
  if (!ctx || !name) return -1;
  if (!strcmp(name, "newton_maxit")) return ctx->newton_maxit;
  if (!strcmp(name, "dsyev_df")) return ctx->dsyev_df;
  for (int p = 0; p < TUNE_NUM; ++p)
    if (!strcmp(name, k_tune_names[p])) return ctx->tune[p][bucket_of(size)];
  return -1;
}

int qk_autotune(qk_ctx* ctx, int N, int nS, int flags) {
  if (!ctx || N <= 0 || nS <= 0) return QK_ERR_ARG;
  (void)flags;
  cudaSetDevice(ctx->device);
  const long long N2 = (long long)N * N;
  double *A = nullptr, *B = nullptr, *Cm = nullptr;
  const size_t nA = (size_t)N2 * nS, nB = (size_t)nS * nS;
  if (cudaMalloc(&A, nA * sizeof(double)) != cudaSuccess) return QK_ERR_NOMEM;
  if (cudaMalloc(&B, 2 * nB * sizeof(double)) != cudaSuccess) { cudaFree(A); return QK_ERR_NOMEM; }
  if (cudaMalloc(&Cm, nA * sizeof(double)) != cudaSuccess) {
    cudaFree(A);
    cudaFree(B);
    return QK_ERR_NOMEM;
  }
  k_fill<<<1024, 256, 0, ctx->stream>>>((long long)nA, A, 1.0, 1);
  k_fill<<<1024, 256, 0, ctx->stream>>>((long long)nB, B, 1.0, 2);
  ctx->launches += 2;
  int st = QK_OK;
  // 1. BF16x3 chunk (the excitation-density shape)
  {
    int best = 2;
    float tbest = 1e30f;
    for (int c : {1, 2, 4}) {
      ctx->tune[TUNE_BF16X3_CHUNK][bucket_of((nS + 63) / 64 * 64)] = c;
      const float t = time_best(ctx, [&] {
        return qk_gemm_bf16x3_nt(ctx, (int)N2, nS, nS, A, N2, B, nS, Cm, N2);
      });
      if (t < tbest) { tbest = t; best = c; }
    }
    ctx->tune[TUNE_BF16X3_CHUNK][bucket_of((nS + 63) / 64 * 64)] = best;
  }
  // 2. split-K multiplier (the back-transformation shape n x 64 x n)
  {
    int best = 2;
    float tbest = 1e30f;
    for (int mlt : {1, 2, 4}) {
      ctx->tune[TUNE_SPLITK_MULT][bucket_of(nS)] = mlt;
      const float t = time_best(ctx, [&] {
        return qk_dgemm(ctx, 'N', 'N', nS, 64, nS, 1.0, B, nS, 0, B + nB, nS, 0, 0.0, Cm, nS, 0, 1);
      });
      if (t < tbest) { tbest = t; best = mlt; }
    }
    ctx->tune[TUNE_SPLITK_MULT][bucket_of(nS)] = best;
  }
  // 3. sigma sweep chunks (rho = A reinterpreted as N x N x nS, energies/Om from B)
  {
    int best = 4;
    float tbest = 1e30f;
    const int nO = N / 8 > 0 ? N / 8 : 1;
    const int nS2 = nO * (N - nO) <= nS ? nO * (N - nO) : nS;
    double* out = Cm;
    for (int cm : {2, 4, 8}) {
      ctx->tune[TUNE_SIGMA_CHUNKS][bucket_of(nS2)] = cm;
      const float t = time_best(ctx, [&] {
        return qk_sigma_diag(ctx, 0, 0.0, 500.0, N, 0, nO, 0, nS2, B, B + N, A, out, out + N,
                             out + 2 * N);
      });
      if (t < tbest) { tbest = t; best = cm; }
    }
    ctx->tune[TUNE_SIGMA_CHUNKS][bucket_of(nS2)] = best;
  }
  // 4. tridiagonalisation grid (eigenvalues only of a random symmetric nS x nS matrix)
  {
    int best = 4;
    float tbest = 1e30f;
    double* w = nullptr;
    st = qk_wst(ctx, W_TUNE, (size_t)nS + 16, &w);
    if (st == QK_OK) {
      for (int gq : {2, 3, 4}) {
        ctx->tune[TUNE_SYTRD_GRID][bucket_of(nS)] = gq;
        const float t = time_best(ctx, [&] {
          k_fill<<<1024, 256, 0, ctx->stream>>>((long long)nB, B + nB, 1.0, 3);
          k_symmetrise<<<1024, 256, 0, ctx->stream>>>(nS, B + nB);
          ctx->launches += 2;
          const bool tm = ctx->time_eig;
          ctx->time_eig = false;
          const int r = qk_eig_sym(ctx, nS, B + nB, nS, w, nullptr, 0);
          ctx->time_eig = tm;
          return r;
        }, 1);
        if (t < tbest) { tbest = t; best = gq; }
      }
      ctx->tune[TUNE_SYTRD_GRID][bucket_of(nS)] = best;
    }
  }
  // 5. k-section width of the bisection (eigenvalues of a random symmetric nS x nS matrix; the
  //    tridiagonalisation is part of each timing and the same for every candidate)
  if (st == QK_OK) {
    double* w = nullptr;
    st = qk_wst(ctx, W_TUNE, (size_t)nS + 16, &w);
    if (st == QK_OK) {
      int best = 0;
      float tbest = 1e30f;
      for (int kk : {2, 4, 8}) {
        ctx->tune[TUNE_STEBZ_K][bucket_of(nS)] = kk;
        const float t = time_best(ctx, [&] {
          k_fill<<<1024, 256, 0, ctx->stream>>>((long long)nB, B + nB, 1.0, 3);
          k_symmetrise<<<1024, 256, 0, ctx->stream>>>(nS, B + nB);
          ctx->launches += 2;
          const bool tm = ctx->time_eig;
          ctx->time_eig = false;
          const int r = qk_eig_sym(ctx, nS, B + nB, nS, w, nullptr, 0);
          ctx->time_eig = tm;
          return r;
        }, 1);
        if (t < tbest) { tbest = t; best = kk; }
      }
      ctx->tune[TUNE_STEBZ_K][bucket_of(nS)] = best;
    }
  }
  // 6. FP64 GEMM path on the back-transformation shapes and the FP64 excitation density
  {
    struct Shape { int m, n, k; };
    const Shape shapes[3] = {{nS, 128, nS}, {nS, nS, 128}, {(int)N2, nS, nS}};
    for (const Shape& sh : shapes) {
      const long long key = (long long)sh.m * sh.n;
      int best = 1;
      float tbest = 1e30f;
      for (int path : {1, 2}) {
        ctx->tune[TUNE_DGEMM_PATH][bucket_of(key)] = path;
        const float t = time_best(ctx, [&] {
          return qk_dgemm(ctx, 'N', 'N', sh.m, sh.n, sh.k, 1.0, sh.m == (int)N2 ? A : B, sh.m, 0,
                          B + nB, sh.k, 0, 0.0, Cm, sh.m, 0, 1);
        }, 1);
        if (t < tbest) { tbest = t; best = path; }
      }
      ctx->tune[TUNE_DGEMM_PATH][bucket_of(key)] = best;
    }
  }
  cudaStreamSynchronize(ctx->stream);
  cudaFree(A);
  cudaFree(B);
  cudaFree(Cm);
  return st;
}

int qk_tune_save(const qk_ctx* ctx, const char* path) {
  if (!ctx || !path) return QK_ERR_ARG;
  FILE* f = fopen(path, "w");
  if (!f) return QK_ERR_ARG;
  fprintf(f, "{\"version\": 1, \"entries\": [");
  bool first = true;
  for (int p = 0; p < TUNE_NUM; ++p)
    for (int b = 0; b < TUNE_BUCKETS; ++b)
      if (ctx->tune[p][b] > 0) {
        fprintf(f, "%s\n  {\"param\": \"%s\", \"bucket\": %d, \"value\": %d}", first ? "" : ",",
                k_tune_names[p], b, ctx->tune[p][b]);
        first = false;
      }
  fprintf(f, "\n]}\n");
  fclose(f);
  return QK_OK;
}

int qk_tune_load(qk_ctx* ctx, const char* path) {
  if (!ctx || !path) return QK_ERR_ARG;
  FILE* f = fopen(path, "r");
  if (!f) return QK_ERR_ARG;
  std::string txt;
  char buf[4096];
  size_t n;
  while ((n = fread(buf, 1, sizeof(buf), f)) > 0) txt.append(buf, n);
  fclose(f);
  size_t pos = 0;
  int loaded = 0;
  while ((pos = txt.find("\"param\"", pos)) != std::string::npos) {
    const size_t q1 = txt.find('"', txt.find(':', pos) + 1);
    const size_t q2 = txt.find('"', q1 + 1);
    if (q1 == std::string::npos || q2 == std::string::npos) break;
    const std::string name = txt.substr(q1 + 1, q2 - q1 - 1);
    const size_t pb = txt.find("\"bucket\"", q2), pv = txt.find("\"value\"", q2);
    if (pb == std::string::npos || pv == std::string::npos) break;
    const int b = atoi(txt.c_str() + txt.find(':', pb) + 1);
    const int v = atoi(txt.c_str() + txt.find(':', pv) + 1);
    for (int p = 0; p < TUNE_NUM; ++p)
      if (name == k_tune_names[p] && b >= 0 && b < TUNE_BUCKETS && v > 0) {
        ctx->tune[p][b] = v;
        ++loaded;
      }
    pos = pv + 1;
  }
  return loaded > 0 ? QK_OK : QK_ERR_ARG;
}

}  // extern "C"
