// k_gemm64.cu -- FP64 GEMM on the FP64 tensor path (DMMA, mma.sync.m8n8k4.f64).
//
// Column-major C = alpha*op(A)*op(B) + beta*C, strided batch.  Used for the AO->MO quarter
// transforms (AOtoMO/AOtoMO_ERI_RHF.f90:26-53), the FP64 excitation density
// (GW/RGW_excitation_density.f90:48-50) and the blocked back-transformation of the
// eigensolver.  Tile 64x64x16, 4 warps (2x2), each warp a 32x32 block of 4x4 DMMA tiles;
// operands are staged global -> registers -> shared memory with one stage of prefetch.
// On GB300 the FP64 rate (~1.2 TFLOP/s) is the bound for every FP64 contraction here, so the
// kernel is shaped for issue rate (16 DMMA per 8 shared loads), not for bandwidth.
#include "qk_internal.cuh"

namespace {

constexpr int BM = 64, BN = 64, BK = 16, LDS = BM + 4;

__device__ __forceinline__ void dmma884(double& d0, double& d1, double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
      : "+d"(d0), "+d"(d1)
      : "d"(a), "d"(b));
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_dgemm_dmma(int M, int N, int K, double alpha,
                                                     const double* __restrict__ A, long long lda,
                                                     long long sA, const double* __restrict__ B,
                                                     long long ldb, long long sB, double beta,
                                                     double* __restrict__ C, long long ldc,
                                                     long long sC) {
  __shared__ double As[2][BK][LDS];
  __shared__ double Bs[2][BK][LDS];
  const long long bz = blockIdx.z;
  A += bz * sA;
  B += bz * sB;
  C += bz * sC;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp & 1) * 32, wn = (warp >> 1) * 32;
  const int g = lane >> 2, t = lane & 3;

  double acc[4][4][2];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = 0.0;

  double ra[8], rb[8];
  auto ldA = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int idx = tid + r * 128;
      int mm, kk;
      if (!TA) { mm = idx & 63; kk = idx >> 6; } else { kk = idx & 15; mm = idx >> 4; }
      const int gm = m0 + mm, gk = k0 + kk;
      double v = 0.0;
      if (gm < M && gk < K) v = !TA ? A[gm + lda * gk] : A[gk + lda * gm];
      ra[r] = v;
    }
  };
  auto stA = [&](int s) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int idx = tid + r * 128;
      int mm, kk;
      if (!TA) { mm = idx & 63; kk = idx >> 6; } else { kk = idx & 15; mm = idx >> 4; }
      As[s][kk][mm] = ra[r];
    }
  };
  auto ldB = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int idx = tid + r * 128;
      int nn, kk;
      if (!TB) { kk = idx & 15; nn = idx >> 4; } else { nn = idx & 63; kk = idx >> 6; }
      const int gn = n0 + nn, gk = k0 + kk;
      double v = 0.0;
      if (gn < N && gk < K) v = !TB ? B[gk + ldb * gn] : B[gn + ldb * gk];
      rb[r] = v;
    }
  };
  auto stB = [&](int s) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int idx = tid + r * 128;
      int nn, kk;
      if (!TB) { kk = idx & 15; nn = idx >> 4; } else { nn = idx & 63; kk = idx >> 6; }
      Bs[s][kk][nn] = rb[r];
    }
  };

  ldA(0);
  ldB(0);
  stA(0);
  stB(0);
  __syncthreads();
  int s = 0;
  for (int k0 = 0; k0 < K; k0 += BK) {
    const bool more = (k0 + BK) < K;
    if (more) { ldA(k0 + BK); ldB(k0 + BK); }
#pragma unroll
    for (int kk = 0; kk < BK; kk += 4) {
      double af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) af[i] = As[s][kk + t][wm + i * 8 + g];
#pragma unroll
      for (int j = 0; j < 4; ++j) bf[j] = Bs[s][kk + t][wn + j * 8 + g];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) dmma884(acc[i][j][0], acc[i][j][1], af[i], bf[j]);
    }
    if (more) { stA(s ^ 1); stB(s ^ 1); }
    __syncthreads();
    s ^= 1;
  }

#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + wm + i * 8 + g;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int gn = n0 + wn + j * 8 + 2 * t + h;
        if (gn < N) {
          double* c = C + gm + ldc * (long long)gn;
          double v = alpha * acc[i][j][h];
          if (beta != 0.0) v += beta * (*c);
          *c = v;
        }
      }
    }
  }
}

}  // namespace

int qk_dgemm(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha, const double* A,
             long long lda, long long strideA, const double* B, long long ldb, long long strideB,
             double beta, double* C, long long ldc, long long strideC, int batch) {
  if (m <= 0 || n <= 0 || batch <= 0) return QK_OK;
  if (k <= 0) {
    // C = beta*C: only beta == 0 is needed by callers
    if (beta != 0.0) return qk_fail(ctx, QK_ERR_ARG, "qk_dgemm: k=0 with beta!=0");
    for (int b = 0; b < batch; ++b)
      QK_CK(cudaMemset2DAsync(C + b * strideC, ldc * sizeof(double), 0, m * sizeof(double), n,
                              ctx->stream));
    return QK_OK;
  }
  const bool TA = (ta == 'T' || ta == 't'), TB = (tb == 'T' || tb == 't');
  dim3 grid((m + BM - 1) / BM, (n + BN - 1) / BN, batch);
  if (grid.y > 65535 || grid.z > 65535) return qk_fail(ctx, QK_ERR_ARG, "qk_dgemm: grid too large");
  if (!TA && !TB)
    k_dgemm_dmma<false, false><<<grid, 128, 0, ctx->stream>>>(m, n, k, alpha, A, lda, strideA, B, ldb,
                                                             strideB, beta, C, ldc, strideC);
  else if (!TA && TB)
    k_dgemm_dmma<false, true><<<grid, 128, 0, ctx->stream>>>(m, n, k, alpha, A, lda, strideA, B, ldb,
                                                            strideB, beta, C, ldc, strideC);
  else if (TA && !TB)
    k_dgemm_dmma<true, false><<<grid, 128, 0, ctx->stream>>>(m, n, k, alpha, A, lda, strideA, B, ldb,
                                                            strideB, beta, C, ldc, strideC);
  else
    k_dgemm_dmma<true, true><<<grid, 128, 0, ctx->stream>>>(m, n, k, alpha, A, lda, strideA, B, ldb,
                                                           strideB, beta, C, ldc, strideC);
  QK_LAUNCHED();
  return QK_OK;
}
