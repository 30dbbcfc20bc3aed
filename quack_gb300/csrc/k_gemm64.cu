// k_gemm64.cu -- FP64 GEMM: the FP64 tensor path (DMMA, mma.sync.m8n8k4.f64) and a DFMA path,
// plus an FP32-product variant with FP64 operands and result (the mixed tier's eigenvector
// back-transformation).
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
                                                     long long sC, int kc) {
  __shared__ double As[2][BK][LDS];
  __shared__ double Bs[2][BK][LDS];
  const long long bz = blockIdx.z;
  // kc < 0: only the lower triangle of C is wanted, tiles strictly above the diagonal exit
  if (kc < 0 && (int)(blockIdx.x + 1) * BM <= (int)blockIdx.y * BN) return;
  int kbeg = 0, kend = K;
  if (kc > 0) {  // split-K: slice bz covers [bz*kc, min(K, bz*kc+kc)) and writes its own C slice
    kbeg = (int)bz * kc;
    kend = min(K, kbeg + kc);
    C += bz * sC;
  } else {
    A += bz * sA;
    B += bz * sB;
    C += bz * sC;
  }
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
      if (gm < M && gk < kend) v = !TA ? A[gm + lda * gk] : A[gk + lda * gm];
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
      if (gn < N && gk < kend) v = !TB ? B[gk + ldb * gn] : B[gn + ldb * gk];
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

  ldA(kbeg);
  ldB(kbeg);
  stA(0);
  stB(0);
  __syncthreads();
  int s = 0;
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    const bool more = (k0 + BK) < kend;
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

// The same GEMM on the FMA path.  With T = double (DFMA): on GB300 DFMA and DMMA share one FP64
// datapath and DFMA issues slightly faster (1.2 vs 1.05 TFLOP/s measured), so a plain
// register-tiled kernel can beat the tensor path: 256 threads, each a 4x4 block of C (rows
// tx + 16 i, columns ty + 16 j) with 16 independent FMA chains, 8 shared loads per 16 FMA.
// With T = float the FP64 operands are rounded to FP32 as they are staged and the products and
// partial sums are FP32 (64x the FP64 issue rate); C stays FP64 (alpha, beta applied in FP64).
// kscale (FP32 path, batched, no split-K): op(B)(k, n) is scaled by kscale[batch * sK + k] as it
// is staged, i.e. C = alpha op(A) diag(kscale) op(B) + beta C.
template <bool TA, bool TB, typename T>
__global__ void __launch_bounds__(256) k_gemm_simt(int M, int N, int K, double alpha,
                                                     const double* __restrict__ A, long long lda,
                                                     long long sA, const double* __restrict__ B,
                                                     long long ldb, long long sB, double beta,
                                                     double* __restrict__ C, long long ldc,
                                                     long long sC, int kc,
                                                     const float* __restrict__ kscale,
                                                     long long sK) {
  __shared__ T As[2][BK][BM];
  __shared__ T Bs[2][BK][BN];
  const long long bz = blockIdx.z;
  if (kc < 0 && (int)(blockIdx.x + 1) * BM <= (int)blockIdx.y * BN) return;  // lower C only
  int kbeg = 0, kend = K;
  if (kc > 0) {
    kbeg = (int)bz * kc;
    kend = min(K, kbeg + kc);
    C += bz * sC;
  } else {
    A += bz * sA;
    B += bz * sB;
    C += bz * sC;
    if (kscale) kscale += bz * sK;
  }
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;

  constexpr bool kF32 = sizeof(T) == 4;
  // FP32: each k tile's 16 products are summed in FP32 and folded into a compensated (hi, lo)
  // pair by TwoSum, so the rounding of the long sum does not grow with K
  T acc[4][4], lo[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = lo[i][j] = T(0);

  T ra[4], rb[4];
  auto ldA = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + r * 256;
      int mm, kk;
      if (!TA) { mm = idx & 63; kk = idx >> 6; } else { kk = idx & 15; mm = idx >> 4; }
      const int gm = m0 + mm, gk = k0 + kk;
      double v = 0.0;
      if (gm < M && gk < kend) v = !TA ? A[gm + lda * gk] : A[gk + lda * gm];
      ra[r] = (T)v;
    }
  };
  auto stA = [&](int st) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + r * 256;
      int mm, kk;
      if (!TA) { mm = idx & 63; kk = idx >> 6; } else { kk = idx & 15; mm = idx >> 4; }
      As[st][kk][mm] = ra[r];
    }
  };
  auto ldB = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + r * 256;
      int nn, kk;
      if (!TB) { kk = idx & 15; nn = idx >> 4; } else { nn = idx & 63; kk = idx >> 6; }
      const int gn = n0 + nn, gk = k0 + kk;
      double v = 0.0;
      if (gn < N && gk < kend) v = !TB ? B[gk + ldb * gn] : B[gn + ldb * gk];
      rb[r] = (T)v;
      if (sizeof(T) == 4 && kscale && gk < kend) rb[r] *= (T)kscale[gk];
    }
  };
  auto stB = [&](int st) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int idx = tid + r * 256;
      int nn, kk;
      if (!TB) { kk = idx & 15; nn = idx >> 4; } else { nn = idx & 63; kk = idx >> 6; }
      Bs[st][kk][nn] = rb[r];
    }
  };

  ldA(kbeg);
  ldB(kbeg);
  stA(0);
  stB(0);
  __syncthreads();
  int st = 0;
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    const bool more = (k0 + BK) < kend;
    if (more) { ldA(k0 + BK); ldB(k0 + BK); }
    T part[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) part[i][j] = kF32 ? T(0) : acc[i][j];
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) af[i] = As[st][kk][tx + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bf[j] = Bs[st][kk][ty + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) part[i][j] = fma(af[i], bf[j], part[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (kF32) {
          const T a0 = acc[i][j], b0 = part[i][j];
          const T sum = a0 + b0, bp = sum - a0;
          lo[i][j] += (a0 - (sum - bp)) + (b0 - bp);
          acc[i][j] = sum;
        } else {
          acc[i][j] = part[i][j];
        }
      }
    if (more) { stA(st ^ 1); stB(st ^ 1); }
    __syncthreads();
    st ^= 1;
  }

#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + tx + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + ty + 16 * j;
      if (gn < N) {
        double* c = C + gm + ldc * (long long)gn;
        double v = alpha * ((double)acc[i][j] + (double)lo[i][j]);
        if (beta != 0.0) v += beta * (*c);
        *c = v;
      }
    }
  }
}

// DFMA GEMM with tall 128 x 32 tiles for outputs with few columns (the quarter transforms of
// qsGW contract the AO tensor with the nO occupied columns: a 64-wide tile would run mostly on
// padding).  Same contract as k_gemm_simt<TA, TB, double> (split-K slices, strided batches, no
// lower-triangle mode): 256 threads, each a 4 x 4 block of C (rows tx + 32 i, columns ty + 8 j),
// 16 independent FMA chains, 8 shared loads per 16 FMA.
constexpr int TM = 128, TN = 32;
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_gemm_tall(int M, int N, int K, double alpha,
                                                     const double* __restrict__ A, long long lda,
                                                     long long sA, const double* __restrict__ B,
                                                     long long ldb, long long sB, double beta,
                                                     double* __restrict__ C, long long ldc,
                                                     long long sC, int kc) {
  __shared__ double As[2][BK][TM];
  __shared__ double Bs[2][BK][TN];
  const long long bz = blockIdx.z;
  int kbeg = 0, kend = K;
  if (kc > 0) {
    kbeg = (int)bz * kc;
    kend = min(K, kbeg + kc);
    C += bz * sC;
  } else {
    A += bz * sA;
    B += bz * sB;
    C += bz * sC;
  }
  const int m0 = blockIdx.x * TM, n0 = blockIdx.y * TN;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
  double ra[8], rb[2];
  auto ldA = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int idx = tid + r * 256;
      int mm, kk;
      if (!TA) { mm = idx & (TM - 1); kk = idx >> 7; } else { kk = idx & (BK - 1); mm = idx >> 4; }
      const int gm = m0 + mm, gk = k0 + kk;
      ra[r] = (gm < M && gk < kend) ? (!TA ? A[gm + lda * gk] : A[gk + lda * gm]) : 0.0;
    }
  };
  auto stA = [&](int st) {
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int idx = tid + r * 256;
      int mm, kk;
      if (!TA) { mm = idx & (TM - 1); kk = idx >> 7; } else { kk = idx & (BK - 1); mm = idx >> 4; }
      As[st][kk][mm] = ra[r];
    }
  };
  auto ldB = [&](int k0) {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + r * 256;
      int nn, kk;
      if (!TB) { kk = idx & (BK - 1); nn = idx >> 4; } else { nn = idx & (TN - 1); kk = idx >> 5; }
      const int gn = n0 + nn, gk = k0 + kk;
      rb[r] = (gn < N && gk < kend) ? (!TB ? B[gk + ldb * gn] : B[gn + ldb * gk]) : 0.0;
    }
  };
  auto stB = [&](int st) {
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int idx = tid + r * 256;
      int nn, kk;
      if (!TB) { kk = idx & (BK - 1); nn = idx >> 4; } else { nn = idx & (TN - 1); kk = idx >> 5; }
      Bs[st][kk][nn] = rb[r];
    }
  };
  ldA(kbeg);
  ldB(kbeg);
  stA(0);
  stB(0);
  __syncthreads();
  int st = 0;
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    const bool more = (k0 + BK) < kend;
    if (more) { ldA(k0 + BK); ldB(k0 + BK); }
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      double af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) af[i] = As[st][kk][tx + 32 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bf[j] = Bs[st][kk][ty + 8 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(af[i], bf[j], acc[i][j]);
    }
    if (more) { stA(st ^ 1); stB(st ^ 1); }
    __syncthreads();
    st ^= 1;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + tx + 32 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + ty + 8 * j;
      if (gn < N) {
        double* c = C + gm + ldc * (long long)gn;
        double v = alpha * acc[i][j];
        if (beta != 0.0) v += beta * (*c);
        *c = v;
      }
    }
  }
}

// Double-float GEMM (the mixed tier's accurate substitute for FP64 on the FP32 pipe): each FP64
// operand is staged as an FP32 pair a = ah + al (al = fl32(a - ah)), each product is formed
// exactly to 2^-48 by TwoProduct (p = ah bh, e = fma(ah, bh, -p) + ah bl + al bh) and added to a
// (hi, lo) accumulator by TwoSum, so the result is accurate to ~K 2^-48 of sum |a_ik b_kj|
// whatever the cancellation -- about twelve FP32 operations per multiply-add, on a pipe with 64x
// the FP64 issue rate.  Tiles BMt x BNt (64 x 64, or 128 x 32 for outputs with few columns),
// 256 threads, each a 4 x 4 block of C; split-K slices and strided batches as k_gemm_simt.
template <bool TA, bool TB, int BMt, int BNt>
__global__ void __launch_bounds__(256) k_gemm_df(int M, int N, int K, double alpha,
                                                   const double* __restrict__ A, long long lda,
                                                   long long sA, const double* __restrict__ B,
                                                   long long ldb, long long sB, double beta,
                                                   double* __restrict__ C, long long ldc,
                                                   long long sC, int kc) {
  constexpr int RT = BMt / 4, CT = BNt / 4;  // RT * CT = 256
  constexpr int NA = BMt * BK / 256, NB = BNt * BK / 256;
  __shared__ float2 As[2][BK][BMt];
  __shared__ float2 Bs[2][BK][BNt];
  const long long bz = blockIdx.z;
  int kbeg = 0, kend = K;
  if (kc > 0) {
    kbeg = (int)bz * kc;
    kend = min(K, kbeg + kc);
    C += bz * sC;
  } else {
    A += bz * sA;
    B += bz * sB;
    C += bz * sC;
  }
  const int m0 = blockIdx.x * BMt, n0 = blockIdx.y * BNt;
  const int tid = threadIdx.x, tx = tid % RT, ty = tid / RT;
  float hi[4][4], lo[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) hi[i][j] = lo[i][j] = 0.0f;
  auto split = [](double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double)h));
  };
  double ra[NA], rb[NB];
  auto ldA = [&](int k0) {
#pragma unroll
    for (int r = 0; r < NA; ++r) {
      const int idx = tid + r * 256;
      int mm, kk;
      if (!TA) { mm = idx % BMt; kk = idx / BMt; } else { kk = idx % BK; mm = idx / BK; }
      const int gm = m0 + mm, gk = k0 + kk;
      ra[r] = (gm < M && gk < kend) ? (!TA ? A[gm + lda * gk] : A[gk + lda * gm]) : 0.0;
    }
  };
  auto stA = [&](int st) {
#pragma unroll
    for (int r = 0; r < NA; ++r) {
      const int idx = tid + r * 256;
      int mm, kk;
      if (!TA) { mm = idx % BMt; kk = idx / BMt; } else { kk = idx % BK; mm = idx / BK; }
      As[st][kk][mm] = split(ra[r]);
    }
  };
  auto ldB = [&](int k0) {
#pragma unroll
    for (int r = 0; r < NB; ++r) {
      const int idx = tid + r * 256;
      int nn, kk;
      if (!TB) { kk = idx % BK; nn = idx / BK; } else { nn = idx % BNt; kk = idx / BNt; }
      const int gn = n0 + nn, gk = k0 + kk;
      rb[r] = (gn < N && gk < kend) ? (!TB ? B[gk + ldb * gn] : B[gn + ldb * gk]) : 0.0;
    }
  };
  auto stB = [&](int st) {
#pragma unroll
    for (int r = 0; r < NB; ++r) {
      const int idx = tid + r * 256;
      int nn, kk;
      if (!TB) { kk = idx % BK; nn = idx / BK; } else { nn = idx % BNt; kk = idx / BNt; }
      Bs[st][kk][nn] = split(rb[r]);
    }
  };
  ldA(kbeg);
  ldB(kbeg);
  stA(0);
  stB(0);
  __syncthreads();
  int st = 0;
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    const bool more = (k0 + BK) < kend;
    if (more) { ldA(k0 + BK); ldB(k0 + BK); }
#pragma unroll 4
    for (int kk = 0; kk < BK; ++kk) {
      float2 af[4], bf[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) af[i] = As[st][kk][tx + RT * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bf[j] = Bs[st][kk][ty + CT * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          // __fmul_rn / __fadd_rn keep the compiler from contracting hi + ah bh into an FMA,
          // which would break the error-free transformations
          const float p = __fmul_rn(af[i].x, bf[j].x);
          float e = fmaf(af[i].x, bf[j].x, -p);
          e = fmaf(af[i].x, bf[j].y, e);
          e = fmaf(af[i].y, bf[j].x, e);
          const float s = __fadd_rn(hi[i][j], p);
          const float bb = __fsub_rn(s, hi[i][j]);
          const float er = __fadd_rn(__fsub_rn(hi[i][j], __fsub_rn(s, bb)), __fsub_rn(p, bb));
          hi[i][j] = s;
          lo[i][j] += er + e;
        }
    }
    if (more) { stA(st ^ 1); stB(st ^ 1); }
    __syncthreads();
    st ^= 1;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + tx + RT * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + ty + CT * j;
      if (gn < N) {
        double* c = C + gm + ldc * (long long)gn;
        double v = alpha * ((double)hi[i][j] + (double)lo[i][j]);
        if (beta != 0.0) v += beta * (*c);
        *c = v;
      }
    }
  }
}

// C = alpha * sum_s W[s] + beta * C  (split-K reduction, column-major m x n)
__global__ void k_splitk_reduce(int m, int n, int S, const double* __restrict__ W, double alpha,
                                double beta, double* __restrict__ C, long long ldc) {
  const long long total = (long long)m * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int s = 0; s < S; ++s) acc += W[(long long)s * total + i];
    const int r = (int)(i % m);
    const long long c = i / m;
    double* cp = C + r + ldc * c;
    double v = alpha * acc;
    if (beta != 0.0) v += beta * (*cp);
    *cp = v;
  }
}

// path: 0 = DMMA, 1 = DFMA, 2 = FP32 products, 3 = DFMA with tall 128 x 32 tiles,
// 4 / 5 = double-float products (64 x 64 / 128 x 32 tiles)
template <bool TA, bool TB>
void launch(int path, dim3 grid, cudaStream_t st, int m, int n, int k, double alpha,
            const double* A, long long lda, long long sA, const double* B, long long ldb,
            long long sB, double beta, double* C, long long ldc, long long sC, int kc,
            const float* kscale, long long sK) {
  if (path == 3)
    k_gemm_tall<TA, TB><<<grid, 256, 0, st>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C,
                                              ldc, sC, kc);
  else if (path == 4)
    k_gemm_df<TA, TB, 64, 64><<<grid, 256, 0, st>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta,
                                                    C, ldc, sC, kc);
  else if (path == 5)
    k_gemm_df<TA, TB, TM, TN><<<grid, 256, 0, st>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta,
                                                    C, ldc, sC, kc);
  else if (path == 1)
    k_gemm_simt<TA, TB, double><<<grid, 256, 0, st>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB,
                                                      beta, C, ldc, sC, kc, nullptr, 0);
  else if (path == 2)
    k_gemm_simt<TA, TB, float><<<grid, 256, 0, st>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB,
                                                     beta, C, ldc, sC, kc, kscale, sK);
  else
    k_dgemm_dmma<TA, TB><<<grid, 128, 0, st>>>(m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C,
                                               ldc, sC, kc);
}

void launch_any(int path, bool TA, bool TB, dim3 grid, cudaStream_t st, int m, int n, int k,
                double alpha, const double* A, long long lda, long long sA, const double* B,
                long long ldb, long long sB, double beta, double* C, long long ldc, long long sC,
                int kc, const float* ks = nullptr, long long sK = 0) {
  if (!TA && !TB) launch<false, false>(path, grid, st, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, kc, ks, sK);
  else if (!TA && TB) launch<false, true>(path, grid, st, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, kc, ks, sK);
  else if (TA && !TB) launch<true, false>(path, grid, st, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, kc, ks, sK);
  else launch<true, true>(path, grid, st, m, n, k, alpha, A, lda, sA, B, ldb, sB, beta, C, ldc, sC, kc, ks, sK);
}

}  // namespace

namespace {

int gemm_impl(qk_ctx* ctx, bool fp32, char ta, char tb, int m, int n, int k, double alpha,
              const double* A, long long lda, long long strideA, const double* B, long long ldb,
              long long strideB, double beta, double* C, long long ldc, long long strideC,
              int batch, bool lower = false, const float* kscale = nullptr, long long sK = 0,
              bool df = false) {
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
  // FP64 path: 1 = DFMA (default), 2 = DMMA tensor path; tunable per size of the product
  int path = df ? 4 : fp32 ? 2
                        : (qk_tune_get(ctx, TUNE_DGEMM_PATH, (long long)m * n, 1) != 2 ? 1 : 0);
  if (df && (lower || kscale)) return qk_fail(ctx, QK_ERR_ARG, "double-float GEMM: full C only");
  // 128 x 32 tiles where they cover m x n with clearly less padding than 64 x 64 (outputs with
  // few columns): DFMA -> path 3, double-float -> path 5
  if ((path == 1 || path == 4) && !lower && !kscale) {
    const long long a64 = (long long)((m + 63) / 64) * 64 * ((n + 63) / 64) * 64;
    const long long a32 = (long long)((m + TM - 1) / TM) * TM * ((n + TN - 1) / TN) * TN;
    if (8 * a32 < 7 * a64) path = path == 1 ? 3 : 5;
  }
  const bool tall = path == 3 || path == 5;
  const int tm = tall ? TM : BM, tn = tall ? TN : BN;
  dim3 grid((m + tm - 1) / tm, (n + tn - 1) / tn, batch);
  if (grid.y > 65535 || grid.z > 65535) return qk_fail(ctx, QK_ERR_ARG, "qk_dgemm: grid too large");
  const long long tiles = (long long)grid.x * grid.y;
  // fewer output tiles than mult CTAs per SM and a long K: split K and reduce
  const int mult = qk_tune_get(ctx, TUNE_SPLITK_MULT, k, 4);
  if (!lower && !kscale && batch == 1 && tiles < (long long)mult * ctx->num_sms && k >= 4 * BK) {
    int S = (int)(((long long)mult * ctx->num_sms + tiles - 1) / tiles);
    const int maxS = k / (2 * BK);
    if (S > maxS) S = maxS;
    if (S > 32) S = 32;
    if (S >= 2) {
      const int kc = ((k + S - 1) / S + BK - 1) / BK * BK;
      S = (k + kc - 1) / kc;
      double* W = nullptr;
      QK_TRY(qk_wst(ctx, W_SPLITK, (size_t)S * m * n, &W));
      grid.z = S;
      launch_any(path, TA, TB, grid, ctx->stream, m, n, k, 1.0, A, lda, 0, B, ldb, 0, 0.0, W, m,
                 (long long)m * n, kc);
      QK_LAUNCHED();
      long long total = (long long)m * n;
      int blocks = (int)((total + 255) / 256);
      if (blocks > 16 * ctx->num_sms) blocks = 16 * ctx->num_sms;
      k_splitk_reduce<<<blocks, 256, 0, ctx->stream>>>(m, n, S, W, alpha, beta, C, ldc);
      QK_LAUNCHED();
      return QK_OK;
    }
  }
  launch_any(path, TA, TB, grid, ctx->stream, m, n, k, alpha, A, lda, strideA, B, ldb, strideB,
             beta, C, ldc, strideC, lower ? -1 : 0, kscale, sK);
  QK_LAUNCHED();
  return QK_OK;
}

}  // namespace

int qk_dgemm(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha, const double* A,
             long long lda, long long strideA, const double* B, long long ldb, long long strideB,
             double beta, double* C, long long ldc, long long strideC, int batch) {
  return gemm_impl(ctx, false, ta, tb, m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta, C,
                   ldc, strideC, batch);
}

int qk_gemm_df(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha, const double* A,
               long long lda, long long strideA, const double* B, long long ldb,
               long long strideB, double beta, double* C, long long ldc, long long strideC,
               int batch) {
  return gemm_impl(ctx, false, ta, tb, m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta, C,
                   ldc, strideC, batch, false, nullptr, 0, true);
}

int qk_gemm_f32p(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha,
                 const double* A, long long lda, long long strideA, const double* B, long long ldb,
                 long long strideB, double beta, double* C, long long ldc, long long strideC,
                 int batch) {
  return gemm_impl(ctx, true, ta, tb, m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta, C,
                   ldc, strideC, batch);
}

int qk_gemm_f32p_lower(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha,
                       const double* A, long long lda, long long strideA, const double* B,
                       long long ldb, long long strideB, double beta, double* C, long long ldc,
                       long long strideC, int batch, const float* kscale, long long sK) {
  return gemm_impl(ctx, true, ta, tb, m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta, C,
                   ldc, strideC, batch, true, kscale, sK);
}

int qk_dgemm_lower(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha,
                   const double* A, long long lda, long long strideA, const double* B,
                   long long ldb, long long strideB, double beta, double* C, long long ldc,
                   long long strideC, int batch) {
  return gemm_impl(ctx, false, ta, tb, m, n, k, alpha, A, lda, strideA, B, ldb, strideB, beta, C,
                   ldc, strideC, batch, true);
}
