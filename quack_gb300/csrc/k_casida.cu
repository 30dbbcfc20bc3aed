// k_casida.cu -- Casida (dRPA singlet) builders and epilogues.
//
//  k_build_AB   : LR/phRLR_A.f90:43-118 / LR/phRLR_B.f90:34-98 as a tiled, coalesced gather
//                 of the (vo|ov) block of the physicist ERI with a shared-memory transpose.
//  k_casida_M   : the dRPA product M = AmBSq.(A+B).AmBSq of LR/phRLR.f90:50-63 in one pass.
//                 For dRPA, A-B is diagonal bit-for-bit (A and B carry the same 2*ERI term), so
//                 dsyev/ADAt reduce to AmBSq = diag(sqrt(fl(A_ii-B_ii))) exactly; the builder
//                 reproduces every rounding of the reference product order:
//                 M(ia,jb) = s_ia * ((A+B)(ia,jb) * s_jb).
//  k_xpy        : XpY = DA(1/sqrt(Om), Z^T.AmBSq), XmY = DA(sqrt(Om), Z^T.AmBIv)  (phRLR.f90:76-81)
//  k_slab       : tmp(p,q,jb) = ERI(p,j,q,b)  (GW/RGW_excitation_density.f90:30-46)
#include <cmath>
#include "qk_internal.cuh"

namespace {

constexpr int TB = 32;

// which: 0 -> A, 1 -> B.   out(ia,jb) at ia + nS*jb.
__global__ void __launch_bounds__(TB * 8) k_build_AB(int which, int ispin, double ct1, double ct2,
                                                      int N, int nC, int nO, int nR,
                                                      const double* __restrict__ e,
                                                      const double* __restrict__ ERI,
                                                      double* __restrict__ out) {
  __shared__ double t1[TB][TB + 1];
  __shared__ double t2[TB][TB + 1];
  const int no = nO - nC, nv = N - nO - nR;
  const long long nS = (long long)no * nv;
  const int ij = blockIdx.z;
  const int ip = ij / no, jp = ij - ip * no;  // i' and j'
  const int i = ip + nC, j = jp + nC;
  const int a0 = blockIdx.x * TB, b0 = blockIdx.y * TB;
  const long long N1 = N, N2 = N1 * N1, N3 = N2 * N1;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  // read: tx -> b (contiguous), ty -> a
  for (int r = ty; r < TB; r += 8) {
    const int ap = a0 + r, bp = b0 + tx;
    double v1 = 0.0, v2 = 0.0;
    if (ap < nv && bp < nv) {
      const long long a = ap + nO, b = bp + nO;
      if (ispin == 1) v1 = __ldg(ERI + b + N1 * i + N2 * j + N3 * a);  // ERI(b,i,j,a)
      if (ct2 != 0.0) {
        if (which == 0) v2 = __ldg(ERI + b + N1 * j + N2 * a + N3 * i);  // ERI(b,j,a,i)
        else            v2 = __ldg(ERI + b + N1 * j + N2 * i + N3 * a);  // ERI(b,j,i,a)
      }
    }
    t1[r][tx] = v1;
    t2[r][tx] = v2;
  }
  __syncthreads();
  // write: tx -> a (contiguous in ia), ty -> b
  for (int r = ty; r < TB; r += 8) {
    const int ap = a0 + tx, bp = b0 + r;
    if (ap < nv && bp < nv) {
      double v = ct1 * t1[tx][r] + ct2 * t2[tx][r];
      if (which == 0 && ip == jp && ap == bp) v = (v + e[ap + nO]) - e[i];
      const long long ia = (long long)ip * nv + ap, jb = (long long)jp * nv + bp;
      out[ia + nS * jb] = v;
    }
  }
}

// s_ia = sqrt(fl(A_ii - B_ii)) with A_ii = (2K+e_a)-e_i, B_ii = 2K; trace of A.
__global__ void k_casida_diag(int N, int nC, int nO, int nR, const double* __restrict__ e,
                              const double* __restrict__ ERI, double* __restrict__ sq,
                              double* __restrict__ trA, int* status) {
  __shared__ double red[32];
  const int no = nO - nC, nv = N - nO - nR;
  const int nS = no * nv;
  const long long N1 = N, N2 = N1 * N1, N3 = N2 * N1;
  double tr = 0.0;
  for (int ia = threadIdx.x; ia < nS; ia += blockDim.x) {
    const int ip = ia / nv, ap = ia - ip * nv;
    const long long i = ip + nC, a = ap + nO;
    const double K2 = 2.0 * ERI[a + N1 * i + N2 * i + N3 * a];  // 2*ERI(a,i,i,a)
    const double Aii = (K2 + e[a]) - e[i];
    const double d = Aii - K2;
    if (d < 0.0) atomicOr(status, QKD_NEG_AMB);
    sq[ia] = sqrt(d);
    tr += Aii;
  }
  tr = qk_block_sum(tr, red);
  if (threadIdx.x == 0) *trA = tr;
}

// M(ia,jb) = s_ia * ((A+B)(ia,jb) * s_jb), A+B = 4K off-diagonal, ((2K+e_a)-e_i)+2K on it.
__global__ void __launch_bounds__(TB * 8) k_casida_M(int N, int nC, int nO, int nR,
                                                      const double* __restrict__ e,
                                                      const double* __restrict__ ERI,
                                                      const double* __restrict__ sq,
                                                      double* __restrict__ M) {
  __shared__ double t1[TB][TB + 1];
  const int no = nO - nC, nv = N - nO - nR;
  const long long nS = (long long)no * nv;
  const int ij = blockIdx.z;
  const int ip = ij / no, jp = ij - ip * no;
  const int i = ip + nC, j = jp + nC;
  const int a0 = blockIdx.x * TB, b0 = blockIdx.y * TB;
  const long long N1 = N, N2 = N1 * N1, N3 = N2 * N1;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < TB; r += 8) {
    const int ap = a0 + r, bp = b0 + tx;
    double v = 0.0;
    if (ap < nv && bp < nv) v = __ldg(ERI + (bp + nO) + N1 * i + N2 * j + N3 * (ap + nO));
    t1[r][tx] = v;
  }
  __syncthreads();
  for (int r = ty; r < TB; r += 8) {
    const int ap = a0 + tx, bp = b0 + r;
    if (ap < nv && bp < nv) {
      const double K2 = 2.0 * t1[tx][r];
      double A = K2;
      if (ip == jp && ap == bp) A = (A + e[ap + nO]) - e[i];
      const double ApB = A + K2;
      const long long ia = (long long)ip * nv + ap, jb = (long long)jp * nv + bp;
      M[ia + nS * jb] = sq[ia] * (ApB * sq[jb]);
    }
  }
}

// general A, B given (dRPA-diagonal A-B checked by the caller)
__global__ void k_casida_diag_AB(int nS, const double* __restrict__ A, const double* __restrict__ B,
                                 double* __restrict__ sq, double* __restrict__ trA, int* status) {
  __shared__ double red[32];
  double tr = 0.0;
  for (int ia = threadIdx.x; ia < nS; ia += blockDim.x) {
    const long long d = (long long)ia * nS + ia;
    const double v = A[d] - B[d];
    if (v < 0.0) atomicOr(status, QKD_NEG_AMB);
    sq[ia] = sqrt(v);
    tr += A[d];
  }
  tr = qk_block_sum(tr, red);
  if (threadIdx.x == 0) *trA = tr;
}

__global__ void k_casida_M_AB(int nS, const double* __restrict__ A, const double* __restrict__ B,
                              const double* __restrict__ sq, double* __restrict__ M) {
  const long long total = (long long)nS * nS;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int ia = (int)(idx % nS), jb = (int)(idx / nS);
    M[idx] = sq[ia] * ((A[idx] + B[idx]) * sq[jb]);
  }
}

__global__ void k_xpy(int nS, const double* __restrict__ w, const double* __restrict__ Zt,
                      const double* __restrict__ sq, double* __restrict__ Om,
                      double* __restrict__ XpY, double* __restrict__ XmY, int* status) {
  const long long total = (long long)nS * nS;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(idx % nS), ia = (int)(idx / nS);
    const double om = sqrt(fabs(w[m]));
    const double z = Zt[idx];
    const double s = sq[ia];
    if (XpY) XpY[idx] = (z * s) * (1.0 / sqrt(om));
    if (XmY) XmY[idx] = (z * (1.0 / s)) * sqrt(om);
    if (ia == 0) {
      Om[m] = om;
      if (w[m] < 0.0) atomicOr(status, QKD_NEG_OMEGA);
    }
  }
}

__global__ void k_sum_sqrt(int n, const double* __restrict__ w, double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += sqrt(fabs(w[i]));
  s = qk_block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

// S[pq + N^2*jb] = ERI(p,j,q,b), pq = p + N*q
__global__ void k_slab(int N, int nC, int nO, int nR, const double* __restrict__ ERI,
                       double* __restrict__ S) {
  const int no = nO - nC, nv = N - nO - nR;
  const long long N1 = N, N2 = N1 * N1, N3 = N2 * N1;
  const int jb = blockIdx.y;
  const int jp = jb / nv, bp = jb - jp * nv;
  const long long j = jp + nC, b = bp + nO;
  (void)no;
  const double* src = ERI + N1 * j + N3 * b;
  double* dst = S + N2 * jb;
  for (long long pq = blockIdx.x * (long long)blockDim.x + threadIdx.x; pq < N2;
       pq += (long long)gridDim.x * blockDim.x) {
    const long long q = pq / N1, p = pq - q * N1;
    dst[pq] = __ldg(src + p + N2 * q);
  }
}

// Lov(jb, P) = L(j, b, P): occupied-virtual block of the factor, (nS x naux) column-major
__global__ void k_gather_ov(int N, int nC, int nO, int nR, int naux, const double* __restrict__ L,
                            double* __restrict__ Lov) {
  const int no = nO - nC, nv = N - nO - nR;
  const long long nS = (long long)no * nv;
  const long long N2 = (long long)N * N;
  const long long total = nS * naux;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long P = idx / nS, jb = idx - P * nS;
    const int jp = (int)(jb / nv), bp = (int)(jb - (long long)jp * nv);
    Lov[idx] = __ldg(L + (jp + nC) + (long long)N * (bp + nO) + N2 * P);
  }
}

// diagonal quantities from K = (ia|jb): s_ia = sqrt(fl(A_ii - B_ii)), tr A
__global__ void k_casida_diag_K(int nS, int nv, int nC, int nO, const double* __restrict__ e,
                                const double* __restrict__ K, double* __restrict__ sq,
                                double* __restrict__ trA, int* status) {
  __shared__ double red[32];
  double tr = 0.0;
  for (int ia = threadIdx.x; ia < nS; ia += blockDim.x) {
    const int ip = ia / nv, ap = ia - ip * nv;
    const double K2 = 2.0 * K[(long long)ia * nS + ia];
    const double Aii = (K2 + e[ap + nO]) - e[ip + nC];
    const double d = Aii - K2;
    if (d < 0.0) atomicOr(status, QKD_NEG_AMB);
    sq[ia] = sqrt(d);
    tr += Aii;
  }
  tr = qk_block_sum(tr, red);
  if (threadIdx.x == 0) *trA = tr;
}

// M from the lower triangle of K (so that M is exactly symmetric whatever produced K):
// tiles (bi >= bj) are read once, written to (bi,bj) and transposed to (bj,bi).
__global__ void __launch_bounds__(TB * 8) k_casida_M_K(int nS, int nv, int nC, int nO,
                                                        const double* __restrict__ e,
                                                        const double* __restrict__ K,
                                                        const double* __restrict__ sq,
                                                        double* __restrict__ M) {
  __shared__ double t[TB][TB + 1];
  // linear lower-triangular tile index -> (bi, bj)
  const long long lin = blockIdx.x;
  int bi = (int)((sqrt(8.0 * (double)lin + 1.0) - 1.0) * 0.5);
  while ((long long)(bi + 1) * (bi + 2) / 2 <= lin) ++bi;
  while ((long long)bi * (bi + 1) / 2 > lin) --bi;
  const int bj = (int)(lin - (long long)bi * (bi + 1) / 2);
  const int r0 = bi * TB, c0 = bj * TB;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int r = ty; r < TB; r += 8) {
    const int row = r0 + tx, col = c0 + r;
    double v = 0.0;
    if (row < nS && col < nS) {
      // element (row, col) of the lower triangle (row >= col holds for off-diagonal tiles)
      v = (row >= col) ? K[row + (long long)nS * col] : K[col + (long long)nS * row];
    }
    t[r][tx] = v;  // t[col offset][row offset]
  }
  __syncthreads();
  for (int r = ty; r < TB; r += 8) {
    const int row = r0 + tx, col = c0 + r;
    if (row < nS && col < nS) {
      const double K2 = 2.0 * t[r][tx];
      double A = K2;
      if (row == col) {
        const int ip = row / nv, ap = row - ip * nv;
        A = (A + e[ap + nO]) - e[ip + nC];
      }
      M[row + (long long)nS * col] = sq[row] * ((A + K2) * sq[col]);
    }
    // transposed element (col, row) for the upper triangle: same K value
    const int row2 = c0 + tx, col2 = r0 + r;  // row2 < col2 region
    if (bi != bj && row2 < nS && col2 < nS) {
      const double K2 = 2.0 * t[tx][r];
      M[row2 + (long long)nS * col2] = sq[row2] * ((K2 + K2) * sq[col2]);
    }
  }
}

// Y(r,c) = f(d_r) X(r,c), f: 0 -> d, 1 -> 1/sqrt(|d|) ; rows x cols, column-major
__global__ void k_rowscale2(int rows, int cols, const double* __restrict__ d, int mode,
                            const double* __restrict__ X, long long ldx, double* __restrict__ Y,
                            long long ldy) {
  const long long total = (long long)rows * cols;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i % rows);
    const long long c = i / rows;
    const double f = mode == 0 ? d[r] : 1.0 / sqrt(sqrt(fabs(d[r])));
    Y[r + ldy * c] = f * X[r + ldx * c];
  }
}

__global__ void k_omega(int nS, const double* __restrict__ w, double* __restrict__ Om, int* status) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nS; m += gridDim.x * blockDim.x) {
    Om[m] = sqrt(fabs(w[m]));  // phRLR.f90:76
    if (w[m] < 0.0) atomicOr(status, QKD_NEG_OMEGA);
  }
}

}  // namespace

int qk_launch_omega(qk_ctx* ctx, int nS, const double* w, double* Om) {
  k_omega<<<(nS + 255) / 256, 256, 0, ctx->stream>>>(nS, w, Om, ctx->d_status);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_rowscale(qk_ctx* ctx, int rows, int cols, const double* d, int mode,
                       const double* X, long long ldx, double* Y, long long ldy) {
  const long long total = (long long)rows * cols;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 32 * ctx->num_sms) blocks = 32 * ctx->num_sms;
  if (blocks < 1) blocks = 1;
  k_rowscale2<<<blocks, 256, 0, ctx->stream>>>(rows, cols, d, mode, X, ldx, Y, ldy);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_gather_ov(qk_ctx* ctx, int N, int nC, int nO, int nR, int naux, const double* L,
                        double* Lov) {
  const long long nS = (long long)(nO - nC) * (N - nO - nR);
  int blocks = (int)((nS * naux + 255) / 256);
  if (blocks > 32 * ctx->num_sms) blocks = 32 * ctx->num_sms;
  if (blocks < 1) blocks = 1;
  k_gather_ov<<<blocks, 256, 0, ctx->stream>>>(N, nC, nO, nR, naux, L, Lov);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_casida_M_K(qk_ctx* ctx, int N, int nC, int nO, int nR, const double* e,
                         const double* K, double* M, double* sq, double* trA) {
  const int no = nO - nC, nv = N - nO - nR;
  const int nS = no * nv;
  if (nS <= 0) return QK_OK;
  k_casida_diag_K<<<1, 1024, 0, ctx->stream>>>(nS, nv, nC, nO, e, K, sq, trA, ctx->d_status);
  QK_LAUNCHED();
  const long long nt = (nS + TB - 1) / TB;
  const long long tiles = nt * (nt + 1) / 2;
  k_casida_M_K<<<(unsigned)tiles, dim3(TB, 8), 0, ctx->stream>>>(nS, nv, nC, nO, e, K, sq, M);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_build_AB(qk_ctx* ctx, int which, int ispin, int dRPA, int N, int nC, int nO, int nR,
                       double lambda, const double* e, const double* ERI, double* out) {
  const int no = nO - nC, nv = N - nO - nR;
  if (no <= 0 || nv <= 0) return QK_OK;
  const double delta = dRPA ? 1.0 : 0.0;
  const double ct1 = (ispin == 1) ? 2.0 * lambda : 0.0;
  const double ct2 = -(1.0 - delta) * lambda;
  dim3 grid((nv + TB - 1) / TB, (nv + TB - 1) / TB, no * no);
  if (grid.z > 65535) return qk_fail(ctx, QK_ERR_ARG, "too many occupied pairs");
  k_build_AB<<<grid, dim3(TB, 8), 0, ctx->stream>>>(which, ispin, ct1, ct2, N, nC, nO, nR, e, ERI,
                                                    out);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_casida_M(qk_ctx* ctx, int N, int nC, int nO, int nR, const double* e,
                       const double* ERI, double* M, double* sq, double* trA) {
  const int no = nO - nC, nv = N - nO - nR;
  if (no <= 0 || nv <= 0) return QK_OK;
  k_casida_diag<<<1, 1024, 0, ctx->stream>>>(N, nC, nO, nR, e, ERI, sq, trA, ctx->d_status);
  QK_LAUNCHED();
  dim3 grid((nv + TB - 1) / TB, (nv + TB - 1) / TB, no * no);
  if (grid.z > 65535) return qk_fail(ctx, QK_ERR_ARG, "too many occupied pairs");
  k_casida_M<<<grid, dim3(TB, 8), 0, ctx->stream>>>(N, nC, nO, nR, e, ERI, sq, M);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_casida_M_from_AB(qk_ctx* ctx, int nS, const double* A, const double* B, double* M,
                               double* sq, double* trA) {
  k_casida_diag_AB<<<1, 1024, 0, ctx->stream>>>(nS, A, B, sq, trA, ctx->d_status);
  QK_LAUNCHED();
  const long long total = (long long)nS * nS;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 8 * ctx->num_sms * 8) blocks = 8 * ctx->num_sms * 8;
  k_casida_M_AB<<<blocks, 256, 0, ctx->stream>>>(nS, A, B, sq, M);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_xpy(qk_ctx* ctx, int nS, const double* w, const double* Zt, const double* sq,
                  double* Om, double* XpY, double* XmY, int want_xmy) {
  const long long total = (long long)nS * nS;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 8 * ctx->num_sms * 8) blocks = 8 * ctx->num_sms * 8;
  k_xpy<<<blocks, 256, 0, ctx->stream>>>(nS, w, Zt, sq, Om, XpY, want_xmy ? XmY : nullptr,
                                         ctx->d_status);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_sum_sqrt(qk_ctx* ctx, int nS, const double* w, double* out) {
  k_sum_sqrt<<<1, 1024, 0, ctx->stream>>>(nS, w, out);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_launch_slab_gather(qk_ctx* ctx, int N, int nC, int nO, int nR, const double* ERI,
                          double* S) {
  const int no = nO - nC, nv = N - nO - nR;
  const int nS = no * nv;
  if (nS <= 0) return QK_OK;
  const long long N2 = (long long)N * N;
  int bx = (int)((N2 + 255) / 256);
  if (bx > 64) bx = 64;
  if (nS > 65535) return qk_fail(ctx, QK_ERR_ARG, "nS too large for slab gather grid");
  k_slab<<<dim3(bx, nS), 256, 0, ctx->stream>>>(N, nC, nO, nR, ERI, S);
  QK_LAUNCHED();
  return QK_OK;
}
