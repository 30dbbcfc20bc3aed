// qk_api.cu -- the extern "C" entry points: stage-level drop-ins for the Fortran subroutines of
// the restricted G0W0/evGW call chain and the device-resident drivers.
#include <cmath>
#include <cstring>
#include <vector>
#include <climits>
#include "qk_internal.cuh"

namespace {

struct Dims {
  int N, nC, nO, nR, nS, no, nv;
};

// the drivers' screening form for the duration of one call (the Casida helpers read ctx->tda_w)
struct TdaScope {
  qk_ctx* ctx;
  bool old;
  TdaScope(qk_ctx* c, bool on) : ctx(c), old(c->tda_w) { c->tda_w = on; }
  ~TdaScope() { ctx->tda_w = old; }
};

int check_dims(qk_ctx* ctx, int nBas, int nOrb, int nC, int nO, int nV, int nR, int nS, Dims* d) {
  (void)nV;
  if (nBas != nOrb)
    return qk_fail(ctx, QK_ERR_ARG, "nBas (%d) != nOrb (%d): the restricted GW path dimensions "
                   "its arrays with nBas and nOrb interchangeably (RGW_self_energy_diag.f90:22-27)",
                   nBas, nOrb);
  const int N = nOrb;
  const int no = nO - nC, nv = N - nO - nR;
  if (N <= 0 || nC < 0 || nR < 0 || no <= 0 || nv <= 0)
    return qk_fail(ctx, QK_ERR_ARG, "invalid orbital partition N=%d nC=%d nO=%d nR=%d", N, nC, nO, nR);
  if ((long long)no * nv != nS)
    return qk_fail(ctx, QK_ERR_ARG, "nS=%d does not equal (nO-nC)*(nOrb-nO-nR)=%lld", nS,
                   (long long)no * nv);
  d->N = N; d->nC = nC; d->nO = nO; d->nR = nR; d->nS = nS; d->no = no; d->nv = nv;
  return QK_OK;
}

int h2d(qk_ctx* ctx, void* dst, const void* src, size_t bytes) {
  QK_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return QK_OK;
}
// Upload only the part of ERI(p,q,r,s) the G0W0/evGW drivers read: q occupied (active), s
// virtual (active), all p and r -- the excitation-density slab ERI(p,j,q,b), which contains the
// Casida block ERI(b,i,j,a) as well.  For fixed (r, s) the entries with q in the occupied range
// and any p are one contiguous run of no*N doubles, so each virtual s is one 2D copy of N such
// runs; the other entries of the device tensor are never read.  At N=200, nO=20 that is
// 1.15 GB instead of 12.8.
int h2d_eri_used(qk_ctx* ctx, double* dERI, const double* hERI, const Dims& d) {
  const size_t N = d.N, N2 = N * N, N3 = N2 * N;
  const size_t run = (size_t)(d.nO - d.nC) * N * sizeof(double);
  for (int s = d.nO; s < d.N - d.nR; ++s) {
    const size_t off = N3 * s + N * d.nC;
    QK_CK(cudaMemcpy2DAsync(dERI + off, N2 * sizeof(double), hERI + off, N2 * sizeof(double), run,
                            N, cudaMemcpyHostToDevice, ctx->stream));
  }
  return QK_OK;
}

// The same block in two parts for the G0W0 driver: the rows r of the Casida matrix's sub-block
// ERI(b,i,j,a) (r = j occupied, 1/N of the bytes per occupied row) on the compute stream, the
// other rows -- only the excitation-density slab reads them -- on the copy stream, where they
// overlap with the Casida eigensolve; the slab gather waits for ctx->ev_copy.
int h2d_eri_split(qk_ctx* ctx, double* dERI, const double* hERI, const Dims& d) {
  if (!ctx->copy_stream) {
    QK_CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    QK_CK(cudaEventCreateWithFlags(&ctx->ev_copy, cudaEventDisableTiming));
  }
  const size_t N = d.N, N2 = N * N, N3 = N2 * N;
  const size_t run = (size_t)(d.nO - d.nC) * N * sizeof(double);
  for (int s = d.nO; s < d.N - d.nR; ++s) {
    const size_t off = N3 * s + N * d.nC + N2 * d.nC;
    QK_CK(cudaMemcpy2DAsync(dERI + off, N2 * sizeof(double), hERI + off, N2 * sizeof(double), run,
                            d.nO - d.nC, cudaMemcpyHostToDevice, ctx->stream));
  }
  // the copy stream starts after the compute stream's earlier work (which may read dERI)
  QK_CK(cudaEventRecord(ctx->ev_copy, ctx->stream));
  QK_CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_copy, 0));
  for (int s = d.nO; s < d.N - d.nR; ++s) {
    const size_t base = N3 * s + N * d.nC;
    if (d.nC > 0)
      QK_CK(cudaMemcpy2DAsync(dERI + base, N2 * sizeof(double), hERI + base, N2 * sizeof(double),
                              run, d.nC, cudaMemcpyHostToDevice, ctx->copy_stream));
    const size_t off = base + N2 * d.nO;
    QK_CK(cudaMemcpy2DAsync(dERI + off, N2 * sizeof(double), hERI + off, N2 * sizeof(double), run,
                            d.N - d.nO, cudaMemcpyHostToDevice, ctx->copy_stream));
  }
  QK_CK(cudaEventRecord(ctx->ev_copy, ctx->copy_stream));
  ctx->eri_pending = true;
  return QK_OK;
}

int d2h(qk_ctx* ctx, void* dst, const void* src, size_t bytes) {
  QK_CK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  return QK_OK;
}

// small elementwise helpers used by the general (non-diagonal A-B) Casida path
__global__ void k_axpby(long long n, double a, const double* __restrict__ x, double b,
                        const double* __restrict__ y, double* __restrict__ z) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    z[i] = a * x[i] + b * y[i];
}
// rows of X (n x n, column-major) scaled: X(r,c) *= f(d[r]); mode 0: sqrt, 1: 1/sqrt, 2: identity
__global__ void k_rowscale(int n, const double* __restrict__ d, int mode, const double* __restrict__ X,
                           double* __restrict__ Y) {
  const long long total = (long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i % n);
    double f = d[r];
    if (mode == 0) f = 1.0 * sqrt(f);
    else if (mode == 1) f = 1.0 / sqrt(f);
    Y[i] = f * X[i];
  }
}
__global__ void k_offdiag_maxabs(int n, const double* __restrict__ A, const double* __restrict__ B,
                                 double* out) {
  double m = 0.0;
  const long long total = (long long)n * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i % n), c = (int)(i / n);
    if (r != c) m = fmax(m, fabs(A[i] - B[i]));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0) {
    // non-negative doubles order like their bit patterns
    atomicMax((unsigned long long*)out, (unsigned long long)__double_as_longlong(m));
  }
}
__global__ void k_trace(int n, const double* __restrict__ A, double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += A[(long long)i * n + i];
  s = qk_block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}
// dRPA singlet A = Delta + 2K from K = (ia|jb) (phRLR_A.f90:43-72, evaluation order (2K + e_a) - e_i)
__global__ void k_build_A_from_K(int nS, int nv, int nC, int nO, const double* __restrict__ e,
                                 const double* __restrict__ K, double* __restrict__ A) {
  const long long total = (long long)nS * nS;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i % nS), c = (int)(i / nS);
    double v = 2.0 * K[i];
    if (r == c) {
      const int ip = r / nv, ap = r - ip * nv;
      v = (v + e[ap + nO]) - e[ip + nC];
    }
    A[i] = v;
  }
}
__global__ void k_vsum_om(int n, const double* __restrict__ w, double* __restrict__ Om,
                          double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    s += w[i];
    if (Om) Om[i] = w[i];
  }
  s = qk_block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}
__global__ void k_xpy_general(int nS, const double* __restrict__ w, double* __restrict__ Om,
                              double* __restrict__ XpY, double* __restrict__ XmY, int* status) {
  const long long total = (long long)nS * nS;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(i % nS);
    const double om = sqrt(fabs(w[m]));
    XpY[i] *= 1.0 / sqrt(om);
    XmY[i] *= 1.0 * sqrt(om);
    if (i < nS) {
      Om[m] = om;
      if (w[m] < 0.0) atomicOr(status, QKD_NEG_OMEGA);
    }
  }
}
__global__ void k_ecrpa(const double* sumOm, const double* trA, double* out) {
  *out = 0.5 * (*sumOm - *trA);
}

int grid_for(qk_ctx* ctx, long long total) {
  long long b = (total + 255) / 256;
  const long long cap = 64LL * ctx->num_sms;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// the excitation density rho = slab * XpY^T for the chosen precision tier
int rho_gemm(qk_ctx* ctx, int prec, int N, int nS, const double* S, const double* XpY, double* rho) {
  const long long N2 = (long long)N * N;
  if (prec == QK_PREC_BF16X3)
    return qk_gemm_bf16x3_nt(ctx, (int)N2, nS, nS, S, N2, XpY, nS, rho, N2);
  return qk_dgemm(ctx, 'N', 'T', (int)N2, nS, nS, 1.0, S, N2, 0, XpY, nS, 0, 0.0, rho, N2, 0, 1);
}

// contractions of the factorised integrals:
//   Lov(jb,P) = L(j,b,P);  K = Lov Lov^T = (ia|jb)  (always FP64: the Casida matrix stays exact)
int factor_prep(qk_ctx* ctx, const Dims& d, int naux, const double* L, double** K_out,
                double** Lov_out) {
  const int N = d.N, nS = d.nS;
  double *Lov, *K;
  QK_TRY(qk_wst(ctx, W_VEC2, (size_t)nS * naux, &Lov));
  QK_TRY(qk_wst(ctx, W_KMAT, (size_t)nS * nS, &K));
  qk_tic(ctx, T_SLAB);
  QK_TRY(qk_launch_gather_ov(ctx, N, d.nC, d.nO, d.nR, naux, L, Lov));
  QK_TRY(qk_dgemm(ctx, 'N', 'T', nS, nS, naux, 1.0, Lov, nS, 0, Lov, nS, 0, 0.0, K, nS, 0, 1));
  qk_toc(ctx, T_SLAB);
  *K_out = K;
  *Lov_out = Lov;
  return QK_OK;
}

// Excitation densities through the factor (RGW_excitation_density.f90:48-50 re-associated):
//   rho(pq,m) = sum_jb (pq|jb) XpY(m,jb) = sum_P L(pq,P) T(m,P),   T = XpY Lov  (nS x naux)
// and, with XpY = D_Om^-1/2 Z_M^T D_s and Z_M = Q Z_T (Householder Q, tridiagonal vectors Z_T):
//   T = D_Om^-1/2 Z_T^T (Q^T (D_s Lov)),
// so the eigenvectors of M are never back-transformed: Q^T is applied to the nS x naux factor
// (2 nS^2 naux flops instead of 2 nS^3) -- the same numbers in another order, with FP64
// products (FP32 products in the mixed tier, whose excitation densities are BF16x3).
int casida_factored(qk_ctx* ctx, int prec, const Dims& d, const double* e, const double* K,
                    const double* Lov, int naux, double* Om, double* T, double* scal) {
  const int nS = d.nS;
  const size_t S2 = (size_t)nS * nS;
  double *M = nullptr, *Zt = nullptr, *sq = nullptr, *X = nullptr;
  QK_TRY(qk_wst(ctx, W_M, S2, &M));
  QK_TRY(qk_wst(ctx, W_E, 2 * (size_t)nS + 64, &sq));
  QK_TRY(qk_wst(ctx, W_ZT, S2, &Zt));
  QK_TRY(qk_wst(ctx, W_TMAT2, (size_t)nS * naux, &X));
  double* w = sq + nS;
  const int f32 = prec == QK_PREC_BF16X3;  // mixed tier: FP32 products, FP64 storage
  if (ctx->tda_w) {
    // Tamm-Dancoff screening (phRLR.f90 with TDA): Om = eig(A), XpY = Z^T = Z_T^T Q^T, so
    // T = Z_T^T (Q^T Lov)
    qk_tic(ctx, T_BUILD);
    k_build_A_from_K<<<grid_for(ctx, (long long)nS * nS), 256, 0, ctx->stream>>>(
        nS, d.nv, d.nC, d.nO, e, K, M);
    QK_LAUNCHED();
    k_trace<<<1, 1024, 0, ctx->stream>>>(nS, M, scal + 0);
    QK_LAUNCHED();
    qk_toc(ctx, T_BUILD);
    QK_TRY(qk_eig_sym(ctx, nS, M, nS, w, Zt, 1, 0, f32));
    qk_tic(ctx, T_BACKTRANS);
    QK_CK(cudaMemcpyAsync(X, Lov, (size_t)nS * naux * sizeof(double), cudaMemcpyDeviceToDevice,
                          ctx->stream));
    QK_TRY(qk_eig_apply_qt(ctx, nS, X, nS, naux, f32));
    QK_TRY((f32 ? qk_gemm_f32p : qk_dgemm)(ctx, 'N', 'N', nS, naux, nS, 1.0, Zt, nS, 0, X, nS, 0,
                                           0.0, T, nS, 0, 1));
    qk_toc(ctx, T_BACKTRANS);
    k_vsum_om<<<1, 1024, 0, ctx->stream>>>(nS, w, Om, scal + 1);
    QK_LAUNCHED();
    k_ecrpa<<<1, 1, 0, ctx->stream>>>(scal + 1, scal + 0, scal + 2);
    QK_LAUNCHED();
    return QK_OK;
  }
  qk_tic(ctx, T_BUILD);
  QK_TRY(qk_launch_casida_M_K(ctx, d.N, d.nC, d.nO, d.nR, e, K, M, sq, scal + 0));
  qk_toc(ctx, T_BUILD);
  QK_TRY(qk_eig_sym(ctx, nS, M, nS, w, Zt, 1, 0, f32));
  QK_TRY(qk_launch_omega(ctx, nS, w, Om));
  qk_tic(ctx, T_BACKTRANS);
  QK_TRY(qk_launch_rowscale(ctx, nS, naux, sq, 0, Lov, nS, X, nS));           // D_s Lov
  QK_TRY(qk_eig_apply_qt(ctx, nS, X, nS, naux, f32));                        // Q^T (.)
  QK_TRY((f32 ? qk_gemm_f32p : qk_dgemm)(ctx, 'N', 'N', nS, naux, nS, 1.0, Zt, nS, 0, X, nS, 0,
                                         0.0, T, nS, 0, 1));
  QK_TRY(qk_launch_rowscale(ctx, nS, naux, w, 1, T, nS, T, nS));             // D_Om^-1/2
  qk_toc(ctx, T_BACKTRANS);
  QK_TRY(qk_launch_sum_sqrt(ctx, nS, w, scal + 1));
  k_ecrpa<<<1, 1, 0, ctx->stream>>>(scal + 1, scal + 0, scal + 2);
  QK_LAUNCHED();
  return QK_OK;
}

// rho(pq,m) = sum_P L(pq,P) T(m,P) in the precision tier
int rho_from_T(qk_ctx* ctx, int prec, const Dims& d, int naux, const double* L, const double* T,
               double* rho) {
  const int N = d.N, nS = d.nS;
  const long long N2 = (long long)N * N;
  if (prec == QK_PREC_BF16X3)
    return qk_gemm_bf16x3_nt(ctx, (int)N2, nS, naux, L, N2, T, nS, rho, N2);
  return qk_dgemm(ctx, 'N', 'T', (int)N2, nS, naux, 1.0, L, N2, 0, T, nS, 0, 0.0, rho, N2, 0, 1);
}

// Casida with eigenvectors for the dRPA singlet screening at energies e.
// Outputs: Om (nS), XpY (nS*nS), optional XmY, sumOm/trA (device scalars) for EcRPA.
int casida_dev(qk_ctx* ctx, const Dims& d, const double* e, const double* ERI, double* Om,
               double* XpY, double* XmY, double* scal /* [0]=trA [1]=sumOm [2]=EcRPA */,
               int want_vectors, const double* K = nullptr, int prec = QK_PREC_FP64) {
  const size_t S2 = (size_t)d.nS * d.nS;
  double *M = nullptr, *Zt = nullptr, *sq = nullptr;
  QK_TRY(qk_wst(ctx, W_M, S2, &M));
  QK_TRY(qk_wst(ctx, W_E, 2 * (size_t)d.nS + 64, &sq));
  double* w = sq + d.nS;
  if (ctx->tda_w) {
    // Tamm-Dancoff screening (phRLR.f90 with TDA): Om = eig(A), XpY = XmY = eigenvectors as rows
    qk_tic(ctx, T_BUILD);
    if (K) {
      k_build_A_from_K<<<grid_for(ctx, (long long)S2), 256, 0, ctx->stream>>>(d.nS, d.nv, d.nC,
                                                                               d.nO, e, K, M);
      QK_LAUNCHED();
    } else {
      QK_TRY(qk_launch_build_AB(ctx, 0, 1, 1, d.N, d.nC, d.nO, d.nR, 1.0, e, ERI, M));
    }
    k_trace<<<1, 1024, 0, ctx->stream>>>(d.nS, M, scal + 0);
    QK_LAUNCHED();
    qk_toc(ctx, T_BUILD);
    ctx->time_eig = want_vectors != 0;
    const int est = qk_eig_sym(ctx, d.nS, M, d.nS, w, want_vectors ? XpY : nullptr, want_vectors,
                               prec == QK_PREC_BF16X3 ? 2 : 1, prec == QK_PREC_BF16X3);
    ctx->time_eig = true;
    QK_TRY(est);
    if (want_vectors && XmY)
      QK_CK(cudaMemcpyAsync(XmY, XpY, S2 * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    k_vsum_om<<<1, 1024, 0, ctx->stream>>>(d.nS, w, Om, scal + 1);
    QK_LAUNCHED();
    k_ecrpa<<<1, 1, 0, ctx->stream>>>(scal + 1, scal + 0, scal + 2);
    QK_LAUNCHED();
    return QK_OK;
  }
  qk_tic(ctx, T_BUILD);
  if (K)
    QK_TRY(qk_launch_casida_M_K(ctx, d.N, d.nC, d.nO, d.nR, e, K, M, sq, scal + 0));
  else
    QK_TRY(qk_launch_casida_M(ctx, d.N, d.nC, d.nO, d.nR, e, ERI, M, sq, scal + 0));
  qk_toc(ctx, T_BUILD);
  if (want_vectors) QK_TRY(qk_wst(ctx, W_ZT, S2, &Zt));
  ctx->time_eig = want_vectors != 0;
  // the mixed tier tridiagonalises in double-float on the FP32 pipe and back-transforms the
  // eigenvectors with FP32 products (they feed the BF16x3 excitation densities); the tridiagonal
  // eigenproblem, and so Om and EcRPA, is FP64 in every tier
  const int est = qk_eig_sym(ctx, d.nS, M, d.nS, w, Zt, want_vectors,
                             prec == QK_PREC_BF16X3 ? 2 : 1, prec == QK_PREC_BF16X3);
  ctx->time_eig = true;
  QK_TRY(est);
  if (want_vectors) QK_TRY(qk_launch_xpy(ctx, d.nS, w, Zt, sq, Om, XpY, XmY, XmY != nullptr));
  QK_TRY(qk_launch_sum_sqrt(ctx, d.nS, w, scal + 1));
  k_ecrpa<<<1, 1, 0, ctx->stream>>>(scal + 1, scal + 0, scal + 2);
  QK_LAUNCHED();
  return QK_OK;
}

// The mixed tier evaluates the pole sums with FP32 far-pole terms (eta = 0 and no SRG only;
// otherwise, and in the FP64 tier, every term is FP64).
int sigma_tier(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, const double* rho,
               const double* Om, qk_sigma_ff* ff, const qk_sigma_ff** use) {
  *use = nullptr;
  if (prm->precision != QK_PREC_BF16X3 || prm->eta != 0.0 || prm->doSRG) return QK_OK;
  QK_TRY(qk_sigma_ff_prep(ctx, d.N, d.nS, rho, Om, ff));
  *use = ff;
  return QK_OK;
}

// Newton QP of RG0W0 (reference start eGWlin) or, with prm->qp_guess, from the learned guess (1)
// or from eHF (2, a comparison baseline); captures the per-orbital features when requested.
int g0w0_qp(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, double flow, const double* eHF,
            const double* Om, const double* rho, const double* SigC, double* Z,
            const double* eGWlin, double* eGW, const qk_sigma_ff* ff) {
  const int N = d.N, nS = d.nS;
  float* F = nullptr;
  double* gbuf = nullptr;  // [0, N): start; [N, 2N): Halley step; then N ints: fromref
  const bool need_f = ctx->capture_features || prm->qp_guess == 1;
  if (need_f) {
    QK_TRY(qk_wst(ctx, W_FEAT, (size_t)N * QK_MLP_NIN + 16, &F));
    QK_TRY(qk_wst(ctx, W_GUESS, (size_t)3 * N + 16, &gbuf));
    QK_TRY(qk_features(ctx, N, d.nC, d.nO, d.nR, nS, eHF, eGWlin, Om, rho, SigC, Z, F, gbuf + N));
    if (ctx->capture_features) {
      ctx->features.resize((size_t)N * QK_MLP_NIN);
      QK_CK(cudaMemcpyAsync(ctx->features.data(), F, sizeof(float) * N * QK_MLP_NIN,
                            cudaMemcpyDeviceToHost, ctx->stream));
      QK_CK(cudaStreamSynchronize(ctx->stream));
    }
  }
  double* w0 = nullptr;
  int* fromref = nullptr;
  if (prm->qp_guess == 1 && !prm->linearize) {
    w0 = gbuf;
    fromref = (int*)(gbuf + 2 * N);
    QK_TRY(qk_guess_from_model(ctx, N, F, eGWlin, gbuf + N, w0, fromref));
  }
  if (prm->qp_guess == 2 && !prm->linearize) {
    // comparison start: the HF energies, same 8-step protocol as the learned guess
    QK_TRY(qk_wst(ctx, W_GUESS, (size_t)3 * N + 16, &gbuf));
    w0 = gbuf;
    QK_CK(cudaMemcpyAsync(w0, eHF, N * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  }
  if (prm->linearize) {
    QK_CK(cudaMemcpyAsync(eGW, eGWlin, N * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    return QK_OK;
  }
  return qk_qp_newton(ctx, prm->doSRG, prm->eta, flow, N, d.nC, d.nO, d.nR, nS, eHF, Om, rho,
                      eGWlin, eHF, eGW, Z, w0, 8, ff, fromref);
}

int g0w0_dev(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, const double* eHF,
             const double* ERI, double* eGW, double* SigC, double* Z, double* Om, double* hEcRPA,
             double* hEcGM) {
  TdaScope tda(ctx, prm->TDA_W != 0);
  const double flow = 500.0;  // RG0W0.f90:98
  const int N = d.N, nS = d.nS;
  const size_t S2 = (size_t)nS * nS, N2S = (size_t)N * N * nS;
  double *XpY, *slab, *rho, *scal, *eGWlin;
  QK_TRY(qk_wst(ctx, W_XPY, S2, &XpY));
  QK_TRY(qk_wst(ctx, W_SLAB, N2S, &slab));
  QK_TRY(qk_wst(ctx, W_RHO, N2S, &rho));
  double* small = nullptr;
  QK_TRY(qk_wst(ctx, W_HOST_B, (size_t)2 * N + 16, &small));
  scal = small;
  eGWlin = small + 16;
  double* EcGM_d = scal + 8;
  qk_timings_clear(ctx);
  // screening at eHF
  QK_TRY(casida_dev(ctx, d, eHF, ERI, Om, XpY, nullptr, scal, 1, nullptr, prm->precision));
  // excitation densities (the slab reads rows of ERI that may still be arriving)
  if (ctx->eri_pending) {
    QK_CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_copy, 0));
    ctx->eri_pending = false;
  }
  qk_tic(ctx, T_SLAB);
  QK_TRY(qk_launch_slab_gather(ctx, N, d.nC, d.nO, d.nR, ERI, slab));
  qk_toc(ctx, T_SLAB);
  qk_tic(ctx, T_RHO);
  QK_TRY(rho_gemm(ctx, prm->precision, N, nS, slab, XpY, rho));
  qk_toc(ctx, T_RHO);
  // self-energy
  qk_tic(ctx, T_SIGMA);
  qk_sigma_ff ff;
  const qk_sigma_ff* ffp = nullptr;
  QK_TRY(sigma_tier(ctx, prm, d, rho, Om, &ff, &ffp));
  QK_TRY(qk_sigma_diag(ctx, prm->doSRG, prm->eta, flow, N, d.nC, d.nO, d.nR, nS, eHF, Om, rho, SigC,
                       Z, EcGM_d, ffp));
  QK_TRY(qk_qp_linear(ctx, N, eHF, Z, SigC, 1, eGWlin));
  qk_toc(ctx, T_SIGMA);
  qk_tic(ctx, T_QP);
  QK_TRY(g0w0_qp(ctx, prm, d, flow, eHF, Om, rho, SigC, Z, eGWlin, eGW, ffp));
  qk_toc(ctx, T_QP);
  // second Casida at eGW for EcRPA (RG0W0.f90:222-225): eigenvalues only; the mixed tier
  // takes the frequency quadrature of the same energy (r x r problems instead of nS x nS).
  // Both tiers first check the QP gap: a virtual level below an occupied one makes A - B
  // indefinite and the energy NaN (phRLR's square roots), which needs no eigenproblem.
  qk_tic(ctx, T_CASIDA2);
  int quad = 0;
  if (!prm->TDA_W)  // (with TDA screening A - B plays no part: no square roots, no quadrature)
    QK_TRY(qk_rpa_ec_quad(ctx, N, d.nC, d.nO, d.nR, eGW, ERI, nullptr, 0, scal + 5, &quad,
                          prm->precision != QK_PREC_BF16X3));
  if (!quad) QK_TRY(casida_dev(ctx, d, eGW, ERI, nullptr, nullptr, nullptr, scal + 3, 0));
  qk_toc(ctx, T_CASIDA2);
  double h[16];
  QK_TRY(d2h(ctx, h, scal, 16 * sizeof(double)));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  qk_timings_collect(ctx);
  if (hEcRPA) *hEcRPA = h[5];
  if (hEcGM) *hEcGM = h[8];
  return QK_OK;
}

// ---------------------------------------------------------------------------------------------
// evGW cycle (evRGW.f90:119-180) without host synchronisation, so that it can be enqueued
// eagerly or captured once into a CUDA graph and replayed by a device-side WHILE loop.
// dstate (device ints): [0] nSCF, [1] n_diis, [2] continue flag.  scal[9] = Conv.
// ---------------------------------------------------------------------------------------------
__global__ void k_diis_count(int* st, int max_diis) {
  st[1] = st[1] + 1 < max_diis ? st[1] + 1 : max_diis;
}

__global__ void k_cycle_end(int* st, const double* conv, double thresh, int maxSCF,
                            cudaGraphConditionalHandle h, int use_handle) {
  st[0] += 1;
  const int cont = (*conv > thresh) && (st[0] <= maxSCF);  // evRGW.f90:119
  st[2] = cont;
  if (use_handle) cudaGraphSetConditional(h, cont ? 1u : 0u);
}

struct EvBufs {
  const double* ERI;   // full-ERI path (or nullptr)
  const double* K;     // factorised path (or nullptr)
  const double* slab;  // full-ERI path: (pq|jb)
  const double* eHF;
  double *eGW, *eOld, *SigC, *Z, *Om, *XpY, *rho, *scal, *errv, *err_hist, *e_hist;
  int* dstate;
  const double* L = nullptr;    // factorised path: L(pq,P) and Lov(jb,P)
  const double* Lov = nullptr;
  int naux = 0;
};

int evgw_cycle(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, const EvBufs& b,
               cudaGraphConditionalHandle h, int use_handle) {
  const double flow = 500.0;
  const int N = d.N, nS = d.nS;
  if (b.L) {
    double* T = nullptr;
    QK_TRY(qk_wst(ctx, W_TMAT, (size_t)nS * b.naux, &T));
    QK_TRY(casida_factored(ctx, prm->precision, d, b.eGW, b.K, b.Lov, b.naux, b.Om, T, b.scal));
    qk_tic(ctx, T_RHO);
    QK_TRY(rho_from_T(ctx, prm->precision, d, b.naux, b.L, T, b.rho));
    qk_toc(ctx, T_RHO);
  } else {
    QK_TRY(casida_dev(ctx, d, b.eGW, b.ERI, b.Om, b.XpY, nullptr, b.scal, 1, b.K, prm->precision));
    qk_tic(ctx, T_RHO);
    QK_TRY(rho_gemm(ctx, prm->precision, N, nS, b.slab, b.XpY, b.rho));
    qk_toc(ctx, T_RHO);
  }
  qk_tic(ctx, T_SIGMA);
  qk_sigma_ff ff;
  const qk_sigma_ff* ffp = nullptr;
  QK_TRY(sigma_tier(ctx, prm, d, b.rho, b.Om, &ff, &ffp));
  QK_TRY(qk_sigma_diag(ctx, prm->doSRG, prm->eta, flow, N, d.nC, d.nO, d.nR, nS, b.eGW, b.Om,
                       b.rho, b.SigC, b.Z, b.scal + 8, ffp));
  qk_toc(ctx, T_SIGMA);
  qk_tic(ctx, T_QP);
  if (prm->linearize) {
    QK_TRY(qk_qp_linear(ctx, N, b.eHF, b.Z, b.SigC, 0, b.eGW));  // evRGW.f90:147
  } else {
    QK_TRY(qk_qp_newton(ctx, prm->doSRG, prm->eta, flow, N, d.nC, d.nO, d.nR, nS, b.eHF, b.Om,
                        b.rho, b.eOld, b.eOld, b.eGW, b.Z, nullptr, 8, ffp));  // evRGW.f90:154
  }
  qk_toc(ctx, T_QP);
  QK_TRY(qk_max_abs_diff(ctx, N, b.eGW, b.eOld, b.scal + 9));  // evRGW.f90:160
  if (prm->max_diis > 1) {  // evRGW.f90:166-171
    k_diis_count<<<1, 1, 0, ctx->stream>>>(b.dstate, prm->max_diis);
    QK_LAUNCHED();
    QK_TRY(qk_sub(ctx, N, b.eGW, b.eOld, b.errv));
    QK_TRY(qk_diis_dev(ctx, N, N, prm->max_diis, b.err_hist, b.e_hist, b.errv, b.eGW, b.scal + 10,
                       b.dstate + 1));
  }
  QK_CK(cudaMemcpyAsync(b.eOld, b.eGW, N * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  k_cycle_end<<<1, 1, 0, ctx->stream>>>(b.dstate, b.scal + 9, prm->thresh, prm->maxSCF, h, use_handle);
  QK_LAUNCHED();
  return QK_OK;
}

// Build (or reuse) a graph whose WHILE node replays evgw_cycle until the device flag drops.
int evgw_graph_run(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, const EvBufs& b) {
  std::vector<long long> key = {(long long)d.N, d.nC, d.nO, d.nR, prm->precision, prm->linearize,
                                prm->doSRG, prm->max_diis, prm->maxSCF,
                                (long long)(prm->thresh * 1e15), (long long)(prm->eta * 1e15),
                                (long long)b.ERI, (long long)b.K, (long long)b.slab,
                                (long long)b.eHF, (long long)b.eGW, (long long)b.dstate,
                                (long long)b.L, (long long)b.naux, prm->TDA_W};
  if (!ctx->evgw_exec || ctx->evgw_key != key) {
    if (ctx->evgw_exec) {
      cudaGraphExecDestroy(ctx->evgw_exec);
      ctx->evgw_exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    QK_CK(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle h;
    QK_CK(cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    QK_CK(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    QK_CK(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0,
                                        cudaStreamCaptureModeRelaxed));
    ctx->capturing = true;
    const int st = evgw_cycle(ctx, prm, d, b, h, 1);
    ctx->capturing = false;
    cudaGraph_t captured = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &captured);
    if (st != QK_OK) {
      cudaGraphDestroy(graph);
      return st;
    }
    QK_CK(ec);
    cudaGraphExec_t exec = nullptr;
    const cudaError_t ei = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    QK_CK(ei);
    ctx->evgw_exec = exec;
    ctx->evgw_key = key;
  }
  QK_CK(cudaGraphLaunch(ctx->evgw_exec, ctx->stream));
  return QK_OK;
}

// cycles of evGW: the first eagerly (it sizes every workspace), the rest either eagerly or from
// the graph; returns nSCF and Conv read back from the device
int evgw_loop(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, const EvBufs& b, int* hnSCF,
              double* hConv) {
  QK_CK(cudaMemsetAsync(b.dstate, 0, 4 * sizeof(int), ctx->stream));
  cudaGraphConditionalHandle none = 0;
  int hst[4] = {0, 0, 1, 0};
  double conv = 1.0;
  QK_TRY(evgw_cycle(ctx, prm, d, b, none, 0));
  QK_CK(cudaMemcpyAsync(hst, b.dstate, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QK_CK(cudaMemcpyAsync(&conv, b.scal + 9, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  if (hst[2]) {
    if (ctx->graph_mode) {
      QK_TRY(evgw_graph_run(ctx, prm, d, b));
    } else {
      while (hst[2]) {
        QK_TRY(evgw_cycle(ctx, prm, d, b, none, 0));
        QK_CK(cudaMemcpyAsync(hst, b.dstate, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        QK_CK(cudaStreamSynchronize(ctx->stream));
      }
    }
    QK_CK(cudaMemcpyAsync(hst, b.dstate, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QK_CK(cudaMemcpyAsync(&conv, b.scal + 9, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QK_CK(cudaStreamSynchronize(ctx->stream));
  }
  *hnSCF = hst[0];
  *hConv = conv;
  return QK_OK;
}

int evgw_dev(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, const double* eHF,
             const double* ERI, double* eGW, double* SigC, double* Z, double* hEcRPA,
             double* hEcGM, int* hnSCF, double* hConv) {
  TdaScope tda(ctx, prm->TDA_W != 0);
  const int N = d.N, nS = d.nS;
  const size_t S2 = (size_t)nS * nS, N2S = (size_t)N * N * nS;
  const int maxd = prm->max_diis > 1 ? prm->max_diis : 1;
  double *XpY, *slab, *rho, *small;
  QK_TRY(qk_wst(ctx, W_XPY, S2, &XpY));
  QK_TRY(qk_wst(ctx, W_SLAB, N2S, &slab));
  QK_TRY(qk_wst(ctx, W_RHO, N2S, &rho));
  QK_TRY(qk_wst(ctx, W_HOST_B, (size_t)(6 + 2 * maxd) * N + nS + 64 + 8, &small));
  double* scal = small;            // [0]=trA [1]=sumOm [2]=EcRPA [8]=EcGM [9]=Conv [10]=rcond
  double* eOld = small + 64;
  double* errv = eOld + N;
  double* Om = errv + N;
  double* err_hist = Om + nS;
  double* e_hist = err_hist + (size_t)N * maxd;
  int* dstate = (int*)(e_hist + (size_t)N * maxd);
  QK_CK(cudaMemsetAsync(err_hist, 0, sizeof(double) * 2 * (size_t)N * maxd, ctx->stream));
  QK_CK(cudaMemcpyAsync(eGW, eHF, N * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  QK_CK(cudaMemcpyAsync(eOld, eHF, N * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  qk_timings_clear(ctx);
  // the slab of (pq|jb) does not depend on the energies: gather it once
  qk_tic(ctx, T_SLAB);
  QK_TRY(qk_launch_slab_gather(ctx, N, d.nC, d.nO, d.nR, ERI, slab));
  qk_toc(ctx, T_SLAB);
  EvBufs bb{ERI, nullptr, slab, eHF, eGW, eOld, SigC, Z, Om, XpY, rho, scal, errv,
            err_hist, e_hist, dstate};
  int nSCF = 0;
  double Conv = 1.0;
  QK_TRY(evgw_loop(ctx, prm, d, bb, &nSCF, &Conv));
  double h[16];
  QK_TRY(d2h(ctx, h, scal, 16 * sizeof(double)));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  qk_timings_collect(ctx);
  if (hEcRPA) *hEcRPA = h[2];
  if (hEcGM) *hEcGM = h[8];
  if (hnSCF) *hnSCF = nSCF;
  if (hConv) *hConv = Conv;
  if (nSCF == prm->maxSCF + 1)  // evRGW.f90:190-198
    return qk_fail(ctx, QK_ERR_NO_CONV, "evGW convergence failed after %d cycles (Conv=%g)", nSCF, Conv);
  return QK_OK;
}

int g0w0_L_dev(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, int naux, const double* L,
               const double* eHF, double* eGW, double* SigC, double* Z, double* Om,
               double* hEcRPA, double* hEcGM) {
  TdaScope tda(ctx, prm->TDA_W != 0);
  const double flow = 500.0;
  const int N = d.N, nS = d.nS;
  const size_t N2S = (size_t)N * N * nS;
  double *rho, *small, *K, *Lov;
  qk_timings_clear(ctx);
  QK_TRY(factor_prep(ctx, d, naux, L, &K, &Lov));
  QK_TRY(qk_wst(ctx, W_RHO, N2S, &rho));
  QK_TRY(qk_wst(ctx, W_HOST_B, (size_t)2 * N + 16, &small));
  double* scal = small;
  double* eGWlin = small + 16;
  double* T = nullptr;
  QK_TRY(qk_wst(ctx, W_TMAT, (size_t)nS * naux, &T));
  QK_TRY(casida_factored(ctx, prm->precision, d, eHF, K, Lov, naux, Om, T, scal));
  qk_tic(ctx, T_RHO);
  QK_TRY(rho_from_T(ctx, prm->precision, d, naux, L, T, rho));
  qk_toc(ctx, T_RHO);
  qk_tic(ctx, T_SIGMA);
  qk_sigma_ff ff;
  const qk_sigma_ff* ffp = nullptr;
  QK_TRY(sigma_tier(ctx, prm, d, rho, Om, &ff, &ffp));
  QK_TRY(qk_sigma_diag(ctx, prm->doSRG, prm->eta, flow, N, d.nC, d.nO, d.nR, nS, eHF, Om, rho, SigC,
                       Z, scal + 8, ffp));
  QK_TRY(qk_qp_linear(ctx, N, eHF, Z, SigC, 1, eGWlin));
  qk_toc(ctx, T_SIGMA);
  qk_tic(ctx, T_QP);
  QK_TRY(g0w0_qp(ctx, prm, d, flow, eHF, Om, rho, SigC, Z, eGWlin, eGW, ffp));
  qk_toc(ctx, T_QP);
  qk_tic(ctx, T_CASIDA2);
  int quad = 0;
  if (!prm->TDA_W)
    QK_TRY(qk_rpa_ec_quad(ctx, N, d.nC, d.nO, d.nR, eGW, nullptr, Lov, naux, scal + 5, &quad,
                          prm->precision != QK_PREC_BF16X3));
  if (!quad) QK_TRY(casida_dev(ctx, d, eGW, nullptr, nullptr, nullptr, nullptr, scal + 3, 0, K));
  qk_toc(ctx, T_CASIDA2);
  double h[16];
  QK_TRY(d2h(ctx, h, scal, 16 * sizeof(double)));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  qk_timings_collect(ctx);
  if (hEcRPA) *hEcRPA = h[5];
  if (hEcGM) *hEcGM = h[8];
  return QK_OK;
}

int evgw_L_dev(qk_ctx* ctx, const qk_gw_params* prm, const Dims& d, int naux, const double* L,
               const double* eHF, double* eGW, double* SigC, double* Z, double* hEcRPA,
               double* hEcGM, int* hnSCF, double* hConv) {
  TdaScope tda(ctx, prm->TDA_W != 0);
  const int N = d.N, nS = d.nS;
  const size_t N2S = (size_t)N * N * nS;
  const int maxd = prm->max_diis > 1 ? prm->max_diis : 1;
  double *rho, *small, *K, *Lov;
  qk_timings_clear(ctx);
  QK_TRY(factor_prep(ctx, d, naux, L, &K, &Lov));
  QK_TRY(qk_wst(ctx, W_RHO, N2S, &rho));
  QK_TRY(qk_wst(ctx, W_HOST_B, (size_t)(6 + 2 * maxd) * N + nS + 64 + 8, &small));
  double* scal = small;
  double* eOld = small + 64;
  double* errv = eOld + N;
  double* Om = errv + N;
  double* err_hist = Om + nS;
  double* e_hist = err_hist + (size_t)N * maxd;
  int* dstate = (int*)(e_hist + (size_t)N * maxd);
  QK_CK(cudaMemsetAsync(err_hist, 0, sizeof(double) * 2 * (size_t)N * maxd, ctx->stream));
  QK_CK(cudaMemcpyAsync(eGW, eHF, N * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  QK_CK(cudaMemcpyAsync(eOld, eHF, N * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  EvBufs bb{nullptr, K, nullptr, eHF, eGW, eOld, SigC, Z, Om, nullptr, rho, scal, errv,
            err_hist, e_hist, dstate};
  bb.L = L;
  bb.Lov = Lov;
  bb.naux = naux;
  int nSCF = 0;
  double Conv = 1.0;
  QK_TRY(evgw_loop(ctx, prm, d, bb, &nSCF, &Conv));
  double h[16];
  QK_TRY(d2h(ctx, h, scal, 16 * sizeof(double)));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  qk_timings_collect(ctx);
  if (hEcRPA) *hEcRPA = h[2];
  if (hEcGM) *hEcGM = h[8];
  if (hnSCF) *hnSCF = nSCF;
  if (hConv) *hConv = Conv;
  if (nSCF == prm->maxSCF + 1)
    return qk_fail(ctx, QK_ERR_NO_CONV, "evGW convergence failed after %d cycles (Conv=%g)", nSCF, Conv);
  return QK_OK;
}

}  // namespace

int qk_g0w0_L(qk_ctx* ctx, const qk_gw_params* prm, int N, int nC, int nO, int nR, int naux,
              const double* L, const double* eHF, double* eGW, double* SigC, double* Z, double* Om,
              double* EcRPA, double* EcGM) {
  Dims d;
  const int nS = (nO - nC) * (N - nO - nR);
  QK_TRY(check_dims(ctx, N, N, nC, nO, N - nO, nR, nS, &d));
  return g0w0_L_dev(ctx, prm, d, naux, L, eHF, eGW, SigC, Z, Om, EcRPA, EcGM);
}

int qk_evgw_L(qk_ctx* ctx, const qk_gw_params* prm, int N, int nC, int nO, int nR, int naux,
              const double* L, const double* eHF, double* eGW, double* SigC, double* Z,
              double* EcRPA, double* EcGM, int* nSCF, double* Conv) {
  Dims d;
  const int nS = (nO - nC) * (N - nO - nR);
  QK_TRY(check_dims(ctx, N, N, nC, nO, N - nO, nR, nS, &d));
  return evgw_L_dev(ctx, prm, d, naux, L, eHF, eGW, SigC, Z, EcRPA, EcGM, nSCF, Conv);
}

namespace {

__global__ void k_vsum(int n, const double* __restrict__ v, double* out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += v[i];
  s = qk_block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

__global__ void k_copy_om(int n, const double* __restrict__ w, double* __restrict__ Om) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) Om[i] = w[i];
}

}  // namespace

// Casida solve on device buffers (LR/phRLR.f90:45-95): A (and B unless TDA) nS x nS column-major,
// A and B are overwritten.  TDA: Om = eig(A), XpY = XmY = eigenvectors as rows.  Otherwise the
// diagonal-A-B (dRPA) fast path or the general path eig(A-B) -> AmBSq, AmBIv -> eig(AmBSq (A+B)
// AmBSq).  scal[0] = tr A, [1] = sum Om, [2] = EcRPA = (sum Om - tr A)/2.  want_vectors = 0 skips
// the eigenvectors of the final eigenproblem (and XpY, XmY); *XpY / *XmY point at the context's
// buffers on return.
int phrlr_dev(qk_ctx* ctx, int TDA, int nS, double* dA, double* dB, double* dOm, double** XpY,
              double** XmY, double* scal, int want_vectors) {
  const size_t S2 = (size_t)nS * nS;
  double *dM, *dZt = nullptr, *dX = nullptr, *dY = nullptr, *sm;
  QK_TRY(qk_wst(ctx, W_M, S2, &dM));
  QK_TRY(qk_wst(ctx, W_E, 3 * (size_t)nS + 64, &sm));
  if (want_vectors) {
    QK_TRY(qk_wst(ctx, W_ZT, S2, &dZt));
    QK_TRY(qk_wst(ctx, W_XPY, S2, &dX));
    QK_TRY(qk_wst(ctx, W_XMY, S2, &dY));
  }
  double* sq = sm;
  double* w = sm + nS;
  QK_CK(cudaMemsetAsync(scal, 0, 4 * sizeof(double), ctx->stream));
  if (XpY) *XpY = want_vectors ? (TDA ? dZt : dX) : nullptr;
  if (XmY) *XmY = want_vectors ? (TDA ? dZt : dY) : nullptr;
  if (TDA) {
    k_trace<<<1, 1024, 0, ctx->stream>>>(nS, dA, scal + 0);
    QK_LAUNCHED();
    QK_TRY(qk_eig_sym(ctx, nS, dA, nS, w, dZt, want_vectors));  // Om = eig(A)
    k_copy_om<<<grid_for(ctx, nS), 256, 0, ctx->stream>>>(nS, w, dOm);
    QK_LAUNCHED();
    k_vsum<<<1, 1024, 0, ctx->stream>>>(nS, w, scal + 1);
    QK_LAUNCHED();
    k_ecrpa<<<1, 1, 0, ctx->stream>>>(scal + 1, scal + 0, scal + 2);
    QK_LAUNCHED();
    return QK_OK;
  }
  k_offdiag_maxabs<<<grid_for(ctx, (long long)S2), 256, 0, ctx->stream>>>(nS, dA, dB, scal + 3);
  QK_LAUNCHED();
  double offmax = 0.0;
  QK_TRY(d2h(ctx, &offmax, scal + 3, 8));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  if (offmax == 0.0) {
    // A-B diagonal (dRPA): M = AmBSq.(A+B).AmBSq directly
    QK_TRY(qk_launch_casida_M_from_AB(ctx, nS, dA, dB, dM, sq, scal + 0));
    QK_TRY(qk_eig_sym(ctx, nS, dM, nS, w, dZt, want_vectors));
    if (want_vectors) {
      QK_TRY(qk_launch_xpy(ctx, nS, w, dZt, sq, dOm, dX, dY, 1));
    } else {
      QK_TRY(qk_launch_omega(ctx, nS, w, dOm));
    }
  } else {
    // general A-B (phRLR.f90:50-81): eig(A-B), AmBSq = U sqrt(l) U^T, AmBIv = U l^-1/2 U^T
    double *amb, *sqm, *ivm, *tmp, *ut;
    QK_TRY(qk_wst(ctx, W_SLAB, 4 * S2, &amb));
    sqm = amb + S2;
    ivm = sqm + S2;
    tmp = ivm + S2;
    QK_TRY(qk_wst(ctx, W_BSEU, S2, &ut));  // U^T of A-B
    k_axpby<<<grid_for(ctx, (long long)S2), 256, 0, ctx->stream>>>((long long)S2, 1.0, dA, -1.0, dB, amb);
    QK_LAUNCHED();
    k_trace<<<1, 1024, 0, ctx->stream>>>(nS, dA, scal + 0);
    QK_LAUNCHED();
    double* lam = sm + 2 * nS;
    QK_TRY(qk_eig_sym(ctx, nS, amb, nS, lam, ut, 1));
    // AmBSq = U diag(sqrt l) U^T = Ut^T (D Ut)
    k_rowscale<<<grid_for(ctx, (long long)S2), 256, 0, ctx->stream>>>(nS, lam, 0, ut, tmp);
    QK_LAUNCHED();
    QK_TRY(qk_dgemm(ctx, 'T', 'N', nS, nS, nS, 1.0, ut, nS, 0, tmp, nS, 0, 0.0, sqm, nS, 0, 1));
    if (want_vectors) {
      k_rowscale<<<grid_for(ctx, (long long)S2), 256, 0, ctx->stream>>>(nS, lam, 1, ut, tmp);
      QK_LAUNCHED();
      QK_TRY(qk_dgemm(ctx, 'T', 'N', nS, nS, nS, 1.0, ut, nS, 0, tmp, nS, 0, 0.0, ivm, nS, 0, 1));
    }
    // ApB into amb, tmp = ApB.AmBSq, M = AmBSq.tmp
    k_axpby<<<grid_for(ctx, (long long)S2), 256, 0, ctx->stream>>>((long long)S2, 1.0, dA, 1.0, dB, amb);
    QK_LAUNCHED();
    QK_TRY(qk_dgemm(ctx, 'N', 'N', nS, nS, nS, 1.0, amb, nS, 0, sqm, nS, 0, 0.0, tmp, nS, 0, 1));
    QK_TRY(qk_dgemm(ctx, 'N', 'N', nS, nS, nS, 1.0, sqm, nS, 0, tmp, nS, 0, 0.0, dM, nS, 0, 1));
    QK_TRY(qk_eig_sym(ctx, nS, dM, nS, w, dZt, want_vectors));  // dZt = Z^T
    if (want_vectors) {
      QK_TRY(qk_dgemm(ctx, 'N', 'N', nS, nS, nS, 1.0, dZt, nS, 0, sqm, nS, 0, 0.0, dX, nS, 0, 1));
      QK_TRY(qk_dgemm(ctx, 'N', 'N', nS, nS, nS, 1.0, dZt, nS, 0, ivm, nS, 0, 0.0, dY, nS, 0, 1));
      k_xpy_general<<<grid_for(ctx, (long long)S2), 256, 0, ctx->stream>>>(nS, w, dOm, dX, dY, ctx->d_status);
      QK_LAUNCHED();
    } else {
      QK_TRY(qk_launch_omega(ctx, nS, w, dOm));
    }
  }
  QK_TRY(qk_launch_sum_sqrt(ctx, nS, w, scal + 1));
  k_ecrpa<<<1, 1, 0, ctx->stream>>>(scal + 1, scal + 0, scal + 2);
  QK_LAUNCHED();
  return QK_OK;
}

namespace {

int begin(qk_ctx* ctx) {
  if (!ctx) return QK_ERR_ARG;
  (void)cudaGetLastError();  // drop a non-sticky error left in this host thread by an earlier call
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return qk_cuda_fail(ctx, e, "cudaSetDevice", __FILE__, __LINE__);
  ctx->err.clear();
  QK_TRY(qk_order_after_default(ctx));
  return qk_status_reset(ctx);
}

constexpr int FATAL = QKD_BARRIER_TIMEOUT | QKD_BAD_INDEX | QKD_MBAR_TIMEOUT;

int end(qk_ctx* ctx, int st) {
  if (st != QK_OK && st != QK_ERR_NO_CONV) {
    cudaStreamSynchronize(ctx->stream);
    return st;
  }
  int s2 = qk_status_check(ctx, FATAL);
  return s2 != QK_OK ? s2 : st;
}

}  // namespace

extern "C" {

// ---------------------------------------------------------------------------------------------
// stage-level drop-ins
// ---------------------------------------------------------------------------------------------
int qk_phRLR_A(qk_ctx* ctx, int ispin, int dRPA, int nBas, int nC, int nO, int nV, int nR, int nS,
               double lambda, const double* e, const double* ERI, double* Aph) {
  QK_TRY(begin(ctx));
  (void)nV;
  if (ispin != 1 && ispin != 2) return qk_fail(ctx, QK_ERR_ARG, "ispin must be 1 or 2");
  const int no = nO - nC, nv = nBas - nO - nR;
  if (no <= 0 || nv <= 0 || (long long)no * nv != nS) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  const size_t N = nBas, N4 = N * N * N * N, S2 = (size_t)nS * nS;
  double *dERI, *de, *dA;
  QK_TRY(qk_wst(ctx, W_ERI, N4, &dERI));
  QK_TRY(qk_wst(ctx, W_HOST_B, N + 16, &de));
  QK_TRY(qk_wst(ctx, W_M, S2, &dA));
  QK_TRY(h2d(ctx, dERI, ERI, N4 * 8));
  QK_TRY(h2d(ctx, de, e, N * 8));
  QK_TRY(qk_launch_build_AB(ctx, 0, ispin, dRPA, nBas, nC, nO, nR, lambda, de, dERI, dA));
  QK_TRY(d2h(ctx, Aph, dA, S2 * 8));
  return end(ctx, QK_OK);
}

int qk_phRLR_B(qk_ctx* ctx, int ispin, int dRPA, int nBas, int nC, int nO, int nV, int nR, int nS,
               double lambda, const double* ERI, double* Bph) {
  QK_TRY(begin(ctx));
  (void)nV;
  if (ispin != 1 && ispin != 2) return qk_fail(ctx, QK_ERR_ARG, "ispin must be 1 or 2");
  const int no = nO - nC, nv = nBas - nO - nR;
  if (no <= 0 || nv <= 0 || (long long)no * nv != nS) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  const size_t N = nBas, N4 = N * N * N * N, S2 = (size_t)nS * nS;
  double *dERI, *dB;
  QK_TRY(qk_wst(ctx, W_ERI, N4, &dERI));
  QK_TRY(qk_wst(ctx, W_M, S2, &dB));
  QK_TRY(h2d(ctx, dERI, ERI, N4 * 8));
  QK_TRY(qk_launch_build_AB(ctx, 1, ispin, dRPA, nBas, nC, nO, nR, lambda, nullptr, dERI, dB));
  QK_TRY(d2h(ctx, Bph, dB, S2 * 8));
  return end(ctx, QK_OK);
}

int qk_phRLR(qk_ctx* ctx, int TDA, int nS, const double* Aph, const double* Bph, double* EcRPA,
             double* Om, double* XpY, double* XmY) {
  QK_TRY(begin(ctx));
  if (nS <= 0) return qk_fail(ctx, QK_ERR_ARG, "nS must be positive");
  const size_t S2 = (size_t)nS * nS;
  double *dA, *dOm, *scal;
  QK_TRY(qk_wst(ctx, W_HOST_A, 2 * S2, &dA));
  double* dB = dA + S2;
  QK_TRY(qk_wst(ctx, W_BSE, (size_t)nS + 16, &dOm));
  scal = dOm + nS;
  QK_TRY(h2d(ctx, dA, Aph, S2 * 8));
  if (!TDA) QK_TRY(h2d(ctx, dB, Bph, S2 * 8));
  double *dX = nullptr, *dY = nullptr;
  QK_TRY(phrlr_dev(ctx, TDA, nS, dA, dB, dOm, &dX, &dY, scal, 1));
  QK_TRY(d2h(ctx, Om, dOm, nS * 8));
  QK_TRY(d2h(ctx, XpY, dX, S2 * 8));
  QK_TRY(d2h(ctx, XmY, TDA ? dX : dY, S2 * 8));
  QK_TRY(d2h(ctx, EcRPA, scal + 2, 8));
  return end(ctx, QK_OK);
}

int qk_RGW_excitation_density(qk_ctx* ctx, int nOrb, int nC, int nO, int nR, int nS,
                              const double* ERI, const double* XpY, double* rho) {
  QK_TRY(begin(ctx));
  Dims d;
  QK_TRY(check_dims(ctx, nOrb, nOrb, nC, nO, nOrb - nO, nR, nS, &d));
  const size_t N = nOrb, N4 = N * N * N * N, S2 = (size_t)nS * nS, N2S = N * N * nS;
  double *dERI, *dX, *dS, *dR;
  QK_TRY(qk_wst(ctx, W_ERI, N4, &dERI));
  QK_TRY(qk_wst(ctx, W_XPY, S2, &dX));
  QK_TRY(qk_wst(ctx, W_SLAB, N2S, &dS));
  QK_TRY(qk_wst(ctx, W_RHO, N2S, &dR));
  QK_TRY(h2d(ctx, dERI, ERI, N4 * 8));
  QK_TRY(h2d(ctx, dX, XpY, S2 * 8));
  QK_TRY(qk_launch_slab_gather(ctx, nOrb, nC, nO, nR, dERI, dS));
  QK_TRY(rho_gemm(ctx, ctx->stage_precision, nOrb, nS, dS, dX, dR));
  QK_TRY(d2h(ctx, rho, dR, N2S * 8));
  return end(ctx, QK_OK);
}

static int sigma_stage(qk_ctx* ctx, int doSRG, double eta, double flow, int nBas, int nC, int nO,
                       int nR, int nS, const double* e, const double* Om, const double* rho,
                       double* EcGM, double* Sig, double* Z) {
  QK_TRY(begin(ctx));
  const int no = nO - nC, nv = nBas - nO - nR;
  if (no <= 0 || nv <= 0 || (long long)no * nv != nS) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  const size_t N = nBas, N2S = N * N * nS;
  double *dR, *sm;
  QK_TRY(qk_wst(ctx, W_RHO, N2S, &dR));
  QK_TRY(qk_wst(ctx, W_HOST_A, 4 * N + nS + 16, &sm));
  double* de = sm;
  double* dSig = sm + N;
  double* dZ = sm + 2 * N;
  double* dOm = sm + 3 * N;
  double* dGM = dOm + nS;
  QK_TRY(h2d(ctx, dR, rho, N2S * 8));
  QK_TRY(h2d(ctx, de, e, N * 8));
  QK_TRY(h2d(ctx, dOm, Om, nS * 8));
  qk_sigma_ff ff;
  const qk_sigma_ff* ffp = nullptr;
  if (ctx->stage_precision == QK_PREC_BF16X3 && eta == 0.0 && !doSRG) {
    QK_TRY(qk_sigma_ff_prep(ctx, nBas, nS, dR, dOm, &ff));
    ffp = &ff;
  }
  QK_TRY(qk_sigma_diag(ctx, doSRG, eta, flow, nBas, nC, nO, nR, nS, de, dOm, dR, dSig, dZ, dGM,
                       ffp));
  QK_TRY(d2h(ctx, Sig, dSig, N * 8));
  QK_TRY(d2h(ctx, Z, dZ, N * 8));
  QK_TRY(d2h(ctx, EcGM, dGM, 8));
  return end(ctx, QK_OK);
}

// full (N x N) correlation self-energy, Z and EcGM (RGW_self_energy.f90 / RGW_SRG_self_energy.f90)
static int sigma_full_stage(qk_ctx* ctx, int doSRG, double eta, double flow, int nOrb, int nC,
                            int nO, int nR, int nS, const double* e, const double* Om,
                            const double* rho, double* EcGM, double* Sig, double* Z) {
  QK_TRY(begin(ctx));
  const int no = nO - nC, nv = nOrb - nO - nR;
  if (no <= 0 || nv <= 0 || (long long)no * nv != nS) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  const size_t N = nOrb, N2 = N * N, N2S = N2 * nS;
  double *dR, *W, *sm;
  QK_TRY(qk_wst(ctx, W_RHO, N2S, &dR));
  QK_TRY(qk_wst(ctx, W_QSR1, N2S, &W));
  QK_TRY(qk_wst(ctx, W_HOST_A, N2 + 3 * N + nS + 16, &sm));
  double* dSig = sm;
  double* de = sm + N2;
  double* dd = de + N;
  double* dZ = dd + N;
  double* dOm = dZ + N;
  double* dGM = dOm + nS;
  QK_TRY(h2d(ctx, dR, rho, N2S * 8));
  QK_TRY(h2d(ctx, de, e, N * 8));
  QK_TRY(h2d(ctx, dOm, Om, nS * 8));
  QK_TRY(qk_qs_sigma(ctx, doSRG, eta, flow, nOrb, nC, nO, nR, nS, de, dOm, dR, W, dSig, 0));
  QK_TRY(qk_qs_mask(ctx, nOrb, nC, nR, dSig));
  QK_TRY(qk_sigma_diag(ctx, doSRG, eta, flow, nOrb, nC, nO, nR, nS, de, dOm, dR, dd, dZ, dGM));
  QK_TRY(d2h(ctx, Sig, dSig, N2 * 8));
  QK_TRY(d2h(ctx, Z, dZ, N * 8));
  QK_TRY(d2h(ctx, EcGM, dGM, 8));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  return end(ctx, QK_OK);
}

// J or K of a density in the AO basis (one pass over the tensor computes both)
static int jk_stage(qk_ctx* ctx, int nBas, const double* P, const double* ERI, double* J,
                    double* K) {
  QK_TRY(begin(ctx));
  if (nBas <= 0) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  const size_t B = nBas, B2 = B * B, B3 = B2 * B, B4 = B2 * B2;
  double *dE, *part, *sm;
  QK_TRY(qk_wst(ctx, W_ERI, B4, &dE));
  QK_TRY(qk_wst(ctx, W_QSJK, 2 * B3, &part));
  QK_TRY(qk_wst(ctx, W_HOST_A, 3 * B2 + 16, &sm));
  double* dP = sm;
  double* dJ = sm + B2;
  double* dK = dJ + B2;
  QK_TRY(h2d(ctx, dE, ERI, B4 * 8));
  QK_TRY(h2d(ctx, dP, P, B2 * 8));
  QK_TRY(qk_qs_jk(ctx, nBas, dE, dP, part, dJ, dK));
  if (J) QK_TRY(d2h(ctx, J, dJ, B2 * 8));
  if (K) QK_TRY(d2h(ctx, K, dK, B2 * 8));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  return end(ctx, QK_OK);
}

int qk_set_stage_precision(qk_ctx* ctx, int precision) {
  if (!ctx || (precision != QK_PREC_FP64 && precision != QK_PREC_BF16X3)) return QK_ERR_ARG;
  ctx->stage_precision = precision;
  return QK_OK;
}

int qk_RGW_self_energy_diag(qk_ctx* ctx, double eta, int nBas, int nOrb, int nC, int nO, int nV,
                            int nR, int nS, const double* e, const double* Om, const double* rho,
                            double* EcGM, double* Sig, double* Z) {
  (void)nOrb; (void)nV;
  return sigma_stage(ctx, 0, eta, 500.0, nBas, nC, nO, nR, nS, e, Om, rho, EcGM, Sig, Z);
}

int qk_RGW_self_energy(qk_ctx* ctx, double eta, int nBas, int nOrb, int nC, int nO, int nV,
                       int nR, int nS, const double* e, const double* Om, const double* rho,
                       double* EcGM, double* SigC, double* Z) {
  (void)nBas; (void)nV;
  return sigma_full_stage(ctx, 0, eta, 500.0, nOrb, nC, nO, nR, nS, e, Om, rho, EcGM, SigC, Z);
}

int qk_RGW_SRG_self_energy(qk_ctx* ctx, double flow, int nBas, int nOrb, int nC, int nO, int nV,
                           int nR, int nS, const double* e, const double* Om, const double* rho,
                           double* EcGM, double* SigC, double* Z) {
  (void)nBas; (void)nV;
  return sigma_full_stage(ctx, 1, 0.0, flow, nOrb, nC, nO, nR, nS, e, Om, rho, EcGM, SigC, Z);
}

int qk_Hartree_matrix_AO_basis(qk_ctx* ctx, int nBas, const double* P, const double* ERI,
                               double* H) {
  return jk_stage(ctx, nBas, P, ERI, H, nullptr);
}

int qk_exchange_matrix_AO_basis(qk_ctx* ctx, int nBas, const double* P, const double* ERI,
                                double* K) {
  return jk_stage(ctx, nBas, P, ERI, nullptr, K);
}

int qk_RGW_SRG_self_energy_diag(qk_ctx* ctx, double flow, int nBas, int nOrb, int nC, int nO,
                                int nV, int nR, int nS, const double* e, const double* Om,
                                const double* rho, double* EcGM, double* SigC, double* Z) {
  (void)nBas; (void)nV;
  // RGW_SRG_self_energy_diag.f90 dimensions its arrays with nOrb
  return sigma_stage(ctx, 1, 0.0, flow, nOrb, nC, nO, nR, nS, e, Om, rho, EcGM, SigC, Z);
}

int qk_RGW_QP_graph(qk_ctx* ctx, int doSRG, double eta, double flow, int nBas, int nC, int nO,
                    int nV, int nR, int nS, const double* eHF, const double* Om, const double* rho,
                    const double* eGWlin, const double* eOld, double* eGW, double* Z) {
  QK_TRY(begin(ctx));
  (void)nV;
  const int no = nO - nC, nv = nBas - nO - nR;
  if (no <= 0 || nv <= 0 || (long long)no * nv != nS) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  const size_t N = nBas, N2S = N * N * nS;
  double *dR, *sm;
  QK_TRY(qk_wst(ctx, W_RHO, N2S, &dR));
  QK_TRY(qk_wst(ctx, W_HOST_A, 6 * N + nS + 16, &sm));
  double* deHF = sm;
  double* dlin = sm + N;
  double* dold = sm + 2 * N;
  double* dGW = sm + 3 * N;
  double* dZ = sm + 4 * N;
  double* dOm = sm + 5 * N;
  QK_TRY(h2d(ctx, dR, rho, N2S * 8));
  QK_TRY(h2d(ctx, deHF, eHF, N * 8));
  QK_TRY(h2d(ctx, dlin, eGWlin, N * 8));
  QK_TRY(h2d(ctx, dold, eOld, N * 8));
  QK_TRY(h2d(ctx, dZ, Z, N * 8));
  QK_TRY(h2d(ctx, dGW, eGWlin, N * 8));
  QK_TRY(h2d(ctx, dOm, Om, nS * 8));
  qk_sigma_ff ff;
  const qk_sigma_ff* ffp = nullptr;
  if (ctx->stage_precision == QK_PREC_BF16X3 && eta == 0.0 && !doSRG) {
    QK_TRY(qk_sigma_ff_prep(ctx, nBas, nS, dR, dOm, &ff));
    ffp = &ff;
  }
  QK_TRY(qk_qp_newton(ctx, doSRG, eta, flow, nBas, nC, nO, nR, nS, deHF, dOm, dR, dlin, dold, dGW, dZ,
                      nullptr, 8, ffp));
  QK_TRY(d2h(ctx, eGW, dGW, N * 8));
  QK_TRY(d2h(ctx, Z, dZ, N * 8));
  return end(ctx, QK_OK);
}

namespace {

// four dgemm('T','N') quarter transforms (AOtoMO_ERI_RHF.f90:26-53) on device buffers; X holds
// the AO tensor and is overwritten, Y is scratch; returns the buffer that holds the result
int aotomo_dev(qk_ctx* ctx, int nBas, int nOrb, const double* dc, double* X, double* Y,
               double** result) {
  const size_t B = nBas, O = nOrb;
  long long R[4] = {(long long)(B * B * B), (long long)(B * B * O), (long long)(B * O * O),
                    (long long)(O * O * O)};
  double* src = X;
  double* dst = Y;
  // stage precision BF16X3: the quarter transforms in double-float (FP32 pairs, exact products;
  // ~1e-13 of sum |a b|) -- the MO coefficients of near-linearly-dependent bases cancel too much
  // for the BF16x3 / FP32-product tiers (the reason qsGW's mixed tier uses it as well)
  const bool df = ctx->stage_precision == QK_PREC_BF16X3;
  for (int s = 0; s < 4; ++s) {
    if (R[s] > INT_MAX) return qk_fail(ctx, QK_ERR_ARG, "AO->MO quarter transform too large");
    if (df)
      QK_TRY(qk_gemm_df(ctx, 'T', 'N', (int)R[s], nOrb, nBas, 1.0, src, nBas, 0, dc, nBas, 0, 0.0,
                        dst, R[s], 0, 1));
    else
      QK_TRY(qk_dgemm(ctx, 'T', 'N', (int)R[s], nOrb, nBas, 1.0, src, nBas, 0, dc, nBas, 0, 0.0,
                      dst, R[s], 0, 1));
    double* t = src;
    src = dst;
    dst = t;
  }
  *result = src;
  return QK_OK;
}

// ---------------------------------------------------------------------------------------------
// quasiparticle self-consistent GW@RHF (GW/qsRGW.f90:193-359, nBas = nOrb; the linearised
// density-matrix correction, dipoles and the post-processing BSE are not part of this path)
// ---------------------------------------------------------------------------------------------
struct QsIn {
  const double *eHF, *cHF, *PHF, *S, *T, *V, *Hc, *X, *ERI;
};
struct QsOut {
  double *eGW, *c, *P, *SigC, *Z;
  double *EqsGW, *EcRPA, *EcGM;
  int* nSCF;
  double* Conv;
};

int qsgw_dev(qk_ctx* ctx, const qk_gw_params* prm, int nBas, const Dims& d, const QsIn& in,
             const QsOut& out) {
  if (prm->maxSCF < 0) return qk_fail(ctx, QK_ERR_ARG, "maxSCF must be >= 0");
  if (prm->max_diis > 32) return qk_fail(ctx, QK_ERR_ARG, "max_diis above 32");
  if (nBas < d.N) return qk_fail(ctx, QK_ERR_ARG, "nBas (%d) < nOrb (%d)", nBas, d.N);
  TdaScope tda(ctx, prm->TDA_W != 0);
  const int N = d.N, nS = d.nS, B = nBas;
  const bool proj = B != N;  // the reference's nBas /= nOrb branch (qsRGW.f90:281-284,328-333)
  // mixed tier: the quarter transforms and the full-Sigma GEMM in double-float (FP32 pairs with
  // exact products: ~1e-13 of sum |terms|, where plain FP32 products left ~1e-5 Ha of noise in F
  // and stalled the SCF); ρ BF16x3 and the eigenvector back-transformation on FP32 products as in
  // G0W0; eigenvalues, the N x N algebra and the DIIS stay FP64
  const int mixed = prm->precision == QK_PREC_BF16X3;
  const double flow = 500.0;
  const size_t N1 = N, N2 = N1 * N1, B1 = B, B2 = B1 * B1, B3 = B2 * B1;
  const size_t rw = B3 * d.no > N2 * nS ? B3 * d.no : N2 * nS;
  double *W1, *W2, *part, *mat, *slab, *rho, *Kmat, *XpY, *hist = nullptr;
  QK_TRY(qk_wst(ctx, W_QSR1, rw, &W1));
  QK_TRY(qk_wst(ctx, W_QSR2, rw, &W2));
  QK_TRY(qk_wst(ctx, W_QSJK, 2 * B3, &part));
  QK_TRY(qk_wst(ctx, W_QSMAT, 14 * B2 + N1 + nS + 64, &mat));
  QK_TRY(qk_wst(ctx, W_SLAB, N2 * nS, &slab));
  QK_TRY(qk_wst(ctx, W_RHO, N2 * nS, &rho));
  QK_TRY(qk_wst(ctx, W_KMAT, (size_t)nS * nS, &Kmat));
  QK_TRY(qk_wst(ctx, W_XPY, (size_t)nS * nS, &XpY));
  // every matrix slot holds nBas^2 doubles; AO matrices are nBas x nBas (ld nBas), MO matrices
  // nOrb x nOrb (ld nOrb), mixed ones nBas x nOrb (ld nBas)
  double* J = mat;
  double* K = J + B2;
  double* F = K + B2;
  double* err = F + B2;
  double* Sraw = err + B2;
  double* Smo = Sraw + B2;
  double* SigCp = Smo + B2;
  double* T1 = SigCp + B2;
  double* T2 = T1 + B2;
  double* Fp = T2 + B2;
  double* Zt = Fp + B2;
  double* SC = Zt + B2;
  double* PS = SC + B2;
  double* SP = PS + B2;
  double* sdiag = SP + B2;
  double* Om = sdiag + N1;
  double* sm = Om + nS;  // [0..2] Casida scalars, [8] EcGM, [16..21] energies + max|err|, [24] rcond
  const int md = prm->max_diis;
  if (md > 1) {
    QK_TRY(qk_wst(ctx, W_QSDIIS, 2 * B2 * md, &hist));
    QK_CK(cudaMemsetAsync(hist, 0, 2 * B2 * md * sizeof(double), ctx->stream));
  }
  QK_CK(cudaMemsetAsync(sm, 0, 64 * sizeof(double), ctx->stream));
  if (out.eGW != in.eHF)
    QK_CK(cudaMemcpyAsync(out.eGW, in.eHF, N1 * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  if (out.c != in.cHF)
    QK_CK(cudaMemcpyAsync(out.c, in.cHF, B1 * N1 * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  if (out.P != in.PHF)
    QK_CK(cudaMemcpyAsync(out.P, in.PHF, B2 * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  auto gemm = [&](char ta, char tb, int m, int n, int k, double alpha, const double* A, int lda,
                  const double* Bm, int ldb, double beta, double* C, int ldc) {
    return qk_dgemm(ctx, ta, tb, m, n, k, alpha, A, lda, 0, Bm, ldb, 0, beta, C, ldc, 0, 1);
  };
  int nSCF = -1, n_diis = 0;
  double Conv = 1.0, hs[32] = {0.0};
  while (Conv > prm->thresh && nSCF < prm->maxSCF) {  // qsRGW.f90:193
    ++nSCF;
    QK_TRY(qk_qs_jk(ctx, B, in.ERI, out.P, part, J, K));                             // :201-202
    QK_TRY(qk_qs_mo_slab(ctx, B, N, d.nC, d.nO, d.nR, out.c, in.ERI, W1, W2, slab, Kmat,
                         mixed));                                                    // :210
    QK_TRY(casida_dev(ctx, d, out.eGW, nullptr, Om, XpY, nullptr, sm, 1, Kmat,
                      prm->precision));                                              // :214-217
    QK_TRY(rho_gemm(ctx, prm->precision, N, nS, slab, XpY, rho));                    // :220
    QK_TRY(qk_qs_sigma(ctx, prm->doSRG, prm->eta, flow, N, d.nC, d.nO, d.nR, nS, out.eGW, Om,
                       rho, W1, Sraw, mixed));                                       // :255-264
    QK_TRY(qk_sigma_diag(ctx, prm->doSRG, prm->eta, flow, N, d.nC, d.nO, d.nR, nS, out.eGW, Om,
                         rho, sdiag, out.Z, sm + 8));                                // Z, EcGM
    QK_TRY(qk_qs_sym(ctx, N, d.nC, d.nR, Sraw, Smo));                                // :269
    QK_TRY(gemm('N', 'N', B, N, B, 1.0, in.S, B, out.c, B, 0.0, SC, B));             // :276
    QK_TRY(gemm('N', 'N', B, N, N, 1.0, SC, B, Smo, N, 0.0, T1, B));
    QK_TRY(gemm('N', 'T', B, B, N, 1.0, T1, B, SC, B, 0.0, SigCp, B));
    QK_TRY(qk_qs_fock(ctx, B, in.Hc, J, K, SigCp, F));                               // :280
    if (proj) {                                                                      // :281-284
      QK_TRY(gemm('N', 'N', B, N, B, 1.0, F, B, out.c, B, 0.0, T2, B));
      QK_TRY(gemm('T', 'N', N, N, B, 1.0, out.c, B, T2, B, 0.0, Fp, N));
      QK_TRY(gemm('N', 'N', B, N, N, 1.0, SC, B, Fp, N, 0.0, T1, B));
      QK_TRY(gemm('N', 'T', B, B, N, 1.0, T1, B, SC, B, 0.0, F, B));
    }
    QK_TRY(gemm('N', 'N', B, B, B, 1.0, out.P, B, in.S, B, 0.0, PS, B));             // :288
    QK_TRY(gemm('N', 'N', B, B, B, 1.0, F, B, PS, B, 0.0, err, B));
    QK_TRY(gemm('N', 'N', B, B, B, 1.0, in.S, B, out.P, B, 0.0, SP, B));
    QK_TRY(gemm('N', 'N', B, B, B, -1.0, SP, B, F, B, 1.0, err, B));
    QK_TRY(qk_qs_energy(ctx, B, out.P, in.T, in.V, J, K, err, sm + 16));             // :290-310
    if (md > 1) {                                                                    // :314-319
      n_diis = n_diis + 1 < md ? n_diis + 1 : md;
      QK_TRY(qk_diis_dev(ctx, (int)B2, (int)B2, n_diis, hist, hist + B2 * md, err, F, sm + 24));
    }
    if (!proj) {                                                                     // :323-327
      QK_TRY(gemm('N', 'N', N, N, N, 1.0, F, N, in.X, N, 0.0, T2, N));
      QK_TRY(gemm('T', 'N', N, N, N, 1.0, in.X, N, T2, N, 0.0, Fp, N));
      QK_TRY(qk_eig_sym(ctx, N, Fp, N, out.eGW, Zt, 1, 1));
      QK_TRY(gemm('N', 'T', N, N, N, 1.0, in.X, N, Zt, N, 0.0, out.c, N));
    } else {                                                                         // :328-333
      QK_TRY(gemm('N', 'N', B, N, B, 1.0, F, B, out.c, B, 0.0, T2, B));
      QK_TRY(gemm('T', 'N', N, N, B, 1.0, out.c, B, T2, B, 0.0, Fp, N));
      QK_TRY(qk_eig_sym(ctx, N, Fp, N, out.eGW, Zt, 1, 1));
      QK_TRY(gemm('N', 'T', B, N, N, 1.0, out.c, B, Zt, N, 0.0, T1, B));
      QK_CK(cudaMemcpyAsync(out.c, T1, B1 * N1 * 8, cudaMemcpyDeviceToDevice, ctx->stream));
    }
    QK_TRY(gemm('N', 'T', B, B, d.nO, 2.0, out.c, B, out.c, B, 0.0, out.P, B));      // :339
    QK_CK(cudaMemcpyAsync(hs, sm, 32 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    QK_CK(cudaStreamSynchronize(ctx->stream));
    if (nSCF > 1) Conv = hs[21];                                                     // :290
  }
  if (out.SigC) {                                                                    // :335
    QK_TRY(gemm('N', 'N', B, N, B, 1.0, SigCp, B, out.c, B, 0.0, T1, B));
    QK_TRY(gemm('T', 'N', N, N, B, 1.0, out.c, B, T1, B, 0.0, out.SigC, N));
  }
  if (out.EqsGW) *out.EqsGW = hs[20];
  if (out.EcRPA) *out.EcRPA = hs[2];
  if (out.EcGM) *out.EcGM = hs[8];
  if (out.nSCF) *out.nSCF = nSCF;
  if (out.Conv) *out.Conv = Conv;
  return nSCF == prm->maxSCF ? QK_ERR_NO_CONV : QK_OK;  // :354
}

}  // namespace

int qk_AOtoMO_ERI_RHF(qk_ctx* ctx, int nBas, int nOrb, const double* c, const double* ERI_AO,
                      double* ERI_MO) {
  QK_TRY(begin(ctx));
  if (nBas <= 0 || nOrb <= 0 || nOrb > nBas) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  const size_t B = nBas, O = nOrb, B4 = B * B * B * B;
  double *X, *Y, *dc, *res;
  QK_TRY(qk_wst(ctx, W_ERI, B4, &X));
  QK_TRY(qk_wst(ctx, W_SLAB, B4, &Y));
  QK_TRY(qk_wst(ctx, W_HOST_A, B * O, &dc));
  QK_TRY(h2d(ctx, X, ERI_AO, B4 * 8));
  QK_TRY(h2d(ctx, dc, c, B * O * 8));
  QK_TRY(aotomo_dev(ctx, nBas, nOrb, dc, X, Y, &res));
  QK_TRY(d2h(ctx, ERI_MO, res, O * O * O * O * 8));
  return end(ctx, QK_OK);
}

int qk_AOtoMO_ERI_RHF_dev(qk_ctx* ctx, int nBas, int nOrb, const double* d_c,
                          const double* d_ERI_AO, double* d_ERI_MO) {
  QK_TRY(begin(ctx));
  if (nBas <= 0 || nOrb <= 0 || nOrb > nBas) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  const size_t B = nBas, O = nOrb, B4 = B * B * B * B;
  double *X, *Y, *res;
  QK_TRY(qk_wst(ctx, W_ERI, B4, &X));
  QK_TRY(qk_wst(ctx, W_SLAB, B4, &Y));
  QK_CK(cudaMemcpyAsync(X, d_ERI_AO, B4 * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  QK_TRY(aotomo_dev(ctx, nBas, nOrb, d_c, X, Y, &res));
  QK_CK(cudaMemcpyAsync(d_ERI_MO, res, O * O * O * O * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  return end(ctx, QK_OK);
}

int qk_DIIS_extrapolation(qk_ctx* ctx, double* rcond, int n_err, int n_e, int n_diis,
                          double* error, double* e, const double* error_in, double* e_inout) {
  QK_TRY(begin(ctx));
  if (n_err <= 0 || n_e <= 0 || n_diis <= 0) return qk_fail(ctx, QK_ERR_ARG, "bad sizes");
  double* sm;
  const size_t need = (size_t)n_err * n_diis + (size_t)n_e * n_diis + n_err + n_e + 8;
  QK_TRY(qk_wst(ctx, W_HOST_A, need, &sm));
  double* dErr = sm;
  double* dE = dErr + (size_t)n_err * n_diis;
  double* dIn = dE + (size_t)n_e * n_diis;
  double* dIO = dIn + n_err;
  double* dRc = dIO + n_e;
  QK_TRY(h2d(ctx, dErr, error, (size_t)n_err * n_diis * 8));
  QK_TRY(h2d(ctx, dE, e, (size_t)n_e * n_diis * 8));
  QK_TRY(h2d(ctx, dIn, error_in, n_err * 8));
  QK_TRY(h2d(ctx, dIO, e_inout, n_e * 8));
  QK_TRY(qk_diis_dev(ctx, n_err, n_e, n_diis, dErr, dE, dIn, dIO, dRc));
  QK_TRY(d2h(ctx, error, dErr, (size_t)n_err * n_diis * 8));
  QK_TRY(d2h(ctx, e, dE, (size_t)n_e * n_diis * 8));
  QK_TRY(d2h(ctx, e_inout, dIO, n_e * 8));
  QK_TRY(d2h(ctx, rcond, dRc, 8));
  return end(ctx, QK_OK);
}

// ---------------------------------------------------------------------------------------------
// drivers
// ---------------------------------------------------------------------------------------------
int qk_RG0W0_dev(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
                 int nR, int nS, const double* d_eHF, const double* d_ERI, double* d_eGW,
                 double* d_SigC, double* d_Z, double* d_Om, double* EcRPA, double* EcGM) {
  QK_TRY(begin(ctx));
  if (!prm) return qk_fail(ctx, QK_ERR_ARG, "params required");
  Dims d;
  QK_TRY(check_dims(ctx, nBas, nOrb, nC, nO, nV, nR, nS, &d));
  const int st = g0w0_dev(ctx, prm, d, d_eHF, d_ERI, d_eGW, d_SigC, d_Z, d_Om, EcRPA, EcGM);
  return end(ctx, st);
}

int qk_evRGW_dev(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
                 int nR, int nS, const double* d_eHF, const double* d_ERI, double* d_eGW,
                 double* d_SigC, double* d_Z, double* EcRPA, double* EcGM, int* nSCF,
                 double* Conv) {
  QK_TRY(begin(ctx));
  if (!prm) return qk_fail(ctx, QK_ERR_ARG, "params required");
  Dims d;
  QK_TRY(check_dims(ctx, nBas, nOrb, nC, nO, nV, nR, nS, &d));
  const int st = evgw_dev(ctx, prm, d, d_eHF, d_ERI, d_eGW, d_SigC, d_Z, EcRPA, EcGM, nSCF, Conv);
  return end(ctx, st);
}

int qk_RG0W0(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
             int nR, int nS, const double* eHF, const double* ERI, double* eGW, double* SigC,
             double* Z, double* Om, double* EcRPA, double* EcGM) {
  QK_TRY(begin(ctx));
  if (!prm) return qk_fail(ctx, QK_ERR_ARG, "params required");
  Dims d;
  QK_TRY(check_dims(ctx, nBas, nOrb, nC, nO, nV, nR, nS, &d));
  const size_t N = nOrb, N4 = N * N * N * N;
  double *dERI, *io;
  QK_TRY(qk_wst(ctx, W_ERI, N4, &dERI));
  QK_TRY(qk_wst(ctx, W_HOST_A, 4 * N + nS + 16, &io));
  double* de = io;
  double* dGW = io + N;
  double* dSig = io + 2 * N;
  double* dZ = io + 3 * N;
  double* dOm = io + 4 * N;
  QK_TRY(h2d(ctx, de, eHF, N * 8));
  QK_TRY(h2d_eri_split(ctx, dERI, ERI, d));
  int st = g0w0_dev(ctx, prm, d, de, dERI, dGW, dSig, dZ, dOm, EcRPA, EcGM);
  if (ctx->eri_pending) {  // an early return: the copies still end before the next call
    cudaStreamWaitEvent(ctx->stream, ctx->ev_copy, 0);
    ctx->eri_pending = false;
  }
  if (st != QK_OK) return end(ctx, st);
  QK_TRY(d2h(ctx, eGW, dGW, N * 8));
  QK_TRY(d2h(ctx, SigC, dSig, N * 8));
  QK_TRY(d2h(ctx, Z, dZ, N * 8));
  QK_TRY(d2h(ctx, Om, dOm, (size_t)nS * 8));
  return end(ctx, QK_OK);
}

int qk_evRGW(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
             int nR, int nS, const double* eHF, const double* ERI, double* eGW, double* SigC,
             double* Z, double* EcRPA, double* EcGM, int* nSCF, double* Conv) {
  QK_TRY(begin(ctx));
  if (!prm) return qk_fail(ctx, QK_ERR_ARG, "params required");
  Dims d;
  QK_TRY(check_dims(ctx, nBas, nOrb, nC, nO, nV, nR, nS, &d));
  const size_t N = nOrb, N4 = N * N * N * N;
  double *dERI, *io;
  QK_TRY(qk_wst(ctx, W_ERI, N4, &dERI));
  QK_TRY(qk_wst(ctx, W_HOST_A, 4 * N + 16, &io));
  double* de = io;
  double* dGW = io + N;
  double* dSig = io + 2 * N;
  double* dZ = io + 3 * N;
  QK_TRY(h2d_eri_used(ctx, dERI, ERI, d));
  QK_TRY(h2d(ctx, de, eHF, N * 8));
  int st = evgw_dev(ctx, prm, d, de, dERI, dGW, dSig, dZ, EcRPA, EcGM, nSCF, Conv);
  if (st != QK_OK && st != QK_ERR_NO_CONV) return end(ctx, st);
  QK_TRY(d2h(ctx, eGW, dGW, N * 8));
  QK_TRY(d2h(ctx, SigC, dSig, N * 8));
  QK_TRY(d2h(ctx, Z, dZ, N * 8));
  return end(ctx, st);
}

int qk_dgemm_dev(qk_ctx* ctx, char transa, char transb, int m, int n, int k, double alpha,
                 const double* d_A, int lda, const double* d_B, int ldb, double beta, double* d_C,
                 int ldc) {
  QK_TRY(begin(ctx));
  const int st = qk_dgemm(ctx, transa, transb, m, n, k, alpha, d_A, lda, 0, d_B, ldb, 0, beta, d_C,
                          ldc, 0, 1);
  return end(ctx, st);
}

int qk_RGW_phBSE_dev(qk_ctx* ctx, const qk_bse_params* prm, int nOrb, int nC, int nO, int nR,
                     const double* d_ERI, const double* d_eW, const double* d_eGW, double* EcBSE,
                     double* d_OmBSE_singlet, double* d_OmBSE_triplet) {
  QK_TRY(begin(ctx));
  if (!prm || !d_ERI || !d_eW || !d_eGW) return qk_fail(ctx, QK_ERR_ARG, "inputs required");
  Dims d;
  const int nS = (nO - nC) * (nOrb - nO - nR);
  QK_TRY(check_dims(ctx, nOrb, nOrb, nC, nO, nOrb - nO, nR, nS, &d));
  const int st = qk_bse_dev(ctx, prm->TDA_W, prm->TDA, prm->singlet, prm->triplet,
                            prm->exchange_kernel, prm->eta, nOrb, nC, nO, nR, d_ERI, d_eW, d_eGW,
                            EcBSE, d_OmBSE_singlet, d_OmBSE_triplet);
  return end(ctx, st);
}

int qk_RGW_phACFDT_dev(qk_ctx* ctx, const qk_bse_params* prm, int doXBS, int nOrb, int nC, int nO,
                       int nR, const double* d_ERI, const double* d_eW, const double* d_eGW,
                       double* EcAC) {
  QK_TRY(begin(ctx));
  if (!prm || !d_ERI || !d_eW || !d_eGW || !EcAC)
    return qk_fail(ctx, QK_ERR_ARG, "inputs and EcAC required");
  Dims d;
  const int nS = (nO - nC) * (nOrb - nO - nR);
  QK_TRY(check_dims(ctx, nOrb, nOrb, nC, nO, nOrb - nO, nR, nS, &d));
  const int st = qk_bse_acfdt_dev(ctx, prm->exchange_kernel, doXBS, prm->TDA_W, prm->TDA,
                                  prm->singlet, prm->triplet, prm->eta, nOrb, nC, nO, nR, d_ERI,
                                  d_eW, d_eGW, EcAC);
  return end(ctx, st);
}

int qk_RGW_phACFDT(qk_ctx* ctx, const qk_bse_params* prm, int doXBS, int nBas, int nOrb, int nC,
                   int nO, int nV, int nR, int nS, const double* ERI, const double* eW,
                   const double* eGW, double* EcAC) {
  QK_TRY(begin(ctx));
  if (!prm || !ERI || !eW || !eGW || !EcAC) return qk_fail(ctx, QK_ERR_ARG, "inputs required");
  Dims d;
  QK_TRY(check_dims(ctx, nBas, nOrb, nC, nO, nV, nR, nS, &d));
  const size_t N = nOrb, N4 = N * N * N * N;
  double *dERI, *io;
  QK_TRY(qk_wst(ctx, W_ERI, N4, &dERI));
  QK_TRY(qk_wst(ctx, W_HOST_B, 2 * N + 16, &io));
  QK_TRY(h2d(ctx, dERI, ERI, N4 * 8));
  QK_TRY(h2d(ctx, io, eW, N * 8));
  QK_TRY(h2d(ctx, io + N, eGW, N * 8));
  const int st = qk_bse_acfdt_dev(ctx, prm->exchange_kernel, doXBS, prm->TDA_W, prm->TDA,
                                  prm->singlet, prm->triplet, prm->eta, nOrb, nC, nO, nR, dERI,
                                  io, io + N, EcAC);
  return end(ctx, st);
}

int qk_RGW_phBSE(qk_ctx* ctx, const qk_bse_params* prm, int nBas, int nOrb, int nC, int nO,
                 int nV, int nR, int nS, const double* ERI, const double* eW, const double* eGW,
                 double* EcBSE, double* OmBSE_singlet, double* OmBSE_triplet) {
  QK_TRY(begin(ctx));
  if (!prm || !ERI || !eW || !eGW) return qk_fail(ctx, QK_ERR_ARG, "inputs required");
  Dims d;
  QK_TRY(check_dims(ctx, nBas, nOrb, nC, nO, nV, nR, nS, &d));
  const size_t N = nOrb, N4 = N * N * N * N;
  double *dERI, *io;
  QK_TRY(qk_wst(ctx, W_ERI, N4, &dERI));
  QK_TRY(qk_wst(ctx, W_HOST_B, 2 * N + 2 * (size_t)nS + 16, &io));
  double* deW = io;
  double* deGW = io + N;
  double* dOS = io + 2 * N;
  double* dOT = dOS + nS;
  QK_TRY(h2d(ctx, dERI, ERI, N4 * 8));
  QK_TRY(h2d(ctx, deW, eW, N * 8));
  QK_TRY(h2d(ctx, deGW, eGW, N * 8));
  const int st = qk_bse_dev(ctx, prm->TDA_W, prm->TDA, prm->singlet, prm->triplet,
                            prm->exchange_kernel, prm->eta, nOrb, nC, nO, nR, dERI, deW, deGW,
                            EcBSE, OmBSE_singlet ? dOS : nullptr, OmBSE_triplet ? dOT : nullptr);
  if (st != QK_OK) return end(ctx, st);
  if (OmBSE_singlet) QK_TRY(d2h(ctx, OmBSE_singlet, dOS, (size_t)nS * 8));
  if (OmBSE_triplet) QK_TRY(d2h(ctx, OmBSE_triplet, dOT, (size_t)nS * 8));
  return end(ctx, QK_OK);
}

int qk_RPA_ecorr_quad_dev(qk_ctx* ctx, int nOrb, int nC, int nO, int nR, int naux,
                          const double* d_e, const double* d_ERI, const double* d_L,
                          double* EcRPA, int* applied) {
  QK_TRY(begin(ctx));
  if (!EcRPA || !applied || (!d_ERI) == (!d_L) || (d_L && naux <= 0))
    return qk_fail(ctx, QK_ERR_ARG, "one of ERI / L (with naux > 0) and the outputs required");
  Dims d;
  const int nS = (nO - nC) * (nOrb - nO - nR);
  QK_TRY(check_dims(ctx, nOrb, nOrb, nC, nO, nOrb - nO, nR, nS, &d));
  double* Lov = nullptr;
  if (d_L) {
    QK_TRY(qk_wst(ctx, W_VEC2, (size_t)nS * naux, &Lov));
    QK_TRY(qk_launch_gather_ov(ctx, nOrb, nC, nO, nR, naux, d_L, Lov));
  }
  double* dEc = nullptr;
  QK_TRY(qk_wst(ctx, W_HOST_A, 8, &dEc));
  int used = 0;
  const int st = qk_rpa_ec_quad(ctx, nOrb, nC, nO, nR, d_e, d_ERI, Lov, naux, dEc, &used);
  if (st != QK_OK) return end(ctx, st);
  *applied = used;
  *EcRPA = 0.0;
  if (used) QK_TRY(d2h(ctx, EcRPA, dEc, sizeof(double)));
  return end(ctx, QK_OK);
}

int qk_gauss_legendre(int n, double* x, double* w) {
  if (n < 1 || n > 4096 || !x || !w) return QK_ERR_ARG;
  qk_gauss_legendre_host(n, x, w);
  return QK_OK;
}

int qk_dgemm_df_dev(qk_ctx* ctx, char transa, char transb, int m, int n, int k, double alpha,
                    const double* d_A, int lda, const double* d_B, int ldb, double beta,
                    double* d_C, int ldc) {
  QK_TRY(begin(ctx));
  const int st = qk_gemm_df(ctx, transa, transb, m, n, k, alpha, d_A, lda, 0, d_B, ldb, 0, beta,
                            d_C, ldc, 0, 1);
  return end(ctx, st);
}

int qk_dgemm_f32p_dev(qk_ctx* ctx, char transa, char transb, int m, int n, int k, double alpha,
                      const double* d_A, int lda, const double* d_B, int ldb, double beta,
                      double* d_C, int ldc) {
  QK_TRY(begin(ctx));
  const int st = qk_gemm_f32p(ctx, transa, transb, m, n, k, alpha, d_A, lda, 0, d_B, ldb, 0, beta,
                              d_C, ldc, 0, 1);
  return end(ctx, st);
}

int qk_gemm_bf16x3_dev(qk_ctx* ctx, int m, int n, int k, const double* d_A, int lda,
                       const double* d_B, int ldb, double* d_C, int ldc) {
  QK_TRY(begin(ctx));
  if (lda < m || ldb < n || ldc < m) return qk_fail(ctx, QK_ERR_ARG, "bad leading dimensions");
  const int st = qk_gemm_bf16x3_nt(ctx, m, n, k, d_A, lda, d_B, ldb, d_C, ldc);
  return end(ctx, st);
}

int qk_gemm_bf16x3_ex_dev(qk_ctx* ctx, char transa, char transb, int m, int n, int k,
                          double alpha, const double* d_A, int lda, const double* d_B, int ldb,
                          double beta, double* d_C, int ldc) {
  QK_TRY(begin(ctx));
  const bool TA = (transa == 'T' || transa == 't'), TB = (transb == 'T' || transb == 't');
  if (lda < (TA ? k : m) || ldb < (TB ? n : k) || ldc < m)
    return qk_fail(ctx, QK_ERR_ARG, "bad leading dimensions");
  const int st = qk_gemm_bf16x3(ctx, transa, transb, m, n, k, alpha, d_A, lda, 0, d_B, ldb, 0,
                                nullptr, 0, beta, d_C, ldc, 0, 1, false);
  return end(ctx, st);
}

int qk_RG0W0_L_dev(qk_ctx* ctx, const qk_gw_params* prm, int nOrb, int nC, int nO, int nR,
                   int naux, const double* d_L, const double* d_eHF, double* d_eGW, double* d_SigC,
                   double* d_Z, double* d_Om, double* EcRPA, double* EcGM) {
  QK_TRY(begin(ctx));
  if (!prm || naux <= 0) return qk_fail(ctx, QK_ERR_ARG, "params/naux required");
  Dims d;
  const int nS = (nO - nC) * (nOrb - nO - nR);
  QK_TRY(check_dims(ctx, nOrb, nOrb, nC, nO, nOrb - nO, nR, nS, &d));
  const int st = g0w0_L_dev(ctx, prm, d, naux, d_L, d_eHF, d_eGW, d_SigC, d_Z, d_Om, EcRPA, EcGM);
  return end(ctx, st);
}

int qk_evRGW_L_dev(qk_ctx* ctx, const qk_gw_params* prm, int nOrb, int nC, int nO, int nR,
                   int naux, const double* d_L, const double* d_eHF, double* d_eGW, double* d_SigC,
                   double* d_Z, double* EcRPA, double* EcGM, int* nSCF, double* Conv) {
  QK_TRY(begin(ctx));
  if (!prm || naux <= 0) return qk_fail(ctx, QK_ERR_ARG, "params/naux required");
  Dims d;
  const int nS = (nO - nC) * (nOrb - nO - nR);
  QK_TRY(check_dims(ctx, nOrb, nOrb, nC, nO, nOrb - nO, nR, nS, &d));
  const int st = evgw_L_dev(ctx, prm, d, naux, d_L, d_eHF, d_eGW, d_SigC, d_Z, EcRPA, EcGM, nSCF,
                            Conv);
  return end(ctx, st);
}

}  // extern "C"

extern "C" {

int qk_qsRGW_dev(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
                 int nR, int nS, const double* d_eHF, const double* d_cHF, const double* d_PHF,
                 const double* d_S, const double* d_T, const double* d_V, const double* d_Hc,
                 const double* d_X, const double* d_ERI_AO, double* d_eGW, double* d_c,
                 double* d_P, double* d_SigC, double* d_Z, double* EqsGW, double* EcRPA,
                 double* EcGM, int* nSCF, double* Conv) {
  QK_TRY(begin(ctx));
  if (!prm || !d_eHF || !d_cHF || !d_PHF || !d_S || !d_T || !d_V || !d_Hc || !d_X || !d_ERI_AO ||
      !d_eGW || !d_c || !d_P || !d_Z)
    return qk_fail(ctx, QK_ERR_ARG, "inputs and eGW, c, P, Z required");
  Dims d;
  if (nBas < nOrb) return qk_fail(ctx, QK_ERR_ARG, "nBas (%d) < nOrb (%d)", nBas, nOrb);
  QK_TRY(check_dims(ctx, nOrb, nOrb, nC, nO, nV, nR, nS, &d));
  const QsIn in{d_eHF, d_cHF, d_PHF, d_S, d_T, d_V, d_Hc, d_X, d_ERI_AO};
  const QsOut out{d_eGW, d_c, d_P, d_SigC, d_Z, EqsGW, EcRPA, EcGM, nSCF, Conv};
  return end(ctx, qsgw_dev(ctx, prm, nBas, d, in, out));
}

int qk_qsRGW(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
             int nR, int nS, const double* eHF, const double* cHF, const double* PHF,
             const double* S, const double* T, const double* V, const double* Hc, const double* X,
             const double* ERI_AO, double* eGW, double* c, double* P, double* SigC, double* Z,
             double* EqsGW, double* EcRPA, double* EcGM, int* nSCF, double* Conv) {
  QK_TRY(begin(ctx));
  if (!prm || !eHF || !cHF || !PHF || !S || !T || !V || !Hc || !X || !ERI_AO || !eGW)
    return qk_fail(ctx, QK_ERR_ARG, "inputs and eGW required");
  Dims d;
  if (nBas < nOrb) return qk_fail(ctx, QK_ERR_ARG, "nBas (%d) < nOrb (%d)", nBas, nOrb);
  QK_TRY(check_dims(ctx, nOrb, nOrb, nC, nO, nV, nR, nS, &d));
  const size_t N = nOrb, N2 = N * N, Bn = nBas, B2 = Bn * Bn, B4 = B2 * B2;
  double *dERI, *io;
  QK_TRY(qk_wst(ctx, W_ERI, B4, &dERI));
  QK_TRY(qk_wst(ctx, W_QSIN, 8 * B2 + 2 * N + 16, &io));
  double* dS = io;
  double* dT = dS + B2;
  double* dV = dT + B2;
  double* dHc = dV + B2;
  double* dX = dHc + B2;     // nBas x nOrb
  double* dc = dX + B2;      // nBas x nOrb
  double* dP = dc + B2;
  double* dSig = dP + B2;    // nOrb x nOrb
  double* de = dSig + B2;
  double* dZ = de + N;
  QK_TRY(h2d(ctx, dERI, ERI_AO, B4 * 8));
  QK_TRY(h2d(ctx, dS, S, B2 * 8));
  QK_TRY(h2d(ctx, dT, T, B2 * 8));
  QK_TRY(h2d(ctx, dV, V, B2 * 8));
  QK_TRY(h2d(ctx, dHc, Hc, B2 * 8));
  QK_TRY(h2d(ctx, dX, X, Bn * N * 8));
  QK_TRY(h2d(ctx, dc, cHF, Bn * N * 8));
  QK_TRY(h2d(ctx, dP, PHF, B2 * 8));
  QK_TRY(h2d(ctx, de, eHF, N * 8));
  const QsIn in{de, dc, dP, dS, dT, dV, dHc, dX, dERI};
  const QsOut out{de, dc, dP, SigC ? dSig : nullptr, dZ, EqsGW, EcRPA, EcGM, nSCF, Conv};
  const int st = qsgw_dev(ctx, prm, nBas, d, in, out);
  if (st != QK_OK && st != QK_ERR_NO_CONV) return end(ctx, st);
  QK_TRY(d2h(ctx, eGW, de, N * 8));
  if (c) QK_TRY(d2h(ctx, c, dc, Bn * N * 8));
  if (P) QK_TRY(d2h(ctx, P, dP, B2 * 8));
  if (SigC) QK_TRY(d2h(ctx, SigC, dSig, N2 * 8));
  if (Z) QK_TRY(d2h(ctx, Z, dZ, N * 8));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  return end(ctx, st);
}

}  // extern "C"
