// k_bse.cu -- static Bethe-Salpeter excitation energies on top of GW (phBSE@GW, singlet and
// triplet, full or Tamm-Dancoff), GW/RGW_phBSE.f90:83-190 without the second-order kernel and
// the dynamical correction.
//
// Screening: the dRPA singlet Casida at the energies eW gives Om and XpY, then rho (FP64), as in
// the G0W0 path.  The static kernels (RGW_phBSE_static_kernel_A/B.f90:32-52)
//   KA(ia,jb) = 4 sum_kc rho(i,j,kc) rho(a,b,kc) Om_kc/(Om_kc^2 + eta^2)
//   KB(ia,jb) = 4 sum_kc rho(i,b,kc) rho(a,j,kc) Om_kc/(Om_kc^2 + eta^2)
// are two FP64 GEMMs over kc: the rho blocks (occ,occ), (vir,vir), (occ,vir), (vir,occ) are
// gathered as matrices with kc as the inner dimension, the weight folded into one side, and
// the products (o^2 x v^2, 2 nS^3 flop each) are added into A and B with the (ia, jb) index
// permutation.  Per spin, A = phRLR_A(ispin, dRPA = false, eGW) + KA and B = phRLR_B + KB go
// through the general (non-diagonal A - B) Casida solve for the excitation energies.
#include "qk_internal.cuh"

namespace {

// f = 4 lam^2 Om/(Om^2 + eta^2) (RGW_phBSE_static_kernel_A.f90:45, the kernel's lambda^2)
__global__ void k_bse_weights(int nS, double eta, double lam2, const double* __restrict__ Om,
                              double* __restrict__ f) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nS; k += gridDim.x * blockDim.x)
    f[k] = (4.0 * lam2) * (Om[k] / (Om[k] * Om[k] + eta * eta));
}

// out[pp + np*qq + np*nq*kc] = rho(p0+pp, q0+qq, kc) * (f ? f[kc] : 1)
__global__ void k_rho_block(int N, int nS, int p0, int np_, int q0, int nq_,
                            const double* __restrict__ rho, const double* __restrict__ f,
                            double* __restrict__ out) {
  const long long per = (long long)np_ * nq_;
  const long long total = per * nS;
  const long long N1 = N, N2 = N1 * N1;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int kc = (int)(idx / per);
    const long long r = idx - per * kc;
    const int qq = (int)(r / np_), pp = (int)(r - (long long)qq * np_);
    const double x = rho[(p0 + pp) + N1 * (q0 + qq) + N2 * kc];
    out[idx] = f ? x * f[kc] : x;
  }
}

// A[(i nv + a) + nS (j nv + b)] += G1[(i + no j) + no^2 (a + nv b)]
__global__ void k_bse_add_KA(int no, int nv, const double* __restrict__ G1, double* __restrict__ A) {
  const long long nS = (long long)no * nv, total = nS * nS, o2 = (long long)no * no;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long jb = idx / nS, ia = idx - jb * nS;
    const int i = (int)(ia / nv), a = (int)(ia - (long long)i * nv);
    const int j = (int)(jb / nv), b = (int)(jb - (long long)j * nv);
    A[idx] += G1[(i + (long long)no * j) + o2 * (a + (long long)nv * b)];
  }
}

// B[(i nv + a) + nS (j nv + b)] += G2[(i + no b) + nS (a + nv j)]
__global__ void k_bse_add_KB(int no, int nv, const double* __restrict__ G2, double* __restrict__ B) {
  const long long nS = (long long)no * nv, total = nS * nS;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long jb = idx / nS, ia = idx - jb * nS;
    const int i = (int)(ia / nv), a = (int)(ia - (long long)i * nv);
    const int j = (int)(jb / nv), b = (int)(jb - (long long)j * nv);
    B[idx] += G2[(i + (long long)no * b) + nS * (a + (long long)nv * j)];
  }
}

// ACFDT integrand matrices (RPA/phACFDT_correlation_energy.f90:56-70), ia = i nv + a:
//   Ap(ia,jb) = c1 ERI(i,b,a,j) - c2 ERI(i,b,j,a),  Bp(ia,jb) = c1 ERI(i,j,a,b) - c2 ERI(i,j,b,a)
__global__ void k_acfdt_ApBp(int N, int nC, int nO, int nv, double c1, double c2,
                             const double* __restrict__ E, double* __restrict__ Ap,
                             double* __restrict__ Bp) {
  const long long nS = (long long)(nO - nC) * nv, total = nS * nS, N1 = N;
  auto at = [&](long long p, long long q, long long r, long long t) {
    return E[p + N1 * (q + N1 * (r + N1 * t))];
  };
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long ia = idx % nS, jb = idx / nS;
    const long long i = nC + ia / nv, a = nO + ia % nv;
    const long long j = nC + jb / nv, b = nO + jb % nv;
    Ap[idx] = c1 * at(i, b, a, j) - c2 * at(i, b, j, a);
    Bp[idx] = c1 * at(i, j, a, b) - c2 * at(i, j, b, a);
  }
}

// Z = [X; Y] (2nS x nS, column-major, ld 2nS) with X = (XpY + XmY)/2, Y = (XpY - XmY)/2
__global__ void k_acfdt_xy(int nS, const double* __restrict__ XpY, const double* __restrict__ XmY,
                           double* __restrict__ Z) {
  const long long n = (long long)nS, total = n * n;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long m = idx % n, ia = idx / n;
    const double p = XpY[idx], q = XmY[idx];
    Z[m + 2 * n * ia] = 0.5 * (p + q);
    Z[n + m + 2 * n * ia] = 0.5 * (p - q);
  }
}

// out = tr(X Bp Y^T + Y Bp X^T) + tr(X Ap X^T + Y Ap Y^T) as Frobenius products with
// ZB = Z Bp^T and ZA = Z Ap^T (one block, fixed order)
__global__ void k_acfdt_dots(int nS, const double* __restrict__ Z, const double* __restrict__ ZB,
                             const double* __restrict__ ZA, double* __restrict__ out) {
  __shared__ double red[32];
  const long long n = (long long)nS, total = n * n;
  double s = 0.0;
  for (long long idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const long long m = idx % n, ia = idx / n;
    const long long ox = m + 2 * n * ia, oy = ox + n;
    s += Z[ox] * ZB[oy] + Z[oy] * ZB[ox] + Z[ox] * ZA[ox] + Z[oy] * ZA[oy];
  }
  s = qk_block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

__global__ void k_trace_d(int n, const double* __restrict__ A, double* __restrict__ out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += A[(long long)i * (n + 1)];
  s = qk_block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

int grid_1d(qk_ctx* ctx, long long total) {
  long long b = (total + 255) / 256;
  const long long cap = 64LL * ctx->num_sms;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

// Screening at lambda (dRPA singlet at eW, RGW_phBSE.f90:89-95 / RGW_phACFDT.f90:94-103) and
// the two static-kernel products G1 (-> KA) and G2 (-> KB, unless TDA), with the kernel's
// lambda^2.  dA, dB (nS^2 each) are scratch.
static int bse_kernels(qk_ctx* ctx, int TDA_W, int TDA, double eta, double lam, int N, int nC,
                       int nO, int nR, const double* ERI, const double* eW, double* dA,
                       double* dB, double** G1_out, double** G2_out) {
  const int no = nO - nC, nv = N - nO - nR, nS = no * nv;
  const size_t S2 = (size_t)nS * nS, N2 = (size_t)N * N;
  double* sm;
  QK_TRY(qk_wst(ctx, W_BSE, 3 * (size_t)nS + 32, &sm));
  double* OmRPA = sm;
  double* f = sm + nS;
  double* scal = sm + 3 * nS;
  QK_TRY(qk_launch_build_AB(ctx, 0, 1, 1, N, nC, nO, nR, lam, eW, ERI, dA));
  if (!TDA_W) QK_TRY(qk_launch_build_AB(ctx, 1, 1, 1, N, nC, nO, nR, lam, eW, ERI, dB));
  double* XpY = nullptr;
  QK_TRY(phrlr_dev(ctx, TDA_W, nS, dA, dB, OmRPA, &XpY, nullptr, scal, 1));
  double *slab, *rho;
  QK_TRY(qk_wst(ctx, W_SLAB, N2 * nS, &slab));
  QK_TRY(qk_wst(ctx, W_RHO, N2 * nS, &rho));
  QK_TRY(qk_launch_slab_gather(ctx, N, nC, nO, nR, ERI, slab));
  QK_TRY(qk_dgemm(ctx, 'N', 'T', (int)N2, nS, nS, 1.0, slab, (long long)N2, 0, XpY, nS, 0, 0.0,
                  rho, (long long)N2, 0, 1));
  // ---- static kernels (RGW_phBSE_static_kernel_A/B.f90:32-52) ----
  k_bse_weights<<<grid_1d(ctx, nS), 256, 0, ctx->stream>>>(nS, eta, lam * lam, OmRPA, f);
  QK_LAUNCHED();
  const size_t o2 = (size_t)no * no, v2 = (size_t)nv * nv;
  double *R, *G;
  QK_TRY(qk_wst(ctx, W_BSER, (o2 + v2 + 2 * (size_t)nS) * nS, &R));
  QK_TRY(qk_wst(ctx, W_BSEK, 2 * S2, &G));
  double* Roo = R;
  double* Rvv = Roo + o2 * nS;
  double* Rov = Rvv + v2 * nS;
  double* Rvo = Rov + (size_t)nS * nS;
  double* G1 = G;
  double* G2 = G + S2;
  k_rho_block<<<grid_1d(ctx, (long long)o2 * nS), 256, 0, ctx->stream>>>(N, nS, nC, no, nC, no,
                                                                          rho, f, Roo);
  QK_LAUNCHED();
  k_rho_block<<<grid_1d(ctx, (long long)v2 * nS), 256, 0, ctx->stream>>>(N, nS, nO, nv, nO, nv,
                                                                          rho, nullptr, Rvv);
  QK_LAUNCHED();
  QK_TRY(qk_dgemm(ctx, 'N', 'T', (int)o2, (int)v2, nS, 1.0, Roo, (long long)o2, 0, Rvv,
                  (long long)v2, 0, 0.0, G1, (long long)o2, 0, 1));
  if (!TDA) {
    k_rho_block<<<grid_1d(ctx, (long long)S2), 256, 0, ctx->stream>>>(N, nS, nC, no, nO, nv, rho,
                                                                       f, Rov);
    QK_LAUNCHED();
    k_rho_block<<<grid_1d(ctx, (long long)S2), 256, 0, ctx->stream>>>(N, nS, nO, nv, nC, no, rho,
                                                                       nullptr, Rvo);
    QK_LAUNCHED();
    QK_TRY(qk_dgemm(ctx, 'N', 'T', nS, nS, nS, 1.0, Rov, nS, 0, Rvo, nS, 0, 0.0, G2, nS, 0, 1));
  }
  *G1_out = G1;
  *G2_out = G2;
  return QK_OK;
}

int qk_bse_dev(qk_ctx* ctx, int TDA_W, int TDA, int singlet, int triplet, int exchange_kernel,
               double eta, int N, int nC, int nO, int nR, const double* ERI, const double* eW,
               const double* eGW, double* hEcBSE, double* OmS, double* OmT) {
  const int no = nO - nC, nv = N - nO - nR, nS = no * nv;
  if (no <= 0 || nv <= 0) return qk_fail(ctx, QK_ERR_ARG, "bad orbital counts");
  const size_t S2 = (size_t)nS * nS;
  double *dA, *sm, *G1, *G2;
  QK_TRY(qk_wst(ctx, W_HOST_A, 2 * S2, &dA));
  double* dB = dA + S2;
  QK_TRY(bse_kernels(ctx, TDA_W, TDA, eta, 1.0, N, nC, nO, nR, ERI, eW, dA, dB, &G1, &G2));
  QK_TRY(qk_wst(ctx, W_BSE, 3 * (size_t)nS + 32, &sm));
  double* OmBSE = sm + 2 * nS;
  double* scal = sm + 3 * nS;
  // ---- singlet and triplet manifolds (RGW_phBSE.f90:106-178) ----
  double ec[2] = {0.0, 0.0};
  for (int ispin = 1; ispin <= 2; ++ispin) {
    if ((ispin == 1 && !singlet) || (ispin == 2 && !triplet)) continue;
    QK_TRY(qk_launch_build_AB(ctx, 0, ispin, 0, N, nC, nO, nR, 1.0, eGW, ERI, dA));
    k_bse_add_KA<<<grid_1d(ctx, (long long)S2), 256, 0, ctx->stream>>>(no, nv, G1, dA);
    QK_LAUNCHED();
    if (!TDA) {
      QK_TRY(qk_launch_build_AB(ctx, 1, ispin, 0, N, nC, nO, nR, 1.0, eGW, ERI, dB));
      k_bse_add_KB<<<grid_1d(ctx, (long long)S2), 256, 0, ctx->stream>>>(no, nv, G2, dB);
      QK_LAUNCHED();
    }
    QK_TRY(phrlr_dev(ctx, TDA, nS, dA, dB, OmBSE, nullptr, nullptr, scal, 0));
    double* dst = ispin == 1 ? OmS : OmT;
    if (dst)
      QK_CK(cudaMemcpyAsync(dst, OmBSE, nS * sizeof(double), cudaMemcpyDeviceToDevice,
                            ctx->stream));
    QK_CK(cudaMemcpyAsync(&ec[ispin - 1], scal + 2, sizeof(double), cudaMemcpyDeviceToHost,
                          ctx->stream));
    QK_CK(cudaStreamSynchronize(ctx->stream));
  }
  ec[1] *= 3.0;  // RGW_phBSE.f90:184
  if (exchange_kernel) {
    ec[0] *= 0.5;
    ec[1] *= 0.5;
  }
  if (hEcBSE) {
    hEcBSE[0] = ec[0];
    hEcBSE[1] = ec[1];
  }
  return QK_OK;
}

// Adiabatic-connection correlation energy of phBSE@GW (GW/RGW_phACFDT.f90:1-219): per spin, a
// 21-point Gauss-Legendre quadrature over the coupling strength lambda in [0, 1] (the nodes and
// weights of include/quadrature.h, computed here) of
//   Ec(lambda) = tr(X Bp Y^T + Y Bp X^T) + tr(X Ap X^T + Y Ap Y^T) - tr(Ap)
// (RPA/phACFDT_correlation_energy.f90:56-80), with X, Y from the BSE Casida at lambda:
// A = phRLR_A(ispin, dRPA = false, lambda, eGW) + KA, B = phRLR_B(...) + KB, the kernels at
// lambda = 1 or, with doXBS, rebuilt from a lambda-scaled screening at every node.
// EcAC = 1/2 sum_k w_k Ec(lambda_k), scaled by 1/2 (singlet) or 3/2 (triplet) with the exchange
// kernel, as the reference does.  Each node: two nS^3 GEMMs of [X; Y] with Bp^T and Ap^T.
int qk_bse_acfdt_dev(qk_ctx* ctx, int exchange_kernel, int doXBS, int TDA_W, int TDA, int singlet,
                     int triplet, double eta, int N, int nC, int nO, int nR, const double* ERI,
                     const double* eW, const double* eGW, double* hEcAC) {
  const int no = nO - nC, nv = N - nO - nR, nS = no * nv;
  if (no <= 0 || nv <= 0) return qk_fail(ctx, QK_ERR_ARG, "bad orbital counts");
  constexpr int NAC = 21;  // include/quadrature.h: nAC
  double x[NAC], wq[NAC];
  qk_gauss_legendre_host(NAC, x, wq);
  const size_t S2 = (size_t)nS * nS;
  double *dA, *acf, *G1 = nullptr, *G2 = nullptr;
  QK_TRY(qk_wst(ctx, W_HOST_A, 2 * S2, &dA));
  double* dB = dA + S2;
  if (!doXBS)
    QK_TRY(bse_kernels(ctx, TDA_W, TDA, eta, 1.0, N, nC, nO, nR, ERI, eW, dA, dB, &G1, &G2));
  QK_TRY(qk_wst(ctx, W_ACF, 8 * S2 + (size_t)nS + 64, &acf));
  double* Ap = acf;
  double* Bp = Ap + S2;
  double* Z = Bp + S2;
  double* ZB = Z + 2 * S2;
  double* ZA = ZB + 2 * S2;
  double* Om = ZA + 2 * S2;
  double* sm = Om + nS;  // [0] tr(Ap), [1] dots, [8..] Casida scalars
  double ec_out[2] = {0.0, 0.0};
  for (int ispin = 1; ispin <= 2; ++ispin) {
    if ((ispin == 1 && !singlet) || (ispin == 2 && !triplet)) continue;
    const double c1 = ispin == 1 ? 2.0 : 0.0;  // 1 + delta_spin
    const double c2 = exchange_kernel ? 1.0 : 0.0;
    k_acfdt_ApBp<<<grid_1d(ctx, (long long)S2), 256, 0, ctx->stream>>>(N, nC, nO, nv, c1, c2, ERI,
                                                                        Ap, Bp);
    QK_LAUNCHED();
    k_trace_d<<<1, 1024, 0, ctx->stream>>>(nS, Ap, sm);
    QK_LAUNCHED();
    double sum = 0.0;
    for (int k = 0; k < NAC; ++k) {
      const double lam = 0.5 * (1.0 + x[k]);
      if (doXBS)
        QK_TRY(bse_kernels(ctx, TDA_W, TDA, eta, lam, N, nC, nO, nR, ERI, eW, dA, dB, &G1, &G2));
      QK_TRY(qk_launch_build_AB(ctx, 0, ispin, 0, N, nC, nO, nR, lam, eGW, ERI, dA));
      k_bse_add_KA<<<grid_1d(ctx, (long long)S2), 256, 0, ctx->stream>>>(no, nv, G1, dA);
      QK_LAUNCHED();
      if (!TDA) {
        QK_TRY(qk_launch_build_AB(ctx, 1, ispin, 0, N, nC, nO, nR, lam, eGW, ERI, dB));
        k_bse_add_KB<<<grid_1d(ctx, (long long)S2), 256, 0, ctx->stream>>>(no, nv, G2, dB);
        QK_LAUNCHED();
      }
      double *XpY = nullptr, *XmY = nullptr;
      QK_TRY(phrlr_dev(ctx, TDA, nS, dA, dB, Om, &XpY, &XmY, sm + 8, 1));
      k_acfdt_xy<<<grid_1d(ctx, (long long)S2), 256, 0, ctx->stream>>>(nS, XpY, XmY, Z);
      QK_LAUNCHED();
      QK_TRY(qk_dgemm(ctx, 'N', 'T', 2 * nS, nS, nS, 1.0, Z, 2 * nS, 0, Bp, nS, 0, 0.0, ZB,
                      2 * nS, 0, 1));
      QK_TRY(qk_dgemm(ctx, 'N', 'T', 2 * nS, nS, nS, 1.0, Z, 2 * nS, 0, Ap, nS, 0, 0.0, ZA,
                      2 * nS, 0, 1));
      k_acfdt_dots<<<1, 1024, 0, ctx->stream>>>(nS, Z, ZB, ZA, sm + 1);
      QK_LAUNCHED();
      double h[2];
      QK_CK(cudaMemcpyAsync(h, sm, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      QK_CK(cudaStreamSynchronize(ctx->stream));
      sum += (0.5 * wq[k]) * (h[1] - h[0]);  // wAC = w/2 on [0, 1]
    }
    double ec = 0.5 * sum;                                     // RGW_phACFDT.f90:151, :208
    if (exchange_kernel) ec *= ispin == 1 ? 0.5 : 1.5;         // :153, :210
    ec_out[ispin - 1] = ec;
  }
  if (hEcAC) {
    hEcAC[0] = ec_out[0];
    hEcAC[1] = ec_out[1];
  }
  return QK_OK;
}
