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

__global__ void k_bse_weights(int nS, double eta, const double* __restrict__ Om,
                              double* __restrict__ f) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nS; k += gridDim.x * blockDim.x)
    f[k] = 4.0 * (Om[k] / (Om[k] * Om[k] + eta * eta));
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

int grid_1d(qk_ctx* ctx, long long total) {
  long long b = (total + 255) / 256;
  const long long cap = 64LL * ctx->num_sms;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace

int qk_bse_dev(qk_ctx* ctx, int TDA_W, int TDA, int singlet, int triplet, int exchange_kernel,
               double eta, int N, int nC, int nO, int nR, const double* ERI, const double* eW,
               const double* eGW, double* hEcBSE, double* OmS, double* OmT) {
  const int no = nO - nC, nv = N - nO - nR, nS = no * nv;
  if (no <= 0 || nv <= 0) return qk_fail(ctx, QK_ERR_ARG, "bad orbital counts");
  const size_t S2 = (size_t)nS * nS, N2 = (size_t)N * N;
  double *dA, *sm;
  QK_TRY(qk_wst(ctx, W_HOST_A, 2 * S2, &dA));
  double* dB = dA + S2;
  QK_TRY(qk_wst(ctx, W_BSE, 3 * (size_t)nS + 32, &sm));
  double* OmRPA = sm;
  double* f = sm + nS;
  double* OmBSE = sm + 2 * nS;
  double* scal = sm + 3 * nS;
  // ---- screening: dRPA singlet at eW (RGW_phBSE.f90:89-95) ----
  QK_TRY(qk_launch_build_AB(ctx, 0, 1, 1, N, nC, nO, nR, 1.0, eW, ERI, dA));
  if (!TDA_W) QK_TRY(qk_launch_build_AB(ctx, 1, 1, 1, N, nC, nO, nR, 1.0, eW, ERI, dB));
  double* XpY = nullptr;
  QK_TRY(phrlr_dev(ctx, TDA_W, nS, dA, dB, OmRPA, &XpY, nullptr, scal, 1));
  double *slab, *rho;
  QK_TRY(qk_wst(ctx, W_SLAB, N2 * nS, &slab));
  QK_TRY(qk_wst(ctx, W_RHO, N2 * nS, &rho));
  QK_TRY(qk_launch_slab_gather(ctx, N, nC, nO, nR, ERI, slab));
  QK_TRY(qk_dgemm(ctx, 'N', 'T', (int)N2, nS, nS, 1.0, slab, (long long)N2, 0, XpY, nS, 0, 0.0,
                  rho, (long long)N2, 0, 1));
  // ---- static kernels (RGW_phBSE_static_kernel_A/B.f90:32-52) ----
  k_bse_weights<<<grid_1d(ctx, nS), 256, 0, ctx->stream>>>(nS, eta, OmRPA, f);
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
