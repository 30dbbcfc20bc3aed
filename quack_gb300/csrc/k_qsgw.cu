// k_qsgw.cu -- the AO-basis kernels of quasiparticle self-consistent GW (GW/qsRGW.f90:193-345).
//
// Per cycle the driver (qk_api.cu) needs, besides the Casida / excitation-density machinery of
// the G0W0 path:
//   * J and K from the density (AOtoMO/Hartree_matrix_AO_basis.f90:22-32,
//     AOtoMO/exchange_matrix_AO_basis.f90:22-31) -- one pass over the nBas^4 AO tensor;
//   * the MO integrals that the screening and the self-energy read.  The reference transforms
//     the whole tensor (AOtoMO_ERI_RHF.f90, 4 x 2 N^5 flop); only <pj|qb> with j active occupied
//     and b active virtual is read (the excitation-density slab, which holds the Casida block
//     (ia|jb) too), so the driver runs the four quarter transformations with the occupied and
//     virtual coefficient blocks in the positions that shrink the tensor first:
//         <j p|b q> = sum c(mu,j) c(la,p) c(nu,b) c(si,q) <mu la|nu si>
//     (4 N^4 no + 4 N^3 no nv flop; FP64 GEMMs, double-float ones in the mixed tier), and the
//     kernels below permute it into the slab layout and
//     the Casida K -- <pj|qb> = <jp|bq> is the particle-exchange symmetry of any two-electron
//     integral, (ia|jb) = <ji|ba> with real orbitals;
//   * the full correlation self-energy (RGW_self_energy.f90:40-84):
//         Sig(p,q) = sum_(x,m) [2 rho(p,x,m) eps_pxm/(eps_pxm^2 + eta^2)] rho(q,x,m)
//     the weighted factor is formed once (k_qs_weight) and the sum over (x,m) is one GEMM of
//     k = nOrb nS (split over k; FP64, or double-float in the mixed tier like the quarter
//     transforms); the SRG form (RGW_SRG_self_energy.f90:40-80), whose weight
//     depends on p and q together, is a tiled kernel (k_qs_srg_sigma);
//   * symmetrisation, the Fock matrix, and the energy traces (qsRGW.f90:269-310).
#include "qk_internal.cuh"

namespace {

int grid_1d(qk_ctx* ctx, long long total) {
  long long b = (total + 255) / 256;
  const long long cap = 64LL * ctx->num_sms;
  return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// One block per AO slab (r, s) = (third, fourth index), 32 lanes over mu x 8 groups over la:
//   Jp[mu + N (r + N s)] = sum_la ERI(mu,la,r,s) P(la,s)     (J(mu,r) = sum_s Jp)
//   Kp[mu + N (s + N r)] = sum_la ERI(mu,la,r,s) P(la,r)     (K(mu,s) = -sum_r Kp)
// so the tensor is read once, coalesced, for both matrices.
constexpr int JK_LANES = 32, JK_GROUPS = 8;
__global__ void __launch_bounds__(JK_LANES* JK_GROUPS)
    k_qs_jk_slabs(int N, const double* __restrict__ ERI, const double* __restrict__ P,
                  double* __restrict__ Jp, double* __restrict__ Kp) {
  extern __shared__ double sm[];
  double* Ps = sm;          // P(:, s)
  double* Pr = sm + N;      // P(:, r)
  double* red = sm + 2 * N; // [2][GROUPS][LANES]
  const long long N1 = N, N2 = N1 * N1;
  const int r = blockIdx.x % N, s = blockIdx.x / N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    Ps[i] = P[i + N1 * s];
    Pr[i] = P[i + N1 * r];
  }
  __syncthreads();
  const double* slab = ERI + N2 * (r + N1 * s);
  const int lane = threadIdx.x % JK_LANES, g = threadIdx.x / JK_LANES;
  for (int m0 = 0; m0 < N; m0 += JK_LANES) {
    const int mu = m0 + lane;
    double a = 0.0, b = 0.0;
    if (mu < N) {
      for (int la = g; la < N; la += JK_GROUPS) {
        const double x = slab[mu + N1 * la];
        a = fma(x, Ps[la], a);
        b = fma(x, Pr[la], b);
      }
    }
    red[g * JK_LANES + lane] = a;
    red[(JK_GROUPS + g) * JK_LANES + lane] = b;
    __syncthreads();
    if (g == 0 && mu < N) {
      double sa = 0.0, sb = 0.0;
      for (int k = 0; k < JK_GROUPS; ++k) {
        sa += red[k * JK_LANES + lane];
        sb += red[(JK_GROUPS + k) * JK_LANES + lane];
      }
      Jp[mu + N1 * (r + N1 * s)] = sa;
      Kp[mu + N1 * (s + N1 * r)] = sb;
    }
    __syncthreads();
  }
}

// out[i] = scale * sum_k in[i + n k]
__global__ void k_qs_sum_last(long long n, int nk, const double* __restrict__ in, double scale,
                              double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nk; ++k) s += in[i + n * k];
    out[i] = scale * s;
  }
}

// slab[p + N q + N^2 (jl nv + bl)] = R[jl + no (p + N (bl + nv q))]      (R = <j p|b q>)
__global__ void k_qs_slab(int N, int no, int nv, const double* __restrict__ R,
                          double* __restrict__ slab) {
  const long long N1 = N, N2 = N1 * N1, total = N2 * no * nv;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long pq = idx % N2, jb = idx / N2;
    const int p = (int)(pq % N1), q = (int)(pq / N1);
    const int jl = (int)(jb / nv), bl = (int)(jb % nv);
    slab[idx] = R[jl + no * (p + N1 * (bl + (long long)nv * q))];
  }
}

// K[ia + nS jb] = (ia|jb) = <j i|b a> = R[jl + no (i + N (bl + nv a))]
__global__ void k_qs_kmat(int N, int nC, int nO, int no, int nv, const double* __restrict__ R,
                          double* __restrict__ K) {
  const long long nS = (long long)no * nv, total = nS * nS, N1 = N;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long ia = idx % nS, jb = idx / nS;
    const int il = (int)(ia / nv), al = (int)(ia % nv);
    const int jl = (int)(jb / nv), bl = (int)(jb % nv);
    K[idx] = R[jl + no * ((nC + il) + N1 * (bl + (long long)nv * (nO + al)))];
  }
}

// A[p + N x + N^2 m] = 2 rho(p,x,m) eps/(eps^2 + eta^2), eps = e_p - e_x + Om_m (x occupied) or
// e_p - e_x - Om_m (x virtual); 0 unless p and x are active (RGW_self_energy.f90:47-82).
__global__ void k_qs_weight(int N, int nC, int nO, int nR, int nS, double eta,
                            const double* __restrict__ e, const double* __restrict__ Om,
                            const double* __restrict__ rho, double* __restrict__ A) {
  const long long N1 = N, N2 = N1 * N1, total = N2 * nS;
  const double eta2 = eta * eta;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const long long px = idx % N2;
    const int m = (int)(idx / N2);
    const int p = (int)(px % N1), x = (int)(px / N1);
    double v = 0.0;
    if (p >= nC && p < N - nR && x >= nC && x < N - nR) {
      const double eps = x < nO ? (e[p] - e[x]) + Om[m] : (e[p] - e[x]) - Om[m];
      v = 2.0 * rho[idx] * (eps / (eps * eps + eta2));
    }
    A[idx] = v;
  }
}

// Sym(p,q) = (Sig(p,q) + Sig(q,p))/2 on the active block, 0 elsewhere (qsRGW.f90:269)
__global__ void k_qs_sym(int N, int nC, int nR, const double* __restrict__ Sig,
                         double* __restrict__ out) {
  const long long N1 = N, total = N1 * N1;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int p = (int)(idx % N1), q = (int)(idx / N1);
    const bool act = p >= nC && p < N - nR && q >= nC && q < N - nR;
    out[idx] = act ? 0.5 * (Sig[idx] + Sig[q + N1 * p]) : 0.0;
  }
}

// zero the rows and columns of inactive orbitals in place (RGW_self_energy.f90:38-84 fills the
// active block only)
__global__ void k_qs_mask(int N, int nC, int nR, double* __restrict__ Sig) {
  const long long N1 = N, total = N1 * N1;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    const int p = (int)(idx % N1), q = (int)(idx / N1);
    if (!(p >= nC && p < N - nR && q >= nC && q < N - nR)) Sig[idx] = 0.0;
  }
}

// SRG-regularised full self-energy (RGW_SRG_self_energy.f90:40-80), tiled over (p,q):
//   Sig(p,q) = sum_(x,m) 2 rho(p,x,m) rho(q,x,m) (1 - g_p g_q) (D_p + D_q)/(D_p^2 + D_q^2),
//   D_p = e_p - e_x +- Om_m, g_p = exp(-s D_p^2).
// A 16 x 16 thread tile of (p,q) per block; the (x,m) range is split over gridDim.z slices whose
// partial sums the caller adds.  Per (x,m) chunk the block stages rho, D and g of its 16 rows
// and 16 columns in shared memory.
constexpr int SRG_T = 16, SRG_CH = 64;
__global__ void __launch_bounds__(SRG_T* SRG_T)
    k_qs_srg_sigma(int N, int nC, int nO, int nR, int nS, double s, const double* __restrict__ e,
                   const double* __restrict__ Om, const double* __restrict__ rho,
                   double* __restrict__ part) {
  __shared__ double rp[SRG_CH][SRG_T], dp[SRG_CH][SRG_T], gp[SRG_CH][SRG_T];
  __shared__ double rq[SRG_CH][SRG_T], dq[SRG_CH][SRG_T], gq[SRG_CH][SRG_T];
  const long long N1 = N, N2 = N1 * N1;
  const int p0 = blockIdx.x * SRG_T, q0 = blockIdx.y * SRG_T;
  const int tx = threadIdx.x % SRG_T, ty = threadIdx.x / SRG_T;
  const int lo = nC, hi = N - nR;               // active orbitals
  const long long nx = hi - lo, K = nx * nS;   // (x, m) pairs, x fastest
  const long long per = (K + gridDim.z - 1) / gridDim.z;
  const long long k0 = per * blockIdx.z, k1 = k0 + per < K ? k0 + per : K;
  double acc = 0.0;
  for (long long kc = k0; kc < k1; kc += SRG_CH) {
    for (int t = threadIdx.x; t < SRG_CH * SRG_T; t += blockDim.x) {
      const int kk = t / SRG_T, r = t % SRG_T;
      const long long k = kc + kk;
      double vr = 0.0, vd = 1.0, vg = 0.0, wr = 0.0, wd = 1.0, wg = 0.0;
      if (k < k1) {
        const int x = lo + (int)(k % nx), m = (int)(k / nx);
        const double om = x < nO ? Om[m] : -Om[m];
        const int p = p0 + r, q = q0 + r;
        if (p >= lo && p < hi) {
          vr = rho[p + N1 * x + N2 * m];
          vd = (e[p] - e[x]) + om;
          vg = exp(-s * vd * vd);
        }
        if (q >= lo && q < hi) {
          wr = rho[q + N1 * x + N2 * m];
          wd = (e[q] - e[x]) + om;
          wg = exp(-s * wd * wd);
        }
      }
      rp[kk][r] = vr; dp[kk][r] = vd; gp[kk][r] = vg;
      rq[kk][r] = wr; dq[kk][r] = wd; gq[kk][r] = wg;
    }
    __syncthreads();
    const int nk = (int)(k1 - kc < SRG_CH ? k1 - kc : SRG_CH);
    for (int kk = 0; kk < nk; ++kk) {
      const double a = rp[kk][tx], b = rq[kk][ty];
      if (a != 0.0 && b != 0.0) {
        const double Dp = dp[kk][tx], Dq = dq[kk][ty];
        const double f = (1.0 - gp[kk][tx] * gq[kk][ty]) * (Dp + Dq) / (Dp * Dp + Dq * Dq);
        acc = fma(2.0 * a * b, f, acc);
      }
    }
    __syncthreads();
  }
  const int p = p0 + tx, q = q0 + ty;
  if (p < N && q < N) part[p + N1 * q + N2 * blockIdx.z] = acc;
}

// F = Hc + J + K/2 + SigCp (qsRGW.f90:280)
__global__ void k_qs_fock(long long n, const double* __restrict__ Hc, const double* __restrict__ J,
                          const double* __restrict__ K, const double* __restrict__ SigCp,
                          double* __restrict__ F) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    F[i] = ((Hc[i] + J[i]) + 0.5 * K[i]) + SigCp[i];
}

// out[0..3] = tr(P T), tr(P V), tr(P J)/2, tr(P K)/4; out[4] = their sum (EqsGW);
// out[5] = max |err| (qsRGW.f90:290-310).  One block.
__global__ void k_qs_energy(int N, const double* __restrict__ P, const double* __restrict__ T,
                            const double* __restrict__ V, const double* __restrict__ J,
                            const double* __restrict__ K, const double* __restrict__ err,
                            double* __restrict__ out) {
  __shared__ double red[32];
  const long long N1 = N, total = N1 * N1;
  double s[4] = {0.0, 0.0, 0.0, 0.0}, mx = 0.0;
  for (long long idx = threadIdx.x; idx < total; idx += blockDim.x) {
    const int i = (int)(idx % N1), j = (int)(idx / N1);
    const long long ji = j + N1 * i;
    const double pij = P[idx];
    s[0] = fma(pij, T[ji], s[0]);
    s[1] = fma(pij, V[ji], s[1]);
    s[2] = fma(pij, J[ji], s[2]);
    s[3] = fma(pij, K[ji], s[3]);
    mx = fmax(mx, fabs(err[idx]));
  }
  double r[4];
  for (int k = 0; k < 4; ++k) r[k] = qk_block_sum(s[k], red);
  const double m = qk_block_max(mx, red);
  if (threadIdx.x == 0) {
    out[0] = r[0];
    out[1] = r[1];
    out[2] = 0.5 * r[2];
    out[3] = 0.25 * r[3];
    out[4] = ((out[0] + out[1]) + out[2]) + out[3];
    out[5] = m;
  }
}

}  // namespace

int qk_qs_jk(qk_ctx* ctx, int N, const double* ERI, const double* P, double* part, double* J,
             double* K) {
  const size_t N1 = N, N3 = N1 * N1 * N1;
  double* Jp = part;
  double* Kp = part + N3;
  const size_t smem = (2 * N1 + 2 * JK_GROUPS * JK_LANES) * sizeof(double);
  if (smem > 48 * 1024) return qk_fail(ctx, QK_ERR_ARG, "qk_qs_jk: nBas %d too large", N);
  k_qs_jk_slabs<<<(unsigned)(N1 * N1), JK_LANES * JK_GROUPS, smem, ctx->stream>>>(N, ERI, P, Jp,
                                                                                  Kp);
  QK_LAUNCHED();
  const long long n2 = (long long)N1 * N1;
  k_qs_sum_last<<<grid_1d(ctx, n2), 256, 0, ctx->stream>>>(n2, N, Jp, 1.0, J);
  QK_LAUNCHED();
  k_qs_sum_last<<<grid_1d(ctx, n2), 256, 0, ctx->stream>>>(n2, N, Kp, -1.0, K);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qs_mo_slab(qk_ctx* ctx, int nBas, int N, int nC, int nO, int nR, const double* c,
                  const double* ERI, double* W1, double* W2, double* slab, double* Kmat, int df) {
  const int no = nO - nC, nv = N - nO - nR;
  const long long N1 = N, B = nBas;
  const double* cocc = c + B * nC;
  const double* cvir = c + B * nO;
  auto gemm = df ? qk_gemm_df : qk_dgemm;
  // <mu la|nu si> -> (la,nu,si,j) -> (nu,si,j,p) -> (si,j,p,b) -> (j,p,b,q); c is nBas x nOrb
  QK_TRY(gemm(ctx, 'T', 'N', (int)(B * B * B), no, nBas, 1.0, ERI, B, 0, cocc, B, 0, 0.0, W1,
              B * B * B, 0, 1));
  QK_TRY(gemm(ctx, 'T', 'N', (int)(B * B * no), N, nBas, 1.0, W1, B, 0, c, B, 0, 0.0, W2,
              B * B * no, 0, 1));
  QK_TRY(gemm(ctx, 'T', 'N', (int)(B * no * N1), nv, nBas, 1.0, W2, B, 0, cvir, B, 0, 0.0, W1,
              B * no * N1, 0, 1));
  QK_TRY(gemm(ctx, 'T', 'N', (int)((long long)no * N1 * nv), N, nBas, 1.0, W1, B, 0, c, B, 0, 0.0,
              W2, (long long)no * N1 * nv, 0, 1));
  const long long nS = (long long)no * nv;
  k_qs_slab<<<grid_1d(ctx, N1 * N1 * nS), 256, 0, ctx->stream>>>(N, no, nv, W2, slab);
  QK_LAUNCHED();
  k_qs_kmat<<<grid_1d(ctx, nS * nS), 256, 0, ctx->stream>>>(N, nC, nO, no, nv, W2, Kmat);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qs_sigma(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                int nS, const double* e, const double* Om, const double* rho, double* W,
                double* Sig, int df) {
  const long long N1 = N, N2 = N1 * N1;
  if (!doSRG) {
    k_qs_weight<<<grid_1d(ctx, N2 * nS), 256, 0, ctx->stream>>>(N, nC, nO, nR, nS, eta, e, Om,
                                                                  rho, W);
    QK_LAUNCHED();
    auto gemm = df ? qk_gemm_df : qk_dgemm;
    return gemm(ctx, 'N', 'T', N, N, (int)(N1 * nS), 1.0, W, N1, 0, rho, N1, 0, 0.0, Sig, N1, 0,
                1);
  }
  const int tiles = (N + SRG_T - 1) / SRG_T;
  const long long K = (long long)(N - nC - nR) * nS;
  long long z = (4LL * ctx->num_sms + (long long)tiles * tiles - 1) / ((long long)tiles * tiles);
  const long long zmax = (K + 4 * SRG_CH - 1) / (4 * SRG_CH);
  if (z > zmax) z = zmax;
  if (z < 1) z = 1;
  if (z > 64) z = 64;
  if (z > nS) z = nS;  // W holds N^2 nS partial sums
  dim3 grid(tiles, tiles, (unsigned)z);
  k_qs_srg_sigma<<<grid, SRG_T * SRG_T, 0, ctx->stream>>>(N, nC, nO, nR, nS, flow, e, Om, rho, W);
  QK_LAUNCHED();
  k_qs_sum_last<<<grid_1d(ctx, N2), 256, 0, ctx->stream>>>(N2, (int)z, W, 1.0, Sig);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qs_sym(qk_ctx* ctx, int N, int nC, int nR, const double* Sig, double* out) {
  k_qs_sym<<<grid_1d(ctx, (long long)N * N), 256, 0, ctx->stream>>>(N, nC, nR, Sig, out);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qs_mask(qk_ctx* ctx, int N, int nC, int nR, double* Sig) {
  k_qs_mask<<<grid_1d(ctx, (long long)N * N), 256, 0, ctx->stream>>>(N, nC, nR, Sig);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qs_fock(qk_ctx* ctx, int N, const double* Hc, const double* J, const double* K,
               const double* SigCp, double* F) {
  const long long n = (long long)N * N;
  k_qs_fock<<<grid_1d(ctx, n), 256, 0, ctx->stream>>>(n, Hc, J, K, SigCp, F);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qs_energy(qk_ctx* ctx, int N, const double* P, const double* T, const double* V,
                 const double* J, const double* K, const double* err, double* out) {
  k_qs_energy<<<1, 1024, 0, ctx->stream>>>(N, P, T, V, J, K, err, out);
  QK_LAUNCHED();
  return QK_OK;
}
