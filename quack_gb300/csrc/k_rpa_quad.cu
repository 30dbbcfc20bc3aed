// k_rpa_quad.cu -- dRPA correlation energy by imaginary-frequency quadrature.
//
// The reference computes EcRPA = (sum_m Omega_m - tr A) / 2 from the eigenvalues of the Casida
// problem (LR/phRLR.f90, called a second time at the G0W0 energies by RG0W0.f90:222-225).  With
// D = diag(e_a - e_i) and K = (ia|jb), the singlet dRPA problem is M = D^1/2 (D + 4K) D^1/2,
// Omega^2 = eig(M), tr A = tr D + 2 tr K, and for any factor K = L L^T (L: nS x r)
//   det(M + w^2) / det(D^2 + w^2) = det(I_r + Q(w)),   Q(w) = 4 L^T diag(d / (d^2 + w^2)) L,
// while  int_0^inf ln((x + w^2)/(y + w^2)) dw = pi (sqrt(x) - sqrt(y))  and
// int_0^inf tr Q(w) dw = 2 pi tr K, so that
//   EcRPA = 1/(2 pi) int_0^inf [ ln det(I + Q(w)) - tr Q(w) ] dw
// exactly.  The integrand is smooth and decays as w^-4; Gauss-Legendre on w = w0 (1+x)/(1-x)
// with w0 = sqrt(d_min d_max) and 24-128 points (by the width d_max/d_min of the spectrum)
// reproduces the eigenvalue route to ~1e-10 Ha.  Cost: r x r problems instead of nS x nS:
//   * the factor: Lov (factorised integrals, r = naux) or a pivoted Cholesky of K (ERI input,
//     stopped at 1e-12 of the largest diagonal; r = the numerical rank);
//   * Q for all points: one batched GEMM with compensated FP32 products, the weights applied
//     as the operand is staged (error ~1e-9 Ha);
//   * ln det(I + Q) - tr Q: blocked FP64 Cholesky carried on S = (Schur complement) - I, so that
//     each pivot contributes (log1p(s) - s) - (Q_ii - s), both second order in Q: no
//     cancellation of the two first-order terms at large w.
// Used by the mixed tier for the EcRPA of the G0W0 energies; every other EcRPA comes from the
// Casida eigenvalues.
#include <cmath>
#include <mutex>
#include <vector>
#include "qk_internal.cuh"

namespace {

constexpr int CB = 64;  // Cholesky block

// d_ia = e_a - e_i (ia = i * nv + a, the Casida ordering) and [min, max] of d
__global__ void k_quad_delta(int nS, int nv, int nC, int nO, const double* __restrict__ e,
                             double* __restrict__ dd, double* __restrict__ mm) {
  __shared__ double smin[32], smax[32];
  double lo = INFINITY, hi = -INFINITY;
  for (int ia = threadIdx.x; ia < nS; ia += blockDim.x) {
    const int ip = ia / nv, ap = ia - ip * nv;
    const double v = e[ap + nO] - e[ip + nC];
    dd[ia] = v;
    lo = fmin(lo, v);
    hi = fmax(hi, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) { smin[w] = lo; smax[w] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) { lo = fmin(lo, smin[i]); hi = fmax(hi, smax[i]); }
    mm[0] = fmin(lo, smin[0]);
    mm[1] = fmax(hi, smax[0]);
  }
}

// K(ia, jb) = (ia|jb) = ERI(b, i, j, a) (Fortran ERI(p,q,r,s) at p + N q + N^2 r + N^3 s),
// column-major nS x nS; tiles of 32 a x 32 b for one (i, j), read along b, written along a.
__global__ void k_gather_K(int N, int nC, int nO, int nR, const double* __restrict__ ERI,
                           double* __restrict__ K) {
  __shared__ double t[32][33];
  const int no = nO - nC, nv = N - nO - nR;
  const long long nS = (long long)no * nv;
  const int ij = blockIdx.z;
  const int ip = ij / no, jp = ij - ip * no;
  const long long N1 = N, N2 = N1 * N1, N3 = N2 * N1;
  const int a0 = blockIdx.x * 32, b0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  for (int r = ty; r < 32; r += 8) {
    const int ap = a0 + r, bp = b0 + tx;
    t[r][tx] = (ap < nv && bp < nv)
                   ? __ldg(ERI + (bp + nO) + N1 * (ip + nC) + N2 * (jp + nC) + N3 * (ap + nO))
                   : 0.0;
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int ap = a0 + tx, bp = b0 + r;
    if (ap < nv && bp < nv) K[(long long)ip * nv + ap + nS * ((long long)jp * nv + bp)] = t[tx][r];
  }
}

struct PcArgs {
  const double* K;
  long long ldk;
  int nS, rmax;
  double tol_rel;
  double* Lt;                // rmax x nS, column-major: Lt[t + rmax * i] = L(i, t)
  double* r;                 // residual diagonal
  int* done;                 // pivoted rows
  unsigned long long* gkey;  // pivot candidates of three consecutive steps (zeroed before launch)
  int* rank;
  unsigned* bar;
  int* status;
};

// Pivot candidate key: the residual rounded to FP32 (whose bit pattern orders non-negative
// values) in the high word, the complemented row index (ties to the lowest row) in the low word;
// integer max then selects a pivot of (to FP32 rounding) the largest residual.
__device__ __forceinline__ unsigned long long pc_key(double v, int i) {
  const float f = v > 0.0 ? (float)v : 0.0f;
  return ((unsigned long long)__float_as_uint(f) << 32) |
         (unsigned long long)(0xFFFFFFFFu - (unsigned)i);
}

// Left-looking pivoted Cholesky of K in one cooperative launch.  Per pivot: thread 0 of every
// CTA reads the winning key of the previous step and the pivot's exact residual, each warp forms
// one row of the new column (l_i = (K_ip - L_i . L_p) / sqrt(r_p)) and folds its residual's key into the CTA's shared maximum, and one bounded grid barrier
// -- whose arrival carries the CTA's key to a global atomic maximum -- closes the step.  The
// factor does not depend on the order of the atomics: every CTA reads the same final maximum.
// The pivot row is staged in shared memory and each row's entries are loaded 4 per lane at once,
// so a step costs a few L2 round trips plus the barrier (~12 us per pivot at nS = 3600).
__global__ void __launch_bounds__(1024, 1) k_pchol(PcArgs a) {
  extern __shared__ double lp[];  // the pivot row of L (a.rmax doubles)
  __shared__ unsigned long long s_key;
  __shared__ double s_rp, s_inv, s_tol;
  __shared__ int s_p, s_ok;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int gw = blockIdx.x * 32 + warp, totw = gridDim.x * 32;
  unsigned epoch = 0;
  // grid barrier (bounded) that first publishes the CTA's candidate into gkey[slot]
  auto barrier = [&](int slot) -> bool {
    __syncthreads();
    if (tid == 0) {
      int ok = 1;
      atomicMax(a.gkey + slot, s_key);
      s_key = 0ull;
      epoch++;
      const unsigned target = epoch * gridDim.x;
      const unsigned limit = qk_spin_limit(a.status);
      __threadfence();
      atomicAdd(a.bar, 1u);
      unsigned spins = 0;
      while (qk_ld_acquire(a.bar) < target) {
        if (++spins > limit) { atomicOr(a.status, QKD_BARRIER_TIMEOUT); ok = 0; break; }
        if (spins > 64) __nanosleep(32);
      }
      if (ok && (*((volatile int*)a.status) & QKD_BARRIER_TIMEOUT)) ok = 0;
      __threadfence();
      s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
  };

  if (tid == 0) s_key = 0ull;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + tid; i < a.nS; i += gridDim.x * blockDim.x) {
    const double x = a.K[i + a.ldk * i];
    a.r[i] = x;
    a.done[i] = 0;
    atomicMax(&s_key, pc_key(x, i));
  }
  if (!barrier(0)) return;
  int q = 0;
  for (; q < a.rmax; ++q) {
    if (tid == 0) {
      const unsigned long long k = __ldcg(a.gkey + q % 3);
      const int p = (int)(0xFFFFFFFFu - (unsigned)(k & 0xFFFFFFFFull));
      double rp = -1.0;
      if (k != 0ull && p >= 0 && p < a.nS) rp = __ldcg(a.r + p);
      s_p = p;
      s_rp = rp;
      s_inv = rp > 0.0 ? qk_rsqrt(rp) : 0.0;
      if (q == 0) s_tol = a.tol_rel * rp;  // relative to the largest diagonal
      if (blockIdx.x == 0) a.gkey[(q + 2) % 3] = 0ull;  // read two steps ago, written next step
    }
    __syncthreads();
    const double rp = s_rp, tol = s_tol, inv = s_inv;
    const int p = s_p;
    if (!(rp > tol) || p < 0 || p >= a.nS) break;  // uniform: every CTA read the same key
    for (int t = tid; t < q; t += blockDim.x) lp[t] = __ldcg(a.Lt + t + (long long)a.rmax * p);
    __syncthreads();
    for (int i = gw; i < a.nS; i += totw) {
      double* li = a.Lt + (long long)a.rmax * i;
      const double kip = lane == 0 ? a.K[i + a.ldk * p] : 0.0;  // issued ahead of the dot
      double s0 = 0.0, s1 = 0.0;
      // the row's entries in batches of 4 loads per lane, issued before their FMAs
      for (int t0 = 0; t0 < q; t0 += 128) {
        double x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int t = t0 + lane + 32 * u;
          x[u] = t < q ? li[t] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 4; u += 2) {
          const int t = t0 + lane + 32 * u;
          if (t < q) s0 = fma(x[u], lp[t], s0);
          if (t + 32 < q) s1 = fma(x[u + 1], lp[t + 32], s1);
        }
      }
      double s = s0 + s1;
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      if (lane == 0) {
        double l = 0.0, rn = a.r[i];
        if (i == p) {
          l = sqrt(rp);  // L_pp
          rn = 0.0;
          a.done[i] = 1;
        } else if (!a.done[i]) {
          l = (kip - s) * inv;
          rn = rn - l * l;
          atomicMax(&s_key, pc_key(rn, i));
        }
        li[q] = l;
        a.r[i] = rn;
      }
    }
    if (!barrier((q + 1) % 3)) return;
  }
  if (blockIdx.x == 0 && tid == 0) *a.rank = q;
}

// L (nS x r, column-major) from Lt (rmax x nS): 32 x 32 tiles through shared memory
__global__ void k_lt_transpose(int nS, int r, int rmax, const double* __restrict__ Lt,
                               double* __restrict__ L) {
  __shared__ double t[32][33];
  const int i0 = blockIdx.x * 32, t0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;
  for (int k = ty; k < 32; k += 8) {
    const int i = i0 + k, tt = t0 + tx;
    t[k][tx] = (i < nS && tt < r) ? Lt[tt + (long long)rmax * i] : 0.0;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int i = i0 + tx, tt = t0 + k;
    if (i < nS && tt < r) L[i + (long long)nS * tt] = t[tx][k];
  }
}

// FP32 weights c_q(i) = 4 d_i / (d_i^2 + w_q^2) of every point (Q_q = L^T diag(c_q) L)
__global__ void k_quad_weights(int nS, int nq, const double* __restrict__ dd,
                               const double* __restrict__ om, float* __restrict__ wq) {
  const int total = nS * nq;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int q = idx / nS, i = idx - q * nS;
    const double d = dd[i], w = om[q];
    wq[idx] = (float)(4.0 * d / fma(d, d, w * w));
  }
}

// diag(Q_q) saved before the factorisation overwrites it
__global__ void k_quad_diag(int r, int nch, const double* __restrict__ Q, double* __restrict__ qd) {
  const int total = r * nch;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const int q = idx / r, i = idx - q * r;
    qd[idx] = Q[(long long)q * r * r + i + (long long)r * i];
  }
}

// Diagonal block kb..kb+nb of every matrix: unblocked Cholesky of I + S (S stored, the identity
// implicit), L11 written back, and the pivots' contributions to ln det(I+Q) - tr Q added to acc.
__global__ void __launch_bounds__(256) k_chol_blk(int r, int kb, int nb, double* __restrict__ S,
                                                  const double* __restrict__ qd,
                                                  double* __restrict__ acc) {
  __shared__ double A[CB][CB + 1];
  __shared__ double sv[CB];
  __shared__ double s_inv;
  __shared__ double red[8];
  const int q = blockIdx.x, tid = threadIdx.x;
  double* Sq = S + (long long)q * r * r;
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int j = idx % nb, k = idx / nb;
    A[j][k] = (j >= k) ? Sq[(kb + j) + (long long)r * (kb + k)] : 0.0;
  }
  __syncthreads();
  for (int c = 0; c < nb; ++c) {
    if (tid == 0) {
      const double s = A[c][c];
      sv[c] = s;
      const double l = sqrt(1.0 + s);
      A[c][c] = l;
      s_inv = 1.0 / l;
    }
    __syncthreads();
    const double inv = s_inv;
    for (int j = c + 1 + tid; j < nb; j += blockDim.x) A[j][c] *= inv;
    __syncthreads();
    const int m = nb - c - 1;
    for (int idx = tid; idx < m * m; idx += blockDim.x) {
      const int jj = idx % m, kk = idx / m;
      if (jj >= kk) {
        const int j = c + 1 + jj, k = c + 1 + kk;
        A[j][k] = fma(-A[j][c], A[k][c], A[j][k]);
      }
    }
    __syncthreads();
  }
  double t = 0.0;
  for (int c = tid; c < nb; c += blockDim.x) {
    const double s = sv[c];
    t += (log1p(s) - s) - (qd[(long long)q * r + kb + c] - s);
  }
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((tid & 31) == 0) red[tid >> 5] = t;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
    acc[q] += s;
  }
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int j = idx % nb, k = idx / nb;
    if (j >= k) Sq[(kb + j) + (long long)r * (kb + k)] = A[j][k];
  }
}

// Panel below the diagonal block: P = S(rows, kb:kb+nb) L11^-T, one row per thread, held in
// registers; column-oriented so that the updates of one step are independent.
constexpr int TRSM_THREADS = 128;
constexpr size_t TRSM_SMEM = sizeof(double) * ((size_t)CB * (CB + 1) + CB + (size_t)CB * TRSM_THREADS);

// Rows below the diagonal block: S_row <- S_row L^-T (forward substitution over the block's
// columns, one thread per row).  The row being solved lives in shared memory (column c of all
// the CTA's rows contiguous, so the accesses are conflict-free): a CB-long row in registers
// spilled, as the compiler keeps the unrolled loop's operands live.
__global__ void __launch_bounds__(TRSM_THREADS) k_chol_trsm(int r, int kb, int nb,
                                                            double* __restrict__ S) {
  extern __shared__ double sm_trsm[];
  double* L = sm_trsm;                      // CB x (CB + 1)
  double* rinv = L + CB * (CB + 1);         // CB
  double* xs = rinv + CB;                   // CB x TRSM_THREADS
  const int q = blockIdx.y, tid = threadIdx.x;
  double* Sq = S + (long long)q * r * r;
  for (int idx = tid; idx < nb * nb; idx += blockDim.x) {
    const int j = idx % nb, k = idx / nb;
    L[j * (CB + 1) + k] = (j >= k) ? Sq[(kb + j) + (long long)r * (kb + k)] : 0.0;
  }
  __syncthreads();
  for (int c = tid; c < nb; c += blockDim.x) rinv[c] = 1.0 / L[c * (CB + 1) + c];
  __syncthreads();
  const int row = kb + nb + blockIdx.x * blockDim.x + tid;
  if (row >= r) return;
  double* x = xs + tid;
  for (int c = 0; c < nb; ++c) x[c * TRSM_THREADS] = Sq[row + (long long)r * (kb + c)];
  for (int c = 0; c < nb; ++c) {
    const double xc = x[c * TRSM_THREADS] * rinv[c];
    x[c * TRSM_THREADS] = xc;
    for (int k = c + 1; k < nb; ++k)
      x[k * TRSM_THREADS] = fma(-xc, L[k * (CB + 1) + c], x[k * TRSM_THREADS]);
  }
  for (int c = 0; c < nb; ++c) Sq[row + (long long)r * (kb + c)] = x[c * TRSM_THREADS];
}

__global__ void k_quad_final(int nq, const double* __restrict__ wt, const double* __restrict__ acc,
                             double* __restrict__ Ec) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < nq; ++q) s = fma(wt[q], acc[q], s);
    *Ec = s * (0.5 / M_PI);
  }
}

// points for the width d_max / d_min of the spectrum (0: too wide, use the eigenvalues); the
// table keeps the quadrature error below ~1e-9 Ha on dRPA problems of each width
int quad_points(double ratio) {
  if (ratio <= 40.0) return 24;
  if (ratio <= 250.0) return 32;
  if (ratio <= 2000.0) return 48;
  if (ratio <= 6000.0) return 64;
  if (ratio <= 20000.0) return 96;
  if (ratio <= 60000.0) return 128;
  return 0;
}

__global__ void k_quad_nan(double* Ec, int* status) {
  *Ec = NAN;
  atomicOr(status, QKD_NEG_AMB);
}

}  // namespace

void qk_gauss_legendre_host(int n, double* x, double* w) {
  // roots of P_n by Newton from the asymptotic guesses cos(pi (k - 1/4) / (n + 1/2)); P_n and
  // P_n' by the three-term recurrence; weights 2 / ((1 - x^2) P_n'(x)^2); nodes ascending
  for (int k = 0; k < (n + 1) / 2; ++k) {
    double z = cos(M_PI * (k + 0.75) / (n + 0.5));
    double dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = z;
      for (int j = 2; j <= n; ++j) {
        const double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1.0; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
      const double dz = p1 / dp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    {
      double p0 = 1.0, p1 = z;
      for (int j = 2; j <= n; ++j) {
        const double p2 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p0) / j;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1.0; }
      dp = n * (z * p1 - p0) / (z * z - 1.0);
    }
    const double wk = 2.0 / ((1.0 - z * z) * dp * dp);
    x[k] = -z;
    x[n - 1 - k] = z;
    w[k] = w[n - 1 - k] = wk;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

int qk_rpa_ec_quad(qk_ctx* ctx, int N, int nC, int nO, int nR, const double* e, const double* ERI,
                   const double* Lov, int naux, double* Ec, int* applied, bool gap_only) {
  *applied = 0;
  const int no = nO - nC, nv = N - nO - nR, nS = no * nv;
  if (nS <= 0 || (!ERI && !Lov)) return QK_OK;
  double *dd = nullptr, *small = nullptr;
  QK_TRY(qk_wst(ctx, W_QUAD, (size_t)nS + 1024, &dd));
  small = dd + nS;  // [0,2): d range; [8,136): nodes; [136,264): weights; [264,392): acc
  k_quad_delta<<<1, 1024, 0, ctx->stream>>>(nS, nv, nC, nO, e, dd, small);
  QK_LAUNCHED();
  double mm[2];
  QK_CK(cudaMemcpyAsync(mm, small, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  if (mm[0] < 0.0) {
    // some e_a < e_i: A - B is not positive definite and the Casida energy is not a number
    // (its square roots are of negative values); no factorisation is needed to say so
    k_quad_nan<<<1, 1, 0, ctx->stream>>>(Ec, ctx->d_status);
    QK_LAUNCHED();
    *applied = 1;
    return QK_OK;
  }
  if (gap_only || !(mm[0] > 0.0) || !(mm[1] >= mm[0])) return QK_OK;
  const int nq = quad_points(mm[1] / mm[0]);
  if (nq == 0) return QK_OK;

  // the factor L (nS x r)
  const double* L = Lov;
  long long ldl = nS;
  int r = naux;
  if (!Lov) {
    const int rmax = nS / 3 > (nS < 64 ? nS : 64) ? nS / 3 : (nS < 64 ? nS : 64);
    double *K = nullptr, *Lt = nullptr, *Lc = nullptr, *pv = nullptr;
    QK_TRY(qk_wst(ctx, W_M, (size_t)nS * nS, &K));
    QK_TRY(qk_wst(ctx, W_QLT, (size_t)rmax * nS, &Lt));
    QK_TRY(qk_wst(ctx, W_QPV, (size_t)2 * nS + 64, &pv));
    dim3 gg((nv + 31) / 32, (nv + 31) / 32, no * no);
    if (gg.z > 65535) return QK_OK;
    k_gather_K<<<gg, dim3(32, 8), 0, ctx->stream>>>(N, nC, nO, nR, ERI, K);
    QK_LAUNCHED();
    PcArgs pa;
    pa.K = K;
    pa.ldk = nS;
    pa.nS = nS;
    pa.rmax = rmax;
    pa.tol_rel = 1e-12;
    pa.Lt = Lt;
    pa.r = pv;
    pa.done = (int*)(pv + nS);
    pa.gkey = (unsigned long long*)(pv + 2 * nS);  // 3 keys
    pa.rank = (int*)(pv + 2 * nS + 4);
    pa.bar = ctx->d_bar;
    pa.status = ctx->d_status;
    int grid = (nS + 31) / 32;
    if (grid > ctx->num_sms) grid = ctx->num_sms;
    const size_t smem = (size_t)rmax * sizeof(double);
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
      attr_err = cudaFuncSetAttribute(k_pchol, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      160 * 1024);
    });
    QK_CK(attr_err);
    if (smem > 160 * 1024) return QK_OK;
    int per_sm = 0;
    QK_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pchol, 1024, smem));
    if (per_sm < 1) return QK_OK;
    QK_CK(cudaMemsetAsync(ctx->d_bar, 0, 16 * sizeof(unsigned), ctx->stream));
    QK_CK(cudaMemsetAsync(pa.gkey, 0, 3 * sizeof(unsigned long long), ctx->stream));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(1024);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    QK_CK(cudaLaunchKernelEx(&cfg, k_pchol, pa));
    ctx->launches++;
    int rank = 0;
    QK_CK(cudaMemcpyAsync(&rank, pa.rank, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    QK_CK(cudaStreamSynchronize(ctx->stream));
    int hst = 0;
    QK_CK(cudaMemcpy(&hst, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (hst & QKD_BARRIER_TIMEOUT)
      return qk_fail(ctx, QK_ERR_DEVICE, "pivoted Cholesky: grid barrier timed out");
    if (rank <= 0 || rank >= rmax) return QK_OK;  // numerically full rank: eigenvalue route
    QK_TRY(qk_wst(ctx, W_QL, (size_t)nS * rank, &Lc));
    dim3 tg((nS + 31) / 32, (rank + 31) / 32);
    k_lt_transpose<<<tg, dim3(32, 8), 0, ctx->stream>>>(nS, rank, rmax, Lt, Lc);
    QK_LAUNCHED();
    L = Lc;
    ldl = nS;
    r = rank;
  }

  // quadrature points
  std::vector<double> x(nq), wg(nq), hb(2 * nq);
  qk_gauss_legendre_host(nq, x.data(), wg.data());
  const double w0 = sqrt(mm[0] * mm[1]);
  for (int k = 0; k < nq; ++k) {
    hb[k] = w0 * (1.0 + x[k]) / (1.0 - x[k]);
    hb[nq + k] = wg[k] * 2.0 * w0 / ((1.0 - x[k]) * (1.0 - x[k]));
  }
  double* om = small + 8;
  double* wt = small + 136;
  double* acc = small + 264;
  QK_CK(cudaMemcpyAsync(om, hb.data(), nq * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  QK_CK(cudaMemcpyAsync(wt, hb.data() + nq, nq * sizeof(double), cudaMemcpyHostToDevice,
                        ctx->stream));
  QK_CK(cudaMemsetAsync(acc, 0, nq * sizeof(double), ctx->stream));
  // the host copies above read hb before this function returns
  QK_CK(cudaStreamSynchronize(ctx->stream));

  // weights of all points; chunks of points with their Q (nch x r x r) at most ~2 GB
  float* wq = nullptr;
  QK_TRY(qk_wst(ctx, W_QX, (size_t)nS * nq, &wq));
  k_quad_weights<<<(nS * nq + 255) / 256, 256, 0, ctx->stream>>>(nS, nq, dd, om, wq);
  QK_LAUNCHED();
  const long long r2 = (long long)r * r;
  int nch = (int)((size_t)(256u << 20) / (size_t)r2);
  if (nch < 1) nch = 1;
  if (nch > nq) nch = nq;
  double *Q = nullptr, *qd = nullptr;
  {
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
      attr_err = cudaFuncSetAttribute(k_chol_trsm, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)TRSM_SMEM);
    });
    QK_CK(attr_err);
  }
  QK_TRY(qk_wst(ctx, W_QQ, (size_t)r2 * nch, &Q));
  QK_TRY(qk_wst(ctx, W_QD, (size_t)r * nch, &qd));
  for (int q0 = 0; q0 < nq; q0 += nch) {
    const int nc = nq - q0 < nch ? nq - q0 : nch;
    // the lower triangle of Q_q = L^T diag(c_q) L (all the factorisation reads), compensated FP32
    // products.  (The BF16x3 tensor-core GEMM was measured at 1.3e-5 Ha here: its FP32 tensor-
    // memory accumulation leaves ~1e-6 relative errors in Q, and ln det(1 + Q) - tr Q, second order
    // in Q, does not forgive first-order errors.)
    QK_TRY(qk_gemm_f32p_lower(ctx, 'T', 'N', r, r, nS, 1.0, L, ldl, 0, L, ldl, 0, 0.0, Q, r, r2,
                              nc, wq + (size_t)q0 * nS, nS));
    k_quad_diag<<<(r * nc + 255) / 256, 256, 0, ctx->stream>>>(r, nc, Q, qd);
    QK_LAUNCHED();
    for (int kb = 0; kb < r; kb += CB) {
      const int nb = r - kb < CB ? r - kb : CB;
      k_chol_blk<<<nc, 256, 0, ctx->stream>>>(r, kb, nb, Q, qd, acc + q0);
      QK_LAUNCHED();
      const int m = r - kb - nb;
      if (m <= 0) break;
      k_chol_trsm<<<dim3((m + TRSM_THREADS - 1) / TRSM_THREADS, nc), TRSM_THREADS, TRSM_SMEM,
                    ctx->stream>>>(r, kb, nb, Q);
      QK_LAUNCHED();
      double* P = Q + (kb + nb) + (long long)r * kb;
      double* S22 = Q + (kb + nb) + (long long)r * (kb + nb);
      QK_TRY(qk_dgemm_lower(ctx, 'N', 'T', m, m, nb, -1.0, P, r, r2, P, r, r2, 1.0, S22, r, r2, nc));
    }
  }
  k_quad_final<<<1, 32, 0, ctx->stream>>>(nq, wt, acc, Ec);
  QK_LAUNCHED();
  *applied = 1;
  return QK_OK;
}
