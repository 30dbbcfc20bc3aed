// k_sigma.cu -- diagonal correlation self-energy, renormalisation factor, Galitskii-Migdal
// energy, Newton/graphical QP solve, linearised QP, DIIS and small reductions.
//
// Pole sums (GW/RGW_self_energy_diag.f90:44-111, GW/RGW_Re_SigC.f90:30-50,
// GW/RGW_Re_dSigC.f90:30-50 and the SRG twins GW/RGW_SRG_*.f90):
//   Sig_p(w)  = sum_m [ sum_i 2 rho_pim^2 f(w - e_i + Om_m) + sum_a 2 rho_pam^2 f(w - e_a - Om_m) ]
//   dSig_p(w) = same with f'
// One thread owns one orbital p (32 consecutive p per warp, so every rho(p,q,m) load is a
// coalesced 256-byte row segment), the 8 warps of a CTA split the excitations m, and CTAs are
// spread over (p tile, m chunk).  Partials per (m chunk, p) are summed in a fixed order by a
// finalising kernel, so results are deterministic.  The occupied-part partial of a virtual p
// evaluated at w = e_p is exactly the Galitskii-Migdal summand (RGW_self_energy_diag.f90:88-107),
// so EcGM comes out of the same sweep: EcGM = -2 * sum_{a} SigOcc_a.
#include <cmath>
#include <cfloat>
#include "qk_internal.cuh"

namespace {

// 1/x in FP64: the hardware's approximate FP64 reciprocal (rcp.approx.ftz.f64) refined by two
// Newton-Raphson steps r <- r (2 - x r), each of which squares the relative error, ending within
// a few ulps of the correctly rounded quotient.  Inputs outside [1e-300, 1e300] in magnitude
// (where the approximation flushes) fall back to the IEEE division.
__device__ __forceinline__ double rcp_nr(double x) {
  const double ax = fabs(x);
  if (!(ax > 1e-300 && ax < 1e300)) return 1.0 / x;
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  r = r * fma(-x, r, 2.0);
  r = r * fma(-x, r, 2.0);
  return r;
}

constexpr int SIG_WARPS = 8;
constexpr int QP_MAXIT = 64;        // RGW_QP_graph.f90:38
constexpr double QP_THRESH = 1e-6;  // RGW_QP_graph.f90:39

struct SigArgs {
  int N, nC, nO, nR, nS;
  int nchunks, mper;  // m chunks and m per chunk
  int doSRG;
  double eta, flow;
  const double* eq;    // energies in the poles (e or eOld)
  const double* wp;    // evaluation energy per p (nullptr -> eq[p])
  const double* Om;
  const double* rho;
  const int* list;     // compacted list of active p (nullptr -> all p in [nC, N-nR))
  const int* nact;     // length of list (nullptr -> ignore)
  double* part;        // 3 * nchunks * N : sig, dsig, occ-part
};

__global__ void __launch_bounds__(SIG_WARPS * 32) k_sigma_partial(SigArgs a) {
  extern __shared__ double se[];  // N energies
  __shared__ double ssig[SIG_WARPS][32], sds[SIG_WARPS][32], socc[SIG_WARPS][32];
  const int nl = a.nact ? *a.nact : 0;
  if (a.list && (int)blockIdx.x * 32 >= nl) return;  // no active orbital in this tile
  const int N = a.N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) se[i] = a.eq[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pend = N - a.nR;
  int p;
  bool pok;
  if (a.list) {
    const int idx = blockIdx.x * 32 + lane;
    pok = idx < nl;
    p = pok ? a.list[idx] : pend;
  } else {
    p = a.nC + blockIdx.x * 32 + lane;
    pok = p < pend;
  }
  __syncthreads();
  double sig = 0.0, ds = 0.0, socc_acc = 0.0;
  if (pok) {
    const double w = a.wp ? a.wp[p] : se[p];
    const double eta2 = a.eta * a.eta;
    const long long N1 = N, N2 = N1 * N1;
    const int m0 = blockIdx.y * a.mper;
    const int m1 = min(a.nS, m0 + a.mper);
    for (int m = m0 + warp; m < m1; m += SIG_WARPS) {
      const double om = __ldg(a.Om + m);
      const double* r = a.rho + p + N2 * m;
      double so = 0.0;
      // eta = 0 takes the fast path; otherwise occupied part: eps = w - e_i + Om_m
      if (!a.doSRG && a.eta == 0.0) {
        // eta = 0: num*eps/(eps^2) = num/eps and num*eps^2/(eps^2)^2 = num/eps^2
        double s1 = 0.0, s2 = 0.0, d1 = 0.0;
        for (int q = a.nC; q < a.nO; ++q) {
          const double x = __ldg(r + N1 * q);
          const double ir = rcp_nr(w - se[q] + om);
          const double t = (x * x) * ir;
          s1 += t;
          d1 = fma(t, ir, d1);
        }
        for (int q = a.nO; q < pend; ++q) {
          const double x = __ldg(r + N1 * q);
          const double ir = rcp_nr(w - se[q] - om);
          const double t = (x * x) * ir;
          s2 += t;
          d1 = fma(t, ir, d1);
        }
        socc_acc += 2.0 * s1;
        sig += 2.0 * s2;
        ds -= 2.0 * d1;
        continue;
      }
      for (int q = a.nC; q < a.nO; ++q) {
        const double x = __ldg(r + N1 * q);
        const double num = 2.0 * x * x;
        const double eps = w - se[q] + om;
        if (!a.doSRG) {
          const double e2 = eps * eps;
          const double rr = rcp_nr(e2 + eta2);
          so += num * eps * rr;
          ds -= num * (e2 - eta2) * rr * rr;
        } else {
          const double reg = 1.0 - exp(-2.0 * a.flow * eps * eps);
          const double ie = rcp_nr(eps);
          so += num * reg * ie;
          ds -= num * reg * ie * ie;
        }
      }
      socc_acc += so;
      // virtual part: eps = w - e_a - Om_m
      for (int q = a.nO; q < pend; ++q) {
        const double x = __ldg(r + N1 * q);
        const double num = 2.0 * x * x;
        const double eps = w - se[q] - om;
        if (!a.doSRG) {
          const double e2 = eps * eps;
          const double rr = rcp_nr(e2 + eta2);
          sig += num * eps * rr;
          ds -= num * (e2 - eta2) * rr * rr;
        } else {
          const double reg = 1.0 - exp(-2.0 * a.flow * eps * eps);
          const double ie = rcp_nr(eps);
          sig += num * reg * ie;
          ds -= num * reg * ie * ie;
        }
      }
    }
    sig += socc_acc;
  }
  ssig[warp][lane] = sig;
  sds[warp][lane] = ds;
  socc[warp][lane] = socc_acc;
  __syncthreads();
  if (warp == 0 && p < pend) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int w = 0; w < SIG_WARPS; ++w) {
      s0 += ssig[w][lane];
      s1 += sds[w][lane];
      s2 += socc[w][lane];
    }
    const size_t o = (size_t)blockIdx.y * N + p;
    const size_t stride = (size_t)a.nchunks * N;
    a.part[o] = s0;
    a.part[o + stride] = s1;
    a.part[o + 2 * stride] = s2;
  }
}

// diag mode: Sig, Z = 1/(1 - dSig), EcGM
__global__ void k_sigma_final(int N, int nC, int nO, int nR, int nchunks,
                              const double* __restrict__ part, double* __restrict__ Sig,
                              double* __restrict__ Z, double* __restrict__ EcGM) {
  __shared__ double red[32];
  const size_t stride = (size_t)nchunks * N;
  double gm = 0.0;
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    double s = 0.0, d = 0.0, o = 0.0;
    if (p >= nC && p < N - nR) {
      for (int c = 0; c < nchunks; ++c) {
        s += part[(size_t)c * N + p];
        d += part[(size_t)c * N + p + stride];
        o += part[(size_t)c * N + p + 2 * stride];
      }
      if (p >= nO) gm += o;
    }
    Sig[p] = s;
    Z[p] = 1.0 / (1.0 - d);
  }
  gm = qk_block_sum(gm, red);
  if (threadIdx.x == 0 && EcGM) *EcGM = -2.0 * gm;
}

// Newton bookkeeping state (device): w, df, nIt, active, nact
struct QPState {
  double* w;
  double* df;
  int* nit;
  int* active;
  int* nact;
  int* list;   // compacted active orbitals, ascending
  int* conv;   // 1 if the last evaluation met |f| <= thresh
  int* evals;  // Sigma evaluations per orbital, all phases
};

// rebuild the compacted active list (one block; warp 0 walks the orbitals 32 at a time)
__device__ void qp_compact(int N, QPState& s) {
  __syncthreads();
  if (threadIdx.x < 32) {
    int base = 0;
    for (int p0 = 0; p0 < N; p0 += 32) {
      const int p = p0 + threadIdx.x;
      const bool act = p < N && s.active[p] != 0;
      const unsigned b = __ballot_sync(0xffffffffu, act);
      if (act) s.list[base + __popc(b & ((1u << threadIdx.x) - 1u))] = p;
      base += __popc(b);
    }
    if (threadIdx.x == 0) *s.nact = base;
  }
}

__global__ void k_qp_init(int N, int nC, int nR, const double* __restrict__ w0, QPState s) {
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    s.w[p] = w0[p];
    s.df[p] = 0.0;
    s.nit[p] = 0;
    s.conv[p] = 0;
    s.evals[p] = 0;
    s.active[p] = (p >= nC && p < N - nR);
  }
  qp_compact(N, s);
}

// Orbitals whose guess-started search did not converge, or converged outside the trust region
// |w - eGWlin| <= |eGWlin - eHF| + 0.02 Ha around the reference start, restart from the
// reference start (the root must stay the one the linearised solution points at).
__global__ void k_qp_restart(int N, int nC, int nR, const double* __restrict__ eGWlin,
                             const double* __restrict__ eHF, QPState s) {
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    const double trust = fabs(eGWlin[p] - eHF[p]) + 0.02;
    const double wnew = s.w[p];
    const bool keep = s.conv[p] && fabs(wnew - eGWlin[p]) <= trust;
    const bool act = (p >= nC && p < N - nR) && !keep;
    if (act) {
      s.w[p] = eGWlin[p];
      s.nit[p] = 0;
    }
    s.active[p] = act;
  }
  qp_compact(N, s);
}

// one Newton step for every still-active p (RGW_QP_graph.f90:56-76)
__global__ void k_qp_update(int N, int nchunks, const double* __restrict__ part,
                            const double* __restrict__ eHF, QPState s, int maxit) {
  if (*s.nact == 0) return;
  const size_t stride = (size_t)nchunks * N;
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    if (!s.active[p]) continue;
    double sig = 0.0, dsig = 0.0;
    for (int c = 0; c < nchunks; ++c) {
      sig += part[(size_t)c * N + p];
      dsig += part[(size_t)c * N + p + stride];
    }
    const int nIt = s.nit[p] + 1;
    s.nit[p] = nIt;
    s.evals[p] += 1;
    const double w = s.w[p];
    const double f = w - eHF[p] - sig;
    const double df = 1.0 / (1.0 - dsig);
    s.w[p] = w - df * f;
    s.df[p] = df;
    const bool ok = !(fabs(f) > QP_THRESH);
    if (ok || nIt >= maxit) {
      s.active[p] = 0;
      s.conv[p] = ok;
    }
  }
  qp_compact(N, s);
}

__global__ void k_qp_finish(int N, int nC, int nR, const double* __restrict__ eGWlin, QPState s,
                            double* __restrict__ eGW, double* __restrict__ Z, int* status) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    if (p < nC || p >= N - nR) continue;
    if (s.nit[p] == QP_MAXIT) {
      eGW[p] = eGWlin[p];
      atomicOr(status, QKD_QP_NOCONV);
    } else {
      eGW[p] = s.w[p];
      Z[p] = s.df[p];
    }
  }
}

__global__ void k_qp_linear(int N, const double* __restrict__ eHF, const double* __restrict__ Z,
                            const double* __restrict__ Sig, int use_z, double* __restrict__ eGW) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x)
    eGW[p] = use_z ? eHF[p] + Z[p] * Sig[p] : eHF[p] + Sig[p];
}

__global__ void k_max_abs_diff(int n, const double* __restrict__ a, const double* __restrict__ b,
                               double* out) {
  double m = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) m = fmax(m, fabs(a[i] - b[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  __shared__ double s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, s[w]);
    *out = m;
  }
}

// DIIS (utils/DIIS_extrapolation.f90:1-61), single block.  hist arrays are (n, nd) column-major
// with leading dimension n.  The bordered (nd+1)^2 system is solved by Gaussian elimination with
// partial pivoting; rcond is the exact reciprocal 1-norm condition number from the explicit
// inverse (dsysvx reports an estimate of the same quantity).
constexpr int DIIS_MAX = 32;
__global__ void k_diis(int n_err, int n_e, int nd_host, double* __restrict__ err,
                       double* __restrict__ e, const double* __restrict__ err_in,
                       double* __restrict__ e_inout, double* __restrict__ rcond_out,
                       const int* __restrict__ nd_dev) {
  const int nd = nd_dev ? *nd_dev : nd_host;
  __shared__ double A[DIIS_MAX + 1][DIIS_MAX + 1];
  __shared__ double wv[DIIS_MAX + 1];
  __shared__ double red[32];
  __shared__ double s_rcond;
  const int tid = threadIdx.x;
  // prepend (utils.f90:506-536): shift columns right, new vector in column 0
  for (int i = tid; i < n_err; i += blockDim.x) {
    for (int c = nd - 1; c >= 1; --c) err[i + (size_t)n_err * c] = err[i + (size_t)n_err * (c - 1)];
    err[i] = err_in[i];
  }
  for (int i = tid; i < n_e; i += blockDim.x) {
    for (int c = nd - 1; c >= 1; --c) e[i + (size_t)n_e * c] = e[i + (size_t)n_e * (c - 1)];
    e[i] = e_inout[i];
  }
  __syncthreads();
  const int M = nd + 1;
  for (int r = 0; r < nd; ++r)
    for (int c = 0; c <= r; ++c) {
      double s = 0.0;
      for (int i = tid; i < n_err; i += blockDim.x)
        s += err[i + (size_t)n_err * r] * err[i + (size_t)n_err * c];
      s = qk_block_sum(s, red);
      if (tid == 0) { A[r][c] = s; A[c][r] = s; }
    }
  if (tid == 0) {
    for (int r = 0; r < nd; ++r) { A[r][nd] = -1.0; A[nd][r] = -1.0; }
    A[nd][nd] = 0.0;
    // 1-norm of A
    double anorm = 0.0;
    for (int c = 0; c < M; ++c) {
      double s = 0.0;
      for (int r = 0; r < M; ++r) s += fabs(A[r][c]);
      anorm = fmax(anorm, s);
    }
    // Gauss-Jordan inverse with partial pivoting
    double W[DIIS_MAX + 1][2 * (DIIS_MAX + 1)];
    for (int r = 0; r < M; ++r)
      for (int c = 0; c < 2 * M; ++c) W[r][c] = (c < M) ? A[r][c] : (c - M == r ? 1.0 : 0.0);
    bool sing = false;
    for (int c = 0; c < M; ++c) {
      int piv = c;
      for (int r = c + 1; r < M; ++r)
        if (fabs(W[r][c]) > fabs(W[piv][c])) piv = r;
      if (W[piv][c] == 0.0) { sing = true; break; }
      if (piv != c)
        for (int k = 0; k < 2 * M; ++k) { double t = W[c][k]; W[c][k] = W[piv][k]; W[piv][k] = t; }
      const double ip = 1.0 / W[c][c];
      for (int k = 0; k < 2 * M; ++k) W[c][k] *= ip;
      for (int r = 0; r < M; ++r) {
        if (r == c) continue;
        const double f = W[r][c];
        if (f != 0.0)
          for (int k = 0; k < 2 * M; ++k) W[r][k] -= f * W[c][k];
      }
    }
    double rc = 0.0;
    if (!sing) {
      double inorm = 0.0;
      for (int c = 0; c < M; ++c) {
        double s = 0.0;
        for (int r = 0; r < M; ++r) s += fabs(W[r][M + c]);
        inorm = fmax(inorm, s);
      }
      rc = (anorm > 0.0 && inorm > 0.0) ? 1.0 / (anorm * inorm) : 0.0;
      // x = A^{-1} b with b = (0,..,0,-1)
      for (int r = 0; r < M; ++r) wv[r] = -W[r][M + nd];
    }
    s_rcond = rc;
    if (rcond_out) *rcond_out = rc;
  }
  __syncthreads();
  if (s_rcond > 10e-14) {  // DIIS_extrapolation.f90:54
    for (int i = tid; i < n_e; i += blockDim.x) {
      double s = 0.0;
      for (int c = 0; c < nd; ++c) s += wv[c] * e[i + (size_t)n_e * c];
      e_inout[i] = s;
    }
  }
}

}  // namespace

static int sigma_sweep(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                       int nS, const double* eq, const double* wp, const double* Om,
                       const double* rho, const int* list, const int* nact, double** part_out,
                       int* nchunks_out) {
  const int nact_p = N - nR - nC;
  const int ptiles = (nact_p + 31) / 32;
  const int cm = qk_tune_get(ctx, TUNE_SIGMA_CHUNKS, (long long)nS, 4);
  int nchunks = (cm * ctx->num_sms + ptiles - 1) / (ptiles > 0 ? ptiles : 1);
  const int maxch = (nS + SIG_WARPS - 1) / SIG_WARPS;
  if (nchunks > maxch) nchunks = maxch;
  if (nchunks < 1) nchunks = 1;
  const int mper = (nS + nchunks - 1) / nchunks;
  nchunks = (nS + mper - 1) / mper;
  double* part = nullptr;
  // every (chunk, p) entry the consumers read is written by the sweep: no clearing needed
  QK_TRY(qk_wst(ctx, W_MISC, (size_t)3 * nchunks * N + 64, &part));
  SigArgs a;
  a.N = N; a.nC = nC; a.nO = nO; a.nR = nR; a.nS = nS;
  a.nchunks = nchunks; a.mper = mper;
  a.doSRG = doSRG; a.eta = eta; a.flow = flow;
  a.eq = eq; a.wp = wp; a.Om = Om; a.rho = rho; a.list = list; a.nact = nact; a.part = part;
  if (ptiles > 0 && nS > 0) {
    k_sigma_partial<<<dim3(ptiles, nchunks), SIG_WARPS * 32, N * sizeof(double), ctx->stream>>>(a);
    QK_LAUNCHED();
  }
  *part_out = part;
  *nchunks_out = nchunks;
  return QK_OK;
}

int qk_sigma_diag(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                  int nS, const double* e, const double* Om, const double* rho, double* Sig,
                  double* Z, double* EcGM) {
  double* part;
  int nch;
  QK_TRY(sigma_sweep(ctx, doSRG, eta, flow, N, nC, nO, nR, nS, e, nullptr, Om, rho, nullptr,
                     nullptr, &part, &nch));
  k_sigma_final<<<1, 1024, 0, ctx->stream>>>(N, nC, nO, nR, nch, part, Sig, Z, EcGM);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qp_newton(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                 int nS, const double* eHF, const double* Om, const double* rho,
                 const double* eGWlin, const double* eOld, double* eGW, double* Z,
                 const double* w_guess, int guess_maxit) {
  double* st = nullptr;
  QK_TRY(qk_wst(ctx, W_M2, (size_t)8 * N + 64, &st));
  QPState s;
  s.w = st;
  s.df = st + N;
  s.nit = (int*)(st + 2 * N);
  s.active = (int*)(st + 3 * N);
  s.list = (int*)(st + 4 * N);
  s.conv = (int*)(st + 5 * N);
  s.evals = (int*)(st + 6 * N);
  s.nact = (int*)(st + 7 * N);
  // phase 1 (learned guess only): at most guess_maxit steps from the guess; phase 2: the
  // reference search (RGW_QP_graph.f90:50-92) from eGWlin for every orbital not yet converged
  k_qp_init<<<1, 1024, 0, ctx->stream>>>(N, nC, nR, w_guess ? w_guess : eGWlin, s);
  QK_LAUNCHED();
  for (int phase = w_guess ? 1 : 2; phase <= 2; ++phase) {
    const int maxit = phase == 1 ? guess_maxit : QP_MAXIT;
    if (phase == 2 && w_guess) {
      k_qp_restart<<<1, 1024, 0, ctx->stream>>>(N, nC, nR, eGWlin, eHF, s);
      QK_LAUNCHED();
    }
    int hact = 1;
    for (int it = 0; it < maxit; ++it) {
      double* part;
      int nch;
      QK_TRY(sigma_sweep(ctx, doSRG, eta, flow, N, nC, nO, nR, nS, eOld, s.w, Om, rho, s.list,
                         s.nact, &part, &nch));
      k_qp_update<<<1, 1024, 0, ctx->stream>>>(N, nch, part, eHF, s, maxit);
      QK_LAUNCHED();
      if (!ctx->capturing && (it & 3) == 3) {  // poll the active count every 4 steps
        QK_CK(cudaMemcpyAsync(&hact, s.nact, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        QK_CK(cudaStreamSynchronize(ctx->stream));
        if (hact == 0) break;
      }
    }
  }
  k_qp_finish<<<(N + 255) / 256, 256, 0, ctx->stream>>>(N, nC, nR, eGWlin, s, eGW, Z, ctx->d_status);
  QK_LAUNCHED();
  if (ctx->capturing) return QK_OK;  // no host readback inside a graph
  // per-orbital Newton step counts and Sigma evaluations for diagnostics (qk_get_qp_iters)
  ctx->qp_iters.resize(N);
  std::vector<int> ev(N);
  QK_CK(cudaMemcpyAsync(ctx->qp_iters.data(), s.nit, N * sizeof(int), cudaMemcpyDeviceToHost,
                        ctx->stream));
  QK_CK(cudaMemcpyAsync(ev.data(), s.evals, N * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  QK_CK(cudaStreamSynchronize(ctx->stream));
  long long tot = 0;
  for (int v : ev) tot += v;
  ctx->qp_evals = tot;
  return QK_OK;
}

// ---------------------------------------------------------------------------------------------
// per-orbital features of the linearised stage for the learned guess
// ---------------------------------------------------------------------------------------------
namespace {

constexpr int NMOM = 6;  // occupied/virtual pole weight, first and second moments

__global__ void __launch_bounds__(SIG_WARPS * 32)
    k_feature_partial(int N, int nC, int nO, int nR, int nS, int nchunks, int mper,
                      const double* __restrict__ e, const double* __restrict__ Om,
                      const double* __restrict__ rho, double* __restrict__ part) {
  extern __shared__ double se[];
  __shared__ double acc[NMOM][SIG_WARPS][32];
  for (int i = threadIdx.x; i < N; i += blockDim.x) se[i] = e[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p = nC + blockIdx.x * 32 + lane;
  const int pend = N - nR;
  __syncthreads();
  double m[NMOM] = {0, 0, 0, 0, 0, 0};
  if (p < pend) {
    const long long N1 = N, N2 = N1 * N1;
    const int m0 = blockIdx.y * mper, m1 = min(nS, m0 + mper);
    for (int mm = m0 + warp; mm < m1; mm += SIG_WARPS) {
      const double om = Om[mm];
      const double* r = rho + p + N2 * mm;
      for (int q = nC; q < nO; ++q) {
        const double x = r[N1 * q], w = x * x, pole = se[q] - om;
        m[0] += w; m[1] += w * pole; m[2] += w * pole * pole;
      }
      for (int q = nO; q < pend; ++q) {
        const double x = r[N1 * q], w = x * x, pole = se[q] + om;
        m[3] += w; m[4] += w * pole; m[5] += w * pole * pole;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < NMOM; ++k) acc[k][warp][lane] = m[k];
  __syncthreads();
  if (warp == 0 && p < pend) {
    const size_t stride = (size_t)nchunks * N;
#pragma unroll
    for (int k = 0; k < NMOM; ++k) {
      double t = 0.0;
      for (int w = 0; w < SIG_WARPS; ++w) t += acc[k][w][lane];
      part[(size_t)k * stride + (size_t)blockIdx.y * N + p] = t;
    }
  }
}

__global__ void k_feature_final(int N, int nC, int nO, int nR, int nchunks,
                                const double* __restrict__ part, const double* __restrict__ e,
                                const double* __restrict__ Om, const double* __restrict__ Sig,
                                const double* __restrict__ Z, float* __restrict__ F) {
  const size_t stride = (size_t)nchunks * N;
  const double eh = e[nO - 1], el = e[nO];
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    double m[NMOM] = {0, 0, 0, 0, 0, 0};
    if (p >= nC && p < N - nR)
      for (int c = 0; c < nchunks; ++c)
        for (int k = 0; k < NMOM; ++k) m[k] += part[(size_t)k * stride + (size_t)c * N + p];
    const double ep = e[p];
    const double co = m[0] > 0 ? m[1] / m[0] : ep, cv = m[3] > 0 ? m[4] / m[3] : ep;
    const double so = m[0] > 0 ? sqrt(fmax(0.0, m[2] / m[0] - co * co)) : 0.0;
    const double sv = m[3] > 0 ? sqrt(fmax(0.0, m[5] / m[3] - cv * cv)) : 0.0;
    float* f = F + (size_t)p * QK_MLP_NIN;
    f[0] = (float)ep;
    f[1] = p < nO ? 1.f : 0.f;
    f[2] = (float)(ep - eh);
    f[3] = (float)(ep - el);
    f[4] = (float)Sig[p];
    f[5] = (float)Z[p];
    f[6] = (float)(Z[p] * Sig[p]);
    f[7] = (float)(1.0 - 1.0 / Z[p]);
    f[8] = (float)m[0];
    f[9] = (float)m[3];
    f[10] = (float)(co - ep);
    f[11] = (float)(cv - ep);
    f[12] = (float)so;
    f[13] = (float)sv;
    f[14] = (float)Om[0];
    f[15] = (float)log((double)N);
  }
}

}  // namespace

int qk_features(qk_ctx* ctx, int N, int nC, int nO, int nR, int nS, const double* e,
                const double* Om, const double* rho, const double* Sig, const double* Z,
                float* F) {
  const int nact = N - nR - nC;
  const int ptiles = (nact + 31) / 32;
  int nchunks = (4 * ctx->num_sms + ptiles - 1) / (ptiles > 0 ? ptiles : 1);
  const int maxch = (nS + SIG_WARPS - 1) / SIG_WARPS;
  if (nchunks > maxch) nchunks = maxch;
  if (nchunks < 1) nchunks = 1;
  const int mper = (nS + nchunks - 1) / nchunks;
  nchunks = (nS + mper - 1) / mper;
  double* part = nullptr;
  QK_TRY(qk_wst(ctx, W_MISC, (size_t)NMOM * nchunks * N + 64, &part));
  QK_CK(cudaMemsetAsync(part, 0, sizeof(double) * NMOM * (size_t)nchunks * N, ctx->stream));
  if (ptiles > 0) {
    k_feature_partial<<<dim3(ptiles, nchunks), SIG_WARPS * 32, N * sizeof(double), ctx->stream>>>(
        N, nC, nO, nR, nS, nchunks, mper, e, Om, rho, part);
    QK_LAUNCHED();
  }
  k_feature_final<<<(N + 127) / 128, 128, 0, ctx->stream>>>(N, nC, nO, nR, nchunks, part, e, Om,
                                                           Sig, Z, F);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qp_linear(qk_ctx* ctx, int N, const double* eHF, const double* Z, const double* Sig,
                 int use_z, double* eGW) {
  k_qp_linear<<<(N + 255) / 256, 256, 0, ctx->stream>>>(N, eHF, Z, Sig, use_z, eGW);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_diis_dev(qk_ctx* ctx, int n_err, int n_e, int n_diis, double* err_hist, double* e_hist,
                const double* err_in, double* e_inout, double* rcond_dev, const int* n_diis_dev) {
  if (n_diis < 1 || n_diis > DIIS_MAX) return qk_fail(ctx, QK_ERR_ARG, "n_diis out of range (1..%d)", DIIS_MAX);
  k_diis<<<1, 256, 0, ctx->stream>>>(n_err, n_e, n_diis, err_hist, e_hist, err_in, e_inout, rcond_dev,
                                     n_diis_dev);
  QK_LAUNCHED();
  return QK_OK;
}

__global__ void k_sub(int n, const double* __restrict__ a, const double* __restrict__ b,
                      double* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = a[i] - b[i];
}

int qk_sub(qk_ctx* ctx, int n, const double* a, const double* b, double* out) {
  k_sub<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, a, b, out);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_max_abs_diff(qk_ctx* ctx, int n, const double* a, const double* b, double* out_dev) {
  k_max_abs_diff<<<1, 1024, 0, ctx->stream>>>(n, a, b, out_dev);
  QK_LAUNCHED();
  return QK_OK;
}
