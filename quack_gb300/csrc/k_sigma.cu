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
#include <mutex>
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
constexpr double QP_THRESH = 1e-6;  // RGW_QP_graph.f90:39

struct SigArgs {
  int N, nC, nO, nR, nS;
  int nchunks, mper;  // chunks (all of them) and m per chunk
  int mchunks, qper;  // mixed sweep: chunk y covers m chunk y % mchunks, q group y / mchunks
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
    // chunk = (m range, q range)
    const int mc = blockIdx.y % a.mchunks, qg = blockIdx.y / a.mchunks;
    const int m0 = mc * a.mper;
    const int m1 = min(a.nS, m0 + a.mper);
    const int qa = a.nC + qg * a.qper, qb = min(pend, qa + a.qper);
    const int qo0 = qa, qo1 = min(a.nO, qb), qv0 = max(a.nO, qa), qv1 = qb;
    for (int m = m0 + warp; m < m1; m += SIG_WARPS) {
      const double om = __ldg(a.Om + m);
      const double* r = a.rho + p + N2 * m;
      double so = 0.0;
      // eta = 0 takes the fast path; otherwise occupied part: eps = w - e_i + Om_m
      if (!a.doSRG && a.eta == 0.0) {
        // eta = 0: num*eps/(eps^2) = num/eps and num*eps^2/(eps^2)^2 = num/eps^2
        double s1 = 0.0, s2 = 0.0, d1 = 0.0;
        for (int q = qo0; q < qo1; ++q) {
          const double x = __ldg(r + N1 * q);
          const double ir = rcp_nr(w - se[q] + om);
          const double t = (x * x) * ir;
          s1 += t;
          d1 = fma(t, ir, d1);
        }
        for (int q = qv0; q < qv1; ++q) {
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
      for (int q = qo0; q < qo1; ++q) {
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
      for (int q = qv0; q < qv1; ++q) {
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

// Mixed-tier sweep (eta = 0, no SRG).  Same outputs as k_sigma_partial (lanes = orbitals p, CTAs
// over (p tile, chunk)), but a chunk is an (m range, q range) pair and the 8 warps split the q
// of their range, each warp running over the whole m range, so that the per-(p,q) setup is done
// once: c = w - e_q as a float pair (c_hi, c_lo) by TwoSum in FP32 from float pairs of w and e_q,
// and the window [lo, hi) of the m with |w - e_q +- Om_m| < tau (Om ascending: two bisections).
// Splitting q over CTAs keeps the GPU busy when only a few orbitals are still searching.  Outside the window, eps = (c_hi +- Om_hi) + (c_lo +- Om_lo) is
// accurate to a few FP32 ulps and the term R/eps with R = 2 rho^2 (FP32) runs on the FP32 pipe;
// the per-(p,q) FP32 partials are added into float-float (TwoSum) accumulators.  Inside the
// window the term is evaluated exactly as in k_sigma_partial (FP64).  All lanes step through the
// same m (the window only masks the reciprocal), so the R loads stay coalesced.
__device__ __forceinline__ float rcp32(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// first m in [lo, hi) with Om_hi(m) >= v, Om_hi(m) = O[m - mb].x (ascending)
__device__ __forceinline__ int om_lower_bound(const float2* __restrict__ O, int mb, int lo, int hi,
                                              float v) {
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (O[mid - mb].x < v) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// (hi, lo) += x, error-free (Knuth's TwoSum) up to the final rounding of lo
__device__ __forceinline__ void ff_add(float& hi, float& lo, float x) {
  const float t = hi + x;
  const float z = t - hi;
  lo += (hi - (t - z)) + (x - z);
  hi = t;
}

struct SigFF {
  const float* Rt;  // R = 2 rho^2 (FP32), p-major: Rt[m + nS (q + N p)]
  const float2* OmF;
  const int* bad;
  float tau;
};

// Mixed-tier sweep over the p-major R: one CTA per (orbital, q group); its warps take the q of
// the group, the lanes the excitations m (contiguous in Rt, so each warp streams 128-byte lines,
// FFT_U loads per lane in flight).  Per (p, q): c = w - e_q as a float pair (TwoSum in FP32) and
// the window of m with |w - e_q +- Om_m| < tau by two bisections on the ascending Om (pairs in
// shared memory); outside the window eps = (c_hi +- Om_hi) + (c_lo +- Om_lo) and R/eps on the FP32
// pipe, the warp's per-(p,q) sums added into float-float (TwoSum) accumulators; inside it the
// FP64 terms of k_sigma_partial.  Same partial-sum layout as k_sigma_partial (chunk = q group).
constexpr int FFT_WARPS = 8;
constexpr int FFT_U = 8;

__global__ void __launch_bounds__(FFT_WARPS * 32) k_sigma_partial_ffT(SigArgs a, SigFF f) {
  // dynamic shared memory: e (N doubles) | e as float pairs (N) | Om pairs (nS)
  extern __shared__ double se[];
  __shared__ double r_sig[FFT_WARPS], r_ds[FFT_WARPS], r_so[FFT_WARPS];
  const int N = a.N, nS = a.nS;
  int p;
  if (a.list) {
    if ((int)blockIdx.x >= *a.nact) return;
    p = a.list[blockIdx.x];
  } else {
    p = a.nC + blockIdx.x;
  }
  float2* eF = (float2*)(se + N);
  float2* oS = eF + N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double e = a.eq[i];
    const float h = (float)e;
    se[i] = e;
    eF[i] = make_float2(h, (float)(e - (double)h));
  }
  for (int i = threadIdx.x; i < nS; i += blockDim.x) oS[i] = f.OmF[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pend = N - a.nR;
  const long long N1 = N, N2 = N1 * N1;
  const bool bad = *f.bad != 0;
  const double w = a.wp ? a.wp[p] : se[p];
  const float w_hi = (float)w;
  const float w_lo = (float)(w - (double)w_hi);
  const float* Rp = f.Rt + (long long)nS * N1 * p;
  const double* rp = a.rho + p;
  float so_h = 0.f, so_l = 0.f, sv_h = 0.f, sv_l = 0.f, d_h = 0.f, d_l = 0.f;
  double Sn_o = 0.0, Sn_v = 0.0, Dn = 0.0;  // window (FP64) parts, per lane
  const int q0 = a.nC + (int)blockIdx.y * a.qper;
  const int q1 = min(pend, q0 + a.qper);
  for (int q = q0 + warp; q < q1; q += FFT_WARPS) {
    const bool occ = q < a.nO;
    const float2 eq = eF[q];
    const float chi = w_hi - eq.x;
    const float bb = chi - w_hi;
    const float clo = ((w_hi - (chi - bb)) + (-eq.x - bb)) + (w_lo - eq.y);
    const float sg = occ ? 1.f : -1.f;
    int lo = 0, hi = nS;
    if (!bad) {
      const float ctr = -sg * chi;  // the pole sits at Om = -c (occupied) or Om = c (virtual)
      lo = om_lower_bound(oS, 0, 0, nS, ctr - f.tau);
      hi = om_lower_bound(oS, 0, lo, nS, ctr + f.tau);
    }
    const float* Rq = Rp + (long long)nS * q;
    float sl = 0.f, dl = 0.f;
    int m0 = 0;
    // batches of FFT_U loads per lane, the next batch's loads issued before the current one is
    // used, so that a lane always has loads in flight; each lane still takes its m in increasing
    // order (the sums are the same bits as with one batch at a time)
    const int nfull = nS / (32 * FFT_U);
    float rv[FFT_U];
    if (nfull > 0) {
#pragma unroll
      for (int u = 0; u < FFT_U; ++u) rv[u] = __ldg(Rq + 32 * u + lane);
    }
    for (int b = 0; b < nfull; ++b, m0 += 32 * FFT_U) {
      float rn[FFT_U];
      const bool more = b + 1 < nfull;
      if (more) {
#pragma unroll
        for (int u = 0; u < FFT_U; ++u) rn[u] = __ldg(Rq + m0 + 32 * FFT_U + 32 * u + lane);
      }
#pragma unroll
      for (int u = 0; u < FFT_U; ++u) {
        const int m = m0 + 32 * u + lane;
        const float2 o = oS[m];
        const float e = fmaf(sg, o.x, chi) + fmaf(sg, o.y, clo);
        float r = rcp32(e);
        r = (m >= lo && m < hi) ? 0.f : r;
        const float t = rv[u] * r;
        sl += t;
        dl = fmaf(t, r, dl);
      }
      if (more) {
#pragma unroll
        for (int u = 0; u < FFT_U; ++u) rv[u] = rn[u];
      }
    }
    for (int m = m0 + lane; m < nS; m += 32) {
      const float2 o = oS[m];
      const float e = fmaf(sg, o.x, chi) + fmaf(sg, o.y, clo);
      float r = rcp32(e);
      r = (m >= lo && m < hi) ? 0.f : r;
      const float t = __ldg(Rq + m) * r;
      sl += t;
      dl = fmaf(t, r, dl);
    }
    for (int o = 16; o > 0; o >>= 1) {
      sl += __shfl_xor_sync(0xffffffffu, sl, o);
      dl += __shfl_xor_sync(0xffffffffu, dl, o);
    }
    if (occ) ff_add(so_h, so_l, sl);
    else ff_add(sv_h, sv_l, sl);
    ff_add(d_h, d_l, dl);
    // the window, in FP64 (RGW_Re_SigC.f90:30-50 / RGW_Re_dSigC.f90:30-50 with eta = 0)
    for (int m = lo + lane; m < hi; m += 32) {
      const double om = __ldg(a.Om + m);
      const double x = __ldg(rp + N1 * q + N2 * m);
      const double ir = rcp_nr(occ ? (w - se[q] + om) : (w - se[q] - om));
      const double t = (2.0 * (x * x)) * ir;
      if (occ) Sn_o += t;
      else Sn_v += t;
      Dn = fma(t, ir, Dn);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    Sn_o += __shfl_xor_sync(0xffffffffu, Sn_o, o);
    Sn_v += __shfl_xor_sync(0xffffffffu, Sn_v, o);
    Dn += __shfl_xor_sync(0xffffffffu, Dn, o);
  }
  // lanes hold identical float-float accumulators (the shuffles gave every lane the sums)
  if (lane == 0) {
    const double so = ((double)so_h + (double)so_l) + Sn_o;
    r_so[warp] = so;
    r_sig[warp] = ((double)sv_h + (double)sv_l) + Sn_v + so;
    r_ds[warp] = -(((double)d_h + (double)d_l) + Dn);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = 0; k < FFT_WARPS; ++k) {
      s0 += r_sig[k];
      s1 += r_ds[k];
      s2 += r_so[k];
    }
    const size_t o = (size_t)blockIdx.y * N + p;
    const size_t stride = (size_t)a.nchunks * N;
    a.part[o] = s0;
    a.part[o + stride] = s1;
    a.part[o + 2 * stride] = s2;
  }
}

// Rt = 2 rho^2 in FP32, p-major: Rt[m + nS (q + N p)] from rho[p + N q + N^2 m], through 32 x 32
// shared-memory tiles of (p, m) per q, both sides coalesced
__global__ void k_sigma_ff_prepT(int N, int nS, const double* __restrict__ rho,
                                 float* __restrict__ Rt) {
  __shared__ float t[32][33];
  const int p0 = blockIdx.x * 32, m0 = blockIdx.y * 32, q = blockIdx.z;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  const long long N1 = N, N2 = N1 * N1;
  for (int i = ty; i < 32; i += 8) {
    const int p = p0 + tx, m = m0 + i;
    float v = 0.f;
    if (p < N && m < nS) {
      const double x = rho[p + N1 * q + N2 * m];
      v = (float)(2.0 * (x * x));
    }
    t[i][tx] = v;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int p = p0 + i, m = m0 + tx;
    if (p < N && m < nS) Rt[m + (long long)nS * (q + N1 * p)] = t[tx][i];
  }
}

// Om split into float pairs; flag Om that is not ascending (or NaN)
__global__ void k_om_pairs(int nS, const double* __restrict__ Om, float2* __restrict__ OmF,
                           int* __restrict__ bad) {
  for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < nS; m += gridDim.x * blockDim.x) {
    const double om = Om[m];
    const float hi = (float)om;
    OmF[m] = make_float2(hi, (float)(om - (double)hi));
    if (!(om >= 0.0) || (m + 1 < nS && !(Om[m + 1] >= om))) atomicOr(bad, 1);
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
  const int* fromref;  // learned-guess mode: 1 where the search started at the reference start
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

// Orbitals whose guess-started search did not converge, or converged to a root that the root
// certificate (k_cert_partial) does not prove to be the reference search's, restart from the
// reference start.  Orbitals that started at the reference start are already on the reference
// trajectory and just continue.
__global__ void k_qp_restart(int N, int nC, int nR, const double* __restrict__ eGWlin,
                             const int* __restrict__ cert, QPState s, int maxit) {
  for (int p = threadIdx.x; p < N; p += blockDim.x) {
    if (s.fromref && s.fromref[p]) {
      s.active[p] = (p >= nC && p < N - nR) && !s.conv[p] && s.nit[p] < maxit;
      continue;
    }
    const bool keep = s.conv[p] && cert[p];
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
  const int nl = *s.nact;
  if (nl == 0) return;
  const size_t stride = (size_t)nchunks * N;
  // one warp per active orbital: the lanes split the chunk partials, then a butterfly
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int idx = warp; idx < nl; idx += nw) {
    const int p = s.list[idx];
    double sig = 0.0, dsig = 0.0;
    for (int c = lane; c < nchunks; c += 32) {
      sig += part[(size_t)c * N + p];
      dsig += part[(size_t)c * N + p + stride];
    }
    for (int o = 16; o > 0; o >>= 1) {
      sig += __shfl_xor_sync(0xffffffffu, sig, o);
      dsig += __shfl_xor_sync(0xffffffffu, dsig, o);
    }
    if (lane != 0) continue;
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

// Persistent Newton solve of the mixed tier (RGW_QP_graph.f90:50-92; eta = 0, no SRG): one CTA
// per orbital, taken from a queue, iterates w <- w - f/(1 - Sigma'(w)) on chip until |f| <= 1e-6
// or maxit steps, so that a search costs no launches and the chaotic orbitals, which run all 64
// steps, no longer hold the whole GPU for two launches per step.  A step sweeps the orbital's
// (q, m) terms: warps over q, lanes over m (Rt is p-major, so the loads are coalesced), the
// same FP32 far-pole / FP64 window split and float-float accumulation as k_sigma_partial_ffT,
// then one block reduction.  The update and the bookkeeping are k_qp_update's.
constexpr size_t NEWT_SMEM_MAX = 200 * 1024;
struct NewtFF {
  int N, nC, nO, nR, nS, maxit;
  const double* eq;     // energies in the poles
  const double* eHF;
  const double* Om;
  const double* rho;
  const float* Rt;      // p-major 2 rho^2
  const float2* OmF;
  const int* bad;
  float tau;
  int* queue;           // next list index to take
};

constexpr int NEWT_WARPS = 32;  // one CTA per SM: its loads must fill the memory pipeline alone
constexpr int NEWT_U = 8;       // R loads per lane issued together
__global__ void __launch_bounds__(NEWT_WARPS * 32) k_qp_newton_ff(NewtFF a, QPState s) {
  // dynamic shared memory: e (N doubles) | e as float pairs (N) | Om as float pairs (nS), so
  // that the two window bisections per (step, q) probe shared memory
  extern __shared__ double se[];
  __shared__ double r_sig[NEWT_WARPS], r_ds[NEWT_WARPS];
  __shared__ double s_w;
  __shared__ int s_p, s_done;
  const int N = a.N, nS = a.nS;
  float2* eF = (float2*)(se + N);
  float2* oS = eF + N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double e = a.eq[i];
    const float h = (float)e;
    se[i] = e;
    eF[i] = make_float2(h, (float)(e - (double)h));
  }
  for (int i = threadIdx.x; i < nS; i += blockDim.x) oS[i] = a.OmF[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int pend = N - a.nR;
  const int nl = *s.nact;
  const bool bad = *a.bad != 0;
  const long long N1 = N, N2 = N1 * N1;
  for (;;) {
    __syncthreads();  // the previous orbital's s_p / s_w / s_done have been read by every thread
    if (threadIdx.x == 0) {
      const int idx = atomicAdd(a.queue, 1);
      s_p = idx < nl ? s.list[idx] : -1;
      s_w = s_p >= 0 ? s.w[s_p] : 0.0;
      s_done = 0;
    }
    __syncthreads();
    const int p = s_p;
    if (p < 0) break;
    const float* Rp = a.Rt + (long long)nS * N1 * p;
    const double* rp = a.rho + p;
    for (;;) {  // at most maxit steps: every step increments nit[p]
      const double w = s_w;
      const float w_hi = (float)w;
      const float w_lo = (float)(w - (double)w_hi);
      float so_h = 0.f, so_l = 0.f, sv_h = 0.f, sv_l = 0.f, d_h = 0.f, d_l = 0.f;
      double Sn = 0.0, Dn = 0.0;  // window (FP64) parts, per lane
      for (int q = a.nC + warp; q < pend; q += NEWT_WARPS) {
        const bool occ = q < a.nO;
        const float2 eq = eF[q];
        const float chi = w_hi - eq.x;
        const float bb = chi - w_hi;
        const float clo = ((w_hi - (chi - bb)) + (-eq.x - bb)) + (w_lo - eq.y);
        const float sg = occ ? 1.f : -1.f;
        int lo = 0, hi = nS;
        if (!bad) {
          const float ctr = -sg * chi;
          lo = om_lower_bound(oS, 0, 0, nS, ctr - a.tau);
          hi = om_lower_bound(oS, 0, lo, nS, ctr + a.tau);
        }
        const float* Rq = Rp + (long long)nS * q;
        float sl = 0.f, dl = 0.f;
        int m0 = 0;
        // batches of NEWT_U coalesced warp loads, the next batch issued before the current one
        // is used (each lane still takes its m in increasing order)
        const int nfull = nS / (32 * NEWT_U);
        float rv[NEWT_U];
        if (nfull > 0) {
#pragma unroll
          for (int u = 0; u < NEWT_U; ++u) rv[u] = __ldg(Rq + 32 * u + lane);
        }
        for (int b = 0; b < nfull; ++b, m0 += 32 * NEWT_U) {
          float rn[NEWT_U];
          const bool more = b + 1 < nfull;
          if (more) {
#pragma unroll
            for (int u = 0; u < NEWT_U; ++u) rn[u] = __ldg(Rq + m0 + 32 * NEWT_U + 32 * u + lane);
          }
#pragma unroll
          for (int u = 0; u < NEWT_U; ++u) {
            const int m = m0 + 32 * u + lane;
            const float2 o = oS[m];
            const float e = fmaf(sg, o.x, chi) + fmaf(sg, o.y, clo);
            float r = rcp32(e);
            r = (m >= lo && m < hi) ? 0.f : r;
            const float t = rv[u] * r;
            sl += t;
            dl = fmaf(t, r, dl);
          }
          if (more) {
#pragma unroll
            for (int u = 0; u < NEWT_U; ++u) rv[u] = rn[u];
          }
        }
        for (int m = m0 + lane; m < nS; m += 32) {
          const float2 o = oS[m];
          const float e = fmaf(sg, o.x, chi) + fmaf(sg, o.y, clo);
          float r = rcp32(e);
          r = (m >= lo && m < hi) ? 0.f : r;
          const float t = __ldg(Rq + m) * r;
          sl += t;
          dl = fmaf(t, r, dl);
        }
        for (int o = 16; o > 0; o >>= 1) {
          sl += __shfl_xor_sync(0xffffffffu, sl, o);
          dl += __shfl_xor_sync(0xffffffffu, dl, o);
        }
        if (occ) ff_add(so_h, so_l, sl);
        else ff_add(sv_h, sv_l, sl);
        ff_add(d_h, d_l, dl);
        // the window, in FP64 (RGW_Re_SigC.f90:30-50 / RGW_Re_dSigC.f90:30-50 with eta = 0)
        for (int m = lo + lane; m < hi; m += 32) {
          const double om = __ldg(a.Om + m);
          const double x = __ldg(rp + N1 * q + N2 * m);
          const double ir = rcp_nr(occ ? (w - se[q] + om) : (w - se[q] - om));
          const double t = (2.0 * (x * x)) * ir;
          Sn += t;
          Dn = fma(t, ir, Dn);
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        Sn += __shfl_xor_sync(0xffffffffu, Sn, o);
        Dn += __shfl_xor_sync(0xffffffffu, Dn, o);
      }
      // lanes hold identical float-float accumulators (the shuffles gave every lane the sums)
      if (lane == 0) {
        r_sig[warp] = (((double)so_h + (double)so_l) + ((double)sv_h + (double)sv_l)) + Sn;
        r_ds[warp] = -(((double)d_h + (double)d_l) + Dn);
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        double sig = 0.0, dsig = 0.0;
        for (int k = 0; k < NEWT_WARPS; ++k) {
          sig += r_sig[k];
          dsig += r_ds[k];
        }
        const int nIt = s.nit[p] + 1;
        s.nit[p] = nIt;
        s.evals[p] += 1;
        const double f = w - a.eHF[p] - sig;
        const double df = 1.0 / (1.0 - dsig);
        const double wn = w - df * f;
        s.w[p] = wn;
        s.df[p] = df;
        const bool ok = !(fabs(f) > QP_THRESH);
        if (ok || nIt >= a.maxit) {
          s.active[p] = 0;
          s.conv[p] = ok;
          s_done = 1;
        }
        s_w = wn;
      }
      __syncthreads();
      if (s_done) break;
    }
  }
}

// RGW_QP_graph.f90:78-86: a search that used all maxIt steps keeps eGWlin (and Z) -- also when
// its last step met the threshold, as the reference tests nIt == maxIt after the loop
__global__ void k_qp_finish(int N, int nC, int nR, const double* __restrict__ eGWlin, QPState s,
                            double* __restrict__ eGW, double* __restrict__ Z, int* status,
                            int maxit) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    if (p < nC || p >= N - nR) continue;
    if (s.nit[p] == maxit) {
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

// Root certificate of a guess-started Newton search (eta = 0, no SRG).  Between consecutive poles
// p_k = e_q -+ Om_m the QP function f(w) = w - eHF - sum_k R_k/(w - p_k) is increasing (f' >= 1)
// and f''(w) = 2 [A(w) - B(w)] with A = sum_{p_k > w} R_k/(p_k - w)^3 (increasing in w) and
// B = sum_{p_k < w} R_k/(w - p_k)^3 (decreasing), so f'' is increasing on any pole-free interval.
// Let r be the root the guess-started search converged to and w0 = eGWlin the reference start.
// If no pole lies between w0 and r, and f''(r) has the sign of w0 - r (then f'' keeps that sign
// on the whole interval between them, f'' being monotone), Newton from w0 converges monotonically
// to r (the classical convex-case theorem): the reference search from eGWlin ends on the same
// root, and the guess-started result is kept.  Otherwise the orbital restarts from eGWlin.  One
// FP64 sweep at r per guess-started orbital that converged: A, B and the count of poles strictly
// between w0 and r (or at either end).
constexpr int CERT_ACC = 3;

__global__ void __launch_bounds__(SIG_WARPS * 32)
    k_cert_partial(int N, int nC, int nO, int nR, int nS, int nchunks, int mper,
                   const double* __restrict__ e, const double* __restrict__ w0s, QPState st,
                   const double* __restrict__ Om, const double* __restrict__ rho,
                   double* __restrict__ part) {
  extern __shared__ double se[];
  __shared__ double acc[CERT_ACC][SIG_WARPS][32];
  for (int i = threadIdx.x; i < N; i += blockDim.x) se[i] = e[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p = nC + blockIdx.x * 32 + lane;
  const int pend = N - nR;
  __syncthreads();
  double sa = 0.0, sb = 0.0, cross = 0.0;
  const bool need = p < pend && st.conv[p] && !(st.fromref && st.fromref[p]);
  if (need) {
    const double w = st.w[p], d0 = w0s[p] - w;
    const long long N1 = N, N2 = N1 * N1;
    const int m0 = blockIdx.y * mper, m1 = min(nS, m0 + mper);
    for (int mm = m0 + warp; mm < m1; mm += SIG_WARPS) {
      const double om = Om[mm];
      const double* r = rho + p + N2 * mm;
      for (int q = nC; q < pend; ++q) {
        const double x = r[N1 * q];
        const double R = 2.0 * (x * x);
        const double eps = q < nO ? (w - se[q] + om) : (w - se[q] - om);  // r - p_k
        const double eps0 = eps + d0;                                      // w0 - p_k (approx.)
        const double ie = rcp_nr(eps);
        const double t = R * ie * ie * ie;
        if (eps > 0.0) sb += t;
        else sa -= t;
        // a pole between w0 and r, or within rounding of either end, voids the certificate
        if (!(eps * eps0 > 0.0) || fabs(eps0) <= 1e-12 * (1.0 + fabs(w))) cross += 1.0;
      }
    }
  }
  acc[0][warp][lane] = sa;
  acc[1][warp][lane] = sb;
  acc[2][warp][lane] = cross;
  __syncthreads();
  if (warp == 0 && p < pend) {
    const size_t stride = (size_t)nchunks * N;
    double a = 0.0, b = 0.0, c = 0.0;
    for (int w = 0; w < SIG_WARPS; ++w) {
      a += acc[0][w][lane];
      b += acc[1][w][lane];
      c += acc[2][w][lane];
    }
    const size_t o = (size_t)blockIdx.y * N + p;
    part[o] = a;
    part[o + stride] = b;
    part[o + 2 * stride] = c;
  }
}

__global__ void k_cert_final(int N, int nC, int nR, int nchunks, const double* __restrict__ part,
                             const double* __restrict__ w0s, QPState st, int* __restrict__ cert) {
  const size_t stride = (size_t)nchunks * N;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    const bool need = p >= nC && p < N - nR && st.conv[p] && !(st.fromref && st.fromref[p]);
    int ok = 0;
    if (need) {
      double a = 0.0, b = 0.0, c = 0.0;
      for (int k = 0; k < nchunks; ++k) {
        const size_t o = (size_t)k * N + p;
        a += part[o];
        b += part[o + stride];
        c += part[o + 2 * stride];
      }
      const double r = st.w[p], w0 = w0s[p], margin = 1e-9 * (a + b);
      // f''(r)/2 = a - b must have the sign of w0 - r (with a margin for rounding)
      const bool convex_ok = (w0 > r && a - b > margin) || (w0 < r && b - a > margin) || w0 == r;
      ok = c == 0.0 && convex_ok && a == a && b == b;
      st.evals[p] += 1;
    }
    cert[p] = ok;
  }
}

}  // namespace

static int sigma_sweep(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                       int nS, const double* eq, const double* wp, const double* Om,
                       const double* rho, const int* list, const int* nact, double** part_out,
                       int* nchunks_out, const qk_sigma_ff* ff = nullptr, int nact_max = -1) {
  // p tiles: all orbitals, or (with a compacted list) an upper bound on the active count.  The
  // partition of every orbital's terms into chunks (the summation order) is fixed by N and nS
  // alone -- never by how many orbitals are still searching -- so an orbital's Sigma(w) is the
  // same bits whatever the other orbitals do (a Newton search started elsewhere for some
  // orbitals must not perturb the chaotic searches of the others)
  int nact_p = N - nR - nC;
  if (list && nact_max >= 0 && nact_max < nact_p) nact_p = nact_max;
  const int cm = qk_tune_get(ctx, TUNE_SIGMA_CHUNKS, (long long)nS, 4);
  const int nq = N - nR - nC;
  const int nall = nq;  // the orbital count the partition is chosen for
  // the mixed sweep keeps e and Om in shared memory; beyond that it takes the FP64 sweep
  const size_t ff_smem = (size_t)N * 16 + (size_t)nS * 8;
  const bool use_ff = ff && !doSRG && eta == 0.0 && ff_smem <= NEWT_SMEM_MAX;
  SigArgs a;
  a.N = N; a.nC = nC; a.nO = nO; a.nR = nR; a.nS = nS;
  a.doSRG = doSRG; a.eta = eta; a.flow = flow;
  a.eq = eq; a.wp = wp; a.Om = Om; a.rho = rho; a.list = list; a.nact = nact;
  double* part = nullptr;
  int nchunks = 1;
  if (use_ff) {
    // a CTA per (orbital, q group): as many groups as fill the resident CTA slots in one wave
    // when every orbital is active (a second, partial wave left SMs idle)
    const int items = nall > 0 ? nall : 1;
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
      attr_err = cudaFuncSetAttribute(k_sigma_partial_ffT,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)NEWT_SMEM_MAX);
    });
    QK_CK(attr_err);
    int ffT_per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ffT_per_sm, k_sigma_partial_ffT,
                                                      FFT_WARPS * 32, ff_smem) != cudaSuccess ||
        ffT_per_sm < 1)
      ffT_per_sm = 1;
    (void)cm;
    int qgroups = ffT_per_sm * ctx->num_sms / items;
    const int gmax = nq / FFT_WARPS > 1 ? nq / FFT_WARPS : 1;
    if (qgroups > gmax) qgroups = gmax;
    if (qgroups < 1) qgroups = 1;
    const int qper = (nq + qgroups - 1) / qgroups;
    qgroups = (nq + qper - 1) / qper;
    if (qgroups < 1) qgroups = 1;
    nchunks = qgroups;
    a.nchunks = nchunks; a.mper = nS; a.mchunks = 1; a.qper = qper;
    // every (chunk, p) entry the consumers read is written by the sweep: no clearing needed
    QK_TRY(qk_wst(ctx, W_MISC, (size_t)3 * nchunks * N + 64, &part));
    a.part = part;
    if (nact_p > 0 && nS > 0) {
      SigFF f{ff->R, ff->OmF, ff->bad, ff->tau};
      k_sigma_partial_ffT<<<dim3(nact_p, nchunks), FFT_WARPS * 32, ff_smem, ctx->stream>>>(a, f);
      QK_LAUNCHED();
    }
  } else {
    const int ptiles = (nact_p + 31) / 32;                // launched
    const int ptiles_all = (nall + 31) / 32 > 0 ? (nall + 31) / 32 : 1;
    int mchunks = (cm * ctx->num_sms + ptiles_all - 1) / ptiles_all;
    const int maxch = (nS + SIG_WARPS - 1) / SIG_WARPS;
    if (mchunks > maxch) mchunks = maxch;
    if (mchunks < 1) mchunks = 1;
    const int mper = (nS + mchunks - 1) / mchunks;
    mchunks = (nS + mper - 1) / mper;
    // two q groups as well, so that the last few still-searching orbitals keep more SMs busy
    // (more groups cost staging overhead when all orbitals are active)
    int qgroups = nq >= 32 ? 2 : 1;
    const int qper = (nq + qgroups - 1) / qgroups;
    qgroups = (nq + qper - 1) / qper;
    nchunks = mchunks * qgroups;
    a.nchunks = nchunks; a.mper = mper; a.mchunks = mchunks; a.qper = qper;
    QK_TRY(qk_wst(ctx, W_MISC, (size_t)3 * nchunks * N + 64, &part));
    a.part = part;
    if (ptiles > 0 && nS > 0) {
      k_sigma_partial<<<dim3(ptiles, nchunks), SIG_WARPS * 32, N * sizeof(double), ctx->stream>>>(a);
      QK_LAUNCHED();
    }
  }
  *part_out = part;
  *nchunks_out = nchunks;
  return QK_OK;
}

int qk_sigma_ff_prep(qk_ctx* ctx, int N, int nS, const double* rho, const double* Om,
                     qk_sigma_ff* ff) {
  const long long n = (long long)N * N * nS;
  float *R = nullptr, *of = nullptr;
  QK_TRY(qk_wst(ctx, W_RHO32, (size_t)n + 32, &R));
  QK_TRY(qk_wst(ctx, W_OMF, 2 * (size_t)nS + 16, &of));
  float2* OmF = (float2*)of;
  int* bad = (int*)(of + 2 * (size_t)nS);
  QK_CK(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  const dim3 tg((N + 31) / 32, (nS + 31) / 32, N);
  if (tg.y > 65535 || tg.z > 65535) return qk_fail(ctx, QK_ERR_ARG, "k_sigma_ff_prepT grid");
  k_sigma_ff_prepT<<<tg, dim3(32, 8), 0, ctx->stream>>>(N, nS, rho, R);
  QK_LAUNCHED();
  k_om_pairs<<<(nS + 255) / 256, 256, 0, ctx->stream>>>(nS, Om, OmF, bad);
  QK_LAUNCHED();
  ff->R = R;
  ff->OmF = OmF;
  ff->bad = bad;
  ff->tau = 0.01f;  // Ha: the FP32-pair denominators are exact to ~1e-12 Ha outside
  return QK_OK;
}

int qk_sigma_diag(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                  int nS, const double* e, const double* Om, const double* rho, double* Sig,
                  double* Z, double* EcGM, const qk_sigma_ff* ff) {
  double* part;
  int nch;
  QK_TRY(sigma_sweep(ctx, doSRG, eta, flow, N, nC, nO, nR, nS, e, nullptr, Om, rho, nullptr,
                     nullptr, &part, &nch, ff));
  k_sigma_final<<<1, 1024, 0, ctx->stream>>>(N, nC, nO, nR, nch, part, Sig, Z, EcGM);
  QK_LAUNCHED();
  return QK_OK;
}

// certificates of the guess-started roots (all 0 where the pole structure of the certificate
// does not hold: eta != 0 or SRG, whose searches then all restart from the reference start)
static int qp_certify(qk_ctx* ctx, int doSRG, double eta, int N, int nC, int nO, int nR, int nS,
                      const double* e, const double* w0, const QPState& s, const double* Om,
                      const double* rho, int* cert) {
  if (doSRG || eta != 0.0) {
    QK_CK(cudaMemsetAsync(cert, 0, sizeof(int) * N, ctx->stream));
    return QK_OK;
  }
  const int nact = N - nR - nC;
  const int ptiles = (nact + 31) / 32;
  int nchunks = (4 * ctx->num_sms + ptiles - 1) / (ptiles > 0 ? ptiles : 1);
  const int maxch = (nS + SIG_WARPS - 1) / SIG_WARPS;
  if (nchunks > maxch) nchunks = maxch;
  if (nchunks < 1) nchunks = 1;
  const int mper = (nS + nchunks - 1) / nchunks;
  nchunks = (nS + mper - 1) / mper;
  double* part = nullptr;
  QK_TRY(qk_wst(ctx, W_MISC, (size_t)CERT_ACC * nchunks * N + 64, &part));
  QK_CK(cudaMemsetAsync(part, 0, sizeof(double) * CERT_ACC * (size_t)nchunks * N, ctx->stream));
  if (ptiles > 0) {
    k_cert_partial<<<dim3(ptiles, nchunks), SIG_WARPS * 32, N * sizeof(double), ctx->stream>>>(
        N, nC, nO, nR, nS, nchunks, mper, e, w0, s, Om, rho, part);
    QK_LAUNCHED();
  }
  k_cert_final<<<(N + 127) / 128, 128, 0, ctx->stream>>>(N, nC, nR, nchunks, part, w0, s, cert);
  QK_LAUNCHED();
  return QK_OK;
}

int qk_qp_newton(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                 int nS, const double* eHF, const double* Om, const double* rho,
                 const double* eGWlin, const double* eOld, double* eGW, double* Z,
                 const double* w_guess, int guess_maxit, const qk_sigma_ff* ff,
                 const int* guess_fromref) {
  double* st = nullptr;
  QK_TRY(qk_wst(ctx, W_M2, (size_t)9 * N + 64, &st));
  QPState s;
  s.w = st;
  s.df = st + N;
  s.nit = (int*)(st + 2 * N);
  s.active = (int*)(st + 3 * N);
  s.list = (int*)(st + 4 * N);
  s.conv = (int*)(st + 5 * N);
  s.evals = (int*)(st + 6 * N);
  s.nact = (int*)(st + 7 * N);
  s.fromref = w_guess ? guess_fromref : nullptr;
  // phase 1 (learned guess only): at most guess_maxit steps from the guess; phase 2: the
  // reference search (RGW_QP_graph.f90:50-92) from eGWlin for every orbital not yet converged
  k_qp_init<<<1, 1024, 0, ctx->stream>>>(N, nC, nR, w_guess ? w_guess : eGWlin, s);
  QK_LAUNCHED();
  // mixed tier: the persistent on-chip search over a p-major copy of R
  const size_t newt_smem = (size_t)N * 16 + (size_t)nS * 8;
  // tunable per nS bucket: 1 (default) = persistent kernel, 2 = per-step sweeps
  const bool persistent = ff && !doSRG && eta == 0.0 && newt_smem <= NEWT_SMEM_MAX &&
                          qk_tune_get(ctx, TUNE_QP_PERSIST, (long long)nS, 1) != 2;
  const float* Rt = ff ? ff->R : nullptr;  // p-major R of qk_sigma_ff_prep
  int* queue = nullptr;
  if (persistent) {
    QK_TRY(qk_wst(ctx, W_QPQUEUE, 16, &queue));
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
      attr_err = cudaFuncSetAttribute(k_qp_newton_ff, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)NEWT_SMEM_MAX);
    });
    QK_CK(attr_err);
  }
  for (int phase = w_guess ? 1 : 2; phase <= 2; ++phase) {
    const int maxit = phase == 1 ? guess_maxit : ctx->newton_maxit;
    if (phase == 2 && w_guess) {
      int* cert = (int*)(st + 8 * N);
      QK_TRY(qp_certify(ctx, doSRG, eta, N, nC, nO, nR, nS, eOld, eGWlin, s, Om, rho, cert));
      k_qp_restart<<<1, 1024, 0, ctx->stream>>>(N, nC, nR, eGWlin, cert, s, ctx->newton_maxit);
      QK_LAUNCHED();
    }
    if (persistent) {
      QK_CK(cudaMemsetAsync(queue, 0, sizeof(int), ctx->stream));
      NewtFF a{N, nC, nO, nR, nS, maxit, eOld, eHF, Om, rho, Rt, ff->OmF, ff->bad, ff->tau, queue};
      const int nq = N - nC - nR;
      int grid = ctx->num_sms;
      // batch workers run several systems at once: each takes its share of the SMs
      if (ctx->sytrd_max_ctas > 0 && grid > ctx->sytrd_max_ctas) grid = ctx->sytrd_max_ctas;
      if (grid > nq) grid = nq;
      if (grid < 1) grid = 1;
      k_qp_newton_ff<<<grid, NEWT_WARPS * 32, newt_smem, ctx->stream>>>(a, s);
      QK_LAUNCHED();
      continue;
    }
    int hact = N;  // upper bound on the active count, refreshed by the polls
    for (int it = 0; it < maxit; ++it) {
      double* part;
      int nch;
      QK_TRY(sigma_sweep(ctx, doSRG, eta, flow, N, nC, nO, nR, nS, eOld, s.w, Om, rho, s.list,
                         s.nact, &part, &nch, ff, hact));
      k_qp_update<<<1, 1024, 0, ctx->stream>>>(N, nch, part, eHF, s, maxit);
      QK_LAUNCHED();
      if (!ctx->capturing && (it & 3) == 3) {  // poll the active count every 4 steps
        QK_CK(cudaMemcpyAsync(&hact, s.nact, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        QK_CK(cudaStreamSynchronize(ctx->stream));
        if (hact == 0) break;
      }
    }
  }
  k_qp_finish<<<(N + 255) / 256, 256, 0, ctx->stream>>>(N, nC, nR, eGWlin, s, eGW, Z, ctx->d_status,
                                                        ctx->newton_maxit);
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

// Per orbital p the feature sweep evaluates the pole sums at the linearised root w = eGWlin_p:
// S0 = sum R/eps, S1 = sum R/eps^2, S2 = sum R/eps^3 (R = 2 rho^2, eps = w - e_q +- Om_m, eta = 0)
// and the nearest pole (min |eps| with its R): one sweep gives the Newton and Halley steps of the
// QP equation f(w) = w - eHF - Sigma(w) from the reference start.
constexpr int NACC = 5;  // S0, S1, S2, min |eps|, R at the minimum

__global__ void __launch_bounds__(SIG_WARPS * 32)
    k_feature_partial(int N, int nC, int nO, int nR, int nS, int nchunks, int mper,
                      const double* __restrict__ e, const double* __restrict__ wlin,
                      const double* __restrict__ Om, const double* __restrict__ rho,
                      double* __restrict__ part) {
  extern __shared__ double se[];
  __shared__ double acc[NACC][SIG_WARPS][32];
  for (int i = threadIdx.x; i < N; i += blockDim.x) se[i] = e[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p = nC + blockIdx.x * 32 + lane;
  const int pend = N - nR;
  __syncthreads();
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, emin = INFINITY, rmin = 0.0;
  if (p < pend) {
    const double w = wlin[p];
    const long long N1 = N, N2 = N1 * N1;
    const int m0 = blockIdx.y * mper, m1 = min(nS, m0 + mper);
    for (int mm = m0 + warp; mm < m1; mm += SIG_WARPS) {
      const double om = Om[mm];
      const double* r = rho + p + N2 * mm;
      for (int q = nC; q < pend; ++q) {
        const double x = r[N1 * q];
        const double R = 2.0 * (x * x);
        const double eps = q < nO ? (w - se[q] + om) : (w - se[q] - om);
        const double ie = rcp_nr(eps);
        const double t = R * ie;
        s0 += t;
        s1 = fma(t, ie, s1);
        s2 = fma(t * ie, ie, s2);
        if (fabs(eps) < emin) {
          emin = fabs(eps);
          rmin = R;
        }
      }
    }
  }
  acc[0][warp][lane] = s0;
  acc[1][warp][lane] = s1;
  acc[2][warp][lane] = s2;
  acc[3][warp][lane] = emin;
  acc[4][warp][lane] = rmin;
  __syncthreads();
  if (warp == 0 && p < pend) {
    const size_t stride = (size_t)nchunks * N;
    double t0 = 0.0, t1 = 0.0, t2 = 0.0, em = INFINITY, rm = 0.0;
    for (int w = 0; w < SIG_WARPS; ++w) {
      t0 += acc[0][w][lane];
      t1 += acc[1][w][lane];
      t2 += acc[2][w][lane];
      if (acc[3][w][lane] < em) {
        em = acc[3][w][lane];
        rm = acc[4][w][lane];
      }
    }
    const size_t o = (size_t)blockIdx.y * N + p;
    part[o] = t0;
    part[o + stride] = t1;
    part[o + 2 * stride] = t2;
    part[o + 3 * stride] = em;
    part[o + 4 * stride] = rm;
  }
}

__device__ __forceinline__ float clampf(double x, double lim) {
  return (float)(x != x ? 0.0 : fmax(-lim, fmin(lim, x)));
}

__global__ void k_feature_final(int N, int nC, int nO, int nR, int nchunks,
                                const double* __restrict__ part, const double* __restrict__ e,
                                const double* __restrict__ wlin, const double* __restrict__ Om,
                                const double* __restrict__ Sig, const double* __restrict__ Z,
                                float* __restrict__ F, double* __restrict__ hal) {
  const size_t stride = (size_t)nchunks * N;
  const double eh = e[nO - 1], el = e[nO];
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < N; p += gridDim.x * blockDim.x) {
    double S0 = 0.0, S1 = 0.0, S2 = 0.0, em = INFINITY, rm = 0.0;
    if (p >= nC && p < N - nR)
      for (int c = 0; c < nchunks; ++c) {
        const size_t o = (size_t)c * N + p;
        S0 += part[o];
        S1 += part[o + stride];
        S2 += part[o + 2 * stride];
        if (part[o + 3 * stride] < em) {
          em = part[o + 3 * stride];
          rm = part[o + 4 * stride];
        }
      }
    const double ep = e[p];
    const double w = wlin[p];
    // f(w) = w - eHF - Sigma(w), f' = 1 - Sigma' = 1 + S1, f'' = -Sigma'' = -2 S2
    const double f0 = w - ep - S0, f1 = 1.0 + S1, f2 = -2.0 * S2;
    const double dn = -f0 / f1;
    const double dh = -2.0 * f0 * f1 / (2.0 * f1 * f1 - f0 * f2);
    if (hal) hal[p] = (dh == dh && fabs(dh) <= 1.0) ? dh : NAN;
    float* f = F + (size_t)p * QK_MLP_NIN;
    f[0] = (float)ep;
    f[1] = p < nO ? 1.f : 0.f;
    f[2] = (float)(ep - eh);
    f[3] = (float)(ep - el);
    f[4] = (float)Sig[p];
    f[5] = (float)Z[p];
    f[6] = (float)(Z[p] * Sig[p]);  // eGWlin - eHF
    f[7] = (float)(1.0 - 1.0 / Z[p]);
    f[8] = clampf(dn, 1.0);          // Newton step from eGWlin
    f[9] = clampf(dh, 1.0);          // Halley step from eGWlin
    f[10] = clampf(f0, 1.0);
    f[11] = clampf(S1, 20.0);
    f[12] = (float)log10(em + 1e-12);
    f[13] = clampf(log10(rm / (em + 1e-300) + 1e-12), 12.0);
    f[14] = (float)Om[0];
    f[15] = (float)log((double)N);
  }
}

}  // namespace

int qk_features(qk_ctx* ctx, int N, int nC, int nO, int nR, int nS, const double* e,
                const double* wlin, const double* Om, const double* rho, const double* Sig,
                const double* Z, float* F, double* hal) {
  const int nact = N - nR - nC;
  const int ptiles = (nact + 31) / 32;
  int nchunks = (4 * ctx->num_sms + ptiles - 1) / (ptiles > 0 ? ptiles : 1);
  const int maxch = (nS + SIG_WARPS - 1) / SIG_WARPS;
  if (nchunks > maxch) nchunks = maxch;
  if (nchunks < 1) nchunks = 1;
  const int mper = (nS + nchunks - 1) / nchunks;
  nchunks = (nS + mper - 1) / mper;
  double* part = nullptr;
  QK_TRY(qk_wst(ctx, W_MISC, (size_t)NACC * nchunks * N + 64, &part));
  QK_CK(cudaMemsetAsync(part, 0, sizeof(double) * NACC * (size_t)nchunks * N, ctx->stream));
  if (ptiles > 0) {
    k_feature_partial<<<dim3(ptiles, nchunks), SIG_WARPS * 32, N * sizeof(double), ctx->stream>>>(
        N, nC, nO, nR, nS, nchunks, mper, e, wlin, Om, rho, part);
    QK_LAUNCHED();
  }
  k_feature_final<<<(N + 127) / 128, 128, 0, ctx->stream>>>(N, nC, nO, nR, nchunks, part, e, wlin,
                                                           Om, Sig, Z, F, hal);
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
