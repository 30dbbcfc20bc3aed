// k_eig.cu -- dense symmetric FP64 eigensolver, written for GB300.
//
// Replaces dsyev('V','U') (utils/wrap_lapack.f90:99-136) as used by LR/phRLR.f90:54,67.
// Pipeline (all on the GPU, no vendor solver):
//   1. k_sytrd: Householder tridiagonalisation (lower variant) in ONE persistent cooperative
//      kernel.  Each iteration fuses the rank-2 update of step k with the symmetric mat-vec of
//      step k+1 on the lower triangle only, so the trailing triangle is streamed once per column
//      (read+write) and every element costs 4 FMAs (LAPACK's 4/3 n^3 flops); every CTA
//      recomputes the O(n) vector work redundantly (bitwise identical in all CTAs), leaving
//      one bounded grid barrier per column.  The mat-vec's partial sums from different CTAs
//      meet in exact (order-independent) accumulators, so the result is the same in every run.
//   2. k_stebz: Sturm-count k-section (K lanes per eigenvalue), full FP64 precision.
//   3. k_stein: inverse iteration on T - lambda I (tridiagonal GEPP), one thread per cluster of
//      close eigenvalues, modified Gram-Schmidt inside clusters; eigenvectors written as rows.
//   The mixed tier runs steps 1 and 2 in double-float arithmetic on the FP32 pipe (k_sytrd_df,
//   sturm_count_df; GB300 issues FP32 at 64x its FP64 rate) and two inverse-iteration steps.
//   4. Blocked back-transformation E <- E * Q^T with compact-WY blocks of 128 reflectors on the
//      FP64 GEMM, or with compensated FP32 products in the mixed tier (all T factors from one
//      batched GEMM and one launch).
// Eigenvalues come out ascending (as dsyev).  Eigenvectors are defined up to sign/rotation in
// degenerate subspaces, which every downstream GW quantity is invariant to.
#include <cmath>
#include <cfloat>
#include <condition_variable>
#include <mutex>
#include <vector>
#include "qk_internal.cuh"

namespace {

constexpr int TRI_THREADS = 1024;
constexpr int TRI_SMEM_MAX = 227 * 1024 - 1024;  // tiles + (when they fit) the three vectors
constexpr int TRI_TC = 16;          // columns per lower-triangle tile of the fused pass
constexpr int TRI_TLD = 33;         // padded leading dimension of a warp's shared tile
constexpr int TRI_TILE_BYTES = (TRI_THREADS / 32) * TRI_TC * TRI_TLD * 8;
constexpr int BT_NB = 128;          // reflectors per compact-WY block
constexpr double CLUSTER_REL = 1e-7;  // eigenvalues closer than this * ||T||_1 share a cluster
constexpr int SB = 16;                // inverse iteration: steps per batch of prefetched loads

// Sum over the CTA with few FP64 operations (the FP64 pipe is the scarce resource here): the
// per-thread partials go to shared memory and warps 0-3 (one per SM sub-partition, so their
// FP64 issue runs in parallel) add the first cnt of them (the rest are zero) in two chains per
// lane, then one butterfly each.  Thread 0 adds the four warp sums and runs fin(total) -- the
// scalar follow-up work, done once instead of by every warp -- before the closing barrier
// publishes its results.  scratch holds blockDim.x + 4 doubles; blockDim.x >= 128.
template <class Fin>
__device__ __forceinline__ void tri_block_sum(double v, double* scratch, int cnt, Fin fin) {
  const int tid = threadIdx.x;
  scratch[tid] = v;
  __syncthreads();
  if (tid < 128) {
    double a0 = 0.0, a1 = 0.0;
    int i = tid;
    for (; i + 128 < cnt; i += 256) {
      a0 += scratch[i];
      a1 += scratch[i + 128];
    }
    if (i < cnt) a0 += scratch[i];
    double t = a0 + a1;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    double* red4 = scratch + blockDim.x;
    if ((tid & 31) == 0) red4[tid >> 5] = t;
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (tid == 0) fin((red4[0] + red4[1]) + (red4[2] + red4[3]));
  }
  __syncthreads();
}

// Order-independent accumulation of the mat-vec partial sums.  Several warps of several CTAs
// add into each element of p, so plain FP64 atomics would make the result depend on their
// order.  Each contribution x is instead split into two parts aligned to fixed binary grids,
// and each grid has its own accumulator: every part is a multiple of its grid's spacing and every
// running sum stays below 2^53 spacings, so all additions are exact and the sums are the same in
// any order.  The grids come from a bound B >= sum of |x| over all contributions to an element
// (B = 2 ||A||_F ||u||_2): the first has spacing 2^g1, g1 = E - 51 (2^E > B), the second 2^g2,
// g2 = E - 92.  A part is its input truncated toward zero to the grid, by clearing low
// significand bits on the integer pipe (FP64 issue is the scarce resource here), and the
// remainder is exact: x = q1 + r1, |r1| < 2^g1; r1 = q2 + (dropped, < 2^g2 = 2^-92 2^E).  Up to
// 2^12 contributions per element keep the second sum exact (n <= 2^16).
__device__ __forceinline__ double tri_trunc(double x, int g) {
  const long long b = __double_as_longlong(x);
  const int k = g - ((int)((b >> 52) & 0x7FF) - 1075);  // low significand bits below 2^g
  const long long keep = k >= 53 ? (long long)0x8000000000000000ULL   // +-0
                                 : (k <= 0 ? -1LL : ~((1LL << k) - 1));
  return __longlong_as_double(b & keep);
}

__device__ __forceinline__ void tri_exact_add(double* b1, double* b2, double x, int g1) {
  const double q1 = tri_trunc(x, g1);
  const double q2 = tri_trunc(__dsub_rn(x, q1), g1 - 41);
  atomicAdd(b1, q1);
  atomicAdd(b2, q2);
}

struct TriArgs {
  double* A;
  long long lda;
  int n;
  double* d;
  double* e;
  double* tau;
  double* V;
  long long ldv;
  int df;        // 1: double-float arithmetic on the FP32 pipe (sytrd_df_body)
  double* vscal;   // df: n slots for the reflectors' scale factors (consumed by k_tri_df_finish)
  double* dfscale; // df: one slot, the power of two that undoes the matrix scaling
  double* pbuf;  // 6*n: three rotating p vectors, each as two exact accumulators (n + n)
  double* fslot; // one partial sum of ||A||_F^2 per CTA of the group
  double* gvec;  // (CTAs of the group) * 3 * n when vectors do not fit in shared memory
  unsigned* bar;
  int* status;
  int use_smem;
};

// CTA group of a tridiagonalisation: the whole grid (k_sytrd; the sizes stay in special
// registers) or a slice of it (k_sytrd_grouped; the sizes live in shared memory)
struct TriGridWhole {
  __device__ __forceinline__ int size() const { return (int)gridDim.x; }
  __device__ __forceinline__ int rank() const { return (int)blockIdx.x; }
};
struct TriGridSlice {
  const int* s;  // shared memory: {size, rank}
  __device__ __forceinline__ int size() const { return *(const volatile int*)s; }
  __device__ __forceinline__ int rank() const { return *(const volatile int*)(s + 1); }
};

// The tridiagonalisation of one matrix by a group of co-resident CTAs.  With kFixed, every
// rounded quantity is independent of the group size: ||A||_F is summed over fixed column chunks
// and each tile's row partial sum is split into the exact accumulators on its own (not summed
// over a warp's run of tiles, whose extent depends on the group size), so the result is the same
// bits for any number of CTAs -- the grouped launch then sizes the groups freely.
template <class Grp, bool kFixed>
__device__ __forceinline__ void sytrd_body(const TriArgs a, const Grp grp) {
  extern __shared__ double sm[];
  __shared__ double s_pj, s_dj, s_alpha, s_sc[7], s_fro;
  __shared__ int s_g1;  // exponent of the first accumulator grid
  const int n = a.n;
  double* ytile = sm;  // one TRI_TC x TRI_TLD tile per warp
  double *vk, *wk, *vk1;
  if (a.use_smem) {
    vk = sm + TRI_TILE_BYTES / 8;
    wk = vk + n;
    vk1 = vk + 2 * n;
  } else {
    double* base = a.gvec + (size_t)grp.rank() * 3 * n;
    vk = base;
    wk = base + n;
    vk1 = base + 2 * n;
  }
  unsigned epoch = 0;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const int totwarps = grp.size() * nwarps;
  const int gthread = grp.rank() * nt + tid, totthreads = grp.size() * nt;
  double tau_k = 0.0, scal_k = 1.0;

  // ---- ||A||_F (bounds every p element's partial sums): fixed per-thread order, per-CTA slot,
  // then every CTA adds the slots in the same order, so all CTAs hold the same value ----
  if (!kFixed) {
    double fs = 0.0;
    for (int c = grp.rank(); c < n; c += grp.size()) {
      const double* col = a.A + a.lda * c;
      for (int i = c + tid; i < n; i += nt) {
        const double x = __ldcg(col + i);
        fs = fma(i == c ? x : x + x, x, fs);
      }
    }
    tri_block_sum(fs, ytile, nt, [&](double t) { __stcg(a.fslot + grp.rank(), t); });
    if (!qk_grid_barrier(a.bar, grp.size(), epoch, a.status)) return;
    if (tid == 0) {
      double t = 0.0;
      for (int b = 0; b < grp.size(); ++b) t += __ldcg(a.fslot + b);
      s_fro = sqrt(t);
    }
    __syncthreads();
  } else {
    // chunks of 32 columns, one slot each (n <= 32768), summed in chunk order
    const int nch = (n + 31) / 32;
    for (int ch = grp.rank(); ch < nch; ch += grp.size()) {
      double fs = 0.0;
      const int c1 = 32 * ch + 32 < n ? 32 * ch + 32 : n;
      for (int c = 32 * ch; c < c1; ++c) {
        const double* col = a.A + a.lda * c;
        for (int i = c + tid; i < n; i += nt) {
          const double x = __ldcg(col + i);
          fs = fma(i == c ? x : x + x, x, fs);
        }
      }
      tri_block_sum(fs, ytile, nt, [&](double t) { __stcg(a.fslot + ch, t); });
    }
    if (!qk_grid_barrier(a.bar, grp.size(), epoch, a.status)) return;
    if (tid == 0) {
      double t = 0.0;
      for (int b = 0; b < nch; ++b) t += __ldcg(a.fslot + b);
      s_fro = sqrt(t);
    }
    __syncthreads();
  }
  const double fro = s_fro;

  for (int k = -1; k <= n - 2; ++k) {
    // ---- zero the p accumulator used two iterations ahead (triple buffering) ----
    {
      double* pz = a.pbuf + (size_t)((k + 2) % 3) * n;
      double* pz2 = pz + 3 * (size_t)n;
      for (int i = gthread; i < n; i += totthreads) {
        __stcg(pz + i, 0.0);
        __stcg(pz2 + i, 0.0);
      }
    }
    // ---- small phase (redundant in every CTA): step k's scalars, then v_{k+1} from column j ----
    // FP64 is the scarce resource (one warp instruction per 64 cycles per SM sub-partition), so
    // the O(n) work is kept to 4 FMAs per element.  The reflector is kept unscaled, u = v / scal
    // with u_{j+1} = 1/scal: the scale factor goes into the scalars of the next step instead of
    // a pass over the vector (the big pass computes p~ = A' u, so p = scal p~).  The rank-2
    // update A - u w^T - w u^T with w = a1 p~ - a2 u is never formed through w: it is
    //   A_ic - (a1 u_i) p~_c - (a1 p~_i - 2 a2 u_i) u_c,
    // two FMAs per element with row scalars, and the column j it exposes is
    //   A_ij + (a2 u_j - w_j) u_i - (a1 u_j) p~_i.
    const int j = k + 1;
    const int cnt = n - j < nt ? n - j : nt;  // threads holding a non-zero partial sum
    double tau1 = 0.0, scal1 = 1.0;
    double a1 = 0.0, a2x2 = 0.0;  // step k's update scalars, kept for the big pass
    {
      const double* p = a.pbuf + (size_t)((k + 3) % 3) * n;
      double dot = 0.0;
      // four elements per thread per round, their loads issued together
      for (int i0 = j + tid; i0 < n; i0 += 4 * nt) {
        double xv[4], pv[4], uv[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int i = i0 + r * nt;
          xv[r] = i < n ? __ldcg(a.A + i + a.lda * j) : 0.0;
          pv[r] = (k >= 0 && i < n) ? __ldcg(p + i) + __ldcg(p + 3 * (size_t)n + i) : 0.0;
          uv[r] = (k >= 0 && i < n) ? vk[i] : 0.0;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int i = i0 + r * nt;
          if (i < n) {
            vk1[i] = xv[r];
            if (k >= 0) {
              wk[i] = pv[r];
              if (i == j) s_pj = pv[r];
              dot = fma(pv[r], uv[r], dot);
            }
          }
        }
      }
      if (k >= 0) {
        // (the barriers publish vk1, wk and s_pj as well)
        tri_block_sum(dot, ytile, cnt, [&](double t) {
          // true dot p.v = scal^2 p~.u;  c = tau^2 dot / 2;  w = scal^2 (tau p~ - c u)
          const double s2 = scal_k * scal_k;
          const double cc = 0.5 * tau_k * tau_k * (s2 * t);
          const double b1 = tau_k * s2, b2 = cc * s2;
          const double u = vk[j];
          const double wj = b1 * s_pj - b2 * u;
          s_sc[0] = b1;
          s_sc[1] = b2 + b2;
          s_sc[2] = b2 * u - wj;  // coefficient of u_i in column j
          s_sc[6] = -b1 * u;      // coefficient of p~_i in column j
        });
      } else {
        if (tid == 0) s_sc[0] = s_sc[1] = s_sc[2] = s_sc[6] = 0.0;
        __syncthreads();
      }
      a1 = s_sc[0];
      a2x2 = s_sc[1];
      const double cu = s_sc[2], cp = s_sc[6];
      double ss = 0.0;
      for (int i = j + tid; i < n; i += nt) {
        double x = vk1[i];
        if (k >= 0) {
          x = fma(cp, wk[i], fma(cu, vk[i], x));
          vk1[i] = x;
        }
        if (i == j) s_dj = x;
        else if (i == j + 1) s_alpha = x;
        else ss = fma(x, x, ss);
      }
      // Householder reflector of the updated column (dlarfg), computed once by thread 0
      tri_block_sum(ss, ytile, cnt, [&](double sigma) {
        double beta = 0.0, t1 = 0.0, scal = 1.0, inv = 1.0, unrm = 1.0;
        if (j <= n - 2) {
          const double alpha = s_alpha;
          if (sigma == 0.0) {
            beta = alpha;
          } else {
            beta = -copysign(sqrt(alpha * alpha + sigma), alpha);
            // reciprocals by qk_rcp (a few ulps) instead of IEEE divisions: this runs on the
            // per-column critical path, where each FP64 instruction costs ~64 cycles
            t1 = (beta - alpha) * qk_rcp(beta);
            inv = alpha - beta;
            scal = qk_rcp(inv);
            unrm = sqrt(fma(inv, inv, sigma));
          }
          vk1[j + 1] = inv;  // u_{j+1} = 1/scal, so that scal * u_{j+1} = 1
        }
        s_sc[3] = beta;
        s_sc[4] = t1;
        s_sc[5] = scal;
        // grids of the exact accumulators for p~ = A' u: |A'_ic| <= ||A||_F, so the partial
        // sums of every element are bounded by ||A||_F ||u||_2; twice that absorbs rounding
        int ex = 0;
        const double bnd = 2.0 * fro * unrm;
        if (bnd > 0.0 && bnd <= DBL_MAX) frexp(bnd, &ex);
        ex = ex < -960 ? -960 : (ex > 1000 ? 1000 : ex);
        s_g1 = ex - 51;
      });
      const double dj = s_dj;
      tau1 = s_sc[4];
      scal1 = s_sc[5];
      if (j <= n - 2) {
        // every CTA holds the reflector: the V column is written by all of them, a slice each
        if (grp.rank() == 0 && tid == 0) { a.e[j] = s_sc[3]; a.tau[j] = tau1; }
        for (int i = j + 1 + gthread; i < n; i += totthreads)
          a.V[i + a.ldv * j] = (i == j + 1) ? 1.0 : vk1[i] * scal1;
      }
      if (grp.rank() == 0 && tid == 0) a.d[j] = dj;
    }
    // ---- big pass: rank-2 update of step k fused with p_{k+1} = A' v_{k+1}, lower triangle ----
    // The trailing lower triangle is cut into tiles of 32 rows x TRI_TC columns (row block bi
    // holds tiles t = 0..2bi+1; tiles are numbered row block after row block).  Each warp takes a
    // contiguous range of tiles.  Lane = row i: it updates A(i,c) for c <= i, accumulates the row
    // part of p_i, and parks the strictly lower y(i,c) in its warp's shared tile; the lanes then
    // read the tile by columns for the transposed part of p_c.  Every element costs the two FMAs
    // of the update and one FMA for each of its two appearances in the symmetric mat-vec.
    const int r0 = k + 2;
    const int mm = n - r0;
    if (mm > 0) {
      double* pnext = a.pbuf + (size_t)((k + 1) % 3) * n;
      double* pnext2 = pnext + 3 * (size_t)n;
      const bool upd = (k >= 0);
      const bool wantp = (j <= n - 2);
      const int nb = (mm + 31) >> 5;
      const int items = nb * (nb + 1);  // < 2^31 for every n this kernel can hold
      const int per = (items + totwarps - 1) / totwarps;
      // warps numbered across CTAs first, so that a short tile list still spreads over all SMs
      const int it0 = (warp * grp.size() + grp.rank()) * per;
      const int it1 = it0 + per < items ? it0 + per : items;
      double* tile = ytile + (size_t)warp * (TRI_TC * TRI_TLD);
      if (it0 < it1) {
        int bi = (int)((sqrtf(4.0f * (float)it0 + 1.0f) - 1.0f) * 0.5f);
        while (bi > 0 && bi * (bi + 1) > it0) --bi;
        while ((bi + 1) * (bi + 2) <= it0) ++bi;
        int off = bi * (bi + 1);
        int cur = -1;
        int i = 0;
        bool rowok = false;
        double ri = 0.0, si = 0.0, rowacc = 0.0;
        double rb1 = 0.0, rb2 = 0.0;  // kFixed: the row's tile sums, already split (exact)
        for (int it = it0; it < it1; ++it) {
          while (it >= off + 2 * bi + 2) {
            off += 2 * bi + 2;
            ++bi;
          }
          if (bi != cur) {
            if (kFixed) {
              if (cur >= 0 && wantp && rowok) {
                atomicAdd(pnext + i, rb1);
                atomicAdd(pnext2 + i, rb2);
              }
              rb1 = rb2 = 0.0;
            } else if (cur >= 0 && wantp && rowok) {
              tri_exact_add(pnext + i, pnext2 + i, rowacc, s_g1);
            }
            cur = bi;
            i = r0 + 32 * bi + lane;
            rowok = i < n;
            const double ui = (upd && rowok) ? vk[i] : 0.0;
            const double pi = (upd && rowok) ? wk[i] : 0.0;
            ri = a1 * ui;                  // row scalars of the rank-2 update
            si = fma(a1, pi, -a2x2 * ui);
            rowacc = 0.0;
          }
          const int c0 = r0 + TRI_TC * (it - off);
          double* col = a.A + i;
#pragma unroll 1
          for (int h = 0; h < TRI_TC; h += 8) {
            // loads first, in a batch, ahead of the dependent stores
            double x[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int c = c0 + h + u;
              x[u] = (rowok && c <= i) ? __ldcg(col + a.lda * c) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const int c = c0 + h + u;
              const bool ok = rowok && c <= i;
              double y = 0.0;
              if (ok) {
                y = upd ? x[u] - ri * wk[c] - si * vk[c] : x[u];
                __stcg(col + a.lda * c, y);
                rowacc += y * vk1[c];
              }
              tile[(h + u) * TRI_TLD + lane] = (ok && c < i) ? y : 0.0;
            }
          }
          __syncwarp();
          if (wantp) {
            // transposed part: lanes 0-15 sum rows 0-15 and lanes 16-31 rows 16-31 of column u
            const int u = lane & (TRI_TC - 1), hh = lane >> 4;
            const int rb = r0 + 32 * bi + 16 * hh;
            const double* tp = tile + u * TRI_TLD + 16 * hh;
            double cs = 0.0;
#pragma unroll
            for (int r = 0; r < 16; ++r) cs += tp[r] * (rb + r < n ? vk1[rb + r] : 0.0);
            cs += __shfl_xor_sync(0xffffffffu, cs, 16);
            const int c = c0 + u;
            if (hh == 0 && c < n && c <= r0 + 32 * bi + 31)
              tri_exact_add(pnext + c, pnext2 + c, cs, s_g1);
            if (kFixed) {
              // this tile's row sum into the row's exact register accumulators
              const int g1 = s_g1;
              const double q1 = tri_trunc(rowacc, g1);
              rb1 = __dadd_rn(rb1, q1);
              rb2 = __dadd_rn(rb2, tri_trunc(__dsub_rn(rowacc, q1), g1 - 41));
              rowacc = 0.0;
            }
          }
          __syncwarp();
        }
        if (kFixed) {
          if (wantp && rowok) {
            atomicAdd(pnext + i, rb1);
            atomicAdd(pnext2 + i, rb2);
          }
        } else if (wantp && rowok) {
          tri_exact_add(pnext + i, pnext2 + i, rowacc, s_g1);
        }
      }
    }
    if (!qk_grid_barrier(a.bar, grp.size(), epoch, a.status)) return;
    // rotate vectors: v_{k+1} becomes v_k
    double* t = vk;
    vk = vk1;
    vk1 = t;
    tau_k = tau1;
    scal_k = scal1;
  }
}

__global__ void __launch_bounds__(TRI_THREADS) k_sytrd(TriArgs a) {
  sytrd_body<TriGridWhole, false>(a, TriGridWhole{});
}

// ---------------------------------------------------------------------------------------------
// Double-float tridiagonalisation (the mixed tier).  GB300 issues one FP64 warp instruction per
// 64 cycles per SM sub-partition but one FP32 instruction per cycle, so the O(n^3) passes run in
// double-float arithmetic instead: a value is an unevaluated sum hi + lo of two floats (about 47
// significant bits), kept in the 8 bytes of the double it replaces.  Products use the exact FP32
// product error from an FMA (Dekker's two-product), sums use Knuth's two-sum; the lo x lo term
// and the rounding of the lo parts are dropped ("sloppy" double-float, relative error of each
// operation about 2^-46 of its operands), so the factorisation stays backward stable with unit
// roundoff about 2^-46 instead of 2^-53.  The scalar work of each column (reflector, dot
// products, grid exponents) and every quantity that leaves the kernel (d, e, tau, V) stay FP64;
// the mat-vec partial sums go into the same exact accumulators as in the FP64 kernel, so the
// results repeat bitwise too.  Explicit __f*_rn intrinsics keep nvcc from contracting the
// error-free transformations into FMAs.
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ float2 df_fma(float2 acc, float2 a, float2 b) {  // acc + a b
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float s = __fadd_rn(acc.x, p);
  const float bb = __fsub_rn(s, acc.x);
  float t = __fadd_rn(__fsub_rn(acc.x, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  t = __fadd_rn(t, __fadd_rn(acc.y, e));
  const float h = __fadd_rn(s, t);
  return make_float2(h, __fsub_rn(t, __fsub_rn(h, s)));
}

__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  float t = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  t = __fadd_rn(t, __fadd_rn(a.y, b.y));
  const float h = __fadd_rn(s, t);
  return make_float2(h, __fsub_rn(t, __fsub_rn(h, s)));
}

__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float h = __fadd_rn(p, e);
  return make_float2(h, __fsub_rn(e, __fsub_rn(h, p)));
}

__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }

// acc += a b for a dot product, compensated (Ogita, Rump and Oishi's Dot2): acc.x is the running
// float sum, acc.y collects the exact errors of its additions and the products' error terms,
// unnormalised -- the dependency chain per term is one addition on each part instead of a full
// double-float renormalisation, and the result is as accurate as double-float accumulation.
__device__ __forceinline__ void dot2_acc(float2& acc, float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = fmaf(a.x, b.x, -p);
  e = fmaf(a.x, b.y, e);
  e = fmaf(a.y, b.x, e);
  const float t = __fadd_rn(acc.x, p);
  const float bb = __fsub_rn(t, acc.x);
  const float err = __fadd_rn(__fsub_rn(acc.x, __fsub_rn(t, bb)), __fsub_rn(p, bb));
  acc.x = t;
  acc.y = __fadd_rn(acc.y, __fadd_rn(err, e));
}

// two Dot2 partial sums into one (same unnormalised form)
__device__ __forceinline__ float2 dot2_merge(float2 a, float2 b) {
  const float t = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(t, a.x);
  const float err = __fadd_rn(__fsub_rn(a.x, __fsub_rn(t, bb)), __fsub_rn(b.x, bb));
  return make_float2(t, __fadd_rn(__fadd_rn(a.y, b.y), err));
}

// x + n1 w + n2 v in one pass: the two exact products, two two-sums on the leading parts, all
// low-order terms added once, one renormalisation
__device__ __forceinline__ float2 df_upd2(float2 x, float2 n1, float2 w, float2 n2, float2 v) {
  const float p1 = __fmul_rn(n1.x, w.x);
  float e1 = fmaf(n1.x, w.x, -p1);
  e1 = fmaf(n1.x, w.y, e1);
  e1 = fmaf(n1.y, w.x, e1);
  const float p2 = __fmul_rn(n2.x, v.x);
  float e2 = fmaf(n2.x, v.x, -p2);
  e2 = fmaf(n2.x, v.y, e2);
  e2 = fmaf(n2.y, v.x, e2);
  const float s1 = __fadd_rn(x.x, p1);
  const float b1 = __fsub_rn(s1, x.x);
  const float t1 = __fadd_rn(__fsub_rn(x.x, __fsub_rn(s1, b1)), __fsub_rn(p1, b1));
  const float s2 = __fadd_rn(s1, p2);
  const float b2 = __fsub_rn(s2, s1);
  const float t2 = __fadd_rn(__fsub_rn(s1, __fsub_rn(s2, b2)), __fsub_rn(p2, b2));
  const float lo = __fadd_rn(__fadd_rn(__fadd_rn(x.y, e1), __fadd_rn(e2, t1)), t2);
  const float h = __fadd_rn(s2, lo);
  return make_float2(h, __fsub_rn(lo, __fsub_rn(h, s2)));
}
__device__ __forceinline__ float2 df_sub(float2 a, float2 b) { return df_add(a, df_neg(b)); }
// times a power of two (exact)
__device__ __forceinline__ float2 df_scale(float2 a, float s) {
  return make_float2(__fmul_rn(a.x, s), __fmul_rn(a.y, s));
}

// 1/b: the float reciprocal refined by one Newton step whose residual 1 - b r is formed exactly
// enough in double-float (1 - fl(b.x r) is exact near 1), relative error about 2^-46
__device__ __forceinline__ float2 df_rcp(float2 b) {
  const float r = __frcp_rn(b.x);
  const float p = __fmul_rn(b.x, r);
  const float pe = fmaf(b.x, r, -p);
  const float e = __fsub_rn(__fsub_rn(__fsub_rn(1.0f, p), pe), __fmul_rn(b.y, r));
  const float c = __fmul_rn(r, e);
  const float h = __fadd_rn(r, c);
  return make_float2(h, __fsub_rn(c, __fsub_rn(h, r)));
}

// sqrt(a), a >= 0: the float square root refined by one Newton step on the exact residual
// a - s^2 (Dekker's product), relative error about 2^-46
__device__ __forceinline__ float2 df_sqrt(float2 a) {
  if (!(a.x > 0.f)) return make_float2(a.x == 0.f ? 0.f : __fsqrt_rn(a.x), 0.f);
  const float s = __fsqrt_rn(a.x);
  const float p = __fmul_rn(s, s);
  const float pe = fmaf(s, s, -p);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.x, p), pe), a.y);
  const float c = __fdiv_rn(r, __fadd_rn(s, s));
  const float h = __fadd_rn(s, c);
  return make_float2(h, __fsub_rn(c, __fsub_rn(h, s)));
}

// Sum over the CTA in double-float, in a fixed order (butterflies within each warp, then warp 0
// over the warp sums; df_add is commutative to the bit, so every lane of a butterfly holds the
// same value); fin(total) runs on thread 0 before the closing barrier publishes its results.
template <class Fin>
__device__ __forceinline__ void df_block_sum(float2 v, float2* red, Fin fin) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    float2 w;
    w.x = __shfl_xor_sync(0xffffffffu, v.x, o);
    w.y = __shfl_xor_sync(0xffffffffu, v.y, o);
    v = df_add(v, w);
  }
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < (int)(blockDim.x >> 5) ? red[lane] : make_float2(0.f, 0.f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      float2 w;
      w.x = __shfl_xor_sync(0xffffffffu, v.x, o);
      w.y = __shfl_xor_sync(0xffffffffu, v.y, o);
      v = df_add(v, w);
    }
    if (lane == 0) fin(v);
  }
  __syncthreads();
}

// FP64 -> double-float by bit operations on the integer pipe (no FP64 issue): hi = x truncated
// to 24 significant bits, lo = the next 23 bits of x.  |x| < 2^-126 gives 0 (and lo = 0 below
// 2^-80); infinities and NaN come through in hi.  Callers keep magnitudes inside float's range
// (the kernel checks ||A||_F first).
__device__ __forceinline__ float2 df_from_double(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hw = (unsigned)(b >> 32);
  const unsigned sgn = hw & 0x80000000u;
  const int e = (int)((hw >> 20) & 0x7FFu);
  const unsigned m = (unsigned)(b >> 29) & 0x7FFFFFu;
  if (e == 0x7FF) return make_float2(__uint_as_float(sgn | 0x7F800000u | (m ? 0x400000u : 0u)), 0.f);
  const int fe = e - 896;  // float's biased exponent
  if (fe <= 0) return make_float2(0.f, 0.f);
  if (fe >= 255) return make_float2(__uint_as_float(sgn | 0x7F800000u), 0.f);
  const float h = __uint_as_float(sgn | ((unsigned)fe << 23) | m);
  float l = 0.f;
  if (e >= 943) {
    // the 23 bits below hi's last one: r * 2^(e - 1069), r < 2^23 converted exactly through
    // the 2^23 exponent pattern
    const unsigned r = ((unsigned)b & 0x1FFFFFFFu) >> 6;
    const float rf = __fsub_rn(__uint_as_float(0x4B000000u | r), 8388608.0f);
    l = __fmul_rn(rf, __uint_as_float((unsigned)(e - 942) << 23));
    l = __uint_as_float(__float_as_uint(l) | sgn);
  }
  return make_float2(h, l);
}

// float -> double by bit operations (exact; zeros and subnormals give 0, which only drops
// magnitudes below 2^-126)
__device__ __forceinline__ double df_f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xFFu;
  if (e == 0xFFu) return (double)f;
  const unsigned long long d =
      e == 0u ? ((unsigned long long)(u & 0x80000000u) << 32)
              : ((unsigned long long)(u & 0x80000000u) << 32) |
                    ((unsigned long long)(e + 896u) << 52) |
                    ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}

// hi + lo as a double: exact (|lo| < ulp(hi), 48 bits in all), one FP64 addition
__device__ __forceinline__ double df_to_double(float2 a) { return __dadd_rn(df_f2d(a.x), df_f2d(a.y)); }

// The same factorisation as sytrd_body (the same fused rank-2 update and symmetric mat-vec over
// the same tiles, the same reflector formulas and exact accumulators), with the matrix and the
// vectors u_k, p~_k, u_{k+1} in double-float.  The lower triangle of A is converted in place
// (float2 in each double's slot) after the Frobenius norm has been found, scaled by the power of
// two 2^-ex that brings ||A||_F into [1/2, 1): every double-float intermediate (entries, mat-vec
// products up to ||A||^2, dot products up to n ||A||^3) then stays far inside float's range, and
// the scaling is exact.  The per-column scalars (dot products, reflector, update coefficients)
// are double-float as well, so that no FP64 latency sits on the per-column critical path: the
// outputs d, e, tau, the reflector scale factors and the unscaled reflectors are stored as
// double-floats in the slots of their doubles, and k_tri_df_finish converts them afterwards (d and
// e scaled back by 2^ex; the reflectors do not depend on the scaling).
template <class Grp, bool kFixed>
__device__ __forceinline__ void sytrd_df_body(const TriArgs a, const Grp grp) {
  extern __shared__ double sm[];
  __shared__ double s_fro;
  __shared__ float2 s_df[4];  // a1, a2x2, cu, cp of the current step
  __shared__ float2 s_pj, s_dj, s_alpha, s_beta, s_t1, s_scal;
  __shared__ float2 s_red[32];
  __shared__ int s_g1;
  const int n = a.n;
  float2* ytile = reinterpret_cast<float2*>(sm);  // one TRI_TC x TRI_TLD tile per warp
  float2 *vk, *wk, *vk1;
  if (a.use_smem) {
    vk = reinterpret_cast<float2*>(sm) + (blockDim.x >> 5) * (TRI_TC * TRI_TLD);
    wk = vk + n;
    vk1 = vk + 2 * n;
  } else {
    float2* base = reinterpret_cast<float2*>(a.gvec + (size_t)grp.rank() * 3 * n);
    vk = base;
    wk = base + n;
    vk1 = base + 2 * n;
  }
  float2* A2 = reinterpret_cast<float2*>(a.A);
  unsigned epoch = 0;
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
  const int totwarps = grp.size() * nwarps;
  const int gthread = grp.rank() * nt + tid, totthreads = grp.size() * nt;
  const float2 zero2 = make_float2(0.f, 0.f), one2 = make_float2(1.f, 0.f);
  float2* V2 = reinterpret_cast<float2*>(a.V);
  float2 tau_k = zero2, scal_k = one2;

  // ---- ||A||_F exactly as the FP64 body computes it (fixed orders) ----
  const int nch = kFixed ? (n + 31) / 32 : 0;
  if (!kFixed) {
    double fs = 0.0;
    for (int c = grp.rank(); c < n; c += grp.size()) {
      const double* col = a.A + a.lda * c;
      for (int i = c + tid; i < n; i += nt) {
        const double x = __ldcg(col + i);
        fs = fma(i == c ? x : x + x, x, fs);
      }
    }
    tri_block_sum(fs, sm, nt, [&](double t) { __stcg(a.fslot + grp.rank(), t); });
  } else {
    for (int ch = grp.rank(); ch < nch; ch += grp.size()) {
      double fs = 0.0;
      const int c1 = 32 * ch + 32 < n ? 32 * ch + 32 : n;
      for (int c = 32 * ch; c < c1; ++c) {
        const double* col = a.A + a.lda * c;
        for (int i = c + tid; i < n; i += nt) {
          const double x = __ldcg(col + i);
          fs = fma(i == c ? x : x + x, x, fs);
        }
      }
      tri_block_sum(fs, sm, nt, [&](double t) { __stcg(a.fslot + ch, t); });
    }
  }
  if (!qk_grid_barrier(a.bar, grp.size(), epoch, a.status)) return;
  if (tid == 0) {
    double t = 0.0;
    const int ns = kFixed ? nch : grp.size();
    for (int b = 0; b < ns; ++b) t += __ldcg(a.fslot + b);
    s_fro = sqrt(t);
  }
  __syncthreads();
  // power-of-two scaling (1 for a zero, infinite or NaN norm: those propagate as in FP64)
  int ex = 0;
  if (s_fro > 0.0 && s_fro <= DBL_MAX) frexp(s_fro, &ex);
  const double sc = ldexp(1.0, -ex);
  const float fro = (float)(s_fro * sc);  // only bounds the accumulator grids
  if (grp.rank() == 0 && tid == 0) *a.dfscale = ldexp(1.0, ex);
  // ---- the lower triangle to double-float, in place (each CTA its own columns) ----
  for (int c = grp.rank(); c < n; c += grp.size()) {
    double* col = a.A + a.lda * c;
    for (int i = c + tid; i < n; i += nt)
      __stcg(A2 + a.lda * c + i, df_from_double(__ldcg(col + i) * sc));
  }
  if (!qk_grid_barrier(a.bar, grp.size(), epoch, a.status)) return;

  for (int k = -1; k <= n - 2; ++k) {
    {
      double* pz = a.pbuf + (size_t)((k + 2) % 3) * n;
      double* pz2 = pz + 3 * (size_t)n;
      for (int i = gthread; i < n; i += totthreads) {
        __stcg(pz + i, 0.0);
        __stcg(pz2 + i, 0.0);
      }
    }
    // ---- small phase (redundant in every CTA), as in sytrd_body, on the FP32 pipe ----
    const int j = k + 1;
    float2 tau1, scal1;
    {
      const double* p = a.pbuf + (size_t)((k + 3) % 3) * n;
      float2 dot = zero2;
      // four elements per thread per round, loads issued together
      for (int i0 = j + tid; i0 < n; i0 += 4 * nt) {
        float2 xv[4], uv[4];
        double pv[4], pv2[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int i = i0 + r * nt;
          xv[r] = i < n ? __ldcg(A2 + i + a.lda * j) : zero2;
          pv[r] = (k >= 0 && i < n) ? __ldcg(p + i) : 0.0;
          pv2[r] = (k >= 0 && i < n) ? __ldcg(p + 3 * (size_t)n + i) : 0.0;
          uv[r] = (k >= 0 && i < n) ? vk[i] : zero2;
        }
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int i = i0 + r * nt;
          if (i < n) {
            vk1[i] = xv[r];
            if (k >= 0) {
              // the two exact accumulators, each split on the integer pipe, added in double-float
              const float2 pf = df_add(df_from_double(pv[r]), df_from_double(pv2[r]));
              wk[i] = pf;
              if (i == j) s_pj = pf;
              dot = df_fma(dot, pf, uv[r]);
            }
          }
        }
      }
      if (k >= 0) {
        df_block_sum(dot, s_red, [&](float2 t) {
          // true dot p.v = scal^2 p~.u;  c = tau^2 dot / 2;  w = scal^2 (tau p~ - c u)
          const float2 s2 = df_mul(scal_k, scal_k);
          const float2 cc = df_scale(df_mul(df_mul(tau_k, tau_k), df_mul(s2, t)), 0.5f);
          const float2 b1 = df_mul(tau_k, s2), b2 = df_mul(cc, s2);
          const float2 u = vk[j];
          const float2 wj = df_sub(df_mul(b1, s_pj), df_mul(b2, u));
          s_df[0] = b1;
          s_df[1] = df_scale(b2, 2.0f);
          s_df[2] = df_sub(df_mul(b2, u), wj);  // coefficient of u_i in column j
          s_df[3] = df_neg(df_mul(b1, u));      // coefficient of p~_i in column j
        });
      } else {
        if (tid < 4) s_df[tid] = zero2;
        __syncthreads();
      }
      const float2 cu = s_df[2], cp = s_df[3];
      float2 ss = zero2;
      for (int i = j + tid; i < n; i += nt) {
        float2 x = vk1[i];
        if (k >= 0) {
          x = df_fma(df_fma(x, cu, vk[i]), cp, wk[i]);
          vk1[i] = x;
        }
        if (i == j) s_dj = x;
        else if (i == j + 1) s_alpha = x;
        else ss = df_fma(ss, x, x);
      }
      // Householder reflector of the updated column (dlarfg) in double-float, by thread 0
      df_block_sum(ss, s_red, [&](float2 sigma) {
        float2 beta = zero2, t1 = zero2, scal = one2, inv = one2;
        float unrm = 1.0f;
        if (j <= n - 2) {
          const float2 alpha = s_alpha;
          if (sigma.x == 0.f) {
            beta = alpha;
          } else {
            const float2 r = df_sqrt(df_fma(sigma, alpha, alpha));
            beta = (__float_as_uint(alpha.x) >> 31) ? r : df_neg(r);  // -copysign(r, alpha)
            t1 = df_mul(df_sub(beta, alpha), df_rcp(beta));
            inv = df_sub(alpha, beta);
            scal = df_rcp(inv);
            // ||u||_2 from the leading parts, rounded up well past float's rounding
            unrm = __fmul_ru(__fsqrt_ru(fmaf(inv.x, inv.x, sigma.x)), 1.0001f);
          }
          vk1[j + 1] = inv;  // u_{j+1} = 1/scal, so that scal * u_{j+1} = 1
        }
        s_beta = beta;
        s_t1 = t1;
        s_scal = scal;
        // grids of the exact accumulators for p~ = A' u (bound 2 ||A||_F ||u||_2, as in FP64)
        int e2x = 0;
        const float bnd = __fmul_ru(__fmul_ru(2.0f, fro), unrm);
        if (bnd > 0.f && bnd <= FLT_MAX) frexpf(bnd, &e2x);
        s_g1 = e2x - 51;
      });
      tau1 = s_t1;
      scal1 = s_scal;
      // outputs as double-floats (k_tri_df_finish converts them); the reflector unscaled, its
      // scale factor beside tau
      if (grp.rank() == 0 && tid == 0) {
        reinterpret_cast<float2*>(a.d)[j] = s_dj;
        if (j <= n - 2) {
          reinterpret_cast<float2*>(a.e)[j] = s_beta;
          reinterpret_cast<float2*>(a.tau)[j] = tau1;
          reinterpret_cast<float2*>(a.vscal)[j] = scal1;
        }
      }
      if (j <= n - 2)
        for (int i = j + 2 + gthread; i < n; i += totthreads) V2[i + a.ldv * j] = vk1[i];
    }
    // ---- big pass: the FP64 body's tiles and order, double-float arithmetic ----
    const int r0 = k + 2;
    const int mm = n - r0;
    if (mm > 0) {
      double* pnext = a.pbuf + (size_t)((k + 1) % 3) * n;
      double* pnext2 = pnext + 3 * (size_t)n;
      const bool upd = (k >= 0);
      const bool wantp = (j <= n - 2);
      const float2 a1 = s_df[0], a2x2 = s_df[1];
      const int nb = (mm + 31) >> 5;
      const int items = nb * (nb + 1);
      const int per = (items + totwarps - 1) / totwarps;
      const int it0 = (warp * grp.size() + grp.rank()) * per;
      const int it1 = it0 + per < items ? it0 + per : items;
      float2* tile = ytile + (size_t)warp * (TRI_TC * TRI_TLD);
      if (it0 < it1) {
        int bi = (int)((sqrtf(4.0f * (float)it0 + 1.0f) - 1.0f) * 0.5f);
        while (bi > 0 && bi * (bi + 1) > it0) --bi;
        while ((bi + 1) * (bi + 2) <= it0) ++bi;
        int off = bi * (bi + 1);
        int cur = -1;
        int i = 0;
        bool rowok = false;
        // -(a1 u_i), -(a1 p~_i - a2x2 u_i); the row's mat-vec sum as a Dot2 pair
        float2 nri = zero2, nsi = zero2, rowacc = zero2;
        double rb1 = 0.0, rb2 = 0.0;
        // interior tiles prefetch the next interior tile's 16 elements into x while they finish
        // their column sums, so that its L2 latency overlaps them
        float2 x[TRI_TC];
        bool have_next = false;
        for (int it = it0; it < it1; ++it) {
          while (it >= off + 2 * bi + 2) {
            off += 2 * bi + 2;
            ++bi;
          }
          if (bi != cur) {
            if (kFixed) {
              if (cur >= 0 && wantp && rowok) {
                atomicAdd(pnext + i, rb1);
                atomicAdd(pnext2 + i, rb2);
              }
              rb1 = rb2 = 0.0;
            } else if (cur >= 0 && wantp && rowok) {
              tri_exact_add(pnext + i, pnext2 + i, df_to_double(rowacc), s_g1);
            }
            cur = bi;
            i = r0 + 32 * bi + lane;
            rowok = i < n;
            const float2 ui = (upd && rowok) ? vk[i] : zero2;
            const float2 pi = (upd && rowok) ? wk[i] : zero2;
            nri = df_neg(df_mul(a1, ui));
            nsi = df_neg(df_fma(df_mul(a1, pi), df_neg(a2x2), ui));
            rowacc = zero2;
          }
          const int c0 = r0 + TRI_TC * (it - off);
          float2* col = A2 + i;
          if (upd && wantp && it - off < 2 * bi && r0 + 32 * bi + 32 <= n) {
            // interior tile (the common case): every element strictly below the diagonal and
            // inside the matrix, so no per-element predicates or index tests; all 16 loads are
            // issued before the first use
            const float2* wc = wk + c0;
            const float2* vc = vk + c0;
            const float2* v1c = vk1 + c0;
            float2* q = col + a.lda * c0;
            if (!have_next) {
              const float2* qq = q;
#pragma unroll
              for (int u = 0; u < TRI_TC; ++u) {
                x[u] = __ldcg(qq);
                qq += a.lda;
              }
            }
#pragma unroll
            for (int u = 0; u < TRI_TC; ++u) {
              const float2 y = df_upd2(x[u], nri, wc[u], nsi, vc[u]);
              __stcg(q, y);
              q += a.lda;
              dot2_acc(rowacc, y, v1c[u]);
              tile[u * TRI_TLD + lane] = y;
            }
            // the next item: the same row block or the next one (rows blocks grow by 2 tiles)
            have_next = false;
            if (it + 1 < it1) {
              int bn = bi, on = off;
              if (it + 1 >= off + 2 * bi + 2) {
                on = off + 2 * bi + 2;
                ++bn;
              }
              if (it + 1 - on < 2 * bn && r0 + 32 * bn + 32 <= n) {
                const float2* qq = A2 + (r0 + 32 * bn + lane) + a.lda * (r0 + TRI_TC * (it + 1 - on));
#pragma unroll
                for (int u = 0; u < TRI_TC; ++u) {
                  x[u] = __ldcg(qq);
                  qq += a.lda;
                }
                have_next = true;
              }
            }
            __syncwarp();
            const int u = lane & (TRI_TC - 1), hh = lane >> 4;
            const float2* tp = tile + u * TRI_TLD + 16 * hh;
            const float2* vr = vk1 + r0 + 32 * bi + 16 * hh;
            float2 cs = zero2;
#pragma unroll
            for (int r = 0; r < 16; ++r) dot2_acc(cs, tp[r], vr[r]);
            float2 o;
            o.x = __shfl_xor_sync(0xffffffffu, cs.x, 16);
            o.y = __shfl_xor_sync(0xffffffffu, cs.y, 16);
            cs = dot2_merge(cs, o);
            if (hh == 0) tri_exact_add(pnext + c0 + u, pnext2 + c0 + u, df_to_double(cs), s_g1);
            if (kFixed) {
              const int g1 = s_g1;
              const double ra = df_to_double(rowacc);
              const double q1 = tri_trunc(ra, g1);
              rb1 = __dadd_rn(rb1, q1);
              rb2 = __dadd_rn(rb2, tri_trunc(__dsub_rn(ra, q1), g1 - 41));
              rowacc = zero2;
            }
            __syncwarp();
            continue;
          }
          // edge tile (the diagonal ones, the last, partial row block, the first and the last
          // column): the same loads-first schedule and arithmetic with per-element masks, without
          // branches: masked elements load A(0,0) and read clamped vector entries (both in
          // bounds), and their results are discarded by selects and a predicated store
          {
            const float2* qq = col + a.lda * c0;
#pragma unroll
            for (int u = 0; u < TRI_TC; ++u) {
              x[u] = __ldcg((rowok && c0 + u <= i) ? qq : A2);
              qq += a.lda;
            }
            float2* q = col + a.lda * c0;
#pragma unroll
            for (int u = 0; u < TRI_TC; ++u) {
              const int c = c0 + u;
              const int cc = c < n ? c : n - 1;
              const bool ok = rowok && c <= i;
              float2 y = upd ? df_upd2(x[u], nri, wk[cc], nsi, vk[cc]) : x[u];
              y = ok ? y : zero2;
              if (ok) __stcg(q, y);
              dot2_acc(rowacc, y, vk1[cc]);
              q += a.lda;
              tile[u * TRI_TLD + lane] = c < i ? y : zero2;
            }
          }
          __syncwarp();
          if (wantp) {
            const int u = lane & (TRI_TC - 1), hh = lane >> 4;
            const int rb = r0 + 32 * bi + 16 * hh;
            const float2* tp = tile + u * TRI_TLD + 16 * hh;
            float2 cs = zero2;
#pragma unroll
            for (int r = 0; r < 16; ++r) dot2_acc(cs, tp[r], vk1[rb + r < n ? rb + r : n - 1]);
            float2 o;
            o.x = __shfl_xor_sync(0xffffffffu, cs.x, 16);
            o.y = __shfl_xor_sync(0xffffffffu, cs.y, 16);
            cs = dot2_merge(cs, o);
            const int c = c0 + u;
            if (hh == 0 && c < n && c <= r0 + 32 * bi + 31)
              tri_exact_add(pnext + c, pnext2 + c, df_to_double(cs), s_g1);
            if (kFixed) {
              const int g1 = s_g1;
              const double ra = df_to_double(rowacc);
              const double q1 = tri_trunc(ra, g1);
              rb1 = __dadd_rn(rb1, q1);
              rb2 = __dadd_rn(rb2, tri_trunc(__dsub_rn(ra, q1), g1 - 41));
              rowacc = zero2;
            }
          }
          __syncwarp();
        }
        if (kFixed) {
          if (wantp && rowok) {
            atomicAdd(pnext + i, rb1);
            atomicAdd(pnext2 + i, rb2);
          }
        } else if (wantp && rowok) {
          tri_exact_add(pnext + i, pnext2 + i, df_to_double(rowacc), s_g1);
        }
      }
    }
    if (!qk_grid_barrier(a.bar, grp.size(), epoch, a.status)) return;
    float2* t = vk;
    vk = vk1;
    vk1 = t;
    tau_k = tau1;
    scal_k = scal1;
  }
}

// 512 threads per CTA (DF_THREADS): the double-float arithmetic needs up to 128 registers a thread
__global__ void __launch_bounds__(512) k_sytrd_df(TriArgs a) {
  sytrd_df_body<TriGridWhole, false>(a, TriGridWhole{});
}

// FP64 outputs of the double-float tridiagonalisation, in place: block j converts column j of V
// (V(j+1, j) = 1, V(i, j) = u_i * scal_j below) and d_j, e_j, tau_j (d and e scaled back).
__global__ void k_tri_df_finish(int n, double* __restrict__ d, double* __restrict__ e,
                                double* __restrict__ tau, double* __restrict__ V, long long ldv,
                                const double* __restrict__ vscal,
                                const double* __restrict__ dfscale) {
  const int j = blockIdx.x;
  const double unsc = *dfscale;
  if (threadIdx.x == 0) {
    d[j] = df_to_double(reinterpret_cast<const float2*>(d)[j]) * unsc;
    if (j <= n - 2) {
      e[j] = df_to_double(reinterpret_cast<const float2*>(e)[j]) * unsc;
      tau[j] = df_to_double(reinterpret_cast<const float2*>(tau)[j]);
    }
  }
  if (j > n - 2) return;
  const double sj = df_to_double(reinterpret_cast<const float2*>(vscal)[j]);
  double* col = V + ldv * j;
  for (int i = j + 1 + threadIdx.x; i < n; i += blockDim.x)
    col[i] = i == j + 1 ? 1.0 : df_to_double(reinterpret_cast<const float2*>(col)[i]) * sj;
}

// Many tridiagonalisations in one cooperative launch: request r owns the CTAs
// [cta0[r], cta0[r+1]) and synchronises them with its own bounded group barrier (its own counter),
// so the per-column latency of small systems overlaps instead of queueing for the whole GPU.
constexpr int TRI_GROUP_MAX = 32;
struct TriGroup {
  int nreq;
  int cta0[TRI_GROUP_MAX + 1];
  TriArgs req[TRI_GROUP_MAX];
};

__global__ void __launch_bounds__(TRI_THREADS) k_sytrd_grouped(const __grid_constant__ TriGroup g) {
  __shared__ int s_grp[2];
  int r = 0;
  while (r + 1 < g.nreq && (int)blockIdx.x >= g.cta0[r + 1]) ++r;
  if ((int)blockIdx.x >= g.cta0[g.nreq]) return;
  if (threadIdx.x == 0) {
    s_grp[0] = g.cta0[r + 1] - g.cta0[r];
    s_grp[1] = (int)blockIdx.x - g.cta0[r];
  }
  __syncthreads();
  sytrd_body<TriGridSlice, true>(g.req[r], TriGridSlice{s_grp});
}

// the same for double-float requests (the mixed tier), DF_THREADS per CTA
constexpr int DF_THREADS = 512;
__global__ void __launch_bounds__(DF_THREADS)
    k_sytrd_df_grouped(const __grid_constant__ TriGroup g) {
  __shared__ int s_grp[2];
  int r = 0;
  while (r + 1 < g.nreq && (int)blockIdx.x >= g.cta0[r + 1]) ++r;
  if ((int)blockIdx.x >= g.cta0[g.nreq]) return;
  if (threadIdx.x == 0) {
    s_grp[0] = g.cta0[r + 1] - g.cta0[r];
    s_grp[1] = (int)blockIdx.x - g.cta0[r];
  }
  __syncthreads();
  sytrd_df_body<TriGridSlice, true>(g.req[r], TriGridSlice{s_grp});
}

// Gershgorin bounds, pivmin, ||T||_1 and e^2 (single block).  T is first scaled in place by the
// power of two that brings max(|d_i|, |e_i|) into [1/2, 1), so that the Sturm recurrence's
// rescaling (every 4 steps, 2^+-400) never meets overflow or underflow whatever the matrix's
// magnitude; out[4] = the inverse factor, which k_tri_unscale applies to the eigenvalues.
__global__ void k_tri_prep(int n, double* __restrict__ d, double* __restrict__ e,
                           double* __restrict__ e2,
                           double* __restrict__ out /* gl, gu, pivmin, tnrm, unscale */) {
  __shared__ double red[32];
  __shared__ double s_sc;
  {
    double m = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
      m = fmax(m, fmax(fabs(d[i]), i < n - 1 ? fabs(e[i]) : 0.0));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, red[w]);
      int ex = 0;
      if (m > 0.0 && m <= DBL_MAX) frexp(m, &ex);
      s_sc = ldexp(1.0, -ex);
      out[4] = ldexp(1.0, ex);
    }
    __syncthreads();
    const double sc = s_sc;
    if (sc != 1.0)
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        d[i] *= sc;
        if (i < n - 1) e[i] *= sc;
      }
    __syncthreads();
  }
  double gl = INFINITY, gu = -INFINITY, emax = 0.0, tn = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double el = i > 0 ? fabs(e[i - 1]) : 0.0;
    const double er = i < n - 1 ? fabs(e[i]) : 0.0;
    gl = fmin(gl, d[i] - el - er);
    gu = fmax(gu, d[i] + el + er);
    tn = fmax(tn, fabs(d[i]) + el + er);
    if (i < n - 1) {
      e2[i] = e[i] * e[i];
      emax = fmax(emax, e[i] * e[i]);
    }
  }
  // max/min reductions via shuffles
  for (int o = 16; o > 0; o >>= 1) {
    gl = fmin(gl, __shfl_xor_sync(0xffffffffu, gl, o));
    gu = fmax(gu, __shfl_xor_sync(0xffffffffu, gu, o));
    emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
  }
  __shared__ double s4[4][32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) { s4[0][wid] = gl; s4[1][wid] = gu; s4[2][wid] = emax; s4[3][wid] = tn; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < nw; ++w) {
      gl = fmin(gl, s4[0][w]);
      gu = fmax(gu, s4[1][w]);
      emax = fmax(emax, s4[2][w]);
      tn = fmax(tn, s4[3][w]);
    }
    const double safmin = DBL_MIN;
    const double pivmin = safmin * fmax(1.0, emax);
    const double tnorm = fmax(fabs(gl), fabs(gu));
    const double fudge = 2.0 * DBL_EPSILON * tnorm * n + 4.0 * pivmin;
    out[0] = gl - fudge - 2.0 * DBL_EPSILON * fabs(gl);
    out[1] = gu + fudge + 2.0 * DBL_EPSILON * fabs(gu);
    out[2] = pivmin;
    out[3] = tn > 0.0 ? tn : 1.0;
  }
}

// eigenvalues of the scaled T back to the matrix's scale (exact: a power of two)
__global__ void k_tri_unscale(int n, const double* __restrict__ prep, double* __restrict__ w) {
  const double f = prep[4];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    w[i] *= f;
}

// Number of eigenvalues of T below x: sign changes of the leading principal minors
// p_0 = 1, p_1 = d_0 - x, p_{i+1} = (d_i - x) p_i - e_{i-1}^2 p_{i-1} (Sturm sequence of the
// characteristic polynomials).  Division-free, and the sign and zero tests read the bits, so a
// step costs 3 FP64 operations.  A zero minor takes the sign opposite to its predecessor (the
// convention that a zero pivot counts as negative), and every 4 steps the pair (p_i, p_{i-1}) is
// rescaled by an exact power of two when it drifts towards overflow or underflow (signs and
// ratios are unchanged by the scaling).
__device__ __forceinline__ int sign_bit(double v, int prev_neg) {
  const int hi = __double2hiint(v), lo = __double2loint(v);
  return (((hi & 0x7fffffff) | lo) == 0) ? !prev_neg : (hi < 0);
}

__device__ __forceinline__ int sturm_count(int n, const double* __restrict__ d,
                                           const double* __restrict__ e2, double x) {
  double p0 = 1.0, p1 = __ldg(d) - x;
  int neg = sign_bit(p1, 0);
  int c = neg;
  for (int i = 1; i < n; ++i) {
    const double p2 = fma(__ldg(d + i) - x, p1, -(__ldg(e2 + i - 1) * p0));
    const int n2 = sign_bit(p2, neg);
    c += (n2 != neg);
    neg = n2;
    p0 = p1;
    p1 = p2;
    if ((i & 3) == 0) {
      const int ex1 = (__double2hiint(p1) >> 20) & 0x7ff;
      const int ex0 = (__double2hiint(p0) >> 20) & 0x7ff;
      const int ex = ex1 > ex0 ? ex1 : ex0;
      if (ex > 1023 + 400) {
        p0 *= 0x1p-400;
        p1 *= 0x1p-400;
      } else if (ex < 1023 - 400) {
        p0 *= 0x1p+400;
        p1 *= 0x1p+400;
      }
    }
  }
  return c;
}

// The same Sturm count in double-float on the FP32 pipe (the mixed tier), with d and e^2 as
// double-float pairs.  A step is d_i - x (a two-sum) and the fused two-product difference
// (d_i - x) p_i - e^2 p_{i-1} with one renormalisation; float's exponent range is narrow, so the
// pair is brought back towards 1 by an exact power of two whenever its larger member leaves
// [2^-30, 2^30] (checked every step: one step changes magnitudes by at most a few units for the
// scaled T, or by the size of a tiny e^2 or d_i - x).
__device__ __forceinline__ float2 df_dif2(float2 a, float2 b, float2 c, float2 d) {  // ab - cd
  const float p1 = __fmul_rn(a.x, b.x);
  float e1 = fmaf(a.x, b.x, -p1);
  e1 = fmaf(a.x, b.y, e1);
  e1 = fmaf(a.y, b.x, e1);
  const float p2 = __fmul_rn(c.x, d.x);
  float e2 = fmaf(c.x, d.x, -p2);
  e2 = fmaf(c.x, d.y, e2);
  e2 = fmaf(c.y, d.x, e2);
  const float s = __fsub_rn(p1, p2);
  const float bb = __fsub_rn(s, p1);
  const float t = __fsub_rn(__fsub_rn(p1, __fsub_rn(s, bb)), __fadd_rn(p2, bb));
  const float lo = __fadd_rn(t, __fsub_rn(e1, e2));
  const float h = __fadd_rn(s, lo);
  return make_float2(h, __fsub_rn(lo, __fsub_rn(h, s)));
}

__device__ __forceinline__ int sturm_count_df(int n, const float2* __restrict__ d,
                                              const float2* __restrict__ e2, float2 x) {
  float2 p0 = make_float2(1.f, 0.f), p1 = df_sub(__ldg(d), x);
  int neg = p1.x == 0.f ? 1 : (int)(__float_as_uint(p1.x) >> 31);
  int c = neg;
  for (int i = 1; i < n; ++i) {
    const float2 p2 = df_dif2(df_sub(__ldg(d + i), x), p1, __ldg(e2 + i - 1), p0);
    const int n2 = p2.x == 0.f ? !neg : (int)(__float_as_uint(p2.x) >> 31);
    c += (n2 != neg);
    neg = n2;
    p0 = p1;
    p1 = p2;
    const int e1x = (int)((__float_as_uint(p1.x) >> 23) & 0xFF);
    const int e0x = (int)((__float_as_uint(p0.x) >> 23) & 0xFF);
    const int ex = e1x > e0x ? e1x : e0x;
    if (ex > 127 + 30) {
      p0 = df_scale(p0, 0x1p-60f);
      p1 = df_scale(p1, 0x1p-60f);
    } else if (ex < 127 - 30) {
      p0 = df_scale(p0, 0x1p+60f);
      p1 = df_scale(p1, 0x1p+60f);
    }
  }
  return c;
}

// d and e^2 of the scaled T as double-float pairs, for the double-float bisection
__global__ void k_tri_df_copy(int n, const double* __restrict__ d, const double* __restrict__ e2,
                              float2* __restrict__ dd, float2* __restrict__ ee) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    dd[i] = df_from_double(d[i]);
    ee[i] = i < n - 1 ? df_from_double(e2[i]) : make_float2(0.f, 0.f);
  }
}

// k-section on the Sturm count: K consecutive lanes share eigenvalue j and test K interior points
// of the bracket per step (log2(K+1) bits per step), to full FP64 precision.  Sturm counts are
// monotone in x in IEEE arithmetic, so the points with count <= j form a prefix and the new
// bracket follows from a popcount of the group's ballot.  K trades extra sweeps for parallelism:
// the FP64 pipe of an SM sub-partition issues one warp instruction per 64 cycles, so the launch
// picks the largest K whose warps still fit one per sub-partition.
// Sturm counts at G+1 equally spaced points of the Gershgorin interval (one thread per point):
// every eigenvalue then starts its k-section from the grid cell that holds it, log2(G) halvings
// below the full interval.
// DF: the counts in double-float (dd, ee), the bracket closed to double-float's precision
// (2^-45 relative, or 2^-47 ||T||_1 near zero) instead of FP64's.
constexpr int STEBZ_GRID = 16384;
template <bool DF>
__global__ void k_stebz_grid(int n, const double* __restrict__ d, const double* __restrict__ e2,
                             const float2* __restrict__ dd, const float2* __restrict__ ee,
                             const double* __restrict__ prep, int G, int* __restrict__ cnt) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g > G) return;
  const double lo = prep[0], hi = prep[1];
  const double h = (hi - lo) / G;
  const double x = lo + h * g;
  cnt[g] = g == 0 ? 0
                  : (g == G ? n
                            : (DF ? sturm_count_df(n, dd, ee, df_from_double(x))
                                  : sturm_count(n, d, e2, x)));
}

template <int K, bool DF>
__global__ void __launch_bounds__(128) k_stebz(int n, const double* __restrict__ d,
                                               const double* __restrict__ e2,
                                               const float2* __restrict__ dd,
                                               const float2* __restrict__ ee,
                                               const double* __restrict__ prep,
                                               const int* __restrict__ cnt, int G,
                                               double* __restrict__ w) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = gt / K, t = gt % K;
  const bool valid = j < n;
  const int lane = threadIdx.x & 31;
  const unsigned gmask = (K == 32 ? 0xffffffffu : ((1u << K) - 1u)) << (lane & ~(K - 1));
  double lo = prep[0], hi = prep[1];
  const double pivmin = prep[2];
  if (cnt && valid) {
    // the cell [x_g, x_{g+1}) with cnt[g] <= j < cnt[g+1] (cnt[0] = 0, cnt[G] = n)
    int a = 0, b = G;
    while (b - a > 1) {
      const int mid = (a + b) >> 1;
      if (cnt[mid] <= j) a = mid;
      else b = mid;
    }
    const double h = (hi - lo) / G;
    const double x0 = lo + h * a;
    const double x1 = b == G ? hi : lo + h * b;
    lo = x0;
    hi = x1;
  }
  const double rtol = DF ? 0x1p-45 : 2.0 * DBL_EPSILON;
  const double atol = DF ? 0x1p-47 * prep[3] : 2.0 * pivmin;
  for (int it = 0; it < 128; ++it) {
    if (hi - lo <= rtol * fmax(fabs(lo), fabs(hi)) + atol) break;
    const double h = (hi - lo) / (K + 1);
    const double x = lo + h * (t + 1);
    const int c = !valid ? 0
                         : (DF ? sturm_count_df(n, dd, ee, df_from_double(x))
                               : sturm_count(n, d, e2, x));
    const unsigned le = __ballot_sync(gmask, c <= j) & gmask;
    const int k = __popc(le);
    const double nlo = k > 0 ? lo + h * k : lo;
    const double nhi = k < K ? lo + h * (k + 1) : hi;
    if (!(nlo < nhi) || (nlo == lo && nhi == hi)) break;
    lo = nlo;
    hi = nhi;
  }
  if (valid && t == 0) w[j] = 0.5 * (lo + hi);
}

void launch_stebz(qk_ctx* ctx, int n, const double* d, const double* e2, const float2* dd,
                  const float2* ee, const double* prep, const int* cnt, int G, double* w) {
  const int blocks8 = (int)((8 * (long long)n + 127) / 128);
  if (dd) {
    // double-float counts: the FP32 pipe has issue to spare, so 16 lanes per eigenvalue (4.1
    // bits per sweep) while the warps fit eight per SM sub-partition, else 8
    const long long slots = 8LL * 4 * 32 * ctx->num_sms;
    if (slots >= 16LL * n)
      k_stebz<16, true><<<(int)((16 * (long long)n + 127) / 128), 128, 0, ctx->stream>>>(
          n, d, e2, dd, ee, prep, cnt, G, w);
    else
      k_stebz<8, true><<<blocks8, 128, 0, ctx->stream>>>(n, d, e2, dd, ee, prep, cnt, G, w);
    return;
  }
  const long long slots = 4LL * 32 * ctx->num_sms;  // one warp per SM sub-partition
  int K = slots >= 8LL * n ? 8 : slots >= 4LL * n ? 4 : slots >= 2LL * n ? 2 : 1;
  const int tk = qk_tune_get(ctx, TUNE_STEBZ_K, n, 0);  // tuned width, if any
  if (tk == 1 || tk == 2 || tk == 4 || tk == 8) K = tk;
  const int blocks = (int)((K * (long long)n + 127) / 128);
  switch (K) {
    case 8: k_stebz<8, false><<<blocks, 128, 0, ctx->stream>>>(n, d, e2, nullptr, nullptr, prep,
                                                              cnt, G, w); break;
    case 4: k_stebz<4, false><<<blocks, 128, 0, ctx->stream>>>(n, d, e2, nullptr, nullptr, prep,
                                                              cnt, G, w); break;
    case 2: k_stebz<2, false><<<blocks, 128, 0, ctx->stream>>>(n, d, e2, nullptr, nullptr, prep,
                                                              cnt, G, w); break;
    default: k_stebz<1, false><<<blocks, 128, 0, ctx->stream>>>(n, d, e2, nullptr, nullptr, prep,
                                                               cnt, G, w); break;
  }
}

__device__ __forceinline__ double rand_pm1(unsigned long long i, unsigned long long j) {
  unsigned long long z = (i * 0x9E3779B97F4A7C15ull) ^ (j + 0x632BE59BD9B4E019ull);
  z ^= z >> 30; z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27; z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return ((double)(z >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
}

// reciprocal of a U pivot, tiny pivots perturbed to +-tiny first (stored once, so that the
// back substitutions multiply instead of divide on their dependency chain)
__device__ __forceinline__ double pivot_rcp(double u, double tiny) {
  if (fabs(u) < tiny) u = (u < 0.0) ? -tiny : tiny;
  return qk_rcp(u);
}

// Inverse iteration.  Thread j leads the cluster that starts at eigenvalue j (clusters are
// maximal runs with consecutive gaps <= CLUSTER_REL*||T||_1).  Workspace W holds five
// interleaved arrays (U0,U1,U2,mult,swap) of n entries per thread: W[(arr*n + i)*n + j].
// The iterate lives directly in the output row Zt[jj + n*i].
__global__ void k_stein(int n, const double* __restrict__ d, const double* __restrict__ e,
                        const double* __restrict__ w, const double* __restrict__ prep,
                        double* __restrict__ W, double* __restrict__ Zt,
                        const int* __restrict__ status, int iters) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  // after a failed tridiagonalisation (barrier expired) T is meaningless -- possibly one cluster
  // of n equal eigenvalues, whose Gram-Schmidt would take seconds: the call fails anyway
  if (*(const volatile int*)status & QKD_BARRIER_TIMEOUT) return;
  const double tnrm = prep[3];
  const double ortol = CLUSTER_REL * tnrm;
  if (j > 0 && w[j] - w[j - 1] <= ortol) return;  // not a cluster leader
  int jend = j;
  while (jend + 1 < n && w[jend + 1] - w[jend] <= ortol) ++jend;

  const size_t N = (size_t)n;
  double* U0 = W + 0 * N * N;
  double* U1 = W + 1 * N * N;
  double* U2 = W + 2 * N * N;
  double* ML = W + 3 * N * N;
  double* SW = W + 4 * N * N;
  auto at = [&](double* arr, int i) -> double& { return arr[(size_t)i * N + j]; };
  const double tiny = DBL_EPSILON * tnrm;
  double xprev = -INFINITY;

  for (int jj = j; jj <= jend; ++jj) {
    double x = w[jj];
    if (jj > j) {
      const double pertol = 10.0 * fabs(DBL_EPSILON * x) + tiny;
      if (x - xprev < pertol) x = xprev + pertol;
    }
    xprev = x;
    // ---- GEPP of T - x I ----
    double r0 = d[0] - x, r1 = n > 1 ? e[0] : 0.0, r2 = 0.0;
    for (int k = 0; k < n - 1; ++k) {
      const double ck = e[k];
      const double ak1 = d[k + 1] - x;
      const double bk1 = (k + 1 < n - 1) ? e[k + 1] : 0.0;
      if (fabs(ck) <= fabs(r0)) {
        const double m = (r0 != 0.0) ? ck * qk_rcp(r0) : 0.0;
        at(U0, k) = pivot_rcp(r0, tiny); at(U1, k) = r1; at(U2, k) = r2; at(ML, k) = m;
        at(SW, k) = 0.0;
        r0 = ak1 - m * r1;
        r1 = bk1 - m * r2;
        r2 = 0.0;
      } else {
        const double m = r0 * qk_rcp(ck);
        at(U0, k) = pivot_rcp(ck, tiny); at(U1, k) = ak1; at(U2, k) = bk1; at(ML, k) = m;
        at(SW, k) = 1.0;
        const double n0 = r1 - m * ak1;
        const double n1 = r2 - m * bk1;
        r0 = n0;
        r1 = n1;
        r2 = 0.0;
      }
    }
    at(U0, n - 1) = pivot_rcp(r0, tiny); at(U1, n - 1) = 0.0; at(U2, n - 1) = 0.0;
    // ---- start vector ----
    for (int i = 0; i < n; ++i) Zt[(size_t)jj + N * i] = rand_pm1(i, jj);
    for (int it = 0; it < iters; ++it) {
      // scale to unit inf-norm
      double mx = 0.0;
      for (int i = 0; i < n; ++i) mx = fmax(mx, fabs(Zt[(size_t)jj + N * i]));
      const double sc = mx > 0.0 ? 1.0 / mx : 1.0;
      // forward: apply P and L^{-1}.  The loads of a batch of SB steps are issued before its
      // stores (they read entries the batch has not written yet), so the memory latency is paid
      // once per batch instead of once per step of the dependency chain.
      double yk = Zt[jj] * sc;
      int k = 0;
      for (; k + SB <= n - 1; k += SB) {
        double zv[SB], mv[SB], sv[SB];
#pragma unroll
        for (int u = 0; u < SB; ++u) {
          zv[u] = Zt[(size_t)jj + N * (k + 1 + u)];
          mv[u] = at(ML, k + u);
          sv[u] = at(SW, k + u);
        }
#pragma unroll
        for (int u = 0; u < SB; ++u) {
          double yk1 = zv[u] * sc;
          if (sv[u] != 0.0) {
            const double t = yk;
            yk = yk1;
            yk1 = t - mv[u] * yk;
          } else {
            yk1 = yk1 - mv[u] * yk;
          }
          Zt[(size_t)jj + N * (k + u)] = yk;
          yk = yk1;
        }
      }
      for (; k < n - 1; ++k) {
        double yk1 = Zt[(size_t)jj + N * (k + 1)] * sc;
        const double m = at(ML, k);
        if (at(SW, k) != 0.0) {
          const double t = yk;
          yk = yk1;
          yk1 = t - m * yk;
        } else {
          yk1 = yk1 - m * yk;
        }
        Zt[(size_t)jj + N * k] = yk;
        yk = yk1;
      }
      Zt[(size_t)jj + N * (n - 1)] = yk;
      // back substitution with U (pivots stored as reciprocals), batched the same way
      double y1 = 0.0, y2 = 0.0;
      k = n - 1;
      for (; k - SB + 1 >= 0; k -= SB) {
        double zv[SB], a0[SB], a1[SB], a2[SB];
#pragma unroll
        for (int u = 0; u < SB; ++u) {
          zv[u] = Zt[(size_t)jj + N * (k - u)];
          a0[u] = at(U0, k - u);
          a1[u] = at(U1, k - u);
          a2[u] = at(U2, k - u);
        }
#pragma unroll
        for (int u = 0; u < SB; ++u) {
          const double yv = (zv[u] - a1[u] * y1 - a2[u] * y2) * a0[u];
          Zt[(size_t)jj + N * (k - u)] = yv;
          y2 = y1;
          y1 = yv;
        }
      }
      for (; k >= 0; --k) {
        const double yv = (Zt[(size_t)jj + N * k] - at(U1, k) * y1 - at(U2, k) * y2) * at(U0, k);
        Zt[(size_t)jj + N * k] = yv;
        y2 = y1;
        y1 = yv;
      }
      // MGS against earlier members of the cluster
      for (int kk = j; kk < jj; ++kk) {
        double dot = 0.0;
        for (int i = 0; i < n; ++i) dot += Zt[(size_t)jj + N * i] * Zt[(size_t)kk + N * i];
        for (int i = 0; i < n; ++i) Zt[(size_t)jj + N * i] -= dot * Zt[(size_t)kk + N * i];
      }
    }
    // normalise (2-norm), largest component positive
    double mx = 0.0, s2 = 0.0;
    int imx = 0;
    for (int i = 0; i < n; ++i) {
      const double v = Zt[(size_t)jj + N * i];
      if (fabs(v) > mx) { mx = fabs(v); imx = i; }
    }
    const double sc0 = mx > 0.0 ? 1.0 / mx : 1.0;
    for (int i = 0; i < n; ++i) {
      const double v = Zt[(size_t)jj + N * i] * sc0;
      s2 += v * v;
    }
    double sc = sc0 / sqrt(s2);
    if (Zt[(size_t)jj + N * imx] < 0.0) sc = -sc;
    for (int i = 0; i < n; ++i) Zt[(size_t)jj + N * i] *= sc;
  }
}

// Forward compact-WY T factors (upper triangular, dlarft 'F','C') of every reflector block,
// one CTA per block: T_ii = tau_i, T(0:i, i) = -tau_i T(0:i, 0:i) G(0:i, i) with G = V_b^T V_b.
// G and T are BT_NB x BT_NB per block (leading dimension BT_NB); the last block may hold fewer
// than BT_NB reflectors (the rest of its T is zero).
constexpr int LARFT_SMEM = (BT_NB * (BT_NB + 1) + BT_NB) * 8;
__global__ void __launch_bounds__(BT_NB) k_larft_all(int nref, const double* __restrict__ G,
                                                     const double* __restrict__ tau,
                                                     double* __restrict__ T) {
  extern __shared__ double lsm[];
  double* sT = lsm;                       // [BT_NB][BT_NB + 1]
  double* z = lsm + BT_NB * (BT_NB + 1);  // [BT_NB]
  const int b = blockIdx.x, t = threadIdx.x;
  const int kb = b * BT_NB;
  const int nb = (nref - kb) < BT_NB ? (nref - kb) : BT_NB;
  const double* Gb = G + (size_t)b * BT_NB * BT_NB;
  const double* tb = tau + kb;
  for (int idx = t; idx < BT_NB * (BT_NB + 1); idx += blockDim.x) sT[idx] = 0.0;
  __syncthreads();
  for (int i = 0; i < nb; ++i) {
    if (t < i) z[t] = Gb[t + BT_NB * i];
    __syncthreads();
    if (t < i) {
      double s0 = 0.0, s1 = 0.0;
      int c = t;
      for (; c + 1 < i; c += 2) {
        s0 = fma(sT[t * (BT_NB + 1) + c], z[c], s0);
        s1 = fma(sT[t * (BT_NB + 1) + c + 1], z[c + 1], s1);
      }
      if (c < i) s0 = fma(sT[t * (BT_NB + 1) + c], z[c], s0);
      sT[t * (BT_NB + 1) + i] = -tb[i] * (s0 + s1);
    }
    if (t == 0) sT[i * (BT_NB + 1) + i] = tb[i];
    __syncthreads();
  }
  double* Tb = T + (size_t)b * BT_NB * BT_NB;
  for (int idx = t; idx < BT_NB * BT_NB; idx += blockDim.x) {
    const int r = idx % BT_NB, c = idx / BT_NB;
    Tb[idx] = sT[r * (BT_NB + 1) + c];
  }
}

// The two large products of a back-transformation block: FP64 GEMM, or (mixed tier) the
// compensated FP32-product GEMM.  (The BF16x3 tensor-core GEMM is ~7x less accurate here: its
// FP32 tensor-memory accumulator sums 6 x 128 products per chunk against 16 per compensated
// tile, and over the 28 blocks of nS = 3600 that moved the linearised QP energies past 1 meV.)
int bt_big_gemm(qk_ctx* ctx, bool mixed, char ta, char tb, int m, int n, int k, double alpha,
                const double* A, long long lda, const double* B, long long ldb, double beta,
                double* C, long long ldc) {
  if (mixed)
    return qk_gemm_f32p(ctx, ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1);
  return qk_dgemm(ctx, ta, tb, m, n, k, alpha, A, lda, 0, B, ldb, 0, beta, C, ldc, 0, 1);
}

// T factors of all reflector blocks of the last tridiagonalisation on this context:
// G_b = V_b^T V_b for the full blocks in one batched GEMM (V is zero above its unit diagonal,
// so all n rows can be used), the last partial block on its own, then k_larft_all.
int eig_tfactors(qk_ctx* ctx, int n, const double* V, const double* tau, const double** T_out,
                 bool fp32) {
  const int nref = n - 2;
  const int nblk = (nref + BT_NB - 1) / BT_NB;
  const size_t B2 = (size_t)BT_NB * BT_NB;
  double* buf = nullptr;
  QK_TRY(qk_wst(ctx, W_TFAC, 2 * B2 * nblk + 16, &buf));
  double* G = buf;
  double* T = buf + B2 * nblk;
  const int full = nref / BT_NB;
  const long long bstride = (long long)n * BT_NB;
  auto gemm = fp32 ? qk_gemm_f32p : qk_dgemm;
  if (full > 0)
    QK_TRY(gemm(ctx, 'T', 'N', BT_NB, BT_NB, n, 1.0, V, n, bstride, V, n, bstride, 0.0, G, BT_NB,
                (long long)B2, full));
  if (full < nblk) {
    const int kb = full * BT_NB, nb = nref - kb;
    const double* Vb = V + (size_t)n * kb;
    QK_TRY(gemm(ctx, 'T', 'N', nb, nb, n, 1.0, Vb, n, 0, Vb, n, 0, 0.0, G + B2 * full, BT_NB, 0,
                1));
  }
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_larft_all, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    LARFT_SMEM);
  });
  QK_CK(attr_err);
  k_larft_all<<<nblk, BT_NB, LARFT_SMEM, ctx->stream>>>(nref, G, tau, T);
  QK_LAUNCHED();
  *T_out = T;
  return QK_OK;
}

}  // namespace

// ------------------------------------------------------------------------------------------
// grouped tridiagonalisation of the batch workers
// ------------------------------------------------------------------------------------------
struct qk_tri_service {
  struct Req {
    TriArgs ta;
    cudaStream_t stream;
    cudaEvent_t ready;
  };
  qk_ctx* parent = nullptr;
  std::mutex mu;
  std::condition_variable cv;
  int n_active = 0;
  unsigned long long gen = 0;
  int last_status = QK_OK;
  std::vector<Req> pending;
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  long long launches = 0;
  long long matrices = 0;
};

namespace {

// CTAs per request: proportional to the n^3 work, at least one, at most what the matrix can use
// (one 32 x 128 trailing block per CTA, as in the single-matrix launch), all within one CTA per
// SM.  The grouped kernel's arithmetic does not depend on a group's size (sytrd_body<., true>),
// so this split, which changes with the launch's other matrices, never changes a result.
void tri_split(const std::vector<qk_tri_service::Req>& rq, int sms, int* cta0) {
  const int R = (int)rq.size();
  std::vector<double> wgt(R);
  std::vector<int> g(R), cap(R);
  double tot = 0.0;
  for (int r = 0; r < R; ++r) {
    const double n = rq[r].ta.n;
    wgt[r] = n * n * n;
    tot += wgt[r];
    const long long want = (long long)rq[r].ta.n * rq[r].ta.n / (32 * 128) + 1;
    cap[r] = (int)(want < sms ? want : sms);
  }
  int used = 0;
  for (int r = 0; r < R; ++r) {
    int v = (int)((double)sms * wgt[r] / (tot > 0.0 ? tot : 1.0));
    v = v < 1 ? 1 : (v > cap[r] ? cap[r] : v);
    g[r] = v;
    used += v;
  }
  // hand the SMs left over to the requests with the most work per CTA, below their cap
  while (used < sms) {
    int best = -1;
    for (int r = 0; r < R; ++r)
      if (g[r] < cap[r] && (best < 0 || wgt[r] / g[r] > wgt[best] / g[best])) best = r;
    if (best < 0) break;
    ++g[best];
    ++used;
  }
  while (used > sms) {  // R <= TRI_GROUP_MAX < SMs, so at least one request has g > 1
    int best = 0;
    for (int r = 1; r < R; ++r)
      if (g[r] > g[best]) best = r;
    if (g[best] <= 1) break;
    --g[best];
    --used;
  }
  cta0[0] = 0;
  for (int r = 0; r < R; ++r) cta0[r + 1] = cta0[r] + g[r];
}

// one cooperative launch for the pending requests of one arithmetic (FP64 or double-float)
int tri_launch_part(qk_tri_service* sv, const std::vector<qk_tri_service::Req>& rq, bool df) {
  const int R = (int)rq.size();
  if (R == 0) return QK_OK;
  TriGroup g;
  g.nreq = R;
  size_t smem = 0;
  const int nt = df ? DF_THREADS : TRI_THREADS;
  for (int r = 0; r < R; ++r) {
    g.req[r] = rq[r].ta;
    const size_t need = (size_t)(nt / 32) * TRI_TC * TRI_TLD * 8 + 3 * (size_t)g.req[r].n * 8;
    smem = need > smem ? need : smem;
  }
  tri_split(rq, sv->parent->num_sms, g.cta0);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g.cta0[R]);
  cfg.blockDim = dim3(nt);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = sv->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, df ? k_sytrd_df_grouped : k_sytrd_grouped, g) != cudaSuccess)
    return QK_ERR_CUDA;
  sv->launches++;
  sv->matrices += R;
  return QK_OK;
}

// cooperative launches for all pending requests (called with the lock held): one per arithmetic
// present, one after the other on the service stream, each over all SMs
void tri_launch_locked(qk_tri_service* sv) {
  int st = QK_OK;
  const int R = (int)sv->pending.size();
  std::vector<qk_tri_service::Req> part[2];
  for (int r = 0; r < R; ++r) {
    part[sv->pending[r].ta.df ? 1 : 0].push_back(sv->pending[r]);
    if (cudaStreamWaitEvent(sv->stream, sv->pending[r].ready, 0) != cudaSuccess) st = QK_ERR_CUDA;
  }
  for (int k = 0; k < 2 && st == QK_OK; ++k) st = tri_launch_part(sv, part[k], k == 1);
  if (cudaEventRecord(sv->done, sv->stream) != cudaSuccess) st = QK_ERR_CUDA;
  // every requester's stream continues after the group (enqueued before they wake up)
  for (int r = 0; r < R; ++r)
    if (cudaStreamWaitEvent(sv->pending[r].stream, sv->done, 0) != cudaSuccess) st = QK_ERR_CUDA;
  sv->last_status = st;
  sv->pending.clear();
  sv->gen++;
  sv->cv.notify_all();
}

int tri_submit(qk_tri_service* sv, qk_ctx* ctx, const TriArgs& ta) {
  if (!ctx->ev_tri) QK_CK(cudaEventCreateWithFlags(&ctx->ev_tri, cudaEventDisableTiming));
  QK_CK(cudaEventRecord(ctx->ev_tri, ctx->stream));
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->pending.push_back({ta, ctx->stream, ctx->ev_tri});
  const unsigned long long my = sv->gen;
  if ((int)sv->pending.size() >= sv->n_active || (int)sv->pending.size() >= TRI_GROUP_MAX)
    tri_launch_locked(sv);
  else
    sv->cv.wait(lk, [&] { return sv->gen != my; });
  ctx->launches++;
  if (sv->last_status != QK_OK)
    return qk_fail(ctx, QK_ERR_CUDA, "grouped tridiagonalisation launch failed");
  return QK_OK;
}

}  // namespace

qk_tri_service* qk_tri_service_new(qk_ctx* parent, int n_workers) {
  auto* sv = new qk_tri_service();
  sv->parent = parent;
  sv->n_active = n_workers;
  if (cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&sv->done, cudaEventDisableTiming) != cudaSuccess) {
    qk_tri_service_free(sv);
    return nullptr;
  }
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_sytrd_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TRI_SMEM_MAX);
    cudaFuncSetAttribute(k_sytrd_df_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TRI_SMEM_MAX);
  });
  return sv;
}

void qk_tri_service_worker_done(qk_tri_service* sv) {
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->n_active--;
  if (!sv->pending.empty() && (int)sv->pending.size() >= sv->n_active) tri_launch_locked(sv);
}

void qk_tri_service_free(qk_tri_service* sv) {
  if (!sv) return;
  if (sv->parent) {
    sv->parent->tri_groups = sv->launches;
    sv->parent->tri_grouped = sv->matrices;
  }
  if (sv->stream) {
    cudaStreamSynchronize(sv->stream);
    cudaStreamDestroy(sv->stream);
  }
  if (sv->done) cudaEventDestroy(sv->done);
  delete sv;
}

// ------------------------------------------------------------------------------------------
int qk_eig_sym(qk_ctx* ctx, int n, double* A, int lda, double* w, double* Zt, int want_vectors,
               int backtransform, int tri_df) {
  if (n <= 0) return QK_OK;
  const size_t N = (size_t)n;
  // workspace: V (n*n), small vectors (d, e, tau, e2, pbuf(6n), prep(64), per-CTA slots)
  double *V = nullptr, *tri = nullptr;
  const size_t tri_len = 10 * N + 64 + 1024;
  QK_TRY(qk_wst(ctx, W_V, N * N, &V));
  QK_TRY(qk_wst(ctx, W_TRI, tri_len, &tri));
  double* d = tri;
  double* e = tri + N;
  double* tau = tri + 2 * N;
  double* e2 = tri + 3 * N;
  double* pbuf = tri + 4 * N;
  double* prep = tri + 10 * N;
  double* fslot = tri + 10 * N + 64;
  QK_CK(cudaMemsetAsync(V, 0, N * N * sizeof(double), ctx->stream));
  QK_CK(cudaMemsetAsync(tri, 0, tri_len * sizeof(double), ctx->stream));
  QK_CK(cudaMemsetAsync(ctx->d_bar, 0, 16 * sizeof(unsigned), ctx->stream));

  // ---- 1. tridiagonalisation ----
  const bool tm = ctx->time_eig;
  if (tm) qk_tic(ctx, T_TRIDIAG);
  {
    // threads per CTA: the FP64 kernel 1024, the double-float kernel 512 (its registers)
    const int nt = tri_df ? DF_THREADS : TRI_THREADS;
    const size_t tile_bytes = (size_t)(nt / 32) * TRI_TC * TRI_TLD * 8;
    const size_t smem_need = tile_bytes + 3 * N * sizeof(double);
    const int use_smem = smem_need <= (size_t)TRI_SMEM_MAX;
    const size_t smem = use_smem ? smem_need : tile_bytes;
    // the attribute is global to the kernel: set it once, at its maximum, so that concurrent
    // callers on other streams/threads never see a smaller limit than their launch needs
    static std::once_flag once;
    static cudaError_t attr_err = cudaSuccess;
    std::call_once(once, [] {
      attr_err = cudaFuncSetAttribute(k_sytrd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      TRI_SMEM_MAX);
      if (attr_err == cudaSuccess)
        attr_err = cudaFuncSetAttribute(k_sytrd_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        TRI_SMEM_MAX);
    });
    QK_CK(attr_err);
    void (*kern)(TriArgs) = tri_df ? k_sytrd_df : k_sytrd;
    int per_sm = 0;
    QK_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, smem));
    if (per_sm < 1) return qk_fail(ctx, QK_ERR_CUDA, "k_sytrd cannot be resident");
    // one CTA per SM: the O(n) vector work of each column is repeated by every CTA, so fewer,
    // wider CTAs waste less FP64 issue
    per_sm = 1;
    // CTAs of the cooperative grid: 4/4 of the SMs by default, or the tuned fraction
    const int gq = qk_tune_get(ctx, TUNE_SYTRD_GRID, n, 4);
    int grid = per_sm * ctx->num_sms * gq / 4;
    if (grid < 1) grid = 1;
    // small problems do not need the whole GPU
    const int want = (int)((N * N) / (32 * 128)) + 1;
    if (grid > want) grid = want < 1 ? 1 : want;
    // several systems at once (batch workers): each takes a share of the SMs, so that their
    // latency-bound per-column phases overlap instead of queueing for the whole GPU
    if (ctx->sytrd_max_ctas > 0 && grid > ctx->sytrd_max_ctas) grid = ctx->sytrd_max_ctas;
    double* gvec = nullptr;
    if (!use_smem) QK_TRY(qk_wst(ctx, W_VEC, (size_t)grid * 3 * N, &gvec));
    TriArgs ta;
    ta.A = A;
    ta.lda = lda;
    ta.n = n;
    ta.d = d;
    ta.e = e;
    ta.tau = tau;
    ta.V = V;
    ta.ldv = n;
    ta.df = tri_df != 0;
    ta.vscal = e2;           // free until k_tri_prep fills e^2
    ta.dfscale = prep + 8;   // k_tri_prep writes prep[0..4]
    ta.pbuf = pbuf;
    ta.fslot = fslot;
    ta.gvec = gvec;
    ta.bar = ctx->d_bar;
    ta.status = ctx->d_status;
    ta.use_smem = use_smem;
    if (ctx->tri_service && use_smem && !ctx->capturing) {
      // batch worker: the matrix joins the other workers' in one grouped launch
      QK_TRY(tri_submit(ctx->tri_service, ctx, ta));
    } else {
      // cooperative launch (all CTAs co-resident for the grid barrier); also valid under capture
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(grid);
      cfg.blockDim = dim3(nt);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = ctx->stream;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      QK_CK(cudaLaunchKernelEx(&cfg, kern, ta));
      ctx->launches++;
    }
  }
  if (tri_df) {
    k_tri_df_finish<<<n, 256, 0, ctx->stream>>>(n, d, e, tau, V, n, e2, prep + 8);
    QK_LAUNCHED();
  }
  if (tm) qk_toc(ctx, T_TRIDIAG);

  // ---- 2. eigenvalues by bisection ----
  if (tm) qk_tic(ctx, T_BISECT);
  k_tri_prep<<<1, 1024, 0, ctx->stream>>>(n, d, e, e2, prep);
  QK_LAUNCHED();
  // the mixed tier bisects in double-float: d and e^2 as pairs in the (now free) pbuf area
  float2* dd = nullptr;
  float2* ee = nullptr;
  if (tri_df) {
    dd = reinterpret_cast<float2*>(pbuf);
    ee = dd + n;
    k_tri_df_copy<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, d, e2, dd, ee);
    QK_LAUNCHED();
  }
  int* cnt = nullptr;
  if (n >= 256) {
    QK_TRY(qk_wst(ctx, W_STEBZ, (size_t)STEBZ_GRID + 64, &cnt));
    if (tri_df)
      k_stebz_grid<true><<<(STEBZ_GRID + 128) / 128, 128, 0, ctx->stream>>>(
          n, d, e2, dd, ee, prep, STEBZ_GRID, cnt);
    else
      k_stebz_grid<false><<<(STEBZ_GRID + 128) / 128, 128, 0, ctx->stream>>>(
          n, d, e2, nullptr, nullptr, prep, STEBZ_GRID, cnt);
    QK_LAUNCHED();
  }
  launch_stebz(ctx, n, d, e2, dd, ee, prep, cnt, STEBZ_GRID, w);
  QK_LAUNCHED();
  if (!want_vectors) {
    k_tri_unscale<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, prep, w);
    QK_LAUNCHED();
  }
  if (tm) qk_toc(ctx, T_BISECT);
  if (!want_vectors) return QK_OK;
  // ---- 3. eigenvectors of T by inverse iteration ----
  double* Wst = nullptr;
  QK_TRY(qk_wst(ctx, W_EIGWORK, 5 * N * N, &Wst));
  if (tm) qk_tic(ctx, T_STEIN);
  // one warp per block: the threads' sweeps are latency-bound chains, so the warps go to as
  // many SMs as there are (each with its own load/store and FP64 units)
  // iterations from the random start: three in FP64 (as dstein's convergence plus its two
  // extra steps), two in the mixed tier, whose eigenvalues come from the double-float bisection
  // and whose vectors feed FP32 products
  k_stein<<<(n + 31) / 32, 32, 0, ctx->stream>>>(n, d, e, w, prep, Wst, Zt, ctx->d_status,
                                                 tri_df ? 2 : 3);
  QK_LAUNCHED();
  k_tri_unscale<<<(n + 255) / 256, 256, 0, ctx->stream>>>(n, prep, w);
  QK_LAUNCHED();
  if (tm) qk_toc(ctx, T_STEIN);

  if (!backtransform) return QK_OK;  // caller applies Q^T itself (qk_eig_apply_qt)
  // ---- 4. back-transformation Zt <- Zt * Q^T, blocks from last to first ----
  // (backtransform == 2, the mixed tier: the block products and the T factors with compensated
  // FP32 products; Zt stays FP64)
  auto gemm = backtransform == 2 ? qk_gemm_f32p : qk_dgemm;
  if (tm) qk_tic(ctx, T_BACKTRANS);
  const int nref = n - 2;  // reflectors 0..n-3 can be non-trivial
  if (nref > 0) {
    const double* Tall = nullptr;
    QK_TRY(eig_tfactors(ctx, n, V, tau, &Tall, backtransform == 2));
    double* bt = nullptr;
    QK_TRY(qk_wst(ctx, W_PART, 2 * N * BT_NB, &bt));
    double* W1 = bt;
    double* W2 = bt + N * BT_NB;
    const int nblk = (nref + BT_NB - 1) / BT_NB;
    for (int b = nblk - 1; b >= 0; --b) {
      const int kb = b * BT_NB;
      const int nb = (nref - kb) < BT_NB ? (nref - kb) : BT_NB;
      const int m = n - kb - 1;
      const double* Vb = V + (kb + 1) + N * kb;
      const double* Tb = Tall + (size_t)b * BT_NB * BT_NB;
      double* Es = Zt + N * (kb + 1);
      QK_TRY(bt_big_gemm(ctx, backtransform == 2, 'N', 'N', n, nb, m, 1.0, Es, n, Vb, n, 0.0, W1,
                         n));
      QK_TRY(gemm(ctx, 'N', 'T', n, nb, nb, 1.0, W1, n, 0, Tb, BT_NB, 0, 0.0, W2, n, 0, 1));
      QK_TRY(bt_big_gemm(ctx, backtransform == 2, 'N', 'T', n, m, nb, -1.0, W2, n, Vb, n, 1.0, Es,
                         n));
    }
  }
  if (tm) qk_toc(ctx, T_BACKTRANS);
  return QK_OK;
}

// X (n x ncols, ldx) <- Q^T X with the reflectors of the last qk_eig_sym call on this context
// (Q = H_0 H_1 ... H_{n-3}); compact-WY blocks applied first to last:
//   X <- X - V (T^T (V^T X)) on rows kb+1..n-1;  fp32: the block products in FP32.
int qk_eig_apply_qt(qk_ctx* ctx, int n, double* X, long long ldx, int ncols, int fp32) {
  const int nref = n - 2;
  if (nref <= 0 || ncols <= 0) return QK_OK;
  const size_t N = (size_t)n;
  double *V = nullptr, *tri = nullptr, *bt = nullptr;
  QK_TRY(qk_wst(ctx, W_V, N * N, &V));
  QK_TRY(qk_wst(ctx, W_TRI, 8 * N + 64, &tri));
  double* tau = tri + 2 * N;
  const double* Tall = nullptr;
  QK_TRY(eig_tfactors(ctx, n, V, tau, &Tall, fp32 != 0));
  QK_TRY(qk_wst(ctx, W_PART, 2 * (size_t)ncols * BT_NB, &bt));
  double* W1 = bt;
  double* W2 = bt + (size_t)ncols * BT_NB;
  const int nblk = (nref + BT_NB - 1) / BT_NB;
  auto gemm = fp32 ? qk_gemm_f32p : qk_dgemm;
  for (int b = 0; b < nblk; ++b) {
    const int kb = b * BT_NB;
    const int nb = (nref - kb) < BT_NB ? (nref - kb) : BT_NB;
    const int m = n - kb - 1;
    const double* Vb = V + (kb + 1) + N * kb;
    const double* Tb = Tall + (size_t)b * BT_NB * BT_NB;
    double* Xs = X + (kb + 1);
    // W1 = V^T X (nb x ncols), W2 = T^T W1, X -= V W2
    QK_TRY(bt_big_gemm(ctx, fp32 != 0, 'T', 'N', nb, ncols, m, 1.0, Vb, n, Xs, ldx, 0.0, W1, nb));
    QK_TRY(gemm(ctx, 'T', 'N', nb, ncols, nb, 1.0, Tb, BT_NB, 0, W1, nb, 0, 0.0, W2, nb, 0, 1));
    QK_TRY(bt_big_gemm(ctx, fp32 != 0, 'N', 'N', m, ncols, nb, -1.0, Vb, n, W2, nb, 1.0, Xs, ldx));
  }
  return QK_OK;
}

extern "C" int qk_dsyev_dev(qk_ctx* ctx, int n, double* d_A, int lda, double* d_w, double* d_Zt,
                            int want_vectors) {
  if (!ctx || n < 0 || lda < n) return QK_ERR_ARG;
  cudaSetDevice(ctx->device);
  QK_TRY(qk_order_after_default(ctx));
  QK_TRY(qk_status_reset(ctx));
  QK_TRY(qk_eig_sym(ctx, n, d_A, lda, d_w, d_Zt, want_vectors, 1, ctx->dsyev_df));
  return qk_status_check(ctx, QKD_BARRIER_TIMEOUT | QKD_BAD_INDEX);
}
