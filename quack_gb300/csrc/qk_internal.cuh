// qk_internal.cuh -- shared internals of libqkgw.so (context, workspace, error plumbing,
// device helpers).  Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>
#include "../../include/qkgw.h"

// device status bits (QKD_*, written by kernels instead of trapping) are in qkgw.h

// stage timers (device time via cudaEvents on the context stream)
enum {
  T_BUILD = 0, T_TRIDIAG, T_BISECT, T_STEIN, T_BACKTRANS, T_SLAB, T_RHO, T_SIGMA, T_QP, T_CASIDA2,
  T_MISC, T_NUM
};

// runtime-tunable launch parameters (chosen by qk_autotune, looked up by size bucket)
enum { TUNE_BF16X3_CHUNK = 0, TUNE_SPLITK_MULT, TUNE_SIGMA_CHUNKS, TUNE_SYTRD_GRID, TUNE_DGEMM_PATH, TUNE_STEBZ_K, TUNE_QP_PERSIST, TUNE_NUM };
constexpr int TUNE_BUCKETS = 40;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

enum {
  W_ERI = 0, W_E, W_M, W_V, W_ZT, W_EIGWORK, W_TRI, W_SLAB, W_RHO, W_XPY, W_XMY, W_VEC, W_PART,
  W_MISC, W_HOST_A, W_HOST_B, W_SPLIT_A, W_SPLIT_B, W_M2, W_SPLITK, W_QPLIST, W_VEC2, W_KMAT, W_BATCHIO, W_MLPIO, W_FEAT, W_GUESS, W_TUNE, W_TMAT, W_TMAT2, W_RHO32, W_OMF, W_TFAC, W_STEBZ,
  W_QUAD, W_QLT, W_QPV, W_QL, W_QX, W_QQ, W_QD, W_BSE, W_BSEU, W_BSER, W_BSEK, W_ERIPACK,
  W_QSR1, W_QSR2, W_QSJK, W_QSMAT, W_QSDIIS, W_QSIN, W_QPQUEUE, W_ACF, W_NUMBUF
};

struct qk_tri_service;  // grouped tridiagonalisation for the batch workers (k_eig.cu)

struct qk_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[2 * T_NUM + 2] = {};
  cudaEvent_t ev_in = nullptr;  // orders the stream after the caller's default-stream work
  cudaStream_t copy_stream = nullptr;  // host->device copies overlapped with the kernels
  cudaEvent_t ev_copy = nullptr;       // end of the overlapped ERI upload
  bool eri_pending = false;            // the slab gather must wait for ev_copy first
  bool tda_w = false;                  // the drivers' screening Casida in the Tamm-Dancoff form
  double timings[T_NUM] = {};
  unsigned long long nvtx[T_NUM] = {};  // open NVTX range per stage (0 = none)
  std::string err;
  int* d_status = nullptr;      // device status word
  unsigned* d_bar = nullptr;    // grid-barrier counters (zeroed before each cooperative launch)
  DevBuf buf[W_NUMBUF];
  long long launches = 0;
  int stage_precision = QK_PREC_FP64;
  int sytrd_max_ctas = 0;  // cap on the tridiagonalisation grid (batch workers share the GPU)
  int newton_maxit = 64;   // Newton steps of the graphical QP solve (RGW_QP_graph.f90:38)
  int guess_gate = 0;      // learned-guess start rule (k_guess: 0 Halley agreement, 1, 2)
  int fail_alloc_in = 0;   // > 0: the n-th next growing workspace allocation fails (test hook)
  int dsyev_df = 0;        // qk_dsyev_dev tridiagonalises in double-float (the mixed tier's way)
  qk_tri_service* tri_service = nullptr;  // batch worker: tridiagonalise through the group launch
  cudaEvent_t ev_tri = nullptr;           // end of this context's work before a group launch
  long long tri_groups = 0;               // grouped tridiagonalisation launches of the last batch
  long long tri_grouped = 0;              // matrices they tridiagonalised
  int last_dev_status = 0;
  bool time_eig = true;  // stage timers inside the eigensolver (off for the eigenvalue-only pass)
  std::vector<int> qp_iters;  // Newton steps per orbital of the last QP solve
  std::vector<qk_ctx*> workers;  // per-stream sub-contexts of the batched driver
  qk_mlp* mlp = nullptr;         // learned QP guess model (not owned)
  bool capture_features = false;
  std::vector<float> features;   // last captured N x 16 raw features
  long long qp_evals = 0;        // orbital-evaluations of Sigma in the last Newton solve
  bool timing = true;            // stage events (off while a graph is being captured)
  bool graph_mode = false;       // evGW cycles 2.. replayed from a CUDA graph
  bool capturing = false;        // inside stream capture: no host synchronisation allowed
  int tune[TUNE_NUM][TUNE_BUCKETS] = {};  // 0 = not tuned (defaults apply)
  cudaGraphExec_t evgw_exec = nullptr;
  std::vector<long long> evgw_key;  // shape/pointer key of the cached evGW graph
};

// Factorised-integral drivers on one context (qk_api.cu), reused by the batched driver.
int qk_g0w0_L(qk_ctx* ctx, const qk_gw_params* prm, int N, int nC, int nO, int nR, int naux,
              const double* L, const double* eHF, double* eGW, double* SigC, double* Z, double* Om,
              double* EcRPA, double* EcGM);
int qk_evgw_L(qk_ctx* ctx, const qk_gw_params* prm, int N, int nC, int nO, int nR, int naux,
              const double* L, const double* eHF, double* eGW, double* SigC, double* Z,
              double* EcRPA, double* EcGM, int* nSCF, double* Conv);


// ------------------------------------------------------------------------------------------
// error helpers
// ------------------------------------------------------------------------------------------
int qk_fail(qk_ctx* ctx, int code, const char* fmt, ...);
int qk_cuda_fail(qk_ctx* ctx, cudaError_t e, const char* what, const char* file, int line);

#define QK_CK(call)                                                                  \
  do {                                                                               \
    cudaError_t _e = (call);                                                         \
    if (_e != cudaSuccess) return qk_cuda_fail(ctx, _e, #call, __FILE__, __LINE__);  \
  } while (0)

#define QK_LAUNCHED()                                                                \
  do {                                                                               \
    ctx->launches++;                                                                 \
    cudaError_t _e = cudaGetLastError();                                             \
    if (_e != cudaSuccess) return qk_cuda_fail(ctx, _e, "kernel launch", __FILE__, __LINE__); \
  } while (0)

#define QK_TRY(expr)                  \
  do {                                \
    int _s = (expr);                  \
    if (_s != QK_OK) return _s;       \
  } while (0)

// tuned value of a parameter for a problem size (bucket = floor(log2(size))), or dflt
int qk_tune_get(const qk_ctx* ctx, int param, long long size, int dflt);

// grow-only device workspace slot
int qk_ws(qk_ctx* ctx, int slot, size_t bytes, void** out);
template <class T>
inline int qk_wst(qk_ctx* ctx, int slot, size_t count, T** out) {
  return qk_ws(ctx, slot, count * sizeof(T), (void**)out);
}
// make ctx->stream wait for the work already enqueued on the legacy default stream (where a
// caller such as PyTorch writes the device inputs), without a host synchronisation
int qk_order_after_default(qk_ctx* ctx);
// reset and read back the device status word
int qk_status_reset(qk_ctx* ctx);
int qk_status_check(qk_ctx* ctx, int fatal_mask);

// stage timing
void qk_tic(qk_ctx* ctx, int stage);
void qk_toc(qk_ctx* ctx, int stage);
void qk_timings_clear(qk_ctx* ctx);
void qk_timings_collect(qk_ctx* ctx);

// ------------------------------------------------------------------------------------------
// kernel-level entry points (all enqueue on ctx->stream; device pointers)
// ------------------------------------------------------------------------------------------
// Double-float GEMM (FP32 pairs, exact products, compensated sums; ~1e-13 of sum |a b|): the
// mixed tier's substitute for FP64 where cancellation rules out FP32 products.
int qk_gemm_df(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha, const double* A,
               long long lda, long long strideA, const double* B, long long ldb,
               long long strideB, double beta, double* C, long long ldc, long long strideC,
               int batch);
// FP64 GEMM (DFMA or DMMA), column-major: C = alpha*op(A)*op(B) + beta*C, batched by strides.
int qk_dgemm(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha, const double* A,
             long long lda, long long strideA, const double* B, long long ldb, long long strideB,
             double beta, double* C, long long ldc, long long strideC, int batch);
// The same contract with FP32 products and FP32 partial sums (split-K slices added in FP64);
// the _lower form computes only the tiles touching the lower triangle of C and can scale the
// k index of op(B) by kscale[batch * sK + k] (C = alpha op(A) diag(kscale) op(B) + beta C).
int qk_gemm_f32p(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha,
                 const double* A, long long lda, long long strideA, const double* B, long long ldb,
                 long long strideB, double beta, double* C, long long ldc, long long strideC,
                 int batch);
int qk_gemm_f32p_lower(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha,
                       const double* A, long long lda, long long strideA, const double* B,
                       long long ldb, long long strideB, double beta, double* C, long long ldc,
                       long long strideC, int batch, const float* kscale = nullptr,
                       long long sK = 0);

// FP64 GEMM that computes only the 64x64 tiles of C touching its lower triangle (rows >= cols);
// for symmetric rank-k updates whose consumer reads the lower triangle.
int qk_dgemm_lower(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha,
                   const double* A, long long lda, long long strideA, const double* B,
                   long long ldb, long long strideB, double beta, double* C, long long ldc,
                   long long strideC, int batch);

// dRPA correlation energy at orbital energies e by imaginary-frequency quadrature (k_rpa_quad.cu);
// from the (ia|jb) block of ERI (pivoted Cholesky) or from Lov (nS x naux).  Writes the energy
// to the device scalar Ec.  A negative e_a - e_i writes NaN (what the Casida square roots give).
// *applied = 0 (and nothing written) when the quadrature does not apply (a zero e_a - e_i, a
// spectrum too wide for the grids, or a factor rank above nS/3) or, with gap_only, whenever
// the gap is not negative; the caller then takes the eigenvalue route.
int qk_rpa_ec_quad(qk_ctx* ctx, int N, int nC, int nO, int nR, const double* e, const double* ERI,
                   const double* Lov, int naux, double* Ec, int* applied, bool gap_only = false);
// Gauss-Legendre nodes and weights on [-1, 1] (Newton iteration on P_n).
void qk_gauss_legendre_host(int n, double* x, double* w);

// Casida solve on device buffers (qk_api.cu; LR/phRLR.f90:45-95), A and B overwritten; TDA or
// full; scal[0..2] = tr A, sum Om, EcRPA; want_vectors = 0 skips the final eigenvectors.
int phrlr_dev(qk_ctx* ctx, int TDA, int nS, double* dA, double* dB, double* dOm, double** XpY,
              double** XmY, double* scal, int want_vectors);

// quasiparticle self-consistent GW, AO-basis pieces (k_qsgw.cu):
//   J = Hartree, K = exchange matrix of P over the AO tensor (N = nBas; part: 2 N^3 scratch);
//   slab / Kmat from the partial MO transform with c (nBas x N; W1, W2: max(nBas^3 no, N^2 nS));
//   Sig = full correlation self-energy (unsymmetrised, W: N^2 nS scratch);
//   df: the GEMMs run in double-float (mixed tier) instead of FP64;
//   out[0..5] = ET, EV, EJ, EK, EqsGW, max|err|.
int qk_qs_jk(qk_ctx* ctx, int N, const double* ERI, const double* P, double* part, double* J,
             double* K);
int qk_qs_mo_slab(qk_ctx* ctx, int nBas, int N, int nC, int nO, int nR, const double* c,
                  const double* ERI, double* W1, double* W2, double* slab, double* Kmat, int df);
int qk_qs_sigma(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                int nS, const double* e, const double* Om, const double* rho, double* W,
                double* Sig, int df);
int qk_qs_sym(qk_ctx* ctx, int N, int nC, int nR, const double* Sig, double* out);
int qk_qs_mask(qk_ctx* ctx, int N, int nC, int nR, double* Sig);
int qk_qs_fock(qk_ctx* ctx, int N, const double* Hc, const double* J, const double* K,
               const double* SigCp, double* F);
int qk_qs_energy(qk_ctx* ctx, int N, const double* P, const double* T, const double* V,
                 const double* J, const double* K, const double* err, double* out);

// static phBSE@GW excitation energies (k_bse.cu; GW/RGW_phBSE.f90:83-190): device ERI (full
// N^4), eW (screening energies), eGW; EcBSE[2] on the host; OmS / OmT (device, nS) optional.
// adiabatic-connection (ACFDT) correlation energy of phBSE@GW (k_bse.cu; GW/RGW_phACFDT.f90:1-219):
// EcAC[2] (singlet, triplet) on the host
int qk_bse_acfdt_dev(qk_ctx* ctx, int exchange_kernel, int doXBS, int TDA_W, int TDA, int singlet,
                     int triplet, double eta, int N, int nC, int nO, int nR, const double* ERI,
                     const double* eW, const double* eGW, double* hEcAC);
int qk_bse_dev(qk_ctx* ctx, int TDA_W, int TDA, int singlet, int triplet, int exchange_kernel,
               double eta, int N, int nC, int nO, int nR, const double* ERI, const double* eW,
               const double* eGW, double* hEcBSE, double* OmS, double* OmT);

// dense symmetric eigensolver pieces.  backtransform: 0 = leave Zt as the eigenvectors of the
// tridiagonal matrix, 1 = back-transform in FP64, 2 = back-transform with FP32 products.
// tri_df: tridiagonalise in double-float arithmetic on the FP32 pipe (the mixed tier; the
// tridiagonal matrix, reflectors, eigenvalues and eigenvectors stay FP64); the lower triangle of
// A is overwritten either way.
// Grouped tridiagonalisation service of the batched driver: workers' tridiagonalisations are
// collected until every active worker has submitted one (or finished), then run as ONE
// cooperative launch of k_sytrd_grouped with a CTA group per matrix.
qk_tri_service* qk_tri_service_new(qk_ctx* parent, int n_workers);
void qk_tri_service_worker_done(qk_tri_service* svc);
void qk_tri_service_free(qk_tri_service* svc);
int qk_eig_sym(qk_ctx* ctx, int n, double* A, int lda, double* w, double* Zt, int want_vectors,
               int backtransform = 1, int tri_df = 0);
int qk_eig_apply_qt(qk_ctx* ctx, int n, double* X, long long ldx, int ncols, int fp32 = 0);

// Casida pieces (k_casida.cu)
int qk_launch_build_AB(qk_ctx* ctx, int which, int ispin, int dRPA, int N, int nC, int nO, int nR,
                       double lambda, const double* e, const double* ERI, double* out);
int qk_launch_casida_M(qk_ctx* ctx, int N, int nC, int nO, int nR, const double* e,
                       const double* ERI, double* M, double* sq, double* trA);
int qk_launch_casida_M_from_AB(qk_ctx* ctx, int nS, const double* A, const double* B, double* M,
                               double* sq, double* trA);
int qk_launch_xpy(qk_ctx* ctx, int nS, const double* w, const double* Zt, const double* sq,
                  double* Om, double* XpY, double* XmY, int want_xmy);
int qk_launch_sum_sqrt(qk_ctx* ctx, int nS, const double* w, double* out);
int qk_launch_omega(qk_ctx* ctx, int nS, const double* w, double* Om);
int qk_launch_rowscale(qk_ctx* ctx, int rows, int cols, const double* d, int mode,
                       const double* X, long long ldx, double* Y, long long ldy);
int qk_launch_gather_ov(qk_ctx* ctx, int N, int nC, int nO, int nR, int naux, const double* L,
                        double* Lov);
int qk_launch_casida_M_K(qk_ctx* ctx, int N, int nC, int nO, int nR, const double* e,
                         const double* K, double* M, double* sq, double* trA);
int qk_launch_slab_gather(qk_ctx* ctx, int N, int nC, int nO, int nR, const double* ERI,
                          double* S);

// self-energy / QP pieces (k_sigma.cu)
// Mixed-tier pole sums (eta = 0, no SRG): terms with |eps| >= tau in FP32 from R = 2 rho^2
// (FP32, p-major: R[m + nS (q + N p)]) and Om as (hi, lo) float pairs, the terms within tau of a
// pole in FP64 from rho.
struct qk_sigma_ff {
  const float* R = nullptr;
  const float2* OmF = nullptr;
  const int* bad = nullptr;  // set when Om is not ascending (every term then goes to FP64)
  float tau = 0.1f;
};
int qk_sigma_ff_prep(qk_ctx* ctx, int N, int nS, const double* rho, const double* Om,
                     qk_sigma_ff* ff);
int qk_sigma_diag(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                  int nS, const double* e, const double* Om, const double* rho, double* Sig,
                  double* Z, double* EcGM, const qk_sigma_ff* ff = nullptr);
int qk_qp_newton(qk_ctx* ctx, int doSRG, double eta, double flow, int N, int nC, int nO, int nR,
                 int nS, const double* eHF, const double* Om, const double* rho,
                 const double* eGWlin, const double* eOld, double* eGW, double* Z,
                 const double* w_guess = nullptr, int guess_maxit = 8,
                 const qk_sigma_ff* ff = nullptr, const int* guess_fromref = nullptr);
// per-orbital features of the linearised stage (N x 16 floats, row-major, raw)
// features of the linearised stage (F: N x QK_MLP_NIN); hal (optional): the FP64 Halley step
// of the QP equation from eGWlin (NaN where it is not usable)
int qk_features(qk_ctx* ctx, int N, int nC, int nO, int nR, int nS, const double* e,
                const double* wlin, const double* Om, const double* rho, const double* Sig,
                const double* Z, float* F, double* hal = nullptr);
// learned guess w0 = e + shift(features) with the attached model
// Newton start per orbital from the attached model: eGWlin + Halley step where the network's
// predicted shift agrees with it, else the reference start (fromref = 1)
int qk_guess_from_model(qk_ctx* ctx, int N, const float* F, const double* base, const double* hal,
                        double* w0, int* fromref);
int qk_qp_linear(qk_ctx* ctx, int N, const double* eHF, const double* Z, const double* Sig,
                 int use_z, double* eGW);
int qk_diis_dev(qk_ctx* ctx, int n_err, int n_e, int n_diis, double* err_hist, double* e_hist,
                const double* err_in, double* e_inout, double* rcond_dev,
                const int* n_diis_dev = nullptr);
int qk_sub(qk_ctx* ctx, int n, const double* a, const double* b, double* out);
int qk_max_abs_diff(qk_ctx* ctx, int n, const double* a, const double* b, double* out_dev);

// BF16x3 tensor-core GEMM (k_bf16x3.cu): C(m x n, ldc) = A(m x k) * B(n x k)^T, column-major,
// FP64 in/out, three-way BF16 split, FP32 accumulation in TMEM.
// The general form: C_b = alpha op(A_b) diag(bscale_b) op(B_b) + beta C_b for b < batch (operands
// with stride 0 are shared; bscale, if given, scales the k index of op(B)), lower: only the
// 128x128 tiles touching the lower triangle of C.  Few output tiles with a long k split k over
// CTAs (FP64 slices and one reduction).
int qk_gemm_bf16x3(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha,
                   const double* A, long long lda, long long sA, const double* B, long long ldb,
                   long long sB, const float* bscale, long long sBS, double beta, double* C,
                   long long ldc, long long sC, int batch, bool lower);
int qk_gemm_bf16x3_nt(qk_ctx* ctx, int m, int n, int k, const double* A, long long lda,
                      const double* B, long long ldb, double* C, long long ldc);

// ------------------------------------------------------------------------------------------
// device helpers
// ------------------------------------------------------------------------------------------
#define QK_MAX_SPIN (1u << 25)

// Poll limit of the bounded grid barriers: the context's status block holds an optional
// override in its second word (set by qk_tune_set(ctx, "spin_limit", ., n); 0 = QK_MAX_SPIN),
// so that a test can make a barrier wait run out and check the reported status.
__device__ __forceinline__ unsigned qk_spin_limit(const int* status) {
  const unsigned v = (unsigned)((const volatile int*)status)[1];
  return v ? v : QK_MAX_SPIN;
}

__device__ __forceinline__ unsigned qk_ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Monotone-counter barrier over `nblocks` co-resident CTAs (cooperative launch guarantees
// co-residency).  Bounded: after qk_spin_limit(status) polls it records QKD_BARRIER_TIMEOUT and
// returns false; callers then leave the kernel.  `epoch` counts barriers passed by this CTA.
// Ordering without separate fences: the CTA's writes before the barrier are ordered before
// thread 0's arrival by the first __syncthreads, the arrival is a release RMW at GPU scope (so
// those writes become visible with it), the poll is an acquire load, and the arrivals of all CTAs
// form one release sequence on the counter, so the load that sees the full count synchronises
// with every CTA's arrival; the second __syncthreads passes that on to the whole CTA.
__device__ __forceinline__ bool qk_grid_barrier(unsigned* counter, unsigned nblocks,
                                                unsigned& epoch, int* status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    epoch++;
    unsigned target = epoch * nblocks;
    const unsigned limit = qk_spin_limit(status);
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(counter) : "memory");
    unsigned spins = 0;
    while (qk_ld_acquire(counter) < target) {
      if (++spins > limit) { atomicOr(status, QKD_BARRIER_TIMEOUT); ok = 0; break; }
      if (spins > 64) __nanosleep(64);
    }
    if (ok && (*((volatile int*)status) & QKD_BARRIER_TIMEOUT)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// 1/x in FP64: the hardware's approximate FP64 reciprocal (rcp.approx.ftz.f64) refined by two
// Newton-Raphson steps r <- r (2 - x r), each of which squares the relative error; magnitudes
// outside [1e-300, 1e300] (where the approximation flushes) take the IEEE division.
__device__ __forceinline__ double qk_rcp(double x) {
  const double ax = fabs(x);
  if (!(ax > 1e-300 && ax < 1e300)) return 1.0 / x;
  double r;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  r = r * fma(-x, r, 2.0);
  r = r * fma(-x, r, 2.0);
  return r;
}

// 1/sqrt(x) for x > 0 in FP64: the hardware approximation (rsqrt.approx.ftz.f64) refined by two
// Newton-Raphson steps r <- r (3 - x r^2) / 2; x outside [1e-300, 1e300] takes 1 / sqrt(x).
__device__ __forceinline__ double qk_rsqrt(double x) {
  if (!(x > 1e-300 && x < 1e300)) return 1.0 / sqrt(x);
  double r;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
  const double hx = 0.5 * x;
  r = r * fma(-hx * r, r, 1.5);
  r = r * fma(-hx * r, r, 1.5);
  return r;
}

template <class T>
__device__ __forceinline__ T qk_block_sum(T v, T* red /* >= 32 entries */) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  T s = (T)0;
  if (wid == 0) {
    s = lane < nw ? red[lane] : (T)0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[0] = s;
  }
  __syncthreads();
  s = red[0];
  return s;
}

// block-wide maximum, every thread gets the result (fmax semantics: NaN operands are ignored)
__device__ __forceinline__ double qk_block_max(double v, double* red /* >= 32 entries */) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  if (wid == 0) {
    double s = lane < nw ? red[lane] : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) s = fmax(s, __shfl_xor_sync(0xffffffffu, s, o));
    if (lane == 0) red[0] = s;
  }
  __syncthreads();
  return red[0];
}
