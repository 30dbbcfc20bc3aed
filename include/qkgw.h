/*
 * qkgw.h -- C ABI of the GB300-native restricted G0W0 / evGW library (libqkgw.so).
 *
 * Conventions (the same as QuAcK's existing GPU module, src/cuda/src/ph_drpa_sing.c:17-18
 * bound from Fortran in src/GPU/cu_quack_module.f90:25-36):
 *   - every integer is a C int passed by value (Fortran: integer(c_int), value);
 *   - every array is a double* into a Fortran column-major array, caller-owned;
 *   - host-pointer entry points copy in, compute on the GPU, copy out and return when done;
 *   - *_dev entry points take device pointers and return once the work is complete;
 *   - every function returns a status (QK_OK = 0).  Unlike the reference module, which prints and
 *     calls exit() on a CUDA error (src/cuda/src/utils.cu:10-16), nothing here exits the host.
 *
 * Array meanings (0-based C offsets of the Fortran arrays):
 *   ERI(p,q,r,s) = <pq|rs> at p + N*(q + N*(r + N*s))               (N = nOrb)
 *   Aph/Bph(ia,jb), ia = (i-nC)*nv + (a-nO), at ia + nS*jb          (nv = nOrb-nO-nR)
 *   XpY/XmY(m,ia) at m + nS*ia  (row m = excitation, CPU orientation of LR/phRLR.f90:77-81)
 *   rho(p,q,m) at p + N*(q + N*m)
 *
 * A context is single-stream and not thread-safe: use one per host thread.
 */
#ifndef QKGW_H
#define QKGW_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct qk_ctx qk_ctx;

enum {
  QK_OK = 0,
  QK_ERR_ARG = 1,          /* invalid sizes / unsupported option values */
  QK_ERR_CUDA = 2,         /* a CUDA runtime call failed (see qk_last_error_string) */
  QK_ERR_NOMEM = 3,        /* device allocation failed */
  QK_ERR_NOT_PD = 4,       /* reserved: A-B not positive definite (reported as warning flag) */
  QK_ERR_NO_CONV = 5,      /* evGW did not converge in maxSCF cycles (evRGW.f90:190-198 stops) */
  QK_ERR_UNSUPPORTED = 6,  /* option outside the supported path */
  QK_ERR_DEVICE = 7,       /* a device-side check failed (bounded wait expired, bad index) */
  QK_ERR_NO_DEVICE = 8     /* no CUDA device / library not built for this GPU */
};

/* precision tiers */
enum {
  QK_PREC_FP64 = 0,        /* FP64 throughout (plain form) */
  QK_PREC_BF16X3 = 1       /* mixed: the excitation-density contraction as BF16x3 split products
                              on tcgen05 (FP32 accumulation, compensated) and the eigenvector
                              back-transformation on compensated FP32 products; with eta = 0 and
                              no SRG the pole sums of Sigma/dSigma (linearised stage and Newton)
                              take the terms with |w - e +- Om| >= 0.01 Ha in FP32 and the
                              near-pole terms in FP64; G0W0's EcRPA at eGW by frequency
                              quadrature.  The Casida eigenvalues, the Newton update and DIIS stay
                              FP64. */
};

/* Options of the GW line of QuAcK's input/options (QuAcK/read_options.f90:242-267). */
typedef struct qk_gw_params {
  double eta;        /* eta_GW */
  int linearize;     /* lin_GW */
  int doSRG;         /* reg_GW  (SRG regularisation, flow s = 500, RG0W0.f90:98) */
  int TDA_W;         /* Tamm-Dancoff screening: Om = eig(A), XpY = XmY = eigenvectors */
  int maxSCF;        /* maxSCF_GW (evGW) */
  double thresh;     /* thresh_GW (evGW) */
  int max_diis;      /* max_diis_GW (evGW) */
  int precision;     /* QK_PREC_* */
  int qp_guess;      /* 0: Newton from the reference start (eGWlin); 1: Newton from the learned
                        guess of the context's model (qk_set_qp_model), restarted from the
                        reference start for orbitals that do not converge within 8 steps;
                        2: the same protocol started from eHF (a comparison baseline) */
} qk_gw_params;

/* ---- context ------------------------------------------------------------------------------ */
int qk_init(int device, qk_ctx** ctx);
int qk_finalize(qk_ctx* ctx);
const char* qk_last_error_string(const qk_ctx* ctx);
/* Per-stage device times (ms) of the last driver call; names in qk_timing_name(i). */
int qk_get_timings(const qk_ctx* ctx, double* ms, int n);
const char* qk_timing_name(int i);
int qk_num_timings(void);
/* Device-side status bits of the context's last call (kernels record them instead of trapping;
 * the call returns QK_ERR_DEVICE when a fatal one is set, the others mirror the reference's
 * printed warnings). */
enum {
  QKD_BARRIER_TIMEOUT = 1, /* a bounded grid/group barrier wait expired (fatal) */
  QKD_BAD_INDEX = 2,       /* an index check failed (fatal) */
  QKD_NEG_AMB = 4,         /* A-B had a negative eigenvalue (phRLR.f90:56-58 warns) */
  QKD_NEG_OMEGA = 8,       /* Casida produced a negative Omega^2 (phRLR.f90:70-74 warns) */
  QKD_QP_NOCONV = 16,      /* a Newton QP search used all maxIt steps (RGW_QP_graph.f90:78-81) */
  QKD_MBAR_TIMEOUT = 32    /* an mbarrier wait expired in a tensor-core kernel (fatal) */
};
int qk_last_device_status(const qk_ctx* ctx);
/* Grouped tridiagonalisation launches of the context's last batched call and the matrices they
 * covered (diagnostics: each launch tridiagonalises every worker's current matrix at once). */
int qk_batch_group_stats(const qk_ctx* ctx, long long* launches, long long* matrices);
/* Count of this library's kernel launches since qk_init (diagnostics). */
long long qk_launch_count(const qk_ctx* ctx);
/* Newton steps per orbital of the context's last graphical QP solve (64 = not converged). */
int qk_get_qp_iters(const qk_ctx* ctx, int* iters, int n);
/* Sigma evaluations (orbital x Newton step, all phases) of the last graphical QP solve. */
long long qk_qp_evals(const qk_ctx* ctx);
/* Release cached device workspace. */
int qk_trim(qk_ctx* ctx);
/* evGW execution mode of this context: 0 (default) enqueues every cycle from the host and reads
 * the convergence measure back after each one; 1 runs the first cycle that way and replays all
 * further cycles from one CUDA graph whose device-side loop (a conditional WHILE node) stops at
 * convergence or maxSCF, with the Newton search unrolled to its 64-step bound (finished orbitals
 * drop out on the device).  Results are the same; mode 1 removes the per-cycle host round trips. */
int qk_set_graph_mode(qk_ctx* ctx, int on);
/* Tier of the stage-level drop-ins below (qk_RGW_excitation_density, qk_RGW_self_energy_diag,
 * qk_RGW_QP_graph), which have the Fortran argument lists and so no precision argument:
 * QK_PREC_FP64 (default) or QK_PREC_BF16X3. */
int qk_set_stage_precision(qk_ctx* ctx, int precision);

/* ---- stage-level drop-ins (host pointers) ------------------------------------------------- */
/* LR/phRLR_A.f90:1-138 */
int qk_phRLR_A(qk_ctx* ctx, int ispin, int dRPA, int nBas, int nC, int nO, int nV, int nR, int nS,
               double lambda, const double* e, const double* ERI, double* Aph);
/* LR/phRLR_B.f90:1-98 */
int qk_phRLR_B(qk_ctx* ctx, int ispin, int dRPA, int nBas, int nC, int nO, int nV, int nR, int nS,
               double lambda, const double* ERI, double* Bph);
/* LR/phRLR.f90:1-97 (TDA must be 0) */
int qk_phRLR(qk_ctx* ctx, int TDA, int nS, const double* Aph, const double* Bph,
             double* EcRPA, double* Om, double* XpY, double* XmY);
/* GW/RGW_excitation_density.f90:1-80 */
int qk_RGW_excitation_density(qk_ctx* ctx, int nOrb, int nC, int nO, int nR, int nS,
                              const double* ERI, const double* XpY, double* rho);
/* GW/RGW_self_energy_diag.f90:1-113 */
int qk_RGW_self_energy_diag(qk_ctx* ctx, double eta, int nBas, int nOrb, int nC, int nO, int nV,
                            int nR, int nS, const double* e, const double* Om, const double* rho,
                            double* EcGM, double* Sig, double* Z);
/* GW/RGW_SRG_self_energy_diag.f90:1-160 */
/* GW/RGW_self_energy.f90:1-161 and GW/RGW_SRG_self_energy.f90:1-170: the full (unsymmetrised)
 * correlation self-energy SigC(nOrb,nOrb) (zero outside the active block), Z and EcGM.  FP64. */
int qk_RGW_self_energy(qk_ctx* ctx, double eta, int nBas, int nOrb, int nC, int nO, int nV,
                       int nR, int nS, const double* e, const double* Om, const double* rho,
                       double* EcGM, double* SigC, double* Z);
int qk_RGW_SRG_self_energy(qk_ctx* ctx, double flow, int nBas, int nOrb, int nC, int nO, int nV,
                           int nR, int nS, const double* e, const double* Om, const double* rho,
                           double* EcGM, double* SigC, double* Z);
/* AOtoMO/Hartree_matrix_AO_basis.f90:1-34 and AOtoMO/exchange_matrix_AO_basis.f90:1-34:
 * H(mu,nu) = sum P(la,si) ERI(mu,la,nu,si), K(mu,nu) = -sum P(la,si) ERI(mu,la,si,nu). */
int qk_Hartree_matrix_AO_basis(qk_ctx* ctx, int nBas, const double* P, const double* ERI,
                               double* H);
int qk_exchange_matrix_AO_basis(qk_ctx* ctx, int nBas, const double* P, const double* ERI,
                                double* K);
int qk_RGW_SRG_self_energy_diag(qk_ctx* ctx, double flow, int nBas, int nOrb, int nC, int nO,
                                int nV, int nR, int nS, const double* e, const double* Om,
                                const double* rho, double* EcGM, double* SigC, double* Z);
/* GW/RGW_QP_graph.f90:1-97 (+ RGW_Re_SigC / RGW_Re_dSigC and their SRG twins).
 * Z is in/out: orbitals whose Newton search fails keep their Z, as in the reference. */
int qk_RGW_QP_graph(qk_ctx* ctx, int doSRG, double eta, double flow, int nBas, int nC, int nO,
                    int nV, int nR, int nS, const double* eHF, const double* Om, const double* rho,
                    const double* eGWlin, const double* eOld, double* eGW, double* Z);
/* ---- integrals from the reference's files into device memory --------------------------------
 * qk_read_eri_bin: int/ERI.bin (utils/read_2e_integrals.f90:55-63; nBas^4 doubles, <pq|rs> in
 *   the column-major layout every ERI argument here takes) streamed into d_ERI through two
 *   pinned staging buffers, reading overlapped with the copies.
 * qk_read_eri_chem_bin: int/ERI_chem.bin (read_2e_integrals.f90:85-107; the 8-fold symmetric
 *   chemist integrals, pair(i,j) = i(i+1)/2 + j for i >= j, nested once more over the pairs, as
 *   AOtoMO/Hartree_matrix_AO_basis.f90:71-93 indexes them) streamed to the device and expanded
 *   into the full <pq|rs> tensor d_ERI (nBas^4).
 * qk_unpack_eri_s8_dev: that expansion alone, from a packed array already on the device.
 * qk_AOtoMO_ERI_RHF_dev: the AO->MO transform of qk_AOtoMO_ERI_RHF on device buffers (d_ERI_AO
 *   is left unchanged). */
int qk_read_eri_bin(qk_ctx* ctx, const char* path, int nBas, double* d_ERI);
int qk_read_eri_chem_bin(qk_ctx* ctx, const char* path, int nBas, double* d_ERI);
int qk_unpack_eri_s8_dev(qk_ctx* ctx, int nBas, const double* d_packed, double* d_ERI);
int qk_AOtoMO_ERI_RHF_dev(qk_ctx* ctx, int nBas, int nOrb, const double* d_c,
                          const double* d_ERI_AO, double* d_ERI_MO);

/* AOtoMO/AOtoMO_ERI_RHF.f90:1-55 */
int qk_AOtoMO_ERI_RHF(qk_ctx* ctx, int nBas, int nOrb, const double* c, const double* ERI_AO,
                      double* ERI_MO);
/* utils/DIIS_extrapolation.f90:1-61: error/e are (n,max_diis) histories, updated in place;
 * n_diis is the history length after this call's increment. */
int qk_DIIS_extrapolation(qk_ctx* ctx, double* rcond, int n_err, int n_e, int n_diis,
                          double* error, double* e, const double* error_in, double* e_inout);

/* ---- driver-level (host pointers) --------------------------------------------------------- */
/* ERI(nOrb,nOrb,nOrb,nOrb) is the full MO tensor as in the reference, but the drivers read (and
 * copy to the device) only the entries ERI(p,j,q,b) with j active occupied and b active virtual
 * (the excitation-density slab, which contains the Casida block): nO*nV/nOrb^2 of it. */
/* GW/RG0W0.f90:109-233.  Om receives the screening (first Casida) energies; EcRPA the
 * correlation energy of the second Casida at eGW (the dumped "G0W0 correlation energy"). */
int qk_RG0W0(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
             int nR, int nS, const double* eHF, const double* ERI, double* eGW, double* SigC,
             double* Z, double* Om, double* EcRPA, double* EcGM);
/* GW/evRGW.f90:110-198.  Returns QK_ERR_NO_CONV (results still written) when maxSCF is hit. */
int qk_evRGW(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
             int nR, int nS, const double* eHF, const double* ERI, double* eGW, double* SigC,
             double* Z, double* EcRPA, double* EcGM, int* nSCF, double* Conv);

/* ---- driver-level (device pointers; inputs resident in HBM) ------------------------------- */
int qk_RG0W0_dev(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
                 int nR, int nS, const double* d_eHF, const double* d_ERI, double* d_eGW,
                 double* d_SigC, double* d_Z, double* d_Om, double* EcRPA, double* EcGM);
int qk_evRGW_dev(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
                 int nR, int nS, const double* d_eHF, const double* d_ERI, double* d_eGW,
                 double* d_SigC, double* d_Z, double* EcRPA, double* EcGM, int* nSCF,
                 double* Conv);

/* ---- quasiparticle self-consistent GW (GW/qsRGW.f90:193-359) -------------------------------
 * Replaces the call qsRGW(...) of GW/RGW.f90:116-124, without the linearised density-matrix
 * correction (do_linDM_GW), the dipoles and the post-processing BSE.  nBas >= nOrb: with
 * nOrb < nBas F is projected through c and Fp = c^T F c, as the reference does (qsRGW.f90:281-284,
 * 328-333).  AO inputs: S, T, V, Hc = T + V (nBas^2), X (nBas x nOrb; Fp = X^T F X when nBas = nOrb),
 * cHF (nBas x nOrb), PHF (nBas^2), ERI_AO(nBas^4) = <mu nu|la si>
 * (physicist layout, 8-fold permutational symmetry of real integrals assumed), and the RHF
 * start eHF, cHF, PHF.  prm: eta, doSRG, TDA_W, maxSCF, thresh, max_diis (<= 32) and
 * precision are read.  Outputs: eGW, c, P, SigC = c^T SigCp c (MO basis), Z of the last cycle;
 * EqsGW = ET + EV + EJ + EK (electronic, without ENuc), EcRPA, EcGM of the last cycle, nSCF,
 * Conv.  c, P, SigC and Z may be NULL in the host-pointer form (SigC in both).  Returns
 * QK_ERR_NO_CONV (results written) when nSCF reaches maxSCF, as the reference stops there. */
int qk_qsRGW(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
             int nR, int nS, const double* eHF, const double* cHF, const double* PHF,
             const double* S, const double* T, const double* V, const double* Hc, const double* X,
             const double* ERI_AO, double* eGW, double* c, double* P, double* SigC, double* Z,
             double* EqsGW, double* EcRPA, double* EcGM, int* nSCF, double* Conv);
int qk_qsRGW_dev(qk_ctx* ctx, const qk_gw_params* prm, int nBas, int nOrb, int nC, int nO, int nV,
                 int nR, int nS, const double* d_eHF, const double* d_cHF, const double* d_PHF,
                 const double* d_S, const double* d_T, const double* d_V, const double* d_Hc,
                 const double* d_X, const double* d_ERI_AO, double* d_eGW, double* d_c,
                 double* d_P, double* d_SigC, double* d_Z, double* EqsGW, double* EcRPA,
                 double* EcGM, int* nSCF, double* Conv);

/* ---- factorised-integral drivers (device pointers) ---------------------------------------
 * (pq|rs) = sum_P L(p,q,P) L(r,s,P) with L(nOrb,nOrb,naux) column-major (symmetric in p,q).
 * The slab (pq|jb) and the Casida coupling (ia|jb) are built on the device from L (in the
 * precision tier of prm->precision); everything else is the RG0W0 / evRGW path above.  No
 * counterpart in the reference, which reads the full nOrb^4 tensor; these variants avoid it
 * for large or many systems. */
int qk_RG0W0_L_dev(qk_ctx* ctx, const qk_gw_params* prm, int nOrb, int nC, int nO, int nR,
                   int naux, const double* d_L, const double* d_eHF, double* d_eGW, double* d_SigC,
                   double* d_Z, double* d_Om, double* EcRPA, double* EcGM);
int qk_evRGW_L_dev(qk_ctx* ctx, const qk_gw_params* prm, int nOrb, int nC, int nO, int nR,
                   int naux, const double* d_L, const double* d_eHF, double* d_eGW, double* d_SigC,
                   double* d_Z, double* EcRPA, double* EcGM, int* nSCF, double* Conv);

/* ---- learned quasiparticle guess ----------------------------------------------------------
 * No counterpart in the reference.  A 16 -> 64 -> 64 -> 1 SiLU perceptron predicts the nonlinear
 * part eGW_p - eGWlin_p of the QP shift from 16 per-orbital features of the linearised G0W0 stage
 * (energies, Sigma, Z, and one pole sweep at eGWlin: the Newton and Halley steps from there and
 * the nearest pole); the Newton search then starts at eGWlin_p + prediction.  It is trained on the
 * GPU (FP32, Adam) by this library's own kernels and evaluated in BF16.  Parameters are one flat
 * float vector of QK_MLP_NPARAM entries: W1 (64x16, row-major), b1, W2 (64x64), b2, W3 (1x64), b3.
 * Inputs/targets of train/grad/predict are already normalised; qk_mlp_set_scaling records the
 * normalisation the drivers apply to raw features and predicted shifts. */
#define QK_MLP_NIN 16
#define QK_MLP_NH 64
#define QK_MLP_NPARAM (QK_MLP_NH * QK_MLP_NIN + QK_MLP_NH + QK_MLP_NH * QK_MLP_NH + QK_MLP_NH + QK_MLP_NH + 1)
typedef struct qk_mlp qk_mlp;
int qk_mlp_create(qk_ctx* ctx, unsigned long long seed, qk_mlp** mlp);
int qk_mlp_free(qk_mlp* mlp);
int qk_mlp_params(qk_ctx* ctx, qk_mlp* mlp, float* host_params, int set);
int qk_mlp_set_scaling(qk_mlp* mlp, const float* xmean, const float* xstd, float ymean, float ystd);
int qk_mlp_grad_dev(qk_ctx* ctx, qk_mlp* mlp, int n, const float* d_X, const float* d_T,
                    float* d_grad, float* loss);
int qk_mlp_train_dev(qk_ctx* ctx, qk_mlp* mlp, int n, const float* d_X, const float* d_T,
                     int epochs, int batch, float lr, float* final_loss);
int qk_mlp_predict_dev(qk_ctx* ctx, qk_mlp* mlp, int n, const float* d_X, float* d_Y, int bf16);
/* Attach a model to the context (used when prm->qp_guess = 1); NULL detaches. */
int qk_set_qp_model(qk_ctx* ctx, qk_mlp* mlp);
/* Capture the 16 raw features per orbital of each subsequent G0W0 driver call (on/off) and read
 * the last captured set (N x 16, row-major, host). */
int qk_set_feature_capture(qk_ctx* ctx, int on);
int qk_get_features(const qk_ctx* ctx, float* host, int n);

/* ---- batched drivers (device pointers) ------------------------------------------------------
 * Many independent systems of uneven size in one call (no counterpart in the reference, which
 * runs one molecule per process).  Per system i, desc[i] gives its sizes and the element offsets
 * of its factor L(nOrb,nOrb,naux) in d_L and of its energies in d_eHF / d_eGW.  method 0 = G0W0,
 * 1 = evGW.  The systems are spread over n_workers CUDA streams (one host thread each), largest
 * first.  Per-system results: status[i] (QK_OK, QK_ERR_NO_CONV, ...), EcRPA[i], nSCF[i] (host
 * arrays); a failing system does not stop the others.  Returns the worst status other than
 * QK_ERR_NO_CONV.  The context's tuned launch parameters and attached QP model (qk_set_qp_model,
 * for prm->qp_guess = 1) apply to every system. */
typedef struct qk_sys_desc {
  int nOrb, nC, nO, nR, naux;
  long long offset_L;
  long long offset_e;
} qk_sys_desc;
int qk_gw_batch_L_dev(qk_ctx* ctx, const qk_gw_params* prm, int method, int nsys,
                      const qk_sys_desc* desc, const double* d_L, const double* d_eHF,
                      double* d_eGW, double* EcRPA, int* status, int* nSCF, int n_workers);

/* ---- dense symmetric eigensolver (device pointers; replaces dsyev('V','U') of
 *      utils/wrap_lapack.f90:99-136 on the GPU).  A (n x n, lda) is symmetric and only its
 *      lower triangle is referenced (dsyev('V','U') reads the upper one: the same numbers for
 *      a symmetric matrix); A is destroyed; w ascending;
 *      if want_vectors, Zt receives the eigenvectors as ROWS: Zt[j + n*i] = component i of
 *      eigenvector j. ------------------------------------------------------------------------ */
int qk_dsyev_dev(qk_ctx* ctx, int n, double* d_A, int lda, double* d_w, double* d_Zt,
                 int want_vectors);

/* ---- Bethe-Salpeter excitation energies on top of GW (GW/RGW_phBSE.f90) -------------------
 * qk_RGW_phBSE: static phBSE@GW -- the dRPA singlet screening at the energies eW (the G0W0 caller
 *   passes eHF, GW/RG0W0.f90:241-242), its static kernels KA/KB
 *   (GW/RGW_phBSE_static_kernel_A/B.f90), and per spin the Casida problem of
 *   A = phRLR_A(ispin, dRPA = false, eGW) + KA, B = phRLR_B + KB (full, or TDA).  Outputs the
 *   correlation energies EcBSE[2] (singlet, 3 x triplet; halved with exchange_kernel, :183-187)
 *   and the excitation energies of the manifolds asked for (OmBSE_* of length nS, or NULL).
 *   The second-order kernel (dophBSE2), the dynamical correction (dBSE) and the transition
 *   dipoles are not computed.  All arithmetic FP64.  ERI is the full ERI(nOrb,nOrb,nOrb,nOrb). */
typedef struct {
  int TDA_W;            /* Tamm-Dancoff screening */
  int TDA;              /* Tamm-Dancoff BSE */
  int singlet;          /* compute the singlet manifold */
  int triplet;          /* compute the triplet manifold */
  int exchange_kernel;  /* halve EcBSE (RGW_phBSE.f90:186-187) */
  double eta;           /* the GW broadening of the static kernels */
} qk_bse_params;

/* GW/RGW_phACFDT.f90:1-219 (the doACFDT branch of RG0W0.f90:259-261): adiabatic-connection
 * correlation energy of phBSE@GW, EcAC[2] = (singlet, triplet), by the 21-point Gauss-Legendre
 * lambda quadrature of RPA/phACFDT_correlation_energy.f90; doXBS rebuilds the screening at
 * every lambda.  prm: TDA_W, TDA, singlet, triplet, exchange_kernel, eta. */
int qk_RGW_phACFDT(qk_ctx* ctx, const qk_bse_params* prm, int doXBS, int nBas, int nOrb, int nC,
                   int nO, int nV, int nR, int nS, const double* ERI, const double* eW,
                   const double* eGW, double* EcAC);
int qk_RGW_phACFDT_dev(qk_ctx* ctx, const qk_bse_params* prm, int doXBS, int nOrb, int nC, int nO,
                       int nR, const double* d_ERI, const double* d_eW, const double* d_eGW,
                       double* EcAC);
int qk_RGW_phBSE(qk_ctx* ctx, const qk_bse_params* prm, int nBas, int nOrb, int nC, int nO,
                 int nV, int nR, int nS, const double* ERI, const double* eW, const double* eGW,
                 double* EcBSE, double* OmBSE_singlet, double* OmBSE_triplet);
int qk_RGW_phBSE_dev(qk_ctx* ctx, const qk_bse_params* prm, int nOrb, int nC, int nO, int nR,
                     const double* d_ERI, const double* d_eW, const double* d_eGW, double* EcBSE,
                     double* d_OmBSE_singlet, double* d_OmBSE_triplet);

/* ---- dRPA correlation energy by frequency quadrature (device pointers) ---------------------
 * qk_RPA_ecorr_quad_dev: EcRPA = (sum Omega - tr A)/2 of the singlet dRPA problem at orbital
 *   energies d_e (the quantity phRLR returns, LR/phRLR.f90) without the nS x nS eigenproblem:
 *   EcRPA = 1/(2 pi) int_0^inf [ln det(1 + Q(w)) - tr Q(w)] dw, Q(w) = 4 L^T diag(d/(d^2+w^2)) L
 *   for a factor (ia|jb) = L L^T -- the pivoted Cholesky of the (ia|jb) block of d_ERI
 *   (ERI(nOrb,nOrb,nOrb,nOrb), the block ERI(b,i,j,a) is read), or d_L (L(nOrb,nOrb,naux)); pass
 *   exactly one.  24-128 Gauss-Legendre points by the width of the e_a - e_i spectrum;
 *   Q with compensated FP32 products, ln det by FP64 Cholesky; agrees with the eigenvalue
 *   route to ~1e-8 Ha.  A negative e_a - e_i gives NaN (as the Casida square roots do) and the
 *   QKD_NEG_AMB status.  *applied = 0 (EcRPA untouched) when it does not apply: a zero
 *   e_a - e_i, d_max/d_min > 60000, or a numerical rank of (ia|jb) above nS/3.  The mixed tier
 *   of qk_RG0W0 / qk_RG0W0_L_dev uses it for the EcRPA at the G0W0 energies.
 * qk_gauss_legendre: the quadrature's nodes x (ascending) and weights w on [-1, 1], host only. */
int qk_RPA_ecorr_quad_dev(qk_ctx* ctx, int nOrb, int nC, int nO, int nR, int naux,
                          const double* d_e, const double* d_ERI, const double* d_L,
                          double* EcRPA, int* applied);
int qk_gauss_legendre(int n, double* x, double* w);

/* ---- contraction kernels on device buffers (column-major) --------------------------------
 * qk_dgemm_dev: C = alpha*op(A)*op(B) + beta*C in FP64 (DFMA, or DMMA where tuned); replaces the
 *   dgemm calls of AOtoMO/AOtoMO_ERI_RHF.f90:26-53 and GW/RGW_excitation_density.f90:48-50.
 * qk_dgemm_f32p_dev: the same contract with FP64 operands and result but FP32 products (the
 *   16 products of each k tile summed in FP32, the tiles folded into a compensated FP32 pair);
 *   the mixed tier's eigenvector back-transformation (dsyev's dormtr step).
 * qk_dgemm_df_dev: the same contract in double-float: operands staged as FP32 pairs, products
 *   exact by TwoProduct, sums by TwoSum (~1e-13 of sum |a_ik b_kj| whatever the cancellation, on
 *   the FP32 pipe); the mixed tier's quarter transforms and full self-energy in qsGW.
 * qk_gemm_bf16x3_dev: C = A * B^T with the three-way BF16 split on tcgen05 (FP32 accumulate),
 *   the precision tier of the same excitation-density dgemm.
 * qk_gemm_bf16x3_ex_dev: the qk_dgemm_dev contract (transposes, alpha, beta) on the same tensor-core
 *   path; few output tiles with a long k split k over CTAs.  The mixed tier's back-transformation
 *   and quadrature products use it. */
int qk_dgemm_dev(qk_ctx* ctx, char transa, char transb, int m, int n, int k, double alpha,
                 const double* d_A, int lda, const double* d_B, int ldb, double beta, double* d_C,
                 int ldc);
int qk_dgemm_f32p_dev(qk_ctx* ctx, char transa, char transb, int m, int n, int k, double alpha,
                      const double* d_A, int lda, const double* d_B, int ldb, double beta,
                      double* d_C, int ldc);
int qk_dgemm_df_dev(qk_ctx* ctx, char transa, char transb, int m, int n, int k, double alpha,
                    const double* d_A, int lda, const double* d_B, int ldb, double beta,
                    double* d_C, int ldc);
int qk_gemm_bf16x3_dev(qk_ctx* ctx, int m, int n, int k, const double* d_A, int lda,
                       const double* d_B, int ldb, double* d_C, int ldc);
int qk_gemm_bf16x3_ex_dev(qk_ctx* ctx, char transa, char transb, int m, int n, int k,
                          double alpha, const double* d_A, int lda, const double* d_B, int ldb,
                          double beta, double* d_C, int ldc);

/* ---- allocation-free self-energy (device pointers) -----------------------------------------
 * No counterpart in the reference.  For hosts that own all device memory themselves (one
 * preallocated pool, a hard memory budget, or an allocation-free hot loop such as a Fortran-driven
 * evGW cycle) and therefore cannot let the library call cudaMalloc: computes the same Sig, Z and
 * EcGM as qk_RGW_self_energy_diag (GW/RGW_self_energy_diag.f90) from caller-owned device buffers
 * e(nBas), Om(nS), rho(nBas,nBas,nS) into Sig(nBas), Z(nBas), EcGM(1), enqueued on `stream`
 * (a cudaStream_t, 0 = default stream) and synchronised before returning (so the call cannot be
 * captured into a CUDA graph).  It needs no qk_ctx and
 * calls no cudaMalloc/cudaFree.  Scratch is a static 3 MiB device array, so nBas <= 1024
 * (QK_ERR_ARG beyond that).  QuAcK's counts are checked: nV = nBas - nO (frozen virtuals
 * included) and nO <= nOrb <= nBas, else QK_ERR_ARG.  Each call resolves the array's device
 * address on the current device (no allocation), so it stays valid across cudaDeviceReset.
 * Calls share the array: calls that overlap on the GPU race and must be serialised by the
 * caller. */
int qk_RGW_self_energy_diag_noalloc_dev(double eta, int nBas, int nOrb, int nC, int nO, int nV,
                                        int nR, int nS, const double* d_e, const double* d_Om,
                                        const double* d_rho, double* d_EcGM, double* d_Sig,
                                        double* d_Z, void* stream);

/* ---- autotuner ------------------------------------------------------------------------------
 * No counterpart in the reference.  Runtime launch parameters of this library's kernels, tuned
 * per size bucket floor(log2(size)): "bf16x3_chunk" (k blocks per TMEM chunk of the BF16x3 GEMM,
 * size = K), "splitk_mult" (split-K target CTAs per SM of the DMMA GEMM, size = K),
 * "sigma_chunks" (m chunks of the pole sweeps per SM, size = nS), "sytrd_grid" (quarters of the
 * SMs in the cooperative tridiagonalisation, size = n), "dgemm_path" (1 DFMA, 2 DMMA, size = m n),
 * "stebz_k" (lanes per eigenvalue in the bisection, size = n), "qp_persist" (mixed-tier Newton:
 * 1 persistent kernel, 2 per-step sweeps, size = nS).  qk_autotune times all candidates on
 * problems of the given sizes (allocates temporary buffers) and keeps the fastest; the table
 * can be saved to / loaded from a JSON file.
 * Two context-wide settings share qk_tune_set (size ignored): "newton_maxit" (steps of the
 * graphical QP solve, 1..4096, default 64 = maxIt of RGW_QP_graph.f90:38; a search that uses all
 * of them keeps eGWlin, :78-81) and "spin_limit" (polls of every bounded grid-barrier wait before
 * it gives up and reports QKD_BARRIER_TIMEOUT, QK_ERR_DEVICE from the call; 0 = the built-in
 * limit of about a second) and "fail_alloc" (n > 0: the n-th next workspace allocation that
 * would call cudaMalloc fails instead, with QK_ERR_NOMEM; 0 disarms) -- hooks for the
 * failure-path tests -- and "guess_gate" (learned-guess start rule: 0 where the model agrees with
 * the Halley step from eGWlin, 1 the model's prediction everywhere, 2 the Halley step
 * everywhere; results are the reference start's in every case) and "dsyev_df" (1: qk_dsyev_dev
 * tridiagonalises in double-float arithmetic on the FP32 pipe, as the mixed tier's Casida solve
 * does; 0, the default, in FP64). */
int qk_autotune(qk_ctx* ctx, int nOrb, int nS, int flags);
int qk_tune_set(qk_ctx* ctx, const char* name, long long size, int value);
int qk_tune_query(const qk_ctx* ctx, const char* name, long long size);
int qk_tune_save(const qk_ctx* ctx, const char* path);
int qk_tune_load(qk_ctx* ctx, const char* path);

/* ---- diagnostics ------------------------------------------------------------------------- */
/* The cudaStream_t (as void*) on which the context enqueues all of its kernels. */
void* qk_stream(const qk_ctx* ctx);
/* Measured FP64 peak of this GPU: back-to-back DMMA (mma.sync.m8n8k4.f64) and DFMA in registers,
 * TFLOP/s. */
int qk_probe_fp64_peak(qk_ctx* ctx, double* tflops_dmma, double* tflops_dfma);
/* Measured FP32 FMA peak of this GPU (back-to-back FFMA in registers), TFLOP/s: the roofline of
 * the mixed tier's FP32-product stages. */
int qk_probe_fp32_peak(qk_ctx* ctx, double* tflops_ffma);

#ifdef __cplusplus
}
#endif
#endif /* QKGW_H */
