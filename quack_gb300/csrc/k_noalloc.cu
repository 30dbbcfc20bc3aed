// k_noalloc.cu -- the diagonal GW self-energy without any device allocation.
//
// Who needs this: Fortran/C hosts that own all device memory themselves -- a code that carves
// every buffer out of one preallocated pool, runs under a hard device-memory budget, or drives
// a hot loop (e.g. the evGW cycle) in which the library must not allocate behind its back.
// Such callers cannot let the library call cudaMalloc, so they cannot use the context-based
// entry points (whose workspace is allocated on first use).  This entry point takes only
// caller-owned device buffers and a stream and allocates nothing.
//
// Its only scratch (the per-chunk partial sums of the pole sweep) is the file-scope array
// below: QK_NOALLOC_SCRATCH_DOUBLES doubles (3 MiB), resident on every GPU that loads the
// library until the process exits.  Limits that follow from it: nBas <= 1024 orbitals, and
// at most 128 excitation chunks (chosen internally).
//
// Set-up: every call looks up the array's device address with cudaGetSymbolAddress on the
// device that is current at the call (a host-side lookup that allocates nothing), so the address
// stays right after cudaDeviceReset or a context change.  All calls share the one array and it
// keeps the last call's contents, so calls whose kernels overlap on the GPU (different streams
// or host threads on one device) race with each other; serialise them.
#include "qk_internal.cuh"

#define QK_NOALLOC_MAX_N 1024
#define QK_NOALLOC_MAX_CHUNKS 128
#define QK_NOALLOC_SCRATCH_DOUBLES (3 * QK_NOALLOC_MAX_CHUNKS * QK_NOALLOC_MAX_N)

static __device__ __align__(256) double qk_noalloc_scratch[QK_NOALLOC_SCRATCH_DOUBLES];

namespace {

constexpr int NA_WARPS = 8;

// same pole sums as RGW_self_energy_diag.f90:44-84 (one thread per orbital p, warps split m),
// partials per (m chunk, p) written to part[chunk*N + p] (+ stride for dSig and the occupied part)
__global__ void __launch_bounds__(NA_WARPS * 32)
    k_sigma_partial_noalloc(int N, int nC, int nO, int nR, int nS, int nchunks, int mper, double eta,
                            const double* __restrict__ e, const double* __restrict__ Om,
                            const double* __restrict__ rho, double* __restrict__ part) {
  extern __shared__ double se[];
  __shared__ double s0[NA_WARPS][32], s1[NA_WARPS][32], s2[NA_WARPS][32];
  for (int i = threadIdx.x; i < N; i += blockDim.x) se[i] = e[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int p = nC + blockIdx.x * 32 + lane;
  const int pend = N - nR;
  __syncthreads();
  double sig = 0.0, ds = 0.0, so = 0.0;
  if (p < pend) {
    const double w = se[p], eta2 = eta * eta;
    const long long N1 = N, N2 = N1 * N1;
    const int m0 = blockIdx.y * mper, m1 = min(nS, m0 + mper);
    for (int m = m0 + warp; m < m1; m += NA_WARPS) {
      const double om = Om[m];
      const double* r = rho + p + N2 * m;
      for (int q = nC; q < nO; ++q) {
        const double x = r[N1 * q], num = 2.0 * x * x, eps = w - se[q] + om;
        const double e2 = eps * eps, rr = 1.0 / (e2 + eta2);
        so += num * eps * rr;
        ds -= num * (e2 - eta2) * rr * rr;
      }
      for (int q = nO; q < pend; ++q) {
        const double x = r[N1 * q], num = 2.0 * x * x, eps = w - se[q] - om;
        const double e2 = eps * eps, rr = 1.0 / (e2 + eta2);
        sig += num * eps * rr;
        ds -= num * (e2 - eta2) * rr * rr;
      }
    }
    sig += so;
  }
  s0[warp][lane] = sig;
  s1[warp][lane] = ds;
  s2[warp][lane] = so;
  __syncthreads();
  if (warp == 0 && p < pend) {
    double a = 0.0, b = 0.0, c = 0.0;
    for (int w = 0; w < NA_WARPS; ++w) { a += s0[w][lane]; b += s1[w][lane]; c += s2[w][lane]; }
    const size_t o = (size_t)blockIdx.y * N + p, stride = (size_t)nchunks * N;
    part[o] = a;
    part[o + stride] = b;
    part[o + 2 * stride] = c;
  }
}

__global__ void k_sigma_final_noalloc(int N, int nC, int nO, int nR, int nchunks,
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
  if (threadIdx.x == 0) *EcGM = -2.0 * gm;
}

// device address of the scratch array on the current device (the host-side symbol is only a
// stand-in); resolved on every call, since a reset or a new context may move the module
int scratch_for_current_device(double** out) {
  void* ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, qk_noalloc_scratch) != cudaSuccess || !ptr) return QK_ERR_CUDA;
  *out = (double*)ptr;
  return QK_OK;
}

}  // namespace

extern "C" int qk_RGW_self_energy_diag_noalloc_dev(double eta, int nBas, int nOrb, int nC, int nO,
                                                   int nV, int nR, int nS, const double* d_e,
                                                   const double* d_Om, const double* d_rho,
                                                   double* d_EcGM, double* d_Sig, double* d_Z,
                                                   void* stream) {
  const int N = nBas;
  const int no = nO - nC, nv = N - nO - nR;
  if (N <= 0 || nC < 0 || nR < 0 || no <= 0 || nv <= 0 || (long long)no * nv != nS)
    return QK_ERR_ARG;
  // QuAcK's counts: nV = nBas - nO (frozen virtuals included), nO <= nOrb <= nBas
  if (nV != N - nO || nOrb < nO || nOrb > N) return QK_ERR_ARG;
  if (N > QK_NOALLOC_MAX_N) return QK_ERR_ARG;  // beyond the static scratch (nBas <= 1024)
  if (!d_e || !d_Om || !d_rho || !d_EcGM || !d_Sig || !d_Z) return QK_ERR_ARG;
  double* part = nullptr;
  int st = scratch_for_current_device(&part);
  if (st != QK_OK) return st;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return QK_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return QK_ERR_CUDA;
  const int nact = N - nR - nC;
  const int ptiles = (nact + 31) / 32;
  int nchunks = (4 * sms + ptiles - 1) / ptiles;
  const int maxch = (nS + NA_WARPS - 1) / NA_WARPS;
  if (nchunks > maxch) nchunks = maxch;
  if (nchunks > QK_NOALLOC_MAX_CHUNKS) nchunks = QK_NOALLOC_MAX_CHUNKS;
  if (nchunks < 1) nchunks = 1;
  const int mper = (nS + nchunks - 1) / nchunks;
  nchunks = (nS + mper - 1) / mper;
  cudaStream_t s = (cudaStream_t)stream;
  // the array keeps the previous call's partial sums: clear the part this call reads
  if (cudaMemsetAsync(part, 0, sizeof(double) * 3 * (size_t)nchunks * N, s) != cudaSuccess)
    return QK_ERR_CUDA;
  // launch statuses are taken from the launches themselves, so an earlier error left by the
  // caller's own work is neither reported as this call's nor cleared
  {
    int a0 = N, a1 = nC, a2 = nO, a3 = nR, a4 = nS, a5 = nchunks, a6 = mper;
    double a7 = eta;
    const double *p8 = d_e, *p9 = d_Om, *p10 = d_rho;
    double* p11 = part;
    void* args[] = {&a0, &a1, &a2, &a3, &a4, &a5, &a6, &a7, &p8, &p9, &p10, &p11};
    if (cudaLaunchKernel((const void*)k_sigma_partial_noalloc, dim3(ptiles, nchunks),
                         dim3(NA_WARPS * 32), args, N * sizeof(double), s) != cudaSuccess)
      return QK_ERR_CUDA;
  }
  {
    int a0 = N, a1 = nC, a2 = nO, a3 = nR, a4 = nchunks;
    const double* p5 = part;
    double *p6 = d_Sig, *p7 = d_Z, *p8 = d_EcGM;
    void* args[] = {&a0, &a1, &a2, &a3, &a4, &p5, &p6, &p7, &p8};
    if (cudaLaunchKernel((const void*)k_sigma_final_noalloc, dim3(1), dim3(1024), args, 0, s) !=
        cudaSuccess)
      return QK_ERR_CUDA;
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return QK_ERR_CUDA;
  return QK_OK;
}
