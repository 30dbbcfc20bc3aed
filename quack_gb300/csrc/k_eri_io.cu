// k_eri_io.cu -- two-electron integrals from the reference's files straight into device memory.
//
// int/ERI.bin (utils/read_2e_integrals.f90:55-63): nBas^4 doubles, an unformatted stream that
// Fortran reads as G(nBas,nBas,nBas,nBas) = <pq|rs> -- the same column-major layout as the
// library's ERI argument, so the bytes go to the device unchanged.
// int/ERI_chem.bin (read_2e_integrals.f90:85-107, read by HF/RHF_hpc.f90:107-110): the 8-fold
// symmetric chemist integrals (pq|rs), one per pair of index pairs: pair(i,j) = i(i+1)/2 + j for
// i >= j (0-based) and position pair(P,Q) again for P >= Q -- the indexing of
// AOtoMO/Hartree_matrix_AO_basis.f90:71-93; nBas(nBas+1)/2 (that + 1)/2 doubles.  A kernel
// expands it into the physicist tensor <pq|rs> = (pr|qs).
//
// The files are read in chunks into two pinned host buffers so that reading one chunk overlaps
// the host-to-device copy of the previous one.
#include <cstdio>
#include <string>
#include "qk_internal.cuh"

namespace {

constexpr size_t CHUNK = (size_t)32 << 20;  // bytes per pinned staging buffer

__device__ __forceinline__ long long pair_index(long long i, long long j) {
  return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i;
}

// ERI(p,q,r,s) = <pq|rs> = (pr|qs) = packed[pair(pair(p,r), pair(q,s))]
__global__ void k_unpack_s8(int N, const double* __restrict__ packed, double* __restrict__ ERI) {
  const long long N1 = N, total = N1 * N1 * N1 * N1;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
       idx += (long long)gridDim.x * blockDim.x) {
    long long t = idx;
    const long long p = t % N1;
    t /= N1;
    const long long q = t % N1;
    t /= N1;
    const long long r = t % N1;
    const long long s = t / N1;
    ERI[idx] = packed[pair_index(pair_index(p, r), pair_index(q, s))];
  }
}

// read `bytes` from the file into device memory at d, double-buffered through pinned memory
int stream_file_to_device(qk_ctx* ctx, const char* path, size_t bytes, void* d) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return qk_fail(ctx, QK_ERR_ARG, "cannot open %s", path);
  void* hb[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int rc = QK_OK;
  for (int i = 0; i < 2 && rc == QK_OK; ++i) {
    if (cudaHostAlloc(&hb[i], CHUNK, cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) != cudaSuccess)
      rc = qk_fail(ctx, QK_ERR_NOMEM, "pinned staging buffers");
  }
  size_t off = 0;
  int k = 0;
  while (rc == QK_OK && off < bytes) {
    const int b = k & 1;
    if (k >= 2 && cudaEventSynchronize(ev[b]) != cudaSuccess) {  // its previous copy is done
      rc = qk_fail(ctx, QK_ERR_CUDA, "staging copy failed");
      break;
    }
    const size_t n = bytes - off < CHUNK ? bytes - off : CHUNK;
    if (std::fread(hb[b], 1, n, f) != n) {
      rc = qk_fail(ctx, QK_ERR_ARG, "%s holds fewer than %zu bytes", path, bytes);
      break;
    }
    if (cudaMemcpyAsync((char*)d + off, hb[b], n, cudaMemcpyHostToDevice, ctx->stream) !=
            cudaSuccess ||
        cudaEventRecord(ev[b], ctx->stream) != cudaSuccess) {
      rc = qk_fail(ctx, QK_ERR_CUDA, "host-to-device copy failed");
      break;
    }
    off += n;
    ++k;
  }
  std::fclose(f);
  cudaStreamSynchronize(ctx->stream);
  for (int i = 0; i < 2; ++i) {
    if (ev[i]) cudaEventDestroy(ev[i]);
    if (hb[i]) cudaFreeHost(hb[i]);
  }
  return rc;
}

}  // namespace

extern "C" {

int qk_unpack_eri_s8_dev(qk_ctx* ctx, int nBas, const double* d_packed, double* d_ERI) {
  if (!ctx || nBas <= 0 || !d_packed || !d_ERI) return QK_ERR_ARG;
  cudaSetDevice(ctx->device);
  QK_TRY(qk_order_after_default(ctx));
  QK_TRY(qk_status_reset(ctx));
  const long long N = nBas, total = N * N * N * N;
  long long blocks = (total + 255) / 256;
  if (blocks > 64LL * ctx->num_sms) blocks = 64LL * ctx->num_sms;
  k_unpack_s8<<<(int)blocks, 256, 0, ctx->stream>>>(nBas, d_packed, d_ERI);
  QK_LAUNCHED();
  QK_CK(cudaStreamSynchronize(ctx->stream));
  return QK_OK;
}

int qk_read_eri_bin(qk_ctx* ctx, const char* path, int nBas, double* d_ERI) {
  if (!ctx || !path || nBas <= 0 || !d_ERI) return QK_ERR_ARG;
  cudaSetDevice(ctx->device);
  ctx->err.clear();
  QK_TRY(qk_order_after_default(ctx));
  const size_t N = nBas;
  return stream_file_to_device(ctx, path, N * N * N * N * sizeof(double), d_ERI);
}

int qk_read_eri_chem_bin(qk_ctx* ctx, const char* path, int nBas, double* d_ERI) {
  if (!ctx || !path || nBas <= 0 || !d_ERI) return QK_ERR_ARG;
  cudaSetDevice(ctx->device);
  ctx->err.clear();
  QK_TRY(qk_order_after_default(ctx));
  const size_t N = nBas, npair = N * (N + 1) / 2, nq = npair * (npair + 1) / 2;
  double* packed = nullptr;
  QK_TRY(qk_wst(ctx, W_ERIPACK, nq, &packed));
  QK_TRY(stream_file_to_device(ctx, path, nq * sizeof(double), packed));
  return qk_unpack_eri_s8_dev(ctx, nBas, packed, d_ERI);
}

}  // extern "C"
