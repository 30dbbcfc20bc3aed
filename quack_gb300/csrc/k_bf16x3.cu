// k_bf16x3.cu -- split-precision (BF16x3) GEMM on the 5th-generation tensor cores.
//
// C(m,n) = sum_k A(m,k) B(n,k) for FP64 A (M x K, column-major) and B (N x K, column-major),
// FP64 C.  This is the precision tier for the O(N^2 nS^2) excitation-density contraction
// (GW/RGW_excitation_density.f90:48-50).
//
// Each FP64 operand is split into three BF16 parts, x = x0 + x1 + x2 with x0 = bf16(x),
// x1 = bf16(x - x0), x2 = bf16(x - x0 - x1) (the differences are exact in FP64), and the
// product keeps the six terms down to 2^-16 relative order:
//     A0B0 + A0B1 + A1B0 + A0B2 + A1B1 + A2B0,
// accumulated in FP32 in tensor memory.  Relative error per product is O(2^-24), i.e. FP32-like.
//
// Kernel shape (one 128 x 128 output tile per CTA, 128 threads):
//   warp 0 lane 0 : TMA producer, loads the 3 A parts and 3 B parts of a 64-wide k block into
//                   one pipeline stage (6 x 16 KB, 128B-swizzled K-major tiles)
//   warp 1 lane 0 : MMA issuer, 6 products x 4 k-steps of tcgen05.mma.kind::f16 (M=128,N=128,K=16)
//                   per stage, tcgen05.commit releases the stage / signals the accumulator
//   warp 2        : allocates / frees 128 TMEM columns
//   warps 0-3     : epilogue, tcgen05.ld 32x32b -> FP64 stores (each warp owns 32 TMEM lanes)
// Every mbarrier wait is bounded; on expiry the kernel records QKD_MBAR_TIMEOUT, drains its own
// copies (bounded) and frees TMEM before returning.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <mutex>
#include "qk_internal.cuh"

namespace {

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int STAGES = 2;
constexpr int TILE_BYTES = 128 * BK * 2;           // 16 KB per part tile
constexpr int STAGE_BYTES = 6 * TILE_BYTES;        // 96 KB
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024 + 256;
constexpr uint32_t MBAR_SPIN = 1u << 30;
// k blocks per TMEM accumulation chunk: a template parameter (1, 2 or 4) chosen by the autotuner
constexpr uint32_t TMEM_COLS = 512;                // two chunk accumulators + hi + lo planes
constexpr int NTHREADS = 320;                      // producer, MMA, 8 epilogue warps

__device__ __forceinline__ uint32_t su32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// bounded wait: false (and status bit) if the phase does not complete within ~2 s
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* status) {
  if (mbar_test(bar, parity)) return true;
  const uint64_t t0 = gtimer();
  for (uint32_t i = 0; i < MBAR_SPIN; ++i) {
    if (mbar_test(bar, parity)) return true;
    if ((i & 255) == 255) {
      if (gtimer() - t0 > 2000000000ull) break;
      __nanosleep(32);
    }
  }
  atomicOr(status, QKD_MBAR_TIMEOUT);
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x,
                                            int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          su32(dst)),
      "l"(map), "r"(su32(bar)), "r"(x), "r"(y)
      : "memory");
}

__device__ __forceinline__ uint64_t sdesc_sw128(const void* tile) {
  const uint32_t a = su32(tile);
  uint64_t d = 0;
  d |= (uint64_t)((a & 0x3FFFF) >> 4);      // start address
  d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                   // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                   // 128-byte swizzle
  return d;
}

__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                          uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          su32(bar))
      : "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

// instruction descriptor: D=F32, A=B=BF16, both K-major, N=128, M=128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,"
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15,%16};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
__device__ __forceinline__ void tmem_st_wait() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// the six (A part, B part) pairs, largest terms first
__device__ __constant__ int kPairA[6] = {0, 0, 1, 0, 1, 2};
__device__ __constant__ int kPairB[6] = {0, 1, 0, 2, 1, 0};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}

// error-free FP32 addition (Knuth's TwoSum): s + e == a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bp = s - a;
  e = (a - (s - bp)) + (b - bp);
}

// Launch geometry: blockIdx.x = output tile, blockIdx.y = batch entry, blockIdx.z = k slice.
struct GemmX {
  int M, N, Kpad, rowsA, rowsB;
  int a_batched, b_batched;  // operand planes per batch entry (else shared by all)
  int kb_per_slice;          // k blocks per z slice (split-K), >= the total when not split
  int n_tiles, lower;        // lower: only tiles touching the lower triangle of C
  double alpha, beta;
  double* C;
  long long ldc, sC;         // C of batch entry y at C + y * sC; slice z at C + z * sC too
};

template <int CHUNK_KB>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_gemm_bf16x3(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                  GemmX g, int* status) {
  const int M = g.M, N = g.N, rowsA = g.rowsA, rowsB = g.rowsB;
  const int tile0 = blockIdx.x;
  const int m_tile0 = tile0 / g.n_tiles, n_tile0 = tile0 - m_tile0 * g.n_tiles;
  if (g.lower && (m_tile0 + 1) * BM <= n_tile0 * BN) return;  // strictly above the diagonal
  const int kb_first = (int)blockIdx.z * g.kb_per_slice;
  const int num_kb_all = g.Kpad / BK;
  const int num_kb = min(g.kb_per_slice, num_kb_all - kb_first);
  if (num_kb <= 0) return;
  const int rowA0 = g.a_batched ? (int)blockIdx.y * 3 * rowsA : 0;
  const int rowB0 = g.b_batched ? (int)blockIdx.y * 3 * rowsB : 0;
  double* __restrict__ C = g.C + (long long)(blockIdx.y + blockIdx.z) * g.sC;
  const long long ldc = g.ldc;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = (uint64_t*)(smem + STAGES * STAGE_BYTES);
  uint64_t* empty = full + STAGES;
  uint64_t* acc_full = empty + STAGES;   // [2] chunk finished by the tensor cores
  uint64_t* acc_empty = acc_full + 2;    // [2] chunk drained by the epilogue warps
  uint32_t* tmem_slot = (uint32_t*)(acc_empty + 2);
  int* abort_flag = (int*)(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = m_tile0 * BM, n0 = n_tile0 * BN;
  const int nch = (num_kb + CHUNK_KB - 1) / CHUNK_KB;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 8);  // one arrival per epilogue warp
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     su32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer ----------------
      int issued = 0;
      for (int kb = 0; kb < num_kb; ++kb) {
        const int s = kb % STAGES;
        const uint32_t ph = (kb / STAGES) & 1;
        if (!mbar_wait(&empty[s], ph ^ 1, status)) { *(volatile int*)abort_flag = 1; break; }
        if (*(volatile int*)abort_flag) break;
        uint8_t* st = smem + s * STAGE_BYTES;
        mbar_expect_tx(&full[s], STAGE_BYTES);
        const int k0 = (kb_first + kb) * BK;
        for (int p = 0; p < 3; ++p) {
          tma_load_2d(st + p * TILE_BYTES, &mapA, &full[s], k0, rowA0 + p * rowsA + m0);
          tma_load_2d(st + (3 + p) * TILE_BYTES, &mapB, &full[s], k0, rowB0 + p * rowsB + n0);
        }
        issued = kb + 1;
      }
      // drain: every issued stage must have landed before the CTA may exit
      for (int kb = (issued > STAGES ? issued - STAGES : 0); kb < issued; ++kb)
        mbar_wait(&full[kb % STAGES], (kb / STAGES) & 1, status);
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      bool ok = true;
      for (int ch = 0; ch < nch && ok; ++ch) {
        const int buf = ch & 1;
        if (!mbar_wait(&acc_empty[buf], ((ch >> 1) & 1) ^ 1, status)) {
          *(volatile int*)abort_flag = 1;
          break;
        }
        tc_fence_after();
        const uint32_t dacc = tmem + (uint32_t)(buf * BN);
        const int kb0 = ch * CHUNK_KB;
        const int kb1 = min(num_kb, kb0 + CHUNK_KB);
        for (int kb = kb0; kb < kb1; ++kb) {
          const int s = kb % STAGES;
          const uint32_t ph = (kb / STAGES) & 1;
          if (!mbar_wait(&full[s], ph, status)) { *(volatile int*)abort_flag = 1; ok = false; break; }
          if (*(volatile int*)abort_flag) { ok = false; break; }
          tc_fence_after();
          uint8_t* st = smem + s * STAGE_BYTES;
#pragma unroll
          for (int pr = 0; pr < 6; ++pr) {
            const uint64_t da = sdesc_sw128(st + kPairA[pr] * TILE_BYTES);
            const uint64_t db = sdesc_sw128(st + (3 + kPairB[pr]) * TILE_BYTES);
#pragma unroll
            for (int j = 0; j < BK / 16; ++j)
              umma_bf16(dacc, da + 2 * j, db + 2 * j, IDESC, ((kb - kb0) | pr | j) != 0);
          }
          umma_commit(&empty[s]);
        }
        umma_commit(&acc_full[buf]);  // chunk complete (also fires on abort)
      }
    }
    __syncwarp();
  } else {
    // ---------------- epilogue warps 2..9 ----------------
    const int q = warp & 3;              // TMEM lane quadrant this warp may access
    const int half = (warp - 2) >> 2;    // 64-column half of the tile
    const int row = m0 + q * 32 + lane;
    const uint32_t tq = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(half * 64);
    const uint32_t t_hi = tq + 256, t_lo = tq + 384;
    bool ok = true;
    for (int ch = 0; ch < nch; ++ch) {
      const int buf = ch & 1;
      bool have = mbar_wait(&acc_full[buf], (ch >> 1) & 1, status);
      have = __all_sync(0xffffffffu, have && !*(volatile int*)abort_flag);
      if (!have) { ok = false; break; }
      tc_fence_after();
      const uint32_t t_acc = tq + (uint32_t)(buf * BN);
#pragma unroll 1
      for (int c = 0; c < 4; ++c) {
        uint32_t a[16], h[16], l[16];
        tmem_ld16(t_acc + c * 16, a);
        if (ch == 0) {
#pragma unroll
          for (int j = 0; j < 16; ++j) { h[j] = a[j]; l[j] = 0u; }
        } else {
          tmem_ld16(t_hi + c * 16, h);
          tmem_ld16(t_lo + c * 16, l);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            float s, e;
            two_sum(__uint_as_float(h[j]), __uint_as_float(a[j]), s, e);
            h[j] = __float_as_uint(s);
            l[j] = __float_as_uint(__uint_as_float(l[j]) + e);
          }
        }
        tmem_st16(t_hi + c * 16, h);
        tmem_st16(t_lo + c * 16, l);
      }
      tmem_st_wait();
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[buf]);
    }
    if (ok) {
      tc_fence_after();
#pragma unroll 1
      for (int c = 0; c < 4; ++c) {
        uint32_t h[16], l[16];
        tmem_ld16(t_hi + c * 16, h);
        tmem_ld16(t_lo + c * 16, l);
        if (row < M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int col = n0 + half * 64 + c * 16 + j;
            if (col < N) {
              double* cp = C + (long long)row + ldc * col;
              double v = g.alpha * ((double)__uint_as_float(h[j]) + (double)__uint_as_float(l[j]));
              if (g.beta != 0.0) v += g.beta * *cp;
              *cp = v;
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
}

// Split the FP64 matrix X (rows x K) into three BF16 parts stored K-major:
// P[p*rows_pad*Kpad + r*Kpad + k], zero padded to rows_pad x Kpad.  X(r, k) = X[r + ld*k]
// (trans = 0, read through a shared-memory transpose) or X[k + ld*r] (trans = 1, read along k
// directly); kscale (optional) multiplies X(r, k) by kscale[k] first.
// The split runs in FP32 after one exact-enough FP64 step: x = h + l with h = fl32(x) and
// l = fl32(x - h) (48 bits of x, four FP64-pipe operations), then x0 = bf16(h), the remainder
// r1 = (h - x0) + l (h - x0 is exact in FP32; the addition rounds at 2^-24 |r1| <= 2^-32 |x|),
// x1 = bf16(r1), r2 = r1 - x1 (exact), x2 = bf16(r2): |x - x0 - x1 - x2| <= ~2^-24 |x|, the
// accuracy of a three-way BF16 split, at a third of the FP64 work of splitting in FP64 (the
// kernel is FP64-issue-bound otherwise).
__device__ __forceinline__ void split_store(double x, __nv_bfloat16* __restrict__ P, size_t o,
                                            size_t plane) {
  const float h = __double2float_rn(x);
  const float l = __double2float_rn(x - (double)h);
  const __nv_bfloat16 x0 = __float2bfloat16_rn(h);
  const float r1 = (h - __bfloat162float(x0)) + l;
  const __nv_bfloat16 x1 = __float2bfloat16_rn(r1);
  const float r2 = r1 - __bfloat162float(x1);
  const __nv_bfloat16 x2 = __float2bfloat16_rn(r2);
  P[o] = x0;
  P[o + plane] = x1;
  P[o + 2 * plane] = x2;
}

__global__ void k_split3(int rows, int K, const double* __restrict__ X, long long ld, int trans,
                         const float* __restrict__ kscale, int rows_pad, int Kpad,
                         __nv_bfloat16* __restrict__ P) {
  __shared__ double t[32][33];
  const int r0 = blockIdx.x * 32, k0 = blockIdx.y * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  const size_t plane = (size_t)rows_pad * Kpad;
  if (trans) {
    for (int i = ty; i < 32; i += 8) {
      const int r = r0 + i, k = k0 + tx;
      if (r < rows_pad && k < Kpad) {
        double x = (r < rows && k < K) ? X[(long long)k + ld * r] : 0.0;
        if (kscale && k < K) x *= (double)kscale[k];
        split_store(x, P, (size_t)r * Kpad + k, plane);
      }
    }
    return;
  }
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + tx, k = k0 + i;
    t[i][tx] = (r < rows && k < K) ? X[(long long)r + ld * k] : 0.0;
  }
  __syncthreads();
  for (int i = ty; i < 32; i += 8) {
    const int r = r0 + i, k = k0 + tx;
    if (r < rows_pad && k < Kpad) {
      double x = t[tx][i];
      if (kscale && k < K) x *= (double)kscale[k];
      split_store(x, P, (size_t)r * Kpad + k, plane);
    }
  }
}

// C = alpha * sum_s W[s] + beta * C  (split-K reduction, column-major m x n, W slices m x n)
__global__ void k_bf16x3_reduce(int m, int n, int S, const double* __restrict__ W, double alpha,
                                double beta, double* __restrict__ C, long long ldc) {
  const long long total = (long long)m * n;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    double acc = 0.0;
    for (int s = 0; s < S; ++s) acc += W[(long long)s * total + i];
    const int r = (int)(i % m);
    const long long c = i / m;
    double* cp = C + r + ldc * c;
    double v = alpha * acc;
    if (beta != 0.0) v += beta * (*cp);
    *cp = v;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

int make_map(qk_ctx* ctx, CUtensorMap* map, const void* base, int Kpad, long long rows_total) {
  auto enc = get_encode();
  if (!enc) return qk_fail(ctx, QK_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[2] = {(cuuint64_t)Kpad, (cuuint64_t)rows_total};
  cuuint64_t strides[1] = {(cuuint64_t)Kpad * 2};
  cuuint32_t box[2] = {BK, 128};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return qk_fail(ctx, QK_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return QK_OK;
}

}  // namespace

static int qk_split3(qk_ctx* ctx, int rows, int K, const double* X, long long ld, int trans,
                     const float* kscale, int rows_pad, int Kpad, void* parts) {
  dim3 grid((rows_pad + 31) / 32, (Kpad + 31) / 32);
  if (grid.y > 65535) return qk_fail(ctx, QK_ERR_ARG, "split: K too large");
  k_split3<<<grid, dim3(32, 8), 0, ctx->stream>>>(rows, K, X, ld, trans, kscale, rows_pad, Kpad,
                                                  (__nv_bfloat16*)parts);
  QK_LAUNCHED();
  return QK_OK;
}

namespace {

int launch_gemm(qk_ctx* ctx, const CUtensorMap& ma, const CUtensorMap& mb, const GemmX& g,
                dim3 grid) {
  static std::once_flag once;
  static cudaError_t attr_err = cudaSuccess;
  std::call_once(once, [] {
    attr_err = cudaFuncSetAttribute(k_gemm_bf16x3<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    SMEM_BYTES);
    if (attr_err == cudaSuccess)
      attr_err = cudaFuncSetAttribute(k_gemm_bf16x3<2>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    if (attr_err == cudaSuccess)
      attr_err = cudaFuncSetAttribute(k_gemm_bf16x3<4>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
  });
  QK_CK(attr_err);
  const int chunk = qk_tune_get(ctx, TUNE_BF16X3_CHUNK, g.Kpad, 2);
  if (chunk == 1)
    k_gemm_bf16x3<1><<<grid, NTHREADS, SMEM_BYTES, ctx->stream>>>(ma, mb, g, ctx->d_status);
  else if (chunk == 4)
    k_gemm_bf16x3<4><<<grid, NTHREADS, SMEM_BYTES, ctx->stream>>>(ma, mb, g, ctx->d_status);
  else
    k_gemm_bf16x3<2><<<grid, NTHREADS, SMEM_BYTES, ctx->stream>>>(ma, mb, g, ctx->d_status);
  QK_LAUNCHED();
  return QK_OK;
}

}  // namespace

int qk_gemm_bf16x3(qk_ctx* ctx, char ta, char tb, int m, int n, int k, double alpha,
                   const double* A, long long lda, long long sA, const double* B, long long ldb,
                   long long sB, const float* bscale, long long sBS, double beta, double* C,
                   long long ldc, long long sC, int batch, bool lower) {
  if (m <= 0 || n <= 0 || batch <= 0) return QK_OK;
  if (k <= 0) return qk_fail(ctx, QK_ERR_ARG, "bf16x3: k must be positive");
  const bool TA = (ta == 'T' || ta == 't'), TB = (tb == 'T' || tb == 't');
  const int rowsA = (m + BM - 1) / BM * BM;
  const int rowsB = (n + BN - 1) / BN * BN;
  const int Kpad = (k + BK - 1) / BK * BK;
  const bool a_b = batch > 1 && sA != 0;
  const bool b_b = batch > 1 && (sB != 0 || (bscale && sBS != 0));
  const size_t planeA = (size_t)3 * rowsA * Kpad, planeB = (size_t)3 * rowsB * Kpad;
  __nv_bfloat16 *Ap = nullptr, *Bp = nullptr;
  QK_TRY(qk_wst(ctx, W_SPLIT_A, planeA * (a_b ? batch : 1), &Ap));
  QK_TRY(qk_wst(ctx, W_SPLIT_B, planeB * (b_b ? batch : 1), &Bp));
  // op(A) (m x k) as rows x K: X(i, kk) = A[i + lda kk] ('N') or A[kk + lda i] ('T');
  // op(B)^T (n x k): X(j, kk) = op(B)(kk, j) = B[kk + ldb j] ('N') or B[j + ldb kk] ('T')
  for (int b = 0; b < (a_b ? batch : 1); ++b)
    QK_TRY(qk_split3(ctx, m, k, A + b * sA, lda, TA ? 1 : 0, nullptr, rowsA, Kpad, Ap + b * planeA));
  for (int b = 0; b < (b_b ? batch : 1); ++b)
    QK_TRY(qk_split3(ctx, n, k, B + b * sB, ldb, TB ? 0 : 1, bscale ? bscale + b * sBS : nullptr,
                     rowsB, Kpad, Bp + b * planeB));
  CUtensorMap ma, mb;
  QK_TRY(make_map(ctx, &ma, Ap, Kpad, 3LL * rowsA * (a_b ? batch : 1)));
  QK_TRY(make_map(ctx, &mb, Bp, Kpad, 3LL * rowsB * (b_b ? batch : 1)));
  const int m_tiles = rowsA / BM, n_tiles = rowsB / BN;
  const long long tiles = (long long)m_tiles * n_tiles;
  if (tiles > 0x7fffffffLL || batch > 65535) return qk_fail(ctx, QK_ERR_ARG, "bf16x3: too many tiles");
  GemmX g;
  g.M = m; g.N = n; g.Kpad = Kpad; g.rowsA = rowsA; g.rowsB = rowsB;
  g.a_batched = a_b; g.b_batched = b_b;
  g.n_tiles = n_tiles; g.lower = lower ? 1 : 0;
  const int num_kb = Kpad / BK;
  // few output tiles and a long k: split k over CTAs, FP64 slices, one reduction (not with
  // lower: the reduction would write the skipped upper tiles)
  const long long eff = tiles;
  int S = 1;
  if (!lower && batch == 1 && eff * 2 < ctx->num_sms && num_kb >= 8) {
    S = (int)((ctx->num_sms + eff - 1) / eff);
    if (S > num_kb / 4) S = num_kb / 4;
    if (S > 16) S = 16;
    if (S < 1) S = 1;
  }
  if (S > 1) {
    const int kbs = (num_kb + S - 1) / S;
    S = (num_kb + kbs - 1) / kbs;
    double* W = nullptr;
    QK_TRY(qk_wst(ctx, W_SPLITK, (size_t)S * m * n, &W));
    g.kb_per_slice = kbs;
    g.alpha = 1.0; g.beta = 0.0;
    g.C = W; g.ldc = m; g.sC = (long long)m * n;
    QK_TRY(launch_gemm(ctx, ma, mb, g, dim3((unsigned)tiles, 1, S)));
    const long long total = (long long)m * n;
    int blocks = (int)((total + 255) / 256);
    if (blocks > 16 * ctx->num_sms) blocks = 16 * ctx->num_sms;
    k_bf16x3_reduce<<<blocks, 256, 0, ctx->stream>>>(m, n, S, W, alpha, beta, C, ldc);
    QK_LAUNCHED();
    return QK_OK;
  }
  g.kb_per_slice = num_kb;
  g.alpha = alpha; g.beta = beta;
  g.C = C; g.ldc = ldc; g.sC = sC;
  return launch_gemm(ctx, ma, mb, g, dim3((unsigned)tiles, batch, 1));
}

int qk_gemm_bf16x3_nt(qk_ctx* ctx, int m, int n, int k, const double* A, long long lda,
                      const double* B, long long ldb, double* C, long long ldc) {
  if (m <= 0 || n <= 0 || k <= 0) return QK_OK;
  return qk_gemm_bf16x3(ctx, 'N', 'T', m, n, k, 1.0, A, lda, 0, B, ldb, 0, nullptr, 0, 0.0, C, ldc,
                        0, 1, false);
}
