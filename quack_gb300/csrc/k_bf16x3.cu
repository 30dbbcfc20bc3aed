// k_bf16x3.cu -- placeholder until the tcgen05 kernel lands.
#include "qk_internal.cuh"

int qk_gemm_bf16x3_nt(qk_ctx* ctx, int m, int n, int k, const double* A, long long lda,
                      const double* B, long long ldb, double* C, long long ldc) {
  (void)m; (void)n; (void)k; (void)A; (void)lda; (void)B; (void)ldb; (void)C; (void)ldc;
  return qk_fail(ctx, QK_ERR_UNSUPPORTED, "BF16x3 tier not built");
}
