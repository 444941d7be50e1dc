// Tensor-core layer GEMMs through cuBLAS for the FP32 forms NEB_PREC_TF32 and
// NEB_PREC_BF16X9: the compute type of the current ABI call (a thread-local
// set by GemmScope for the call's duration; 0 selects the SIMT kernels) and
// row-major FP32 GEMM helpers expressed in cuBLAS's column-major terms.
#pragma once
#include <cublas_v2.h>
#include "neb_common.cuh"

namespace neb {

int& gemm_compute();  // 0: SIMT; else a cublasComputeType_t

struct GemmScope {
  int saved;
  explicit GemmScope(int precision) : saved(gemm_compute()) {
    gemm_compute() = precision == NEB_PREC_TF32     ? (int)CUBLAS_COMPUTE_32F_FAST_TF32
                     : precision == NEB_PREC_BF16X9 ? (int)CUBLAS_COMPUTE_32F_EMULATED_16BFX9
                                                    : 0;
  }
  ~GemmScope() { gemm_compute() = saved; }
};

// C = alpha op(A) op(B) + beta C (column-major, FP32 storage), batched with
// the given element strides (a zero stride shares the operand).
int tc_sgemm_batched(cudaStream_t s, cublasOperation_t ta, cublasOperation_t tb, int m,
                     int64_t n, int64_t k, float alpha, const float* A, int lda, int64_t sa,
                     const float* B, int ldb, int64_t sb, float beta, float* C, int ldc,
                     int64_t sc, int batch, const char* name);

}  // namespace neb
