// Tensor-core (tcgen05 + TMA) BF16 GEMM with FP32 accumulation in TMEM.
#pragma once
#include "net.cuh"

namespace dw {

bool tc_available();

// C[M, N] (fp32) = A[M, K] (bf16, row stride lda) @ Wt[N, K]^T (bf16, K-major, row stride = round_up(K, 64))
// with the GemmEpi epilogue (act must be 0 or 1).
int gemm_bf16_tc(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Wt, float* C, int ldc, int M, int N, int K,
                 const GemmEpi& epi, cudaStream_t s);
// Same, bf16 output (used for value-only layers whose output feeds the next GEMM).
int gemm_bf16_tc_act(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Wt, __nv_bfloat16* C, int ldc, int M, int N,
                     int K, const GemmEpi& epi, cudaStream_t s);
// Batched over walkers: A_z = A + z * sA, C_z = C + z * sC (element strides), no epilogue.
int gemm_bf16_tc_batched(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Wt, float* C, int ldc, int M, int N, int K,
                         int batch, int64_t sA, int64_t sC, cudaStream_t s);

// Split-BF16 operands (three MMAs per K step): A is [hi | lo] rows of logical width lda.
int gemm_split_tc(const Split* A, int lda, const __nv_bfloat16* Whi, const __nv_bfloat16* Wlo, float* C, int ldc, int M,
                  int N, int K, const GemmEpi& epi, cudaStream_t s);
int gemm_split_tc_act(const Split* A, int lda, const __nv_bfloat16* Whi, const __nv_bfloat16* Wlo, Split* C, int ldc,
                      int M, int N, int K, const GemmEpi& epi, cudaStream_t s);
int gemm_split_tc_batched(const Split* A, int lda, const __nv_bfloat16* Whi, const __nv_bfloat16* Wlo, float* C, int ldc,
                          int M, int N, int K, int batch, int64_t rows_per_batch, int64_t sC, cudaStream_t s);

}  // namespace dw
