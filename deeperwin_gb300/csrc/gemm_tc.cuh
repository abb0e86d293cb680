// Persistent tcgen05 tensor-core GEMM (TMA loads, TMEM accumulators, TMA stores).
#pragma once
#include "net.cuh"

namespace dw {

bool tc_available();

// C[M, N] = epilogue(A[M, K] @ W[N, K]^T).
// np = 1: A and W are BF16; np = 2: split-BF16 (A is [hi | lo] rows of logical width lda, W = W0 + W1).
// out = 0: fp32 C (row stride ldc); 1: bf16 C; 2: split-BF16 C ([hi | lo] rows of logical width ldc).
// fl = 1: forward-Laplacian tanh epilogue over groups of epi.Tp channel rows (n3 = 3 n_el);
// fl = 0: bias / row bias and optional tanh (epi.act).
// W rows have stride round_up(K, 64).
int gemm_tc(int np, int out, const void* A, int lda, const __nv_bfloat16* W0, const __nv_bfloat16* W1, void* C, int ldc,
            int M, int N, int K, const GemmEpi& epi, int fl, int n3, cudaStream_t s);

// Walker-block operands: per walker `rows` consecutive rows (a multiple of 32) of A (row stride
// np * lda) and C (row stride ldc), walkers a_wstride / c_wstride elements apart.
struct WalkerBlocks {
    int nw, rows;
    int64_t a_wstride, c_wstride;
};
// C (fp32) = A @ W^T over the rows of every walker block, plain epilogue.
int gemm_tc_wb(int np, const void* A, int lda, const __nv_bfloat16* W0, const __nv_bfloat16* W1, float* C, int ldc,
               const WalkerBlocks& wb, int N, int K, cudaStream_t s);

}  // namespace dw
