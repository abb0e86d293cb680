// FP32 CUDA-core GEMM for the plain (FP32 end-to-end) form: C = A @ W with the
// per-row epilogues of the network (value-channel bias, per-walker-channel row bias,
// optional tanh for value-only rows). No TF32: the reference disables it
// (NVIDIA_TF32_OVERRIDE=0, process_molecule.py:20-29).
#include "net.cuh"

namespace dw {

template <int BM, int BN, int BK, int TM, int TN>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
k_gemm_f32(const float* __restrict__ A, int lda, const float* __restrict__ W, int ldw, float* __restrict__ C, int ldc,
           int M, int N, int K, GemmEpi epi, int64_t sA, int64_t sC) {
    constexpr int TR = BM / TM, TC = BN / TN, NT = TR * TC;
    A += blockIdx.z * sA;
    C += blockIdx.z * sC;
    __shared__ float As[2][BK][BM + 4];
    __shared__ float Ws[2][BK][BN + 4];
    const int tid = threadIdx.x;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    const int tr = tid / TC, tc = tid % TC;
    float acc[TM][TN];
    #pragma unroll
    for (int i = 0; i < TM; ++i)
        #pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;

    auto load = [&](int buf, int k0) {
        #pragma unroll 4
        for (int e = tid; e < BM * BK; e += NT) {
            int rr = e / BK, kk = e % BK;
            int gm = m0 + rr, gk = k0 + kk;
            As[buf][kk][rr] = (gm < M && gk < K) ? __ldg(A + (int64_t)gm * lda + gk) : 0.f;
        }
        #pragma unroll 4
        for (int e = tid; e < BK * BN; e += NT) {
            int kk = e / BN, cc = e % BN;
            int gk = k0 + kk, gn = n0 + cc;
            Ws[buf][kk][cc] = (gk < K && gn < N) ? __ldg(W + (int64_t)gk * ldw + gn) : 0.f;
        }
    };
    int nk = (K + BK - 1) / BK;
    load(0, 0);
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
        int buf = kt & 1;
        if (kt + 1 < nk) load(buf ^ 1, (kt + 1) * BK);
        #pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            float a[TM], w[TN];
            #pragma unroll
            for (int i = 0; i < TM; ++i) a[i] = As[buf][kk][tr + i * TR];
            #pragma unroll
            for (int j = 0; j < TN; ++j) w[j] = Ws[buf][kk][tc + j * TC];
            #pragma unroll
            for (int i = 0; i < TM; ++i)
                #pragma unroll
                for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], w[j], acc[i][j]);
        }
        __syncthreads();
    }
    #pragma unroll
    for (int i = 0; i < TM; ++i) {
        int m = m0 + tr + i * TR;
        if (m >= M) continue;
        int t = m % epi.Tp;
        const float* rb = epi.rowbias ? epi.rowbias + ((int64_t)(m / epi.rows_per_walker) * epi.Tp + t) * epi.ldrb : nullptr;
        #pragma unroll
        for (int j = 0; j < TN; ++j) {
            int n = n0 + tc + j * TC;
            if (n >= N) continue;
            float v = acc[i][j];
            if (epi.bias && t == 0) v += epi.bias[n];
            if (rb) v += rb[n];
            if (epi.act == 1) v = tanhf(v);
            C[(int64_t)m * ldc + n] = v;
        }
    }
}

void gemm_f32(const float* A, int lda, const float* W, int ldw, float* C, int ldc, int M, int N, int K,
              const GemmEpi& epi, int batch, int64_t sA, int64_t sC, cudaStream_t s) {
    if (M <= 0 || N <= 0) return;
    if (N <= 32) {
        constexpr int BM = 128, BN = 32;
        dim3 g((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
        k_gemm_f32<BM, BN, 8, 8, 2><<<g, (BM / 8) * (BN / 2), 0, s>>>(A, lda, W, ldw, C, ldc, M, N, K, epi, sA, sC);
    } else {
        constexpr int BM = 128, BN = 64;
        dim3 g((N + BN - 1) / BN, (M + BM - 1) / BM, batch);
        k_gemm_f32<BM, BN, 8, 8, 4><<<g, (BM / 8) * (BN / 4), 0, s>>>(A, lda, W, ldw, C, ldc, M, N, K, epi, sA, sC);
    }
    count_launch();
}

}  // namespace dw
