// Declarations of the network, determinant, MCMC and GEMM launchers.
#pragma once
#include "common.cuh"

namespace dw {

template <class T> __device__ __forceinline__ T from_f(float v);
template <> __device__ __forceinline__ float from_f<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

// net.cu
void launch_ion_maps(const float* P, const ParamLayout& L, const Dims& d, const int32_t* Z, float* him, cudaStream_t s);
template <class Act> void launch_features(const float* r, const float* R, const Dims& d, int B, Act* X0, cudaStream_t s);
void launch_streams(const float* r, const float* R, const float* P, const ParamLayout& L, const Dims& d, int B,
                    float* WP, float* HE, cudaStream_t s);
template <class Act> void launch_spin_means(const Act* X, int ldx, int hw, const Dims& d, int B, Act* M, int mw, cudaStream_t s);
template <class Act> void launch_tanh_fl(const float* Zb, int ldz, int ncols, int groups, const Dims& d, Act* Y, int ldy, cudaStream_t s);
template <class Act> void launch_conv(const float* r, const float* WPl, const float* HM, const float* HEl, const float* himl,
                                      const Dims& d, int l, int B, Act* X, int ldx, cudaStream_t s);
void launch_envelope(const float* r, const float* R, const float* P, const ParamLayout& L, const Dims& d, int B,
                     const float* BF, int ldbf, float* MO, cudaStream_t s);
template <class Act> void launch_jastrow_out(const Act* J2, int ldj, const float* w2, const Dims& d, int B, double* jas, cudaStream_t s);

// gemm_simt.cu: C[m, n] = sum_k A[m, k] W[k, n] with epilogue.
struct GemmEpi {
    const float* bias = nullptr;     // [N], added to rows whose channel (row % Tp) == 0
    const float* rowbias = nullptr;  // [(walker * Tp + channel), N] added to every row
    int ldrb = 0;
    int Tp = 1;                      // channels per electron
    int rows_per_walker = 1;         // n_el * Tp (for rowbias indexing)
    int act = 0;                     // 0: none, 1: tanh (value-only rows)
};
void gemm_f32(const float* A, int lda, const float* W, int ldw, float* C, int ldc, int M, int N, int K,
              const GemmEpi& epi, int batch, int64_t sA, int64_t sC, cudaStream_t s);

// det.cu
template <class S>
void launch_slogdet(const float* MO, const Dims& d, int B, double* logdet, double* sign, float* Ainv, cudaStream_t s);
void launch_det_tangents(const float* MO, const float* Ainv, const double* sign, const Dims& d, int B,
                         double* g, double* lapdet, cudaStream_t s);
void launch_combine(const double* logdet, const double* sign, const double* g, const double* lapdet, const double* jas,
                    const float* r, const float* R, const int32_t* Z, const Dims& d, int B,
                    float* log_psi_sqr, float* phase, float* E_loc, float* grad_out, cudaStream_t s);
void launch_coulomb(const float* r, int B, int n, const float* R, const int32_t* Z, int N, float* E, cudaStream_t s);

}  // namespace dw
