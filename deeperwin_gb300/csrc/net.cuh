// Declarations of the network, determinant, MCMC and GEMM launchers.
#pragma once
#include <type_traits>
#include "common.cuh"

namespace dw {

template <class T> __device__ __forceinline__ T from_f(float v);
template <> __device__ __forceinline__ float from_f<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float to_f(__nv_bfloat16 v) { return __bfloat162float(v); }

// Storage element of split-BF16 activations: a logical row of width ld is stored as
// [hi(0..ld) | lo(0..ld)] with hi = bf16(x), lo = bf16(x - hi); x is recovered as hi + lo
// to about 2^-17 relative. Tensor-core GEMMs consume hi and lo as two BF16 operands.
struct Split { __nv_bfloat16 v; };

// act_store / act_load address element (row, col) of a logical [rows, ld] activation.
template <class Act> struct ActIO {
    static constexpr int kParts = 1;
    __device__ static __forceinline__ void store(Act* b, int64_t row, int ld, int col, float x) {
        b[row * ld + col] = from_f<Act>(x);
    }
    // eight consecutive columns; col % 8 == 0 and the row start 16-byte aligned
    __device__ static __forceinline__ void store8(Act* b, int64_t row, int ld, int col, const float (&x)[8]) {
        if constexpr (std::is_same<Act, float>::value) {
            float4* o = reinterpret_cast<float4*>(b + row * ld + col);
            o[0] = make_float4(x[0], x[1], x[2], x[3]);
            o[1] = make_float4(x[4], x[5], x[6], x[7]);
        } else {
            uint32_t p[4];
            #pragma unroll
            for (int k = 0; k < 4; ++k) {
                __nv_bfloat162 h = __floats2bfloat162_rn(x[2 * k], x[2 * k + 1]);
                p[k] = *reinterpret_cast<uint32_t*>(&h);
            }
            *reinterpret_cast<uint4*>(b + row * ld + col) = make_uint4(p[0], p[1], p[2], p[3]);
        }
    }
    __device__ static __forceinline__ float load(const Act* b, int64_t row, int ld, int col) {
        return to_f(b[row * ld + col]);
    }
};
template <> struct ActIO<Split> {
    static constexpr int kParts = 2;
    __device__ static __forceinline__ void store(Split* b, int64_t row, int ld, int col, float x) {
        __nv_bfloat16 hi = __float2bfloat16_rn(x);
        __nv_bfloat16 lo = __float2bfloat16_rn(x - __bfloat162float(hi));
        b[row * 2 * ld + col].v = hi;
        b[row * 2 * ld + ld + col].v = lo;
    }
    __device__ static __forceinline__ void store8(Split* b, int64_t row, int ld, int col, const float (&x)[8]) {
        uint32_t ph[4], pl[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) {
            __nv_bfloat162 h = __floats2bfloat162_rn(x[2 * k], x[2 * k + 1]);
            __nv_bfloat162 l = __floats2bfloat162_rn(x[2 * k] - __low2float(h), x[2 * k + 1] - __high2float(h));
            ph[k] = *reinterpret_cast<uint32_t*>(&h);
            pl[k] = *reinterpret_cast<uint32_t*>(&l);
        }
        *reinterpret_cast<uint4*>(b + row * 2 * ld + col) = make_uint4(ph[0], ph[1], ph[2], ph[3]);
        *reinterpret_cast<uint4*>(b + row * 2 * ld + ld + col) = make_uint4(pl[0], pl[1], pl[2], pl[3]);
    }
    __device__ static __forceinline__ float load(const Split* b, int64_t row, int ld, int col) {
        return __bfloat162float(b[row * 2 * ld + col].v) + __bfloat162float(b[row * 2 * ld + ld + col].v);
    }
};

// net.cu
void launch_ion_maps(const float* P, const ParamLayout& L, const Dims& d, const int32_t* Z, float* him, cudaStream_t s);
template <class Act> void launch_features(const float* r, const float* R, const int32_t* Z, const Dims& d, int B, Act* X0,
                                          cudaStream_t s);
// him != nullptr (forward passes, when ei_fusable(d)): HE receives the el-ion convolution already
// reduced over the ions, conv_ei[level][walker * n + electron][channels][32], not the stream.
bool ei_fusable(const Dims& d);
void launch_streams(const float* r, const float* R, const int32_t* Z, const float* P, const ParamLayout& L,
                    const Dims& d, int B, float* WP, float* HE, cudaStream_t s, float* HP = nullptr,
                    const float* him = nullptr);
template <class Act> void launch_spin_means(const Act* X, int ldx, int hw, const Dims& d, int B, Act* M, int mw, cudaStream_t s);
template <class Act> void launch_tanh_fl(const float* Zb, int ldz, int ncols, int groups, const Dims& d, Act* Y, int ldy, cudaStream_t s);
// ei_fused = 1: HEl is conv_ei of this level (launch_streams with him), not the el-ion stream.
template <class Act> void launch_conv(const float* r, const float* WPl, const float* HM, const float* HEl, const float* himl,
                                      const Dims& d, int l, int B, Act* X, int ldx, cudaStream_t s, int ei_fused = 0);
// BF rows hold the backflow of each electron; the down-spin electrons' columns start at column
// spin_cols (KN when both spin blocks are stored side by side, 0 when each row holds its own spin's).
void launch_envelope(const float* r, const float* R, const int32_t* Z, const float* P, const ParamLayout& L,
                     const float* sp_alpha, const Dims& d, int B, const float* BF, int ldbf, int spin_cols, float* MO,
                     cudaStream_t s);
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
// C[M, N] (+)= A[M, K] @ W^T where W is [N, K] row-major (ldw); accumulate = 1 adds to C.
void gemm_f32_nt(const float* A, int lda, const float* W, int ldw, float* C, int ldc, int M, int N, int K,
                 int accumulate, cudaStream_t s);
// dW[K, N] += sum_r A[r, k] G[r, n] over rows r (row selector sel[r] == want when sel != NULL),
// dB[N] += sum_r G[r, n] when dB != NULL. Split over rows, atomically accumulated.
void wgrad_f32(const float* A, int lda, const float* G, int ldg, int rows, int K, int N, float* dW, int lddw,
               float* dB, const int8_t* sel, int want, cudaStream_t s);
// K, N <= 32: rows with sel[r] == 1 accumulate into (dW1, dB1), the others into (dW0, dB0), in one
// pass (sel == NULL: every row into output 0).
void wgrad32_sel2(const float* A, int lda, const float* G, int ldg, int rows, int K, int N, const int8_t* sel,
                  float* dW0, float* dB0, float* dW1, float* dB1, int lddw, cudaStream_t s);

// det.cu
template <class S>
void launch_slogdet(const float* MO, const Dims& d, int B, double* logdet, double* sign, float* Ainv, cudaStream_t s);
void launch_det_tangents(const float* MO, const float* Ainv, const double* sign, const Dims& d, int B,
                         double* g, double* lapdet, cudaStream_t s);
void launch_combine(const double* logdet, const double* sign, const double* g, const double* lapdet, const double* jas,
                    const float* r, const float* R, const int32_t* Z, const Dims& d, int B,
                    float* log_psi_sqr, float* phase, float* E_loc, float* grad_out, cudaStream_t s,
                    int coul64 = 0, const int* nvalid = nullptr, float* esc = nullptr);
void launch_coulomb(const float* r, int B, int n, const float* R, const int32_t* Z, int N, float* E, cudaStream_t s);
// FP64 Gauss-Jordan log|det| and inverse of the value-channel Slater matrices (any Dims mode).
void launch_slogdet_inv(const float* MO, const Dims& d, int B, double* logdet, double* sign, float* Ainv, cudaStream_t s);

// api.cu: value-only forward on caller-provided scratch, walker chunks sized against `budget` bytes
size_t value_forward_bytes(const DwArch* a, int precision, int B, size_t budget);
int value_forward(const DwArch* a, int precision, const float* params, const void* prepared, const float* r, int B,
                  const float* R, const int32_t* Z, float* lp, float* phase, void* ws, size_t wsb, size_t budget,
                  cudaStream_t s);

// api.cu: the FP32 row-gathered layer weights (Wmain, Wmean per iteration) of a prepared buffer
void prepared_fp32_layers(const DwArch* a, const void* prepared, const float* main[4], const float* mean[4]);

// fp64.cu: FP64 form (DW_PRECISION_FP64). nvalid (device int, may be null): walkers at or beyond
// *nvalid are skipped; it requires the walkers to fit one chunk.
size_t fp64_plan_bytes(const DwArch* a, int B, bool tang);
int fp64_max_chunk(const DwArch* a, bool tang);     // walkers of one FP64 chunk
// FP64 LU, inverse and determinant tangents of float32 Slater channels (MO layout of the forward
// plans, d.T channels); MO64 holds Bc K T n^2 doubles, Ainv64 Bc K n^2.
int fp64_dets_from_f32(const float* MO, const Dims& d, int Bc, double* MO64, double* Ainv64, double* logdet,
                       double* sign, double* g, double* lapdet, cudaStream_t s);
int fp64_forward_all(const DwArch* a, const float* P, const void* prepared, const float* r, int B, const float* R,
                     const int32_t* Z, float* lp, float* phase, float* E, float* grad, bool tang, void* ws,
                     size_t ws_bytes, cudaStream_t s, const int32_t* seg, int nseg, const int* nvalid);

// api.cu: the FP32 (DW_PRECISION_FP32_DET64) or split-BF16 (DW_PRECISION_MIXED_DET64) network with
// FP64 determinant algebra on a caller region
inline bool det64_form(int precision) {
    return precision == DW_PRECISION_FP32_DET64 || precision == DW_PRECISION_MIXED_DET64;
}
size_t det64_plan_bytes(const DwArch* a, int precision, int B);
int det64_local_energy(const DwArch* a, int precision, const float* P, const void* prepared, const float* r, int B,
                       const float* R, const int32_t* Z, const int32_t* seg, int nseg, float* E, float* lp, float* grad,
                       void* ws, size_t wsb, cudaStream_t s);

// guard.cu: FP64 re-evaluation of the mixed form's flagged walkers (esc: per-walker error scales
// written by the combine kernel, 3 floats per walker)
int guard_capacity(const DwArch* a, int B);
size_t guard_bytes(const DwArch* a, int B);
int tail_guard(const DwArch* a, const float* P, const void* prepared, const float* r, int B, const float* R,
               const int32_t* Z, const int32_t* seg, int nseg, const float* esc, float* E, float* lp, float* grad,
               void* ws, size_t wsb, cudaStream_t s);

// backward.cu
size_t bwd_bytes(const DwArch* a, int B, int* chunk);
int backward_all(const DwArch* a, const float* P, const float* const main[4], const float* const mean[4],
                 const float* bf_cat, const float* sp_alpha, const float* r, int B, const float* R, const int32_t* Z,
                 const float* coeff, float* grad, void* ws, size_t wsb, cudaStream_t s);

}  // namespace dw
