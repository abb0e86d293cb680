// tcgen05 tensor-core GEMM for sm_103a: TMA (128-byte swizzle) loads A and B tiles into a
// multi-stage shared-memory ring, one elected thread issues tcgen05.mma (kind::f16, BF16 in,
// FP32 accumulate in TMEM), and four warps drain TMEM with tcgen05.ld into the fused
// epilogue (value-channel bias, per-walker-channel bias, tanh).
//
// Warp roles: warp 0 lane 0 = TMA producer, warp 1 lane 0 = MMA issuer, warps 0-3 = epilogue.
// Every mbarrier wait is bounded; on timeout the kernel records an error flag, stops
// issuing, drains, frees its TMEM and returns.
#include "gemm_tc.cuh"
#include <cuda.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>

namespace dw {

__device__ int g_tc_error = 0;

namespace {

constexpr int BM = 128, BK = 64;
constexpr uint32_t kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bounded parity wait: returns false after kSpinLimit unsuccessful probes.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    uint32_t addr = smem_u32(bar);
    for (uint32_t it = 0; it < kSpinLimit; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok) : "r"(addr), "r"(parity) : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1) : "memory");
}
// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(const void* p) {
    uint64_t addr = smem_u32(p);
    return ((addr & 0x3FFFFull) >> 4) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) | (2ull << 61);
}
// Instruction descriptor, kind::f16: D=F32, A=B=BF16, both K-major, M=128, N.
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
        ::"r"(tmem_d), "l"(a), "l"(b), "r"(idesc), "r"(accum));
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    #pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

struct TcArgs {
    void* C; int ldc; int M; int N; int K; int BN;
    int64_t a_rows_per_batch;   // row offset of batch z in the A tensor map
    int64_t sC;                 // element offset of batch z in C
    GemmEpi epi;
    int stages;
    uint32_t tmem_cols;
};

// NP = 1: plain BF16 operands, one MMA per 16-wide K step.
// NP = 2: split-BF16 operands A = A_hi + A_lo, W = W_hi + W_lo; three MMAs per K step
//         (A_hi W_hi + A_hi W_lo + A_lo W_hi) into the same FP32 TMEM accumulator.
// OUT = 0: fp32 C; 1: bf16 C; 2: split-BF16 C ([hi | lo] rows of logical width ldc).
template <int NP, int OUT>
__global__ void __launch_bounds__(128, 1)
k_gemm_tc(const __grid_constant__ CUtensorMap tmA0, const __grid_constant__ CUtensorMap tmA1,
          const __grid_constant__ CUtensorMap tmB0, const __grid_constant__ CUtensorMap tmB1, TcArgs a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int S = a.stages, BN = a.BN;
    const uint32_t a_bytes = BM * BK * 2, b_bytes = (uint32_t)BN * BK * 2;
    const uint32_t stage_bytes = NP * (a_bytes + b_bytes);
    // stage s: [A_0 | A_1 | B_0 | B_1]
    auto sA = [&](int s, int part) { return smem + (size_t)s * stage_bytes + (size_t)part * a_bytes; };
    auto sB = [&](int s, int part) { return smem + (size_t)s * stage_bytes + (size_t)NP * a_bytes + (size_t)part * b_bytes; };
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)S * stage_bytes);
    uint64_t* empty = full + S;
    uint64_t* done = empty + S;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
    __shared__ int s_err;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN, z = blockIdx.z;
    const int nk = (a.K + BK - 1) / BK;

    if (threadIdx.x == 0) {
        s_err = 0;
        for (int s = 0; s < S; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     ::"r"(smem_u32(tmem_slot)), "r"(a.tmem_cols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // TMA producer
        const int row_a = (int)(z * a.a_rows_per_batch) + m0;
        for (int kt = 0; kt < nk; ++kt) {
            int s = kt % S;
            if (kt >= S && !mbar_wait(&empty[s], ((kt / S) - 1) & 1)) { atomicExch(&s_err, 1); break; }
            mbar_expect_tx(&full[s], stage_bytes);
            tma_load_2d(sA(s, 0), &tmA0, &full[s], kt * BK, row_a);
            tma_load_2d(sB(s, 0), &tmB0, &full[s], kt * BK, n0);
            if (NP == 2) {
                tma_load_2d(sA(s, 1), &tmA1, &full[s], kt * BK, row_a);
                tma_load_2d(sB(s, 1), &tmB1, &full[s], kt * BK, n0);
            }
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = idesc_bf16(BN);
        for (int kt = 0; kt < nk; ++kt) {
            int s = kt % S;
            if (!mbar_wait(&full[s], (kt / S) & 1)) { atomicExch(&s_err, 1); break; }
            tc_fence_after();
            uint64_t a0 = smem_desc_sw128(sA(s, 0)), b0 = smem_desc_sw128(sB(s, 0));
            uint64_t a1 = smem_desc_sw128(sA(s, NP - 1)), b1 = smem_desc_sw128(sB(s, NP - 1));
            #pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint64_t o = (uint64_t)(kk * 2);
                umma_bf16(tmem, a0 + o, b0 + o, idesc, (kt | kk) ? 1u : 0u);
                if (NP == 2) {
                    umma_bf16(tmem, a0 + o, b1 + o, idesc, 1u);
                    umma_bf16(tmem, a1 + o, b0 + o, idesc, 1u);
                }
            }
            umma_commit(&empty[s]);
        }
        umma_commit(done);
    }
    __syncwarp();
    bool ok = mbar_wait(done, 0);
    tc_fence_after();
    if (!ok) atomicExch(&s_err, 1);

    // Epilogue: warp w owns TMEM lanes (rows) 32w..32w+31.
    const int m = m0 + warp * 32 + lane;
    const GemmEpi& e = a.epi;
    const int t = m % e.Tp;
    const float* rb = (e.rowbias && m < a.M) ? e.rowbias + ((int64_t)(m / e.rows_per_walker) * e.Tp + t) * e.ldrb : nullptr;
    for (int c0 = 0; c0 < BN; c0 += 16) {
        float v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        if (m < a.M && ok) {
            #pragma unroll
            for (int j = 0; j < 16; ++j) {
                int n = n0 + c0 + j;
                if (n < a.N) {
                    float x = v[j];
                    if (e.bias && t == 0) x += e.bias[n];
                    if (rb) x += rb[n];
                    if (e.act == 1) x = tanhf(x);
                    if (OUT == 0) {
                        reinterpret_cast<float*>(a.C)[z * a.sC + (int64_t)m * a.ldc + n] = x;
                    } else if (OUT == 1) {
                        reinterpret_cast<__nv_bfloat16*>(a.C)[z * a.sC + (int64_t)m * a.ldc + n] = __float2bfloat16_rn(x);
                    } else {
                        ActIO<Split>::store(reinterpret_cast<Split*>(a.C) + z * a.sC, m, a.ldc, n, x);
                    }
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (s_err && threadIdx.x == 0) {
        // drain: wait (bounded) for any TMA still in flight before the shared memory is released
        for (int s = 0; s < S; ++s) {
            int last = nk - 1 - ((nk - 1 - s) % S);
            if (last >= s) mbar_wait(&full[s], (last / S) & 1);
        }
        atomicExch(&g_tc_error, 1);
    }
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(a.tmem_cols) : "memory");
    }
}

// ------------------------------------------------------------------ host side
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    }
    return fn;
}

// 2-D bf16 tensor map: dims {cols (inner), rows}, row stride ld elements, box {64, box_rows}.
int make_map(CUtensorMap* map, const void* base, int64_t rows, int cols, int ld, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return DW_ERR_UNSUPPORTED;
    if (((uintptr_t)base & 15) || (ld * 2) % 16) return DW_ERR_ARG;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? DW_OK : DW_ERR_ARG;
}

// A: np parts of a logical [rows, lda] activation (np = 2: [hi | lo] rows of width 2 lda).
// W0/W1: [N, round_up(K, 64)] K-major weight parts.
template <int NP, int OUT>
int launch_tc(const __nv_bfloat16* A, int lda, int64_t a_rows_total, const __nv_bfloat16* W0, const __nv_bfloat16* W1,
              void* C, int ldc, int M, int N, int K, const GemmEpi& epi, int batch, int64_t a_rows_per_batch, int64_t sC,
              cudaStream_t s) {
    if (M <= 0 || N <= 0 || K <= 0) return DW_OK;
    const int bn_max = NP == 2 ? 128 : 256;
    int ntiles = (N + bn_max - 1) / bn_max;
    int BN = round_up((N + ntiles - 1) / ntiles, 16);
    int Kp = round_up(K, 64);
    CUtensorMap ma0, ma1, mb0, mb1;
    const int phys_ld = NP * lda;
    DW_CHECK(make_map(&ma0, A, a_rows_total, K, phys_ld, BM));
    DW_CHECK(make_map(&mb0, W0, N, K, Kp, BN));
    if (NP == 2) {
        DW_CHECK(make_map(&ma1, A + lda, a_rows_total, K, phys_ld, BM));
        DW_CHECK(make_map(&mb1, W1, N, K, Kp, BN));
    } else {
        ma1 = ma0; mb1 = mb0;
    }
    TcArgs a;
    a.C = C; a.ldc = ldc; a.M = M; a.N = N; a.K = K; a.BN = BN;
    a.a_rows_per_batch = a_rows_per_batch; a.sC = sC; a.epi = epi;
    int stage_bytes = NP * (BM * BK * 2 + BN * BK * 2);
    a.stages = std::min(4, (200 * 1024) / stage_bytes);
    a.tmem_cols = 32;
    while ((int)a.tmem_cols < BN) a.tmem_cols <<= 1;
    size_t smem = 1024 + (size_t)a.stages * stage_bytes + (2 * a.stages + 1) * 8 + 16;
    auto kern = k_gemm_tc<NP, OUT>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid(ntiles, (M + BM - 1) / BM, batch);
    kern<<<grid, 128, smem, s>>>(ma0, ma1, mb0, mb1, a);
    count_launch();
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

}  // namespace

bool tc_available() {
    static int cached = -1;
    if (cached < 0) {
        const char* env = getenv("DWGB_DISABLE_TC");
        int dev = 0;
        cudaDeviceProp prop;
        cached = (!(env && env[0] == '1') && cudaGetDevice(&dev) == cudaSuccess &&
                  cudaGetDeviceProperties(&prop, dev) == cudaSuccess && prop.major == 10 && prop.minor == 3 &&
                  encode_fn() != nullptr) ? 1 : 0;
    }
    return cached == 1;
}

int gemm_bf16_tc(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Wt, float* C, int ldc, int M, int N, int K,
                 const GemmEpi& epi, cudaStream_t s) {
    return launch_tc<1, 0>(A, lda, M, Wt, nullptr, C, ldc, M, N, K, epi, 1, 0, 0, s);
}
int gemm_bf16_tc_act(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Wt, __nv_bfloat16* C, int ldc, int M, int N,
                     int K, const GemmEpi& epi, cudaStream_t s) {
    return launch_tc<1, 1>(A, lda, M, Wt, nullptr, C, ldc, M, N, K, epi, 1, 0, 0, s);
}
int gemm_bf16_tc_batched(const __nv_bfloat16* A, int lda, const __nv_bfloat16* Wt, float* C, int ldc, int M, int N, int K,
                         int batch, int64_t sA, int64_t sC, cudaStream_t s) {
    GemmEpi e;
    int64_t rows_per_batch = sA / lda;
    int64_t rows_total = rows_per_batch * (batch - 1) + M;
    return launch_tc<1, 0>(A, lda, rows_total, Wt, nullptr, C, ldc, M, N, K, e, batch, rows_per_batch, sC, s);
}
int gemm_split_tc(const Split* A, int lda, const __nv_bfloat16* Whi, const __nv_bfloat16* Wlo, float* C, int ldc, int M,
                  int N, int K, const GemmEpi& epi, cudaStream_t s) {
    return launch_tc<2, 0>(reinterpret_cast<const __nv_bfloat16*>(A), lda, M, Whi, Wlo, C, ldc, M, N, K, epi, 1, 0, 0, s);
}
int gemm_split_tc_act(const Split* A, int lda, const __nv_bfloat16* Whi, const __nv_bfloat16* Wlo, Split* C, int ldc,
                      int M, int N, int K, const GemmEpi& epi, cudaStream_t s) {
    return launch_tc<2, 2>(reinterpret_cast<const __nv_bfloat16*>(A), lda, M, Whi, Wlo, C, ldc, M, N, K, epi, 1, 0, 0, s);
}
int gemm_split_tc_batched(const Split* A, int lda, const __nv_bfloat16* Whi, const __nv_bfloat16* Wlo, float* C, int ldc,
                          int M, int N, int K, int batch, int64_t rows_per_batch, int64_t sC, cudaStream_t s) {
    GemmEpi e;
    int64_t rows_total = rows_per_batch * (batch - 1) + M;
    return launch_tc<2, 0>(reinterpret_cast<const __nv_bfloat16*>(A), lda, rows_total, Whi, Wlo, C, ldc, M, N, K, e, batch,
                           rows_per_batch, sC, s);
}

}  // namespace dw

extern "C" {

// Test hook: C[M,N] (fp32) = A[M,K] (bf16, row stride lda) @ Wt[N,K]^T (bf16, row stride round_up(K,64)).
// With Wt_lo != NULL, A is split-BF16 ([hi | lo] rows of logical width lda) and W = Wt + Wt_lo.
int dw_debug_gemm_bf16(const void* A, int lda, const void* Wt, const void* Wt_lo, float* C, int ldc, int M, int N, int K,
                       void* stream) {
    if (!dw::tc_available()) return DW_ERR_UNSUPPORTED;
    dw::GemmEpi e;
    if (Wt_lo)
        return dw::gemm_split_tc((const dw::Split*)A, lda, (const __nv_bfloat16*)Wt, (const __nv_bfloat16*)Wt_lo, C, ldc,
                                 M, N, K, e, (cudaStream_t)stream);
    return dw::gemm_bf16_tc((const __nv_bfloat16*)A, lda, (const __nv_bfloat16*)Wt, C, ldc, M, N, K, e, (cudaStream_t)stream);
}

// Reads and clears the device-side error flag of the tensor-core kernels (1 = a bounded wait timed out).
int dw_debug_tc_error_flag(void) {
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, dw::g_tc_error, sizeof(int)) != cudaSuccess) return -1;
    cudaMemcpyToSymbol(dw::g_tc_error, &zero, sizeof(int));
    return v;
}

}  // extern "C"
