// FP32 CUDA-core GEMM for the plain (FP32 end-to-end) form: C = A @ W with the
// per-row epilogues of the network (value-channel bias, per-walker-channel row bias,
// optional tanh for value-only rows). No TF32: the reference disables it
// (NVIDIA_TF32_OVERRIDE=0, process_molecule.py:20-29).
#include "net.cuh"
#include <algorithm>

namespace dw {

static int num_sms_simt() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 148;
    }
    return n;
}

template <int BM, int BN, int BK, int TM, int TN, bool TRANS_W = false, bool ACC = false>
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
            Ws[buf][kk][cc] = (gk < K && gn < N) ? __ldg(TRANS_W ? W + (int64_t)gn * ldw + gk : W + (int64_t)gk * ldw + gn)
                                                 : 0.f;
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
            if (ACC) C[(int64_t)m * ldc + n] += v;
            else C[(int64_t)m * ldc + n] = v;
        }
    }
}

// Wide shapes (N >= 128, K and the leading dimensions multiples of 4, 16-byte aligned operands):
// 128 x 128 tiles, 256 threads with an 8 x 8 patch each (two 4-wide groups per direction, so a
// warp's 16-byte shared reads are consecutive: 4 LDS.128 feed 64 FMAs), 16-byte global loads
// staged through registers into double-buffered shared memory. Same epilogue as k_gemm_f32.
template <bool TRANS_W, bool ACC>
__global__ void __launch_bounds__(256)
k_gemm_f32v(const float* __restrict__ A, int lda, const float* __restrict__ W, int ldw, float* __restrict__ C, int ldc,
            int M, int N, int K, GemmEpi epi, int64_t sA, int64_t sC) {
    constexpr int BM = 128, BN = 128, BK = 8;
    A += blockIdx.z * sA;
    C += blockIdx.z * sC;
    __shared__ __align__(16) float As[2][BK][BM];
    __shared__ __align__(16) float Ws[2][BK][BN];
    const int tid = threadIdx.x, tr = tid / 16, tc = tid % 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    float acc[8][8];
    #pragma unroll
    for (int i = 0; i < 8; ++i)
        #pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
    // per thread: one float4 of A (row tid / 2, k half tid % 2) and one of W
    const int ar = tid / 2, ah = (tid % 2) * 4;
    const int wk = tid / 32, wn = (tid % 32) * 4;          // non-transposed W: [K][N]
    float4 ra, rw;
    auto gload = [&](int k0) {
        const int gm = m0 + ar, gk = k0 + ah;
        ra = (gm < M && gk < K) ? __ldg(reinterpret_cast<const float4*>(A + (int64_t)gm * lda + gk))
                                : make_float4(0.f, 0.f, 0.f, 0.f);
        if (TRANS_W) {
            const int gn = n0 + ar;
            rw = (gn < N && gk < K) ? __ldg(reinterpret_cast<const float4*>(W + (int64_t)gn * ldw + gk))
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
        } else {
            const int kk = k0 + wk, gn = n0 + wn;
            rw = (kk < K && gn < N) ? __ldg(reinterpret_cast<const float4*>(W + (int64_t)kk * ldw + gn))
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    auto sstore = [&](int buf) {
        As[buf][ah + 0][ar] = ra.x; As[buf][ah + 1][ar] = ra.y; As[buf][ah + 2][ar] = ra.z; As[buf][ah + 3][ar] = ra.w;
        if (TRANS_W) {
            Ws[buf][ah + 0][ar] = rw.x; Ws[buf][ah + 1][ar] = rw.y; Ws[buf][ah + 2][ar] = rw.z; Ws[buf][ah + 3][ar] = rw.w;
        } else {
            *reinterpret_cast<float4*>(&Ws[buf][wk][wn]) = rw;
        }
    };
    const int nk = (K + BK - 1) / BK;
    gload(0);
    sstore(0);
    __syncthreads();
    for (int kt = 0; kt < nk; ++kt) {
        const int buf = kt & 1;
        if (kt + 1 < nk) gload((kt + 1) * BK);
        #pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][4 * tr]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + 4 * tr]);
            const float4 b0 = *reinterpret_cast<const float4*>(&Ws[buf][kk][4 * tc]);
            const float4 b1 = *reinterpret_cast<const float4*>(&Ws[buf][kk][64 + 4 * tc]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float b[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
            #pragma unroll
            for (int i = 0; i < 8; ++i)
                #pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        if (kt + 1 < nk) sstore(buf ^ 1);
        __syncthreads();
    }
    #pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int m = m0 + (i < 4 ? 4 * tr + i : 64 + 4 * tr + i - 4);
        if (m >= M) continue;
        const int t = m % epi.Tp;
        const float* rb = epi.rowbias ? epi.rowbias + ((int64_t)(m / epi.rows_per_walker) * epi.Tp + t) * epi.ldrb : nullptr;
        #pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + (j < 4 ? 4 * tc + j : 64 + 4 * tc + j - 4);
            if (n >= N) continue;
            float v = acc[i][j];
            if (epi.bias && t == 0) v += epi.bias[n];
            if (rb) v += rb[n];
            if (epi.act == 1) v = tanhf(v);
            if (ACC) C[(int64_t)m * ldc + n] += v;
            else C[(int64_t)m * ldc + n] = v;
        }
    }
}

static bool vec_ok(const float* A, int lda, const float* W, int ldw, int N, int K, bool trans_w) {
    auto al = [](const void* p) { return ((uintptr_t)p & 15) == 0; };
    return N >= 128 && K % 4 == 0 && lda % 4 == 0 && ldw % 4 == 0 && al(A) && al(W) && (trans_w || N % 4 == 0);
}

void gemm_f32(const float* A, int lda, const float* W, int ldw, float* C, int ldc, int M, int N, int K,
              const GemmEpi& epi, int batch, int64_t sA, int64_t sC, cudaStream_t s) {
    if (M <= 0 || N <= 0) return;
    if (vec_ok(A, lda, W, ldw, N, K, false) && (batch == 1 || (sA % 4 == 0))) {
        dim3 g((N + 127) / 128, (M + 127) / 128, batch);
        k_gemm_f32v<false, false><<<g, 256, 0, s>>>(A, lda, W, ldw, C, ldc, M, N, K, epi, sA, sC);
        count_launch();
        return;
    }
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

void gemm_f32_nt(const float* A, int lda, const float* W, int ldw, float* C, int ldc, int M, int N, int K,
                 int accumulate, cudaStream_t s) {
    if (M <= 0 || N <= 0) return;
    GemmEpi epi;
    if (vec_ok(A, lda, W, ldw, N, K, true)) {
        dim3 g((N + 127) / 128, (M + 127) / 128, 1);
        if (accumulate) k_gemm_f32v<true, true><<<g, 256, 0, s>>>(A, lda, W, ldw, C, ldc, M, N, K, epi, 0, 0);
        else k_gemm_f32v<true, false><<<g, 256, 0, s>>>(A, lda, W, ldw, C, ldc, M, N, K, epi, 0, 0);
        count_launch();
        return;
    }
    constexpr int BM = 128, BN = 64;
    dim3 g((N + BN - 1) / BN, (M + BM - 1) / BM, 1);
    if (accumulate)
        k_gemm_f32<BM, BN, 8, 8, 4, true, true><<<g, (BM / 8) * (BN / 4), 0, s>>>(A, lda, W, ldw, C, ldc, M, N, K, epi, 0, 0);
    else
        k_gemm_f32<BM, BN, 8, 8, 4, true, false><<<g, (BM / 8) * (BN / 4), 0, s>>>(A, lda, W, ldw, C, ldc, M, N, K, epi, 0, 0);
    count_launch();
}

// Weight gradient for narrow shapes: 64 x 64 output tiles, 32-row slabs, a 4 x 4 patch per thread.
__global__ void __launch_bounds__(256)
k_wgrad_f32_64(const float* __restrict__ A, int lda, const float* __restrict__ G, int ldg, int rows, int K, int N,
            float* __restrict__ dW, int lddw, float* __restrict__ dB, const int8_t* __restrict__ sel, int want,
            int rows_per_seg) {
    __shared__ float As[32][64 + 1];
    __shared__ float Gs[32][64 + 1];
    const int k0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    const int r_begin = blockIdx.z * rows_per_seg, r_end = min(rows, r_begin + rows_per_seg);
    const int tid = threadIdx.x, tk = tid / 16, tn = tid % 16;
    float acc[4][4] = {{0.f}};
    float bacc[4] = {0.f, 0.f, 0.f, 0.f};
    for (int r0 = r_begin; r0 < r_end; r0 += 32) {
        for (int e = tid; e < 32 * 64; e += 256) {
            const int rr = e / 64, cc = e % 64, r = r0 + rr;
            bool ok = r < r_end && (!sel || sel[r] == want);
            As[rr][cc] = (ok && k0 + cc < K) ? A[(int64_t)r * lda + k0 + cc] : 0.f;
            Gs[rr][cc] = (ok && n0 + cc < N) ? G[(int64_t)r * ldg + n0 + cc] : 0.f;
        }
        __syncthreads();
        #pragma unroll 4
        for (int rr = 0; rr < 32; ++rr) {
            float a[4], g[4];
            #pragma unroll
            for (int u = 0; u < 4; ++u) { a[u] = As[rr][tk + 16 * u]; g[u] = Gs[rr][tn + 16 * u]; }
            #pragma unroll
            for (int u = 0; u < 4; ++u)
                #pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fmaf(a[u], g[v], acc[u][v]);
            if (dB && blockIdx.y == 0 && tk == 0) {
                #pragma unroll
                for (int v = 0; v < 4; ++v) bacc[v] += g[v];
            }
        }
        __syncthreads();
    }
    #pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int k = k0 + tk + 16 * u;
        if (k >= K) continue;
        #pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int n = n0 + tn + 16 * v;
            if (n < N) atomicAdd(dW + (int64_t)k * lddw + n, acc[u][v]);
        }
    }
    if (dB && blockIdx.y == 0 && tk == 0) {
        #pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int n = n0 + tn + 16 * v;
            if (n < N) atomicAdd(dB + n, bacc[v]);
        }
    }
}

// Weight gradient dW[K, N] += sum_r A[r, k] G[r, n]: 128 x 128 output tiles, rows split into
// segments over grid.z and accumulated atomically; each block stages 16-row slabs of A and G in
// shared memory and accumulates an 8 x 8 patch per thread.
__global__ void __launch_bounds__(256)
k_wgrad_f32(const float* __restrict__ A, int lda, const float* __restrict__ G, int ldg, int rows, int K, int N,
            float* __restrict__ dW, int lddw, float* __restrict__ dB, const int8_t* __restrict__ sel, int want,
            int rows_per_seg) {
    // 128 x 128 tile of dW per block, 8 x 8 per thread (two 4-wide groups in each direction so that
    // the 16-byte shared-memory reads of a warp are consecutive), 16 rows staged per step.
    constexpr int TB = 128, RB = 16;
    __shared__ __align__(16) float As[RB][TB];
    __shared__ __align__(16) float Gs[RB][TB];
    const int k0 = blockIdx.y * TB, n0 = blockIdx.x * TB;
    const int r_begin = blockIdx.z * rows_per_seg, r_end = min(rows, r_begin + rows_per_seg);
    const int tid = threadIdx.x, tk = tid / 16, tn = tid % 16;
    float acc[8][8];
    #pragma unroll
    for (int u = 0; u < 8; ++u)
        #pragma unroll
        for (int v = 0; v < 8; ++v) acc[u][v] = 0.f;
    float bacc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    const bool do_bias = dB && blockIdx.y == 0 && tk == 0;
    for (int r0 = r_begin; r0 < r_end; r0 += RB) {
        for (int e = tid; e < RB * TB; e += 256) {
            const int rr = e / TB, cc = e % TB, r = r0 + rr;
            const bool ok = r < r_end && (!sel || sel[r] == want);
            As[rr][cc] = (ok && k0 + cc < K) ? __ldg(A + (int64_t)r * lda + k0 + cc) : 0.f;
            Gs[rr][cc] = (ok && n0 + cc < N) ? __ldg(G + (int64_t)r * ldg + n0 + cc) : 0.f;
        }
        __syncthreads();
        #pragma unroll 2
        for (int rr = 0; rr < RB; ++rr) {
            const float4 a0 = *reinterpret_cast<const float4*>(&As[rr][4 * tk]);
            const float4 a1 = *reinterpret_cast<const float4*>(&As[rr][64 + 4 * tk]);
            const float4 g0 = *reinterpret_cast<const float4*>(&Gs[rr][4 * tn]);
            const float4 g1 = *reinterpret_cast<const float4*>(&Gs[rr][64 + 4 * tn]);
            const float a[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float g[8] = {g0.x, g0.y, g0.z, g0.w, g1.x, g1.y, g1.z, g1.w};
            #pragma unroll
            for (int u = 0; u < 8; ++u)
                #pragma unroll
                for (int v = 0; v < 8; ++v) acc[u][v] = fmaf(a[u], g[v], acc[u][v]);
            if (do_bias) {
                #pragma unroll
                for (int v = 0; v < 8; ++v) bacc[v] += g[v];
            }
        }
        __syncthreads();
    }
    #pragma unroll
    for (int u = 0; u < 8; ++u) {
        const int k = k0 + (u < 4 ? 4 * tk + u : 64 + 4 * tk + u - 4);
        if (k >= K) continue;
        #pragma unroll
        for (int v = 0; v < 8; ++v) {
            const int n = n0 + (v < 4 ? 4 * tn + v : 64 + 4 * tn + v - 4);
            if (n < N) atomicAdd(dW + (int64_t)k * lddw + n, acc[u][v]);
        }
    }
    if (do_bias) {
        #pragma unroll
        for (int v = 0; v < 8; ++v) {
            const int n = n0 + (v < 4 ? 4 * tn + v : 64 + 4 * tn + v - 4);
            if (n < N) atomicAdd(dB + n, bacc[v]);
        }
    }
}

// Narrow weight gradients (K, N <= 32), one pass over the rows for up to two outputs: rows with
// sel[r] == 1 go to (dW1, dB1), the others to (dW0, dB0) (sel == NULL: all rows to output 0).
// 256 threads = 4 row groups x 64 threads; a thread keeps a 4 x 4 patch of each 32 x 32 output
// (two float4 shared loads feed 16 FMAs per row), the row groups are added in shared memory and
// each block adds its segment with one atomic per output element.
__global__ void __launch_bounds__(256)
k_wgrad32(const float* __restrict__ A, int lda, const float* __restrict__ G, int ldg, int rows, int K, int N,
          const int8_t* __restrict__ sel, float* __restrict__ dW0, float* __restrict__ dB0, float* __restrict__ dW1,
          float* __restrict__ dB1, int lddw, int rows_per_seg) {
    constexpr int RS = 32;                               // rows per shared-memory slab
    __shared__ __align__(16) float As[RS][36];
    __shared__ __align__(16) float Gs[RS][36];
    __shared__ int8_t ss[RS];
    __shared__ __align__(16) float red[4][2][32][33];
    const int tid = threadIdx.x, grp = tid >> 6, t64 = tid & 63, kb = t64 >> 3, nb = t64 & 7;
    const int r_begin = blockIdx.x * rows_per_seg, r_end = min(rows, r_begin + rows_per_seg);
    float acc[2][4][4], bacc[2][4];
    #pragma unroll
    for (int o = 0; o < 2; ++o) {
        #pragma unroll
        for (int u = 0; u < 4; ++u) {
            bacc[o][u] = 0.f;
            #pragma unroll
            for (int v = 0; v < 4; ++v) acc[o][u][v] = 0.f;
        }
    }
    for (int r0 = r_begin; r0 < r_end; r0 += RS) {
        for (int e = tid; e < RS * 32; e += 256) {
            const int rr = e >> 5, cc = e & 31, r = r0 + rr;
            const bool ok = r < r_end;
            As[rr][cc] = (ok && cc < K) ? __ldg(A + (int64_t)r * lda + cc) : 0.f;
            Gs[rr][cc] = (ok && cc < N) ? __ldg(G + (int64_t)r * ldg + cc) : 0.f;
        }
        if (tid < RS) ss[tid] = (sel && r0 + tid < r_end) ? (sel[r0 + tid] == 1 ? 1 : 0) : 0;
        __syncthreads();
        #pragma unroll 2
        for (int rr = grp; rr < RS; rr += 4) {
            const float4 a4 = *reinterpret_cast<const float4*>(&As[rr][4 * kb]);
            const float4 g4 = *reinterpret_cast<const float4*>(&Gs[rr][4 * nb]);
            const float a[4] = {a4.x, a4.y, a4.z, a4.w}, g[4] = {g4.x, g4.y, g4.z, g4.w};
            if (ss[rr]) {
                #pragma unroll
                for (int u = 0; u < 4; ++u)
                    #pragma unroll
                    for (int v = 0; v < 4; ++v) acc[1][u][v] = fmaf(a[u], g[v], acc[1][u][v]);
                #pragma unroll
                for (int v = 0; v < 4; ++v) bacc[1][v] += g[v];
            } else {
                #pragma unroll
                for (int u = 0; u < 4; ++u)
                    #pragma unroll
                    for (int v = 0; v < 4; ++v) acc[0][u][v] = fmaf(a[u], g[v], acc[0][u][v]);
                #pragma unroll
                for (int v = 0; v < 4; ++v) bacc[0][v] += g[v];
            }
        }
        __syncthreads();
    }
    const int nout = sel ? 2 : 1;
    for (int o = 0; o < nout; ++o) {
        #pragma unroll
        for (int u = 0; u < 4; ++u)
            #pragma unroll
            for (int v = 0; v < 4; ++v) red[grp][o][4 * kb + u][4 * nb + v] = acc[o][u][v];
    }
    __syncthreads();
    for (int e = tid; e < nout * 1024; e += 256) {
        const int o = e >> 10, k = (e >> 5) & 31, n = e & 31;
        if (k >= K || n >= N) continue;
        const float v = red[0][o][k][n] + red[1][o][k][n] + red[2][o][k][n] + red[3][o][k][n];
        atomicAdd((o ? dW1 : dW0) + (int64_t)k * lddw + n, v);
    }
    // bias: the kb == 0 threads of each row group hold the column sums of G
    __syncthreads();
    if (kb == 0) {
        for (int o = 0; o < nout; ++o)
            #pragma unroll
            for (int v = 0; v < 4; ++v) red[grp][o][0][4 * nb + v] = bacc[o][v];
    }
    __syncthreads();
    for (int e = tid; e < nout * 32; e += 256) {
        const int o = e >> 5, n = e & 31;
        float* dB = o ? dB1 : dB0;
        if (!dB || n >= N) continue;
        atomicAdd(dB + n, red[0][o][0][n] + red[1][o][0][n] + red[2][o][0][n] + red[3][o][0][n]);
    }
}

void wgrad32_sel2(const float* A, int lda, const float* G, int ldg, int rows, int K, int N, const int8_t* sel,
                  float* dW0, float* dB0, float* dW1, float* dB1, int lddw, cudaStream_t s) {
    if (rows <= 0 || K <= 0 || N <= 0) return;
    int segs = std::max(1, std::min((rows + 127) / 128, 2 * num_sms_simt()));
    int rps = (rows + segs - 1) / segs;
    rps = (rps + 31) / 32 * 32;
    segs = (rows + rps - 1) / rps;
    k_wgrad32<<<segs, 256, 0, s>>>(A, lda, G, ldg, rows, K, N, sel, dW0, dB0, dW1, dB1, lddw, rps);
    count_launch();
}

void wgrad_f32(const float* A, int lda, const float* G, int ldg, int rows, int K, int N, float* dW, int lddw,
               float* dB, const int8_t* sel, int want, cudaStream_t s) {
    if (rows <= 0 || K <= 0 || N <= 0) return;
    if (K <= 32 && N <= 32 && !sel) {
        wgrad32_sel2(A, lda, G, ldg, rows, K, N, nullptr, dW, dB, nullptr, nullptr, lddw, s);
        return;
    }
    if (K < 128 || N < 128) {
        // narrow shapes: 64 x 64 tiles waste less of each thread's patch
        const int tiles = ((K + 63) / 64) * ((N + 63) / 64);
        int segs = std::max(1, std::min((rows + 255) / 256, (4 * num_sms_simt() + tiles - 1) / tiles));
        int rps = (rows + segs - 1) / segs;
        rps = (rps + 31) / 32 * 32;
        segs = (rows + rps - 1) / rps;
        dim3 g((N + 63) / 64, (K + 63) / 64, segs);
        k_wgrad_f32_64<<<g, 256, 0, s>>>(A, lda, G, ldg, rows, K, N, dW, lddw, dB, sel, want, rps);
        count_launch();
        return;
    }
    const int tiles = ((K + 127) / 128) * ((N + 127) / 128);
    // row segments: enough blocks for two waves over the SMs, at least 64 rows per segment
    int segs = std::max(1, std::min((rows + 63) / 64, (2 * num_sms_simt() + tiles - 1) / tiles));
    int rps = (rows + segs - 1) / segs;
    rps = (rps + 15) / 16 * 16;
    segs = (rows + rps - 1) / rps;
    dim3 g((N + 127) / 128, (K + 127) / 128, segs);
    k_wgrad_f32<<<g, 256, 0, s>>>(A, lda, G, ldg, rows, K, N, dW, lddw, dB, sel, want, rps);
    count_launch();
}

}  // namespace dw
