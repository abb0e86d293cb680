// Persistent tcgen05 tensor-core GEMM for sm_103a.
//
//   C[M, N] = epilogue( A[M, K] @ W[N, K]^T )
//
// * A and W are BF16 (NP = 1) or split-BF16 (NP = 2: x = hi + lo, three MMAs per K step:
//   A_hi W_hi + A_hi W_lo + A_lo W_hi, all accumulated in FP32 in TMEM).
// * Warp roles (320 threads): warp 0 = TMA producer, warp 1 = MMA issuer (one elected lane),
//   warps 2-9 = epilogue (warp w drains TMEM lanes 32 (w % 4) .. +31; the two warps of a lane
//   quarter take alternate 32-column chunks).
// * Shared-memory ring of S stages (128-byte swizzled K-major tiles), two TMEM accumulators
//   so the epilogue of tile i overlaps the main loop of tile i + 1, one CTA per SM looping
//   over output tiles.
// * Epilogue: value-channel bias, per-(walker, channel) row bias, and either tanh on value
//   rows or the forward-Laplacian tanh across the Tp channel rows of each electron
//   (y = tanh z; y_t = (1 - y^2) z_t; y_lap = (1 - y^2) z_lap - 2 y (1 - y^2) sum_t z_t^2).
//   Results are written to swizzled shared-memory staging tiles (two per warp, so the staging
//   of one chunk overlaps the TMA store of the previous one) and stored with TMA.
// Every mbarrier wait is bounded; on timeout the kernel records an error flag, stops
// issuing, waits (bounded) for its TMA loads in flight, frees its TMEM and returns.
#include "gemm_tc.cuh"
#include <cuda.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>

namespace dw {

__device__ int g_tc_error = 0;

namespace {

constexpr int BM = 128;
constexpr int kEpiWarps = 8;                         // two per TMEM lane quarter
constexpr int kThreads = 64 + 32 * kEpiWarps;        // producer warp, MMA warp, epilogue warps
constexpr int CW = 32;                               // columns per epilogue chunk / staged store box
constexpr uint32_t kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded parity wait: true once the phase with the given parity has completed.
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
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2) : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, const void* src, int c0, int c1, int c2) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%2, %3, %4}], [%1];"
                 ::"l"(map), "r"(smem_u32(src)), "r"(c0), "r"(c1), "r"(c2) : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, const void* src, int c0, int c1) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%2, %3}], [%1];"
                 ::"l"(map), "r"(smem_u32(src)), "r"(c0), "r"(c1) : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// named barriers: 1 = all epilogue warps, 2 + h = the four epilogue warps of column half h
__device__ __forceinline__ void epi_bar() { asm volatile("bar.sync 1, %0;" ::"n"(32 * kEpiWarps) : "memory"); }
__device__ __forceinline__ void half_bar(int h) { asm volatile("bar.sync %0, 128;" ::"r"(2 + h) : "memory"); }

// UMMA shared-memory descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(const void* p) {
    uint64_t addr = smem_u32(p);
    return ((addr & 0x3FFFFull) >> 4) | (1ull << 16) | ((uint64_t)(1024 >> 4) << 32) | (1ull << 46) | (2ull << 61);
}
// K-major, 64-byte swizzle (32 BF16 per row), 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t smem_desc_sw64(const void* p) {
    uint64_t addr = smem_u32(p);
    return ((addr & 0x3FFFFull) >> 4) | (1ull << 16) | ((uint64_t)(512 >> 4) << 32) | (1ull << 46) | (4ull << 61);
}
// Operand tiles of BK K-columns: 64 -> 128-byte rows, 32 -> 64-byte rows.
template <int BK> __device__ __forceinline__ uint64_t smem_desc(const void* p) {
    return BK == 64 ? smem_desc_sw128(p) : smem_desc_sw64(p);
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

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    #pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 16-byte chunk j of row r in a 128-byte-swizzled staging tile (128-byte rows, 1024-byte aligned).
__device__ __forceinline__ uint32_t swz(int r, int j) { return (uint32_t)(r * 128 + ((j ^ (r & 7)) << 4)); }
// 16-byte chunk j (0..3) of row r in a 64-byte-swizzled staging tile (64-byte rows): the chunk
// index is XORed with address bits 7-8, i.e. with (r >> 1) & 3.
__device__ __forceinline__ uint32_t swz64(int r, int j) { return (uint32_t)(r * 64 + ((j ^ ((r >> 1) & 3)) << 4)); }

// Forward-Laplacian scratch per epilogue warp: four per-column arrays for up to four electron
// groups (value-row z and the coefficient rows d1 = 1 - tanh^2, y0 = tanh(z0),
// cl = -2 y0 d1 sum_t z_t^2), pitch kFlP floats (16-byte aligned), then a zero row.
constexpr int kFlP = CW + 4;
constexpr int kFlWarp = 4 * 4 * kFlP + CW;

struct TcArgs {
    int M, N, K, BN;
    GemmEpi epi;
    int fl;             // forward-Laplacian epilogue (rows grouped by Tp channels)
    int n3;             // 3 n_el: channels 1..n3 are gradients, n3 + 1 the Laplacian
    int stages;
    uint32_t tmem_cols;
    int n_tiles_n, n_tiles;
    // Walker-block mode (nrb > 0): A and C are 3-D tensors {K or N, rows per walker block, walkers};
    // M tile mi covers row block (mi % nrb) of 32 rows in walkers 4 (mi / nrb) .. + 3, and epilogue
    // warp q stores the rows of walker 4 (mi / nrb) + q. Plain epilogue only (no bias, tanh or
    // forward-Laplacian rows).
    int nrb;
};

// OUT: 0 = fp32 C, 1 = bf16 C, 2 = split-BF16 C. BK: K-columns per pipeline stage (64 or 32).
template <int NP, int OUT, int BK>
__global__ void __launch_bounds__(kThreads, 1)
k_gemm_tc(const __grid_constant__ CUtensorMap tmA0, const __grid_constant__ CUtensorMap tmA1,
          const __grid_constant__ CUtensorMap tmB0, const __grid_constant__ CUtensorMap tmB1,
          const __grid_constant__ CUtensorMap tmC0, const __grid_constant__ CUtensorMap tmC1, TcArgs a) {
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    constexpr int SWB = 4096;                          // staging bytes per buffer (32 x CW fp32, or BF16 hi + lo)
    const int S = a.stages, BN = a.BN;
    const uint32_t a_bytes = BM * BK * 2, b_bytes = (uint32_t)BN * BK * 2;
    const uint32_t stage_bytes = NP * (a_bytes + b_bytes);
    auto sA = [&](int s, int part) { return smem + (size_t)s * stage_bytes + (size_t)part * a_bytes; };
    auto sB = [&](int s, int part) { return smem + (size_t)s * stage_bytes + (size_t)NP * a_bytes + (size_t)part * b_bytes; };
    uint8_t* stage_out = smem + (size_t)S * stage_bytes;                   // [epilogue warp][2 buffers][SWB]
    float* xchg = reinterpret_cast<float*>(stage_out + 2 * kEpiWarps * SWB); // [half][2 bufs][2 arrays][4][CW]
    float* flbuf = xchg + 2 * 2 * 2 * 4 * CW;                              // [epilogue warp][kFlWarp]
    uint64_t* full = reinterpret_cast<uint64_t*>(flbuf + kEpiWarps * kFlWarp);
    uint64_t* empty = full + S;
    uint64_t* tfull = empty + S;     // [2]
    uint64_t* tempty = tfull + 2;    // [2]
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tempty + 2);
    __shared__ int s_err;
    __shared__ int s_epi_err;   // written only by epilogue warps, read after their named barrier

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nk = (a.K + BK - 1) / BK;

    if (threadIdx.x == 0) {
        s_err = 0;
        s_epi_err = 0;
        for (int s = 0; s < S; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&tfull[b], 1); mbar_init(&tempty[b], kEpiWarps); }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        fence_async_smem();
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

    if (warp == 0) {
        // ---------------- TMA producer
        if (lane == 0) {
            uint32_t cnt = 0;
            uint32_t issued[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            bool err = false;
            for (int tile = blockIdx.x; tile < a.n_tiles && !err; tile += gridDim.x) {
                const int m0 = (tile / a.n_tiles_n) * BM, n0 = (tile % a.n_tiles_n) * BN;
                for (int kt = 0; kt < nk; ++kt, ++cnt) {
                    const int s = cnt % S;
                    const uint32_t use = cnt / S;
                    if (use > 0 && !mbar_wait(&empty[s], (use - 1) & 1)) { err = true; break; }
                    mbar_expect_tx(&full[s], stage_bytes);
                    if (a.nrb) {
                        const int mi = tile / a.n_tiles_n, rb = (mi % a.nrb) * 32, w0 = (mi / a.nrb) * 4;
                        tma_load_3d(sA(s, 0), &tmA0, &full[s], kt * BK, rb, w0);
                        if (NP == 2) tma_load_3d(sA(s, 1), &tmA1, &full[s], kt * BK, rb, w0);
                    } else {
                        tma_load_2d(sA(s, 0), &tmA0, &full[s], kt * BK, m0);
                        if (NP == 2) tma_load_2d(sA(s, 1), &tmA1, &full[s], kt * BK, m0);
                    }
                    tma_load_2d(sB(s, 0), &tmB0, &full[s], kt * BK, n0);
                    if (NP == 2) tma_load_2d(sB(s, 1), &tmB1, &full[s], kt * BK, n0);
                    issued[s] = use + 1;
                }
            }
            if (err) {
                atomicExch(&s_err, 1);
                for (int s = 0; s < S; ++s)          // drain loads still in flight
                    if (issued[s]) mbar_wait(&full[s], (issued[s] - 1) & 1);
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(BN);
            uint32_t cnt = 0, it = 0;
            bool err = false;
            for (int tile = blockIdx.x; tile < a.n_tiles && !err; tile += gridDim.x, ++it) {
                const uint32_t acc = it & 1;
                if (!mbar_wait(&tempty[acc], ((it >> 1) & 1) ^ 1)) { err = true; break; }
                tc_fence_after();
                const uint32_t d = tmem + acc * (uint32_t)BN;
                for (int kt = 0; kt < nk; ++kt, ++cnt) {
                    const int s = cnt % S;
                    if (!mbar_wait(&full[s], (cnt / S) & 1)) { err = true; break; }
                    tc_fence_after();
                    const uint64_t a0 = smem_desc<BK>(sA(s, 0)), b0 = smem_desc<BK>(sB(s, 0));
                    const uint64_t a1 = smem_desc<BK>(sA(s, NP - 1)), b1 = smem_desc<BK>(sB(s, NP - 1));
                    #pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk) {
                        const uint64_t o = (uint64_t)(kk * 2);
                        umma_bf16(d, a0 + o, b0 + o, idesc, (kt | kk) ? 1u : 0u);
                        if (NP == 2) {
                            umma_bf16(d, a0 + o, b1 + o, idesc, 1u);
                            umma_bf16(d, a1 + o, b0 + o, idesc, 1u);
                        }
                    }
                    umma_commit(&empty[s]);
                }
                umma_commit(&tfull[acc]);
            }
            if (err) atomicExch(&s_err, 1);
        }
    } else {
        // ---------------- epilogue warps: warp w drains TMEM lanes 32 (w % 4) .. +31; the two warps
        // of one lane quarter take alternate CW-column chunks (column half h)
        const int q = warp & 3;                      // TMEM lane quarter
        const int ew = warp - 2, h = ew >> 2;        // epilogue warp index, column half
        const GemmEpi& e = a.epi;
        const int Tp = e.Tp;
        uint32_t nchunk = 0;                         // chunks staged by this warp (selects the buffer)
        uint32_t it = 0;
        int xbuf = 0;
        for (int tile = blockIdx.x; tile < a.n_tiles; tile += gridDim.x, ++it) {
            const int m0 = (tile / a.n_tiles_n) * BM, n0 = (tile % a.n_tiles_n) * BN;
            const uint32_t acc = it & 1;
            const int row = q * 32 + lane;           // row within the tile
            const int m = m0 + row;
            const int t = m % Tp;
            const float* rb = (e.rowbias && m < a.M) ? e.rowbias + ((int64_t)(m / e.rows_per_walker) * Tp + t) * e.ldrb
                                                     : nullptr;
            const bool is_val = t == 0, is_grad = t >= 1 && t <= a.n3, is_lap = a.fl && t == a.n3 + 1;
            // bias / row-bias of one CW-column chunk (vectorized; rows of one walker share their
            // row-bias rows, so neighbouring warps hit in L1)
            float rbv[CW];
            auto load_bias = [&](int c0) {
                const bool full_chunk = n0 + c0 + CW <= a.N;
                #pragma unroll
                for (int j = 0; j < CW; j += 4) {
                    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
                    const int n = n0 + c0 + j;
                    if (rb) {
                        if (full_chunk) x = __ldg(reinterpret_cast<const float4*>(rb + n));
                        else {
                            if (n < a.N) x.x = __ldg(rb + n);
                            if (n + 1 < a.N) x.y = __ldg(rb + n + 1);
                            if (n + 2 < a.N) x.z = __ldg(rb + n + 2);
                            if (n + 3 < a.N) x.w = __ldg(rb + n + 3);
                        }
                    }
                    if (e.bias && is_val) {
                        if (full_chunk) {
                            float4 b4 = __ldg(reinterpret_cast<const float4*>(e.bias + n));
                            x.x += b4.x; x.y += b4.y; x.z += b4.z; x.w += b4.w;
                        } else {
                            if (n < a.N) x.x += __ldg(e.bias + n);
                            if (n + 1 < a.N) x.y += __ldg(e.bias + n + 1);
                            if (n + 2 < a.N) x.z += __ldg(e.bias + n + 2);
                            if (n + 3 < a.N) x.w += __ldg(e.bias + n + 3);
                        }
                    }
                    rbv[j] = x.x; rbv[j + 1] = x.y; rbv[j + 2] = x.z; rbv[j + 3] = x.w;
                }
            };
            if (rb) {
                // pull this row's row-bias chunks into L1 while the accumulator is finished
                for (int c0 = h * CW; c0 < BN && n0 + c0 < a.N; c0 += 2 * CW)
                    asm volatile("prefetch.global.L1 [%0];" ::"l"(rb + n0 + c0));
            }
            const bool ready = mbar_wait(&tfull[acc], (it >> 1) & 1);
            if (!ready && lane == 0) s_epi_err = 1;
            epi_bar();                               // all epilogue warps agree before leaving
            if (*(volatile int*)&s_epi_err) { if (lane == 0) atomicExch(&s_err, 1); break; }
            tc_fence_after();
            for (int c0 = h * CW; c0 < BN; c0 += 2 * CW) {
                float v[CW];
                load_bias(c0);                        // issued before the TMEM reads of this chunk
                const uint32_t base = tmem + acc * (uint32_t)BN + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
                #pragma unroll
                for (int j = 0; j < CW; j += 16) tmem_ld16(base + j, v + j);
                tmem_wait_ld();
                #pragma unroll
                for (int j = 0; j < CW; ++j) v[j] += rbv[j];
                // double-buffered staging: the store issued from this buffer two chunks ago has
                // finished reading it once at most one bulk group (the previous chunk's) is pending
                uint8_t* my_out = stage_out + (size_t)(ew * 2 + (nchunk & 1)) * SWB;
                ++nchunk;
                if (lane == 0) bulk_wait_read1();
                __syncwarp();
                if (a.fl) {
                    // Forward-Laplacian tanh over the Tp channel rows of each electron:
                    // y_0 = tanh(z_0), y_t = d1 z_t (gradients), y_lap = d1 z_lap - 2 y0 d1 sum_t z_t^2,
                    // d1 = 1 - y0^2. Gradient rows stage their squares in the swizzled staging tile (free
                    // here: its last TMA store has finished reading it) and the value row its value
                    // in Z0. Lanes add float4 column chunks over 8-row blocks, the blocks of one electron
                    // are combined in-lane, by shuffles or (Tp > 32) across warps, and the lane holding a
                    // group's column sums writes that group's coefficient rows for its four columns.
                    // Each row then takes y = alpha v + beta with coefficient rows chosen by its type.
                    float* sq = reinterpret_cast<float*>(my_out);          // [32 rows][CW] swizzled by 16 B chunks
                    float* fb = flbuf + (size_t)ew * kFlWarp;
                    float* Z0 = fb;                                       // [group][kFlP]
                    float* D1 = fb + 4 * kFlP;
                    float* Y0 = fb + 8 * kFlP;
                    float* CL = fb + 12 * kFlP;
                    float* ZR = fb + 16 * kFlP;                           // zero row
                    const int grp = Tp < 32 ? lane / Tp : 0;
                    #pragma unroll
                    for (int j4 = 0; j4 < CW / 4; ++j4) {
                        const float4 x4 = make_float4(v[4 * j4], v[4 * j4 + 1], v[4 * j4 + 2], v[4 * j4 + 3]);
                        const float4 s4 = is_grad ? make_float4(x4.x * x4.x, x4.y * x4.y, x4.z * x4.z, x4.w * x4.w)
                                                  : make_float4(0.f, 0.f, 0.f, 0.f);
                        *reinterpret_cast<float4*>(sq + lane * CW + ((j4 ^ (lane & 7)) << 2)) = s4;
                        if (is_val) *reinterpret_cast<float4*>(Z0 + grp * kFlP + 4 * j4) = x4;
                    }
                    if (lane < CW / 4) reinterpret_cast<float4*>(ZR)[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
                    __syncwarp();
                    // lane (rb, jc): column chunk jc (columns 4 jc .. 4 jc + 3), rows [rb RPL, (rb + 1) RPL)
                    constexpr int NCH = CW / 4, RPL = NCH, NS = RPL / 8;
                    const int jc = lane % NCH, rbk = lane / NCH;
                    float4 ps[NS];
                    #pragma unroll
                    for (int s8 = 0; s8 < NS; ++s8) {
                        float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
                        #pragma unroll
                        for (int i = 0; i < 8; ++i) {
                            const int r = rbk * RPL + 8 * s8 + i;            // r & 7 == i
                            const float4 y = *reinterpret_cast<const float4*>(sq + r * CW + ((jc ^ i) << 2));
                            x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w;
                        }
                        ps[s8] = x;
                    }
                    auto coeffs = [&](int g, float4 ss, float4 z0) {
                        const float y[4] = {tanhf(z0.x), tanhf(z0.y), tanhf(z0.z), tanhf(z0.w)};
                        const float sv[4] = {ss.x, ss.y, ss.z, ss.w};
                        float d1[4], cl[4];
                        #pragma unroll
                        for (int k = 0; k < 4; ++k) { d1[k] = 1.f - y[k] * y[k]; cl[k] = -2.f * y[k] * d1[k] * sv[k]; }
                        *reinterpret_cast<float4*>(Y0 + g * kFlP + 4 * jc) = make_float4(y[0], y[1], y[2], y[3]);
                        *reinterpret_cast<float4*>(D1 + g * kFlP + 4 * jc) = make_float4(d1[0], d1[1], d1[2], d1[3]);
                        *reinterpret_cast<float4*>(CL + g * kFlP + 4 * jc) = make_float4(cl[0], cl[1], cl[2], cl[3]);
                    };
                    const int gsz = Tp < 32 ? Tp : 32;                      // rows of a group in this warp
                    const int bpg = gsz / 8;                                // 8-row blocks per group
                    if (bpg >= NS) {
                        // all blocks of this lane lie in one group; add the lanes of the same group
                        float4 g4 = ps[0];
                        #pragma unroll
                        for (int s8 = 1; s8 < NS; ++s8) { g4.x += ps[s8].x; g4.y += ps[s8].y; g4.z += ps[s8].z; g4.w += ps[s8].w; }
                        for (int o = NCH; o < NCH * (bpg / NS); o <<= 1) {
                            g4.x += __shfl_xor_sync(0xffffffffu, g4.x, o);
                            g4.y += __shfl_xor_sync(0xffffffffu, g4.y, o);
                            g4.z += __shfl_xor_sync(0xffffffffu, g4.z, o);
                            g4.w += __shfl_xor_sync(0xffffffffu, g4.w, o);
                        }
                        const int g = (rbk * NS) / bpg;
                        const bool holder = (rbk * NS) % bpg == 0;
                        if (Tp <= 32) {
                            if (holder) coeffs(g, g4, *reinterpret_cast<const float4*>(Z0 + g * kFlP + 4 * jc));
                        } else {
                            // a group spans several warps: exchange the partial sums and the value row
                            float* xs = xchg + (size_t)(h * 2 + xbuf) * 2 * 4 * CW;
                            const bool has_val = (q * 32) % Tp == 0;        // this warp holds the value row
                            if (holder) {
                                *reinterpret_cast<float4*>(xs + q * CW + 4 * jc) = g4;
                                if (has_val)
                                    *reinterpret_cast<float4*>(xs + 4 * CW + q * CW + 4 * jc) =
                                        *reinterpret_cast<const float4*>(Z0 + 4 * jc);
                            }
                            half_bar(h);
                            const int qs = Tp / 32, g0 = (q / qs) * qs;
                            if (holder) {
                                float4 tot = make_float4(0.f, 0.f, 0.f, 0.f);
                                for (int k = 0; k < qs; ++k) {
                                    const float4 pk = *reinterpret_cast<const float4*>(xs + (g0 + k) * CW + 4 * jc);
                                    tot.x += pk.x; tot.y += pk.y; tot.z += pk.z; tot.w += pk.w;
                                }
                                coeffs(0, tot, *reinterpret_cast<const float4*>(xs + 4 * CW + g0 * CW + 4 * jc));
                            }
                            xbuf ^= 1;   // the other exchange buffer is written only after the next barrier
                        }
                    } else {
                        // one 8-row block per group (Tp = 8 with 16 rows per lane)
                        #pragma unroll
                        for (int s8 = 0; s8 < NS; ++s8) {
                            const int g = rbk * NS + s8;
                            coeffs(g, ps[s8], *reinterpret_cast<const float4*>(Z0 + g * kFlP + 4 * jc));
                        }
                    }
                    __syncwarp();
                    // row type -> coefficient rows: value (0, y0), gradient (d1, 0), Laplacian
                    // (d1, cl), padding channels (0, 0)
                    const float* al = (is_grad || is_lap) ? D1 + grp * kFlP : ZR;
                    const float* be = is_val ? Y0 + grp * kFlP : (is_lap ? CL + grp * kFlP : ZR);
                    #pragma unroll
                    for (int j4 = 0; j4 < CW / 4; ++j4) {
                        const float4 a4 = *reinterpret_cast<const float4*>(al + 4 * j4);
                        const float4 b4 = *reinterpret_cast<const float4*>(be + 4 * j4);
                        v[4 * j4] = fmaf(a4.x, v[4 * j4], b4.x);
                        v[4 * j4 + 1] = fmaf(a4.y, v[4 * j4 + 1], b4.y);
                        v[4 * j4 + 2] = fmaf(a4.z, v[4 * j4 + 2], b4.z);
                        v[4 * j4 + 3] = fmaf(a4.w, v[4 * j4 + 3], b4.w);
                    }
                    __syncwarp();
                } else if (e.act == 1) {
                    #pragma unroll
                    for (int j = 0; j < CW; ++j) v[j] = tanhf(v[j]);
                }
                // stage the 32 x CW sub-tile (128-byte swizzle for FP32 rows, 64-byte for BF16 rows) and
                // store it with TMA
                if (OUT == 0) {
                    #pragma unroll
                    for (int j = 0; j < 8; ++j)
                        *reinterpret_cast<float4*>(my_out + swz(lane, j)) =
                            make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                } else {
                    #pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        uint32_t hw_[4], lw_[4];
                        #pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            const float x0 = v[8 * j + 2 * k], x1 = v[8 * j + 2 * k + 1];
                            const __nv_bfloat162 hh = __floats2bfloat162_rn(x0, x1);
                            hw_[k] = *reinterpret_cast<const uint32_t*>(&hh);
                            if (OUT == 2) {
                                const __nv_bfloat162 ll = __floats2bfloat162_rn(x0 - __low2float(hh), x1 - __high2float(hh));
                                lw_[k] = *reinterpret_cast<const uint32_t*>(&ll);
                            } else {
                                lw_[k] = 0u;
                            }
                        }
                        *reinterpret_cast<uint4*>(my_out + swz64(lane, j)) = make_uint4(hw_[0], hw_[1], hw_[2], hw_[3]);
                        if (OUT == 2)
                            *reinterpret_cast<uint4*>(my_out + 2048 + swz64(lane, j)) = make_uint4(lw_[0], lw_[1], lw_[2], lw_[3]);
                    }
                }
                fence_async_smem();
                __syncwarp();
                if (lane == 0) {
                    if (a.nrb) {
                        const int mi = tile / a.n_tiles_n;
                        tma_store_3d(&tmC0, my_out, n0 + c0, (mi % a.nrb) * 32, (mi / a.nrb) * 4 + q);
                    } else {
                        tma_store_2d(&tmC0, my_out, n0 + c0, m0 + q * 32);
                        if (OUT == 2) tma_store_2d(&tmC1, my_out + 2048, n0 + c0, m0 + q * 32);
                    }
                    bulk_commit();
                }
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[acc]);
        }
        if (lane == 0) bulk_wait0();
    }
    tc_fence_before();
    __syncthreads();
    if (s_err && threadIdx.x == 0) atomicExch(&g_tc_error, 1);
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

// 2-D tensor map: dims {cols (inner), rows}, row stride ld elements, box {box_cols, box_rows},
// swizzle of box_cols * element size bytes (128 or 64).
int make_map(CUtensorMap* map, const void* base, int64_t rows, int cols, int64_t ld, int box_cols, int box_rows,
             bool f32) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return DW_ERR_UNSUPPORTED;
    const int es = f32 ? 4 : 2;
    const int span = box_cols * es;
    if (((uintptr_t)base & 15) || (ld * es) % 16 || (span != 128 && span != 64)) return DW_ERR_ARG;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * es};
    cuuint32_t box[2] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                    const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    span == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? DW_OK : DW_ERR_ARG;
}

// 3-D tensor map {cols (inner), rows, walkers}: row stride ld and walker stride wstride elements,
// box {box_cols, box_rows, box_w}, swizzle of box_cols * element size bytes (128 or 64).
int make_map3(CUtensorMap* map, const void* base, int64_t nw, int rows, int cols, int64_t ld, int64_t wstride,
              int box_cols, int box_rows, int box_w, bool f32) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return DW_ERR_UNSUPPORTED;
    const int es = f32 ? 4 : 2;
    const int span = box_cols * es;
    if (((uintptr_t)base & 15) || (ld * es) % 16 || (wstride * es) % 16 || (span != 128 && span != 64)) return DW_ERR_ARG;
    cuuint64_t dims[3] = {(cuuint64_t)cols, (cuuint64_t)rows, (cuuint64_t)nw};
    cuuint64_t strides[2] = {(cuuint64_t)ld * es, (cuuint64_t)wstride * es};
    cuuint32_t box[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, (cuuint32_t)box_w};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, f32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                    const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    span == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? DW_OK : DW_ERR_ARG;
}

int num_sms() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 148;
    }
    return n;
}

// A: NP parts of a logical [M, lda] activation (NP = 2: [hi | lo] rows of width 2 lda).
// W0/W1: [N, round_up(K, 64)] K-major weight parts. C: logical [M, ldc].
// wb != nullptr: walker-block mode (FP32 output, plain epilogue); M is then ignored.
// K-columns per stage of the split-BF16 GEMMs (instrumentation: dw_debug_set_gemm_bk).
int g_split_bk = 64;

template <int NP, int OUT, int BK>
int launch_tc(const __nv_bfloat16* A, int lda, const __nv_bfloat16* W0, const __nv_bfloat16* W1, void* C, int ldc,
              int M, int N, int K, const GemmEpi& epi, int fl, int n3, cudaStream_t s, const WalkerBlocks* wb = nullptr) {
    if (wb) {
        if (OUT != 0 || fl || epi.bias || epi.rowbias || epi.act || wb->rows % 32) return DW_ERR_ARG;
        if (wb->nw <= 0) return DW_OK;
        M = ((wb->nw + 3) / 4) * (wb->rows / 32) * BM;
    }
    if (M <= 0 || N <= 0 || K <= 0) return DW_OK;
    constexpr int BN_MAX = NP == 2 ? 128 : 256;      // keeps >= 2 pipeline stages in shared memory
    int ntn = (N + BN_MAX - 1) / BN_MAX;
    int BN = round_up((N + ntn - 1) / ntn, CW);
    while (BN > BN_MAX) { ntn += 1; BN = round_up((N + ntn - 1) / ntn, CW); }
    const int Kp = round_up(K, 64);
    CUtensorMap ma0, ma1, mb0, mb1, mc0, mc1;
    if (wb) {
        DW_CHECK(make_map3(&ma0, A, wb->nw, wb->rows, K, (int64_t)NP * lda, wb->a_wstride, BK, 32, 4, false));
        if (NP == 2) DW_CHECK(make_map3(&ma1, A + lda, wb->nw, wb->rows, K, (int64_t)NP * lda, wb->a_wstride, BK, 32, 4, false));
        else ma1 = ma0;
    } else {
        DW_CHECK(make_map(&ma0, A, M, K, (int64_t)NP * lda, BK, BM, false));
        if (NP == 2) DW_CHECK(make_map(&ma1, A + lda, M, K, (int64_t)NP * lda, BK, BM, false));
        else ma1 = ma0;
    }
    DW_CHECK(make_map(&mb0, W0, N, K, Kp, BK, BN, false));
    if (NP == 2) DW_CHECK(make_map(&mb1, W1, N, K, Kp, BK, BN, false));
    else mb1 = mb0;
    if (wb) {
        DW_CHECK(make_map3(&mc0, C, wb->nw, wb->rows, N, ldc, wb->c_wstride, 32, 32, 1, true));
        mc1 = mc0;
    } else if (OUT == 0) {
        DW_CHECK(make_map(&mc0, C, M, N, ldc, 32, 32, true));
        mc1 = mc0;
    } else if (OUT == 1) {
        DW_CHECK(make_map(&mc0, C, M, N, ldc, 32, 32, false));
        mc1 = mc0;
    } else {
        DW_CHECK(make_map(&mc0, C, M, N, (int64_t)2 * ldc, 32, 32, false));
        DW_CHECK(make_map(&mc1, reinterpret_cast<const __nv_bfloat16*>(C) + ldc, M, N, (int64_t)2 * ldc, 32, 32, false));
    }
    TcArgs a;
    a.M = M; a.N = N; a.K = K; a.BN = BN; a.epi = epi; a.fl = fl; a.n3 = n3;
    a.nrb = wb ? wb->rows / 32 : 0;
    const int stage_bytes = NP * (BM * BK * 2 + BN * BK * 2);
    const int fixed = 1024 + 2 * kEpiWarps * 4096 + 2 * 2 * 2 * 4 * CW * 4 + kEpiWarps * kFlWarp * 4 + 256;
    a.stages = std::min(8, (220 * 1024 - fixed) / stage_bytes);
    if (a.stages < 2) return DW_ERR_ARCH;
    a.tmem_cols = 32;
    while ((int)a.tmem_cols < 2 * BN) a.tmem_cols <<= 1;
    const int mt = (M + BM - 1) / BM;
    a.n_tiles_n = ntn;
    a.n_tiles = mt * ntn;
    size_t smem = (size_t)fixed + (size_t)a.stages * stage_bytes;
    auto kern = k_gemm_tc<NP, OUT, BK>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int grid = std::min(a.n_tiles, num_sms());
    kern<<<grid, kThreads, smem, s>>>(ma0, ma1, mb0, mb1, mc0, mc1, a);
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

int gemm_tc_wb(int np, const void* A, int lda, const __nv_bfloat16* W0, const __nv_bfloat16* W1, float* C, int ldc,
               const WalkerBlocks& wb, int N, int K, cudaStream_t s) {
    const __nv_bfloat16* a = reinterpret_cast<const __nv_bfloat16*>(A);
    GemmEpi e;
    if (np == 1) return launch_tc<1, 0, 64>(a, lda, W0, W1, C, ldc, 0, N, K, e, 0, 0, s, &wb);
    if (np == 2 && g_split_bk == 32) return launch_tc<2, 0, 32>(a, lda, W0, W1, C, ldc, 0, N, K, e, 0, 0, s, &wb);
    if (np == 2) return launch_tc<2, 0, 64>(a, lda, W0, W1, C, ldc, 0, N, K, e, 0, 0, s, &wb);
    return DW_ERR_ARG;
}

int gemm_tc(int np, int out, const void* A, int lda, const __nv_bfloat16* W0, const __nv_bfloat16* W1, void* C, int ldc,
            int M, int N, int K, const GemmEpi& epi, int fl, int n3, cudaStream_t s) {
    const __nv_bfloat16* a = reinterpret_cast<const __nv_bfloat16*>(A);
    if (np == 1 && out == 0) return launch_tc<1, 0, 64>(a, lda, W0, W1, C, ldc, M, N, K, epi, fl, n3, s);
    if (np == 1 && out == 1) return launch_tc<1, 1, 64>(a, lda, W0, W1, C, ldc, M, N, K, epi, fl, n3, s);
    if (g_split_bk == 32) {
        if (np == 2 && out == 0) return launch_tc<2, 0, 32>(a, lda, W0, W1, C, ldc, M, N, K, epi, fl, n3, s);
        if (np == 2 && out == 2) return launch_tc<2, 2, 32>(a, lda, W0, W1, C, ldc, M, N, K, epi, fl, n3, s);
    }
    if (np == 2 && out == 0) return launch_tc<2, 0, 64>(a, lda, W0, W1, C, ldc, M, N, K, epi, fl, n3, s);
    if (np == 2 && out == 2) return launch_tc<2, 2, 64>(a, lda, W0, W1, C, ldc, M, N, K, epi, fl, n3, s);
    return DW_ERR_ARG;
}

}  // namespace dw

extern "C" {

// Test hook: C[M,N] (fp32) = A[M,K] (bf16, row stride lda) @ Wt[N,K]^T (bf16, row stride round_up(K,64)).
// With Wt_lo != NULL, A is split-BF16 ([hi | lo] rows of logical width lda) and W = Wt + Wt_lo.
int dw_debug_gemm_bf16(const void* A, int lda, const void* Wt, const void* Wt_lo, float* C, int ldc, int M, int N, int K,
                       void* stream) {
    if (!dw::tc_available()) return DW_ERR_UNSUPPORTED;
    dw::GemmEpi e;
    return dw::gemm_tc(Wt_lo ? 2 : 1, 0, A, lda, (const __nv_bfloat16*)Wt, (const __nv_bfloat16*)Wt_lo, C, ldc, M, N, K,
                       e, 0, 0, (cudaStream_t)stream);
}

// Instrumentation: K-columns per pipeline stage of the split-BF16 GEMMs (64: two stages of 64 KB at
// N tiles of 128; 32: four stages of 32 KB). Returns the previous value; other values are ignored.
int dw_debug_set_gemm_bk(int bk) {
    const int prev = dw::g_split_bk;
    if (bk == 32 || bk == 64) dw::g_split_bk = bk;
    return prev;
}

// Reads and clears the device-side error flag of the tensor-core kernels (1 = a bounded wait timed out).
int dw_debug_tc_error_flag(void) {
    int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, dw::g_tc_error, sizeof(int)) != cudaSuccess) return -1;
    cudaMemcpyToSymbol(dw::g_tc_error, &zero, sizeof(int));
    return v;
}

}  // extern "C"
