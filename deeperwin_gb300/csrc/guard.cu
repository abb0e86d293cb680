// Re-evaluation of the ill-conditioned tail of the mixed form's local energies.
//
// The split-BF16 GEMMs of the mixed form carry about 2^-16 relative error per Slater-matrix entry;
// the forward Laplacian turns entry errors into E_L errors amplified by the cancellations of the
// kinetic term (|grad log psi|^2 against Lap log psi near the nodes, and between the determinants
// of the sum). For nearly all walkers that stays below a mHa; for the walkers near a node of the
// wavefunction it reaches Hartrees and dominates the mean energy. The combine kernel reports per
// walker the magnitude of the terms it cancels; walkers whose predicted error (that magnitude
// times the form's relative entry accuracy) exceeds a threshold are gathered into a fixed-capacity
// sub-batch (no host synchronisation), re-evaluated with FP64 determinant algebra, and their E_L,
// log psi^2 and gradient are scattered back. The selection depends only on each walker's own scales, so a walker gets the
// same result in any batch as long as the flagged walkers fit the capacity; beyond it the walkers
// with the largest predicted errors are taken.
#include "net.cuh"
#include <algorithm>

namespace dw {

__device__ unsigned long long g_guard_walkers = 0, g_guard_flagged = 0, g_guard_overflow = 0;

// Predicted E_L error of a mixed-form walker: kGuardRel times the largest magnitude the combine
// kernel cancels (the determinant terms of the Laplacian of log|psi~|, or the terms of E_L). On
// C2H4-shaped walkers (16 electrons, 32 determinants) the measured |E_mixed - E_FP64| / that
// magnitude has median 1.7e-6 and 99th percentile 1.5e-5 (2e-5 to 5e-5 after optimisation steps).
// Walkers predicted above kGuardTol (magnitude above 2,000 Ha) are re-evaluated, those of the
// largest magnitudes first when more than the capacity (1 / 32 of the batch) are flagged.
constexpr float kGuardRel = 1.5e-5f;
constexpr float kGuardTol = 0.03f;
// Re-evaluation form: the plain FP32 network with FP64 determinant algebra (LU, inverse, tangent
// traces). The catastrophic errors of ill-conditioned walkers come from the determinant algebra:
// on 4,096 C2H4-shaped walkers near the initial weights the plain FP32 form is off by up to 14 Ha,
// the same network with FP64 determinants by at most 95 mHa (mean 0.03 mHa), at about 1.5x the
// plain form's cost per walker. The FP64 form (fp64.cu) would cost about 15x more per walker.
constexpr bool kGuardFp64 = false;

// Sort key of a walker (larger = re-evaluate first); NaN scales rank first.
__device__ __forceinline__ float guard_key(const float* sc) {
    const float m = fmaxf(sc[0], sc[1]);
    return m == m ? m : INFINITY;
}

// Flagged walkers into idx[0 .. min(count, cap)), in walker order (one block, deterministic).
// When more than cap are flagged, the walkers with the largest keys are taken: t is the smallest key
// (float bit pattern, binary search) with #{key >= t} <= cap; the walkers with key >= t come first
// and walkers whose key equals the next lower bit pattern (ties, including NaN scales ranked as
// infinity) fill the remaining slots in walker order. counts[0] = walkers to re-evaluate,
// counts[1] = walkers flagged.
__global__ void __launch_bounds__(1024)
k_guard_select(const float* __restrict__ esc, int B, float rel, float tol, int cap, int* __restrict__ idx,
               int* __restrict__ counts) {
    __shared__ int warp_tot[32];
    __shared__ int base;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t thr_flag = __float_as_uint(tol / rel);
    auto key_bits = [&](int b) { return __float_as_uint(guard_key(esc + 3 * (int64_t)b)); };
    // block-wide count of walkers whose key bits are >= t
    auto count_ge = [&](uint32_t t) {
        int c = 0;
        for (int b = threadIdx.x; b < B; b += blockDim.x) c += key_bits(b) >= t;
        c = __reduce_add_sync(0xffffffffu, c);
        __syncthreads();
        if (lane == 0) warp_tot[wid] = c;
        __syncthreads();
        int tot = 0;
        for (int w = 0; w < nw; ++w) tot += warp_tot[w];
        return tot;
    };
    // appends the walkers selected by `pick` in walker order while slots are left
    auto compact = [&](auto pick) {
        for (int b0 = 0; b0 < B; b0 += blockDim.x) {
            const int b = b0 + threadIdx.x;
            const bool f = b < B && pick(b);
            const unsigned m = __ballot_sync(0xffffffffu, f);
            if (lane == 0) warp_tot[wid] = __popc(m);
            __syncthreads();
            int off = base;
            for (int w = 0; w < wid; ++w) off += warp_tot[w];
            const int pos = off + __popc(m & ((1u << lane) - 1u));
            if (f && pos < cap) idx[pos] = b;
            __syncthreads();
            if (threadIdx.x == 0) {
                int tt = 0;
                for (int w = 0; w < nw; ++w) tt += warp_tot[w];
                base += tt;
            }
            __syncthreads();
        }
    };
    // keys are non-negative floats: their bit patterns order as the values
    uint32_t t = thr_flag + 1u;                       // key > tol / rel
    const int flagged = count_ge(t);
    bool fill = false;
    if (flagged > cap) {
        uint32_t lo = t, hi = 0x7F800001u;            // count_ge(hi) = 0 <= cap
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (count_ge(mid) <= cap) hi = mid; else lo = mid + 1;
        }
        fill = lo > t;                                // count_ge(lo - 1) > cap: ties at lo - 1
        t = lo;
    }
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    compact([&](int b) { return key_bits(b) >= t; });
    if (fill) {
        const uint32_t tie = t - 1u;
        compact([&](int b) { return key_bits(b) == tie; });
    }
    if (threadIdx.x == 0) {
        const int sel = min(base, cap);
        counts[0] = sel;
        counts[1] = flagged;
        atomicAdd(&g_guard_walkers, (unsigned long long)B);
        atomicAdd(&g_guard_flagged, (unsigned long long)flagged);
        if (flagged > sel) atomicAdd(&g_guard_overflow, (unsigned long long)(flagged - sel));
    }
}

__global__ void k_guard_gather(const float* __restrict__ r, const int32_t* __restrict__ seg, const int* __restrict__ idx,
                               const int* __restrict__ counts, int n3, float* __restrict__ r_sub,
                               int32_t* __restrict__ seg_sub, int cap, int fill) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = (int)(e / n3), c = (int)(e % n3);
    if (k >= cap || (!fill && k >= counts[0])) return;
    const int b = k < counts[0] ? idx[k] : 0;
    r_sub[(int64_t)k * n3 + c] = r[(int64_t)b * n3 + c];
    if (seg && c == 0) seg_sub[k] = seg[b];
}

__global__ void k_guard_scatter(const float* __restrict__ E_sub, const float* __restrict__ lp_sub,
                                const float* __restrict__ g_sub, const int* __restrict__ idx,
                                const int* __restrict__ counts, int n3, int cap, float* __restrict__ E,
                                float* __restrict__ lp, float* __restrict__ grad) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int k = (int)(e / n3), c = (int)(e % n3);
    if (k >= cap || k >= counts[0]) return;
    const int b = idx[k];
    if (c == 0) {
        E[b] = E_sub[k];
        if (lp) lp[b] = lp_sub[k];
    }
    if (grad) grad[(int64_t)b * n3 + c] = g_sub[(int64_t)k * n3 + c];
}

int guard_capacity(const DwArch* a, int B) {
    // up to 1 / 32 of the batch (at least 16); the FP64 form needs the flagged walkers in one chunk
    // (its kernels skip the unused capacity through the device-side count), the FP32 network with
    // FP64 determinants runs over the whole capacity (unused slots hold a copy of walker 0)
    const int want = std::min(B, std::max(16, (B + 31) / 32));
    return kGuardFp64 ? std::max(1, std::min(want, fp64_max_chunk(a, true))) : want;
}

struct GuardPlan {
    int cap;
    int* idx; int* counts; float* r_sub; int32_t* seg_sub; float* E_sub; float* lp_sub; float* g_sub;
    void* fp64_ws; size_t fp64_bytes;
    size_t bytes;
};

static GuardPlan carve_guard(const DwArch* a, int B, void* ws) {
    GuardPlan g;
    const int n3 = 3 * a->n_el;
    g.cap = guard_capacity(a, B);
    Carver c(ws, (size_t)-1);
    g.idx = c.take<int>((size_t)g.cap);
    g.counts = c.take<int>(2);
    g.r_sub = c.take<float>((size_t)g.cap * n3);
    g.seg_sub = c.take<int32_t>((size_t)g.cap);
    g.E_sub = c.take<float>((size_t)g.cap);
    g.lp_sub = c.take<float>((size_t)g.cap);
    g.g_sub = c.take<float>((size_t)g.cap * n3);
    g.fp64_bytes = kGuardFp64 ? fp64_plan_bytes(a, g.cap, true) : det64_plan_bytes(a, g.cap);
    g.fp64_ws = c.take<unsigned char>(g.fp64_bytes);
    g.bytes = c.used + 256;
    return g;
}

size_t guard_bytes(const DwArch* a, int B) { return carve_guard(a, B, nullptr).bytes; }

int tail_guard(const DwArch* a, const float* P, const void* prepared, const float* r, int B, const float* R,
               const int32_t* Z, const int32_t* seg, int nseg, const float* esc, float* E, float* lp, float* grad,
               void* ws, size_t wsb, cudaStream_t s) {
    GuardPlan g = carve_guard(a, B, ws);
    if (g.bytes > wsb) return DW_ERR_WORKSPACE;
    const int n3 = 3 * a->n_el;
    k_guard_select<<<1, 1024, 0, s>>>(esc, B, kGuardRel, kGuardTol, g.cap, g.idx, g.counts);
    count_launch();
    const int64_t ne = (int64_t)g.cap * n3;
    k_guard_gather<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(r, seg, g.idx, g.counts, n3, g.r_sub,
                                                                 seg ? g.seg_sub : nullptr, g.cap, kGuardFp64 ? 0 : 1);
    count_launch();
    if (kGuardFp64)
        DW_CHECK(fp64_forward_all(a, P, prepared, g.r_sub, g.cap, R, Z, g.lp_sub, nullptr, g.E_sub,
                                  grad ? g.g_sub : nullptr, true, g.fp64_ws, g.fp64_bytes, s, seg ? g.seg_sub : nullptr,
                                  nseg, g.counts));
    else
        DW_CHECK(det64_local_energy(a, P, prepared, g.r_sub, g.cap, R, Z, seg ? g.seg_sub : nullptr, nseg, g.E_sub,
                                    g.lp_sub, grad ? g.g_sub : nullptr, g.fp64_ws, g.fp64_bytes, s));
    k_guard_scatter<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(g.E_sub, g.lp_sub, g.g_sub, g.idx, g.counts, n3, g.cap,
                                                                  E, lp, grad);
    count_launch();
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

}  // namespace dw

extern "C" {

// Cumulative counts of the tail re-evaluation since the last reset: walkers seen, walkers
// flagged, flagged walkers beyond the capacity (kept at their mixed-form values). Synchronizes
// the device. No counterpart in the reference.
int dw_guard_stats(int64_t* walkers, int64_t* flagged, int64_t* overflow, int reset) {
    unsigned long long v[3] = {0, 0, 0};
    if (cudaDeviceSynchronize() != cudaSuccess) return DW_ERR_CUDA;
    if (cudaMemcpyFromSymbol(&v[0], dw::g_guard_walkers, sizeof(v[0])) != cudaSuccess ||
        cudaMemcpyFromSymbol(&v[1], dw::g_guard_flagged, sizeof(v[1])) != cudaSuccess ||
        cudaMemcpyFromSymbol(&v[2], dw::g_guard_overflow, sizeof(v[2])) != cudaSuccess)
        return DW_ERR_CUDA;
    if (walkers) *walkers = (int64_t)v[0];
    if (flagged) *flagged = (int64_t)v[1];
    if (overflow) *overflow = (int64_t)v[2];
    if (reset) {
        unsigned long long z = 0;
        cudaMemcpyToSymbol(dw::g_guard_walkers, &z, sizeof(z));
        cudaMemcpyToSymbol(dw::g_guard_flagged, &z, sizeof(z));
        cudaMemcpyToSymbol(dw::g_guard_overflow, &z, sizeof(z));
    }
    return DW_OK;
}

}  // extern "C"
