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
// log psi^2 and gradient are scattered back. Walkers so close to a node that the FP32 rounding of
// the network itself decides their E_L (magnitudes above kGuardFp64Key) are then re-evaluated by the
// FP64 form (fp64.cu) in a second, smaller sub-batch. The selection depends only on each walker's
// own scales, so a walker gets the same result in any batch as long as the flagged walkers fit the
// capacities; beyond them the walkers with the largest predicted errors are taken.
#include "net.cuh"
#include <algorithm>

namespace dw {

// [tier][walkers seen, walkers flagged, flagged walkers beyond the capacity]
__device__ unsigned long long g_guard_cnt[2][3];

// Predicted E_L error of a mixed-form walker: kGuardRel times the largest magnitude the combine
// kernel cancels (the determinant terms of the Laplacian of log|psi~|, or the terms of E_L). On
// C2H4-shaped walkers (16 electrons, 32 determinants) the measured |E_mixed - E_FP64| / that
// magnitude has median 1.7e-6 and 99th percentile 1.5e-5 (2e-5 to 5e-5 after optimisation steps).
// Walkers predicted above kGuardTol (magnitude above 1,000 Ha) are re-evaluated, those of the
// largest magnitudes first when more than the capacity (1 / 32 of the batch) are flagged. The
// whole capacity is re-evaluated every call whatever the count, so a lower threshold costs nothing
// while the flagged walkers fit: on eleven C2H4 states (initial weights, the end of the optimisation
// bench) lowering it from 2,000 to 1,000 Ha moved the worst batch-mean error from -0.58 to
// -0.38 mHa; below 1,000 Ha nothing changed further.
constexpr float kGuardRel = 1.5e-5f;
constexpr float kGuardTol = 0.015f;
// Re-evaluation form: the plain FP32 network with FP64 determinant algebra (LU, inverse, tangent
// traces). The catastrophic errors of ill-conditioned walkers come from the determinant algebra:
// on 4,096 C2H4-shaped walkers near the initial weights the plain FP32 form is off by up to 14 Ha,
// the same network with FP64 determinants by at most 95 mHa (mean 0.03 mHa), at about 1.5x the
// plain form's cost per walker. The FP64 form (fp64.cu) would cost about 15x more per walker.
// Second tier: walkers whose cancelled magnitude exceeds kGuardFp64Key Ha. At the end of the C2H4
// optimisation bench (random-init weights after 14 Adam steps) 4-37 of 4,096 walkers exceed it; the
// FP32 network with FP64 determinants is off by 0.1-4 Ha on those between 1e5 and 1e7 and by up to
// 57 kHa on the few beyond 1e8 (|E_L| up to 1.4e5 Ha), where only an FP64 network resolves the node.
constexpr float kGuardFp64Key = 1.0e5f;
// Network of the first tier's re-evaluation (DW_PRECISION_FP32_DET64 or DW_PRECISION_MIXED_DET64;
// instrumentation switch dw_debug_set_guard_form).
static int g_guard_form = DW_PRECISION_FP32_DET64;

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
               int* __restrict__ counts, int tier) {
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
        atomicAdd(&g_guard_cnt[tier][0], (unsigned long long)B);
        atomicAdd(&g_guard_cnt[tier][1], (unsigned long long)flagged);
        if (flagged > sel) atomicAdd(&g_guard_cnt[tier][2], (unsigned long long)(flagged - sel));
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
    // first tier: up to 1 / 32 of the batch (at least 16), run over the whole capacity (unused
    // slots hold a copy of walker 0)
    (void)a;
    return std::min(B, std::max(16, (B + 31) / 32));
}

// second tier: up to 1 / 128 of the batch (at least 8) in one FP64 chunk; its kernels skip the
// unused capacity through the device-side count, so it costs FP64 work only for the walkers
// flagged (about 0.6 ms per C2H4-shaped walker)
static int guard64_capacity(const DwArch* a, int B) {
    return std::max(1, std::min(std::min(B, std::max(8, (B + 127) / 128)), fp64_max_chunk(a, true)));
}

struct GuardTier {
    int cap;
    int* idx; int* counts; float* r_sub; int32_t* seg_sub; float* E_sub; float* lp_sub; float* g_sub;
};

struct GuardPlan {
    GuardTier t[2];
    void* region; size_t region_bytes;              // forward workspace, used by one tier at a time
    size_t bytes;
};

static GuardPlan carve_guard(const DwArch* a, int B, void* ws) {
    GuardPlan g;
    const int n3 = 3 * a->n_el;
    Carver c(ws, (size_t)-1);
    for (int k = 0; k < 2; ++k) {
        GuardTier& t = g.t[k];
        t.cap = k == 0 ? guard_capacity(a, B) : guard64_capacity(a, B);
        t.idx = c.take<int>((size_t)t.cap);
        t.counts = c.take<int>(2);
        t.r_sub = c.take<float>((size_t)t.cap * n3);
        t.seg_sub = c.take<int32_t>((size_t)t.cap);
        t.E_sub = c.take<float>((size_t)t.cap);
        t.lp_sub = c.take<float>((size_t)t.cap);
        t.g_sub = c.take<float>((size_t)t.cap * n3);
    }
    g.region_bytes = std::max({det64_plan_bytes(a, DW_PRECISION_FP32_DET64, g.t[0].cap),
                               det64_plan_bytes(a, DW_PRECISION_MIXED_DET64, g.t[0].cap),
                               fp64_plan_bytes(a, g.t[1].cap, true)});
    g.region = c.take<unsigned char>(g.region_bytes);
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
    for (int k = 0; k < 2; ++k) {
        const GuardTier& t = g.t[k];
        // tier 0: predicted error above kGuardTol; tier 1: magnitude above kGuardFp64Key
        k_guard_select<<<1, 1024, 0, s>>>(esc, B, k == 0 ? kGuardRel : 1.0f, k == 0 ? kGuardTol : kGuardFp64Key, t.cap,
                                          t.idx, t.counts, k);
        count_launch();
        const int64_t ne = (int64_t)t.cap * n3;
        k_guard_gather<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(r, seg, t.idx, t.counts, n3, t.r_sub,
                                                                     seg ? t.seg_sub : nullptr, t.cap, k == 0 ? 1 : 0);
        count_launch();
        if (k == 0) {
            DW_CHECK(det64_local_energy(a, g_guard_form, P, prepared, t.r_sub, t.cap, R, Z, seg ? t.seg_sub : nullptr,
                                        nseg, t.E_sub, t.lp_sub, grad ? t.g_sub : nullptr, g.region, g.region_bytes, s));
        } else {
            timer_begin("guard_fp64", s);
            DW_CHECK(fp64_forward_all(a, P, prepared, t.r_sub, t.cap, R, Z, t.lp_sub, nullptr, t.E_sub,
                                      grad ? t.g_sub : nullptr, true, g.region, g.region_bytes, s,
                                      seg ? t.seg_sub : nullptr, nseg, t.counts));
            timer_end("guard_fp64", s, 0.0, 0.0);
        }
        k_guard_scatter<<<(unsigned)((ne + 255) / 256), 256, 0, s>>>(t.E_sub, t.lp_sub, t.g_sub, t.idx, t.counts, n3,
                                                                      t.cap, E, lp, grad);
        count_launch();
    }
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

}  // namespace dw

extern "C" {

// Cumulative counts of the tail re-evaluation since the last reset (tier 0: the FP64-determinant
// re-evaluation, tier 1: the FP64-form re-evaluation): walkers seen, walkers flagged, flagged
// walkers beyond the capacity (kept at the previous tier's values). Synchronizes the device. No
// counterpart in the reference.
int dw_guard_tier_stats(int tier, int64_t* walkers, int64_t* flagged, int64_t* overflow, int reset) {
    if (tier < 0 || tier > 1) return DW_ERR_ARG;
    unsigned long long v[2][3];
    if (cudaDeviceSynchronize() != cudaSuccess) return DW_ERR_CUDA;
    if (cudaMemcpyFromSymbol(v, dw::g_guard_cnt, sizeof(v)) != cudaSuccess) return DW_ERR_CUDA;
    if (walkers) *walkers = (int64_t)v[tier][0];
    if (flagged) *flagged = (int64_t)v[tier][1];
    if (overflow) *overflow = (int64_t)v[tier][2];
    if (reset) {
        for (int k = 0; k < 3; ++k) v[tier][k] = 0;
        if (cudaMemcpyToSymbol(dw::g_guard_cnt, v, sizeof(v)) != cudaSuccess) return DW_ERR_CUDA;
    }
    return DW_OK;
}

// Tier 0 of dw_guard_tier_stats; a reset clears both tiers.
int dw_guard_stats(int64_t* walkers, int64_t* flagged, int64_t* overflow, int reset) {
    DW_CHECK(dw_guard_tier_stats(0, walkers, flagged, overflow, reset));
    return reset ? dw_guard_tier_stats(1, nullptr, nullptr, nullptr, 1) : DW_OK;
}

// Instrumentation: network of the first re-evaluation tier (DW_PRECISION_FP32_DET64, the default,
// or DW_PRECISION_MIXED_DET64). Returns the previous form.
int dw_debug_set_guard_form(int precision) {
    if (!dw::det64_form(precision)) return -DW_ERR_ARG;
    const int old = dw::g_guard_form;
    dw::g_guard_form = precision;
    return old;
}

}  // extern "C"
