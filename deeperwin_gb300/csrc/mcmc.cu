// Metropolis-Hastings accept/propose kernel and FP64 cross-walker reductions.
#include "net.cuh"
#include "mcmc.cuh"
#include <cooperative_groups.h>

namespace dw {

// Counter-based normals for (walker, step): Philox counter {walker, step, group, tag}.
__device__ __forceinline__ void normals4(uint64_t seed, uint32_t walker, uint32_t step, uint32_t group, float (&o)[4]) {
    Philox4 c{walker, step, group, 0xA511E9B3u};
    Philox4 x = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    box_muller(x.x, x.y, o[0], o[1]);
    box_muller(x.z, x.w, o[2], o[3]);
}
__device__ __forceinline__ float uniform1(uint64_t seed, uint32_t walker, uint32_t step) {
    Philox4 c{walker, step, 0u, 0x63D83595u};
    Philox4 x = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return u32_to_unit(x.x);
}

// Step-size rule (mcmc.py:370-387): on steps where step_nr % interval == 0, divide by 1.05
// if the previous running acceptance is below target, else multiply; clip.
__device__ __forceinline__ float next_stepsize(float s, double acc_rate_prev, int step_nr_new, const MhArgs& a) {
    if (a.interval > 0 && step_nr_new % a.interval == 0) {
        s = acc_rate_prev < (double)a.target ? s / 1.05f : s * 1.05f;
        s = fminf(fmaxf(s, a.min_step), a.max_step);
    }
    return s;
}

// phase 0: propose only (r_prop = r + s N); phase 1: accept proposal, then propose the next;
// phase 2: accept only. One warp per walker; each walker follows the scalars of its chain.
__global__ void k_mh(MhArgs a, int phase) {
    __shared__ int blk_seg[32], blk_acc[32];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const int w = blockIdx.x * wpb + wid;
    const int n3 = 3 * a.n;
    int accepted = 0, sg = -1;
    if (w < a.B) {
        sg = a.seg ? clamp_seg(a.seg[w], a.nseg) : 0;
        const DwMcmcScalars* S = a.scalars + sg;
        const double acc_rate = S->acc_rate;
        const float step = S->stepsize;
        const int step_nr = S->step_nr;
        const uint64_t key = a.seeds ? a.seeds[sg] : a.seed;
        const uint32_t wk = a.widx ? (uint32_t)a.widx[w] : (uint32_t)w;
        float* rw = a.r + (int64_t)w * n3;
        float* pw = a.r_prop + (int64_t)w * n3;
        float s_prop = step;
        int nr_prop = step_nr;
        if (phase >= 1) {
            float lp = a.lp[w], lpn = a.lp_prop[w];
            float U = uniform1(key, wk, (uint32_t)step_nr);
            bool acc = expf(lpn - lp) > U;          // mcmc.py:359-362
            int age = a.age[w];
            acc = acc || (age >= a.max_age);        // mcmc.py:363
            if (acc) for (int q = lane; q < n3; q += 32) rw[q] = pw[q];
            if (lane == 0) {
                a.age[w] = acc ? 0 : age + 1;       // mcmc.py:364-365
                if (acc) a.lp[w] = lpn;
            }
            accepted = acc ? 1 : 0;
            nr_prop = step_nr + 1;
            s_prop = next_stepsize(step, acc_rate, nr_prop, a);
            __syncwarp();
        }
        if (phase <= 1) {
            for (int g = lane; g * 4 < n3; g += 32) {
                float z[4];
                normals4(key, wk, (uint32_t)nr_prop, (uint32_t)g, z);
                #pragma unroll
                for (int c = 0; c < 4; ++c) {
                    int q = g * 4 + c;
                    if (q < n3) pw[q] = rw[q] + s_prop * z[c];   // mcmc.py:178-179
                }
            }
        }
    }
    if (phase == 0) return;
    // Integer accept / walker counts per chain (runs of equal chain within the block merged),
    // then the last block turns them into FP64 acceptance rates and the next step sizes.
    if (lane == 0) { blk_seg[wid] = sg; blk_acc[wid] = accepted; }
    __syncthreads();
    if (threadIdx.x == 0) {
        int k = 0;
        while (k < wpb) {
            const int cs = blk_seg[k];
            int acc = 0, cnt = 0;
            for (; k < wpb && blk_seg[k] == cs; ++k) { acc += blk_acc[k]; ++cnt; }
            if (cs >= 0) { atomicAdd(a.counts + 2 * cs, acc); atomicAdd(a.counts + 2 * cs + 1, cnt); }
        }
        __threadfence();
        unsigned t = atomicAdd(&a.scalars[0].ticket, 1u);
        if (t == gridDim.x - 1) {
            __threadfence();
            for (int c = 0; c < a.nseg; ++c) {
                volatile int* cc = a.counts + 2 * c;
                const int acc = cc[0], cnt = cc[1];
                cc[0] = 0; cc[1] = 0;
                if (cnt == 0) continue;              // chain not in this launch
                DwMcmcScalars* S = a.scalars + c;
                const double prev = S->acc_rate;
                const double mean = (double)acc / (double)cnt;
                S->last_acc = mean;
                S->acc_rate = 0.9 * prev + 0.1 * mean;      // mcmc.py:371
                S->stepsize = next_stepsize(S->stepsize, prev, S->step_nr + 1, a);
                S->step_nr = S->step_nr + 1;
            }
            a.scalars[0].ticket = 0u;
            __threadfence();
        }
    }
}

void launch_mh(const MhArgs& a, int phase, cudaStream_t s) {
    const int wpb = 8;
    int blocks = (a.B + wpb - 1) / wpb;
    k_mh<<<blocks, wpb * 32, 0, s>>>(a, phase);
    count_launch();
}
int mh_counts_needed(int nseg) { return 2 * nseg; }

// ------------------------------------------------------------------ FP64 statistics
struct Welford { double n, mean, m2; };
__device__ __forceinline__ Welford wmerge(Welford a, Welford b) {
    if (b.n == 0) return a;
    if (a.n == 0) return b;
    double n = a.n + b.n, dlt = b.mean - a.mean;
    return Welford{n, a.mean + dlt * b.n / n, a.m2 + b.m2 + dlt * dlt * a.n * b.n / n};
}
__device__ Welford block_welford(Welford w) {
    __shared__ double sh[3][32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        Welford x{__shfl_xor_sync(0xffffffffu, w.n, o), __shfl_xor_sync(0xffffffffu, w.mean, o),
                  __shfl_xor_sync(0xffffffffu, w.m2, o)};
        w = (lane & o) ? wmerge(x, w) : wmerge(w, x);
    }
    if (lane == 0) { sh[0][wid] = w.n; sh[1][wid] = w.mean; sh[2][wid] = w.m2; }
    __syncthreads();
    Welford r{0, 0, 0};
    if (threadIdx.x == 0)
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) r = wmerge(r, Welford{sh[0][k], sh[1][k], sh[2][k]});
    return r;
}

// FP64 mean / variance of (optionally clipped) energies with the reference's nanmean semantics
// (loss_function.py:94-99): only NaN entries are dropped; an infinite entry makes the mean that
// infinity and the variance infinite (NaN when both signs occur, or when no finite entry is left).
// One thread-block cluster of kStatsBlocks CTAs on as many SMs (the FP64 tanh of the clipping and
// the merges run on 8 SMs' FP64 pipes instead of one): each thread keeps counts and sums shifted by
// its first finite value, blocks merge their threads by Welford, and block 0 merges the blocks'
// partials through distributed shared memory in rank order, so the result is deterministic and no
// global scratch is needed.
constexpr int kStatsBlocks = 8, kStatsThreads = 512;
struct StatPart { double n, mean, m2, npos, nneg, nnum; };

__global__ void __cluster_dims__(kStatsBlocks, 1, 1) __launch_bounds__(kStatsThreads)
k_stats(const float* __restrict__ E, int n, int clip, double center, double width, double clip_by,
        float* __restrict__ E_clip, double* __restrict__ out) {
    namespace cg = cooperative_groups;
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int stride = kStatsBlocks * kStatsThreads;
    double c0 = 0.0, s1 = 0.0, s2 = 0.0, cnt = 0.0, npos = 0.0, nneg = 0.0;
    bool have = false;
    for (int i = rank * kStatsThreads + threadIdx.x; i < n; i += stride) {
        double x = E[i];
        if (clip) {
            x = center + tanh((x - center) / width) * width;   // loss_function.py:49-51
            E_clip[i] = (float)x;
        }
        if (isnan(x)) continue;
        if (isinf(x)) { if (x > 0) npos += 1.0; else nneg += 1.0; continue; }
        if (!have) { c0 = x; have = true; }
        const double dd = x - c0;
        s1 += dd; s2 = fma(dd, dd, s2); cnt += 1.0;
    }
    Welford w{cnt, cnt > 0 ? c0 + s1 / cnt : 0.0, cnt > 0 ? fmax(s2 - s1 * s1 / cnt, 0.0) : 0.0};
    Welford r = block_welford(w);
    for (int o = 16; o > 0; o >>= 1) {
        npos += __shfl_xor_sync(0xffffffffu, npos, o);
        nneg += __shfl_xor_sync(0xffffffffu, nneg, o);
    }
    __shared__ double inf_sh[2][kStatsThreads / 32];
    __shared__ StatPart part;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { inf_sh[0][wid] = npos; inf_sh[1][wid] = nneg; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double p = 0.0, q = 0.0;
        for (int k = 0; k < kStatsThreads / 32; ++k) { p += inf_sh[0][k]; q += inf_sh[1][k]; }
        part = StatPart{r.n, r.mean, r.m2, p, q, 0.0};
    }
    cl.sync();
    if (rank == 0 && threadIdx.x == 0) {
        Welford t{0, 0, 0};
        double p = 0.0, q = 0.0;
        for (int b = 0; b < kStatsBlocks; ++b) {
            const StatPart* o = cl.map_shared_rank(&part, b);
            t = wmerge(t, Welford{o->n, o->mean, o->m2});
            p += o->npos; q += o->nneg;
        }
        double mean = t.n > 0 ? t.mean : NAN, var = t.n > 0 ? t.m2 / t.n : NAN;
        if (p > 0 && q > 0) { mean = NAN; var = NAN; }
        else if (p > 0) { mean = INFINITY; var = t.n > 0 ? INFINITY : NAN; }
        else if (q > 0) { mean = -INFINITY; var = t.n > 0 ? INFINITY : NAN; }
        out[0] = mean;
        out[1] = var;
        out[2] = t.n + p + q;                  // entries that are not NaN
        if (clip) { out[2] = mean; out[3] = sqrt(var) * clip_by; }
    }
    cl.sync();                                 // keep every block's partial alive until block 0 has read it
}

void launch_stats(const float* E, int n, int clip, double c, double w, double cb, float* Ec, double* out, cudaStream_t s) {
    k_stats<<<kStatsBlocks, kStatsThreads, 0, s>>>(E, n, clip, c, w, cb, Ec, out);
    count_launch();
}

}  // namespace dw
