// Metropolis-Hastings accept/propose kernel and FP64 cross-walker reductions.
#include "net.cuh"
#include "mcmc.cuh"

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

// Single-block FP64 mean / variance / finite count of (optionally clipped) energies.
__global__ void k_stats(const float* __restrict__ E, int n, int clip, double center, double width, double clip_by,
                        float* __restrict__ E_clip, double* __restrict__ out) {
    Welford w{0, 0, 0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double x = E[i];
        if (clip) {
            x = center + tanh((x - center) / width) * width;   // loss_function.py:49-51
            E_clip[i] = (float)x;
        }
        if (isfinite(x)) w = wmerge(w, Welford{1.0, x, 0.0});
    }
    Welford r = block_welford(w);
    if (threadIdx.x == 0) {
        double var = r.n > 0 ? r.m2 / r.n : NAN;
        out[0] = r.n > 0 ? r.mean : NAN;
        out[1] = var;
        out[2] = r.n;
        if (clip) { out[2] = r.mean; out[3] = sqrt(var) * clip_by; }
    }
}

void launch_stats(const float* E, int n, int clip, double c, double w, double cb, float* Ec, double* out, cudaStream_t s) {
    k_stats<<<1, 1024, 0, s>>>(E, n, clip, c, w, cb, Ec, out);
    count_launch();
}

}  // namespace dw
