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
// Four uniforms in (0, 1) for (walker, step, group, tag).
__device__ __forceinline__ void uniforms4(uint64_t seed, uint32_t walker, uint32_t step, uint32_t group, uint32_t tag,
                                          float (&o)[4]) {
    Philox4 x = philox4x32_10(Philox4{walker, step, group, tag}, (uint32_t)seed, (uint32_t)(seed >> 32));
    o[0] = u32_to_unit(x.x); o[1] = u32_to_unit(x.y); o[2] = u32_to_unit(x.z); o[3] = u32_to_unit(x.w);
}
constexpr uint32_t kTagCauchy = 0xC4A3B1E7u, kTagSpin = 0x5F1A9C3Du;

// Standard normal for coordinate q of a walker's proposal at counter `step`.
__device__ __forceinline__ float normal_q(uint64_t key, uint32_t wk, uint32_t step, int q) {
    float z[4];
    normals4(key, wk, step, (uint32_t)(q >> 2), z);
    return z[q & 3];
}

// Local step size and Langevin drift of one electron (mcmc.py:204-215): s = stepsize
// clip(d_closest_ion, r_min, r_max), g = -scale sum_I Z_I (r - R_I) / |r - R_I|.
__device__ __forceinline__ void local_step(const float* x, const float* R, const int32_t* Z, int N, float stepsize,
                                           const MhArgs& a, float& s, float (&g)[3]) {
    float dmin = 3.4e38f;
    g[0] = g[1] = g[2] = 0.f;
    for (int I = 0; I < N; ++I) {
        if (Z[I] <= 0) continue;                 // padding ion of a packed geometry
        const float dx = x[0] - R[3 * I], dy = x[1] - R[3 * I + 1], dz = x[2] - R[3 * I + 2];
        const float d = sqrtf(dx * dx + dy * dy + dz * dz);
        dmin = fminf(dmin, d);
        const float w = -a.langevin_scale * (float)Z[I] / d;
        g[0] += w * dx; g[1] += w * dy; g[2] += w * dz;
    }
    s = stepsize * fminf(fmaxf(dmin, a.r_min), a.r_max);
}

// Proposal of one walker (warp): writes pw and returns the log proposal ratio (lane 0).
__device__ float propose_walker(const MhArgs& a, const float* rw, float* pw, float step, int nr, uint64_t key,
                                uint32_t wk, int sg, int lane) {
    const int n = a.n, n3 = 3 * n;
    const int kind = a.proposal;
    float lq = 0.f;
    if (kind == DW_PROPOSAL_NORMAL || kind == DW_PROPOSAL_NORMAL_ONE_EL) {
        const int one = kind == DW_PROPOSAL_NORMAL_ONE_EL ? nr % n : -1;
        for (int g = lane; g * 4 < n3; g += 32) {
            float z[4];
            normals4(key, wk, (uint32_t)nr, (uint32_t)g, z);
            #pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int q = g * 4 + c;
                if (q < n3) pw[q] = (one < 0 || q / 3 == one) ? rw[q] + step * z[c] : rw[q];   // mcmc.py:178-179, 190-192
            }
        }
    } else if (kind == DW_PROPOSAL_CAUCHY) {
        for (int g = lane; g * 4 < n3; g += 32) {
            float u[4];
            uniforms4(key, wk, (uint32_t)nr, (uint32_t)g, kTagCauchy, u);
            #pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int q = g * 4 + c;
                float sn, cs;
                sincospif(u[c] - 0.5f, &sn, &cs);                   // Cauchy = tan(pi (u - 1/2))
                if (q < n3) pw[q] = rw[q] + step * (sn / cs);       // mcmc.py:199-200
            }
        }
    } else {
        // local step sizes (all electrons, or electron nr mod n) and the Langevin drift
        const float* R = a.R + (size_t)sg * a.N * 3;
        const int32_t* Z = a.Z + (size_t)sg * a.N;
        const int one = kind == DW_PROPOSAL_LOCAL_ONE_EL ? nr % n : -1;
        const bool lang = kind == DW_PROPOSAL_LANGEVIN;
        for (int i = lane; i < n; i += 32) {
            const float* x = rw + 3 * i;
            float* y = pw + 3 * i;
            if (one >= 0 && i != one) { y[0] = x[0]; y[1] = x[1]; y[2] = x[2]; continue; }
            float s, g[3], s2, g2[3];
            local_step(x, R, Z, a.N, step, a, s, g);
            float d_fwd = 0.f;
            for (int c = 0; c < 3; ++c) {
                const float z = normal_q(key, wk, (uint32_t)nr, 3 * i + c);
                const float drift = lang ? g[c] * s * s : 0.f;
                y[c] = x[c] + z * s + drift;                         // mcmc.py:227, :270
                const float e = y[c] - x[c] - drift;
                d_fwd += e * e;
            }
            local_step(y, R, Z, a.N, step, a, s2, g2);
            float d_rev = 0.f;
            for (int c = 0; c < 3; ++c) {
                const float e = x[c] - y[c] - (lang ? g2[c] * s2 * s2 : 0.f);
                d_rev += e * e;
            }
            // 3 (log s - log s') + (|fwd|^2 / s^2 - |rev|^2 / s'^2) / 2 (mcmc.py:230-233, :280-285)
            lq += 3.f * (logf(s) - logf(s2)) + 0.5f * (d_fwd / (s * s) - d_rev / (s2 * s2));
        }
        lq = warp_sum(lq);
    }
    // spin swap / flip of the proposal (mcmc.py:346-356). The swap exchanges an electron of the
    // first n_el // 2 with one of the others, the split the reference uses (mcmc.py:350).
    if (a.p_swap > 0.f || a.p_flip > 0.f) {
        __syncwarp();
        float u[4];
        uniforms4(key, wk, (uint32_t)nr, 0u, kTagSpin, u);
        const int nh = n / 2;
        if (a.p_swap > 0.f && u[0] < a.p_swap && nh > 0) {
            const int iu = min((int)(u[1] * nh), nh - 1);
            const int id = nh + min((int)(u[2] * (n - nh)), n - nh - 1);
            if (lane < 3) {
                const float t = pw[3 * iu + lane];
                pw[3 * iu + lane] = pw[3 * id + lane];
                pw[3 * id + lane] = t;
            }
            __syncwarp();
        }
        if (a.p_flip > 0.f && u[3] < a.p_flip) {
            for (int q = lane; q < 3 * nh; q += 32) {
                const int i = q / 3, c = q % 3;
                const float t = pw[3 * i + c];
                pw[3 * i + c] = pw[3 * (n - 1 - i) + c];
                pw[3 * (n - 1 - i) + c] = t;
            }
            __syncwarp();
        }
    }
    return lq;
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
            const float lq = a.lq ? a.lq[w] : 0.f;
            float U = uniform1(key, wk, (uint32_t)step_nr);
            bool acc = expf(lpn - lp + lq) > U;     // mcmc.py:358-362
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
            const float lq = propose_walker(a, rw, pw, s_prop, nr_prop, key, wk, sg, lane);
            if (a.lq && lane == 0) a.lq[w] = lq;
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
