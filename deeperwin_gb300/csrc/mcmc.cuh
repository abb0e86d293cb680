#pragma once
#include "common.cuh"

namespace dw {

struct MhArgs {
    float* r;              // [B, n, 3] current walkers (updated on accept)
    float* r_prop;         // [B, n, 3] proposal buffer
    float* lp;             // [B] current log psi^2
    const float* lp_prop;  // [B] log psi^2 of the proposals
    int32_t* age;          // [B]
    DwMcmcScalars* scalars;  // [nseg] chain scalars (step size, acceptance, step counter) per segment
    int* counts;           // [2 * nseg] accepted / walker counts of the running step (zero between steps)
    int B, n;
    int max_age, interval;
    float target, min_step, max_step;
    uint64_t seed;
    // Packed chains: walker b belongs to chain seg[b], draws its random numbers as walker
    // widx[b] of that chain, keyed by seeds[seg[b]]. All null: one chain, walker b, key `seed`.
    const int32_t* seg;
    const int32_t* widx;
    const uint64_t* seeds;
    int nseg;
    // Proposal rule (DwProposal) and its parameters; lq[B] holds the log proposal ratio of the
    // pending proposals (asymmetric rules). R / Z / N: nuclei of each segment (local, Langevin).
    int proposal;
    float r_min, r_max, langevin_scale, p_swap, p_flip;
    float* lq;
    const float* R;
    const int32_t* Z;
    int N;
};

void launch_mh(const MhArgs& a, int phase, cudaStream_t s);
int mh_counts_needed(int nseg);
void launch_stats(const float* E, int n, int clip, double c, double w, double cb, float* Ec, double* out, cudaStream_t s);

}  // namespace dw
