#pragma once
#include "common.cuh"

namespace dw {

struct MhArgs {
    float* r;              // [B, n, 3] current walkers (updated on accept)
    float* r_prop;         // [B, n, 3] proposal buffer
    float* lp;             // [B] current log psi^2
    const float* lp_prop;  // [B] log psi^2 of the proposals
    int32_t* age;          // [B]
    DwMcmcScalars* scalars;
    int* partials;         // [blocks] block accept counts
    int B, n;
    int max_age, interval;
    float target, min_step, max_step;
    uint64_t seed;
};

void launch_mh(const MhArgs& a, int phase, cudaStream_t s);
int mh_partials_needed(int B);
void launch_stats(const float* E, int n, int clip, double c, double w, double cb, float* Ec, double* out, cudaStream_t s);

}  // namespace dw
