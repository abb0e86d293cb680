// Shared definitions for the dwgb CUDA library: model dimensions, the packed parameter
// layout, workspace carving, launch accounting and small device helpers.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stddef.h>
#include <math.h>
#include "../../include/dwgb.h"

#define DW_CHECK_CUDA(x)                                   \
    do {                                                   \
        cudaError_t _e = (x);                              \
        if (_e != cudaSuccess) { dw::set_last_cuda_error(_e); return (int)DW_ERR_CUDA; } \
    } while (0)

#define DW_CHECK(x)                                        \
    do { int _s = (x); if (_s != DW_OK) return _s; } while (0)

namespace dw {

void set_last_cuda_error(cudaError_t e);
void count_launch(int n = 1);
int64_t launch_count();
void reset_launch_count();

// Optional per-tag kernel timing with CUDA events recorded on the launching stream
// (enabled by dw_timer_enable; used to measure a kernel's live duration inside a run).
bool timer_on();
void timer_begin(const char* tag, cudaStream_t s);
void timer_end(const char* tag, cudaStream_t s, double flops, double bytes);

constexpr int kAlignFloats = 64;      // packed-parameter alignment (floats)
constexpr int kMaxEl = 64;
constexpr int kMaxIons = 16;

// Index of each tensor in the packed parameter list (same order as params.param_shapes).
struct ParamLayout {
    int64_t ion_embed;
    int64_t w_same_w[4], w_same_b[4], w_diff_w[4], w_diff_b[4];
    int64_t h_map_w[4], h_map_b[4], h_ion_map_w[4], h_ion_map_b[4];
    int64_t h_el_w[4], h_el_b[4];
    int64_t h_same_w[3], h_same_b[3], h_diff_w[3], h_diff_b[3], h_ei_w[3], h_ei_b[3];
    int64_t bf_up, bf_dn, alpha_up, alpha_dn, weights_up, weights_dn;
    int64_t jas_w[3], jas_b[2];
    int64_t total;
    int n_entries;
    int64_t off[128], size[128];
};

// Model dimensions for one launch family.
struct Dims {
    int n, nu, nd, N, K, zmin, zmax;
    int D, E, EI, J0, J1;
    int hw[4];     // width of h_one entering iteration l
    int eiw[4];    // el-ion stream width entering iteration l
    int eew[4];    // 2-el stream width entering iteration l
    int inw[4];    // full symmetric-feature width of h_el_l (3 hw + E + eiw)
    int kw[4];     // row width of the per-electron layer input [h | conv_ee | conv_ei] padded to 64
    int KN;        // n_dets * n_el
    int T;         // channels: 1 (value) or 3n + 2 (value, 3n gradients, Laplacian)
    int Tp;        // padded channel count (power of two >= T)
    int lap;       // index of the Laplacian channel (T-1) or -1
    // Packed launches: walker b of this launch belongs to geometry segment seg[b] (R, Z and the
    // ion maps are per segment; ions with Z = 0 are padding and contribute nothing).
    // seg == nullptr: one geometry for all walkers.
    const int32_t* seg;
    int nseg;
};

constexpr int kMaxSeg = 256;     // geometries per packed launch
// Out-of-range segment indices are clamped so that a bad index cannot read outside the
// geometry arrays; the host wrappers validate seg before the launch.
__host__ __device__ __forceinline__ int clamp_seg(int s, int nseg) { return s < 0 ? 0 : (s >= nseg ? nseg - 1 : s); }
__host__ __device__ __forceinline__ int seg_of(const Dims& d, int64_t b) { return d.seg ? clamp_seg(d.seg[b], d.nseg) : 0; }

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }
inline int next_pow2(int x) { int p = 1; while (p < x) p <<= 1; return p; }

int check_arch(const DwArch* a);
void make_layout(const DwArch* a, ParamLayout* L);
Dims make_dims(const DwArch* a, bool tangents);

// ------------------------------------------------------------------ workspace carving
struct Carver {
    char* base; size_t cap; size_t used; bool dry;
    Carver(void* b, size_t c) : base((char*)b), cap(c), used(0), dry(b == nullptr) {}
    template <class T> T* take(size_t count) {
        size_t off = (used + 255) / 256 * 256;
        used = off + count * sizeof(T);
        if (dry) return nullptr;
        return (T*)(base + off);
    }
    bool ok() const { return dry || used <= cap; }
};

// ------------------------------------------------------------------ device helpers
__device__ __forceinline__ float warp_sum(float v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ float softplus_f(float x) {
    // log(1 + exp(x)), stable form
    return fmaxf(x, 0.f) + log1pf(expf(-fabsf(x)));
}

// Philox-4x32-10 counter-based generator (Salmon, Moraes, Dror, Shaw, "Parallel random
// numbers: as easy as 1, 2, 3", SC'11). Round multipliers and Weyl key increments are
// the published Philox4x32 constants.
struct Philox4 { uint32_t x, y, z, w; };
__device__ __forceinline__ Philox4 philox4x32_10(Philox4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    #pragma unroll
    for (int i = 0; i < 10; ++i) {
        uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        Philox4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += W0; k1 += W1;
    }
    return c;
}
// Uniform in (0, 1): (u + 0.5) / 2^32.
__device__ __forceinline__ float u32_to_unit(uint32_t u) {
    return ((float)(u >> 8) + 0.5f) * (1.0f / 16777216.0f);
}
// Two standard normals from two uniforms (Box-Muller).
__device__ __forceinline__ void box_muller(uint32_t a, uint32_t b, float& n0, float& n1) {
    float u1 = u32_to_unit(a), u2 = u32_to_unit(b);
    float rad = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    n0 = rad * c; n1 = rad * s;
}

}  // namespace dw
