// Hellmann-Feynman forces on the nuclei (hamiltonian.py:294-338 calculate_forces): per walker the
// electron-nucleus attraction with the reference's short-distance cut-off d -> d / tanh(d / R_cut),
// optionally with antithetic sampling (core electrons mirrored through their closest nucleus,
// weighted by psi^2(mirrored) / psi^2), averaged over the walkers in FP64, plus the nucleus-nucleus
// repulsion.
#include "net.cuh"
#include <algorithm>

namespace dw {

// Mirrored walkers: every electron closer than R_core to its closest nucleus is reflected through
// it, r -> r - 2 (r - R_closest) (hamiltonian.py:321-328).
__global__ void k_force_mirror(const float* __restrict__ r, int B, int n, const float* __restrict__ R,
                               const int32_t* __restrict__ Z, int N, float R_core, float* __restrict__ rm) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)B * n) return;
    const float* x = r + e * 3;
    float best = 3.4e38f, dx = 0.f, dy = 0.f, dz = 0.f;
    for (int I = 0; I < N; ++I) {
        if (Z[I] <= 0) continue;
        const float ax = x[0] - R[3 * I], ay = x[1] - R[3 * I + 1], az = x[2] - R[3 * I + 2];
        const float d = sqrtf(ax * ax + ay * ay + az * az);
        if (d < best) { best = d; dx = ax; dy = ay; dz = az; }     // argmin: first of equal distances
    }
    const bool core = best < R_core;
    rm[e * 3] = core ? x[0] - 2.f * dx : x[0];
    rm[e * 3 + 1] = core ? x[1] - 2.f * dy : x[1];
    rm[e * 3 + 2] = core ? x[2] - 2.f * dz : x[2];
}

// sum_i Z_I (r_i - R_I) / d'^3 with d' = d / tanh(d / R_cut) (hamiltonian.py:293-295) of one
// walker for nucleus I, FP64, lanes over electrons.
__device__ __forceinline__ void force_sum(const float* x, int n, const float* RI, double ZI, double R_cut, int lane,
                                          double (&f)[3]) {
    f[0] = f[1] = f[2] = 0.0;
    for (int i = lane; i < n; i += 32) {
        const double ax = (double)x[3 * i] - RI[0], ay = (double)x[3 * i + 1] - RI[1], az = (double)x[3 * i + 2] - RI[2];
        const double d = sqrt(ax * ax + ay * ay + az * az);
        const double dc = d / tanh(d / R_cut);
        const double w = ZI / (dc * dc * dc);
        f[0] += w * ax; f[1] += w * ay; f[2] += w * az;
    }
    for (int c = 0; c < 3; ++c) f[c] = warp_sum(f[c]);
}

// Per-walker forces [B][N][3] (electrons summed), warp per walker.
__global__ void k_force_walkers(const float* __restrict__ r, const float* __restrict__ rm, const float* __restrict__ lp,
                                const float* __restrict__ lpm, int B, int n, const float* __restrict__ R,
                                const int32_t* __restrict__ Z, int N, double R_cut, double* __restrict__ out) {
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= B) return;
    const int64_t b = warp;
    // antithetic weight psi^2(r_m) / psi^2(r) (hamiltonian.py:329)
    const double wm = rm ? exp((double)lpm[b] - (double)lp[b]) : 0.0;
    for (int I = 0; I < N; ++I) {
        double f[3] = {0.0, 0.0, 0.0};
        if (Z[I] > 0) {
            const float RIf[3] = {R[3 * I], R[3 * I + 1], R[3 * I + 2]};
            double fm[3];
            force_sum(r + b * n * 3, n, RIf, (double)Z[I], R_cut, lane, f);
            if (rm) {
                force_sum(rm + b * n * 3, n, RIf, (double)Z[I], R_cut, lane, fm);
                for (int c = 0; c < 3; ++c) f[c] = 0.5 * (f[c] + fm[c] * wm);      // hamiltonian.py:332
            }
        }
        if (lane < 3) out[(b * N + I) * 3 + lane] = f[lane];
    }
}

// Batch mean of the per-walker forces (fixed order, one block per component) plus the
// nucleus-nucleus forces sum_J Z_I Z_J (R_I - R_J) / (|R_I - R_J| + 1e-8)^3 (hamiltonian.py:298-306).
__global__ void k_force_mean(const double* __restrict__ pw, int B, const float* __restrict__ R,
                             const int32_t* __restrict__ Z, int N, double* __restrict__ out) {
    const int comp = blockIdx.x, I = comp / 3, c = comp % 3;
    double s = 0.0;
    for (int b = threadIdx.x; b < B; b += blockDim.x) s += pw[(int64_t)b * N * 3 + comp];
    __shared__ double red[32];
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        double ii = 0.0;
        if (Z[I] > 0) {
            for (int J = 0; J < N; ++J) {
                if (J == I || Z[J] <= 0) continue;
                const double dx = (double)R[3 * I] - R[3 * J], dy = (double)R[3 * I + 1] - R[3 * J + 1],
                             dz = (double)R[3 * I + 2] - R[3 * J + 2];
                const double dist = sqrt(dx * dx + dy * dy + dz * dz) + 1e-8;
                const double dd = c == 0 ? dx : (c == 1 ? dy : dz);
                ii += (double)Z[I] * Z[J] * dd / (dist * dist * dist);
            }
        }
        out[comp] = t / B + ii;
    }
}

}  // namespace dw

using namespace dw;

extern "C" {

size_t dw_forces_workspace_bytes(const DwArch* a, int precision, int n_walkers) {
    if (check_arch(a) != DW_OK || n_walkers <= 0) return 0;
    const size_t fwd = dw_workspace_bytes(a, precision, n_walkers, 0);
    if (fwd == 0) return 0;
    return fwd + 3 * 256 + (size_t)n_walkers * a->n_el * 3 * sizeof(float) + (size_t)n_walkers * sizeof(float) +
           (size_t)n_walkers * a->n_ions * 3 * sizeof(double);
}

int dw_forces(const DwArch* a, int precision, const float* params, const void* prepared, const float* r, int B,
              const float* R, const int32_t* Z, const float* log_psi_sqr, float R_cut, float R_core, int antithetic,
              double* forces, double* per_walker, void* ws, size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!r || !R || !Z || !log_psi_sqr || !forces || B <= 0 || !(R_cut > 0.f) || !(R_core >= 0.f)) return DW_ERR_ARG;
    if (antithetic && (!params || !prepared)) return DW_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const int n = a->n_el, N = a->n_ions;
    const size_t fwd = dw_workspace_bytes(a, precision, B, 0);
    if (fwd == 0) return DW_ERR_ARG;
    Carver c(static_cast<char*>(ws) + fwd, wsb > fwd ? wsb - fwd : 0);
    float* rm = c.take<float>((size_t)B * n * 3);
    float* lpm = c.take<float>((size_t)B);
    double* pw = c.take<double>((size_t)B * N * 3);
    if (!ws || !c.ok()) return DW_ERR_WORKSPACE;
    if (per_walker) pw = per_walker;
    int64_t launches = 0;
    if (antithetic) {
        k_force_mirror<<<(unsigned)(((int64_t)B * n + 255) / 256), 256, 0, s>>>(r, B, n, R, Z, N, R_core, rm);
        DW_CHECK(dw_log_psi_sqr(a, precision, params, prepared, rm, B, R, Z, lpm, nullptr, ws, fwd, stream));
        launches += launch_count() + 1;
    }
    k_force_walkers<<<(unsigned)(((int64_t)B * 32 + 255) / 256), 256, 0, s>>>(r, antithetic ? rm : nullptr, log_psi_sqr,
                                                                           lpm, B, n, R, Z, N, (double)R_cut, pw);
    k_force_mean<<<3 * N, 256, 0, s>>>(pw, B, R, Z, N, forces);
    reset_launch_count();
    count_launch((int)launches + 2);
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

}  // extern "C"
