// FP64 form: the whole forward pass and the forward-Laplacian local energy in double precision
// (DW_PRECISION_FP64). It mirrors the reference's float64 mode (configuration.py:1893
// `float_precision`, applied through jax_enable_x64 in process_molecule.py:20-29): every GEMM,
// activation, convolution, envelope, LU, inverse, determinant tangent and reduction runs in FP64.
// The packed FP32 weights are read as they are (FP32 -> FP64 is exact), as the reference's x64
// mode evaluates float32-initialised weights in double.
//
// Layout. Every per-electron quantity carries C channels: C = 1 in value passes, C = 3n + 2 in
// tangent passes (channel 0 the value, 1 + 3m + c the derivative by coordinate c of electron m,
// C - 1 the Laplacian over all 3n coordinates). Rows are (walker, electron, channel); a linear map
// acts on every channel row alike (the bias only on channel 0) and an elementwise map couples the
// C rows of one (walker, electron). Pair streams depend on r only through d_ij and are carried as
// Taylor triples (f, df/dd, d2f/dd2); el-ion streams depend only on r_i and carry (value, three
// gradients, Laplacian) in r_i. This form is the precision anchor of the mixed form (and the FP64
// GPU rerun of its accuracy checks); it is not tuned for speed: the FP64 pipe of this part issues
// at a small fraction of the FP32 rate.
#include "net.cuh"
#include <algorithm>

namespace dw {

// Launch family of one FP64 pass: dims, channel count, walkers in the chunk and an optional
// device-side count of valid walkers (walkers at or beyond it are skipped by every kernel).
struct Run64 {
    Dims d;
    int C;          // channels per electron
    int B;          // walkers in the chunk
    const int* nvalid;
};
__device__ __forceinline__ int valid_walkers(const Run64& q) {
    return q.nvalid ? min(q.B, max(0, *q.nvalid)) : q.B;
}
__device__ __forceinline__ double softplus_d(double x) { return fmax(x, 0.0) + log1p(exp(-fabs(x))); }

// ------------------------------------------------------------------ GEMM
// C[m, n] = sum_k A[m, k] W[k, n] (+ bias[n] on channel-0 rows, + rowbias[(walker, channel), n]),
// A and C FP64, W the FP32 weights (converted exactly). Batched over blockIdx.z with strides sA /
// sC (batch index = walker when rows_per_walker == 0). 64 x 64 tiles, 16-deep K slices, 256
// threads with a 4 x 4 patch each (rows tr + 16 i, columns tc + 16 j: a warp's shared reads of
// W are 16 consecutive doubles, those of A two broadcasts).
struct Epi64 {
    const float* bias = nullptr;
    const double* rowbias = nullptr;
    int ldrb = 0;
    int rows_per_walker = 0;    // rows of one walker (0: batch index is the walker)
};
__global__ void __launch_bounds__(256)
k64_gemm(const double* __restrict__ A, int lda, int64_t sA, const float* __restrict__ W, int ldw,
         double* __restrict__ Cm, int ldc, int64_t sC, int M, int N, int K, Epi64 e, Run64 q) {
    constexpr int BM = 64, BN = 64, BK = 16;
    const int bz = blockIdx.z;
    const int nv = valid_walkers(q);
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    if (e.rows_per_walker == 0) {
        if (bz >= nv) return;
    } else if ((int64_t)m0 >= (int64_t)nv * e.rows_per_walker) {
        return;
    }
    A += bz * sA;
    Cm += bz * sC;
    __shared__ double As[BK][BM + 1];
    __shared__ double Ws[BK][BN];
    const int tid = threadIdx.x, tr = tid / 16, tc = tid % 16;
    double acc[4][4];
    #pragma unroll
    for (int i = 0; i < 4; ++i)
        #pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    for (int k0 = 0; k0 < K; k0 += BK) {
        #pragma unroll
        for (int u = 0; u < (BM * BK) / 256; ++u) {
            const int idx = tid + u * 256, rr = idx / BK, kk = idx % BK;
            const int gm = m0 + rr, gk = k0 + kk;
            As[kk][rr] = (gm < M && gk < K) ? A[(int64_t)gm * lda + gk] : 0.0;
        }
        #pragma unroll
        for (int u = 0; u < (BK * BN) / 256; ++u) {
            const int idx = tid + u * 256, kk = idx / BN, cc = idx % BN;
            const int gk = k0 + kk, gn = n0 + cc;
            Ws[kk][cc] = (gk < K && gn < N) ? (double)W[(int64_t)gk * ldw + gn] : 0.0;
        }
        __syncthreads();
        #pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], w[4];
            #pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][tr + 16 * i];
            #pragma unroll
            for (int j = 0; j < 4; ++j) w[j] = Ws[kk][tc + 16 * j];
            #pragma unroll
            for (int i = 0; i < 4; ++i)
                #pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], w[j], acc[i][j]);
        }
        __syncthreads();
    }
    #pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + tr + 16 * i;
        if (m >= M) continue;
        const int t = m % q.C;
        const double* rb = nullptr;
        if (e.rowbias && e.rows_per_walker > 0)
            rb = e.rowbias + ((int64_t)(m / e.rows_per_walker) * q.C + t) * e.ldrb;
        #pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + tc + 16 * j;
            if (n >= N) continue;
            double v = acc[i][j];
            if (e.bias && t == 0) v += (double)e.bias[n];
            if (rb) v += rb[n];
            Cm[(int64_t)m * ldc + n] = v;
        }
    }
}

static void gemm64(const double* A, int lda, int64_t sA, const float* W, int ldw, double* C, int ldc, int64_t sC,
                   int M, int N, int K, const Epi64& e, int batch, const Run64& q, cudaStream_t s) {
    dim3 grid((N + 63) / 64, (M + 63) / 64, batch);
    timer_begin("fp64_gemm", s);
    k64_gemm<<<grid, 256, 0, s>>>(A, lda, sA, W, ldw, C, ldc, sC, M, N, K, e, q);
    timer_end("fp64_gemm", s, 2.0 * M * N * K * batch, 0.0);
    count_launch();
}

// ------------------------------------------------------------------ elementwise tanh over channels
// Y = tanh(Z) for the C channel rows of each (walker, electron): value tanh(z0); gradient rows
// s z_t with s = 1 - tanh^2; Laplacian row s z_L - 2 tanh s sum_t z_t^2 (mlp.py:57-66 under the
// forward Laplacian).
__global__ void k64_jet_tanh(const double* __restrict__ Z, int ldz, int ncols, Run64 q, double* __restrict__ Y,
                             int ldy) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t ent = idx / ncols;
    const int col = (int)(idx % ncols);
    if (ent >= (int64_t)valid_walkers(q) * q.d.n) return;
    const int C = q.C;
    const double* z = Z + ent * C * ldz + col;
    double* y = Y + ent * C * ldy + col;
    const double y0 = tanh(z[0]);
    y[0] = y0;
    if (C == 1) return;
    const double sp = 1.0 - y0 * y0;
    double sq = 0.0;
    for (int t = 1; t < C - 1; ++t) {
        const double zt = z[(int64_t)t * ldz];
        sq = fma(zt, zt, sq);
        y[(int64_t)t * ldy] = sp * zt;
    }
    y[(int64_t)(C - 1) * ldy] = sp * z[(int64_t)(C - 1) * ldz] - 2.0 * y0 * sp * sq;
}

static void jet_tanh(const double* Z, int ldz, int ncols, const Run64& q, double* Y, int ldy, cudaStream_t s) {
    const int64_t n = (int64_t)q.B * q.d.n * ncols;
    timer_begin("fp64_tanh", s);
    k64_jet_tanh<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(Z, ldz, ncols, q, Y, ldy);
    timer_end("fp64_tanh", s, 0.0, 0.0);
    count_launch();
}

// ------------------------------------------------------------------ ion maps
// him[seg][l][I][c] = tanh(ion_embed[Z_I - z_min] W_l + b_l)_c for c < eiw[l]
// (ferminet_embedding.py:171-175 h_ion_map, input_features.py:184-191 lookup); zero for Z = 0
// padding ions.
__global__ void k64_ion_maps(const float* __restrict__ P, ParamLayout L, Dims d, const int32_t* __restrict__ Zall,
                             double* __restrict__ him) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int total = d.nseg * 4 * d.N * 32;
    if (idx >= total) return;
    const int c = idx % 32, I = (idx / 32) % d.N, l = (idx / (32 * d.N)) % 4, g = idx / (32 * d.N * 4);
    const int z = Zall[g * d.N + I];
    double v = 0.0;
    if (z > 0 && c < d.eiw[l]) {
        const int zi = min(max(z - d.zmin, 0), d.zmax - d.zmin);
        const float* e = P + L.ion_embed + (int64_t)zi * d.EI;
        const float* w = P + L.h_ion_map_w[l];
        double acc = (double)P[L.h_ion_map_b[l] + c];
        for (int k = 0; k < d.EI; ++k) acc = fma((double)e[k], (double)w[k * d.eiw[l] + c], acc);
        v = tanh(acc);
    }
    him[idx] = v;
}

// ------------------------------------------------------------------ input features
// Layer-0 columns [d_iI, r_i - R_I] per ion, ion-major (input_features.py:41-68, :237-245), with
// their channels: gradients only along electron i's coordinates, Laplacian 2 / d for the distance.
__global__ void k64_features(const float* __restrict__ r, const float* __restrict__ Rall,
                             const int32_t* __restrict__ Zall, Run64 q, double* __restrict__ X, int ldx) {
    const Dims& d = q.d;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int I = (int)(idx % d.N);
    const int64_t row = idx / d.N;                 // (walker, electron, channel)
    const int t = (int)(row % q.C);
    const int64_t be = row / q.C;
    const int i = (int)(be % d.n);
    const int64_t b = be / d.n;
    if (b >= valid_walkers(q)) return;
    const int g = seg_of(d, b);
    const float* R = Rall + (int64_t)g * d.N * 3;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (Zall[g * d.N + I] > 0) {
        double df[3];
        for (int c = 0; c < 3; ++c) df[c] = (double)r[(b * d.n + i) * 3 + c] - (double)R[I * 3 + c];
        const double dist = sqrt(df[0] * df[0] + df[1] * df[1] + df[2] * df[2]);
        if (t == 0) {
            v[0] = dist; v[1] = df[0]; v[2] = df[1]; v[3] = df[2];
        } else if (t == q.C - 1) {
            v[0] = 2.0 / dist;
        } else if ((t - 1) / 3 == i) {
            const int c = (t - 1) % 3;
            v[0] = df[c] / dist;
            v[1 + c] = 1.0;
        }
    }
    double* o = X + row * ldx + I * 4;
    for (int k = 0; k < 4; ++k) o[k] = v[k];
}

// ------------------------------------------------------------------ pair streams (Taylor in d_ij)
// Warp per (walker, i, j), lane = feature column. Level-0 stream h = d_ij (zero with zero
// derivatives on the diagonal: get_distance_matrix pads the diagonal before the norm and zeroes
// it, utils/utils.py:287-305). Per level l: w = tanh(h W_w + b_w) with W_w = w_same / w_diff by
// the spins of i and j (ferminet_embedding.py:118-150); for l < 3 the stream update
// h <- residual(tanh(h W_h + b_h), h) (ferminet_embedding.py:246-262). Output
// WP[l][walker][i][j][{f, f', f''}][32].
__global__ void k64_pair_streams(const float* __restrict__ r, const float* __restrict__ P, ParamLayout L, Run64 q,
                                 double* __restrict__ WP) {
    const Dims& d = q.d;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int j = (int)(warp % d.n), i = (int)((warp / d.n) % d.n);
    const int64_t b = warp / ((int64_t)d.n * d.n);
    if (b >= valid_walkers(q)) return;
    const bool same = (i < d.nu) == (j < d.nu);
    double h0 = 0.0, h1 = 0.0, h2 = 0.0;          // stream component held by this lane
    int width = 1;
    if (i != j && lane == 0) {
        const float* ri = r + (b * d.n + i) * 3;
        const float* rj = r + (b * d.n + j) * 3;
        double s = 0.0;
        for (int c = 0; c < 3; ++c) { const double x = (double)rj[c] - (double)ri[c]; s += x * x; }
        h0 = sqrt(s); h1 = 1.0; h2 = 0.0;
    }
    const int64_t plane = (int64_t)q.B * d.n * d.n * 96;
    for (int l = 0; l < 4; ++l) {
        for (int pass = 0; pass < (l < 3 ? 2 : 1); ++pass) {
            const int64_t wo = pass == 0 ? (same ? L.w_same_w[l] : L.w_diff_w[l]) : (same ? L.h_same_w[l] : L.h_diff_w[l]);
            const int64_t bo = pass == 0 ? (same ? L.w_same_b[l] : L.w_diff_b[l]) : (same ? L.h_same_b[l] : L.h_diff_b[l]);
            double z0 = (double)P[bo + lane], z1 = 0.0, z2 = 0.0;
            for (int k = 0; k < width; ++k) {
                const double x0 = __shfl_sync(0xffffffffu, h0, k), x1 = __shfl_sync(0xffffffffu, h1, k),
                             x2 = __shfl_sync(0xffffffffu, h2, k);
                const double w = (double)P[wo + k * 32 + lane];
                z0 = fma(x0, w, z0); z1 = fma(x1, w, z1); z2 = fma(x2, w, z2);
            }
            const double y0 = tanh(z0), sp = 1.0 - y0 * y0;
            const double y1 = sp * z1, y2 = sp * z2 - 2.0 * y0 * sp * z1 * z1;
            if (pass == 0) {
                double* o = WP + l * plane + (((b * d.n + i) * d.n + j) * 3) * 32 + lane;
                o[0] = y0; o[32] = y1; o[64] = y2;
            } else if (width == 32) {
                const double rs = 0.70710678118654752440;   // (old + new) / sqrt(2), mlp.py:13-17
                h0 = (h0 + y0) * rs; h1 = (h1 + y1) * rs; h2 = (h2 + y2) * rs;
            } else {
                h0 = y0; h1 = y1; h2 = y2;
            }
        }
        width = 32;
    }
}

// ------------------------------------------------------------------ el-ion streams
// Warp per (walker, electron), lane = feature column, loop over ions. Level-0 stream
// [d_iI, r_i - R_I] (width 4) with (value, three gradients, Laplacian) in r_i; per level the
// convolution conv_ei[i] = sum_I h_ei[i, I] * him[l][I] (ferminet_embedding.py:171-175) is
// accumulated, then for l < 3 h_ei <- residual(tanh(h_ei W + b), h_ei). Output
// CE[l][walker][i][5][32].
__global__ void k64_ei_streams(const float* __restrict__ r, const float* __restrict__ Rall,
                               const int32_t* __restrict__ Zall, const float* __restrict__ P, ParamLayout L,
                               const double* __restrict__ him, Run64 q, double* __restrict__ CE) {
    const Dims& d = q.d;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int i = (int)(warp % d.n);
    const int64_t b = warp / d.n;
    if (b >= valid_walkers(q)) return;
    const int g = seg_of(d, b);
    const float* R = Rall + (int64_t)g * d.N * 3;
    double acc[4][5];
    for (int l = 0; l < 4; ++l)
        for (int c = 0; c < 5; ++c) acc[l][c] = 0.0;
    for (int I = 0; I < d.N; ++I) {
        if (Zall[g * d.N + I] <= 0) continue;        // padding ion: contributes nothing
        double df[3];
        for (int c = 0; c < 3; ++c) df[c] = (double)r[(b * d.n + i) * 3 + c] - (double)R[I * 3 + c];
        const double dist = sqrt(df[0] * df[0] + df[1] * df[1] + df[2] * df[2]);
        double h[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        if (lane == 0) {
            h[0] = dist; h[1] = df[0] / dist; h[2] = df[1] / dist; h[3] = df[2] / dist; h[4] = 2.0 / dist;
        } else if (lane < 4) {
            h[0] = df[lane - 1]; h[lane] = 1.0;
        }
        int width = 4;
        for (int l = 0; l < 4; ++l) {
            const double hm = him[(((int64_t)g * 4 + l) * d.N + I) * 32 + lane];
            for (int c = 0; c < 5; ++c) acc[l][c] = fma(h[c], hm, acc[l][c]);
            if (l == 3) break;
            double z[5] = {(double)P[L.h_ei_b[l] + lane], 0.0, 0.0, 0.0, 0.0};
            for (int k = 0; k < width; ++k) {
                const double w = (double)P[L.h_ei_w[l] + k * 32 + lane];
                for (int c = 0; c < 5; ++c) z[c] = fma(__shfl_sync(0xffffffffu, h[c], k), w, z[c]);
            }
            const double y0 = tanh(z[0]), sp = 1.0 - y0 * y0;
            double y[5];
            y[0] = y0;
            y[1] = sp * z[1]; y[2] = sp * z[2]; y[3] = sp * z[3];
            y[4] = sp * z[4] - 2.0 * y0 * sp * (z[1] * z[1] + z[2] * z[2] + z[3] * z[3]);
            const double rs = width == 32 ? 0.70710678118654752440 : 1.0;
            for (int c = 0; c < 5; ++c) h[c] = width == 32 ? (h[c] + y[c]) * rs : y[c];
            width = 32;
        }
    }
    const int64_t plane = (int64_t)q.B * d.n * 5 * 32;
    for (int l = 0; l < 4; ++l)
        for (int c = 0; c < 5; ++c) CE[l * plane + ((b * d.n + i) * 5 + c) * 32 + lane] = acc[l][c];
}

// ------------------------------------------------------------------ SchNet el-el convolution
// conv_ee[i] = sum_j w_ij * h_map_j (ferminet_embedding.py:152-169, self-pair included) with the
// product rule over the channels: w_ij depends on r only through d_ij (gradient u = (r_i - r_j) /
// d_ij along r_i, -u along r_j; |grad d|^2 = 2, Lap d = 4 / d). Thread per (channel, column) of one
// (walker, electron) block; writes columns [col0, col0 + 32) of the layer input.
__global__ void k64_conv_ee(const float* __restrict__ r, const double* __restrict__ WPl, const double* __restrict__ HM,
                            Run64 q, double* __restrict__ X, int ldx, int col0) {
    const Dims& d = q.d;
    const int i = blockIdx.x % d.n;
    const int64_t b = blockIdx.x / d.n;
    if (b >= valid_walkers(q)) return;
    const int C = q.C, n = d.n;
    __shared__ double u_sh[kMaxEl][4];       // u_ij (3) and 1 / d_ij
    for (int j = threadIdx.x; j < n; j += blockDim.x) {
        double df[3], s = 0.0;
        for (int c = 0; c < 3; ++c) {
            df[c] = (double)r[(b * n + i) * 3 + c] - (double)r[(b * n + j) * 3 + c];
            s += df[c] * df[c];
        }
        const double dist = sqrt(s);
        const double inv = j == i ? 0.0 : 1.0 / dist;
        for (int c = 0; c < 3; ++c) u_sh[j][c] = df[c] * inv;
        u_sh[j][3] = inv;
    }
    __syncthreads();
    const double* wp = WPl + ((b * n + i) * n) * 96;      // [j][3][32]
    const double* hm = HM + (b * n) * C * 32;             // [(j, t)][32]
    for (int e = threadIdx.x; e < C * 32; e += blockDim.x) {
        const int t = e / 32, col = e % 32;
        double v = 0.0;
        for (int j = 0; j < n; ++j) v = fma(wp[j * 96 + col], hm[((int64_t)j * C + t) * 32 + col], v);
        if (t > 0 && t < C - 1) {
            const int m = (t - 1) / 3, c = (t - 1) % 3;
            if (m == i) {
                for (int j = 0; j < n; ++j) {
                    if (j == i) continue;
                    v = fma(wp[j * 96 + 32 + col] * u_sh[j][c], hm[((int64_t)j * C) * 32 + col], v);
                }
            } else {
                v = fma(-wp[m * 96 + 32 + col] * u_sh[m][c], hm[((int64_t)m * C) * 32 + col], v);
            }
        } else if (t == C - 1 && C > 1) {
            for (int j = 0; j < n; ++j) {
                if (j == i) continue;
                const double w1 = wp[j * 96 + 32 + col], w2 = wp[j * 96 + 64 + col];
                const double lapw = 2.0 * w2 + 4.0 * w1 * u_sh[j][3];
                double cross = 0.0;
                for (int c = 0; c < 3; ++c)
                    cross = fma(u_sh[j][c], hm[((int64_t)j * C + 1 + 3 * i + c) * 32 + col] -
                                             hm[((int64_t)j * C + 1 + 3 * j + c) * 32 + col], cross);
                v = fma(lapw, hm[((int64_t)j * C) * 32 + col], v);
                v = fma(2.0 * w1, cross, v);
            }
        }
        X[(((b * n + i) * C) + t) * (int64_t)ldx + col0 + col] = v;
    }
}

// conv_ei of one level expanded to the channels: value, electron i's own gradient rows and the
// Laplacian; zero elsewhere. Columns [col0, col0 + width).
__global__ void k64_conv_ei(const double* __restrict__ CEl, Run64 q, int width, double* __restrict__ X, int ldx,
                            int col0) {
    const Dims& d = q.d;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int col = (int)(idx % width);
    const int64_t row = idx / width;
    const int t = (int)(row % q.C);
    const int64_t be = row / q.C;
    const int i = (int)(be % d.n);
    const int64_t b = be / d.n;
    if (b >= valid_walkers(q)) return;
    const double* ce = CEl + be * 5 * 32 + col;
    double v = 0.0;
    if (t == 0) v = ce[0];
    else if (t == q.C - 1) v = ce[4 * 32];
    else if ((t - 1) / 3 == i) v = ce[(1 + (t - 1) % 3) * 32];
    X[row * ldx + col0 + col] = v;
}

// Spin means of the h columns per (walker, channel): M[(b, t)] = [mean over up electrons,
// mean over down electrons] (SymmetricFeatures, ferminet_embedding.py:52-94).
__global__ void k64_spin_means(const double* __restrict__ X, int ldx, int hw, Run64 q, double* __restrict__ M) {
    const Dims& d = q.d;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int col = (int)(idx % hw);
    const int64_t bt = idx / hw;
    const int t = (int)(bt % q.C);
    const int64_t b = bt / q.C;
    if (b >= valid_walkers(q)) return;
    double su = 0.0, sd = 0.0;
    for (int i = 0; i < d.n; ++i) {
        const double x = X[((b * d.n + i) * q.C + t) * (int64_t)ldx + col];
        if (i < d.nu) su += x; else sd += x;
    }
    M[bt * 2 * hw + col] = su / d.nu;
    M[bt * 2 * hw + hw + col] = sd / d.nd;
}

// ------------------------------------------------------------------ envelope orbitals
// MO[b][k][t][i][o] = env_i(k, o) * BF[(b, i, t)][k n + o] with the product rule; the isotropic
// exponential envelope env = sum_I w exp(-softplus(alpha) d_iI) (envelope_orbitals.py:96-127)
// depends only on r_i: gradient -a e u, Laplacian e (a^2 - 2 a / d).
__global__ void k64_envelope_mo(const float* __restrict__ r, const float* __restrict__ Rall,
                                const int32_t* __restrict__ Zall, const float* __restrict__ P, ParamLayout L, Run64 q,
                                const double* __restrict__ BF, int ldbf, double* __restrict__ MO) {
    const Dims& d = q.d;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int n = d.n, C = q.C;
    const int o = (int)(idx % n);
    const int i = (int)((idx / n) % n);
    const int k = (int)((idx / ((int64_t)n * n)) % d.K);
    const int64_t b = idx / ((int64_t)n * n * d.K);
    if (b >= valid_walkers(q)) return;
    const int g = seg_of(d, b);
    const float* R = Rall + (int64_t)g * d.N * 3;
    const bool up = i < d.nu;
    const int64_t col = (int64_t)k * n + o;
    const float* alpha = P + (up ? L.alpha_up : L.alpha_dn);
    const float* wts = P + (up ? L.weights_up : L.weights_dn);
    double e0 = 0.0, eg[3] = {0.0, 0.0, 0.0}, eL = 0.0;
    for (int I = 0; I < d.N; ++I) {
        if (Zall[g * d.N + I] <= 0) continue;
        double df[3];
        for (int c = 0; c < 3; ++c) df[c] = (double)r[(b * n + i) * 3 + c] - (double)R[I * 3 + c];
        const double dist = sqrt(df[0] * df[0] + df[1] * df[1] + df[2] * df[2]);
        const double a = softplus_d((double)alpha[(int64_t)I * d.KN + col]);
        const double e = (double)wts[(int64_t)I * d.KN + col] * exp(-a * dist);
        e0 += e;
        if (C > 1) {
            for (int c = 0; c < 3; ++c) eg[c] -= a * e * df[c] / dist;
            eL += e * (a * a - 2.0 * a / dist);
        }
    }
    const double* bf = BF + ((b * n + i) * C) * (int64_t)ldbf + col;
    double* mo = MO + (((b * d.K + k) * C) * n + i) * (int64_t)n + o;
    const int64_t plane = (int64_t)n * n;
    const double b0 = bf[0];
    mo[0] = e0 * b0;
    if (C == 1) return;
    for (int t = 1; t < C - 1; ++t) {
        double v = e0 * bf[(int64_t)t * ldbf];
        if ((t - 1) / 3 == i) v = fma(eg[(t - 1) % 3], b0, v);
        mo[t * plane] = v;
    }
    double lap = fma(eL, b0, e0 * bf[(int64_t)(C - 1) * ldbf]);
    for (int c = 0; c < 3; ++c) lap = fma(2.0 * eg[c], bf[(int64_t)(1 + 3 * i + c) * ldbf], lap);
    mo[(C - 1) * plane] = lap;
}

// ------------------------------------------------------------------ determinants
// FP64 Gauss-Jordan elimination with partial pivoting of the value-channel Slater matrix of one
// (walker, determinant): log|det|, sign (jnp.linalg.slogdet, wavefunction.py:69-73) and, in
// tangent passes, the inverse. Block of 128 threads, [A | I] in shared memory.
__global__ void __launch_bounds__(128)
k64_slogdet_inv(const double* __restrict__ MO, Run64 q, double* __restrict__ logdet, double* __restrict__ sign,
                double* __restrict__ Ainv) {
    const Dims& d = q.d;
    const int n = d.n, C = q.C, w2 = 2 * n + 1;
    const int64_t mat = blockIdx.x;                  // b * K + k
    if (mat / d.K >= valid_walkers(q)) return;
    extern __shared__ double aug[];                  // [n][2n + 1], then n factors
    double* fac = aug + (int64_t)n * w2;
    __shared__ int s_piv;
    __shared__ double s_logabs, s_sign;
    const int tid = threadIdx.x;
    const double* A = MO + (mat * C) * (int64_t)n * n;
    const bool want_inv = Ainv != nullptr;
    const int cols = want_inv ? 2 * n : n;
    for (int e = tid; e < n * 2 * n; e += blockDim.x) {
        const int rr = e / (2 * n), cc = e % (2 * n);
        aug[rr * w2 + cc] = cc < n ? A[rr * n + cc] : (cc - n == rr ? 1.0 : 0.0);
    }
    if (tid == 0) { s_logabs = 0.0; s_sign = 1.0; }
    __syncthreads();
    bool singular = false;
    for (int p = 0; p < n; ++p) {
        if (tid < 32) {
            double best = -1.0; int bi = p;
            for (int rr = p + tid; rr < n; rr += 32) {
                const double v = fabs(aug[rr * w2 + p]);
                if (v > best) { best = v; bi = rr; }
            }
            for (int off = 16; off > 0; off >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, best, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ov > best || (ov == best && oi < bi)) { best = ov; bi = oi; }
            }
            if (tid == 0) s_piv = bi;
        }
        __syncthreads();
        const int piv = s_piv;
        const double pv = aug[piv * w2 + p];
        if (pv == 0.0 || !isfinite(pv)) { singular = true; break; }
        if (piv != p) {
            for (int cc = p + tid; cc < cols; cc += blockDim.x) {
                const double x = aug[p * w2 + cc];
                aug[p * w2 + cc] = aug[piv * w2 + cc];
                aug[piv * w2 + cc] = x;
            }
        }
        __syncthreads();
        const double inv = 1.0 / pv;
        if (tid == 0) {
            s_logabs += log(fabs(pv));
            s_sign *= (pv < 0.0) != (piv != p) ? -1.0 : 1.0;
        }
        for (int cc = p + 1 + tid; cc < cols; cc += blockDim.x) aug[p * w2 + cc] *= inv;
        for (int rr = tid; rr < n; rr += blockDim.x) fac[rr] = aug[rr * w2 + p];
        __syncthreads();
        const int span = cols - (p + 1);
        for (int e = tid; e < n * span; e += blockDim.x) {
            const int rr = e / span, cc = p + 1 + e % span;
            if (rr == p || (!want_inv && rr < p)) continue;   // value passes: LU rows only
            aug[rr * w2 + cc] = fma(-fac[rr], aug[p * w2 + cc], aug[rr * w2 + cc]);
        }
        __syncthreads();
    }
    if (tid == 0) {
        logdet[mat] = singular ? -INFINITY : s_logabs;
        sign[mat] = singular ? 0.0 : s_sign;
    }
    if (want_inv) {
        double* out = Ainv + mat * (int64_t)n * n;
        for (int e = tid; e < n * n; e += blockDim.x) out[e] = singular ? 0.0 : aug[(e / n) * w2 + n + e % n];
    }
}

// g_t = tr(A^-1 dA_t) over the 3n gradient channels and lap = tr(A^-1 Lap A) - sum_t tr((A^-1 dA_t)^2)
// of one (walker, determinant), all in FP64.
__global__ void __launch_bounds__(128)
k64_det_tangents(const double* __restrict__ MO, const double* __restrict__ Ainv, const double* __restrict__ sign,
                 Run64 q, double* __restrict__ g, double* __restrict__ lapdet) {
    const Dims& d = q.d;
    const int n = d.n, C = q.C, n3 = 3 * n, nn = n * n;
    const int64_t mat = blockIdx.x;
    if (mat / d.K >= valid_walkers(q)) return;
    extern __shared__ double sm[];
    double* Ai = sm;
    double* dA = Ai + nn;
    double* Cm = dA + nn;
    __shared__ double red[2][4];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (sign[mat] == 0.0) {
        for (int t = tid; t < n3; t += blockDim.x) g[mat * n3 + t] = 0.0;
        if (tid == 0) lapdet[mat] = 0.0;
        return;
    }
    for (int e = tid; e < nn; e += blockDim.x) Ai[e] = Ainv[mat * nn + e];
    double lap_acc = 0.0;
    for (int t = 1; t < C; ++t) {
        const double* src = MO + ((mat * C) + t) * (int64_t)nn;
        __syncthreads();
        for (int e = tid; e < nn; e += blockDim.x) dA[e] = src[e];
        __syncthreads();
        double tr = 0.0, tr2 = 0.0;
        for (int e = tid; e < nn; e += blockDim.x) {
            const int a = e / n, c = e % n;
            double acc = 0.0;
            for (int m = 0; m < n; ++m) acc = fma(Ai[a * n + m], dA[m * n + c], acc);
            Cm[e] = acc;
            if (a == c) tr += acc;
        }
        __syncthreads();
        if (t != C - 1)
            for (int e = tid; e < nn; e += blockDim.x) tr2 = fma(Cm[e], Cm[(e % n) * n + e / n], tr2);
        tr = warp_sum(tr); tr2 = warp_sum(tr2);
        if (lane == 0) { red[0][wid] = tr; red[1][wid] = tr2; }
        __syncthreads();
        if (tid == 0) {
            const double s0 = red[0][0] + red[0][1] + red[0][2] + red[0][3];
            const double s1 = red[1][0] + red[1][1] + red[1][2] + red[1][3];
            if (t == C - 1) lap_acc += s0;
            else { g[mat * n3 + (t - 1)] = s0; lap_acc -= s1; }
        }
    }
    if (tid == 0) lapdet[mat] = lap_acc;
}

// Jastrow output: jas[(b, t)] = sum_i sum_c J2[(b, i, t)][c] w2[c] (wavefunction.py:57-59, linear
// output without bias, summed over electrons). Warp per (walker, channel).
__global__ void k64_jastrow_out(const double* __restrict__ J2, int ldj, const float* __restrict__ w2, Run64 q,
                                double* __restrict__ jas) {
    const Dims& d = q.d;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int t = (int)(warp % q.C);
    const int64_t b = warp / q.C;
    if (b >= valid_walkers(q)) return;
    double acc = 0.0;
    for (int i = 0; i < d.n; ++i) {
        const double* row = J2 + ((b * d.n + i) * q.C + t) * (int64_t)ldj;
        for (int c = lane; c < d.J1; c += 32) acc = fma(row[c], (double)w2[c], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) jas[b * q.C + t] = acc;
}

// ------------------------------------------------------------------ plan and launch sequence
struct Plan64 {
    int Bc, C;
    double* him;
    double *XA, *XB, *Zt, *HM, *M, *WB, *WP, *CE, *BF, *MO, *logdet, *sign, *Ainv, *g, *lapdet, *J1, *J2, *jas;
    size_t bytes;
};
static const int kXW64 = 320;    // layer 1..3 input [h (256) | conv_ee (32) | conv_ei (32)]

static Plan64 carve64(const Dims& d, int C, int Bc, void* ws) {
    Carver c(ws, (size_t)-1);
    Plan64 p;
    p.Bc = Bc; p.C = C;
    const int64_t rows = (int64_t)Bc * d.n * C;
    const int w0 = d.hw[0] + d.E + d.eiw[0];
    p.him = c.take<double>((size_t)kMaxSeg * 4 * d.N * 32);
    p.XA = c.take<double>(rows * kXW64);
    p.XB = c.take<double>(rows * std::max(kXW64, w0));
    p.Zt = c.take<double>(rows * std::max(d.D, d.J0));
    p.HM = c.take<double>(rows * 32);
    p.M = c.take<double>((int64_t)Bc * C * 2 * d.D);
    p.WB = c.take<double>((int64_t)Bc * C * d.D);
    p.WP = c.take<double>((int64_t)4 * Bc * d.n * d.n * 96);
    p.CE = c.take<double>((int64_t)4 * Bc * d.n * 5 * 32);
    p.BF = c.take<double>(rows * d.KN);
    p.MO = c.take<double>((int64_t)Bc * d.K * C * d.n * d.n);
    p.logdet = c.take<double>((int64_t)Bc * d.K);
    p.sign = c.take<double>((int64_t)Bc * d.K);
    if (C > 1) {
        p.Ainv = c.take<double>((int64_t)Bc * d.K * d.n * d.n);
        p.g = c.take<double>((int64_t)Bc * d.K * 3 * d.n);
        p.lapdet = c.take<double>((int64_t)Bc * d.K);
    } else {
        p.Ainv = p.g = p.lapdet = nullptr;
    }
    p.J1 = c.take<double>(rows * d.J0);
    p.J2 = c.take<double>(rows * d.J1);
    p.jas = c.take<double>((int64_t)Bc * C);
    p.bytes = c.used;
    return p;
}

static const size_t kChunkBudget64 = (size_t)6 << 30;

static int choose_chunk64(const Dims& d, int C, int B, size_t budget) {
    const size_t one = carve64(d, C, 1, nullptr).bytes, two = carve64(d, C, 2, nullptr).bytes;
    const size_t per = std::max<size_t>(two > one ? two - one : one, 1);
    const size_t fixed = one > per ? one - per : 0;
    const size_t avail = budget > fixed ? budget - fixed : per;
    // batched GEMMs put the walker on grid.z (at most 65535)
    int bc = std::min((int)std::min<size_t>(std::max<size_t>(1, avail / per), 32768), B);
    while (bc > 1 && carve64(d, C, bc, nullptr).bytes > budget) bc -= std::max(1, bc / 32);
    return bc;
}

static inline unsigned blocks_for(int64_t n, int tpb) { return (unsigned)((n + tpb - 1) / tpb); }

// The FP64 forward (value or tangent) of one chunk of walkers.
static int run_chunk64(const Plan64& p, const Dims& d0, int Bc, const float* P, const ParamLayout& L, const float* main_w[4],
                       const float* mean_w[4], const float* r, const float* R, const int32_t* Z, const int32_t* seg,
                       const int* nvalid, float* lp, float* phase, float* E, float* grad, cudaStream_t s) {
    Dims d = d0;
    d.seg = seg;
    Run64 q;
    q.d = d; q.C = p.C; q.B = Bc; q.nvalid = nvalid;
    const int C = p.C, n = d.n;
    const int64_t rows = (int64_t)Bc * n * C;
    const bool tang = C > 1;
    const int w0 = d.hw[0] + d.E + d.eiw[0];
    // layer-0 input [features | conv_ee | conv_ei] in XB (free until layer 1 writes it)
    timer_begin("fp64_streams", s);
    k64_features<<<blocks_for(rows * d.N, 256), 256, 0, s>>>(r, R, Z, q, p.XB, w0);
    count_launch();
    k64_pair_streams<<<blocks_for((int64_t)Bc * n * n * 32, 256), 256, 0, s>>>(r, P, L, q, p.WP);
    count_launch();
    k64_ei_streams<<<blocks_for((int64_t)Bc * n * 32, 256), 256, 0, s>>>(r, R, Z, P, L, p.him, q, p.CE);
    count_launch();
    timer_end("fp64_streams", s, 0.0, 0.0);
    double* xin = p.XB;
    int ldin = w0;
    for (int l = 0; l < 4; ++l) {
        double* xout = (l % 2 == 0) ? p.XA : p.XB;
        const int hw = d.hw[l];
        // h_map = tanh(h W + b) -> HM
        Epi64 em; em.bias = P + L.h_map_b[l]; em.rows_per_walker = n * C;
        gemm64(xin, ldin, 0, P + L.h_map_w[l], d.E, p.Zt, d.E, 0, (int)rows, d.E, hw, em, 1, q, s);
        jet_tanh(p.Zt, d.E, d.E, q, p.HM, 32, s);
        // convolutions into columns [hw, hw + E + eiw)
        timer_begin("fp64_conv", s);
        k64_conv_ee<<<(unsigned)((int64_t)Bc * n), 128, 0, s>>>(r, p.WP + (int64_t)l * Bc * n * n * 96, p.HM, q, xin,
                                                                 ldin, hw);
        timer_end("fp64_conv", s, 0.0, 0.0);
        count_launch();
        k64_conv_ei<<<blocks_for(rows * d.eiw[l], 256), 256, 0, s>>>(p.CE + (int64_t)l * Bc * n * 5 * 32, q, d.eiw[l],
                                                                      xin, ldin, hw + d.E);
        count_launch();
        // spin means and their per-(walker, channel) product with the mean rows (+ the layer bias)
        k64_spin_means<<<blocks_for((int64_t)Bc * C * hw, 256), 256, 0, s>>>(xin, ldin, hw, q, p.M);
        count_launch();
        Epi64 eb; eb.bias = P + L.h_el_b[l]; eb.rows_per_walker = C;
        gemm64(p.M, 2 * hw, 0, mean_w[l], d.D, p.WB, d.D, 0, Bc * C, d.D, 2 * hw, eb, 1, q, s);
        // h_el = tanh([h | conv_ee | conv_ei] W_main + mean term) (ferminet_embedding.py:233-241)
        Epi64 e3; e3.rowbias = p.WB; e3.ldrb = d.D; e3.rows_per_walker = n * C;
        gemm64(xin, ldin, 0, main_w[l], d.D, p.Zt, d.D, 0, (int)rows, d.D, hw + d.E + d.eiw[l], e3, 1, q, s);
        jet_tanh(p.Zt, d.D, d.D, q, xout, kXW64, s);
        xin = xout;
        ldin = kXW64;
    }
    const double* H = xin;
    // backflow per spin (envelope_orbitals.py:46-75): the electrons of one spin are nu * C
    // consecutive rows of each walker
    for (int spin = 0; spin < 2; ++spin) {
        const int i0 = spin == 0 ? 0 : d.nu, ns = spin == 0 ? d.nu : d.nd;
        Epi64 e0;
        gemm64(H + (int64_t)i0 * C * kXW64, kXW64, (int64_t)n * C * kXW64, P + (spin == 0 ? L.bf_up : L.bf_dn), d.KN,
               p.BF + (int64_t)i0 * C * d.KN, d.KN, (int64_t)n * C * d.KN, ns * C, d.KN, d.D, e0, Bc, q, s);
    }
    timer_begin("fp64_envelope", s);
    k64_envelope_mo<<<blocks_for((int64_t)Bc * d.K * n * n, 128), 128, 0, s>>>(r, R, Z, P, L, q, p.BF, d.KN, p.MO);
    timer_end("fp64_envelope", s, 0.0, 0.0);
    count_launch();
    const int nmat = Bc * d.K;
    const size_t sm_lu = ((size_t)n * (2 * n + 1) + n) * sizeof(double);
    if (sm_lu > 48 * 1024) cudaFuncSetAttribute(k64_slogdet_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_lu);
    timer_begin("fp64_lu", s);
    k64_slogdet_inv<<<nmat, 128, sm_lu, s>>>(p.MO, q, p.logdet, p.sign, tang ? p.Ainv : nullptr);
    timer_end("fp64_lu", s, 0.0, 0.0);
    count_launch();
    if (tang) {
        const size_t sm_t = (size_t)3 * n * n * sizeof(double);
        if (sm_t > 48 * 1024) cudaFuncSetAttribute(k64_det_tangents, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_t);
        timer_begin("fp64_det_tangents", s);
        k64_det_tangents<<<nmat, 128, sm_t, s>>>(p.MO, p.Ainv, p.sign, q, p.g, p.lapdet);
        timer_end("fp64_det_tangents", s, 0.0, 0.0);
        count_launch();
    }
    // Jastrow MLP([64, 64, 1]) on the final embedding (wavefunction.py:42-60)
    Epi64 j0; j0.bias = P + L.jas_b[0]; j0.rows_per_walker = n * C;
    gemm64(H, kXW64, 0, P + L.jas_w[0], d.J0, p.Zt, d.J0, 0, (int)rows, d.J0, d.D, j0, 1, q, s);
    jet_tanh(p.Zt, d.J0, d.J0, q, p.J1, d.J0, s);
    Epi64 j1; j1.bias = P + L.jas_b[1]; j1.rows_per_walker = n * C;
    gemm64(p.J1, d.J0, 0, P + L.jas_w[1], d.J1, p.Zt, d.J1, 0, (int)rows, d.J1, d.J0, j1, 1, q, s);
    jet_tanh(p.Zt, d.J1, d.J1, q, p.J2, d.J1, s);
    k64_jastrow_out<<<blocks_for((int64_t)Bc * C * 32, 256), 256, 0, s>>>(p.J2, d.J1, P + L.jas_w[2], q, p.jas);
    count_launch();
    // log-sum-exp over determinants, derivatives of log psi^2, kinetic + FP64 Coulomb energy
    Dims dc = d;
    dc.Tp = C;
    launch_combine(p.logdet, p.sign, p.g, p.lapdet, p.jas, r, R, Z, dc, Bc, lp, phase, E, grad, s, 1, nvalid);
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

// FP64 determinant algebra on float32 Slater-matrix channels MO[b][k][t][i][o] (t < d.T): the
// channels are widened to FP64 in MO64, then the FP64 LU / Gauss-Jordan inverse and the FP64
// determinant tangents of this file give log|det|, sign, the gradient traces and the Laplacian
// term. Used by the plain form's FP64-determinant variant.
__global__ void k64_widen(const float* __restrict__ x, int64_t n, double* __restrict__ y) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (double)x[i];
}

int fp64_dets_from_f32(const float* MO, const Dims& d, int Bc, double* MO64, double* Ainv64, double* logdet,
                       double* sign, double* g, double* lapdet, cudaStream_t s) {
    Run64 q;
    q.d = d; q.C = d.T; q.B = Bc; q.nvalid = nullptr;
    const int n = d.n, nmat = Bc * d.K;
    const int64_t ne = (int64_t)nmat * d.T * n * n;
    k64_widen<<<(unsigned)std::min<int64_t>((ne + 255) / 256, 152 * 32), 256, 0, s>>>(MO, ne, MO64);
    count_launch();
    const bool tang = d.T > 1;
    const size_t sm_lu = ((size_t)n * (2 * n + 1) + n) * sizeof(double);
    if (sm_lu > 48 * 1024) cudaFuncSetAttribute(k64_slogdet_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_lu);
    k64_slogdet_inv<<<nmat, 128, sm_lu, s>>>(MO64, q, logdet, sign, tang ? Ainv64 : nullptr);
    count_launch();
    if (tang) {
        const size_t sm_t = (size_t)3 * n * n * sizeof(double);
        if (sm_t > 48 * 1024) cudaFuncSetAttribute(k64_det_tangents, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_t);
        k64_det_tangents<<<nmat, 128, sm_t, s>>>(MO64, Ainv64, sign, q, g, lapdet);
        count_launch();
    }
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

int fp64_max_chunk(const DwArch* a, bool tang) {
    Dims d = make_dims(a, tang);
    const int C = tang ? 3 * d.n + 2 : 1;
    return choose_chunk64(d, C, 1 << 30, kChunkBudget64);
}

size_t fp64_plan_bytes(const DwArch* a, int B, bool tang) {
    Dims d = make_dims(a, tang);
    const int C = tang ? 3 * d.n + 2 : 1;
    return (carve64(d, C, choose_chunk64(d, C, std::max(B, 1), kChunkBudget64), nullptr).bytes + 4096 + 255) / 256 * 256;
}

int fp64_forward_all(const DwArch* a, const float* P, const void* prepared, const float* r, int B, const float* R,
                     const int32_t* Z, float* lp, float* phase, float* E, float* grad, bool tang, void* ws,
                     size_t ws_bytes, cudaStream_t s, const int32_t* seg, int nseg, const int* nvalid) {
    Dims d = make_dims(a, tang);
    if (nseg < 1 || nseg > kMaxSeg || (nseg > 1 && !seg)) return DW_ERR_ARG;
    const int C = tang ? 3 * d.n + 2 : 1;
    d.T = C; d.Tp = C; d.lap = tang ? C - 1 : -1;
    d.nseg = nseg;
    ParamLayout L;
    make_layout(a, &L);
    const float* main_w[4];
    const float* mean_w[4];
    prepared_fp32_layers(a, prepared, main_w, mean_w);
    const int bc = choose_chunk64(d, C, B, kChunkBudget64);
    if (nvalid && bc < B) return DW_ERR_ARG;       // a device-side walker count needs one chunk
    Plan64 p = carve64(d, C, bc, ws);
    if (p.bytes > ws_bytes) return DW_ERR_WORKSPACE;
    const int total = nseg * 4 * d.N * 32;
    k64_ion_maps<<<(total + 255) / 256, 256, 0, s>>>(P, L, d, Z, p.him);
    count_launch();
    for (int b0 = 0; b0 < B; b0 += bc) {
        const int nb = std::min(bc, B - b0);
        DW_CHECK(run_chunk64(p, d, nb, P, L, main_w, mean_w, r + (int64_t)b0 * d.n * 3, R, Z, seg ? seg + b0 : nullptr,
                             nvalid, lp + b0, phase ? phase + b0 : nullptr, E ? E + b0 : nullptr,
                             grad ? grad + (int64_t)b0 * 3 * d.n : nullptr, s));
    }
    return DW_OK;
}

}  // namespace dw
