// Per-walker network kernels of the dpe4 wavefunction with forward-mode Laplacian.
//
// Channel convention for every per-electron tensor X[(b, i, t), col] (rows ordered walker,
// electron, channel; Tp rows per electron):
//   t = 0            value
//   t = 1 + 3m + c   d/d r_{m,c}   (m = electron, c = x,y,z)
//   t = 3n + 1       Laplacian over all 3n coordinates
//   t > 3n + 1       zero padding up to Tp (a power of two)
// In value-only mode Tp = 1.
//
// The 2-el streams depend on r only through d_ij = |r_j - r_i|, so they are carried in
// 1-D Taylor form (f, df/dd, d2f/dd2) and expanded to the 3n channels where they are
// contracted (SchNet convolution). The el-ion streams depend on r_i - R_I only and carry
// (value, 3 gradients w.r.t. r_i, Laplacian w.r.t. r_i).
#include "common.cuh"
#include "net.cuh"
#include <type_traits>

namespace dw {

// ------------------------------------------------------------------ ion maps (constant per geometry)
// him[l][I][f] = tanh(Embed(Z_I - z_min) @ W_ion_map_l + b)   (ferminet_embedding.py:172-174,
// input_features.py:184-191)
__global__ void k_ion_maps(const float* __restrict__ P, ParamLayout L, Dims d, const int32_t* __restrict__ Z,
                           float* __restrict__ him) {
    // him[seg][l][I][f]; padding ions (Z = 0) map to 0 so they drop out of conv_ei
    for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < d.nseg * 4 * d.N * 32; idx += gridDim.x * blockDim.x) {
        const int sg = idx / (4 * d.N * 32), li = idx % (4 * d.N * 32);
        int l = li / (d.N * 32), rem = li % (d.N * 32), I = rem / 32, f = rem % 32;
        float v = 0.f;
        const int zI = Z[sg * d.N + I];
        if (f < d.eiw[l] && zI > 0) {
            int z = zI - d.zmin;
            z = z < 0 ? 0 : (z > d.zmax - d.zmin ? d.zmax - d.zmin : z);
            const float* emb = P + L.ion_embed + (int64_t)z * d.EI;
            const float* W = P + L.h_ion_map_w[l];
            float acc = P[L.h_ion_map_b[l] + f];
            for (int k = 0; k < d.EI; ++k) acc += emb[k] * W[k * d.eiw[l] + f];
            v = tanhf(acc);
        }
        him[idx] = v;
    }
}

// ------------------------------------------------------------------ input features
// X0[(b,i,t), 4I + q] = [d_iI, (r_i - R_I)_{x,y,z}] with tangents (input_features.py:51-68, :237-239).
// Also zero-fills the padding columns of the layer-0 input.
template <class Act>
__global__ void k_features(const float* __restrict__ r, const float* __restrict__ Rall, const int32_t* __restrict__ Zall,
                           Dims d, int B, Act* __restrict__ X0) {
    __shared__ float geo[16][5];  // per ion: s_x, s_y, s_z, |s|, 1/|s|; |s| < 0 marks a padding ion
    const int bi = blockIdx.x;    // b * n + i
    const int i = bi % d.n;
    const int sg = seg_of(d, bi / d.n);
    const float* R = Rall + (size_t)sg * d.N * 3;
    const int32_t* Z = Zall + (size_t)sg * d.N;
    const float* ri = r + (int64_t)bi * 3;
    if (threadIdx.x < d.N) {
        const int I = threadIdx.x;
        const float sx = ri[0] - R[I * 3 + 0], sy = ri[1] - R[I * 3 + 1], sz = ri[2] - R[I * 3 + 2];
        const float dd = sqrtf(sx * sx + sy * sy + sz * sz);
        geo[I][0] = sx; geo[I][1] = sy; geo[I][2] = sz;
        geo[I][3] = Z[I] > 0 ? dd : -1.f;
        geo[I][4] = 1.f / dd;
    }
    __syncthreads();
    const int width = d.kw[0], nf = 4 * d.N;
    const int64_t row0 = (int64_t)bi * d.Tp;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int t = warp; t < d.Tp; t += nwarps) {
        // channel t: 0 value, 1 + 3 m + c derivative by r_m,c (non-zero for m == i only), lap
        const int c = (t >= 1 && t <= 3 * d.n && (t - 1) / 3 == i) ? (t - 1) % 3 : -1;
        for (int col = lane; col < width; col += 32) {
            if (col >= nf && col < nf + d.E + 4) continue;   // conv columns written by the convolution
            float v = 0.f;
            if (col < nf) {
                const int I = col >> 2, q = col & 3;
                const float dd = geo[I][3];
                if (dd >= 0.f) {
                    if (t == 0) v = q == 0 ? dd : geo[I][q - 1];
                    else if (t == d.lap) v = q == 0 ? 2.f * geo[I][4] : 0.f;
                    else if (c >= 0) v = q == 0 ? geo[I][c] * geo[I][4] : (q - 1 == c ? 1.f : 0.f);
                }
            }
            ActIO<Act>::store(X0, row0 + t, width, col, v);
        }
    }
}

// ------------------------------------------------------------------ 2-el and el-ion streams
// One thread per unordered electron pair (pair streams) or per (electron, ion) (el-ion stream),
// its CH x 32 activations in registers. Pair streams: ferminet_embedding.py:137-150 (w maps)
// and :247-253 (h_same / h_diff MLPs, residual (x+y)/sqrt2 on equal widths, mlp.py:13-17).
// El-ion stream: ferminet_embedding.py:259-262.
//
// The 2-el features depend on r only through d = |r_j - r_i| (use_el_el_differences=False),
// so they carry CH = 3 Taylor channels (f, df/dd, d2f/dd2); the el-ion stream carries
// CH = 5 channels (f, d/dx_i, d/dy_i, d/dz_i, Laplacian_i). Value-only mode: CH = 1.
//
// WP[l][b][i*n+j][ch][32] and HE[l][b][i*N+I][ch][32].

// y = tanh(z) with Taylor / Laplacian channels; CH = 3: 1-D Taylor (f, f', f''), CH = 5:
// (f, 3 gradients, Laplacian), CH = 1: value only.
template <int CH>
__device__ __forceinline__ void tanh_taylor(const float (&z)[CH], float (&y)[CH]) {
    const float t = tanhf(z[0]), d1 = 1.f - t * t;
    y[0] = t;
    if (CH == 3) { y[1] = d1 * z[1]; y[2] = d1 * z[2] - 2.f * t * d1 * z[1] * z[1]; }
    if (CH == 5) {
        const float sq = z[1] * z[1] + z[2] * z[2] + z[3] * z[3];
        y[1] = d1 * z[1]; y[2] = d1 * z[2]; y[3] = d1 * z[3]; y[4] = d1 * z[4] - 2.f * t * d1 * sq;
    }
}

// out[c][f] = tanh-Taylor(sum_k h[c][k] W[k][f] + b[f] [c == 0]) for four output features at a time.
template <int CH>
__device__ __forceinline__ void dense_quad(const float (&h)[CH][32], int in_w, const float* __restrict__ W,
                                           const float* __restrict__ bias, int f, float (&y)[CH][4]) {
    float z[CH][4];
    const float4 b4 = __ldg(reinterpret_cast<const float4*>(bias + f));
    #pragma unroll
    for (int c = 0; c < CH; ++c) { z[c][0] = z[c][1] = z[c][2] = z[c][3] = 0.f; }
    z[0][0] = b4.x; z[0][1] = b4.y; z[0][2] = b4.z; z[0][3] = b4.w;
    #pragma unroll
    for (int k = 0; k < 32; ++k) {
        if (k < in_w) {
            const float4 w = __ldg(reinterpret_cast<const float4*>(W + k * 32 + f));
            #pragma unroll
            for (int c = 0; c < CH; ++c) {
                z[c][0] = fmaf(h[c][k], w.x, z[c][0]); z[c][1] = fmaf(h[c][k], w.y, z[c][1]);
                z[c][2] = fmaf(h[c][k], w.z, z[c][2]); z[c][3] = fmaf(h[c][k], w.w, z[c][3]);
            }
        }
    }
    #pragma unroll
    for (int u = 0; u < 4; ++u) {
        float zz[CH], yy[CH];
        #pragma unroll
        for (int c = 0; c < CH; ++c) zz[c] = z[c][u];
        tanh_taylor<CH>(zz, yy);
        #pragma unroll
        for (int c = 0; c < CH; ++c) y[c][u] = yy[c];
    }
}

// h <- residual(dense(h)) through one shared-memory row per thread (row pitch CH*32 + 1).
template <int CH>
__device__ __forceinline__ void stream_layer(float (&h)[CH][32], int in_w, const float* __restrict__ W,
                                             const float* __restrict__ bias, bool resid, float* row) {
    for (int f = 0; f < 32; f += 4) {
        float y[CH][4];
        dense_quad<CH>(h, in_w, W, bias, f, y);
        #pragma unroll
        for (int c = 0; c < CH; ++c)
            #pragma unroll
            for (int u = 0; u < 4; ++u) row[c * 32 + f + u] = y[c][u];
    }
    const float rs = 0.70710678118654752f;
    #pragma unroll
    for (int c = 0; c < CH; ++c)
        #pragma unroll
        for (int k = 0; k < 32; ++k) h[c][k] = resid ? (h[c][k] + row[c * 32 + k]) * rs : row[c * 32 + k];
}

template <int CH>
__global__ void __launch_bounds__(128)
k_pair_streams(const float* __restrict__ r, const float* __restrict__ P, ParamLayout L, Dims d, int B,
               float* __restrict__ WP, float* __restrict__ HP) {
    extern __shared__ float srow[];
    float* row = srow + threadIdx.x * (CH * 32 + 1);
    const int npair = d.n * (d.n + 1) / 2;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (int64_t)B * npair) return;
    const int b = (int)(gid / npair), p = (int)(gid % npair);
    int i = 0, rem = p;
    while (rem >= d.n - i) { rem -= d.n - i; ++i; }
    const int j = i + rem;
    const bool same = (i < d.nu) == (j < d.nu);
    const float* rb = r + (int64_t)b * d.n * 3;
    float dd = 0.f;
    if (i != j) {
        const float dx = rb[j * 3] - rb[i * 3], dy = rb[j * 3 + 1] - rb[i * 3 + 1], dz = rb[j * 3 + 2] - rb[i * 3 + 2];
        dd = sqrtf(dx * dx + dy * dy + dz * dz);
    }
    float h[CH][32];
    #pragma unroll
    for (int c = 0; c < CH; ++c)
        #pragma unroll
        for (int k = 0; k < 32; ++k) h[c][k] = 0.f;
    // input feature [dist]: value d, d' = 1, d'' = 0; the diagonal is the constant 0 (utils.py:297-300)
    h[0][0] = dd;
    if (CH == 3) h[1][0] = (i != j) ? 1.f : 0.f;
    const int64_t plane = (int64_t)B * d.n * d.n;
    for (int l = 0; l < 4; ++l) {
        const int in_w = d.eew[l];
        const float* Wm = P + (same ? L.w_same_w[l] : L.w_diff_w[l]);
        const float* bm = P + (same ? L.w_same_b[l] : L.w_diff_b[l]);
        float* o1 = WP + ((int64_t)l * plane + (int64_t)b * d.n * d.n + i * d.n + j) * CH * 32;
        float* o2 = WP + ((int64_t)l * plane + (int64_t)b * d.n * d.n + j * d.n + i) * CH * 32;
        for (int f = 0; f < 32; f += 4) {
            float y[CH][4];
            dense_quad<CH>(h, in_w, Wm, bm, f, y);
            #pragma unroll
            for (int c = 0; c < CH; ++c) {
                const float4 v = make_float4(y[c][0], y[c][1], y[c][2], y[c][3]);
                *reinterpret_cast<float4*>(o1 + c * 32 + f) = v;
                if (i != j) *reinterpret_cast<float4*>(o2 + c * 32 + f) = v;
            }
        }
        if (l < 3) {
            const float* Ws = P + (same ? L.h_same_w[l] : L.h_diff_w[l]);
            const float* bs = P + (same ? L.h_same_b[l] : L.h_diff_b[l]);
            stream_layer<CH>(h, in_w, Ws, bs, l > 0, row);
            if (HP && CH == 1) {      // keep h^(l+1) of this unordered pair for the backward pass
                float* o = HP + ((int64_t)l * B * npair + gid) * 32;
                #pragma unroll
                for (int k = 0; k < 32; k += 4)
                    *reinterpret_cast<float4*>(o + k) = make_float4(h[0][k], h[0][k + 1], h[0][k + 2], h[0][k + 3]);
            }
        }
    }
}

// ------------------------------------------------------------------ value-mode stream MLPs
// Value-only 2-el and el-ion streams as block-level MLP chains: a block takes RB = 64 rows
// (unordered electron pairs of one spin type, or electron-ion entries) and keeps their
// activations in shared memory, feature-major, through all layers; each layer is a
// [64 x in] x [in x 32] product with 4 x 4 register tiles per thread (a 16-byte shared load of
// 4 rows and one of 4 weights per k feeds 16 FMAs), the layer's weights staged in shared
// memory. Same mathematics as k_pair_streams<1> / k_ei_streams<1>.
constexpr int kRB = 64;
struct MlpSmem {
    float H[2][32][kRB + 4];     // activations [buffer][feature][row]
    float W[32 * 32];
    float bias[32];
};

__device__ __forceinline__ void mlp_load_w(MlpSmem& sm, const float* __restrict__ W, const float* __restrict__ b,
                                           int in_w) {
    for (int e = threadIdx.x; e < in_w * 32; e += blockDim.x) sm.W[e] = __ldg(W + e);
    if (threadIdx.x < 32) sm.bias[threadIdx.x] = __ldg(b + threadIdx.x);
}

// z[rr][ff] = bias[f] + sum_k H[k][row] W[k][f], rows 4 rg + rr, features 4 fg + ff
__device__ __forceinline__ void mlp_tile(const MlpSmem& sm, int cur, int in_w, int rg, int fg, float (&z)[4][4]) {
    const float4 b4 = *reinterpret_cast<const float4*>(&sm.bias[4 * fg]);
    #pragma unroll
    for (int rr = 0; rr < 4; ++rr) { z[rr][0] = b4.x; z[rr][1] = b4.y; z[rr][2] = b4.z; z[rr][3] = b4.w; }
    #pragma unroll 8
    for (int k = 0; k < in_w; ++k) {
        const float4 h4 = *reinterpret_cast<const float4*>(&sm.H[cur][k][4 * rg]);
        const float4 w4 = *reinterpret_cast<const float4*>(&sm.W[k * 32 + 4 * fg]);
        const float hv[4] = {h4.x, h4.y, h4.z, h4.w};
        #pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
            z[rr][0] = fmaf(hv[rr], w4.x, z[rr][0]); z[rr][1] = fmaf(hv[rr], w4.y, z[rr][1]);
            z[rr][2] = fmaf(hv[rr], w4.z, z[rr][2]); z[rr][3] = fmaf(hv[rr], w4.w, z[rr][3]);
        }
    }
}

// Blocks [0, blocks_same) take same-spin pairs (up-up then down-down, i <= j), the rest the
// up-down pairs. WP[l][b][i n + j][32] gets both orders; HP (optional) the stream levels 1..3
// at the unordered-pair index used by the backward pass.
__global__ void __launch_bounds__(128)
k_pair_mlp(const float* __restrict__ r, const float* __restrict__ P, ParamLayout L, Dims d, int B, int blocks_same,
           float* __restrict__ WP, float* __restrict__ HP) {
    __shared__ __align__(16) MlpSmem sm;
    __shared__ int rw[kRB], ri[kRB], rj[kRB];
    const int tid = threadIdx.x;
    const int n = d.n, nu = d.nu, nd = d.nd;
    const bool same = (int)blockIdx.x < blocks_same;
    const int cu = nu * (nu + 1) / 2;
    const int npt = same ? cu + nd * (nd + 1) / 2 : nu * nd;
    const int64_t g0 = (int64_t)(same ? blockIdx.x : blockIdx.x - blocks_same) * kRB;
    const int64_t total = (int64_t)B * npt;
    for (int q = tid; q < kRB; q += blockDim.x) {
        const int64_t g = g0 + q;
        int b = -1, i = 0, j = 0;
        if (g < total) {
            b = (int)(g / npt);
            int p = (int)(g % npt);
            if (same) {
                int m = nu, base = 0;
                if (p >= cu) { p -= cu; m = nd; base = nu; }
                int a = 0;
                while (p >= m - a) { p -= m - a; ++a; }
                i = base + a; j = base + a + p;
            } else {
                i = p / nd; j = nu + p % nd;
            }
        }
        rw[q] = b; ri[q] = i; rj[q] = j;
        float dd = 0.f;
        if (b >= 0 && i != j) {
            const float* rb = r + (int64_t)b * n * 3;
            const float dx = rb[j * 3] - rb[i * 3], dy = rb[j * 3 + 1] - rb[i * 3 + 1], dz = rb[j * 3 + 2] - rb[i * 3 + 2];
            dd = sqrtf(dx * dx + dy * dy + dz * dz);
        }
        sm.H[0][0][q] = dd;             // input feature [dist] (utils.py:297-300: 0 on the diagonal)
    }
    const int rg = tid >> 3, fg = tid & 7;
    const int64_t plane = (int64_t)B * n * n;
    const int64_t npair_u = (int64_t)n * (n + 1) / 2;
    const float rs = 0.70710678118654752f;
    int cur = 0;
    for (int l = 0; l < 4; ++l) {
        const int in_w = d.eew[l];
        __syncthreads();
        mlp_load_w(sm, P + (same ? L.w_same_w[l] : L.w_diff_w[l]), P + (same ? L.w_same_b[l] : L.w_diff_b[l]), in_w);
        __syncthreads();
        float z[4][4];
        mlp_tile(sm, cur, in_w, rg, fg, z);
        #pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
            const int q = 4 * rg + rr, b = rw[q];
            if (b < 0) continue;
            const int i = ri[q], j = rj[q];
            const float4 v = make_float4(tanhf(z[rr][0]), tanhf(z[rr][1]), tanhf(z[rr][2]), tanhf(z[rr][3]));
            const int64_t wb = (int64_t)l * plane + (int64_t)b * n * n;
            *reinterpret_cast<float4*>(WP + (wb + i * n + j) * 32 + 4 * fg) = v;
            if (i != j) *reinterpret_cast<float4*>(WP + (wb + j * n + i) * 32 + 4 * fg) = v;
        }
        if (l == 3) break;
        __syncthreads();
        mlp_load_w(sm, P + (same ? L.h_same_w[l] : L.h_diff_w[l]), P + (same ? L.h_same_b[l] : L.h_diff_b[l]), in_w);
        __syncthreads();
        mlp_tile(sm, cur, in_w, rg, fg, z);
        #pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
            const int q = 4 * rg + rr;
            float hn[4];
            #pragma unroll
            for (int ff = 0; ff < 4; ++ff) {
                const int f = 4 * fg + ff;
                const float y = tanhf(z[rr][ff]);
                hn[ff] = l > 0 ? (sm.H[cur][f][q] + y) * rs : y;        // residual (mlp.py:13-17)
                sm.H[cur ^ 1][f][q] = hn[ff];
            }
            const int b = rw[q];
            if (HP && b >= 0) {     // keep h^(l+1) of this unordered pair for the backward pass
                const int i = ri[q], j = rj[q];
                const int64_t pu = (int64_t)i * n - (int64_t)i * (i - 1) / 2 + (j - i);
                *reinterpret_cast<float4*>(HP + (((int64_t)l * B + b) * npair_u + pu) * 32 + 4 * fg) =
                    make_float4(hn[0], hn[1], hn[2], hn[3]);
            }
        }
        cur ^= 1;
    }
}

// Value-only el-ion stream: rows (walker, electron, ion); HE[l][row][32] for levels 0..3
// (level 0 the input [d, dx, dy, dz]); padding ions (Z = 0) give zero rows.
__global__ void __launch_bounds__(128)
k_ei_mlp(const float* __restrict__ r, const float* __restrict__ Rall, const int32_t* __restrict__ Zall,
         const float* __restrict__ P, ParamLayout L, Dims d, int B, float* __restrict__ HE) {
    __shared__ __align__(16) MlpSmem sm;
    __shared__ int rok[kRB];
    const int tid = threadIdx.x;
    const int nei = d.n * d.N;
    const int64_t total = (int64_t)B * nei;
    const int64_t g0 = (int64_t)blockIdx.x * kRB;
    for (int q = tid; q < kRB; q += blockDim.x) {
        const int64_t g = g0 + q;
        float f4[4] = {0.f, 0.f, 0.f, 0.f};
        int ok = 0;
        if (g < total) {
            const int b = (int)(g / nei), p = (int)(g % nei), i = p / d.N, I = p % d.N;
            const int sg = seg_of(d, b);
            if (Zall[(size_t)sg * d.N + I] > 0) {
                const float* R = Rall + (size_t)sg * d.N * 3;
                const float* rr = r + ((int64_t)b * d.n + i) * 3;
                f4[1] = rr[0] - R[I * 3]; f4[2] = rr[1] - R[I * 3 + 1]; f4[3] = rr[2] - R[I * 3 + 2];
                f4[0] = sqrtf(f4[1] * f4[1] + f4[2] * f4[2] + f4[3] * f4[3]);   // [d, dx, dy, dz]
                ok = 1;
            } else {
                ok = 2;                  // padding ion: zero rows at every level
            }
        }
        rok[q] = ok;
        #pragma unroll
        for (int k = 0; k < 4; ++k) sm.H[0][k][q] = f4[k];
    }
    __syncthreads();
    const int rg = tid >> 3, fg = tid & 7;
    // level 0: the input features, zero padded to 32
    for (int e = tid; e < kRB * 8; e += blockDim.x) {
        const int q = e / 8, f0 = (e % 8) * 4;
        if (!rok[q]) continue;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (f0 == 0) v = make_float4(sm.H[0][0][q], sm.H[0][1][q], sm.H[0][2][q], sm.H[0][3][q]);
        *reinterpret_cast<float4*>(HE + (g0 + q) * 32 + f0) = v;
    }
    const float rs = 0.70710678118654752f;
    int cur = 0;
    for (int l = 0; l < 3; ++l) {
        const int in_w = d.eiw[l];
        __syncthreads();
        mlp_load_w(sm, P + L.h_ei_w[l], P + L.h_ei_b[l], in_w);
        __syncthreads();
        float z[4][4];
        mlp_tile(sm, cur, in_w, rg, fg, z);
        #pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
            const int q = 4 * rg + rr;
            float hn[4];
            #pragma unroll
            for (int ff = 0; ff < 4; ++ff) {
                const int f = 4 * fg + ff;
                const float y = tanhf(z[rr][ff]);
                hn[ff] = rok[q] == 2 ? 0.f : (l > 0 ? (sm.H[cur][f][q] + y) * rs : y);
                sm.H[cur ^ 1][f][q] = hn[ff];
            }
            if (rok[q])
                *reinterpret_cast<float4*>(HE + ((int64_t)(l + 1) * total + g0 + q) * 32 + 4 * fg) =
                    make_float4(hn[0], hn[1], hn[2], hn[3]);
        }
        cur ^= 1;
    }
}

// ------------------------------------------------------------------ tangent-mode stream MLPs
// The same block-level chains with Taylor channels: every entry (pair or electron-ion) is CH
// consecutive rows (value, derivatives, Laplacian). The dense part of a layer is one
// [rows x in] x [in x 32] product (bias on value rows only) with 4 x 4 register tiles; the
// pre-activations go through shared memory, where one thread per (entry, feature) applies the
// channel-coupling tanh (tanh_taylor) and the residual. Same mathematics as
// k_pair_streams<3> / k_ei_streams<5>.
struct MlpSmemT {
    float H[2][32][kRB + 4];     // activations [buffer][feature][row]
    float Zs[32][kRB + 4];       // pre-activations of the current layer
    float W[32 * 32];
    float bias[32];
};

// Zs[f][row] = sum_k H[cur][k][row] W[k][f] (+ bias[f] on value rows), 4 x 4 tiles
template <int CH>
__device__ __forceinline__ void mlp_tile_t(MlpSmemT& sm, int cur, int in_w) {
    const int rg = threadIdx.x >> 3, fg = threadIdx.x & 7;
    float z[4][4];
    const float4 b4 = *reinterpret_cast<const float4*>(&sm.bias[4 * fg]);
    #pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
        const bool val = ((4 * rg + rr) % CH) == 0;
        z[rr][0] = val ? b4.x : 0.f; z[rr][1] = val ? b4.y : 0.f; z[rr][2] = val ? b4.z : 0.f; z[rr][3] = val ? b4.w : 0.f;
    }
    #pragma unroll 8
    for (int k = 0; k < in_w; ++k) {
        const float4 h4 = *reinterpret_cast<const float4*>(&sm.H[cur][k][4 * rg]);
        const float4 w4 = *reinterpret_cast<const float4*>(&sm.W[k * 32 + 4 * fg]);
        const float hv[4] = {h4.x, h4.y, h4.z, h4.w};
        #pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
            z[rr][0] = fmaf(hv[rr], w4.x, z[rr][0]); z[rr][1] = fmaf(hv[rr], w4.y, z[rr][1]);
            z[rr][2] = fmaf(hv[rr], w4.z, z[rr][2]); z[rr][3] = fmaf(hv[rr], w4.w, z[rr][3]);
        }
    }
    #pragma unroll
    for (int ff = 0; ff < 4; ++ff)
        *reinterpret_cast<float4*>(&sm.Zs[4 * fg + ff][4 * rg]) = make_float4(z[0][ff], z[1][ff], z[2][ff], z[3][ff]);
}

__device__ __forceinline__ void mlp_load_wt(MlpSmemT& sm, const float* __restrict__ W, const float* __restrict__ b,
                                            int in_w) {
    for (int e = threadIdx.x; e < in_w * 32; e += blockDim.x) sm.W[e] = __ldg(W + e);
    if (threadIdx.x < 32) sm.bias[threadIdx.x] = __ldg(b + threadIdx.x);
}

// 2-el streams with 1-D Taylor channels (f, f', f'' in d_ij): EPB = kRB / 3 unordered pairs
// per block; WP[l][b][i n + j][3][32] for both orders.
__global__ void __launch_bounds__(128)
k_pair_mlp_t(const float* __restrict__ r, const float* __restrict__ P, ParamLayout L, Dims d, int B, int blocks_same,
             float* __restrict__ WP) {
    constexpr int CH = 3, EPB = kRB / CH;
    __shared__ __align__(16) MlpSmemT sm;
    __shared__ int rw[EPB], ri[EPB], rj[EPB];
    const int tid = threadIdx.x;
    const int n = d.n, nu = d.nu, nd = d.nd;
    const bool same = (int)blockIdx.x < blocks_same;
    const int cu = nu * (nu + 1) / 2;
    const int npt = same ? cu + nd * (nd + 1) / 2 : nu * nd;
    const int64_t g0 = (int64_t)(same ? blockIdx.x : blockIdx.x - blocks_same) * EPB;
    const int64_t total = (int64_t)B * npt;
    for (int e = tid; e < 32 * (kRB + 4); e += blockDim.x) sm.H[0][e / (kRB + 4)][e % (kRB + 4)] = 0.f;
    __syncthreads();
    for (int q = tid; q < EPB; q += blockDim.x) {
        const int64_t g = g0 + q;
        int b = -1, i = 0, j = 0;
        if (g < total) {
            b = (int)(g / npt);
            int p = (int)(g % npt);
            if (same) {
                int m = nu, base = 0;
                if (p >= cu) { p -= cu; m = nd; base = nu; }
                int a = 0;
                while (p >= m - a) { p -= m - a; ++a; }
                i = base + a; j = base + a + p;
            } else {
                i = p / nd; j = nu + p % nd;
            }
        }
        rw[q] = b; ri[q] = i; rj[q] = j;
        float dd = 0.f;
        if (b >= 0 && i != j) {
            const float* rb = r + (int64_t)b * n * 3;
            const float dx = rb[j * 3] - rb[i * 3], dy = rb[j * 3 + 1] - rb[i * 3 + 1], dz = rb[j * 3 + 2] - rb[i * 3 + 2];
            dd = sqrtf(dx * dx + dy * dy + dz * dz);
        }
        // input feature [dist]: value d, d' = 1, d'' = 0; the diagonal is the constant 0 (utils.py:297-300)
        sm.H[0][0][q * CH] = dd;
        sm.H[0][0][q * CH + 1] = (b >= 0 && i != j) ? 1.f : 0.f;
        sm.H[0][0][q * CH + 2] = 0.f;
    }
    const int64_t plane = (int64_t)B * n * n;
    const float rs = 0.70710678118654752f;
    int cur = 0;
    for (int l = 0; l < 4; ++l) {
        const int in_w = d.eew[l];
        __syncthreads();
        mlp_load_wt(sm, P + (same ? L.w_same_w[l] : L.w_diff_w[l]), P + (same ? L.w_same_b[l] : L.w_diff_b[l]), in_w);
        __syncthreads();
        mlp_tile_t<CH>(sm, cur, in_w);
        __syncthreads();
        for (int it = tid; it < EPB * 32; it += blockDim.x) {
            const int q = it / 32, f = it % 32, b = rw[q];
            if (b < 0) continue;
            float z[CH], y[CH];
            #pragma unroll
            for (int c = 0; c < CH; ++c) z[c] = sm.Zs[f][q * CH + c];
            tanh_taylor<CH>(z, y);
            const int i = ri[q], j = rj[q];
            const int64_t wb = (int64_t)l * plane + (int64_t)b * n * n;
            #pragma unroll
            for (int c = 0; c < CH; ++c) {
                WP[((wb + i * n + j) * CH + c) * 32 + f] = y[c];
                if (i != j) WP[((wb + j * n + i) * CH + c) * 32 + f] = y[c];
            }
        }
        if (l == 3) break;
        __syncthreads();
        mlp_load_wt(sm, P + (same ? L.h_same_w[l] : L.h_diff_w[l]), P + (same ? L.h_same_b[l] : L.h_diff_b[l]), in_w);
        __syncthreads();
        mlp_tile_t<CH>(sm, cur, in_w);
        __syncthreads();
        // consecutive threads take consecutive pairs (row stride CH): conflict-free shared accesses
        for (int it = tid; it < EPB * 32; it += blockDim.x) {
            const int q = it % EPB, f = it / EPB;
            float z[CH], y[CH];
            #pragma unroll
            for (int c = 0; c < CH; ++c) z[c] = sm.Zs[f][q * CH + c];
            tanh_taylor<CH>(z, y);
            #pragma unroll
            for (int c = 0; c < CH; ++c)
                sm.H[cur ^ 1][f][q * CH + c] = l > 0 ? (sm.H[cur][f][q * CH + c] + y[c]) * rs : y[c];
        }
        cur ^= 1;
    }
}

// El-ion stream with (value, 3 gradients w.r.t. r_i, Laplacian) channels: EPB = kRB / 5 entries
// (walker, electron, ion) per block; HE[l][entry][5][32] for levels 0..3; padding ions give
// zero entries.
__global__ void __launch_bounds__(128)
k_ei_mlp_t(const float* __restrict__ r, const float* __restrict__ Rall, const int32_t* __restrict__ Zall,
           const float* __restrict__ P, ParamLayout L, Dims d, int B, float* __restrict__ HE) {
    constexpr int CH = 5, EPB = kRB / CH;
    __shared__ __align__(16) MlpSmemT sm;
    __shared__ int rok[EPB];
    const int tid = threadIdx.x;
    const int nei = d.n * d.N;
    const int64_t total = (int64_t)B * nei;
    const int64_t g0 = (int64_t)blockIdx.x * EPB;
    for (int e = tid; e < 32 * (kRB + 4); e += blockDim.x) sm.H[0][e / (kRB + 4)][e % (kRB + 4)] = 0.f;
    __syncthreads();
    for (int q = tid; q < EPB; q += blockDim.x) {
        const int64_t g = g0 + q;
        int ok = 0;
        if (g < total) {
            const int b = (int)(g / nei), p = (int)(g % nei), i = p / d.N, I = p % d.N;
            const int sg = seg_of(d, b);
            if (Zall[(size_t)sg * d.N + I] > 0) {
                const float* R = Rall + (size_t)sg * d.N * 3;
                const float* rr = r + ((int64_t)b * d.n + i) * 3;
                const float sx = rr[0] - R[I * 3], sy = rr[1] - R[I * 3 + 1], sz = rr[2] - R[I * 3 + 2];
                const float dd = sqrtf(sx * sx + sy * sy + sz * sz);
                const float sv[3] = {sx, sy, sz};
                // [d, sx, sy, sz] (input_features.py:56-66), its gradients and Laplacian in r_i
                sm.H[0][0][q * CH] = dd;
                #pragma unroll
                for (int c = 0; c < 3; ++c) {
                    sm.H[0][1 + c][q * CH] = sv[c];
                    sm.H[0][0][q * CH + 1 + c] = sv[c] / dd;
                    sm.H[0][1 + c][q * CH + 1 + c] = 1.f;
                }
                sm.H[0][0][q * CH + 4] = 2.f / dd;
                ok = 1;
            } else {
                ok = 2;                  // padding ion
            }
        }
        rok[q] = ok;
    }
    __syncthreads();
    // level 0: the input features, zero padded to 32
    for (int it = tid; it < EPB * CH * 32; it += blockDim.x) {
        const int q = it / (CH * 32), rc = it % (CH * 32), c = rc / 32, f = rc % 32;
        if (!rok[q]) continue;
        HE[((g0 + q) * CH + c) * 32 + f] = rok[q] == 2 ? 0.f : sm.H[0][f][q * CH + c];
    }
    const float rs = 0.70710678118654752f;
    int cur = 0;
    for (int l = 0; l < 3; ++l) {
        const int in_w = d.eiw[l];
        __syncthreads();
        mlp_load_wt(sm, P + L.h_ei_w[l], P + L.h_ei_b[l], in_w);
        __syncthreads();
        mlp_tile_t<CH>(sm, cur, in_w);
        __syncthreads();
        for (int it = tid; it < EPB * 32; it += blockDim.x) {
            const int q = it / 32, f = it % 32;
            float z[CH], y[CH];
            #pragma unroll
            for (int c = 0; c < CH; ++c) z[c] = sm.Zs[f][q * CH + c];
            tanh_taylor<CH>(z, y);
            #pragma unroll
            for (int c = 0; c < CH; ++c) {
                const float hn = rok[q] == 2 ? 0.f : (l > 0 ? (sm.H[cur][f][q * CH + c] + y[c]) * rs : y[c]);
                sm.H[cur ^ 1][f][q * CH + c] = hn;
                if (rok[q]) HE[((int64_t)(l + 1) * total * CH + (g0 + q) * CH + c) * 32 + f] = hn;
            }
        }
        cur ^= 1;
    }
}

// El-ion stream fused with its SchNet reduction (forward passes): the block holds the
// electron-ion rows of EPB whole electrons (N ions x CH channels each) and, at every stream level
// l = 0..3, writes conv_ei[l][electron][c][f] = sum_I h_l[electron, I][c][f] * ion_map_l[I][f]
// (ferminet_embedding.py:171-175) instead of the stream itself, N times fewer values. The
// stream layers are those of k_ei_mlp (CH = 1) and k_ei_mlp_t (CH = 5); padding ions (Z = 0)
// have zero rows at every level. Requires N CH <= kRB.
template <int CH>
__global__ void __launch_bounds__(128)
k_ei_conv(const float* __restrict__ r, const float* __restrict__ Rall, const int32_t* __restrict__ Zall,
          const float* __restrict__ P, ParamLayout L, Dims d, int B, const float* __restrict__ him,
          float* __restrict__ CEI) {
    __shared__ __align__(16) MlpSmemT sm;
    __shared__ unsigned char rok[kRB];     // per entry (electron, ion): 1 real ion, 2 padding ion
    const int N = d.N, EPB = kRB / (N * CH);
    const int tid = threadIdx.x;
    const int64_t ne = (int64_t)B * d.n;
    const int64_t e0 = (int64_t)blockIdx.x * EPB;
    for (int e = tid; e < 32 * (kRB + 4); e += blockDim.x) sm.H[0][e / (kRB + 4)][e % (kRB + 4)] = 0.f;
    __syncthreads();
    for (int q = tid; q < EPB * N; q += blockDim.x) {
        const int el = q / N, I = q % N;
        const int64_t e = e0 + el;
        unsigned char ok = 0;
        if (e < ne) {
            const int b = (int)(e / d.n);
            const int sg = seg_of(d, b);
            if (Zall[(size_t)sg * N + I] > 0) {
                const float* R = Rall + (size_t)sg * N * 3;
                const float* rr = r + e * 3;
                const float sx = rr[0] - R[I * 3], sy = rr[1] - R[I * 3 + 1], sz = rr[2] - R[I * 3 + 2];
                const float dd = sqrtf(sx * sx + sy * sy + sz * sz);
                const float sv[3] = {sx, sy, sz};
                const int row = q * CH;
                // [d, sx, sy, sz] (input_features.py:56-66), with CH = 5 its gradients and Laplacian in r_i
                sm.H[0][0][row] = dd;
                #pragma unroll
                for (int c = 0; c < 3; ++c) {
                    sm.H[0][1 + c][row] = sv[c];
                    if (CH == 5) {
                        sm.H[0][0][row + 1 + c] = sv[c] / dd;
                        sm.H[0][1 + c][row + 1 + c] = 1.f;
                    }
                }
                if (CH == 5) sm.H[0][0][row + 4] = 2.f / dd;
                ok = 1;
            } else {
                ok = 2;
            }
        }
        rok[q] = ok;
    }
    __syncthreads();
    auto write_cei = [&](int level, int buf) {
        for (int it = tid; it < EPB * CH * 32; it += blockDim.x) {
            const int el = it / (CH * 32), c = (it / 32) % CH, f = it % 32;
            const int64_t e = e0 + el;
            if (e >= ne) continue;
            const int sg = seg_of(d, (int)(e / d.n));
            const float* hs = him + ((size_t)sg * 4 + level) * N * 32 + f;
            float v = 0.f;
            for (int I = 0; I < N; ++I) v = fmaf(sm.H[buf][f][(el * N + I) * CH + c], __ldg(hs + I * 32), v);
            CEI[(((int64_t)level * ne + e) * CH + c) * 32 + f] = v;
        }
    };
    write_cei(0, 0);
    const float rs = 0.70710678118654752f;
    int cur = 0;
    for (int l = 0; l < 3; ++l) {
        const int in_w = d.eiw[l];
        __syncthreads();
        mlp_load_wt(sm, P + L.h_ei_w[l], P + L.h_ei_b[l], in_w);
        __syncthreads();
        mlp_tile_t<CH>(sm, cur, in_w);
        __syncthreads();
        // consecutive threads take consecutive entries (row stride CH): conflict-free shared accesses
        for (int it = tid; it < EPB * N * 32; it += blockDim.x) {
            const int q = it % (EPB * N), f = it / (EPB * N);
            float z[CH], y[CH];
            #pragma unroll
            for (int c = 0; c < CH; ++c) z[c] = sm.Zs[f][q * CH + c];
            tanh_taylor<CH>(z, y);
            #pragma unroll
            for (int c = 0; c < CH; ++c)
                sm.H[cur ^ 1][f][q * CH + c] =
                    rok[q] == 1 ? (l > 0 ? (sm.H[cur][f][q * CH + c] + y[c]) * rs : y[c]) : 0.f;
        }
        cur ^= 1;
        __syncthreads();
        write_cei(l + 1, cur);
    }
}

template <int CH>
__global__ void __launch_bounds__(128)
k_ei_streams(const float* __restrict__ r, const float* __restrict__ R, const int32_t* __restrict__ Z,
             const float* __restrict__ P, ParamLayout L, Dims d, int B, float* __restrict__ HE) {
    extern __shared__ float srow[];
    float* row = srow + threadIdx.x * (CH * 32 + 1);
    const int nei = d.n * d.N;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (int64_t)B * nei) return;
    const int b = (int)(gid / nei), p = (int)(gid % nei);
    const int i = p / d.N, I = p % d.N;
    const float* ri = r + ((int64_t)b * d.n + i) * 3;
    const int sg = seg_of(d, b);
    R += (size_t)sg * d.N * 3;
    const int64_t plane = (int64_t)B * nei;
    if (Z[sg * d.N + I] <= 0) {       // padding ion: zero stream (its ion map is zero as well)
        for (int l = 0; l < 4; ++l) {
            float4* o = reinterpret_cast<float4*>(HE + ((int64_t)l * plane + (int64_t)b * nei + p) * CH * 32);
            for (int k = 0; k < CH * 8; ++k) o[k] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
        return;
    }
    const float s[3] = {ri[0] - R[I * 3], ri[1] - R[I * 3 + 1], ri[2] - R[I * 3 + 2]};
    const float dd = sqrtf(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
    float h[CH][32];
    #pragma unroll
    for (int c = 0; c < CH; ++c)
        #pragma unroll
        for (int k = 0; k < 32; ++k) h[c][k] = 0.f;
    // [d, sx, sy, sz] (input_features.py:56-66)
    h[0][0] = dd; h[0][1] = s[0]; h[0][2] = s[1]; h[0][3] = s[2];
    if (CH == 5) {
        #pragma unroll
        for (int c = 0; c < 3; ++c) { h[1 + c][0] = s[c] / dd; h[1 + c][1 + c] = 1.f; }
        h[4][0] = 2.f / dd;
    }
    for (int l = 0; l < 4; ++l) {
        float* o = HE + ((int64_t)l * plane + (int64_t)b * nei + p) * CH * 32;
        #pragma unroll
        for (int c = 0; c < CH; ++c)
            #pragma unroll
            for (int k = 0; k < 32; k += 4)
                *reinterpret_cast<float4*>(o + c * 32 + k) = make_float4(h[c][k], h[c][k + 1], h[c][k + 2], h[c][k + 3]);
        if (l == 3) break;
        stream_layer<CH>(h, d.eiw[l], P + L.h_ei_w[l], P + L.h_ei_b[l], l > 0, row);
    }
}

// ------------------------------------------------------------------ spin means of h_one
// M[(b*Tp + t), 0:hw] = mean over up electrons, [hw:2hw] = mean over down electrons
// (SymmetricFeatures, ferminet_embedding.py:60-72). Row width mw (>= 2hw, zero padded).
// Split-BF16 variant, 8 columns per thread with 16-byte hi / lo loads (hw % 8 == 0).
__global__ void k_spin_means_split8(const Split* __restrict__ X, int ldx, int hw, Dims d, Split* __restrict__ M, int mw) {
    const int b = blockIdx.x;
    const int m8 = mw / 8;
    for (int idx = threadIdx.x; idx < d.Tp * m8; idx += blockDim.x) {
        const int t = idx / m8, col = (idx % m8) * 8;
        float v[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        if (col < 2 * hw) {
            const int f = col % hw;
            const int i0 = col < hw ? 0 : d.nu, i1 = col < hw ? d.nu : d.n;
            for (int i = i0; i < i1; ++i) {
                const int64_t row = (int64_t)(b * d.n + i) * d.Tp + t;
                const uint4 h = *reinterpret_cast<const uint4*>(X + row * 2 * ldx + f);
                const uint4 l = *reinterpret_cast<const uint4*>(X + row * 2 * ldx + ldx + f);
                const uint32_t hh[4] = {h.x, h.y, h.z, h.w}, ll[4] = {l.x, l.y, l.z, l.w};
                #pragma unroll
                for (int k = 0; k < 4; ++k) {
                    v[2 * k] += __uint_as_float(hh[k] << 16) + __uint_as_float(ll[k] << 16);
                    v[2 * k + 1] += __uint_as_float(hh[k] & 0xffff0000u) + __uint_as_float(ll[k] & 0xffff0000u);
                }
            }
            const float inv = 1.f / (float)(i1 - i0);
            #pragma unroll
            for (int k = 0; k < 8; ++k) v[k] *= inv;
        }
        const int64_t orow = (int64_t)b * d.Tp + t;
        uint32_t hh[4], ll[4];
        #pragma unroll
        for (int k = 0; k < 4; ++k) {
            __nv_bfloat16 h0 = __float2bfloat16_rn(v[2 * k]), h1 = __float2bfloat16_rn(v[2 * k + 1]);
            __nv_bfloat16 l0 = __float2bfloat16_rn(v[2 * k] - __bfloat162float(h0));
            __nv_bfloat16 l1 = __float2bfloat16_rn(v[2 * k + 1] - __bfloat162float(h1));
            hh[k] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
            ll[k] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
        }
        *reinterpret_cast<uint4*>(M + orow * 2 * mw + col) = make_uint4(hh[0], hh[1], hh[2], hh[3]);
        *reinterpret_cast<uint4*>(M + orow * 2 * mw + mw + col) = make_uint4(ll[0], ll[1], ll[2], ll[3]);
    }
}

template <class Act>
__global__ void k_spin_means(const Act* __restrict__ X, int ldx, int hw, Dims d, Act* __restrict__ M, int mw) {
    int b = blockIdx.x;
    for (int idx = threadIdx.x; idx < d.Tp * mw; idx += blockDim.x) {
        int t = idx / mw, col = idx % mw;
        float v = 0.f;
        if (col < 2 * hw) {
            int f = col % hw;
            int i0 = col < hw ? 0 : d.nu, i1 = col < hw ? d.nu : d.n;
            for (int i = i0; i < i1; ++i) v += ActIO<Act>::load(X, (int64_t)(b * d.n + i) * d.Tp + t, ldx, f);
            v /= (float)(i1 - i0);
        }
        ActIO<Act>::store(M, (int64_t)b * d.Tp + t, mw, col, v);
    }
}

// ------------------------------------------------------------------ tanh with forward Laplacian
// y = tanh(z): y_t = (1 - y^2) z_t, y_lap = (1 - y^2) z_lap - 2 y (1 - y^2) sum_t z_t^2.
template <class Act>
__global__ void k_tanh_fl(const float* __restrict__ Zb, int ldz, int ncols, int nrow_groups, Dims d,
                          Act* __restrict__ Y, int ldy) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nrow_groups * ncols) return;
    int64_t g = idx / ncols;
    int f = idx % ncols;
    const float* z = Zb + g * d.Tp * ldz + f;
    const int64_t r0 = g * d.Tp;
    float z0 = z[0];
    float y0 = tanhf(z0), d1 = 1.f - y0 * y0;
    ActIO<Act>::store(Y, r0, ldy, f, y0);
    if (d.Tp == 1) return;
    float s = 0.f;
    for (int t = 1; t <= 3 * d.n; ++t) {
        float zt = z[(int64_t)t * ldz];
        s += zt * zt;
        ActIO<Act>::store(Y, r0 + t, ldy, f, d1 * zt);
    }
    ActIO<Act>::store(Y, r0 + d.lap, ldy, f, d1 * z[(int64_t)d.lap * ldz] - 2.f * y0 * d1 * s);
    for (int t = d.lap + 1; t < d.Tp; ++t) ActIO<Act>::store(Y, r0 + t, ldy, f, 0.f);
}

// ------------------------------------------------------------------ SchNet convolutions
// conv_ee[i] = sum_j w_ij * hm_j (same/diff spin blocks incl. the self pair,
// ferminet_embedding.py:152-169) and conv_ei[i] = sum_I h_ei[i,I] * him[I] (:171-175),
// with product-rule tangents and Laplacian. Written into columns [hw, hw+E+eiw) of X_l.
template <class Act>
__global__ void k_conv(const float* __restrict__ r, const float* __restrict__ WPl, const float* __restrict__ HM,
                       const float* __restrict__ HEl, const float* __restrict__ himl, Dims d, int l, int B,
                       Act* __restrict__ X, int ldx) {
    int bi = blockIdx.x;
    int b = bi / d.n, i = bi % d.n;
    int hw = d.hw[l], E = d.E, eiw = d.eiw[l];
    int ncol = E + eiw;
    int pch = d.Tp > 1 ? 3 : 1, ech = d.Tp > 1 ? 5 : 1;
    const float* rb = r + (int64_t)b * d.n * 3;
    const float* wrow = WPl + ((int64_t)b * d.n * d.n + (int64_t)i * d.n) * pch * 32;   // w_i,: records
    const float* hmb = HM + (int64_t)b * d.n * d.Tp * 32;
    for (int idx = threadIdx.x; idx < d.Tp * ncol; idx += blockDim.x) {
        int t = idx / ncol, col = idx % ncol;
        float v = 0.f;
        if (t < d.T) {
            if (col < E) {
                int f = col;
                for (int j = 0; j < d.n; ++j) v += wrow[j * pch * 32 + f] * hmb[((int64_t)j * d.Tp + t) * 32 + f];
                if (t >= 1 && t <= 3 * d.n) {
                    int m = (t - 1) / 3, c = (t - 1) % 3;
                    if (m == i) {
                        for (int j = 0; j < d.n; ++j) {
                            if (j == i) continue;
                            float u = rb[j * 3 + c] - rb[i * 3 + c];
                            float dx = rb[j * 3] - rb[i * 3], dy = rb[j * 3 + 1] - rb[i * 3 + 1], dz = rb[j * 3 + 2] - rb[i * 3 + 2];
                            float dist = sqrtf(dx * dx + dy * dy + dz * dz);
                            v -= wrow[j * pch * 32 + 32 + f] * (u / dist) * hmb[(int64_t)j * d.Tp * 32 + f];
                        }
                    } else {
                        float u = rb[m * 3 + c] - rb[i * 3 + c];
                        float dx = rb[m * 3] - rb[i * 3], dy = rb[m * 3 + 1] - rb[i * 3 + 1], dz = rb[m * 3 + 2] - rb[i * 3 + 2];
                        float dist = sqrtf(dx * dx + dy * dy + dz * dz);
                        v += wrow[m * pch * 32 + 32 + f] * (u / dist) * hmb[(int64_t)m * d.Tp * 32 + f];
                    }
                } else if (t == d.lap) {
                    for (int j = 0; j < d.n; ++j) {
                        if (j == i) continue;
                        float dx = rb[j * 3] - rb[i * 3], dy = rb[j * 3 + 1] - rb[i * 3 + 1], dz = rb[j * 3 + 2] - rb[i * 3 + 2];
                        float dist = sqrtf(dx * dx + dy * dy + dz * dz);
                        float inv = 1.f / dist;
                        float w1 = wrow[j * pch * 32 + 32 + f], w2 = wrow[j * pch * 32 + 64 + f];
                        const float* hj = hmb + (int64_t)j * d.Tp * 32 + f;
                        float cross = 0.f;
                        float uu[3] = {dx * inv, dy * inv, dz * inv};
                        #pragma unroll
                        for (int c = 0; c < 3; ++c)
                            cross += uu[c] * (hj[(1 + 3 * j + c) * 32] - hj[(1 + 3 * i + c) * 32]);
                        v += 2.f * (w2 + 2.f * w1 * inv) * hj[0] + 2.f * w1 * cross;
                    }
                }
            } else {
                int f = col - E;
                int ch = -1;
                if (t == 0) ch = 0;
                else if (t == d.lap) ch = 4;
                else if (t >= 1 + 3 * i && t < 4 + 3 * i) ch = t - 3 * i;
                if (ch >= 0) {
                    const float* he = HEl + ((int64_t)b * d.n * d.N + (int64_t)i * d.N) * ech * 32;
                    const float* hs = himl + (size_t)seg_of(d, b) * 4 * d.N * 32;
                    for (int I = 0; I < d.N; ++I) v += he[(I * ech + ch) * 32 + f] * hs[I * 32 + f];
                }
            }
        }
        ActIO<Act>::store(X, (int64_t)bi * d.Tp + t, ldx, hw + col, v);
    }
}

// Register-tiled tangent convolution. Block = (walker, tile of TI = 4 electrons i) with
// NW = Tp / TT warps; lane = feature f, warp w owns channels [w TT, w TT + TT). The main loop
// loads w_ij (4 rows) and h_j (TT channels) once per j and issues 4 TT FMAs. The results are
// staged in shared memory, where the product-rule terms are added with per-(i, j) items spread
// over the warps: single terms w'_im u_im h_m for the channels of the other electrons m, the
// j-sums of the electron's own gradient channels and of the Laplacian. Columns are then written
// eight at a time (16-byte stores). conv_ei is non-zero on 5 channels per electron only. Same
// mathematics as k_conv.
template <class Act, int TT, int TI>
__global__ void __launch_bounds__(512)
k_conv_tile(const float* __restrict__ r, const float* __restrict__ WPl, const float* __restrict__ HM,
            const float* __restrict__ HEl, const float* __restrict__ himl, Dims d, int l, int B, Act* __restrict__ X,
            int ldx, int ei_fused) {
    extern __shared__ __align__(16) float smc[];
    const int n = d.n, Tp = d.Tp, T = d.T;
    const int NW = Tp / TT;
    float* out = smc;                                   // [TI][Tp][32] conv_ee
    float* red = out + TI * Tp * 32;                    // [NW][TI][4][32] own-gradient / Laplacian partials
    float* eiv = red + NW * TI * 4 * 32;                // [TI][5][32] conv_ei channels
    const int f = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ntile = (n + TI - 1) / TI;
    const int b = blockIdx.x / ntile, i0 = (blockIdx.x % ntile) * TI;
    const int ni = min(TI, n - i0);
    const int hw = d.hw[l], E = d.E, eiw = d.eiw[l];
    const int t0 = w * TT;
    const float* rb = r + (size_t)b * n * 3;
    const float* wpb = WPl + (size_t)b * n * n * 96 + f;           // records [i * n + j][3][32]
    const float* hmb = HM + (size_t)b * n * Tp * 32 + f;           // [j][Tp][32]
    {
        float acc[TI][TT];
        #pragma unroll
        for (int ii = 0; ii < TI; ++ii)
            #pragma unroll
            for (int k = 0; k < TT; ++k) acc[ii][k] = 0.f;
        const int i_last = i0 + ni - 1;
        for (int j = 0; j < n; ++j) {
            const float* hj = hmb + (size_t)j * Tp * 32;
            float h[TT];
            #pragma unroll
            for (int k = 0; k < TT; ++k) h[k] = (t0 + k < T) ? __ldg(hj + (t0 + k) * 32) : 0.f;
            #pragma unroll
            for (int ii = 0; ii < TI; ++ii) {
                const int i = min(i0 + ii, i_last);           // rows past the tile repeat the last one
                const float w0 = __ldg(wpb + ((size_t)i * n + j) * 96);
                #pragma unroll
                for (int k = 0; k < TT; ++k) acc[ii][k] = fmaf(w0, h[k], acc[ii][k]);
            }
        }
        #pragma unroll
        for (int ii = 0; ii < TI; ++ii)
            #pragma unroll
            for (int k = 0; k < TT; ++k) out[(ii * Tp + t0 + k) * 32 + f] = acc[ii][k];
    }
    // product-rule partials of the own-gradient channels and the Laplacian, j split over warps
    for (int ii = 0; ii < ni; ++ii) {
        const int i = i0 + ii;
        const float rx = rb[i * 3], ry = rb[i * 3 + 1], rz = rb[i * 3 + 2];
        float o0 = 0.f, o1 = 0.f, o2 = 0.f, ol = 0.f;
        for (int j = w; j < n; j += NW) {
            if (j == i) continue;
            const float* wr = wpb + ((size_t)i * n + j) * 96;
            const float* hj = hmb + (size_t)j * Tp * 32;
            const float w1 = __ldg(wr + 32), w2 = __ldg(wr + 64), h0 = __ldg(hj);
            const float dx = rb[j * 3] - rx, dy = rb[j * 3 + 1] - ry, dz = rb[j * 3 + 2] - rz;
            const float inv = 1.f / sqrtf(dx * dx + dy * dy + dz * dz);
            const float ux = dx * inv, uy = dy * inv, uz = dz * inv;
            o0 += w1 * ux * h0; o1 += w1 * uy * h0; o2 += w1 * uz * h0;
            const float cross = ux * (__ldg(hj + (1 + 3 * j) * 32) - __ldg(hj + (1 + 3 * i) * 32)) +
                                uy * (__ldg(hj + (2 + 3 * j) * 32) - __ldg(hj + (2 + 3 * i) * 32)) +
                                uz * (__ldg(hj + (3 + 3 * j) * 32) - __ldg(hj + (3 + 3 * i) * 32));
            ol += 2.f * (w2 + 2.f * w1 * inv) * h0 + 2.f * w1 * cross;
        }
        float* rr = red + ((w * TI + ii) * 4) * 32 + f;
        rr[0] = o0; rr[32] = o1; rr[64] = o2; rr[96] = ol;
    }
    // conv_ei on its 5 non-zero channels: items (ii, ch) over the warps
    const float* hs = himl + (size_t)seg_of(d, b) * 4 * d.N * 32 + f;
    for (int it = w; it < ni * 5; it += NW) {
        const int ii = it / 5, ch = it % 5;
        float v = 0.f;
        if (ei_fused) {
            // already reduced over the ions by the el-ion stream kernel: CEI[electron][5][32]
            v = __ldg(HEl + (((size_t)b * n + i0 + ii) * 5 + ch) * 32 + f);
        } else {
            const float* he = HEl + ((size_t)b * n * d.N + (size_t)(i0 + ii) * d.N) * 5 * 32 + ch * 32 + f;
            if (f < eiw)
                for (int I = 0; I < d.N; ++I) v += __ldg(he + I * 5 * 32) * __ldg(hs + I * 32);
        }
        eiv[(ii * 5 + ch) * 32 + f] = v;
    }
    __syncthreads();
    // single product-rule terms: channel 1 + 3m + c of electron i gains w'_im u_im,c h_m,0 (m != i)
    for (int it = w; it < ni * n; it += NW) {
        const int ii = it / n, m = it % n, i = i0 + ii;
        float* o = out + (ii * Tp) * 32 + f;
        if (m == i) {
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, sl = 0.f;
            for (int q = 0; q < NW; ++q) {
                const float* rr = red + ((q * TI + ii) * 4) * 32 + f;
                s0 += rr[0]; s1 += rr[32]; s2 += rr[64]; sl += rr[96];
            }
            o[(1 + 3 * i) * 32] -= s0; o[(2 + 3 * i) * 32] -= s1; o[(3 + 3 * i) * 32] -= s2;
            o[d.lap * 32] += sl;
        } else {
            const float dx = rb[m * 3] - rb[i * 3], dy = rb[m * 3 + 1] - rb[i * 3 + 1], dz = rb[m * 3 + 2] - rb[i * 3 + 2];
            const float inv = 1.f / sqrtf(dx * dx + dy * dy + dz * dz);
            const float g = __ldg(wpb + ((size_t)i * n + m) * 96 + 32) * __ldg(hmb + (size_t)m * Tp * 32) * inv;
            o[(1 + 3 * m) * 32] += g * dx; o[(2 + 3 * m) * 32] += g * dy; o[(3 + 3 * m) * 32] += g * dz;
        }
    }
    __syncthreads();
    // stores: row (ii, t), units of 8 columns: 4 units of conv_ee, then conv_ei
    const int ei_units = (eiw + 7) / 8;
    const int units = 4 + ei_units;
    const bool rowvec = (hw % 8) == 0 && (ldx % 8) == 0;      // 16-byte aligned column groups
    for (int it = threadIdx.x; it < ni * Tp * units; it += blockDim.x) {
        const int u = it % units, rt = it / units, t = rt % Tp, ii = rt / Tp, i = i0 + ii;
        const int64_t row = ((int64_t)b * n + i) * Tp + t;
        float v[8];
        int col;
        if (u < 4) {
            const float* src = out + (ii * Tp + t) * 32 + 8 * u;
            #pragma unroll
            for (int k = 0; k < 8; ++k) v[k] = t < T ? src[k] : 0.f;
            col = hw + 8 * u;
        } else {
            int ch = -1;
            if (t == 0) ch = 0;
            else if (t == d.lap) ch = 4;
            else if (t >= 1 + 3 * i && t < 4 + 3 * i) ch = t - 3 * i;
            const float* src = eiv + (ii * 5 + (ch < 0 ? 0 : ch)) * 32 + 8 * (u - 4);
            #pragma unroll
            for (int k = 0; k < 8; ++k) v[k] = ch >= 0 ? src[k] : 0.f;
            col = hw + E + 8 * (u - 4);
        }
        if (rowvec && (u < 4 || eiw - 8 * (u - 4) >= 8)) {
            ActIO<Act>::store8(X, row, ldx, col, v);
        } else {
            const int lim = u < 4 ? 8 : min(8, eiw - 8 * (u - 4));
            #pragma unroll
            for (int k = 0; k < 8; ++k)
                if (k < lim) ActIO<Act>::store(X, row, ldx, col + k, v[k]);
        }
    }
}

// Value rows (Tp = 1): thread per (walker, electron, 8-column octet) of the conv_ee / conv_ei
// block of the layer input. Each thread accumulates its 8 columns over the n pair records (or
// the N ion records) with 16-byte loads of w_ij / h_ei and of h_map_j / the ion map (the latter
// shared by all electrons of a walker, served from L1); no shared-memory staging or barriers.
// Same mathematics as k_conv_walker on value rows.
template <class Act>
__global__ void __launch_bounds__(256)
k_conv_value(const float* __restrict__ WPl, const float* __restrict__ HM, const float* __restrict__ HEl,
             const float* __restrict__ himl, Dims d, int l, int B, Act* __restrict__ X, int ldx) {
    const int n = d.n, N = d.N, E = d.E, eiw = d.eiw[l], hw = d.hw[l];
    const int oe = E / 8, oi = (eiw + 7) / 8, octs = oe + oi;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (int64_t)B * n * octs) return;
    const int oct = (int)(gid % octs);
    const int64_t bi = gid / octs;                 // walker * n + electron
    const int b = (int)(bi / n), i = (int)(bi % n);
    float acc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int col, ncol;
    if (oct < oe) {
        const int f0 = 8 * oct;
        const float* w = WPl + ((int64_t)b * n * n + (int64_t)i * n) * 32 + f0;
        const float* h = HM + (int64_t)b * n * 32 + f0;
        #pragma unroll 4
        for (int j = 0; j < n; ++j) {
            const float4 w0 = __ldg(reinterpret_cast<const float4*>(w + j * 32));
            const float4 w1 = __ldg(reinterpret_cast<const float4*>(w + j * 32 + 4));
            const float4 h0 = __ldg(reinterpret_cast<const float4*>(h + j * 32));
            const float4 h1 = __ldg(reinterpret_cast<const float4*>(h + j * 32 + 4));
            acc[0] = fmaf(w0.x, h0.x, acc[0]); acc[1] = fmaf(w0.y, h0.y, acc[1]);
            acc[2] = fmaf(w0.z, h0.z, acc[2]); acc[3] = fmaf(w0.w, h0.w, acc[3]);
            acc[4] = fmaf(w1.x, h1.x, acc[4]); acc[5] = fmaf(w1.y, h1.y, acc[5]);
            acc[6] = fmaf(w1.z, h1.z, acc[6]); acc[7] = fmaf(w1.w, h1.w, acc[7]);
        }
        col = hw + f0;
        ncol = 8;
    } else {
        const int f0 = 8 * (oct - oe);
        const float* he = HEl + ((int64_t)b * n * N + (int64_t)i * N) * 32 + f0;
        const float* hs = himl + (size_t)seg_of(d, b) * 4 * N * 32 + f0;
        #pragma unroll 4
        for (int I = 0; I < N; ++I) {
            const float4 e0 = __ldg(reinterpret_cast<const float4*>(he + I * 32));
            const float4 e1 = __ldg(reinterpret_cast<const float4*>(he + I * 32 + 4));
            const float4 s0 = __ldg(reinterpret_cast<const float4*>(hs + I * 32));
            const float4 s1 = __ldg(reinterpret_cast<const float4*>(hs + I * 32 + 4));
            acc[0] = fmaf(e0.x, s0.x, acc[0]); acc[1] = fmaf(e0.y, s0.y, acc[1]);
            acc[2] = fmaf(e0.z, s0.z, acc[2]); acc[3] = fmaf(e0.w, s0.w, acc[3]);
            acc[4] = fmaf(e1.x, s1.x, acc[4]); acc[5] = fmaf(e1.y, s1.y, acc[5]);
            acc[6] = fmaf(e1.z, s1.z, acc[6]); acc[7] = fmaf(e1.w, s1.w, acc[7]);
        }
        col = hw + E + f0;
        ncol = min(8, eiw - f0);
    }
    if (ncol == 8 && (col % 8) == 0 && (ldx % 8) == 0) {
        ActIO<Act>::store8(X, bi, ldx, col, acc);
    } else {
        #pragma unroll
        for (int k = 0; k < 8; ++k)
            if (k < ncol) ActIO<Act>::store(X, bi, ldx, col + k, acc[k]);
    }
}

// Block per walker: the walker's h_map tangents (n x Tp x 32) and pair geometry are staged in
// shared memory once, then every (electron, channel, column) output of conv_ee / conv_ei is
// formed from shared memory. Same mathematics as k_conv.
template <class Act>
__global__ void __launch_bounds__(256)
k_conv_walker(const float* __restrict__ r, const float* __restrict__ WPl, const float* __restrict__ HM,
              const float* __restrict__ HEl, const float* __restrict__ himl, Dims d, int l, int B,
              Act* __restrict__ X, int ldx) {
    extern __shared__ float smc[];
    const int b = blockIdx.x;
    const int n = d.n, Tp = d.Tp, T = d.T;
    const int hw = d.hw[l], E = d.E, eiw = d.eiw[l];
    const int ncol = E + eiw;
    const int pch = Tp > 1 ? 3 : 1, ech = Tp > 1 ? 5 : 1;
    float* hm = smc;                                   // [n][Tp][32]
    float* geo = hm + (size_t)n * Tp * 32;             // [n][n][4]: u_x, u_y, u_z, 1/d (0 on the diagonal)
    const float* hmb = HM + (size_t)b * n * Tp * 32;
    for (int e = threadIdx.x; e < n * Tp * 8; e += blockDim.x)
        reinterpret_cast<float4*>(hm)[e] = __ldg(reinterpret_cast<const float4*>(hmb) + e);
    const float* rb = r + (size_t)b * n * 3;
    for (int e = threadIdx.x; e < (Tp > 1 ? n * n : 0); e += blockDim.x) {   // pair geometry: tangent rows only
        const int i = e / n, j = e % n;
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i != j) {
            const float dx = rb[j * 3] - rb[i * 3], dy = rb[j * 3 + 1] - rb[i * 3 + 1], dz = rb[j * 3 + 2] - rb[i * 3 + 2];
            const float inv = 1.f / sqrtf(dx * dx + dy * dy + dz * dz);
            g = make_float4(dx * inv, dy * inv, dz * inv, inv);
        }
        reinterpret_cast<float4*>(geo)[e] = g;
    }
    __syncthreads();
    const float* wpb = WPl + (size_t)b * n * n * pch * 32;
    const float* heb = HEl + (size_t)b * n * d.N * ech * 32;
    const int items = n * Tp * ncol;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int col = it % ncol, t = (it / ncol) % Tp, i = it / (ncol * Tp);
        float v = 0.f;
        if (t < T) {
            if (col < E) {
                const int f = col;
                const float* wrow = wpb + (size_t)i * n * pch * 32 + f;      // record (i, j) at j * pch * 32
                #pragma unroll 4
                for (int j = 0; j < n; ++j) v += __ldg(wrow + j * pch * 32) * hm[(j * Tp + t) * 32 + f];
                if (t >= 1 && t <= 3 * n) {
                    const int m = (t - 1) / 3, c = (t - 1) % 3;
                    if (m == i) {
                        for (int j = 0; j < n; ++j) {
                            if (j == i) continue;
                            v -= __ldg(wrow + j * pch * 32 + 32) * geo[(i * n + j) * 4 + c] * hm[(j * Tp) * 32 + f];
                        }
                    } else {
                        v += __ldg(wrow + m * pch * 32 + 32) * geo[(i * n + m) * 4 + c] * hm[(m * Tp) * 32 + f];
                    }
                } else if (t == d.lap) {
                    for (int j = 0; j < n; ++j) {
                        if (j == i) continue;
                        const float* gg = geo + (i * n + j) * 4;
                        const float w1 = __ldg(wrow + j * pch * 32 + 32), w2 = __ldg(wrow + j * pch * 32 + 64);
                        const float* hj = hm + (size_t)j * Tp * 32 + f;
                        float cross = 0.f;
                        #pragma unroll
                        for (int c = 0; c < 3; ++c) cross += gg[c] * (hj[(1 + 3 * j + c) * 32] - hj[(1 + 3 * i + c) * 32]);
                        v += 2.f * (w2 + 2.f * w1 * gg[3]) * hj[0] + 2.f * w1 * cross;
                    }
                }
            } else {
                const int f = col - E;
                int ch = -1;
                if (t == 0) ch = 0;
                else if (t == d.lap) ch = 4;
                else if (t >= 1 + 3 * i && t < 4 + 3 * i) ch = t - 3 * i;
                if (ch >= 0) {
                    const float* he = heb + (size_t)i * d.N * ech * 32;
                    const float* hs = himl + (size_t)seg_of(d, b) * 4 * d.N * 32;
                    #pragma unroll 4
                    for (int I = 0; I < d.N; ++I) v += __ldg(he + (I * ech + ch) * 32 + f) * __ldg(hs + I * 32 + f);
                }
            }
        }
        ActIO<Act>::store(X, ((int64_t)b * n + i) * Tp + t, ldx, hw + col, v);
    }
}

// ------------------------------------------------------------------ envelope x backflow -> Slater tangents
// mo[b][k][t][i][o] = env[i,(k,o)] * bf[i,(k,o)] with tangents (envelope_orbitals.py:91-127).
// env = sum_I w_I exp(-softplus(alpha_I) d_iI); grad/Laplacian w.r.t. r_i only.
__global__ void k_envelope(const float* __restrict__ r, const float* __restrict__ Rall, const int32_t* __restrict__ Zall,
                           const float* __restrict__ P, ParamLayout L, const float* __restrict__ spA, Dims d, int B,
                           const float* __restrict__ BF, int ldbf, int spin_cols, float* __restrict__ MO) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * d.n * d.KN) return;
    int col = idx % d.KN;
    int64_t bi = idx / d.KN;
    int i = bi % d.n, b = bi / d.n;
    int k = col / d.n, o = col % d.n;
    bool up = i < d.nu;
    const float* spa = spA + (up ? 0 : d.N * d.KN);          // softplus(alpha), prepared
    const float* wts = P + (up ? L.weights_up : L.weights_dn);
    const float* ri = r + bi * 3;
    const int sg = seg_of(d, b);
    const float* R = Rall + (size_t)sg * d.N * 3;
    const int32_t* Z = Zall + (size_t)sg * d.N;
    float env = 0.f, g[3] = {0.f, 0.f, 0.f}, lapv = 0.f;
    for (int I = 0; I < d.N; ++I) {
        if (Z[I] <= 0) continue;                                  // padding ion
        float s0 = ri[0] - R[I * 3], s1 = ri[1] - R[I * 3 + 1], s2 = ri[2] - R[I * 3 + 2];
        float dd = sqrtf(s0 * s0 + s1 * s1 + s2 * s2);
        float a = __ldg(spa + I * d.KN + col);
        float e = wts[I * d.KN + col] * expf(-a * dd);
        env += e;
        if (d.Tp > 1) {
            float gs = -a * e / dd;
            g[0] += gs * s0; g[1] += gs * s1; g[2] += gs * s2;
            lapv += e * (a * a - 2.f * a / dd);
        }
    }
    const float* bf = BF + bi * d.Tp * ldbf + (up ? 0 : spin_cols) + col;
    int64_t mstride = (int64_t)d.n * d.n;                    // per channel
    float* mo = MO + (((int64_t)b * d.K + k) * d.T) * mstride + i * d.n + o;
    float bf0 = bf[0];
    mo[0] = env * bf0;
    if (d.Tp == 1) return;
    // gradient channels four at a time (the four backflow loads in flight together); the
    // electron's own three coordinates also carry the envelope gradient times the value row
    const int n3 = 3 * d.n;
    for (int t0 = 1; t0 <= n3; t0 += 4) {
        float bv[4];
        #pragma unroll
        for (int u = 0; u < 4; ++u) bv[u] = t0 + u <= n3 ? __ldg(bf + (int64_t)(t0 + u) * ldbf) : 0.f;
        #pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int t = t0 + u;
            if (t > n3) break;
            float v = env * bv[u];
            const unsigned c = (unsigned)(t - 1 - 3 * i);
            if (c < 3u) v += (c == 0 ? g[0] : (c == 1 ? g[1] : g[2])) * bf0;
            mo[t * mstride] = v;
        }
    }
    float vl = env * bf[(int64_t)d.lap * ldbf] + lapv * bf0;
    for (int c = 0; c < 3; ++c) vl += 2.f * g[c] * bf[(int64_t)(1 + 3 * i + c) * ldbf];
    mo[d.lap * mstride] = vl;
}

// ------------------------------------------------------------------ Jastrow output layer + electron sum
// jas[b][t] = sum_i sum_f J2[(b,i,t), f] * w2[f]  (wavefunction.py:58-59, linear output, no bias)
template <class Act>
__global__ void k_jastrow_out(const Act* __restrict__ J2, int ldj, const float* __restrict__ w2, Dims d, int B,
                              double* __restrict__ jas) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= B * d.Tp) return;
    int b = warp / d.Tp, t = warp % d.Tp;
    float acc = 0.f;
    for (int i = 0; i < d.n; ++i) {
        const int64_t row = (int64_t)(b * d.n + i) * d.Tp + t;
        for (int f = lane; f < d.J1; f += 32) acc += ActIO<Act>::load(J2, row, ldj, f) * w2[f];
    }
    acc = warp_sum(acc);
    if (lane == 0) jas[(int64_t)b * d.Tp + t] = acc;
}

// ------------------------------------------------------------------ launch wrappers
void launch_ion_maps(const float* P, const ParamLayout& L, const Dims& d, const int32_t* Z, float* him, cudaStream_t s) {
    const int n = d.nseg * 4 * d.N * 32;
    k_ion_maps<<<(n + 255) / 256, 256, 0, s>>>(P, L, d, Z, him); count_launch();
}
template <class Act>
void launch_features(const float* r, const float* R, const int32_t* Z, const Dims& d, int B, Act* X0, cudaStream_t s) {
    const int fthreads = std::min(256, 32 * d.Tp);        // one warp per channel row, up to 8 warps
    k_features<Act><<<B * d.n, fthreads, 0, s>>>(r, R, Z, d, B, X0); count_launch();
}
// The fused el-ion reduction needs whole electrons in one block and a convolution kernel that
// reads it (k_conv_tile, 8 <= Tp <= 128). It is used in tangent passes only: for value rows the
// separate k_ei_mlp + k_conv_value pair measured faster (the fused kernel's extra shared-memory
// pass costs more than the stream traffic it saves).
bool ei_fusable(const Dims& d) {
    return d.E == 32 && d.EI == 32 && d.Tp >= 8 && d.Tp <= 128 && d.N * 5 <= kRB;
}

void launch_streams(const float* r, const float* R, const int32_t* Z, const float* P, const ParamLayout& L,
                    const Dims& d, int B, float* WP, float* HE, cudaStream_t s, float* HP, const float* him) {
    const bool tang = d.Tp > 1;
    if (him && !ei_fusable(d)) him = nullptr;
    const int64_t npair = (int64_t)B * d.n * (d.n + 1) / 2, nei = (int64_t)B * d.n * d.N;
    auto blocks = [](int64_t n) { return (unsigned)((n + 127) / 128); };
    if (tang) {
        size_t sm3 = 128 * (3 * 32 + 1) * sizeof(float), sm5 = 128 * (5 * 32 + 1) * sizeof(float);
        cudaFuncSetAttribute(k_ei_streams<5>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm5);
        cudaFuncSetAttribute(k_pair_streams<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm3);
        if (d.E == 32 && d.EI == 32) {
            constexpr int EP = kRB / 3, EE = kRB / 5;
            const int64_t same_rows = (int64_t)B * (d.nu * (d.nu + 1) / 2 + d.nd * (d.nd + 1) / 2);
            const int64_t diff_rows = (int64_t)B * d.nu * d.nd;
            const int bs = (int)((same_rows + EP - 1) / EP), bd = (int)((diff_rows + EP - 1) / EP);
            k_pair_mlp_t<<<bs + bd, 128, 0, s>>>(r, P, L, d, B, bs, WP);
            if (him) {
                const int epb = kRB / (d.N * 5);
                k_ei_conv<5><<<(unsigned)(((int64_t)B * d.n + epb - 1) / epb), 128, 0, s>>>(r, R, Z, P, L, d, B, him, HE);
            } else {
                k_ei_mlp_t<<<(unsigned)((nei + EE - 1) / EE), 128, 0, s>>>(r, R, Z, P, L, d, B, HE);
            }
        } else {
            k_pair_streams<3><<<blocks(npair), 128, sm3, s>>>(r, P, L, d, B, WP, nullptr);
            k_ei_streams<5><<<blocks(nei), 128, sm5, s>>>(r, R, Z, P, L, d, B, HE);
        }
    } else {
        const int64_t same_rows = (int64_t)B * (d.nu * (d.nu + 1) / 2 + d.nd * (d.nd + 1) / 2);
        const int64_t diff_rows = (int64_t)B * d.nu * d.nd;
        const int bs = (int)((same_rows + kRB - 1) / kRB), bd = (int)((diff_rows + kRB - 1) / kRB);
        k_pair_mlp<<<bs + bd, 128, 0, s>>>(r, P, L, d, B, bs, WP, HP);
        if (him) {
            const int epb = kRB / d.N;
            k_ei_conv<1><<<(unsigned)(((int64_t)B * d.n + epb - 1) / epb), 128, 0, s>>>(r, R, Z, P, L, d, B, him, HE);
        } else {
            k_ei_mlp<<<(unsigned)((nei + kRB - 1) / kRB), 128, 0, s>>>(r, R, Z, P, L, d, B, HE);
        }
    }
    count_launch(2);
}
template <class Act>
void launch_spin_means(const Act* X, int ldx, int hw, const Dims& d, int B, Act* M, int mw, cudaStream_t s) {
    if constexpr (std::is_same<Act, Split>::value) {
        if (hw % 8 == 0) { k_spin_means_split8<<<B, 256, 0, s>>>(X, ldx, hw, d, M, mw); count_launch(); return; }
    }
    k_spin_means<Act><<<B, 256, 0, s>>>(X, ldx, hw, d, M, mw); count_launch();
}
template <class Act>
void launch_tanh_fl(const float* Zb, int ldz, int ncols, int groups, const Dims& d, Act* Y, int ldy, cudaStream_t s) {
    int64_t n = (int64_t)groups * ncols;
    k_tanh_fl<Act><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(Zb, ldz, ncols, groups, d, Y, ldy); count_launch();
}
template <class Act>
void launch_conv(const float* r, const float* WPl, const float* HM, const float* HEl, const float* himl, const Dims& d,
                 int l, int B, Act* X, int ldx, cudaStream_t s, int ei_fused) {
    if (d.Tp >= 8 && d.Tp <= 128 && d.E == 32) {
        // 4 electrons per block (8 or 5 per block measured slower: larger shared-memory tiles and
        // product-rule loops outweigh the extra reuse of each h_map load)
        constexpr int TI = 4;
        const unsigned grid = (unsigned)B * ((d.n + TI - 1) / TI);
        const int TT = d.Tp >= 64 ? 8 : d.Tp / 8;
        const int NW = d.Tp / TT;
        const size_t smem = ((size_t)TI * d.Tp * 32 + (size_t)NW * TI * 4 * 32 + (size_t)TI * 5 * 32) * sizeof(float);
        auto go = [&](auto kern) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kern<<<grid, NW * 32, smem, s>>>(r, WPl, HM, HEl, himl, d, l, B, X, ldx, ei_fused);
        };
        auto pick = [&](auto ti) {
            constexpr int T_I = decltype(ti)::value;
            switch (TT) {
                case 1: go(k_conv_tile<Act, 1, T_I>); break;
                case 2: go(k_conv_tile<Act, 2, T_I>); break;
                case 4: go(k_conv_tile<Act, 4, T_I>); break;
                default: go(k_conv_tile<Act, 8, T_I>); break;
            }
        };
        pick(std::integral_constant<int, TI>());
        count_launch();
        return;
    }
    if (d.Tp == 1 && d.E % 8 == 0 && !ei_fused) {
        const int octs = d.E / 8 + (d.eiw[l] + 7) / 8;
        const int64_t threads = (int64_t)B * d.n * octs;
        k_conv_value<Act><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(WPl, HM, HEl, himl, d, l, B, X, ldx);
        count_launch();
        return;
    }
    const size_t smem = ((size_t)d.n * d.Tp * 32 + (size_t)d.n * d.n * 4) * sizeof(float);
    if (smem <= 200 * 1024) {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(k_conv_walker<Act>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        k_conv_walker<Act><<<B, 256, smem, s>>>(r, WPl, HM, HEl, himl, d, l, B, X, ldx);
    } else {
        k_conv<Act><<<B * d.n, 256, 0, s>>>(r, WPl, HM, HEl, himl, d, l, B, X, ldx);
    }
    count_launch();
}
// Envelopes by rows: grid (walker groups of kEnvWG, column chunks, spin); each thread owns one
// orbital column (k, o) of one spin. softplus(alpha) and the weight of every ion for that column
// stay in registers across all rows of the block; per (electron, ion) the difference vector,
// distance and inverse distance are formed once in shared memory (a negative distance marks a
// padding ion of a packed geometry). Same mathematics as k_envelope.
// NI bounds the ions held in registers; with NI = 8 four blocks fit an SM, which doubles the loads
// in flight of this memory-bound kernel.
constexpr int kEnvWG = 4;
constexpr int kEnvMaxIons = 16;
template <int NI>
__global__ void __launch_bounds__(256, NI <= 8 ? 4 : 2)
k_envelope_rows(const float* __restrict__ r, const float* __restrict__ Rall, const int32_t* __restrict__ Zall,
                const float* __restrict__ P, ParamLayout L, const float* __restrict__ spA, Dims d, int B,
                const float* __restrict__ BF, int ldbf, int spin_cols, float* __restrict__ MO) {
    extern __shared__ float se[];                            // [row][ion][5]: dx, dy, dz, dist, 1/dist
    const int spin = blockIdx.z;
    const int ns = spin == 0 ? d.nu : d.nd, i0 = spin == 0 ? 0 : d.nu;
    const int b0 = blockIdx.x * kEnvWG;
    const int nb = min(kEnvWG, B - b0);
    const int rows = nb * ns, N = d.N;
    for (int e = threadIdx.x; e < rows * N; e += blockDim.x) {
        const int rr = e / N, I = e % N;
        const int b = b0 + rr / ns, i = i0 + rr % ns;
        const int sg = seg_of(d, b);
        const float* R = Rall + (size_t)sg * N * 3;
        const float* ri = r + ((int64_t)b * d.n + i) * 3;
        const float s0 = ri[0] - R[I * 3], s1 = ri[1] - R[I * 3 + 1], s2 = ri[2] - R[I * 3 + 2];
        const float dd = sqrtf(s0 * s0 + s1 * s1 + s2 * s2);
        float* o = se + (size_t)e * 5;
        o[0] = s0; o[1] = s1; o[2] = s2;
        o[3] = Zall[(size_t)sg * N + I] > 0 ? dd : -1.f;
        o[4] = 1.f / dd;
    }
    __syncthreads();
    const int col = blockIdx.y * blockDim.x + threadIdx.x;
    if (col >= d.KN) return;
    const float* spa = spA + (spin ? (size_t)N * d.KN : 0);   // softplus(alpha), prepared
    const float* wts = P + (spin ? L.weights_dn : L.weights_up);
    float av[NI], wv[NI];
    #pragma unroll
    for (int I = 0; I < NI; ++I) {
        av[I] = I < N ? __ldg(spa + (size_t)I * d.KN + col) : 0.f;
        wv[I] = I < N ? __ldg(wts + (size_t)I * d.KN + col) : 0.f;
    }
    const int k = col / d.n, o = col - (col / d.n) * d.n;
    const int64_t mstride = (int64_t)d.n * d.n;              // per channel
    const bool tang = d.Tp > 1;
    if (!tang) {
        // value rows four at a time: the four backflow loads are in flight together
        for (int r4 = 0; r4 < rows; r4 += 4) {
            float bfv[4], env4[4];
            #pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int rr = min(r4 + u, rows - 1);
                const int b = b0 + rr / ns, i = i0 + rr % ns;
                bfv[u] = __ldg(BF + ((int64_t)b * d.n + i) * ldbf + (spin ? spin_cols : 0) + col);
            }
            #pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float* gv = se + (size_t)min(r4 + u, rows - 1) * N * 5;
                float env = 0.f;
                #pragma unroll
                for (int I = 0; I < NI; ++I) {
                    if (I >= N) break;
                    const float dd = gv[I * 5 + 3];
                    if (dd < 0.f) continue;                  // padding ion
                    env += wv[I] * expf(-av[I] * dd);
                }
                env4[u] = env;
            }
            #pragma unroll
            for (int u = 0; u < 4; ++u) {
                if (r4 + u >= rows) break;
                const int rr = r4 + u, b = b0 + rr / ns, i = i0 + rr % ns;
                MO[((int64_t)b * d.K + k) * mstride + i * d.n + o] = env4[u] * bfv[u];
            }
        }
        return;
    }
    for (int rr = 0; rr < rows; ++rr) {
        const int b = b0 + rr / ns, i = i0 + rr % ns;
        const float* gv = se + (size_t)rr * N * 5;
        float env = 0.f, g0 = 0.f, g1 = 0.f, g2 = 0.f, lapv = 0.f;
        #pragma unroll
        for (int I = 0; I < NI; ++I) {
            if (I >= N) break;
            const float dd = gv[I * 5 + 3];
            if (dd < 0.f) continue;                          // padding ion
            const float a = av[I];
            const float e = wv[I] * expf(-a * dd);
            env += e;
            if (tang) {
                const float inv = gv[I * 5 + 4];
                const float gs = -a * e * inv;
                g0 += gs * gv[I * 5]; g1 += gs * gv[I * 5 + 1]; g2 += gs * gv[I * 5 + 2];
                lapv += e * (a * a - 2.f * a * inv);
            }
        }
        const float* bf = BF + ((int64_t)b * d.n + i) * d.Tp * ldbf + (spin ? spin_cols : 0) + col;
        float* mo = MO + (((int64_t)b * d.K + k) * d.T) * mstride + i * d.n + o;
        const float bf0 = bf[0];
        mo[0] = env * bf0;
        if (!tang) continue;
        for (int t = 1; t <= 3 * d.n; ++t) {
            float v = env * bf[(int64_t)t * ldbf];
            const unsigned c = (unsigned)(t - 1 - 3 * i);     // own coordinate channels
            if (c < 3u) v += (c == 0 ? g0 : (c == 1 ? g1 : g2)) * bf0;
            mo[t * mstride] = v;
        }
        float vl = env * bf[(int64_t)d.lap * ldbf] + lapv * bf0;
        vl += 2.f * (g0 * bf[(int64_t)(1 + 3 * i) * ldbf] + g1 * bf[(int64_t)(2 + 3 * i) * ldbf] +
                     g2 * bf[(int64_t)(3 + 3 * i) * ldbf]);
        mo[d.lap * mstride] = vl;
    }
}

void launch_envelope(const float* r, const float* R, const int32_t* Z, const float* P, const ParamLayout& L,
                     const float* sp_alpha, const Dims& d, int B, const float* BF, int ldbf, int spin_cols, float* MO,
                     cudaStream_t s) {
    // value-only rows: row-blocked form (the tangent form writes 3n + 2 channels per element and
    // keeps one thread per element for parallelism)
    if (d.N <= kEnvMaxIons && d.Tp == 1) {
        const int threads = std::min(256, round_up(d.KN, 32));
        const int ns_max = std::max(d.nu, d.nd);
        const size_t sm = (size_t)kEnvWG * ns_max * d.N * 5 * sizeof(float);
        dim3 grid((unsigned)((B + kEnvWG - 1) / kEnvWG), (unsigned)((d.KN + threads - 1) / threads), d.nd > 0 ? 2 : 1);
        if (d.N <= 8) k_envelope_rows<8><<<grid, threads, sm, s>>>(r, R, Z, P, L, sp_alpha, d, B, BF, ldbf, spin_cols, MO);
        else k_envelope_rows<16><<<grid, threads, sm, s>>>(r, R, Z, P, L, sp_alpha, d, B, BF, ldbf, spin_cols, MO);
        count_launch();
        return;
    }
    int64_t n = (int64_t)B * d.n * d.KN;
    k_envelope<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(r, R, Z, P, L, sp_alpha, d, B, BF, ldbf, spin_cols, MO);
    count_launch();
}
template <class Act>
void launch_jastrow_out(const Act* J2, int ldj, const float* w2, const Dims& d, int B, double* jas, cudaStream_t s) {
    int64_t warps = (int64_t)B * d.Tp;
    k_jastrow_out<Act><<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(J2, ldj, w2, d, B, jas); count_launch();
}

#define DW_INST(Act)                                                                                          \
    template void launch_features<Act>(const float*, const float*, const int32_t*, const Dims&, int, Act*,    \
                                       cudaStream_t);                                                         \
    template void launch_spin_means<Act>(const Act*, int, int, const Dims&, int, Act*, int, cudaStream_t);    \
    template void launch_tanh_fl<Act>(const float*, int, int, int, const Dims&, Act*, int, cudaStream_t);     \
    template void launch_conv<Act>(const float*, const float*, const float*, const float*, const float*,      \
                                   const Dims&, int, int, Act*, int, cudaStream_t, int);                      \
    template void launch_jastrow_out<Act>(const Act*, int, const float*, const Dims&, int, double*, cudaStream_t);
DW_INST(float)
DW_INST(__nv_bfloat16)
DW_INST(Split)

}  // namespace dw
