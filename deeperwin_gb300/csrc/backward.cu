// Hand-written reverse mode for the parameter gradient of  L = sum_b c_b log psi^2_b.
//
// With c_b = (E_clip,b - mean E_clip) / B this is the VMC gradient of
// optimization/loss_function.py:141-153 (the custom JVP of total_energy). Per walker chunk the
// value-only forward is recomputed (activations are not kept from any earlier call) with its
// intermediates held in the workspace, then the adjoints run backwards:
//   sum of determinants (wavefunction.py:63-83)  ->  dA_k = g_k A_k^-T (FP64 Gauss-Jordan inverse)
//   envelopes x backflow (envelope_orbitals.py:91-127) -> alpha, weights, W_up, W_dn
//   Jastrow MLP (wavefunction.py:48-60)
//   four h_el layers with spin means and SchNet convolutions (ferminet_embedding.py:52-262)
//   2-el same/diff streams and w maps, el-ion stream, ion maps and ion embedding.
// Weight gradients are reductions over rows (walker x electron / pair) done by split-row
// FP32 kernels with atomic accumulation into the caller's (zeroed) packed gradient.
#include "net.cuh"
#include <algorithm>
#include <string.h>

namespace dw {

namespace {

struct Bwd {
    Dims d;
    int Bc, rows, npair, nei;
    float* him;                       // [4][N][32]
    float* X[4];                      // layer inputs [rows, kw_l]
    float* Mc[4];                     // spin means [Bc, mw_l]
    float* WB;                        // [Bc, D]
    float* HM[4];                     // h_map outputs [rows, 32]
    float* H4;                        // final embedding [rows, D]
    float* WP;                        // [4][Bc n n][32]
    float* HE;                        // [4][Bc n N][32]
    float* HP;                        // [3][Bc npair][32] stream levels 1..3
    float* HP0;                       // [Bc npair] the input distance of each unordered pair
    int8_t* sel;                      // [Bc npair] 1 = same-spin pair
    float *J1, *J2;                   // [rows, 64]
    float* BF;                        // [rows, 2 KN]
    float* MO;                        // [Bc, K, n, n]
    double *logdet, *sign;
    float* Ainv;                      // [Bc, K, n, n]
    float* crow;                      // [rows] per-row coefficient c_b
    // adjoints
    float *dH, *dZ, *dX, *dZw, *dMc, *dHM, *dMO, *dBF, *dENV, *dJ;
    float* dWP;                       // [4][Bc n n][32] ordered (i, j) adjoints of w_ij
    float* dHE;                       // [4][Bc n N][32]
    float* dZp;                       // [7][Bc npair][32]: w maps l = 0..3, streams l = 0..2
    float* dZe;                       // [3][Bc nei][32]
    float* dHIM;                      // [4][N][32]
    size_t bytes;
};

inline int mean_w(const Dims& d, int l) { return round_up(2 * d.hw[l], 64); }

Bwd carve_bwd(const Dims& d, int Bc, void* ws) {
    Carver c(ws, (size_t)-1);
    Bwd b;
    b.d = d; b.Bc = Bc;
    b.rows = Bc * d.n;
    b.npair = Bc * d.n * (d.n + 1) / 2;
    b.nei = Bc * d.n * d.N;
    const int64_t rows = b.rows;
    b.him = c.take<float>(4 * d.N * 32);
    for (int l = 0; l < 4; ++l) {
        b.X[l] = c.take<float>(rows * d.kw[l]);
        b.Mc[l] = c.take<float>((int64_t)Bc * mean_w(d, l));
        b.HM[l] = c.take<float>(rows * 32);
    }
    b.WB = c.take<float>((int64_t)Bc * d.D);
    b.H4 = c.take<float>(rows * d.D);
    b.WP = c.take<float>((int64_t)4 * Bc * d.n * d.n * 32);
    b.HE = c.take<float>((int64_t)4 * b.nei * 32);
    b.HP = c.take<float>((int64_t)3 * b.npair * 32);
    b.HP0 = c.take<float>(b.npair);
    b.sel = c.take<int8_t>(b.npair);
    b.J1 = c.take<float>(rows * d.J0);
    b.J2 = c.take<float>(rows * d.J1);
    b.BF = c.take<float>(rows * 2 * d.KN);
    b.MO = c.take<float>((int64_t)Bc * d.K * d.n * d.n);
    b.logdet = c.take<double>((int64_t)Bc * d.K);
    b.sign = c.take<double>((int64_t)Bc * d.K);
    b.Ainv = c.take<float>((int64_t)Bc * d.K * d.n * d.n);
    b.crow = c.take<float>(rows);
    int kwmax = 0, mwmax = 0;
    for (int l = 0; l < 4; ++l) { kwmax = std::max(kwmax, d.kw[l]); mwmax = std::max(mwmax, mean_w(d, l)); }
    b.dH = c.take<float>(rows * d.D);
    b.dZ = c.take<float>(rows * std::max(d.D, 2 * d.KN));
    b.dX = c.take<float>(rows * kwmax);
    b.dZw = c.take<float>((int64_t)Bc * d.D);
    b.dMc = c.take<float>((int64_t)Bc * mwmax);
    b.dHM = c.take<float>(rows * 32);
    b.dMO = c.take<float>((int64_t)Bc * d.K * d.n * d.n);
    b.dBF = c.take<float>(rows * 2 * d.KN);
    b.dENV = c.take<float>(rows * d.KN);
    b.dJ = c.take<float>(rows * std::max(d.J0, d.J1));
    b.dWP = c.take<float>((int64_t)4 * Bc * d.n * d.n * 32);
    b.dHE = c.take<float>((int64_t)4 * b.nei * 32);
    b.dZp = c.take<float>((int64_t)7 * b.npair * 32);
    b.dZe = c.take<float>((int64_t)3 * b.nei * 32);
    b.dHIM = c.take<float>(4 * d.N * 32);
    b.bytes = c.used;
    return b;
}

// ---------------------------------------------------------------- determinant adjoints
// Block per walker: g_k = d(2 f)/d l_k with f = log(|sum_k s_k e^{l_k - l_max}| + 1e-8) + l_max
// (derivative of the max taken at the first maximal determinant, as in the forward), then
// dA_k = c_b g_k A_k^-T.
__global__ void k_bwd_dets(const double* __restrict__ logdet, const double* __restrict__ sign,
                           const float* __restrict__ Ainv, const float* __restrict__ coeff, int K, int n,
                           float* __restrict__ dMO) {
    __shared__ double gk[128];
    const int b = blockIdx.x;
    if (threadIdx.x == 0) {
        const double* ld = logdet + (int64_t)b * K;
        const double* sg = sign + (int64_t)b * K;
        double lmax = -INFINITY; int ks = 0;
        for (int k = 0; k < K; ++k) if (ld[k] > lmax) { lmax = ld[k]; ks = k; }
        double psi = 0.0;
        for (int k = 0; k < K; ++k) psi += sg[k] * exp(ld[k] - lmax);
        const double eps = 1e-8, u = fabs(psi), sgn = psi < 0 ? -1.0 : 1.0;
        for (int k = 0; k < K; ++k) {
            double g = sgn * sg[k] * exp(ld[k] - lmax) / (u + eps);
            if (k == ks) g += eps / (u + eps);
            gk[k] = 2.0 * g * (double)coeff[b];
        }
    }
    __syncthreads();
    const int nn = n * n;
    for (int e = threadIdx.x; e < K * nn; e += blockDim.x) {
        const int k = e / nn, io = e % nn, i = io / n, o = io % n;
        const float* ai = Ainv + ((int64_t)b * K + k) * nn;
        dMO[((int64_t)b * K + k) * nn + io] = (float)gk[k] * ai[o * n + i];
    }
}

// Envelope x backflow adjoints per (walker, electron, column): dBF (in the spin's half of the
// [W_up | W_dn] columns, zero in the other) and dENV = dmo * bf.
__global__ void k_bwd_envelope(const float* __restrict__ r, const float* __restrict__ R, const float* __restrict__ P,
                               ParamLayout L, const float* __restrict__ spA, Dims d, int B, const float* __restrict__ BF,
                               const float* __restrict__ dMO, float* __restrict__ dBF, float* __restrict__ dENV) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * d.n * d.KN) return;
    const int col = idx % d.KN;
    const int64_t bi = idx / d.KN;
    const int i = bi % d.n, b = bi / d.n;
    const int k = col / d.n, o = col % d.n;
    const bool up = i < d.nu;
    const float* spa = spA + (up ? 0 : d.N * d.KN);
    const float* wts = P + (up ? L.weights_up : L.weights_dn);
    const float* ri = r + bi * 3;
    float env = 0.f;
    for (int I = 0; I < d.N; ++I) {
        const float s0 = ri[0] - R[I * 3], s1 = ri[1] - R[I * 3 + 1], s2 = ri[2] - R[I * 3 + 2];
        const float dd = sqrtf(s0 * s0 + s1 * s1 + s2 * s2);
        env += wts[I * d.KN + col] * expf(-spa[I * d.KN + col] * dd);
    }
    const float dmo = dMO[(((int64_t)b * d.K + k) * d.n + i) * d.n + o];
    const float bf = BF[bi * 2 * d.KN + (up ? 0 : d.KN) + col];
    dBF[bi * 2 * d.KN + (up ? 0 : d.KN) + col] = dmo * env;
    dBF[bi * 2 * d.KN + (up ? d.KN : 0) + col] = 0.f;
    dENV[bi * d.KN + col] = dmo * bf;
}

// alpha / weights gradients: block per (spin, ion, 32 columns, row segment), the segment's rows of
// that spin strided over the block's 8 row lanes, then a shared-memory reduction and one atomic
// add per column and segment.
__global__ void k_bwd_env_params(const float* __restrict__ r, const float* __restrict__ R, const float* __restrict__ P,
                                 ParamLayout L, Dims d, int B, const float* __restrict__ dENV,
                                 float* __restrict__ grad, int col_chunks, int rows_per_seg) {
    __shared__ float red[2][8][33];
    const int spin = blockIdx.z, I = blockIdx.y, lane8 = threadIdx.x >> 5;
    const int cchunk = blockIdx.x % col_chunks, seg = blockIdx.x / col_chunks;
    const int col = cchunk * 32 + (threadIdx.x & 31);
    const int i0 = spin == 0 ? 0 : d.nu, ns = spin == 0 ? d.nu : d.nd;
    const int e_begin = seg * rows_per_seg, e_end = min(B * ns, e_begin + rows_per_seg);
    float ga = 0.f, gw = 0.f;
    if (col < d.KN) {
        const float al = P[(spin == 0 ? L.alpha_up : L.alpha_dn) + I * d.KN + col];
        const float w = P[(spin == 0 ? L.weights_up : L.weights_dn) + I * d.KN + col];
        const float a = softplus_f(al), sig = 1.f / (1.f + expf(-al));
        for (int e = e_begin + lane8; e < e_end; e += 8) {
            const int b = e / ns, i = i0 + e % ns;
            const int64_t bi = (int64_t)b * d.n + i;
            const float* ri = r + bi * 3;
            const float s0 = ri[0] - R[I * 3], s1 = ri[1] - R[I * 3 + 1], s2 = ri[2] - R[I * 3 + 2];
            const float dd = sqrtf(s0 * s0 + s1 * s1 + s2 * s2);
            const float ex = expf(-a * dd);
            const float g = dENV[bi * d.KN + col];
            gw += g * ex;
            ga += g * w * ex * (-dd) * sig;
        }
    }
    red[0][lane8][threadIdx.x & 31] = ga;
    red[1][lane8][threadIdx.x & 31] = gw;
    __syncthreads();
    if (lane8 == 0 && col < d.KN) {
        float sa = 0.f, sw = 0.f;
        for (int k = 0; k < 8; ++k) { sa += red[0][k][threadIdx.x]; sw += red[1][k][threadIdx.x]; }
        atomicAdd(grad + (spin == 0 ? L.alpha_up : L.alpha_dn) + I * d.KN + col, sa);
        atomicAdd(grad + (spin == 0 ? L.weights_up : L.weights_dn) + I * d.KN + col, sw);
    }
}

// y = tanh(z) adjoint: dz = dy (1 - y^2); dz may alias dy.
__global__ void k_tanh_bwd(const float* __restrict__ dy, int lddy, const float* __restrict__ y, int ldy, int rows,
                           int cols, float* __restrict__ dz, int lddz) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)rows * cols) return;
    const int64_t rr = idx / cols;
    const int c = idx % cols;
    const float yy = y[rr * ldy + c];
    dz[rr * lddz + c] = dy[rr * lddy + c] * (1.f - yy * yy);
}

// per-walker sums of the layer pre-activation adjoints (the spin-mean term is shared by all
// electrons of a walker)
__global__ void k_walker_sum(const float* __restrict__ dz, int ld, int n, int cols, int B, float* __restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * cols) return;
    const int b = idx / cols, c = idx % cols;
    float s = 0.f;
    for (int i = 0; i < n; ++i) s += dz[((int64_t)b * n + i) * ld + c];
    out[idx] = s;
}

// dh[(b,i), f] = dX[(b,i), f] + dMc[b, spin(i) * hw + f] / n_spin   (SymmetricFeatures means)
__global__ void k_means_bwd(const float* __restrict__ dX, int ldx, const float* __restrict__ dMc, int ldm, Dims d,
                            int hw, int B, float* __restrict__ dh, int ldh) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)B * d.n * hw) return;
    const int64_t bi = idx / hw;
    const int f = idx % hw;
    const int i = bi % d.n, b = bi / d.n;
    const bool up = i < d.nu;
    dh[bi * ldh + f] = dX[bi * ldx + f] + dMc[(int64_t)b * ldm + (up ? 0 : hw) + f] / (float)(up ? d.nu : d.nd);
}

// SchNet convolution adjoints, block per walker:
//   dhm[j] = sum_i dconv_ee[i] * w_ij,  dw_ij = dconv_ee[i] * hm[j],
//   de_iI = dconv_ei[i] * him_I,        dhim_I += sum_i dconv_ei[i] * e_iI.
__global__ void k_conv_bwd(const float* __restrict__ dX, int ldx, const float* __restrict__ WPl,
                           const float* __restrict__ HMl, const float* __restrict__ HEl, const float* __restrict__ himl,
                           Dims d, int l, int B, float* __restrict__ dHM, float* __restrict__ dWPl,
                           float* __restrict__ dHEl, float* __restrict__ dHIMl) {
    const int b = blockIdx.x, n = d.n, E = d.E, eiw = d.eiw[l], hw = d.hw[l];
    const float* dxb = dX + (int64_t)b * n * ldx;
    const float* wpb = WPl + (int64_t)b * n * n * 32;
    const float* hmb = HMl + (int64_t)b * n * 32;
    for (int e = threadIdx.x; e < n * E; e += blockDim.x) {
        const int j = e / E, f = e % E;
        float s = 0.f;
        for (int i = 0; i < n; ++i) s += dxb[(int64_t)i * ldx + hw + f] * wpb[((int64_t)i * n + j) * 32 + f];
        dHM[((int64_t)b * n + j) * 32 + f] = s;
    }
    for (int e = threadIdx.x; e < n * n * E; e += blockDim.x) {
        const int ij = e / E, f = e % E, i = ij / n, j = ij % n;
        dWPl[((int64_t)b * n * n + ij) * 32 + f] = dxb[(int64_t)i * ldx + hw + f] * hmb[j * 32 + f];
    }
    const float* heb = HEl + (int64_t)b * n * d.N * 32;
    for (int e = threadIdx.x; e < n * d.N * 32; e += blockDim.x) {
        const int iI = e / 32, f = e % 32, i = iI / d.N, I = iI % d.N;
        dHEl[((int64_t)b * n * d.N + iI) * 32 + f] = f < eiw ? dxb[(int64_t)i * ldx + hw + E + f] * himl[I * 32 + f] : 0.f;
    }
    for (int e = threadIdx.x; e < d.N * eiw; e += blockDim.x) {
        const int I = e / eiw, f = e % eiw;
        float s = 0.f;
        for (int i = 0; i < n; ++i) s += dxb[(int64_t)i * ldx + hw + E + f] * heb[((int64_t)i * d.N + I) * 32 + f];
        atomicAdd(dHIMl + I * 32 + f, s);
    }
}

// Pair streams adjoint, thread per unordered pair (i <= j), reverse through
// w^(l) = tanh(h^(l) W_wm + b) (l = 0..3) and h^(l+1) = res(tanh(h^(l) W_hs + b), h^(l)).
// Writes the pre-activation adjoints dZp[l] (w maps) and dZp[4 + l] (streams) per pair. A layer's
// four weight matrices (map and stream, opposite- and same-spin) are staged in shared memory, the
// copies 16 bytes apart modulo the bank width so that the two spin kinds of a warp read different
// banks, and read as float4 broadcasts (four FMAs per load); pair rows move as float4.
__global__ void __launch_bounds__(128)
k_pair_bwd(const float* __restrict__ r, const float* __restrict__ P, ParamLayout L, Dims d, int B,
           const float* __restrict__ WP, const float* __restrict__ HP, const float* __restrict__ dWP,
           float* __restrict__ dZp, float* __restrict__ HP0, int8_t* __restrict__ sel) {
    constexpr int WPITCH = 32 * 32 + 4;
    __shared__ __align__(16) float Wsh[4 * WPITCH];   // map diff, map same, stream diff, stream same
    const int npw = d.n * (d.n + 1) / 2;
    const int64_t npair = (int64_t)B * npw;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = gid < npair;
    int b = 0, i = 0, j = 0;
    bool same = false;
    if (live) {
        b = (int)(gid / npw);
        int rem = (int)(gid % npw);
        while (rem >= d.n - i) { rem -= d.n - i; ++i; }
        j = i + rem;
        same = (i < d.nu) == (j < d.nu);
        const float* rb = r + (int64_t)b * d.n * 3;
        float dd = 0.f;
        if (i != j) {
            const float dx = rb[j * 3] - rb[i * 3], dy = rb[j * 3 + 1] - rb[i * 3 + 1], dz = rb[j * 3 + 2] - rb[i * 3 + 2];
            dd = sqrtf(dx * dx + dy * dy + dz * dz);
        }
        HP0[gid] = dd;
        sel[gid] = same ? 1 : 0;
    }
    const int64_t plane = (int64_t)B * d.n * d.n;
    const float rs = 0.70710678118654752f;
    float dh[32];
    #pragma unroll
    for (int k = 0; k < 32; ++k) dh[k] = 0.f;
    for (int l = 3; l >= 0; --l) {
        const int in_w = d.eew[l];
        const int in_prev = l > 0 ? d.eew[l - 1] : 0;
        __syncthreads();                              // the previous layer's readers are done
        for (int e = threadIdx.x; e < 4 * 1024; e += blockDim.x) {
            const int m = e >> 10, kf = e & 1023, k = kf >> 5;
            float v = 0.f;
            if (m < 2) {
                if (k < in_w) v = P[(m ? L.w_same_w[l] : L.w_diff_w[l]) + kf];
            } else if (k < in_prev) {
                v = P[(m == 3 ? L.h_same_w[l - 1] : L.h_diff_w[l - 1]) + kf];
            }
            Wsh[m * WPITCH + kf] = v;
        }
        __syncthreads();
        if (!live) continue;
        // w map adjoint
        const float* Wm = Wsh + (same ? WPITCH : 0);
        const int64_t oij = (int64_t)l * plane + (int64_t)b * d.n * d.n + i * d.n + j;
        const int64_t oji = (int64_t)l * plane + (int64_t)b * d.n * d.n + j * d.n + i;
        const float4* w4 = reinterpret_cast<const float4*>(WP + oij * 32);
        const float4* g14 = reinterpret_cast<const float4*>(dWP + oij * 32);
        const float4* g24 = reinterpret_cast<const float4*>(dWP + oji * 32);
        float4* dzw4 = reinterpret_cast<float4*>(dZp + ((int64_t)l * npair + gid) * 32);
        float dz[32];
        #pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float4 wv = w4[q], ga = g14[q];
            const float4 gb = i != j ? g24[q] : make_float4(0.f, 0.f, 0.f, 0.f);
            dz[4 * q] = (ga.x + gb.x) * (1.f - wv.x * wv.x);
            dz[4 * q + 1] = (ga.y + gb.y) * (1.f - wv.y * wv.y);
            dz[4 * q + 2] = (ga.z + gb.z) * (1.f - wv.z * wv.z);
            dz[4 * q + 3] = (ga.w + gb.w) * (1.f - wv.w * wv.w);
            dzw4[q] = make_float4(dz[4 * q], dz[4 * q + 1], dz[4 * q + 2], dz[4 * q + 3]);
        }
        #pragma unroll
        for (int k = 0; k < 32; ++k) {
            if (k < in_w) {
                const float4* wr = reinterpret_cast<const float4*>(Wm + k * 32);
                float acc = 0.f;
                #pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 wq = wr[q];
                    acc = fmaf(dz[4 * q], wq.x, acc);
                    acc = fmaf(dz[4 * q + 1], wq.y, acc);
                    acc = fmaf(dz[4 * q + 2], wq.z, acc);
                    acc = fmaf(dz[4 * q + 3], wq.w, acc);
                }
                dh[k] += acc;
            }
        }
        if (l == 0) continue;
        // stream adjoint: h^(l) = res(y, h^(l-1)), y = tanh(h^(l-1) W_hs + b)
        const bool resid = l - 1 > 0;
        const float* Ws = Wsh + (same ? 3 : 2) * WPITCH;
        const float4* hl4 = reinterpret_cast<const float4*>(HP + ((int64_t)(l - 1) * npair + gid) * 32);   // h^(l)
        const float4* hp4 = reinterpret_cast<const float4*>(HP + ((int64_t)(resid ? l - 2 : 0) * npair + gid) * 32);
        float4* dzs4 = reinterpret_cast<float4*>(dZp + ((int64_t)(4 + l - 1) * npair + gid) * 32);
        float dzh[32];
        #pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float4 hv = hl4[q];
            const float4 pv = resid ? hp4[q] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float h4[4] = {hv.x, hv.y, hv.z, hv.w}, p4[4] = {pv.x, pv.y, pv.z, pv.w};
            #pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int f = 4 * q + u;
                const float y = resid ? 1.41421356237309505f * h4[u] - p4[u] : h4[u];
                const float dy = resid ? dh[f] * rs : dh[f];
                dzh[f] = dy * (1.f - y * y);
            }
            dzs4[q] = make_float4(dzh[4 * q], dzh[4 * q + 1], dzh[4 * q + 2], dzh[4 * q + 3]);
        }
        float dn[32];
        #pragma unroll
        for (int k = 0; k < 32; ++k) {
            float acc = resid ? dh[k] * rs : 0.f;
            if (k < in_prev) {
                const float4* wr = reinterpret_cast<const float4*>(Ws + k * 32);
                #pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 wq = wr[q];
                    acc = fmaf(dzh[4 * q], wq.x, acc);
                    acc = fmaf(dzh[4 * q + 1], wq.y, acc);
                    acc = fmaf(dzh[4 * q + 2], wq.z, acc);
                    acc = fmaf(dzh[4 * q + 3], wq.w, acc);
                }
            }
            dn[k] = acc;
        }
        #pragma unroll
        for (int k = 0; k < 32; ++k) dh[k] = dn[k];
    }
}

// El-ion stream adjoint, thread per (walker, electron, ion): e^(l+1) = res(tanh(e^(l) W + b), e^(l)).
__global__ void __launch_bounds__(128)
k_ei_bwd(const float* __restrict__ P, ParamLayout L, Dims d, int B, const float* __restrict__ HE,
         const float* __restrict__ dHE, float* __restrict__ dZe) {
    const int64_t nei = (int64_t)B * d.n * d.N;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= nei) return;
    const float rs = 0.70710678118654752f;
    float de[32];
    #pragma unroll
    for (int k = 0; k < 32; ++k) de[k] = dHE[((int64_t)3 * nei + gid) * 32 + k];
    for (int l = 3; l >= 1; --l) {
        const bool resid = l - 1 > 0;
        const float* el = HE + ((int64_t)l * nei + gid) * 32;
        const float* ep = HE + ((int64_t)(l - 1) * nei + gid) * 32;
        float dz[32];
        float* dzo = dZe + ((int64_t)(l - 1) * nei + gid) * 32;
        #pragma unroll
        for (int f = 0; f < 32; ++f) {
            const float y = resid ? 1.41421356237309505f * el[f] - ep[f] : el[f];
            dz[f] = (resid ? de[f] * rs : de[f]) * (1.f - y * y);
            dzo[f] = dz[f];
        }
        const float* W = P + L.h_ei_w[l - 1];
        const int in_prev = d.eiw[l - 1];
        float dn[32];
        #pragma unroll
        for (int k = 0; k < 32; ++k) {
            float s = (resid ? de[k] * rs : 0.f) + dHE[((int64_t)(l - 1) * nei + gid) * 32 + k];
            if (k < in_prev) {
                #pragma unroll
                for (int f = 0; f < 32; ++f) s = fmaf(dz[f], __ldg(W + k * 32 + f), s);
            }
            dn[k] = s;
        }
        #pragma unroll
        for (int k = 0; k < 32; ++k) de[k] = dn[k];
    }
}

// Ion maps and ion embedding adjoints (one block): him_l = tanh(emb[Z_I] W_l + b_l).
__global__ void k_ion_bwd(const float* __restrict__ P, ParamLayout L, Dims d, const int32_t* __restrict__ Z,
                          const float* __restrict__ him, const float* __restrict__ dHIM, float* __restrict__ grad) {
    for (int l = 0; l < 4; ++l) {
        const int w = d.eiw[l];
        for (int e = threadIdx.x; e < d.N * w; e += blockDim.x) {
            const int I = e / w, f = e % w;
            const float y = him[(l * d.N + I) * 32 + f];
            const float dz = dHIM[(l * d.N + I) * 32 + f] * (1.f - y * y);
            int z = Z[I] - d.zmin;
            z = z < 0 ? 0 : (z > d.zmax - d.zmin ? d.zmax - d.zmin : z);
            const float* emb = P + L.ion_embed + (int64_t)z * d.EI;
            atomicAdd(grad + L.h_ion_map_b[l] + f, dz);
            for (int k = 0; k < d.EI; ++k) {
                atomicAdd(grad + L.h_ion_map_w[l] + k * w + f, emb[k] * dz);
                atomicAdd(grad + L.ion_embed + (int64_t)z * d.EI + k, dz * P[L.h_ion_map_w[l] + k * w + f]);
            }
        }
    }
}

__global__ void k_row_coeff(const float* __restrict__ coeff, int n, int rows, float* __restrict__ crow) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < rows) crow[idx] = coeff[idx / n];
}
__global__ void k_outer_row(const float* __restrict__ crow, const float* __restrict__ w, int rows, int cols,
                            float* __restrict__ out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx < (int64_t)rows * cols) out[idx] = crow[idx / cols] * w[idx % cols];
}

inline unsigned nblk(int64_t n, int t = 256) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void launch_slogdet_inv(const float* MO, const Dims& d, int B, double* logdet, double* sign, float* Ainv, cudaStream_t s);

static int backward_chunk(const Bwd& w, int Bc, const float* P, const ParamLayout& L, const float* prepared_f32_main[4],
                          const float* prepared_f32_mean[4], const float* bf_cat, const float* spA, const float* r,
                          const float* R, const int32_t* Z, const float* coeff, float* grad, cudaStream_t s) {
    const Dims& d = w.d;
    const int rows = Bc * d.n;
    const int npw = d.n * (d.n + 1) / 2;
    const int64_t npair = (int64_t)Bc * npw, nei = (int64_t)Bc * d.n * d.N;
    // ---------------- forward with stored activations (value only, FP32)
    launch_ion_maps(P, L, d, Z, w.him, s);
    launch_features<float>(r, R, Z, d, Bc, w.X[0], s);
    launch_streams(r, R, Z, P, L, d, Bc, w.WP, w.HE, s, w.HP);
    for (int l = 0; l < 4; ++l) {
        const int hw = d.hw[l], mw = mean_w(d, l);
        launch_spin_means<float>(w.X[l], d.kw[l], hw, d, Bc, w.Mc[l], mw, s);
        GemmEpi e1; e1.bias = P + L.h_el_b[l]; e1.Tp = 1; e1.rows_per_walker = 1;
        gemm_f32(w.Mc[l], mw, prepared_f32_mean[l], d.D, w.WB, d.D, Bc, d.D, mw, e1, 1, 0, 0, s);
        GemmEpi e2; e2.bias = P + L.h_map_b[l]; e2.act = 1;
        gemm_f32(w.X[l], d.kw[l], P + L.h_map_w[l], d.E, w.HM[l], 32, rows, d.E, hw, e2, 1, 0, 0, s);
        const int64_t wpp = (int64_t)Bc * d.n * d.n * 32, hep = nei * 32;
        launch_conv<float>(r, w.WP + l * wpp, w.HM[l], w.HE + l * hep, w.him + l * d.N * 32, d, l, Bc, w.X[l], d.kw[l], s);
        GemmEpi e3; e3.rowbias = w.WB; e3.ldrb = d.D; e3.Tp = 1; e3.rows_per_walker = d.n; e3.act = 1;
        float* out = l < 3 ? w.X[l + 1] : w.H4;
        const int ldo = l < 3 ? d.kw[l + 1] : d.D;
        gemm_f32(w.X[l], d.kw[l], prepared_f32_main[l], d.D, out, ldo, rows, d.D, d.kw[l], e3, 1, 0, 0, s);
    }
    GemmEpi e0;
    gemm_f32(w.H4, d.D, bf_cat, 2 * d.KN, w.BF, 2 * d.KN, rows, 2 * d.KN, d.D, e0, 1, 0, 0, s);
    launch_envelope(r, R, Z, P, L, spA, d, Bc, w.BF, 2 * d.KN, d.KN, w.MO, s);
    launch_slogdet_inv(w.MO, d, Bc, w.logdet, w.sign, w.Ainv, s);
    GemmEpi j0; j0.bias = P + L.jas_b[0]; j0.act = 1;
    GemmEpi j1; j1.bias = P + L.jas_b[1]; j1.act = 1;
    gemm_f32(w.H4, d.D, P + L.jas_w[0], d.J0, w.J1, d.J0, rows, d.J0, d.D, j0, 1, 0, 0, s);
    gemm_f32(w.J1, d.J0, P + L.jas_w[1], d.J1, w.J2, d.J1, rows, d.J1, d.J0, j1, 1, 0, 0, s);

    // ---------------- adjoints
    k_row_coeff<<<nblk(rows), 256, 0, s>>>(coeff, d.n, rows, w.crow);
    // determinants -> Slater matrices -> backflow / envelopes
    k_bwd_dets<<<Bc, 256, 0, s>>>(w.logdet, w.sign, w.Ainv, coeff, d.K, d.n, w.dMO);
    k_bwd_envelope<<<nblk((int64_t)rows * d.KN), 256, 0, s>>>(r, R, P, L, spA, d, Bc, w.BF, w.dMO, w.dBF, w.dENV);
    {
        // row segments: about four blocks per SM in total
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        sms = sms > 0 ? sms : 152;
        const int cc = (d.KN + 31) / 32, ns_max = std::max(d.nu, d.nd);
        int segs = std::max(1, std::min((Bc * ns_max + 63) / 64, (4 * sms + cc * d.N * 2 - 1) / (cc * d.N * 2)));
        const int rps = (Bc * ns_max + segs - 1) / segs;
        k_bwd_env_params<<<dim3(cc * segs, d.N, 2), 256, 0, s>>>(r, R, P, L, d, Bc, w.dENV, grad, cc, rps);
    }
    wgrad_f32(w.H4, d.D, w.dBF, 2 * d.KN, rows, d.D, d.KN, grad + L.bf_up, d.KN, nullptr, nullptr, 0, s);
    wgrad_f32(w.H4, d.D, w.dBF + d.KN, 2 * d.KN, rows, d.D, d.KN, grad + L.bf_dn, d.KN, nullptr, nullptr, 0, s);
    gemm_f32_nt(w.dBF, 2 * d.KN, bf_cat, 2 * d.KN, w.dH, d.D, rows, d.D, 2 * d.KN, 0, s);
    // Jastrow: J = sum_i j2_i . w2 ; j2 = tanh(j1 W1 + b1) ; j1 = tanh(h W0 + b0)
    wgrad_f32(w.J2, d.J1, w.crow, 1, rows, d.J1, 1, grad + L.jas_w[2], 1, nullptr, nullptr, 0, s);
    k_outer_row<<<nblk((int64_t)rows * d.J1), 256, 0, s>>>(w.crow, P + L.jas_w[2], rows, d.J1, w.dJ);
    k_tanh_bwd<<<nblk((int64_t)rows * d.J1), 256, 0, s>>>(w.dJ, d.J1, w.J2, d.J1, rows, d.J1, w.dJ, d.J1);
    wgrad_f32(w.J1, d.J0, w.dJ, d.J1, rows, d.J0, d.J1, grad + L.jas_w[1], d.J1, grad + L.jas_b[1], nullptr, 0, s);
    gemm_f32_nt(w.dJ, d.J1, P + L.jas_w[1], d.J1, w.dZ, d.J0, rows, d.J0, d.J1, 0, s);
    k_tanh_bwd<<<nblk((int64_t)rows * d.J0), 256, 0, s>>>(w.dZ, d.J0, w.J1, d.J0, rows, d.J0, w.dZ, d.J0);
    wgrad_f32(w.H4, d.D, w.dZ, d.J0, rows, d.D, d.J0, grad + L.jas_w[0], d.J0, grad + L.jas_b[0], nullptr, 0, s);
    gemm_f32_nt(w.dZ, d.J0, P + L.jas_w[0], d.J0, w.dH, d.D, rows, d.D, d.J0, 1, s);
    // embedding layers, last to first; w.dH holds dL/dh_{l+1}
    DW_CHECK_CUDA(cudaMemsetAsync(w.dHIM, 0, sizeof(float) * 4 * d.N * 32, s));
    for (int l = 3; l >= 0; --l) {
        const int hw = d.hw[l], mw = mean_w(d, l), kw = d.kw[l];
        const float* hout = l < 3 ? w.X[l + 1] : w.H4;
        const int ldh = l < 3 ? d.kw[l + 1] : d.D;
        k_tanh_bwd<<<nblk((int64_t)rows * d.D), 256, 0, s>>>(w.dH, d.D, hout, ldh, rows, d.D, w.dZ, d.D);
        // weights of the per-electron part: rows [h | conv_ee | conv_ei] of h_el_l.w
        wgrad_f32(w.X[l], kw, w.dZ, d.D, rows, hw, d.D, grad + L.h_el_w[l], d.D, grad + L.h_el_b[l], nullptr, 0, s);
        wgrad_f32(w.X[l] + hw, kw, w.dZ, d.D, rows, d.E + d.eiw[l], d.D, grad + L.h_el_w[l] + (int64_t)3 * hw * d.D,
                  d.D, nullptr, nullptr, 0, s);
        // spin-mean part: rows [mean_up | mean_dn]
        k_walker_sum<<<nblk((int64_t)Bc * d.D), 256, 0, s>>>(w.dZ, d.D, d.n, d.D, Bc, w.dZw);
        wgrad_f32(w.Mc[l], mw, w.dZw, d.D, Bc, 2 * hw, d.D, grad + L.h_el_w[l] + (int64_t)hw * d.D, d.D, nullptr,
                  nullptr, 0, s);
        gemm_f32_nt(w.dZ, d.D, prepared_f32_main[l], d.D, w.dX, kw, rows, kw, d.D, 0, s);
        gemm_f32_nt(w.dZw, d.D, prepared_f32_mean[l], d.D, w.dMc, mw, Bc, mw, d.D, 0, s);
        // convolution adjoints
        const int64_t wpp = (int64_t)Bc * d.n * d.n * 32, hep = nei * 32;
        k_conv_bwd<<<Bc, 256, 0, s>>>(w.dX, kw, w.WP + l * wpp, w.HM[l], w.HE + l * hep, w.him + l * d.N * 32, d, l, Bc,
                                      w.dHM, w.dWP + l * wpp, w.dHE + l * hep, w.dHIM + l * d.N * 32);
        // dh_l = dX[:, :hw] + mean adjoints + h_map adjoint
        if (l > 0) k_means_bwd<<<nblk((int64_t)rows * hw), 256, 0, s>>>(w.dX, kw, w.dMc, mw, d, hw, Bc, w.dH, d.D);
        k_tanh_bwd<<<nblk((int64_t)rows * 32), 256, 0, s>>>(w.dHM, 32, w.HM[l], 32, rows, 32, w.dHM, 32);
        wgrad_f32(w.X[l], kw, w.dHM, 32, rows, hw, d.E, grad + L.h_map_w[l], d.E, grad + L.h_map_b[l], nullptr, 0, s);
        if (l > 0) gemm_f32_nt(w.dHM, 32, P + L.h_map_w[l], d.E, w.dH, d.D, rows, hw, d.E, 1, s);
    }
    // 2-el streams
    k_pair_bwd<<<nblk(npair, 128), 128, 0, s>>>(r, P, L, d, Bc, w.WP, w.HP, w.dWP, w.dZp, w.HP0, w.sel);
    for (int l = 0; l < 4; ++l) {
        const float* A = l == 0 ? w.HP0 : w.HP + (int64_t)(l - 1) * npair * 32;
        const int lda = l == 0 ? 1 : 32, in_w = d.eew[l];
        // one pass over the pairs per weight: same-spin pairs (sel 1) and opposite-spin pairs (sel 0)
        wgrad32_sel2(A, lda, w.dZp + (int64_t)l * npair * 32, 32, (int)npair, in_w, 32, w.sel,
                     grad + L.w_diff_w[l], grad + L.w_diff_b[l], grad + L.w_same_w[l], grad + L.w_same_b[l], 32, s);
        if (l < 3)
            wgrad32_sel2(A, lda, w.dZp + (int64_t)(4 + l) * npair * 32, 32, (int)npair, in_w, 32, w.sel,
                         grad + L.h_diff_w[l], grad + L.h_diff_b[l], grad + L.h_same_w[l], grad + L.h_same_b[l], 32, s);
    }
    // el-ion stream
    k_ei_bwd<<<nblk(nei, 128), 128, 0, s>>>(P, L, d, Bc, w.HE, w.dHE, w.dZe);
    for (int l = 0; l < 3; ++l)
        wgrad_f32(w.HE + (int64_t)l * nei * 32, 32, w.dZe + (int64_t)l * nei * 32, 32, (int)nei, d.eiw[l], 32,
                  grad + L.h_ei_w[l], 32, grad + L.h_ei_b[l], nullptr, 0, s);
    // ion maps / embedding
    k_ion_bwd<<<1, 256, 0, s>>>(P, L, d, Z, w.him, w.dHIM, grad);
    count_launch(40);
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

size_t bwd_bytes(const DwArch* a, int B, int* chunk) {
    Dims d = make_dims(a, false);
    const size_t per = carve_bwd(d, 1, nullptr).bytes;
    const size_t budget = (size_t)4 << 30;
    int bc = (int)std::max<size_t>(1, budget / std::max<size_t>(per, 1));
    bc = std::min(bc, std::max(B, 1));
    if (chunk) *chunk = bc;
    return carve_bwd(d, bc, nullptr).bytes + 4096;
}

int backward_all(const DwArch* a, const float* P, const float* const main[4], const float* const mean[4],
                 const float* bf_cat, const float* sp_alpha, const float* r, int B, const float* R, const int32_t* Z,
                 const float* coeff, float* grad, void* ws, size_t wsb, cudaStream_t s) {
    Dims d = make_dims(a, false);
    ParamLayout L;
    make_layout(a, &L);
    int bc = 0;
    size_t need = bwd_bytes(a, B, &bc);
    if (need > wsb) return DW_ERR_WORKSPACE;
    Bwd w = carve_bwd(d, bc, ws);
    const float* m4[4] = {main[0], main[1], main[2], main[3]};
    const float* n4[4] = {mean[0], mean[1], mean[2], mean[3]};
    for (int b0 = 0; b0 < B; b0 += bc) {
        const int nb = std::min(bc, B - b0);
        Bwd wc = w;
        wc.Bc = nb; wc.rows = nb * d.n; wc.npair = nb * d.n * (d.n + 1) / 2; wc.nei = nb * d.n * d.N;
        DW_CHECK(backward_chunk(wc, nb, P, L, m4, n4, bf_cat, sp_alpha, r + (int64_t)b0 * d.n * 3, R, Z, coeff + b0,
                                grad, s));
    }
    return DW_OK;
}

}  // namespace dw
