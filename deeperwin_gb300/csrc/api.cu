// extern "C" entry points: workspace planning and the launch sequences of the forward
// pass, the forward-Laplacian local energy and the Metropolis-Hastings chain.
#include "net.cuh"
#include "mcmc.cuh"
#include "gemm_tc.cuh"
#include <string.h>
#include <algorithm>
#include <type_traits>

namespace dw {

// ------------------------------------------------------------------ prepared weights
// Per iteration l: Wmain_l [kw_l, D] = rows of h_el_l.w for (h_one, conv_ee, conv_ei) and
// Wmean_l [mw_l, D] = rows for (mean_up, mean_dn) (the spin means are identical for all
// electrons of a walker, so their product is formed once per walker and channel).
// Mixed precision additionally keeps BF16 K-major copies ([N, K]) for the tensor-core GEMMs.
// Tensor-core paths keep BF16 K-major copies ([N, K]) of every GEMM weight: hi = bf16(w) and,
// for the split (mixed) form, lo = bf16(w - hi).
struct WRef {
    const float* f32 = nullptr; int ldw = 0;                // [K, N] row-major FP32
    const __nv_bfloat16* hi = nullptr; const __nv_bfloat16* lo = nullptr;
};
struct Prepared {
    float* main[4]; float* mean[4];
    float* bf_cat;                                   // [D, 2 KN] = [W_up | W_dn]
    float* sp_alpha;                                 // [2][N][KN] softplus(alpha_up), softplus(alpha_dn)
    __nv_bfloat16* main_bf[2][4]; __nv_bfloat16* mean_bf[2][4]; __nv_bfloat16* map_bf[2][4];
    __nv_bfloat16* bf_bf[2]; __nv_bfloat16* jas0[2]; __nv_bfloat16* jas1[2];
    size_t bytes;
};
static inline int tc_parts(int precision) {
    return (precision == DW_PRECISION_MIXED || precision == DW_PRECISION_MIXED_DET64) ? 2
                                                                                      : (precision == DW_PRECISION_BF16 ? 1 : 0);
}
static inline int mean_width(const Dims& d, int l) { return round_up(2 * d.hw[l], 64); }

static Prepared carve_prepared(const DwArch* a, int precision, void* base) {
    Dims d = make_dims(a, false);
    Carver c(base, (size_t)-1);
    Prepared p;
    memset(&p, 0, sizeof(p));
    for (int l = 0; l < 4; ++l) {
        p.main[l] = c.take<float>((size_t)d.kw[l] * d.D);
        p.mean[l] = c.take<float>((size_t)mean_width(d, l) * d.D);
    }
    p.bf_cat = c.take<float>((size_t)d.D * 2 * d.KN);
    p.sp_alpha = c.take<float>((size_t)2 * d.N * d.KN);
    for (int part = 0; part < tc_parts(precision); ++part) {
        for (int l = 0; l < 4; ++l) {
            p.main_bf[part][l] = c.take<__nv_bfloat16>((size_t)d.kw[l] * d.D);
            p.mean_bf[part][l] = c.take<__nv_bfloat16>((size_t)mean_width(d, l) * d.D);
            p.map_bf[part][l] = c.take<__nv_bfloat16>((size_t)round_up(d.hw[l], 64) * d.E);
        }
        p.bf_bf[part] = c.take<__nv_bfloat16>((size_t)d.D * round_up(2 * d.KN, 16));
        p.jas0[part] = c.take<__nv_bfloat16>((size_t)d.D * d.J0);
        p.jas1[part] = c.take<__nv_bfloat16>((size_t)d.J0 * d.J1);
    }
    p.bytes = c.used;
    return p;
}

// softplus of the envelope exponents (parameters only, computed once per parameter update)
__global__ void k_softplus(const float* __restrict__ a_up, const float* __restrict__ a_dn, int n, float* __restrict__ out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 2 * n) return;
    out[idx] = softplus_f(idx < n ? a_up[idx] : a_dn[idx - n]);
}

// Row gather for the prepared FP32 layer weights: mode 0 builds Wmain (rows h, conv_ee,
// conv_ei of h_el_l.w), mode 1 builds Wmean (rows mean_up, mean_dn); other rows are zero.
__global__ void k_gather_rows(const float* __restrict__ src, int cols, int rows, int hw, int nconv, int mode,
                              float* __restrict__ dst) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)rows * cols) return;
    int r = idx / cols, c = idx % cols;
    int sr;
    if (mode == 0) sr = r < hw ? r : (r < hw + nconv ? 2 * hw + r : -1);
    else sr = r < 2 * hw ? hw + r : -1;
    dst[idx] = sr >= 0 ? src[(int64_t)sr * cols + c] : 0.f;
}
// dstT[c][r] = bf16 part of src[r][c] (part 0: hi = bf16(x), part 1: lo = bf16(x - hi)) for
// r < rows_src; zero for rows_src <= r < rows_pad and c >= cols (padding).
__global__ void k_transpose_bf16(const float* __restrict__ src, int rows_src, int rows_pad, int cols, int cols_pad,
                                 int part, __nv_bfloat16* __restrict__ dst) {
    int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)rows_pad * cols_pad) return;
    int c = idx / rows_pad, r = idx % rows_pad;
    float v = (r < rows_src && c < cols) ? src[(int64_t)r * cols + c] : 0.f;
    __nv_bfloat16 hi = __float2bfloat16_rn(v);
    dst[idx] = part == 0 ? hi : __float2bfloat16_rn(v - __bfloat162float(hi));
}

static int prepare(const DwArch* a, int precision, const float* P, void* prep, size_t bytes, cudaStream_t s) {
    Dims d = make_dims(a, false);
    ParamLayout L;
    make_layout(a, &L);
    Prepared p = carve_prepared(a, precision, prep);
    if (p.bytes > bytes) return DW_ERR_WORKSPACE;
    for (int l = 0; l < 4; ++l) {
        for (int which = 0; which < 2; ++which) {
            int rows = which == 0 ? d.kw[l] : mean_width(d, l);
            float* dst = which == 0 ? p.main[l] : p.mean[l];
            int64_t n = (int64_t)rows * d.D;
            k_gather_rows<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(P + L.h_el_w[l], d.D, rows, d.hw[l],
                                                                     d.E + d.eiw[l], which, dst);
            count_launch();
        }
    }
    k_softplus<<<(2 * d.N * d.KN + 255) / 256, 256, 0, s>>>(P + L.alpha_up, P + L.alpha_dn, d.N * d.KN, p.sp_alpha);
    count_launch();
    for (int half = 0; half < 2; ++half) {
        DW_CHECK_CUDA(cudaMemcpy2DAsync(p.bf_cat + half * d.KN, sizeof(float) * 2 * d.KN,
                                        P + (half == 0 ? L.bf_up : L.bf_dn), sizeof(float) * d.KN,
                                        sizeof(float) * d.KN, d.D, cudaMemcpyDeviceToDevice, s));
    }
    for (int part = 0; part < tc_parts(precision); ++part) {
        auto tr = [&](const float* src, int rows_src, int rows_pad, int cols, int cols_pad, __nv_bfloat16* dst) {
            int64_t n = (int64_t)rows_pad * cols_pad;
            k_transpose_bf16<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, rows_src, rows_pad, cols, cols_pad, part, dst);
            count_launch();
        };
        for (int l = 0; l < 4; ++l) {
            tr(p.main[l], d.kw[l], d.kw[l], d.D, d.D, p.main_bf[part][l]);
            tr(p.mean[l], mean_width(d, l), mean_width(d, l), d.D, d.D, p.mean_bf[part][l]);
            tr(P + L.h_map_w[l], d.hw[l], round_up(d.hw[l], 64), d.E, d.E, p.map_bf[part][l]);
        }
        tr(p.bf_cat, d.D, d.D, 2 * d.KN, round_up(2 * d.KN, 16), p.bf_bf[part]);
        tr(P + L.jas_w[0], d.D, d.D, d.J0, d.J0, p.jas0[part]);
        tr(P + L.jas_w[1], d.J0, d.J0, d.J1, d.J1, p.jas1[part]);
    }
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

// ------------------------------------------------------------------ forward plan
template <class Act>
struct Plan {
    Dims d;
    int Bc;             // walkers per chunk
    int rows;           // Bc * n * Tp
    float* him;
    Act* X0; Act* XA; Act* XB;
    Act* Mcat; float* WB; float* HM; float* Zb;
    float* WP; float* HE;
    float* BF; float* MO;
    double* logdet; double* sign; float* Ainv; double* g; double* lapdet;
    Act* J1; Act* J2; double* jas;
    size_t bytes;
};

static const int kXW = 320;   // row width of the layer-1..3 inputs: 256 (h) + 32 (conv_ee) + 32 (conv_ei)

template <class Act>
static Plan<Act> carve_plan(const Dims& d, int Bc, void* ws) {
    Carver c(ws, (size_t)-1);
    const int64_t np = ActIO<Act>::kParts;
    Plan<Act> p;
    p.d = d; p.Bc = Bc;
    int64_t rows = (int64_t)Bc * d.n * d.Tp;
    p.rows = (int)rows;
    int mw = 0;
    for (int l = 0; l < 4; ++l) mw = std::max(mw, mean_width(d, l));
    int zw = std::max(std::max(d.D, d.J0), d.KN);
    p.him = c.take<float>((size_t)kMaxSeg * 4 * d.N * 32);   // [segment][iteration][ion][32]
    p.X0 = c.take<Act>(np * rows * d.kw[0]);
    p.XA = c.take<Act>(np * rows * kXW);
    p.XB = c.take<Act>(np * rows * kXW);
    p.Mcat = c.take<Act>(np * Bc * d.Tp * mw);
    p.WB = c.take<float>((int64_t)Bc * d.Tp * d.D);
    p.HM = c.take<float>(rows * d.E);
    p.Zb = std::is_same<Act, float>::value ? c.take<float>(rows * std::max(d.D, d.J0)) : nullptr;
    int pc = d.Tp > 1 ? 3 : 1, ec = d.Tp > 1 ? 5 : 1;
    p.WP = c.take<float>((int64_t)4 * Bc * d.n * d.n * pc * 32);
    p.HE = c.take<float>((int64_t)4 * Bc * d.n * d.N * ec * 32);
    p.BF = c.take<float>(rows * round_up(2 * d.KN, 4));   // row pitch padded to 16 bytes (TMA stores)
    p.MO = c.take<float>((int64_t)Bc * d.K * d.T * d.n * d.n);
    p.logdet = c.take<double>((int64_t)Bc * d.K);
    p.sign = c.take<double>((int64_t)Bc * d.K);
    if (d.Tp > 1) {
        p.Ainv = c.take<float>((int64_t)Bc * d.K * d.n * d.n);
        p.g = c.take<double>((int64_t)Bc * d.K * 3 * d.n);
        p.lapdet = c.take<double>((int64_t)Bc * d.K);
    } else {
        p.Ainv = nullptr; p.g = nullptr; p.lapdet = nullptr;
    }
    p.J1 = c.take<Act>(np * rows * d.J0);
    p.J2 = c.take<Act>(np * rows * d.J1);
    p.jas = c.take<double>((int64_t)Bc * d.Tp);
    (void)zw;
    p.bytes = c.used;
    return p;
}

static const size_t kChunkBudget = (size_t)6 << 30;   // bytes of activations per walker chunk

// Walkers per chunk: the marginal workspace of one walker (the plan also holds fixed buffers,
// such as the per-geometry ion maps, that do not grow with the chunk) against the budget.
template <class Act>
static int choose_chunk(const Dims& d, int B, size_t budget = kChunkBudget) {
    const size_t one = carve_plan<Act>(d, 1, nullptr).bytes, two = carve_plan<Act>(d, 2, nullptr).bytes;
    const size_t per = std::max<size_t>(two > one ? two - one : one, 1);
    const size_t fixed = one > per ? one - per : 0;
    const size_t avail = budget > fixed ? budget - fixed : per;
    int bc = std::min((int)std::max<size_t>(1, avail / per), B);
    // buffers below the 256-byte carve granularity grow unseen in the two-walker estimate
    while (bc > 1 && carve_plan<Act>(d, bc, nullptr).bytes > budget) bc -= std::max(1, bc / 32);
    return bc;
}

// ------------------------------------------------------------------ GEMM dispatch by activation type
// mm:      C (fp32) = A W + epilogue
// mm_act:  C (Act)  = act(A W + epilogue)            (value-only layers)
// mm_bat:  batched over walkers, no epilogue
template <class Act> struct MM;
template <> struct MM<float> {
    static int mm(const float* A, int lda, const WRef& W, float* C, int ldc, int M, int N, int K, const GemmEpi& e,
                  cudaStream_t s) {
        gemm_f32(A, lda, W.f32, W.ldw, C, ldc, M, N, K, e, 1, 0, 0, s);
        return DW_OK;
    }
    template <class Out>
    static int mm_fl(const float* A, int lda, const WRef& W, Out* C, int ldc, int M, int N, int K, const GemmEpi& e,
                     const Dims& d, float* Zb, cudaStream_t s) {
        gemm_f32(A, lda, W.f32, W.ldw, Zb, N, M, N, K, e, 1, 0, 0, s);
        launch_tanh_fl<Out>(Zb, N, N, M / d.Tp, d, C, ldc, s);
        return DW_OK;
    }
};
template <class Act> struct MMTC {
    static constexpr int np = ActIO<Act>::kParts;
    static constexpr int out_act = np == 2 ? 2 : 1;
    static int mm(const Act* A, int lda, const WRef& W, float* C, int ldc, int M, int N, int K, const GemmEpi& e,
                  cudaStream_t s) {
        return gemm_tc(np, 0, A, lda, W.hi, W.lo, C, ldc, M, N, K, e, 0, 0, s);
    }
    static int mm(const Act* A, int lda, const WRef& W, Act* C, int ldc, int M, int N, int K, const GemmEpi& e,
                  cudaStream_t s) {
        return gemm_tc(np, out_act, A, lda, W.hi, W.lo, C, ldc, M, N, K, e, 0, 0, s);
    }
    static int mm_fl(const Act* A, int lda, const WRef& W, float* C, int ldc, int M, int N, int K, const GemmEpi& e,
                     const Dims& d, float*, cudaStream_t s) {
        return gemm_tc(np, 0, A, lda, W.hi, W.lo, C, ldc, M, N, K, e, 1, 3 * d.n, s);
    }
    static int mm_fl(const Act* A, int lda, const WRef& W, Act* C, int ldc, int M, int N, int K, const GemmEpi& e,
                     const Dims& d, float*, cudaStream_t s) {
        return gemm_tc(np, out_act, A, lda, W.hi, W.lo, C, ldc, M, N, K, e, 1, 3 * d.n, s);
    }
};
template <> struct MM<__nv_bfloat16> : MMTC<__nv_bfloat16> {};
template <> struct MM<Split> : MMTC<Split> {};

// Runs `stmt` between per-tag timer events (no-ops unless dw_timer_enable(1)).
#define DW_TIMED(tag, stmt) do { timer_begin(tag, s); stmt; timer_end(tag, s, 0.0, 0.0); } while (0)

// Element offset of row `row` in a logical-width-ld activation buffer of type Act.
template <class Act> static inline int64_t act_off(int64_t row, int ld) { return row * ld * ActIO<Act>::kParts; }

// The forward (value or tangent) of one chunk of walkers.
template <class Act>
static int run_chunk(const Plan<Act>& p, int Bc, int precision, const float* P, const ParamLayout& L,
                     const Prepared& pre, const float* r, const float* R, const int32_t* Z, const int32_t* seg,
                     float* lp, float* phase, float* E_loc, float* grad, cudaStream_t s, float* esc = nullptr) {
    Dims d = p.d;
    d.seg = seg;          // walker -> geometry segment of this chunk (null: one geometry)
    const int rows = Bc * d.n * d.Tp;
    const bool tang = d.Tp > 1;
    const int pt = tc_parts(precision);
    auto wref = [&](const float* f32, int ldw, __nv_bfloat16* const* bf, int l) {
        WRef w; w.f32 = f32; w.ldw = ldw;
        if (pt >= 1) w.hi = bf[0 * 4 + l];
        if (pt >= 2) w.lo = bf[1 * 4 + l];
        return w;
    };
    auto wref1 = [&](const float* f32, int ldw, __nv_bfloat16* const* bf) {
        WRef w; w.f32 = f32; w.ldw = ldw;
        if (pt >= 1) w.hi = bf[0];
        if (pt >= 2) w.lo = bf[1];
        return w;
    };
    DW_TIMED("features", launch_features<Act>(r, R, Z, d, Bc, p.X0, s));
    // el-ion stream reduced over the ions inside the stream kernel where possible (conv_ei per
    // electron and level in the HE buffer instead of the full stream)
    const bool ei_fused = ei_fusable(d);
    DW_TIMED("streams", launch_streams(r, R, Z, P, L, d, Bc, p.WP, p.HE, s, nullptr, ei_fused ? p.him : nullptr));
    Act* xin = p.X0;
    int ldin = d.kw[0];
    int pc = tang ? 3 : 1, ec = tang ? 5 : 1;
    for (int l = 0; l < 4; ++l) {
        Act* xout = (l % 2 == 0) ? p.XA : p.XB;
        int hw = d.hw[l], mw = mean_width(d, l);
        // (a) spin means and their per-walker contribution (+ the layer bias on the value channel)
        DW_TIMED("spin_means", launch_spin_means<Act>(xin, ldin, hw, d, Bc, p.Mcat, mw, s));
        GemmEpi e1; e1.bias = P + L.h_el_b[l]; e1.Tp = d.Tp; e1.rows_per_walker = d.Tp;
        DW_TIMED("mean_gemm", DW_CHECK(MM<Act>::mm(p.Mcat, mw, wref(pre.mean[l], d.D, &pre.mean_bf[0][0], l), p.WB, d.D,
                                                   Bc * d.Tp, d.D, mw, e1, s)));
        // (b) h_map = tanh(h_one W + b)
        GemmEpi e2; e2.bias = P + L.h_map_b[l]; e2.Tp = d.Tp; e2.rows_per_walker = d.n * d.Tp; e2.act = tang ? 0 : 1;
        WRef wmap = wref(P + L.h_map_w[l], d.E, &pre.map_bf[0][0], l);
        if (tang) DW_TIMED("map_gemm", DW_CHECK(MM<Act>::mm_fl(xin, ldin, wmap, p.HM, d.E, rows, d.E, hw, e2, d, p.Zb, s)));
        else DW_TIMED("map_gemm", DW_CHECK(MM<Act>::mm(xin, ldin, wmap, p.HM, d.E, rows, d.E, hw, e2, s)));
        // (c) SchNet convolutions into the input columns [hw, hw + E + eiw)
        int64_t wp_plane = (int64_t)Bc * d.n * d.n * pc * 32;
        int64_t he_plane = ei_fused ? (int64_t)Bc * d.n * ec * 32 : (int64_t)Bc * d.n * d.N * ec * 32;
        DW_TIMED("conv", launch_conv<Act>(r, p.WP + l * wp_plane, p.HM, p.HE + l * he_plane, p.him + l * d.N * 32, d, l,
                                          Bc, xin, ldin, s, ei_fused ? 1 : 0));
        // (d) h_el = tanh([h | conv_ee | conv_ei] W_main + per-walker mean term)
        GemmEpi e3; e3.rowbias = p.WB; e3.ldrb = d.D; e3.Tp = d.Tp; e3.rows_per_walker = d.n * d.Tp; e3.act = tang ? 0 : 1;
        WRef wm = wref(pre.main[l], d.D, &pre.main_bf[0][0], l);
        if (tang) {
            // algorithmic work of this launch: 2 M N K over the T = 3n + 2 channel rows of each
            // electron (not the Tp - T zero padding rows the launch also moves) and the unpadded K,
            // A and C streamed once
            const double kreal = hw + d.E + d.eiw[l];
            const double rows_alg = (double)Bc * d.n * d.T;
            const double flops = 2.0 * rows_alg * d.D * kreal;
            const double esz = (double)sizeof(Act) * ActIO<Act>::kParts;
            const double bytes = rows_alg * (kreal + d.D) * esz + kreal * d.D * esz;
            // the tail re-evaluation's FP32 layers are timed apart from the production form's
            const char* tag = det64_form(precision) ? "guard_layer_gemm" : "layer_gemm";
            timer_begin(tag, s);
            DW_CHECK(MM<Act>::mm_fl(xin, ldin, wm, xout, kXW, rows, d.D, d.kw[l], e3, d, p.Zb, s));
            timer_end(tag, s, flops, bytes);
        } else {
            DW_TIMED("layer_gemm_value", DW_CHECK(MM<Act>::mm(xin, ldin, wm, xout, kXW, rows, d.D, d.kw[l], e3, s)));
        }
        xin = xout;
        ldin = kXW;
    }
    const Act* H = xin;   // final embedding, logical row width kXW
    // backflow (envelope_orbitals.py:46-75). Tensor-core tangent passes: one GEMM per spin over
    // that spin's electron rows of every walker (walker-block tensor maps), so each row gets only
    // its own spin's KN columns. Otherwise every row times [W_up | W_dn] and the envelope kernel
    // takes the half that matches the electron's spin.
    int ldbf = round_up(2 * d.KN, 4), spin_cols = d.KN;
    const bool per_spin = tang && pt >= 1 && (d.nu * d.Tp) % 32 == 0 && (d.nd * d.Tp) % 32 == 0 && d.KN % 4 == 0;
    if (per_spin) {
        ldbf = d.KN;
        spin_cols = 0;
        timer_begin("backflow_gemm", s);
        for (int spin = 0; spin < 2; ++spin) {
            const int i0 = spin == 0 ? 0 : d.nu, ns = spin == 0 ? d.nu : d.nd;
            WalkerBlocks wb;
            wb.nw = Bc;
            wb.rows = ns * d.Tp;
            wb.a_wstride = (int64_t)d.n * d.Tp * kXW * ActIO<Act>::kParts;
            wb.c_wstride = (int64_t)d.n * d.Tp * d.KN;
            const int64_t wrow = (int64_t)spin * d.KN * d.D;           // W_up / W_dn rows of the K-major copy
            DW_CHECK(gemm_tc_wb(pt, H + act_off<Act>((int64_t)i0 * d.Tp, kXW), kXW, pre.bf_bf[0] + wrow,
                                pt >= 2 ? pre.bf_bf[1] + wrow : nullptr, p.BF + (int64_t)i0 * d.Tp * d.KN, d.KN, wb,
                                d.KN, d.D, s));
        }
        timer_end("backflow_gemm", s, 0.0, 0.0);
    } else {
        GemmEpi e0; e0.Tp = d.Tp; e0.rows_per_walker = d.n * d.Tp;
        WRef wb; wb.f32 = pre.bf_cat; wb.ldw = 2 * d.KN;
        if (pt >= 1) wb.hi = pre.bf_bf[0];
        if (pt >= 2) wb.lo = pre.bf_bf[1];
        DW_TIMED("backflow_gemm", DW_CHECK(MM<Act>::mm(H, kXW, wb, p.BF, ldbf, rows, 2 * d.KN, d.D, e0, s)));
    }
    DW_TIMED("envelope", launch_envelope(r, R, Z, P, L, pre.sp_alpha, d, Bc, p.BF, ldbf, spin_cols, p.MO, s));
    if (det64_form(precision) && tang) {
        // FP64 LU, inverse and tangent traces of the FP32 Slater channels; the widened channels use
        // the backflow buffer (consumed by the envelope kernel, at least twice the Slater channels'
        // size) and the inverses the layer buffer XA (the embedding H is in XB)
        DW_TIMED("det_tangents", DW_CHECK(fp64_dets_from_f32(p.MO, d, Bc, reinterpret_cast<double*>(p.BF),
                                                             reinterpret_cast<double*>(p.XA), p.logdet, p.sign, p.g,
                                                             p.lapdet, s)));
    } else {
        if (precision == DW_PRECISION_FP32) DW_TIMED("slogdet", launch_slogdet<float>(p.MO, d, Bc, p.logdet, p.sign, p.Ainv, s));
        else DW_TIMED("slogdet", launch_slogdet<double>(p.MO, d, Bc, p.logdet, p.sign, p.Ainv, s));
        if (tang) DW_TIMED("det_tangents", launch_det_tangents(p.MO, p.Ainv, p.sign, d, Bc, p.g, p.lapdet, s));
    }
    // Jastrow MLP([64, 64, 1]) on the final embedding
    GemmEpi j0; j0.bias = P + L.jas_b[0]; j0.Tp = d.Tp; j0.rows_per_walker = d.n * d.Tp; j0.act = tang ? 0 : 1;
    GemmEpi j1 = j0; j1.bias = P + L.jas_b[1];
    WRef wj0 = wref1(P + L.jas_w[0], d.J0, pre.jas0), wj1 = wref1(P + L.jas_w[1], d.J1, pre.jas1);
    timer_begin("jastrow", s);
    if (tang) {
        DW_CHECK(MM<Act>::mm_fl(H, kXW, wj0, p.J1, d.J0, rows, d.J0, d.D, j0, d, p.Zb, s));
        DW_CHECK(MM<Act>::mm_fl(p.J1, d.J0, wj1, p.J2, d.J1, rows, d.J1, d.J0, j1, d, p.Zb, s));
    } else {
        DW_CHECK(MM<Act>::mm(H, kXW, wj0, p.J1, d.J0, rows, d.J0, d.D, j0, s));
        DW_CHECK(MM<Act>::mm(p.J1, d.J0, wj1, p.J2, d.J1, rows, d.J1, d.J0, j1, s));
    }
    launch_jastrow_out<Act>(p.J2, d.J1, P + L.jas_w[2], d, Bc, p.jas, s);
    timer_end("jastrow", s, 0.0, 0.0);
    DW_TIMED("combine", launch_combine(p.logdet, p.sign, p.g, p.lapdet, p.jas, r, R, Z, d, Bc, lp, phase, E_loc, grad, s,
                                       0, nullptr, esc));
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

// Calls f(tag) with a null pointer of the activation type of the precision form (double: the FP64
// form of fp64.cu).
template <class F>
static int with_act(int precision, bool need_device, F&& f) {
    switch (precision) {
        case DW_PRECISION_FP32: return f((float*)nullptr);
        case DW_PRECISION_FP32_DET64: return f((float*)nullptr);
        case DW_PRECISION_FP64: return f((double*)nullptr);
        case DW_PRECISION_MIXED:
        case DW_PRECISION_MIXED_DET64:
            if (need_device && !tc_available()) return DW_ERR_UNSUPPORTED;
            return f((Split*)nullptr);
        case DW_PRECISION_BF16:
            if (need_device && !tc_available()) return DW_ERR_UNSUPPORTED;
            return f((__nv_bfloat16*)nullptr);
        default: return DW_ERR_ARG;
    }
}
template <class T> using act_of = typename std::remove_pointer<T>::type;

template <class Act>
static size_t plan_bytes(const DwArch* a, int B, bool tang, size_t budget = kChunkBudget) {
    Dims d = make_dims(a, tang);
    return (carve_plan<Act>(d, choose_chunk<Act>(d, std::max(B, 1), budget), nullptr).bytes + 4096 + 255) / 256 * 256;
}

// Mixed-form local energies: the forward's plan (or the tail re-evaluation, which reuses that
// region once the forward is done) followed by the per-walker error scales.
static size_t guarded_bytes(const DwArch* a, int B, size_t plan) {
    return (std::max(plan, guard_bytes(a, B)) + 255) / 256 * 256 + (size_t)3 * B * sizeof(float) + 256;
}

// Workspace of one forward (value or tangent) and the forward itself, for every precision form.
template <class Act>
static size_t plan_bytes_any(const DwArch* a, int B, bool tang) {
    if constexpr (std::is_same<Act, double>::value) return fp64_plan_bytes(a, B, tang);
    else return plan_bytes<Act>(a, B, tang);
}

template <class Act>
static size_t ws_bytes_t(const DwArch* a, int n_walkers, int mode) {
    if (mode == 3) return bwd_bytes(a, n_walkers, nullptr);
    if (mode == 2) {
        size_t b = plan_bytes_any<Act>(a, n_walkers, false);
        b += (size_t)n_walkers * a->n_el * 3 * sizeof(float) + 256;      // proposals
        b += (size_t)n_walkers * sizeof(float) + 256;                    // proposal log psi^2
        b += (size_t)n_walkers * sizeof(float) + 256;                    // log proposal ratios
        b += (size_t)mh_counts_needed(kMaxSeg) * sizeof(int) + 256;
        return b;
    }
    size_t b = plan_bytes_any<Act>(a, n_walkers, mode == 1);
    if (mode == 1 && std::is_same<Act, Split>::value) b = guarded_bytes(a, n_walkers, b);
    if (mode == 1) b += (size_t)n_walkers * sizeof(float) + 256;         // log psi^2 when not requested
    return b;
}

template <class Act>
static int forward_all(const DwArch* a, int precision, const float* P, const void* prepared, const float* r, int B,
                       const float* R, const int32_t* Z, float* lp, float* phase, float* E, float* grad, bool tang,
                       void* ws, size_t ws_bytes, cudaStream_t s, const int32_t* seg = nullptr, int nseg = 1,
                       size_t budget = kChunkBudget, float* esc = nullptr) {
    Dims d = make_dims(a, tang);
    if (nseg < 1 || nseg > kMaxSeg || (nseg > 1 && !seg)) return DW_ERR_ARG;
    // the fused forward-Laplacian epilogue keeps one electron's channels inside a 128-row tile
    if (tang && !std::is_same<Act, float>::value && d.Tp > 128) return DW_ERR_ARCH;
    ParamLayout L;
    make_layout(a, &L);
    Prepared pre = carve_prepared(a, precision, const_cast<void*>(prepared));
    int bc = choose_chunk<Act>(d, B, budget);
    Plan<Act> p = carve_plan<Act>(d, bc, ws);
    if (p.bytes > ws_bytes) return DW_ERR_WORKSPACE;
    d.nseg = nseg;
    p.d.nseg = nseg;      // the chunks index geometries through the plan's dims
    launch_ion_maps(P, L, d, Z, p.him, s);
    for (int b0 = 0; b0 < B; b0 += bc) {
        int nb = std::min(bc, B - b0);
        DW_CHECK(run_chunk<Act>(p, nb, precision, P, L, pre, r + (int64_t)b0 * d.n * 3, R, Z, seg ? seg + b0 : nullptr,
                                lp + b0,
                                phase ? phase + b0 : nullptr, E ? E + b0 : nullptr,
                                grad ? grad + (int64_t)b0 * 3 * d.n : nullptr, s, esc ? esc + 3 * (int64_t)b0 : nullptr));
    }
    return DW_OK;
}

template <class Act>
static int forward_any(const DwArch* a, int precision, const float* P, const void* prepared, const float* r, int B,
                       const float* R, const int32_t* Z, float* lp, float* phase, float* E, float* grad, bool tang,
                       void* ws, size_t ws_bytes, cudaStream_t s, const int32_t* seg = nullptr, int nseg = 1) {
    if constexpr (std::is_same<Act, double>::value)
        return fp64_forward_all(a, P, prepared, r, B, R, Z, lp, phase, E, grad, tang, ws, ws_bytes, s, seg, nseg, nullptr);
    else
        return forward_all<Act>(a, precision, P, prepared, r, B, R, Z, lp, phase, E, grad, tang, ws, ws_bytes, s, seg, nseg);
}

// Local energies of one or several geometries. Workspace: [forward plan | log psi^2 when not
// requested], and for the mixed form [plan or tail re-evaluation | log psi^2 | error scales]: the
// mixed form's walkers whose predicted E_L error exceeds the tolerance are re-evaluated in FP64
// (guard.cu).
static int local_energy_impl(const DwArch* a, int precision, const float* params, const void* prepared, const float* r,
                             int B, const float* R, const int32_t* Z, const int32_t* seg, int nseg, float* E, float* lp,
                             float* grad, void* ws, size_t wsb, cudaStream_t s) {
    return with_act(precision, true, [&](auto tag) {
        using Act = act_of<decltype(tag)>;
        const size_t pb = plan_bytes_any<Act>(a, B, true);
        const bool guarded = std::is_same<Act, Split>::value && precision == DW_PRECISION_MIXED;
        const size_t region = guarded ? (std::max(pb, guard_bytes(a, B)) + 255) / 256 * 256 : pb;
        char* tail = static_cast<char*>(ws) + region;
        float* lpo = lp;
        if (!lpo) {   // log psi^2 output is optional; it then lives after the plan
            lpo = reinterpret_cast<float*>(tail);
            tail += ((size_t)B * sizeof(float) + 255) / 256 * 256;
        }
        float* esc = guarded ? reinterpret_cast<float*>(tail) : nullptr;
        if (guarded) tail += (size_t)3 * B * sizeof(float);
        if ((size_t)(tail - static_cast<char*>(ws)) > wsb) return (int)DW_ERR_WORKSPACE;
        if constexpr (std::is_same<Act, double>::value) {
            return fp64_forward_all(a, params, prepared, r, B, R, Z, lpo, nullptr, E, grad, true, ws, region, s, seg, nseg,
                                    nullptr);
        } else {
            DW_CHECK(forward_all<Act>(a, precision, params, prepared, r, B, R, Z, lpo, nullptr, E, grad, true, ws, region,
                                      s, seg, nseg, kChunkBudget, esc));
            if (!guarded) return (int)DW_OK;
            timer_begin("guard", s);
            const int st = tail_guard(a, params, prepared, r, B, R, Z, seg, nseg, esc, E, lpo, grad, ws, region, s);
            timer_end("guard", s, 0.0, 0.0);
            return st;
        }
    });
}

// Local energy with FP64 determinant algebra on a caller region (DW_PRECISION_FP32_DET64: plain
// FP32 network, DW_PRECISION_MIXED_DET64: split-BF16 network): the mixed form's re-evaluation of
// flagged walkers (guard.cu).
size_t det64_plan_bytes(const DwArch* a, int precision, int B) {
    return precision == DW_PRECISION_MIXED_DET64 ? plan_bytes<Split>(a, B, true) : plan_bytes<float>(a, B, true);
}
int det64_local_energy(const DwArch* a, int precision, const float* P, const void* prepared, const float* r, int B,
                       const float* R, const int32_t* Z, const int32_t* seg, int nseg, float* E, float* lp, float* grad,
                       void* ws, size_t wsb, cudaStream_t s) {
    if (precision == DW_PRECISION_MIXED_DET64)
        return forward_all<Split>(a, precision, P, prepared, r, B, R, Z, lp, nullptr, E, grad, true, ws, wsb, s, seg,
                                  nseg);
    return forward_all<float>(a, DW_PRECISION_FP32_DET64, P, prepared, r, B, R, Z, lp, nullptr, E, grad, true, ws, wsb,
                              s, seg, nseg);
}

// FP32 row-gathered layer weights of a prepared buffer (the same offsets in every precision form).
void prepared_fp32_layers(const DwArch* a, const void* prepared, const float* main[4], const float* mean[4]) {
    Prepared p = carve_prepared(a, DW_PRECISION_FP32, const_cast<void*>(prepared));
    for (int l = 0; l < 4; ++l) { main[l] = p.main[l]; mean[l] = p.mean[l]; }
}

// Value-only forward for the workspace-free entry point (noalloc.cu): bytes of scratch it needs
// and the call itself on a caller-supplied scratch region.
// Scratch bytes and call of the value-only forward with walker chunks sized against `budget`
// bytes (the workspace-free entry point passes its fixed array, so a large batch runs in several
// chunks instead of being refused). The FP64 form is not offered there.
size_t value_forward_bytes(const DwArch* a, int precision, int B, size_t budget) {
    size_t out = 0;
    with_act(precision, false, [&](auto tag) {
        using Act = act_of<decltype(tag)>;
        if constexpr (!std::is_same<Act, double>::value) out = plan_bytes<Act>(a, B, false, budget);
        return 0;
    });
    return out;
}
int value_forward(const DwArch* a, int precision, const float* params, const void* prepared, const float* r, int B,
                  const float* R, const int32_t* Z, float* lp, float* phase, void* ws, size_t wsb, size_t budget,
                  cudaStream_t s) {
    return with_act(precision, true, [&](auto tag) {
        using Act = act_of<decltype(tag)>;
        if constexpr (std::is_same<Act, double>::value) return (int)DW_ERR_ARG;
        else return forward_all<Act>(a, precision, params, prepared, r, B, R, Z, lp, phase, nullptr, nullptr, false, ws,
                                     wsb, s, nullptr, 1, budget);
    });
}

}  // namespace dw

using namespace dw;

extern "C" {

size_t dw_prepared_bytes(const DwArch* a, int precision) {
    if (check_arch(a) != DW_OK) return 0;
    return carve_prepared(a, precision, nullptr).bytes + 256;
}

int dw_prepare_params(const DwArch* a, int precision, const float* params, void* prepared, size_t bytes, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared) return DW_ERR_ARG;
    if (precision < DW_PRECISION_FP32 || precision > DW_PRECISION_MIXED_DET64) return DW_ERR_ARG;
    return prepare(a, precision, params, prepared, bytes, (cudaStream_t)stream);
}

size_t dw_workspace_bytes(const DwArch* a, int precision, int n_walkers, int mode) {
    if (check_arch(a) != DW_OK || n_walkers <= 0) return 0;
    size_t out = 0;
    with_act(precision, false, [&](auto tag) { out = ws_bytes_t<act_of<decltype(tag)>>(a, n_walkers, mode); return 0; });
    return out;
}

int dw_log_psi_sqr(const DwArch* a, int precision, const float* params, const void* prepared, const float* r,
                   int B, const float* R, const int32_t* Z, float* lp, float* phase, void* ws, size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared || !r || !R || !Z || !lp || B <= 0) return DW_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    return with_act(precision, true, [&](auto tag) {
        using Act = act_of<decltype(tag)>;
        return forward_any<Act>(a, precision, params, prepared, r, B, R, Z, lp, phase, nullptr, nullptr, false, ws, wsb, s);
    });
}

int dw_local_energy(const DwArch* a, int precision, const float* params, const void* prepared, const float* r, int B,
                    const float* R, const int32_t* Z, float* E, float* lp, float* grad, void* ws, size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared || !r || !R || !Z || !E || B <= 0) return DW_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    return local_energy_impl(a, precision, params, prepared, r, B, R, Z, nullptr, 1, E, lp, grad, ws, wsb, s);
}

int dw_potential_energy(const float* r, int B, int n, const float* R, const int32_t* Z, int N, float* E, void* stream) {
    reset_launch_count();
    if (!r || !R || !Z || !E || B <= 0 || n <= 0 || N <= 0) return DW_ERR_ARG;
    launch_coulomb(r, B, n, R, Z, N, E, (cudaStream_t)stream);
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

}  // extern "C"

namespace dw {

// Proposal rule and its parameters within their domains.
static bool mcmc_config_ok(const DwMcmcConfig* c) {
    if (c->proposal < DW_PROPOSAL_NORMAL || c->proposal > DW_PROPOSAL_LOCAL_ONE_EL) return false;
    const bool local = c->proposal == DW_PROPOSAL_LANGEVIN || c->proposal == DW_PROPOSAL_LOCAL ||
                       c->proposal == DW_PROPOSAL_LOCAL_ONE_EL;
    if (local && !(c->r_min > 0.f && c->r_max >= c->r_min)) return false;
    return c->p_spin_swap >= 0.f && c->p_spin_swap <= 1.f && c->p_spin_flip >= 0.f && c->p_spin_flip <= 1.f;
}

// Metropolis-Hastings chains (mcmc.py:390-396 run_mcmc_steps): optional re-evaluation of log psi^2
// at the current walkers, then n_steps x (forward at the proposals, accept / propose).
static int mcmc_impl(const DwArch* a, int precision, const float* params, const void* prepared, float* r, int B,
                     const float* R, const int32_t* Z, int nseg, const int32_t* seg, const int32_t* widx,
                     const uint64_t* seeds, float* lp, int32_t* age, DwMcmcScalars* scalars, const DwMcmcConfig* cfg,
                     void* ws, size_t wsb, cudaStream_t s) {
    return with_act(precision, true, [&](auto tag) {
        using Act = act_of<decltype(tag)>;
        if (wsb < ws_bytes_t<Act>(a, B, 2)) return (int)DW_ERR_WORKSPACE;
        size_t fwd = plan_bytes_any<Act>(a, B, false);
        Carver c(static_cast<char*>(ws) + fwd, wsb - fwd);
        float* r_prop = c.take<float>((size_t)B * a->n_el * 3);
        float* lp_prop = c.take<float>((size_t)B);
        float* lq = c.take<float>((size_t)B);
        int* counts = c.take<int>((size_t)mh_counts_needed(kMaxSeg));
        if (!c.ok()) return (int)DW_ERR_WORKSPACE;
        auto fwd_call = [&](const float* rr, float* out) {
            return forward_any<Act>(a, precision, params, prepared, rr, B, R, Z, out, nullptr, nullptr, nullptr, false,
                                    ws, fwd, s, seg, nseg);
        };
        int64_t launches = 0;
        if (cfg->reevaluate) { DW_CHECK(fwd_call(r, lp)); launches += launch_count(); }   // mcmc.py:396
        if (cfg->n_steps == 0) { reset_launch_count(); count_launch((int)launches); return (int)DW_OK; }
        DW_CHECK_CUDA(cudaMemsetAsync(counts, 0, (size_t)mh_counts_needed(nseg) * sizeof(int), s));
        MhArgs m;
        m.r = r; m.r_prop = r_prop; m.lp = lp; m.lp_prop = lp_prop; m.age = age; m.scalars = scalars;
        m.counts = counts; m.B = B; m.n = a->n_el; m.max_age = cfg->max_age;
        m.interval = cfg->stepsize_update_interval; m.target = cfg->target_acceptance_rate;
        m.min_step = cfg->min_stepsize; m.max_step = cfg->max_stepsize; m.seed = cfg->seed;
        m.seg = seg; m.widx = widx; m.seeds = seeds; m.nseg = nseg;
        m.proposal = cfg->proposal;
        m.r_min = cfg->r_min; m.r_max = cfg->r_max; m.langevin_scale = cfg->langevin_scale;
        m.p_swap = cfg->p_spin_swap; m.p_flip = cfg->p_spin_flip;
        const bool asym = cfg->proposal == DW_PROPOSAL_LANGEVIN || cfg->proposal == DW_PROPOSAL_LOCAL ||
                          cfg->proposal == DW_PROPOSAL_LOCAL_ONE_EL;
        m.lq = asym ? lq : nullptr;
        m.R = R; m.Z = Z; m.N = a->n_ions;
        reset_launch_count();
        DW_TIMED("mh", launch_mh(m, 0, s));
        launches += launch_count();
        for (int k = 0; k < cfg->n_steps; ++k) {
            reset_launch_count();
            DW_CHECK(fwd_call(r_prop, lp_prop));
            DW_TIMED("mh", launch_mh(m, k + 1 < cfg->n_steps ? 1 : 2, s));
            launches += launch_count();
        }
        reset_launch_count();
        count_launch((int)launches);
        DW_CHECK_CUDA(cudaGetLastError());
        return (int)DW_OK;
    });
}

}  // namespace dw

extern "C" {

int dw_mcmc_steps(const DwArch* a, int precision, const float* params, const void* prepared, float* r, int B,
                  const float* R, const int32_t* Z, float* lp, int32_t* age, DwMcmcScalars* scalars,
                  const DwMcmcConfig* cfg, void* ws, size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared || !r || !R || !Z || !lp || !age || !scalars || !cfg || B <= 0) return DW_ERR_ARG;
    if (cfg->n_steps < 0 || !mcmc_config_ok(cfg)) return DW_ERR_ARG;
    return mcmc_impl(a, precision, params, prepared, r, B, R, Z, 1, nullptr, nullptr, nullptr, lp, age, scalars, cfg,
                     ws, wsb, (cudaStream_t)stream);
}

int dw_mcmc_steps_packed(const DwArch* a, int precision, const float* params, const void* prepared, float* r, int B,
                         const float* R, const int32_t* Z, int nseg, const int32_t* seg, const int32_t* walker_index,
                         const uint64_t* seeds, float* lp, int32_t* age, DwMcmcScalars* scalars,
                         const DwMcmcConfig* cfg, void* ws, size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared || !r || !R || !Z || !seg || !walker_index || !seeds || !lp || !age || !scalars || !cfg ||
        B <= 0)
        return DW_ERR_ARG;
    if (cfg->n_steps < 0 || nseg < 1 || nseg > kMaxSeg || !mcmc_config_ok(cfg)) return DW_ERR_ARG;
    return mcmc_impl(a, precision, params, prepared, r, B, R, Z, nseg, seg, walker_index, seeds, lp, age, scalars, cfg,
                     ws, wsb, (cudaStream_t)stream);
}

int dw_log_psi_sqr_packed(const DwArch* a, int precision, const float* params, const void* prepared, const float* r,
                          int B, const float* R, const int32_t* Z, int nseg, const int32_t* seg, float* lp,
                          float* phase, void* ws, size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared || !r || !R || !Z || !seg || !lp || B <= 0 || nseg < 1 || nseg > kMaxSeg)
        return DW_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    return with_act(precision, true, [&](auto tag) {
        using Act = act_of<decltype(tag)>;
        return forward_any<Act>(a, precision, params, prepared, r, B, R, Z, lp, phase, nullptr, nullptr, false, ws, wsb, s,
                                seg, nseg);
    });
}

int dw_local_energy_packed(const DwArch* a, int precision, const float* params, const void* prepared, const float* r,
                           int B, const float* R, const int32_t* Z, int nseg, const int32_t* seg, float* E, float* lp,
                           float* grad, void* ws, size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared || !r || !R || !Z || !seg || !E || B <= 0 || nseg < 1 || nseg > kMaxSeg)
        return DW_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    return local_energy_impl(a, precision, params, prepared, r, B, R, Z, seg, nseg, E, lp, grad, ws, wsb, s);
}

int dw_log_psi_sqr_backward(const DwArch* a, int precision, const float* params, const void* prepared, const float* r,
                            int B, const float* R, const int32_t* Z, const float* coeff, float* grad, void* ws,
                            size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared || !r || !R || !Z || !coeff || !grad || B <= 0) return DW_ERR_ARG;
    if (precision == DW_PRECISION_FP64) return DW_ERR_UNSUPPORTED;   // the backward runs in FP32
    if (precision < DW_PRECISION_FP32 || precision > DW_PRECISION_BF16) return DW_ERR_ARG;
    Prepared pre = carve_prepared(a, precision, const_cast<void*>(prepared));
    const float* m4[4] = {pre.main[0], pre.main[1], pre.main[2], pre.main[3]};
    const float* n4[4] = {pre.mean[0], pre.mean[1], pre.mean[2], pre.mean[3]};
    timer_begin("backward", (cudaStream_t)stream);
    const int st = backward_all(a, params, m4, n4, pre.bf_cat, pre.sp_alpha, r, B, R, Z, coeff, grad, ws, wsb,
                                (cudaStream_t)stream);
    timer_end("backward", (cudaStream_t)stream, 0.0, 0.0);
    return st;
}

int dw_energy_stats(const float* E, int n, double* out, void* stream) {
    reset_launch_count();
    if (!E || !out || n <= 0) return DW_ERR_ARG;
    launch_stats(E, n, 0, 0.0, 1.0, 1.0, nullptr, out, (cudaStream_t)stream);
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

// Instrumentation: the local energy of dw_local_energy plus three per-walker error scales
// (scales[3 b .. 3 b + 2]: the magnitude S of the terms summed into E_L, the magnitude of the
// determinant terms summed into the Laplacian of log|sum of determinants|, and 1 / (|psi~| + 1e-8)
// with psi~ the determinant sum relative to its largest term). FP32, mixed and BF16 forms.
int dw_debug_local_energy_scales(const DwArch* a, int precision, const float* params, const void* prepared,
                                 const float* r, int B, const float* R, const int32_t* Z, float* E, float* lp,
                                 float* scales, void* ws, size_t wsb, void* stream) {
    reset_launch_count();
    DW_CHECK(check_arch(a));
    if (!params || !prepared || !r || !R || !Z || !E || !lp || !scales || B <= 0) return DW_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    return with_act(precision, true, [&](auto tag) {
        using Act = act_of<decltype(tag)>;
        if constexpr (std::is_same<Act, double>::value) return (int)DW_ERR_ARG;
        else return forward_all<Act>(a, precision, params, prepared, r, B, R, Z, lp, nullptr, E, nullptr, true, ws, wsb,
                                     s, nullptr, 1, kChunkBudget, scales);
    });
}

int dw_clip_energies(const float* E, int n, double center, double width, double clip_by, float* E_clip, double* out,
                     void* stream) {
    reset_launch_count();
    if (!E || !out || !E_clip || n <= 0 || !(width > 0)) return DW_ERR_ARG;
    launch_stats(E, n, 1, center, width, clip_by, E_clip, out, (cudaStream_t)stream);
    DW_CHECK_CUDA(cudaGetLastError());
    return DW_OK;
}

}  // extern "C"
