// Determinants, their forward-mode derivatives, the multi-determinant combine, the
// Jastrow add, the kinetic energy and the Coulomb potential.
#include "net.cuh"
#include "ff.cuh"
#include <type_traits>

namespace dw {

// ------------------------------------------------------------------ slogdet (+ inverse)
// Shared FP64 helpers of the LU kernels.
// 1/d by Newton-Raphson iteration x <- x + x (1 - d x), seeded with the approximate FP32
// reciprocal (about 2^-22 relative); each step squares the relative error, so two steps reach
// FP64 precision. Divisions stay exact outside the FP32 exponent range.
__device__ __forceinline__ double recip_nr(double d) {
    const double ad = fabs(d);
    if (!(ad > 1e-30 && ad < 1e30)) return 1.0 / d;
    double x = (double)__fdividef(1.0f, (float)d);
    x = fma(x, fma(-d, x, 1.0), x);
    x = fma(x, fma(-d, x, 1.0), x);
    return x;
}
__device__ __forceinline__ float recip_nr(float d) { return 1.0f / d; }

template <class S> __device__ __forceinline__ int mag_key(S v);
template <> __device__ __forceinline__ int mag_key<double>(double v) { return __double2hiint(v) & 0x7fffffff; }
template <> __device__ __forceinline__ int mag_key<float>(float v) { return __float_as_int(v) & 0x7fffffff; }

// Multiplies the pivot-product mantissa by |pivot| and renormalises it to [0.5, 1) with
// integer operations on the exponent field (the library frexp only for subnormal / overflow).
__device__ __forceinline__ double mant_mul_norm(double mant, double a, int& expo) {
    double m = mant * a;                                  // a = |pivot| > 0, mant in [0.5, 1)
    const int hi = __double2hiint(m), lo = __double2loint(m);
    const int eb = (hi >> 20) & 0x7ff;
    if (eb == 0 || eb == 0x7ff) {                         // subnormal / overflow: library frexp
        int e;
        m = frexp(m, &e);
        expo += e;
        return m;
    }
    expo += eb - 1022;
    return __hiloint2double((hi & 0x800fffff) | 0x3fe00000, lo);
}

// Scalar operations of the elimination kernels, for S = double (FP64) and S = FF (float-float).
// Pivot keys: non-negative floating-point magnitudes order as their bit patterns.
__device__ __forceinline__ long long lu_key(double v) { return __double_as_longlong(v) & 0x7fffffffffffffffll; }
__device__ __forceinline__ int lu_key(FF v) { return __float_as_int(v.hi) & 0x7fffffff; }
template <class S> __device__ __forceinline__ S lu_from(float x);
template <> __device__ __forceinline__ double lu_from<double>(float x) { return (double)x; }
template <> __device__ __forceinline__ FF lu_from<FF>(float x) { return ff_make(x); }
__device__ __forceinline__ bool lu_neg(double v) { return v < 0.0; }
__device__ __forceinline__ bool lu_neg(FF v) { return v.hi < 0.f; }
__device__ __forceinline__ double lu_negate(double v) { return -v; }
__device__ __forceinline__ FF lu_negate(FF v) { return ff_neg(v); }
__device__ __forceinline__ double lu_fnma(double l, double u, double a) { return fma(-l, u, a); }   // a - l u
__device__ __forceinline__ FF lu_fnma(FF l, FF u, FF a) { return ff_fnma(l, u, a); }
__device__ __forceinline__ float lu_to_float(double v) { return (float)v; }
__device__ __forceinline__ float lu_to_float(FF v) { return __fadd_rn(v.hi, v.lo); }
// A pivot p with its reciprocal; lu_quot(a, q) = a / p. The float-float form divides instead of
// multiplying when 1 / p.hi leaves the normal FP32 range (|p| < 2^-125 or > 2^125).
struct PivD { double p, rp; };
struct PivF { FF p, rp; bool ok; };
__device__ __forceinline__ PivD lu_pivot(double p) { return PivD{p, recip_nr(p)}; }
__device__ __forceinline__ PivF lu_pivot(FF p) {
    const bool ok = ff_recip_ok(p);
    return PivF{p, ok ? ff_recip(p) : FF{0.f, 0.f}, ok};
}
__device__ __forceinline__ double lu_quot(double a, const PivD& q) { return a * q.rp; }
__device__ __forceinline__ FF lu_quot(FF a, const PivF& q) { return q.ok ? ff_mul(a, q.rp) : ff_div(a, q.p); }
// Pivot-magnitude product as mantissa [0.5, 1) and binary exponent; one log per matrix.
__device__ __forceinline__ void lu_mant_mul(double& m, double p, int& e) { m = mant_mul_norm(m, fabs(p), e); }
__device__ __forceinline__ void lu_mant_mul(FF& m, FF p, int& e) { ff_mant_mul(m, p, e); }
__device__ __forceinline__ double lu_log(double m, int e) { return log(m) + (double)e * 0.69314718055994530942; }
__device__ __forceinline__ double lu_log(FF m, int e) { return ff_log_mant(m, e); }

// One warp per (walker, determinant). Gauss-Jordan elimination with partial pivoting
// (first maximal |pivot| wins, as LAPACK getrf) on [A | I] in scalar type S; in value-only
// mode an LU elimination on A alone. Mirrors jnp.linalg.slogdet in
// evaluate_sum_of_determinants (model/wavefunction.py:63-73).
template <class S>
__global__ void k_slogdet(const float* __restrict__ MO, int n, int T, int nmat, int want_inv,
                          double* __restrict__ logdet, double* __restrict__ sign, float* __restrict__ Ainv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const int mat = blockIdx.x * wpb + wid;
    if (mat >= nmat) return;
    const int nc = want_inv ? 2 * n : n;
    S* M = reinterpret_cast<S*>(smem_raw) + (size_t)wid * n * nc;
    const float* A = MO + (int64_t)mat * T * n * n;      // channel 0 of this (walker, det)
    for (int e = lane; e < n * nc; e += 32) {
        int r = e / nc, c = e % nc;
        M[e] = c < n ? (S)A[r * n + c] : (S)((c - n) == r ? 1 : 0);
    }
    __syncwarp();
    double ld = 0.0, sg = 1.0;
    bool singular = false;
    for (int c = 0; c < n; ++c) {
        // pivot search over rows c..n-1
        S best = (S)-1; int bi = n;
        for (int r = c + lane; r < n; r += 32) {
            S v = M[r * nc + c]; v = v < 0 ? -v : v;
            if (v > best) { best = v; bi = r; }
        }
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            S ob = __shfl_xor_sync(0xffffffffu, best, o);
            int oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (!(best > (S)0)) { singular = true; break; }
        if (bi != c) {
            for (int j = lane; j < nc; j += 32) {
                S t = M[c * nc + j]; M[c * nc + j] = M[bi * nc + j]; M[bi * nc + j] = t;
            }
            sg = -sg;
            __syncwarp();
        }
        S piv = M[c * nc + c];
        ld += log(fabs((double)piv));
        if (piv < (S)0) sg = -sg;
        S inv = (S)1 / piv;
        for (int j = c + 1 + lane; j < nc; j += 32) M[c * nc + j] *= inv;
        __syncwarp();
        int r0 = want_inv ? 0 : c + 1;
        for (int r = r0; r < n; ++r) {
            if (r == c) continue;
            S f = M[r * nc + c];
            if (f != (S)0)
                for (int j = c + 1 + lane; j < nc; j += 32) M[r * nc + j] -= f * M[c * nc + j];
        }
        __syncwarp();
    }
    if (lane == 0) {
        logdet[mat] = singular ? -INFINITY : ld;
        sign[mat] = singular ? 0.0 : sg;
    }
    if (want_inv) {
        float* out = Ainv + (int64_t)mat * n * n;
        for (int e = lane; e < n * n; e += 32) {
            int r = e / n, c = e % n;
            out[e] = singular ? 0.f : (float)M[r * nc + n + c];
        }
    }
}

// Value-mode log|det| for 32 < n <= 64: warp per matrix, the matrix in shared memory (row pitch
// n + 1), LU with partial pivoting (first row of maximal |a|, as LAPACK getrf). Each step scales
// the L column and then spreads the (n - k - 1)^2 elements of the trailing update over all 32
// lanes in row-major order, so the lanes stay busy as the trailing block shrinks (the row-at-a-
// time form of k_slogdet leaves most lanes idle once fewer than 32 columns remain). Rows are
// exchanged from the pivot column on (the L factors are not needed for the determinant); the
// pivot magnitudes accumulate as a normalised mantissa and a binary exponent, one log per matrix.
__device__ __forceinline__ long long wide_key(double v) { return __double_as_longlong(v) & 0x7fffffffffffffffll; }
__device__ __forceinline__ long long wide_key(float v) { return (long long)(__float_as_int(v) & 0x7fffffff); }
__device__ __forceinline__ double wide_fnma(double l, double u, double a) { return fma(-l, u, a); }
__device__ __forceinline__ float wide_fnma(float l, float u, float a) { return fmaf(-l, u, a); }

template <class S>
__global__ void __launch_bounds__(256)
k_slogdet_wide(const float* __restrict__ MO, int n, int T, int nmat, double* __restrict__ logdet,
               double* __restrict__ sign) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const int mat = blockIdx.x * wpb + wid;
    if (mat >= nmat) return;                              // the whole warp
    const int ld = n + 1;
    S* M = reinterpret_cast<S*>(smem_raw) + (size_t)wid * n * ld;
    const float* A = MO + (int64_t)mat * T * n * n;       // channel 0 of this (walker, det)
    for (int e = lane; e < n * n; e += 32) {
        const int r = e / n, c = e - r * n;
        M[r * ld + c] = (S)__ldg(A + e);
    }
    __syncwarp();
    double mant = 1.0, sg = 1.0;
    int expo = 0;
    bool singular = false;
    for (int k = 0; k < n; ++k) {
        long long best = -1;
        int p = n;
        for (int r = k + lane; r < n; r += 32) {
            const long long v = wide_key(M[r * ld + k]);
            if (v > best) { best = v; p = r; }
        }
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int op = __shfl_xor_sync(0xffffffffu, p, o);
            if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
        }
        if (best <= 0) { singular = true; break; }        // the same in every lane
        if (p != k) {
            for (int j = k + lane; j < n; j += 32) {
                const S t = M[k * ld + j]; M[k * ld + j] = M[p * ld + j]; M[p * ld + j] = t;
            }
            sg = -sg;
            __syncwarp();
        }
        const S piv = M[k * ld + k];
        if (piv < (S)0) sg = -sg;
        mant = mant_mul_norm(mant, fabs((double)piv), expo);
        const S rp = recip_nr(piv);
        for (int r = k + 1 + lane; r < n; r += 32) M[r * ld + k] *= rp;
        __syncwarp();
        const int m = n - k - 1;
        if (m > 0) {
            // element e = lane + 32 s of the m x m trailing block: row e / m, column e % m,
            // advanced by 32 = dr m + dc with a carry instead of a division per element
            int r = lane / m, c = lane - r * m;
            const int dr = 32 / m, dc = 32 - dr * m;
            for (int e = lane; e < m * m; e += 32) {
                S* row = M + (k + 1 + r) * ld;
                row[k + 1 + c] = wide_fnma(row[k], M[k * ld + k + 1 + c], row[k + 1 + c]);
                r += dr;
                c += dc;
                if (c >= m) { c -= m; ++r; }
            }
        }
        __syncwarp();
    }
    if (lane == 0) {
        logdet[mat] = singular ? -INFINITY : log(mant) + (double)expo * 0.69314718055994530942;
        sign[mat] = singular ? 0.0 : sg;
    }
}

// log|det| and the inverse for 32 < n <= 64: Gauss-Jordan elimination on [A | I] with partial
// pivoting, warp per matrix in shared memory (row pitch 2n + 1). At step k the columns left of k
// of the A half are unit vectors and are neither stored nor touched: the pivot row is scaled on
// the columns right of k and every other row is updated there, the (n - 1)(2n - k - 1) elements
// spread over all 32 lanes. The right half ends as A^-1 (row exchanges act on both halves).
template <class S>
__global__ void __launch_bounds__(256)
k_slogdet_wide_inv(const float* __restrict__ MO, int n, int T, int nmat, double* __restrict__ logdet,
                   double* __restrict__ sign, float* __restrict__ Ainv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const int mat = blockIdx.x * wpb + wid;
    if (mat >= nmat) return;                              // the whole warp
    const int nc = 2 * n, ld = nc + 1;
    S* M = reinterpret_cast<S*>(smem_raw) + (size_t)wid * n * ld;
    const float* A = MO + (int64_t)mat * T * n * n;
    for (int e = lane; e < n * nc; e += 32) {
        const int r = e / nc, c = e - r * nc;
        M[r * ld + c] = c < n ? (S)__ldg(A + r * n + c) : (S)((c - n) == r ? 1 : 0);
    }
    __syncwarp();
    double mant = 1.0, sg = 1.0;
    int expo = 0;
    bool singular = false;
    for (int k = 0; k < n; ++k) {
        long long best = -1;
        int p = n;
        for (int r = k + lane; r < n; r += 32) {
            const long long v = wide_key(M[r * ld + k]);
            if (v > best) { best = v; p = r; }
        }
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const long long ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int op = __shfl_xor_sync(0xffffffffu, p, o);
            if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
        }
        if (best <= 0) { singular = true; break; }        // the same in every lane
        if (p != k) {
            for (int j = k + lane; j < nc; j += 32) {
                const S t = M[k * ld + j]; M[k * ld + j] = M[p * ld + j]; M[p * ld + j] = t;
            }
            sg = -sg;
            __syncwarp();
        }
        const S piv = M[k * ld + k];
        if (piv < (S)0) sg = -sg;
        mant = mant_mul_norm(mant, fabs((double)piv), expo);
        const S rp = recip_nr(piv);
        for (int j = k + 1 + lane; j < nc; j += 32) M[k * ld + j] *= rp;
        __syncwarp();
        const int w = nc - k - 1;                         // columns right of k
        // element e = lane + 32 s: row q = e / w of the n - 1 other rows, column e % w
        int q = lane / w, c = lane - q * w;
        const int dq = 32 / w, dc = 32 - dq * w;
        for (int e = lane; e < (n - 1) * w; e += 32) {
            const int r = q < k ? q : q + 1;
            S* row = M + r * ld;
            row[k + 1 + c] = wide_fnma(row[k], M[k * ld + k + 1 + c], row[k + 1 + c]);
            q += dq;
            c += dc;
            if (c >= w) { c -= w; ++q; }
        }
        __syncwarp();
    }
    if (lane == 0) {
        logdet[mat] = singular ? -INFINITY : log(mant) + (double)expo * 0.69314718055994530942;
        sign[mat] = singular ? 0.0 : sg;
    }
    float* out = Ainv + (int64_t)mat * n * n;
    for (int e = lane; e < n * n; e += 32) {
        const int r = e / n, c = e - r * n;
        out[e] = singular ? 0.f : (float)M[r * ld + n + c];
    }
}

// Register-resident variant for n <= NMAX <= 32: a team of n lanes per matrix (32 / n
// matrices per warp), lane c owning column c of A (and of the identity block when INV).
// Partial pivoting: the owner of the pivot column finds the first row of maximal |a| at or
// below the diagonal (as LAPACK getrf) and broadcasts it; every lane swaps and eliminates
// its own column. The pivot product is kept as an FP64 mantissa and a binary exponent
// (frexp) so only one log is taken per matrix; divisions happen on the pivot owner only.
template <class S, int NMAX, bool INV>
__global__ void __launch_bounds__(128)
k_slogdet_reg(const float* __restrict__ MO, int n, int T, int nmat, double* __restrict__ logdet,
              double* __restrict__ sign, float* __restrict__ Ainv) {
    const int lane = threadIdx.x & 31;
    const int teams = 32 / n;
    const int team = lane / n, c = lane % n;
    const bool lane_on = team < teams;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int mat = gw * teams + (lane_on ? team : 0);
    const bool active = lane_on && mat < nmat;
    const int src_base = (lane_on ? team : 0) * n;
    S col[NMAX], icol[NMAX];
    const float* A = MO + (int64_t)(active ? mat : 0) * T * n * n;
    #pragma unroll
    for (int r = 0; r < NMAX; ++r) {
        col[r] = (active && r < n) ? (S)A[r * n + c] : (S)0;
        if (INV) icol[r] = (r == c) ? (S)1 : (S)0;
    }
    double mant = 1.0, sg = 1.0;
    int expo = 0;
    bool singular = false;
    // All loops are unrolled over NMAX (== n for the exact-size instances, so no predicated-off
    // FP64 work is issued). Every lane runs all steps (teams of one warp share the shuffles); a
    // singular matrix only sets its flag and continues with a unit pivot.
    #pragma unroll
    for (int k = 0; k < NMAX; ++k) {
        if (k >= n) break;
        const int owner = src_base + k;
        // pivot search on magnitude bit patterns (non-negative IEEE values order as integers; no
        // FP64 instructions), first maximum wins; only the owner's result is used
        long long best = -1; int p = k;
        #pragma unroll
        for (int r = k; r < NMAX; ++r) {
            const long long v = std::is_same<S, double>::value
                                    ? (__double_as_longlong((double)col[r]) & 0x7fffffffffffffffll)
                                    : (long long)(__float_as_int((float)col[r]) & 0x7fffffff);
            if (r < n && v > best) { best = v; p = r; }
        }
        p = __shfl_sync(0xffffffffu, p, owner);
        best = __shfl_sync(0xffffffffu, best, owner);
        bool sing_now = !(best > 0);
        if (p != k) {
            S xk = col[k], xp = 0, ik = INV ? icol[k] : (S)0, ip = 0;
            #pragma unroll
            for (int r = k + 1; r < NMAX; ++r) if (r == p) { xp = col[r]; if (INV) ip = icol[r]; }
            col[k] = xp;
            if (INV) icol[k] = ip;
            #pragma unroll
            for (int r = k + 1; r < NMAX; ++r) if (r == p) { col[r] = xk; if (INV) icol[r] = ik; }
            sg = -sg;
        }
        S pk = __shfl_sync(0xffffffffu, col[k], owner);
        sing_now = sing_now || pk == (S)0;
        singular = singular || sing_now;
        if (sing_now) pk = (S)1;
        S inv = 0;
        if (c == k) inv = recip_nr(pk);
        inv = __shfl_sync(0xffffffffu, inv, owner);
        mant = mant_mul_norm(mant, fabs((double)pk), expo);
        if (pk < (S)0) sg = -sg;
        if (INV) {
            // Gauss-Jordan: scale row k, eliminate all other rows with the broadcast column-k entries
            col[k] *= inv;
            icol[k] *= inv;
            const S rk = col[k], irk = icol[k];
            #pragma unroll
            for (int r = 0; r < NMAX; ++r) {
                if (r == k) continue;
                const S f = __shfl_sync(0xffffffffu, col[r], owner);
                if (r < n) { col[r] -= f * rk; icol[r] -= f * irk; }
            }
        } else {
            // LU: eliminate the rows below the pivot; the owner pre-scales its column by 1/pivot
            const S rk = col[k];
            #pragma unroll
            for (int r = k + 1; r < NMAX; ++r) {
                const S f = __shfl_sync(0xffffffffu, col[r] * inv, owner);
                if (r < n) col[r] -= f * rk;
            }
        }
    }
    if (active && c == 0) {
        logdet[mat] = singular ? -INFINITY : log(mant) + (double)expo * 0.69314718055994530942;
        sign[mat] = singular ? 0.0 : sg;
    }
    if (INV && active) {
        float* out = Ainv + (int64_t)mat * n * n;
        #pragma unroll
        for (int r = 0; r < NMAX; ++r)
            if (r < n) out[r * n + c] = singular ? 0.f : (float)icol[r];
    }
}

// Value-only log|det| with rows in lanes: a team of n lanes per matrix (32 / n matrices per
// warp), lane r owning row r of A. Per pivot k: a segmented shuffle argmax over the team picks
// the first row of maximal |a_rk| at or below the diagonal (as LAPACK getrf; magnitudes are
// compared through their IEEE bit patterns, which order non-negative values), the two rows are
// exchanged by shuffles, the pivot row is broadcast one entry at a time and every lane below
// the pivot eliminates its own row: (n - k - 1) FMAs per lane, the minimum for LU. After each
// step the rows shift one column to the left, so the pivot column is always register a[0] and
// every register index is static (the pivot loop itself is not unrolled). The pivot product is
// kept as a mantissa and a binary exponent (frexp), with one log per matrix.
template <class S, int NMAX>
__global__ void __launch_bounds__(128)
k_slogdet_rows(const float* __restrict__ MO, int n, int T, int nmat, double* __restrict__ logdet,
               double* __restrict__ sign) {
    const int lane = threadIdx.x & 31;
    const int teams = 32 / n;
    const int team = lane / n, r = lane % n;
    const bool lane_on = team < teams;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int mat = gw * teams + (lane_on ? team : 0);
    const bool active = lane_on && mat < nmat;
    const int base = (lane_on ? team : 0) * n;
    S a[NMAX];
    const float* A = MO + (int64_t)(active ? mat : 0) * T * n * n + (int64_t)r * n;
    #pragma unroll
    for (int c = 0; c < NMAX; ++c) a[c] = (active && c < n) ? (S)__ldg(A + c) : (S)0;
    double mant = 1.0, sg = 1.0;
    int expo = 0;
    bool singular = false;
    #pragma unroll 1
    for (int k = 0; k < n; ++k) {
        const int rem = n - k;                       // live columns a[0 .. rem)
        // team argmax of |a_r0| over rows r >= k (ties: lowest row)
        int key = (lane_on && r >= k) ? mag_key<S>(a[0]) : -1, row = r;
        #pragma unroll
        for (int off = 1; off < NMAX; off <<= 1) {
            const int ok = __shfl_down_sync(0xffffffffu, key, off);
            const int orow = __shfl_down_sync(0xffffffffu, row, off);
            if (r + off < n && (ok > key || (ok == key && orow < row))) { key = ok; row = orow; }
        }
        const int p = __shfl_sync(0xffffffffu, row, base);
        const int kmax = __shfl_sync(0xffffffffu, key, base);
        bool sing_now = kmax <= 0;
        // row exchange; the shuffles run warp-wide whenever any team of the warp swaps
        const bool swap = p != k;
        if (__any_sync(0xffffffffu, swap)) {
            const int src = base + (swap ? (r == k ? p : (r == p ? k : r)) : r);
            #pragma unroll
            for (int c = 0; c < NMAX; ++c) {
                if (c >= rem) break;
                a[c] = __shfl_sync(0xffffffffu, a[c], src);
            }
        }
        if (swap) sg = -sg;
        S pk = __shfl_sync(0xffffffffu, a[0], base + k);
        sing_now = sing_now || pk == (S)0;
        singular = singular || sing_now;
        if (sing_now) pk = (S)1;
        int e;
        mant *= frexp(fabs((double)pk), &e);
        expo += e;
        mant = frexp(mant, &e);
        expo += e;
        if (pk < (S)0) sg = -sg;
        const bool below = r > k;
        const S l = below ? a[0] * recip_nr(pk) : (S)0;
        #pragma unroll
        for (int c = 1; c < NMAX; ++c) {
            if (c >= rem) break;
            const S pc = __shfl_sync(0xffffffffu, a[c], base + k);
            if (below) a[c] -= l * pc;
        }
        #pragma unroll
        for (int c = 0; c + 1 < NMAX; ++c) a[c] = a[c + 1];
    }
    if (active && r == 0) {
        logdet[mat] = singular ? -INFINITY : log(mant) + (double)expo * 0.69314718055994530942;
        sign[mat] = singular ? 0.0 : sg;
    }
}

// log|det| with one matrix per thread, in FP64 (S = double) or float-float (S = FF). On this
// part FP64 arithmetic issues at about 1/100 of the FP32 rate, so the FP64 form is bound by the
// number of FP64 instructions. The production forms use FP64: the LU is one of the steps kept in
// FP64 for stability near nodal surfaces. The float-float instances (about 15 FP32 instructions
// per elimination step, ~48-bit significands; measured 1.3-2.5x faster for n = 10..16, with
// log|det| within ~1e-9 of FP64 on random matrices) are an evaluated alternative, reachable
// through dw_debug_slogdet_small and tested there. Giving each thread a whole matrix issues
// exactly the (n-k-1)^2 trailing-update steps and (n-k-1) multipliers of pivot k, plus one
// reciprocal and one mantissa product per pivot, with no lanes idling above the pivot.
// The matrices live in shared memory, element (i, j) of thread t at
// sm[(i * NMAX + j) * LD + t] with LD = TPB + 1 (8-byte elements): accesses of one element by
// all threads are consecutive, and the odd stride keeps the cooperative staging of the
// row-major input free of bank conflicts. Partial pivoting takes the first row of maximal
// |a_ik| at or below the diagonal (as LAPACK getrf), comparing magnitude bit patterns (the
// leading FP32 word in the float-float form); rows are exchanged physically, so ties are
// resolved in the current row order exactly as getrf does. The pivot product is kept as a
// mantissa in [0.5, 1) and a binary exponent, normalised with integer operations, and one log
// is taken per matrix.
template <class S, int NMAX, int TPB>
__global__ void __launch_bounds__(TPB)
k_slogdet_thread(const float* __restrict__ MO, int n, int T, int nmat, double* __restrict__ logdet,
                 double* __restrict__ sign) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int LD = TPB + 1;
    static_assert(sizeof(S) == 8, "8-byte elements");
    S* sm = reinterpret_cast<S*>(smem_raw);
    const int tid = threadIdx.x;
    const int mat0 = blockIdx.x * TPB;
    const int nm = min(TPB, nmat - mat0);
    const int nn = n * n;
    // cooperative staging: matrix m of the block is n*n contiguous floats at MO + (mat0+m) T n^2
    for (int q = tid; q < nm * nn; q += TPB) {
        const int m = q / nn, e = q - m * nn;
        const int i = e / n, j = e - i * n;
        sm[(i * NMAX + j) * LD + m] = lu_from<S>(__ldg(MO + (int64_t)(mat0 + m) * T * nn + e));
    }
    __syncthreads();
    if (tid >= nm) return;
    S* a = sm + tid;
    auto at = [&](int i, int j) -> S& { return a[(i * NMAX + j) * LD]; };
    S mant = lu_from<S>(1.f);
    double sg = 1.0;
    int expo = 0;
    bool singular = false;
    #pragma unroll 1
    for (int k = 0; k < n; ++k) {
        auto best = lu_key(at(k, k));
        int p = k;
        #pragma unroll 1
        for (int i = k + 1; i < n; ++i) {
            const auto v = lu_key(at(i, k));
            if (v > best) { best = v; p = i; }
        }
        if (best == 0) { singular = true; break; }
        if (p != k) {
            #pragma unroll 1
            for (int j = k; j < n; ++j) { const S t = at(k, j); at(k, j) = at(p, j); at(p, j) = t; }
            sg = -sg;
        }
        const S pk = at(k, k);
        if (lu_neg(pk)) sg = -sg;
        lu_mant_mul(mant, pk, expo);
        const auto piv = lu_pivot(pk);
        const int rem = n - k - 1;                       // trailing columns k+1 .. n-1
        S u[NMAX - 1];
        #pragma unroll
        for (int c = 0; c < NMAX - 1; ++c) {
            if (c >= rem) break;
            u[c] = at(k, k + 1 + c);
        }
        #pragma unroll 1
        for (int i = k + 1; i < n; ++i) {
            S* row = &at(i, k);
            const S l = lu_quot(row[0], piv);
            #pragma unroll
            for (int c = 0; c < NMAX - 1; ++c) {
                if (c >= rem) break;
                row[(c + 1) * LD] = lu_fnma(l, u[c], row[(c + 1) * LD]);
            }
        }
    }
    logdet[mat0 + tid] = singular ? -INFINITY : lu_log(mant, expo);
    sign[mat0 + tid] = singular ? 0.0 : sg;
}

// log|det| and inverse with one matrix per thread (S = double or FF, as k_slogdet_thread):
// in-place Gauss-Jordan elimination with partial pivoting (first row of maximal |a_ik| at or
// below the diagonal, rows exchanged physically as getrf does), n^3 update steps per matrix.
// Pivot k: row k is scaled by 1/a_kk, every other row i loses a_ik times it, and column k
// becomes the inverse's column (1/a_kk on the diagonal, -a_ik/a_kk elsewhere). The result is
// (PA)^-1 = A^-1 P^T, so the recorded row exchanges are undone on the columns in reverse order.
// Shared-memory layout and log-det bookkeeping as in k_slogdet_thread; the inverse is written
// in FP32 (zeros when singular).
template <class S, int NMAX, int TPB>
__global__ void __launch_bounds__(TPB)
k_slogdet_inv_thread(const float* __restrict__ MO, int n, int T, int nmat, double* __restrict__ logdet,
                     double* __restrict__ sign, float* __restrict__ Ainv) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int LD = TPB + 1;
    static_assert(sizeof(S) == 8, "8-byte elements");
    S* sm = reinterpret_cast<S*>(smem_raw);
    unsigned char* pivs = smem_raw + (size_t)NMAX * NMAX * LD * sizeof(S);   // [k][thread]
    const int tid = threadIdx.x;
    const int mat0 = blockIdx.x * TPB;
    const int nm = min(TPB, nmat - mat0);
    const int nn = n * n;
    for (int q = tid; q < nm * nn; q += TPB) {
        const int m = q / nn, e = q - m * nn;
        const int i = e / n, j = e - i * n;
        sm[(i * NMAX + j) * LD + m] = lu_from<S>(__ldg(MO + (int64_t)(mat0 + m) * T * nn + e));
    }
    __syncthreads();
    if (tid >= nm) return;
    S* a = sm + tid;
    auto at = [&](int i, int j) -> S& { return a[(i * NMAX + j) * LD]; };
    const S one = lu_from<S>(1.f);
    S mant = one;
    double sg = 1.0;
    int expo = 0;
    bool singular = false;
    #pragma unroll 1
    for (int k = 0; k < n; ++k) {
        auto best = lu_key(at(k, k));
        int p = k;
        #pragma unroll 1
        for (int i = k + 1; i < n; ++i) {
            const auto v = lu_key(at(i, k));
            if (v > best) { best = v; p = i; }
        }
        if (best == 0) { singular = true; break; }
        pivs[k * TPB + tid] = (unsigned char)p;
        if (p != k) {
            #pragma unroll 1
            for (int j = 0; j < n; ++j) { const S t = at(k, j); at(k, j) = at(p, j); at(p, j) = t; }
            sg = -sg;
        }
        const S pk = at(k, k);
        if (lu_neg(pk)) sg = -sg;
        lu_mant_mul(mant, pk, expo);
        const auto piv = lu_pivot(pk);
        // scaled pivot row in registers (column k itself becomes 1 / a_kk)
        S u[NMAX];
        #pragma unroll
        for (int j = 0; j < NMAX; ++j) {
            if (j >= n) break;
            u[j] = lu_quot(j == k ? one : at(k, j), piv);
            at(k, j) = u[j];
        }
        #pragma unroll 1
        for (int i = 0; i < n; ++i) {
            if (i == k) continue;
            S* row = &at(i, 0);
            const S f = row[k * LD];
            #pragma unroll
            for (int j = 0; j < NMAX; ++j) {
                if (j >= n) break;
                if (j == k) continue;
                row[j * LD] = lu_fnma(f, u[j], row[j * LD]);
            }
            row[k * LD] = lu_negate(lu_quot(f, piv));
        }
    }
    const int mat = mat0 + tid;
    logdet[mat] = singular ? -INFINITY : lu_log(mant, expo);
    sign[mat] = singular ? 0.0 : sg;
    float* out = Ainv + (int64_t)mat * nn;
    if (singular) {
        for (int e = 0; e < nn; ++e) out[e] = 0.f;
        return;
    }
    // undo the row exchanges on the columns, last exchange first
    #pragma unroll 1
    for (int k = n - 1; k >= 0; --k) {
        const int p = pivs[k * TPB + tid];
        if (p == k) continue;
        #pragma unroll 1
        for (int i = 0; i < n; ++i) { const S t = at(i, k); at(i, k) = at(i, p); at(i, p) = t; }
    }
    #pragma unroll 1
    for (int i = 0; i < n; ++i)
        #pragma unroll 1
        for (int j = 0; j < n; ++j) out[i * n + j] = lu_to_float(at(i, j));
}

// log|det| (and, with INV, the inverse) with SPLIT lanes per matrix, S = double or FF: the
// lanes of a matrix own its rows cyclically (row i belongs to lane i % SPLIT) and run the same
// elimination as k_slogdet_thread (LU) / k_slogdet_inv_thread (Gauss-Jordan) on their rows,
// exchanging the pivot choice by shuffles and sharing rows through shared memory. For n > 12
// the per-matrix shared memory limits an SM to about a hundred matrices, so a single lane per
// matrix leaves the arithmetic pipes short of warps; splitting the rows multiplies the warps
// at nearly the same instruction count. Lanes of padding matrices (past nmat) eliminate an
// identity matrix so that every lane runs every shuffle.
template <class S, int NMAX, int SPLIT, bool INV>
__global__ void __launch_bounds__(32 * SPLIT)
k_slogdet_split(const float* __restrict__ MO, int n, int T, int nmat, double* __restrict__ logdet,
                double* __restrict__ sign, float* __restrict__ Ainv) {
    constexpr int TPB = 32 * SPLIT, MPB = 32, LD = MPB + 1;
    static_assert(sizeof(S) == 8, "8-byte elements");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    S* sm = reinterpret_cast<S*>(smem_raw);
    unsigned char* pivs = smem_raw + (size_t)NMAX * NMAX * LD * sizeof(S);    // [k][matrix]
    const int tid = threadIdx.x, m = tid / SPLIT, h = tid % SPLIT;
    const int mat0 = blockIdx.x * MPB;
    const int nm = min(MPB, nmat - mat0);
    const int nn = n * n;
    for (int q = tid; q < MPB * nn; q += TPB) {
        const int mm = q / nn, e = q - mm * nn;
        const int i = e / n, j = e - i * n;
        sm[(i * NMAX + j) * LD + mm] = lu_from<S>(mm < nm ? __ldg(MO + (int64_t)(mat0 + mm) * T * nn + e)
                                                          : (i == j ? 1.f : 0.f));
    }
    __syncthreads();
    S* a = sm + m;
    auto at = [&](int i, int j) -> S& { return a[(i * NMAX + j) * LD]; };
    const S one = lu_from<S>(1.f);
    S mant = one;
    double sg = 1.0;
    int expo = 0;
    bool singular = false;
    #pragma unroll 1
    for (int k = 0; k < n; ++k) {
        // first own row at or below the diagonal
        const int i0 = k + ((h - k % SPLIT) + SPLIT) % SPLIT;
        decltype(lu_key(one)) best = -1;
        int p = n;
        #pragma unroll 1
        for (int i = i0; i < n; i += SPLIT) {
            const auto v = lu_key(at(i, k));
            if (v > best) { best = v; p = i; }
        }
        #pragma unroll
        for (int o = 1; o < SPLIT; o <<= 1) {
            const auto ob = __shfl_xor_sync(0xffffffffu, best, o);
            const int op = __shfl_xor_sync(0xffffffffu, p, o);
            if (ob > best || (ob == best && op < p)) { best = ob; p = op; }
        }
        const bool sing_now = best <= 0;
        singular = singular || sing_now;
        if (sing_now) p = k;
        if (INV && h == 0) pivs[k * MPB + m] = (unsigned char)p;
        if (p != k) {
            #pragma unroll 1
            for (int j = (INV ? 0 : k) + h; j < n; j += SPLIT) {
                const S t = at(k, j); at(k, j) = at(p, j); at(p, j) = t;
            }
            sg = -sg;
        }
        __syncwarp();
        S pk = at(k, k);
        if (sing_now) pk = one;
        if (lu_neg(pk)) sg = -sg;
        lu_mant_mul(mant, pk, expo);
        const auto piv = lu_pivot(pk);
        if (!INV) {
            const int rem = n - k - 1;
            S u[NMAX - 1];
            #pragma unroll
            for (int c = 0; c < NMAX - 1; ++c) {
                if (c >= rem) break;
                u[c] = at(k, k + 1 + c);
            }
            #pragma unroll 1
            for (int i = i0 + (i0 == k ? SPLIT : 0); i < n; i += SPLIT) {
                S* row = &at(i, k);
                const S l = lu_quot(row[0], piv);
                #pragma unroll
                for (int c = 0; c < NMAX - 1; ++c) {
                    if (c >= rem) break;
                    row[(c + 1) * LD] = lu_fnma(l, u[c], row[(c + 1) * LD]);
                }
            }
        } else {
            S u[NMAX];
            #pragma unroll
            for (int j = 0; j < NMAX; ++j) {
                if (j >= n) break;
                u[j] = lu_quot(j == k ? one : at(k, j), piv);
            }
            __syncwarp();                                     // row k read by every lane of the matrix
            if (k % SPLIT == h) {
                #pragma unroll
                for (int j = 0; j < NMAX; ++j) {
                    if (j >= n) break;
                    at(k, j) = u[j];
                }
            }
            #pragma unroll 1
            for (int i = h; i < n; i += SPLIT) {
                if (i == k) continue;
                S* row = &at(i, 0);
                const S f = row[k * LD];
                #pragma unroll
                for (int j = 0; j < NMAX; ++j) {
                    if (j >= n) break;
                    if (j == k) continue;
                    row[j * LD] = lu_fnma(f, u[j], row[j * LD]);
                }
                row[k * LD] = lu_negate(lu_quot(f, piv));
            }
        }
        __syncwarp();
    }
    const bool active = m < nm;
    const int mat = mat0 + m;
    if (active && h == 0) {
        logdet[mat] = singular ? -INFINITY : lu_log(mant, expo);
        sign[mat] = singular ? 0.0 : sg;
    }
    if (!INV) return;
    // undo the row exchanges on the columns, last exchange first (own rows)
    #pragma unroll 1
    for (int k = n - 1; k >= 0; --k) {
        const int p = pivs[k * MPB + m];
        if (p == k) continue;
        #pragma unroll 1
        for (int i = h; i < n; i += SPLIT) { const S t = at(i, k); at(i, k) = at(i, p); at(i, p) = t; }
    }
    if (!active) return;
    float* out = Ainv + (int64_t)mat * nn;
    #pragma unroll 1
    for (int i = h; i < n; i += SPLIT)
        #pragma unroll 1
        for (int j = 0; j < n; ++j) out[i * n + j] = singular ? 0.f : lu_to_float(at(i, j));
}

template <class S, int NMAX, int SPLIT, bool INV>
static void launch_slogdet_split(const float* MO, int n, int T, int nmat, double* logdet, double* sign, float* Ainv,
                                 cudaStream_t s) {
    const size_t smem = (size_t)NMAX * NMAX * 33 * sizeof(S) + (size_t)NMAX * 32;
    cudaFuncSetAttribute(k_slogdet_split<S, NMAX, SPLIT, INV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_slogdet_split<S, NMAX, SPLIT, INV><<<(unsigned)((nmat + 31) / 32), 32 * SPLIT, smem, s>>>(MO, n, T, nmat, logdet,
                                                                                             sign, Ainv);
}

template <class S, int NMAX, int TPB>
static void launch_slogdet_inv_thread(const float* MO, int n, int T, int nmat, double* logdet, double* sign, float* Ainv,
                                      cudaStream_t s) {
    const size_t smem = (size_t)NMAX * NMAX * (TPB + 1) * sizeof(S) + (size_t)NMAX * TPB;
    cudaFuncSetAttribute(k_slogdet_inv_thread<S, NMAX, TPB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_slogdet_inv_thread<S, NMAX, TPB><<<(unsigned)((nmat + TPB - 1) / TPB), TPB, smem, s>>>(MO, n, T, nmat, logdet,
                                                                                          sign, Ainv);
}

template <class S, int NMAX, int TPB>
static void launch_slogdet_thread(const float* MO, int n, int T, int nmat, double* logdet, double* sign, cudaStream_t s) {
    const size_t smem = (size_t)NMAX * NMAX * (TPB + 1) * sizeof(S);
    cudaFuncSetAttribute(k_slogdet_thread<S, NMAX, TPB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_slogdet_thread<S, NMAX, TPB><<<(unsigned)((nmat + TPB - 1) / TPB), TPB, smem, s>>>(MO, n, T, nmat, logdet, sign);
}

// Elimination kernels for n <= 16 in scalar type S (double or FF). FP64: one matrix per thread
// up to n = 12 (the FP64 pipe is the bound, and a thread per matrix issues the fewest FP64
// instructions), four lanes per matrix above. Float-float: one matrix per thread up to n = 8,
// four lanes per matrix above -- its ~15-instruction update chains are latency-bound at the
// 8 warps per SM that a thread per matrix leaves in shared memory, and four lanes per matrix
// measured 1.2-2.1x faster for n = 10 and 12 (two or eight lanes: slower than four).
template <class S>
static void launch_slogdet_small(const float* MO, int n, int T, int nmat, double* logdet, double* sign, float* Ainv,
                                 bool want_inv, cudaStream_t s) {
    constexpr bool ff = std::is_same<S, FF>::value;
    if (n <= 8 || (!ff && n <= 12)) {
        if (!want_inv) {
            if (n <= 4) launch_slogdet_thread<S, 4, 64>(MO, n, T, nmat, logdet, sign, s);
            else if (n <= 8) launch_slogdet_thread<S, 8, 64>(MO, n, T, nmat, logdet, sign, s);
            else if (n <= 10) launch_slogdet_thread<S, 10, 64>(MO, n, T, nmat, logdet, sign, s);
            else launch_slogdet_thread<S, 12, 64>(MO, n, T, nmat, logdet, sign, s);
        } else {
            if (n <= 4) launch_slogdet_inv_thread<S, 4, 64>(MO, n, T, nmat, logdet, sign, Ainv, s);
            else if (n <= 8) launch_slogdet_inv_thread<S, 8, 64>(MO, n, T, nmat, logdet, sign, Ainv, s);
            else if (n <= 10) launch_slogdet_inv_thread<S, 10, 64>(MO, n, T, nmat, logdet, sign, Ainv, s);
            else launch_slogdet_inv_thread<S, 12, 64>(MO, n, T, nmat, logdet, sign, Ainv, s);
        }
        return;
    }
    auto go = [&](auto nmax) {
        constexpr int NM = decltype(nmax)::value;
        if (want_inv) launch_slogdet_split<S, NM, 4, true>(MO, n, T, nmat, logdet, sign, Ainv, s);
        else launch_slogdet_split<S, NM, 4, false>(MO, n, T, nmat, logdet, sign, nullptr, s);
    };
    if constexpr (ff) {
        if (n <= 10) go(std::integral_constant<int, 10>());
        else if (n <= 12) go(std::integral_constant<int, 12>());
        else go(std::integral_constant<int, 16>());
    } else {
        go(std::integral_constant<int, 16>());
    }
}

template <class S>
void launch_slogdet_impl(const float* MO, const Dims& d, int B, double* logdet, double* sign, float* Ainv, int want_inv,
                         cudaStream_t s);
template <class S>
void launch_slogdet(const float* MO, const Dims& d, int B, double* logdet, double* sign, float* Ainv, cudaStream_t s) {
    launch_slogdet_impl<S>(MO, d, B, logdet, sign, Ainv, d.Tp > 1 ? 1 : 0, s);
}
void launch_slogdet_inv(const float* MO, const Dims& d, int B, double* logdet, double* sign, float* Ainv, cudaStream_t s) {
    launch_slogdet_impl<double>(MO, d, B, logdet, sign, Ainv, 1, s);
}
template <class S>
void launch_slogdet_impl(const float* MO, const Dims& d, int B, double* logdet, double* sign, float* Ainv, int want_inv,
                         cudaStream_t s) {
    int n = d.n;
    int nmat = B * d.K;
    if (n <= 32) {
        const int teams = 32 / n;
        const int64_t warps = (nmat + teams - 1) / teams;
        const unsigned blocks = (unsigned)((warps * 32 + 127) / 128);
        // the high-precision form (S = double): FP64 elimination, one matrix per thread or four
        // lanes per matrix, up to n = 16
        if (std::is_same<S, double>::value && n <= 16) {
            launch_slogdet_small<double>(MO, n, d.T, nmat, logdet, sign, Ainv, want_inv != 0, s);
            count_launch();
            return;
        }
        if (!want_inv) {
            auto rows = [&](auto kern) { kern<<<blocks, 128, 0, s>>>(MO, n, d.T, nmat, logdet, sign); };
            if (n <= 4) rows(k_slogdet_rows<S, 4>);
            else if (n <= 8) rows(k_slogdet_rows<S, 8>);
            else if (n <= 10) rows(k_slogdet_rows<S, 10>);
            else if (n <= 12) rows(k_slogdet_rows<S, 12>);
            else if (n <= 16) rows(k_slogdet_rows<S, 16>);
            else if (n <= 24) rows(k_slogdet_rows<S, 24>);
            else rows(k_slogdet_rows<S, 32>);
            count_launch();
            return;
        }
        auto go = [&](auto kern) { kern<<<blocks, 128, 0, s>>>(MO, n, d.T, nmat, logdet, sign, Ainv); };
        if (n <= 8) { if (want_inv) go(k_slogdet_reg<S, 8, true>); else go(k_slogdet_reg<S, 8, false>); }
        else if (n <= 16) { if (want_inv) go(k_slogdet_reg<S, 16, true>); else go(k_slogdet_reg<S, 16, false>); }
        else if (n <= 24) { if (want_inv) go(k_slogdet_reg<S, 24, true>); else go(k_slogdet_reg<S, 24, false>); }
        else { if (want_inv) go(k_slogdet_reg<S, 32, true>); else go(k_slogdet_reg<S, 32, false>); }
        count_launch();
        return;
    }
    if (!want_inv && n <= 64) {
        const size_t per = (size_t)n * (n + 1) * sizeof(S);
        int wpb = (int)(96 * 1024 / per);
        wpb = wpb < 1 ? 1 : (wpb > 8 ? 8 : wpb);
        const size_t sm = per * wpb;
        if (sm > 48 * 1024) cudaFuncSetAttribute(k_slogdet_wide<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_slogdet_wide<S><<<(nmat + wpb - 1) / wpb, wpb * 32, sm, s>>>(MO, n, d.T, nmat, logdet, sign);
        count_launch();
        return;
    }
    if (want_inv && n <= 64) {
        const size_t per = (size_t)n * (2 * n + 1) * sizeof(S);
        int wpb = (int)(96 * 1024 / per);
        wpb = wpb < 1 ? 1 : (wpb > 8 ? 8 : wpb);
        const size_t sm = per * wpb;
        if (sm > 48 * 1024)
            cudaFuncSetAttribute(k_slogdet_wide_inv<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_slogdet_wide_inv<S><<<(nmat + wpb - 1) / wpb, wpb * 32, sm, s>>>(MO, n, d.T, nmat, logdet, sign, Ainv);
        count_launch();
        return;
    }
    int nc = want_inv ? 2 * n : n;
    size_t per = (size_t)n * nc * sizeof(S);
    int wpb = (int)(96 * 1024 / per);
    wpb = wpb < 1 ? 1 : (wpb > 8 ? 8 : wpb);
    size_t sm = per * wpb;
    if (sm > 48 * 1024) cudaFuncSetAttribute(k_slogdet<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_slogdet<S><<<(nmat + wpb - 1) / wpb, wpb * 32, sm, s>>>(MO, n, d.T, nmat, want_inv, logdet, sign, Ainv);
    count_launch();
}
template void launch_slogdet<float>(const float*, const Dims&, int, double*, double*, float*, cudaStream_t);
template void launch_slogdet<double>(const float*, const Dims&, int, double*, double*, float*, cudaStream_t);

// ------------------------------------------------------------------ determinant tangents
// g_t = tr(A^-1 dA_t), lap = tr(A^-1 Lap A) - sum_t tr((A^-1 dA_t)^2), traces accumulated in FP64.
__global__ void k_det_tangents(const float* __restrict__ MO, const float* __restrict__ Ainv,
                               const double* __restrict__ sign, int n, int T, int nmat,
                               double* __restrict__ g, double* __restrict__ lapdet) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* Ai = reinterpret_cast<float*>(smem_raw);
    float* dA = Ai + n * n;
    float* C = dA + n * n;
    __shared__ double red[2][32];
    const int mat = blockIdx.x;
    const int tid = threadIdx.x, nt = blockDim.x;
    if (sign[mat] == 0.0) {
        for (int t = tid; t < 3 * n; t += nt) g[(int64_t)mat * 3 * n + t] = 0.0;
        if (tid == 0) lapdet[mat] = 0.0;
        return;
    }
    for (int e = tid; e < n * n; e += nt) Ai[e] = Ainv[(int64_t)mat * n * n + e];
    double lap_acc = 0.0;
    for (int t = 1; t < T; ++t) {
        const float* src = MO + ((int64_t)mat * T + t) * n * n;
        __syncthreads();
        for (int e = tid; e < n * n; e += nt) dA[e] = src[e];
        __syncthreads();
        double tr = 0.0, tr2 = 0.0;
        for (int e = tid; e < n * n; e += nt) {
            int a = e / n, c = e % n;
            float acc = 0.f;
            for (int m = 0; m < n; ++m) acc = fmaf(Ai[a * n + m], dA[m * n + c], acc);
            C[e] = acc;
            if (a == c) tr += acc;
        }
        __syncthreads();
        if (t != T - 1) {
            for (int e = tid; e < n * n; e += nt) {
                int a = e / n, c = e % n;
                tr2 += (double)C[a * n + c] * (double)C[c * n + a];
            }
        }
        tr = warp_sum(tr); tr2 = warp_sum(tr2);
        if ((tid & 31) == 0) { red[0][tid >> 5] = tr; red[1][tid >> 5] = tr2; }
        __syncthreads();
        if (tid == 0) {
            double s0 = 0, s1 = 0;
            for (int w = 0; w < (nt + 31) / 32; ++w) { s0 += red[0][w]; s1 += red[1][w]; }
            if (t == T - 1) lap_acc += s0;
            else { g[(int64_t)mat * 3 * n + (t - 1)] = s0; lap_acc -= s1; }
        }
    }
    if (tid == 0) lapdet[mat] = lap_acc;
}

// Warp per (walker, determinant) for n <= 32: A^-1 staged in shared memory, lanes split into
// G = 32 / n groups, each group takes one tangent channel at a time and lane j of a group owns
// column j of dA_t and of C_t = A^-1 dA_t. tr(C_t) and tr(C_t^2) are accumulated in FP64.
__global__ void __launch_bounds__(128)
k_det_tangents_warp(const float* __restrict__ MO, const float* __restrict__ Ainv, const double* __restrict__ sign,
                    int n, int T, int nmat, double* __restrict__ g, double* __restrict__ lapdet) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const int mat = blockIdx.x * wpb + wid;
    const int G = 32 / n;                 // channel groups per warp
    // per warp: A^-1 (ais floats) then G group areas of cgs floats (C_t with row pitch n + 1, later
    // reused for 2 n double partials); both sizes are even so the doubles stay 8-byte aligned
    const int ais = (n * n + 1) & ~1, cgs = ((n * (n + 1) > 4 * n ? n * (n + 1) : 4 * n) + 1) & ~1;
    float* Ai = reinterpret_cast<float*>(smem_raw) + (size_t)wid * (ais + G * cgs);
    float* Cs = Ai + ais;
    if (mat >= nmat) return;
    if (sign[mat] == 0.0) {
        for (int t = lane; t < 3 * n; t += 32) g[(int64_t)mat * 3 * n + t] = 0.0;
        if (lane == 0) lapdet[mat] = 0.0;
        return;
    }
    for (int e = lane; e < n * n; e += 32) Ai[e] = Ainv[(int64_t)mat * n * n + e];
    __syncwarp();
    const int grp = lane / n, j = lane % n;
    const bool on = grp < G;
    float* Cg = Cs + (size_t)(on ? grp : 0) * cgs;
    double lap_acc = 0.0;
    for (int t0 = 1; t0 < T; t0 += G) {
        const int t = t0 + grp;
        const bool valid = on && t < T;
        float col[32];
        const float* src = MO + ((int64_t)mat * T + (valid ? t : 0)) * n * n;
        #pragma unroll
        for (int m = 0; m < 32; ++m) col[m] = (valid && m < n) ? src[m * n + j] : 0.f;
        for (int a = 0; a < n; ++a) {
            float acc = 0.f;
            #pragma unroll
            for (int m = 0; m < 32; ++m) if (m < n) acc = fmaf(Ai[a * n + m], col[m], acc);
            if (valid) Cg[a * (n + 1) + j] = acc;
        }
        __syncwarp();
        // lane j: C[j][j] and sum_a C[a][j] C[j][a]; the group leader adds the n lane partials
        // lane partials in FP32 (n products of one row/column pair); the cross-lane and
        // cross-channel trace sums below are accumulated in FP64
        double p0 = 0.0, p1 = 0.0;
        if (valid) {
            p0 = (double)Cg[j * (n + 1) + j];
            if (t != T - 1) {
                float q = 0.f;
                for (int a = 0; a < n; ++a) q = fmaf(Cg[a * (n + 1) + j], Cg[j * (n + 1) + a], q);
                p1 = (double)q;
            }
        }
        __syncwarp();
        double* part = reinterpret_cast<double*>(Cg);     // reuse the C area as [n][2] doubles
        if (valid) { part[2 * j] = p0; part[2 * j + 1] = p1; }
        __syncwarp();
        if (valid && j == 0) {
            double s0 = 0.0, s1 = 0.0;
            for (int jj = 0; jj < n; ++jj) { s0 += part[2 * jj]; s1 += part[2 * jj + 1]; }
            if (t == T - 1) lap_acc += s0;
            else { g[(int64_t)mat * 3 * n + (t - 1)] = s0; lap_acc -= s1; }
        }
        __syncwarp();
    }
    // combine the group-leader partial Laplacian sums
    for (int o = 16; o > 0; o >>= 1) lap_acc += __shfl_xor_sync(0xffffffffu, lap_acc, o);
    if (lane == 0) lapdet[mat] = lap_acc;
}

// Register-tiled determinant tangents, one block of 128 threads per (walker, determinant).
// For every channel t: C_t = A^-1 D_t (D_t = channel t of the Slater matrix), g_t = tr C_t and,
// for the 3n gradient channels, tr(C_t^2) = sum_aj C_aj C_ja. Each thread forms one 4 x 4 tile
// of C_t from float4 shared-memory loads (16 FMAs per two 16-byte loads), stages it, reads the
// transposed tile for its part of tr(C_t^2). A channel's traces are FP32 sums of products of
// FP32 entries (as C_t itself is FP32), formed from the tile partials by one lane per channel;
// the traces of all channels are accumulated in FP64 into
// lap = tr(A^-1 Lap A) - sum_t tr(C_t^2). Matrices are zero-padded to NP = round_up(n, 4) for n <= 32
// and to 40 for n = 33..40 (a channel's 100 tiles then leave 28 of the 128 threads idle).
template <int NP>
__global__ void __launch_bounds__(128)
k_det_tangents_tile(const float* __restrict__ MO, const float* __restrict__ Ainv, const double* __restrict__ sign,
                    int n, int T, double* __restrict__ g, double* __restrict__ lapdet) {
    constexpr int NB = NP / 4;                   // tile rows / columns
    constexpr int TPC = NB * NB;                 // tiles (threads) per channel
    constexpr int CPR = 128 / TPC;               // channels per round
    constexpr int PP = NP * NP + 4;              // channel plane pitch (floats), offset to spread banks
    __shared__ __align__(16) float AT[NP * NP];  // AT[k][a] = Ainv[a][k]
    __shared__ __align__(16) float Ds[CPR * PP];
    __shared__ float part[2][128];
    __shared__ double tr1[3 * NP + 2], tr2[3 * NP + 2];
    const int mat = blockIdx.x, tid = threadIdx.x;
    if (sign[mat] == 0.0) {
        for (int t = tid; t < 3 * n; t += 128) g[(int64_t)mat * 3 * n + t] = 0.0;
        if (tid == 0) lapdet[mat] = 0.0;
        return;
    }
    for (int e = tid; e < NP * NP; e += 128) {
        const int k = e / NP, a = e % NP;
        AT[e] = (k < n && a < n) ? __ldg(Ainv + (int64_t)mat * n * n + a * n + k) : 0.f;
    }
    const int c = tid / TPC, tile = tid % TPC, ab = tile / NB, jb = tile % NB;
    const int nn = n * n;
    // n == NP (a multiple of 4): every channel plane is one contiguous, 16-byte aligned block
    const bool vec_planes = n == NP && (((uintptr_t)MO) & 15) == 0;
    for (int t0 = 1; t0 < T; t0 += CPR) {
        const int nc = min(CPR, T - t0);
        __syncthreads();                         // previous round's readers of Ds are done
        // stage channels t0 .. t0 + nc - 1 (contiguous in MO), zero-padded to NP x NP
        const float* src = MO + ((int64_t)mat * T + t0) * nn;
        if (vec_planes) {
            // a plain copy: consecutive threads move consecutive 16-byte words of a plane
            constexpr int Q = NP * NP / 4;
            for (int q = tid; q < CPR * Q; q += 128) {
                const int cc = q / Q, r4 = q - cc * Q;
                float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                if (cc < nc) v = __ldg(reinterpret_cast<const float4*>(src + (int64_t)cc * nn) + r4);
                *reinterpret_cast<float4*>(Ds + cc * PP + 4 * r4) = v;
            }
        } else {
            // one matrix row (channel cc, row i) per thread, its padding zeroed
            for (int q = tid; q < CPR * NP; q += 128) {
                const int cc = q / NP, i = q - cc * NP;
                float* dst = Ds + cc * PP + i * NP;
                const bool live = cc < nc && i < n;
                const float* srow = src + (int64_t)cc * nn + i * n;
                #pragma unroll
                for (int j = 0; j < NP; ++j) dst[j] = (live && j < n) ? __ldg(srow + j) : 0.f;
            }
        }
        __syncthreads();
        float acc[4][4];
        #pragma unroll
        for (int x = 0; x < 4; ++x)
            #pragma unroll
            for (int y = 0; y < 4; ++y) acc[x][y] = 0.f;
        const bool on = c < nc;
        if (on) {
            const float* dp = Ds + c * PP + 4 * jb;
            const float* ap = AT + 4 * ab;
            #pragma unroll 4
            for (int k = 0; k < n; ++k) {
                const float4 av = *reinterpret_cast<const float4*>(ap + k * NP);
                const float4 dv = *reinterpret_cast<const float4*>(dp + k * NP);
                const float a4[4] = {av.x, av.y, av.z, av.w}, d4[4] = {dv.x, dv.y, dv.z, dv.w};
                #pragma unroll
                for (int x = 0; x < 4; ++x)
                    #pragma unroll
                    for (int y = 0; y < 4; ++y) acc[x][y] = fmaf(a4[x], d4[y], acc[x][y]);
            }
        }
        __syncthreads();                         // Ds is reused for C
        if (on) {
            float* cp = Ds + c * PP;
            #pragma unroll
            for (int x = 0; x < 4; ++x)
                *reinterpret_cast<float4*>(cp + (4 * ab + x) * NP + 4 * jb) =
                    make_float4(acc[x][0], acc[x][1], acc[x][2], acc[x][3]);
        }
        __syncthreads();
        float p1 = 0.f, p2 = 0.f;
        if (on) {
            // transposed tile: C[4 jb + y][4 ab + x]
            const float* cp = Ds + c * PP;
            #pragma unroll
            for (int y = 0; y < 4; ++y) {
                const float4 ct = *reinterpret_cast<const float4*>(cp + (4 * jb + y) * NP + 4 * ab);
                p2 = fmaf(acc[0][y], ct.x, p2);
                p2 = fmaf(acc[1][y], ct.y, p2);
                p2 = fmaf(acc[2][y], ct.z, p2);
                p2 = fmaf(acc[3][y], ct.w, p2);
            }
            if (ab == jb) p1 = acc[0][0] + acc[1][1] + acc[2][2] + acc[3][3];
        }
        part[0][tid] = p1;
        part[1][tid] = p2;
        __syncthreads();
        if (tid < nc) {
            float s1 = 0.f, s2 = 0.f;
            #pragma unroll 4
            for (int q = 0; q < TPC; ++q) { s1 += part[0][tid * TPC + q]; s2 += part[1][tid * TPC + q]; }
            tr1[t0 + tid] = (double)s1;
            tr2[t0 + tid] = (double)s2;
        }
    }
    __syncthreads();
    for (int t = 1 + tid; t < T - 1; t += 128) g[(int64_t)mat * 3 * n + (t - 1)] = tr1[t];
    if (tid < 32) {
        double s = 0.0;
        for (int t = 1 + tid; t < T - 1; t += 32) s += tr2[t];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (tid == 0) lapdet[mat] = tr1[T - 1] - s;
    }
}

// Instrumentation: run the single-buffer tile kernel for every n (dw_debug_set_det_tangents_kernel).
static bool g_det_tangents_tile = false;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// The traces of k_det_tangents_tile for n == NP in {4, 8, 16} (a channel's 4 x 4 tiles within one
// warp): the channel planes stream through three shared-memory buffers by cp.async (the planes of
// round r + 2 load while round r's products run), the transposed partner tile comes by shuffles
// instead of a shared-memory round trip, and a channel's partial traces are reduced by shuffles,
// so a round needs one barrier. The same products and FP32 partial sums, FP64 accumulation over
// the channels.
template <int NP>
__global__ void __launch_bounds__(128)
k_det_tangents_pipe(const float* __restrict__ MO, const float* __restrict__ Ainv, const double* __restrict__ sign,
                    int T, double* __restrict__ g, double* __restrict__ lapdet) {
    constexpr int n = NP, nn = NP * NP;
    constexpr int NB = NP / 4, TPC = NB * NB, CPR = 128 / TPC, PP = NP * NP + 4, Q = NP * NP / 4;
    static_assert(32 % TPC == 0, "a channel's tiles lie in one warp");
    __shared__ __align__(16) float AT[NP * NP];
    __shared__ __align__(16) float Ds[3][CPR * PP];
    __shared__ double tr1[3 * 32 + 2], tr2[3 * 32 + 2];
    const int mat = blockIdx.x, tid = threadIdx.x;
    if (sign[mat] == 0.0) {
        for (int t = tid; t < 3 * n; t += 128) g[(int64_t)mat * 3 * n + t] = 0.0;
        if (tid == 0) lapdet[mat] = 0.0;
        return;
    }
    const int nrounds = (T - 1 + CPR - 1) / CPR;
    // round r stages channels 1 + r CPR .. (contiguous in MO) into buffer r % 3; an empty group
    // keeps the group count uniform past the last round
    auto stage = [&](int r) {
        if (r < nrounds) {
            const int t0 = 1 + r * CPR, nc = min(CPR, T - t0);
            const float* src = MO + ((int64_t)mat * T + t0) * nn;
            float* dst = Ds[r % 3];
            for (int q = tid; q < nc * Q; q += 128) {
                const int cc = q / Q, r4 = q - cc * Q;
                cp_async16(dst + cc * PP + 4 * r4, src + (int64_t)cc * nn + 4 * r4);
            }
        }
        cp_async_commit();
    };
    stage(0);
    stage(1);
    for (int e = tid; e < nn; e += 128) {
        const int k = e / NP, a = e % NP;
        AT[e] = __ldg(Ainv + (int64_t)mat * nn + a * n + k);
    }
    const int c = tid / TPC, tile = tid % TPC, ab = tile / NB, jb = tile % NB;
    const int partner = (tid & 31 & ~(TPC - 1)) | (jb * NB + ab);      // lane of the transposed tile
    for (int r = 0; r < nrounds; ++r) {
        const int t0 = 1 + r * CPR, nc = min(CPR, T - t0);
        cp_async_wait1();                        // this thread's copies of round r have landed
        __syncthreads();                         // everyone's; round r - 1's buffer is free again
        stage(r + 2);
        const bool on = c < nc;
        float acc[4][4];
        #pragma unroll
        for (int x = 0; x < 4; ++x)
            #pragma unroll
            for (int y = 0; y < 4; ++y) acc[x][y] = 0.f;
        if (on) {
            const float* dp = Ds[r % 3] + c * PP + 4 * jb;
            const float* ap = AT + 4 * ab;
            #pragma unroll
            for (int k = 0; k < n; ++k) {
                const float4 av = *reinterpret_cast<const float4*>(ap + k * NP);
                const float4 dv = *reinterpret_cast<const float4*>(dp + k * NP);
                const float a4[4] = {av.x, av.y, av.z, av.w}, d4[4] = {dv.x, dv.y, dv.z, dv.w};
                #pragma unroll
                for (int x = 0; x < 4; ++x)
                    #pragma unroll
                    for (int y = 0; y < 4; ++y) acc[x][y] = fmaf(a4[x], d4[y], acc[x][y]);
            }
        }
        // tr(C^2) part of this tile: sum_xy C[4 ab + x][4 jb + y] C[4 jb + y][4 ab + x], the second
        // factor being the partner's acc[y][x]
        float p2 = 0.f;
        #pragma unroll
        for (int x = 0; x < 4; ++x)
            #pragma unroll
            for (int y = 0; y < 4; ++y) p2 = fmaf(acc[x][y], __shfl_sync(0xffffffffu, acc[y][x], partner), p2);
        float p1 = ab == jb ? acc[0][0] + acc[1][1] + acc[2][2] + acc[3][3] : 0.f;
        #pragma unroll
        for (int o = TPC / 2; o > 0; o >>= 1) {
            p1 += __shfl_xor_sync(0xffffffffu, p1, o);
            p2 += __shfl_xor_sync(0xffffffffu, p2, o);
        }
        if (on && tile == 0) {
            tr1[t0 + c] = (double)p1;
            tr2[t0 + c] = (double)p2;
        }
    }
    __syncthreads();
    for (int t = 1 + tid; t < T - 1; t += 128) g[(int64_t)mat * 3 * n + (t - 1)] = tr1[t];
    if (tid < 32) {
        double sacc = 0.0;
        for (int t = 1 + tid; t < T - 1; t += 32) sacc += tr2[t];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) sacc += __shfl_xor_sync(0xffffffffu, sacc, o);
        if (tid == 0) lapdet[mat] = tr1[T - 1] - sacc;
    }
}

void launch_det_tangents(const float* MO, const float* Ainv, const double* sign, const Dims& d, int B,
                         double* g, double* lapdet, cudaStream_t s) {
    int nmat = B * d.K;
    if ((d.n == 4 || d.n == 8 || d.n == 16) && d.T == 3 * d.n + 2 && (((uintptr_t)MO) & 15) == 0 && !g_det_tangents_tile) {
        auto go = [&](auto kern) { kern<<<nmat, 128, 0, s>>>(MO, Ainv, sign, d.T, g, lapdet); };
        if (d.n == 4) go(k_det_tangents_pipe<4>);
        else if (d.n == 8) go(k_det_tangents_pipe<8>);
        else go(k_det_tangents_pipe<16>);
        count_launch();
        return;
    }
    if ((d.n <= 32 || (d.n <= 40 && !g_det_tangents_tile)) && d.T == 3 * d.n + 2) {
        auto go = [&](auto kern) { kern<<<nmat, 128, 0, s>>>(MO, Ainv, sign, d.n, d.T, g, lapdet); };
        if (d.n <= 4) go(k_det_tangents_tile<4>);
        else if (d.n <= 8) go(k_det_tangents_tile<8>);
        else if (d.n <= 12) go(k_det_tangents_tile<12>);
        else if (d.n <= 16) go(k_det_tangents_tile<16>);
        else if (d.n <= 20) go(k_det_tangents_tile<20>);
        else if (d.n <= 24) go(k_det_tangents_tile<24>);
        else if (d.n <= 28) go(k_det_tangents_tile<28>);
        else if (d.n <= 32) go(k_det_tangents_tile<32>);
        else go(k_det_tangents_tile<40>);
        count_launch();
        return;
    }
    if (d.n <= 32) {
        const int n = d.n, G = 32 / n, wpb = 4;
        const int ais = (n * n + 1) & ~1, cgs = ((n * (n + 1) > 4 * n ? n * (n + 1) : 4 * n) + 1) & ~1;
        size_t sm = (size_t)wpb * (ais + G * cgs) * sizeof(float);
        if (sm > 48 * 1024) cudaFuncSetAttribute(k_det_tangents_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_det_tangents_warp<<<(nmat + wpb - 1) / wpb, wpb * 32, sm, s>>>(MO, Ainv, sign, n, d.T, nmat, g, lapdet);
        count_launch();
        return;
    }
    size_t sm = 3 * (size_t)d.n * d.n * sizeof(float);
    if (sm > 48 * 1024) cudaFuncSetAttribute(k_det_tangents, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_det_tangents<<<nmat, 128, sm, s>>>(MO, Ainv, sign, d.n, d.T, nmat, g, lapdet);
    count_launch();
}

// ------------------------------------------------------------------ Coulomb (hamiltonian.py:17-39)
// Pair terms in FP32 (each difference of two FP32 coordinates is correctly rounded, so every
// 1/r carries a few FP32 ulps of relative error, as in the reference's FP32 arithmetic), summed
// in FP64.
__device__ double coulomb_walker(const float* rb, int n, const float* R, const int32_t* Z, int N, int lane) {
    double e = 0.0;
    for (int p = lane; p < n * n; p += 32) {
        int i = p / n, j = p % n;
        if (j <= i) continue;
        const float dx = rb[j * 3] - rb[i * 3], dy = rb[j * 3 + 1] - rb[i * 3 + 1], dz = rb[j * 3 + 2] - rb[i * 3 + 2];
        e += (double)(1.f / sqrtf(dx * dx + dy * dy + dz * dz));
    }
    for (int p = lane; p < n * N; p += 32) {
        int i = p / N, I = p % N;
        if (Z[I] <= 0) continue;                                  // padding ion
        const float dx = rb[i * 3] - R[I * 3], dy = rb[i * 3 + 1] - R[I * 3 + 1], dz = rb[i * 3 + 2] - R[I * 3 + 2];
        e -= (double)((float)Z[I] / sqrtf(dx * dx + dy * dy + dz * dz));
    }
    for (int p = lane; p < N * N; p += 32) {
        int I = p / N, J = p % N;
        if (J <= I || Z[I] <= 0 || Z[J] <= 0) continue;
        const float dx = R[J * 3] - R[I * 3], dy = R[J * 3 + 1] - R[I * 3 + 1], dz = R[J * 3 + 2] - R[I * 3 + 2];
        e += (double)((float)(Z[I] * Z[J]) / sqrtf(dx * dx + dy * dy + dz * dz));
    }
    return warp_sum(e);
}

// The same sums with every difference, distance and quotient in FP64 (FP64 form).
__device__ double coulomb_walker64(const float* rb, int n, const float* R, const int32_t* Z, int N, int lane) {
    double e = 0.0;
    for (int p = lane; p < n * n; p += 32) {
        int i = p / n, j = p % n;
        if (j <= i) continue;
        const double dx = (double)rb[j * 3] - rb[i * 3], dy = (double)rb[j * 3 + 1] - rb[i * 3 + 1],
                     dz = (double)rb[j * 3 + 2] - rb[i * 3 + 2];
        e += 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
    }
    for (int p = lane; p < n * N; p += 32) {
        int i = p / N, I = p % N;
        if (Z[I] <= 0) continue;
        const double dx = (double)rb[i * 3] - R[I * 3], dy = (double)rb[i * 3 + 1] - R[I * 3 + 1],
                     dz = (double)rb[i * 3 + 2] - R[I * 3 + 2];
        e -= (double)Z[I] / sqrt(dx * dx + dy * dy + dz * dz);
    }
    for (int p = lane; p < N * N; p += 32) {
        int I = p / N, J = p % N;
        if (J <= I || Z[I] <= 0 || Z[J] <= 0) continue;
        const double dx = (double)R[J * 3] - R[I * 3], dy = (double)R[J * 3 + 1] - R[I * 3 + 1],
                     dz = (double)R[J * 3 + 2] - R[I * 3 + 2];
        e += (double)(Z[I] * Z[J]) / sqrt(dx * dx + dy * dy + dz * dz);
    }
    return warp_sum(e);
}

__global__ void k_coulomb(const float* __restrict__ r, int B, int n, const float* __restrict__ R,
                          const int32_t* __restrict__ Z, int N, float* __restrict__ E) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= B) return;
    double e = coulomb_walker(r + (int64_t)warp * n * 3, n, R, Z, N, lane);
    if (lane == 0) E[warp] = (float)e;
}

void launch_coulomb(const float* r, int B, int n, const float* R, const int32_t* Z, int N, float* E, cudaStream_t s) {
    k_coulomb<<<(B * 32 + 255) / 256, 256, 0, s>>>(r, B, n, R, Z, N, E);
    count_launch();
}

// ------------------------------------------------------------------ combine
// log psi^2 = 2 (log(|sum_k s_k e^{l_k - l_max}| + 1e-8) + l_max) + J   (wavefunction.py:77-81, :127-128)
// With tangents: grad/Laplacian of f = log(|psi~| + eps) + l_{k*} (k* = argmax), all in FP64;
// E_kin = -1/2 (1/2 Lap log psi^2 + 1/4 |grad log psi^2|^2) (hamiltonian.py:216).
__global__ void k_combine(const double* __restrict__ logdet, const double* __restrict__ sign,
                          const double* __restrict__ g, const double* __restrict__ lapdet,
                          const double* __restrict__ jas, const float* __restrict__ r, const float* __restrict__ R,
                          const int32_t* __restrict__ Z, Dims d, int B, float* __restrict__ log_psi_sqr,
                          float* __restrict__ phase, float* __restrict__ E_loc, float* __restrict__ grad_out,
                          int coul64, const int* __restrict__ nvalid, float* __restrict__ esc) {
    int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= B || (nvalid && warp >= *nvalid)) return;
    const int b = warp, K = d.K, n3 = 3 * d.n;
    const double* ld = logdet + (int64_t)b * K;
    const double* sg = sign + (int64_t)b * K;
    // lane-parallel log-sum-exp over the determinants: first maximal log|det| (ties: lowest k)
    double lmax = -INFINITY; int ks = 0;
    for (int k = lane; k < K; k += 32) if (ld[k] > lmax) { lmax = ld[k]; ks = k; }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, lmax, o);
        const int oi = __shfl_xor_sync(0xffffffffu, ks, o);
        if (ov > lmax || (ov == lmax && oi < ks)) { lmax = ov; ks = oi; }
    }
    double psi = 0.0;
    for (int k = lane; k < K; k += 32) psi += sg[k] * exp(ld[k] - lmax);
    psi = warp_sum(psi);
    const double eps = 1e-8;
    double u = fabs(psi), sgn = psi < 0 ? -1.0 : 1.0;
    double f = log(u + eps) + lmax;
    const double* jb = jas + (int64_t)b * d.Tp;
    if (lane == 0) {
        log_psi_sqr[b] = (float)(2.0 * f + jb[0]);
        if (phase) phase[b] = psi < 0 ? 3.14159265358979323846f : 0.f;
    }
    if (d.Tp == 1) return;
    // tangents; a_k = s_k e^{l_k - l_max} once per walker
    __shared__ double a_sh[8][128];
    double* ak = a_sh[threadIdx.x >> 5];
    for (int k = lane; k < K; k += 32) ak[k] = sg[k] * exp(ld[k] - lmax);
    __syncwarp();
    const double* gb = g + (int64_t)b * K * n3;
    const double* gs = gb + (int64_t)ks * n3;
    double grad_sq = 0.0, gpsi_sq = 0.0;
    // lane-parallel over coordinates
    for (int t = lane; t < n3; t += 32) {
        double gp = 0.0;
        for (int k = 0; k < K; ++k) gp += ak[k] * (gb[(int64_t)k * n3 + t] - gs[t]);
        double gf = sgn * gp / (u + eps) + gs[t];
        double gl = 2.0 * gf + jb[1 + t];
        grad_sq += gl * gl;
        gpsi_sq += gp * gp;
        if (grad_out) grad_out[(int64_t)b * n3 + t] = (float)gl;
    }
    // Laplacian of psi~
    double lp = 0.0, lpa = 0.0;
    for (int k = lane; k < K; k += 32) {
        double dg2 = 0.0;
        for (int t = 0; t < n3; ++t) { double dd = gb[(int64_t)k * n3 + t] - gs[t]; dg2 += dd * dd; }
        const double dl = lapdet[(int64_t)b * K + k] - lapdet[(int64_t)b * K + ks];
        lp += ak[k] * (dl + dg2);
        lpa += fabs(ak[k]) * (fabs(dl) + dg2);
    }
    grad_sq = warp_sum(grad_sq); gpsi_sq = warp_sum(gpsi_sq); lp = warp_sum(lp);
    if (esc) lpa = warp_sum(lpa);
    double lapf = sgn * lp / (u + eps) - gpsi_sq / ((u + eps) * (u + eps)) + lapdet[(int64_t)b * K + ks];
    double lap = 2.0 * lapf + jb[d.lap];
    double ekin = -0.5 * (0.5 * lap + 0.25 * grad_sq);
    const int gs_ = seg_of(d, b);
    const float* rb = r + (int64_t)b * d.n * 3;
    const float* Rg = R + (size_t)gs_ * d.N * 3;
    const int32_t* Zg = Z + (size_t)gs_ * d.N;
    double epot = coul64 ? coulomb_walker64(rb, d.n, Rg, Zg, d.N, lane) : coulomb_walker(rb, d.n, Rg, Zg, d.N, lane);
    if (lane == 0) E_loc[b] = (float)(ekin + epot);
    if (esc && lane == 0) {
        // error scales of this walker: the magnitude S of the terms summed into E_L, the magnitude
        // of the determinant terms summed into Lap log|psi~| (cancellation across determinants),
        // and 1 / (|psi~| + eps) (closeness to a node of the determinant sum)
        const double ue = u + eps;
        esc[3 * (int64_t)b] = (float)(0.25 * fabs(lap) + 0.125 * grad_sq + fabs(epot));
        esc[3 * (int64_t)b + 1] = (float)(lpa / ue + gpsi_sq / (ue * ue) + fabs(lapdet[(int64_t)b * K + ks]));
        esc[3 * (int64_t)b + 2] = (float)(1.0 / ue);
    }
}

void launch_combine(const double* logdet, const double* sign, const double* g, const double* lapdet, const double* jas,
                    const float* r, const float* R, const int32_t* Z, const Dims& d, int B,
                    float* log_psi_sqr, float* phase, float* E_loc, float* grad_out, cudaStream_t s, int coul64,
                    const int* nvalid, float* esc) {
    k_combine<<<(B * 32 + 255) / 256, 256, 0, s>>>(logdet, sign, g, lapdet, jas, r, R, Z, d, B, log_psi_sqr, phase,
                                                   E_loc, grad_out, coul64, nvalid, esc);
    count_launch();
}

}  // namespace dw

extern "C" {
// Test entry: the elimination kernels for n <= 16 in a chosen scalar type (0 = FP64,
// 1 = float-float) on nmat matrices of n x n FP32 entries at MO + m T n^2, with (want_inv) or
// without the FP32 inverse. Lets the two forms be compared on the same inputs.
int dw_debug_slogdet_small(const float* MO, int n, int T, int nmat, int scalar, int want_inv, double* logdet,
                           double* sign, float* Ainv, void* stream) {
    if (!MO || !logdet || !sign || n < 1 || n > 16 || T < 1 || nmat < 1 || (scalar != 0 && scalar != 1) ||
        (want_inv && !Ainv))
        return DW_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (scalar == 0) dw::launch_slogdet_small<double>(MO, n, T, nmat, logdet, sign, Ainv, want_inv != 0, s);
    else dw::launch_slogdet_small<dw::FF>(MO, n, T, nmat, logdet, sign, Ainv, want_inv != 0, s);
    return cudaGetLastError() == cudaSuccess ? DW_OK : DW_ERR_CUDA;
}

// Instrumentation: determinant-tangent kernels (0: the default choice; 1: the single-buffer tile
// kernel for n in {4, 8, 16} instead of the pipelined one, and the general kernel instead of the
// tile kernel for n = 33..40). Returns the previous choice.
int dw_debug_set_det_tangents_kernel(int which) {
    if (which != 0 && which != 1) return -DW_ERR_ARG;
    const int old = dw::g_det_tangents_tile ? 1 : 0;
    dw::g_det_tangents_tile = which == 1;
    return old;
}
}  // extern "C"
