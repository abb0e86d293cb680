// Float-float ("double-FP32") arithmetic for the determinant kernels.
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with |lo| <= ulp(hi) / 2, about 48
// significant bits. On this part FP64 arithmetic issues at about 1/100 of the FP32 rate, so an
// elimination step of ~15 FP32 instructions is several times cheaper than one FP64 FMA.
// The error-free transformations are the published ones: TwoSum (Knuth, TAOCP vol. 2, 4.2.2),
// Fast2Sum (Dekker 1971) and the exact product error of an FMA (fma(a, b, -ab)); the
// add / multiply compositions follow the "sloppy" double-word forms of Dekker's add2 / mul2
// (also the dd_real forms of Hida, Li and Bailey's QD library): relative error a few 2^-48 of
// the operands. Every rounding step is an explicit round-to-nearest intrinsic so the compiler
// cannot contract a product and a sum into one FMA (which would break the error-free steps).
// Range: the low words stay normal while the values exceed ~1e-30; for smaller values (an
// envelope of 1e-30 is an electron ~50 bohr from every nucleus) they become subnormal and the
// accuracy falls gradually toward FP32's.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace dw {

#if defined(__CUDA_ARCH__)
#define DW_FADD(a, b) __fadd_rn((a), (b))
#define DW_FSUB(a, b) __fsub_rn((a), (b))
#define DW_FMUL(a, b) __fmul_rn((a), (b))
#define DW_FDIV(a, b) __fdiv_rn((a), (b))
#else
#define DW_FADD(a, b) ((a) + (b))
#define DW_FSUB(a, b) ((a) - (b))
#define DW_FMUL(a, b) ((a) * (b))
#define DW_FDIV(a, b) ((a) / (b))
#endif

struct __align__(8) FF {
    float hi, lo;
};

__host__ __device__ __forceinline__ FF ff_make(float x) { return FF{x, 0.f}; }

// Fast2Sum: h + l with |h| >= |l| (or h == 0) as a normalised pair
__host__ __device__ __forceinline__ FF ff_norm(float h, float l) {
    const float s = DW_FADD(h, l);
    return FF{s, DW_FSUB(l, DW_FSUB(s, h))};
}

// a * b
__host__ __device__ __forceinline__ FF ff_mul(FF a, FF b) {
    const float p = DW_FMUL(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return ff_norm(p, e);
}

// a + b
__host__ __device__ __forceinline__ FF ff_add(FF a, FF b) {
    const float s = DW_FADD(a.hi, b.hi);                     // TwoSum(a.hi, b.hi) = s + t exactly
    const float v = DW_FSUB(s, a.hi);
    const float t = DW_FADD(DW_FSUB(a.hi, DW_FSUB(s, v)), DW_FSUB(b.hi, v));
    return ff_norm(s, DW_FADD(t, DW_FADD(a.lo, b.lo)));
}

// a - l u (the elimination update)
__host__ __device__ __forceinline__ FF ff_fnma(FF l, FF u, FF a) {
    const float p = DW_FMUL(l.hi, u.hi);
    float pe = fmaf(l.hi, u.hi, -p);                          // l u = p + pe (to ~2^-48)
    pe = fmaf(l.hi, u.lo, pe);
    pe = fmaf(l.lo, u.hi, pe);
    const float s = DW_FSUB(a.hi, p);                         // TwoSum(a.hi, -p) = s + t exactly
    const float v = DW_FSUB(s, a.hi);
    const float t = DW_FADD(DW_FSUB(a.hi, DW_FSUB(s, v)), DW_FSUB(-p, v));
    return ff_norm(s, DW_FADD(t, DW_FSUB(a.lo, pe)));
}

__host__ __device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.hi, -a.lo}; }

// 1 / p for |p.hi| in the normal range: the correctly rounded FP32 reciprocal r plus one
// Newton correction r (1 - p r), whose residual an FMA forms exactly (relative error ~2^-46)
__host__ __device__ __forceinline__ FF ff_recip(FF p) {
#if defined(__CUDA_ARCH__)
    const float r = __frcp_rn(p.hi);
#else
    const float r = 1.0f / p.hi;
#endif
    float e = fmaf(-p.hi, r, 1.0f);
    e = fmaf(-p.lo, r, e);
    return ff_norm(r, DW_FMUL(r, e));
}

// a / b by long division: q1 = a.hi / b.hi, q2 = (a - q1 b).hi / b.hi
__host__ __device__ __forceinline__ FF ff_div(FF a, FF b) {
    const float q1 = DW_FDIV(a.hi, b.hi);
    const FF r = ff_fnma(ff_make(q1), b, a);
    return ff_norm(q1, DW_FDIV(r.hi, b.hi));
}

// Whether 1 / p.hi is a normal FP32 number (|p.hi| in [2^-125, 2^125]), so that a * (1 / p)
// can stand in for a / p.
__host__ __device__ __forceinline__ bool ff_recip_ok(FF p) {
    const float a = fabsf(p.hi);
    return a >= 2.35098870e-38f && a <= 4.25352959e+37f;
}

// Splits |a| into 2^e f with f in [1, 2) (hi part), scaling both parts by the same power of two.
__host__ __device__ __forceinline__ FF ff_frexp1(FF a, int& e) {
    const float h = fabsf(a.hi), l = a.hi < 0.f ? -a.lo : a.lo;
#if defined(__CUDA_ARCH__)
    const int b = __float_as_int(h) >> 23;                    // biased exponent of |hi|
    if (b >= 2 && b <= 252) {
        const float s = __int_as_float((254 - b) << 23);      // 2^(127 - b), a normal number
        e += b - 127;
        return FF{DW_FMUL(h, s), DW_FMUL(l, s)};
    }
#endif
    int k;
    const float f = frexpf(h, &k);                            // h = f 2^k, f in [0.5, 1)
    e += k - 1;
    return FF{2.f * f, ldexpf(l, 1 - k)};
}

// Running product of pivot magnitudes as a mantissa in [0.5, 1) and a binary exponent.
__host__ __device__ __forceinline__ void ff_mant_mul(FF& mant, FF p, int& expo) {
    const FF f = ff_frexp1(p, expo);                          // [1, 2)
    FF m = ff_mul(mant, f);                                   // [0.5, 2)
    if (m.hi >= 1.f) { m.hi *= 0.5f; m.lo *= 0.5f; ++expo; }
    mant = m;
}

// FF constants c = hi + lo (hi the nearest float, lo the nearest float to the rest)
#define DW_FF_CONST(name, v) \
    constexpr float name##_hi = (float)(v); \
    constexpr float name##_lo = (float)((v) - (double)(float)(v));
DW_FF_CONST(kFfThird, 1.0 / 3.0)
DW_FF_CONST(kFfFifth, 1.0 / 5.0)
DW_FF_CONST(kFfSeventh, 1.0 / 7.0)
#undef DW_FF_CONST

// log(mant) + expo ln 2 for mant in [0.5, 1). With m = mant (or 2 mant below 1/sqrt 2, and one
// ln 2 less) in [1/sqrt 2, sqrt 2): log m = 2 atanh z = 2 (z + z^3/3 + z^5/5 + ...),
// z = (m - 1) / (m + 1), |z| <= 0.1716 (z^2 <= 0.0295). The terms from z^9 on (together below
// 1e-7 of the sum) are summed in FP32, the leading ones in float-float; truncation after z^21
// leaves < 1e-17. The sum with expo ln 2 is formed in FP64 (absolute error ~1e-14).
__host__ __device__ __forceinline__ double ff_log_mant(FF mant, int expo) {
    if (mant.hi < 0.70710678f) { mant.hi *= 2.f; mant.lo *= 2.f; --expo; }
    const FF num = ff_norm(DW_FSUB(mant.hi, 1.f), mant.lo);   // m.hi - 1 is exact (Sterbenz)
    const FF den = ff_add(mant, ff_make(1.f));
    const FF z = ff_div(num, den);
    const FF z2 = ff_mul(z, z);
    const float w = z2.hi;
    float tail = 1.f / 21.f;                                  // z^8 (1/9 + z^2/11 + ... + z^12/21)
    tail = fmaf(tail, w, 1.f / 19.f);
    tail = fmaf(tail, w, 1.f / 17.f);
    tail = fmaf(tail, w, 1.f / 15.f);
    tail = fmaf(tail, w, 1.f / 13.f);
    tail = fmaf(tail, w, 1.f / 11.f);
    tail = fmaf(tail, w, 1.f / 9.f);
    FF s = ff_add(ff_mul(ff_make(tail), z2), FF{kFfSeventh_hi, kFfSeventh_lo});
    s = ff_add(ff_mul(s, z2), FF{kFfFifth_hi, kFfFifth_lo});
    s = ff_add(ff_mul(s, z2), FF{kFfThird_hi, kFfThird_lo});
    s = ff_add(ff_mul(s, z2), ff_make(1.f));
    const FF lm = ff_mul(z, s);                               // log m / 2
    return 2.0 * ((double)lm.hi + (double)lm.lo) + (double)expo * 0.69314718055994530942;
}

}  // namespace dw
