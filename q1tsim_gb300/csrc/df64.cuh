// Complex128 arithmetic without the FP64 pipe.
//
// GB300 runs FP64 at about 2 FMA per clock per SM, so a complex 2x2 update
// of a complex128 amplitude pair (16 FMA) costs about three times its HBM
// traffic.  Here a double x is split with integer operations into two floats
// x = h + l (h = x rounded to 24 significant bits, l = x - h rounded to 24),
// products are formed exactly with FMA (TwoProd) and
// summed with error-free TwoSum (Knuth), and the result h + l is assembled
// back into a double with integer operations.  The relative error of a
// product is about 2^-47 and of a 4-term dot product about 2^-46 of its
// largest term: an absolute error of a few 1e-15 for amplitudes of modulus
// <= 1, against the complex128 tolerance of 1e-12 for whole circuits.
//
// The fast range is |x| < 2^126; split_f64 reports larger values, and callers
// then use FP64 arithmetic for that element.  Amplitudes below 2^-126 are
// flushed to zero (an absolute error under 1.2e-38).
#pragma once
#include <cstdint>
#include <cmath>
#include <cstring>

namespace q1g {

struct DF {
    float h, l;   // value h + l
};

__host__ __device__ __forceinline__ float bits_to_float(uint32_t u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    std::memcpy(&f, &u, 4);
    return f;
#endif
}

__host__ __device__ __forceinline__ uint32_t float_to_bits(float f)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
#endif
}

__host__ __device__ __forceinline__ float f_mul(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}

__host__ __device__ __forceinline__ float f_add(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}

__host__ __device__ __forceinline__ float f_sub(float a, float b)
{
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}

__host__ __device__ __forceinline__ float f_fma(float a, float b, float c)
{
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

__host__ __device__ __forceinline__ int f_to_int_rn(float f)
{
#ifdef __CUDA_ARCH__
    return __float2int_rn(f);
#else
    return (int)nearbyintf(f);
#endif
}

// x (IEEE double bits) -> h + l.  False when |x| >= 2^126 (callers then use
// FP64 for that element).  |x| < 2^-126 is flushed to a signed zero and
// 2^-126 <= |x| < 2^-74 keeps only h: absolute errors below 2^-98, far under
// the 1e-12 amplitude contract.
__host__ __device__ __forceinline__ bool split_f64(uint64_t bits, DF& out)
{
    const uint32_t hw = (uint32_t)(bits >> 32), lw = (uint32_t)bits;
    const uint32_t e = (hw >> 20) & 0x7FFu;
    const uint32_t sign = hw & 0x80000000u;
    if (e > 1149u) return false;
    if (e < 897u) {
        out.h = bits_to_float(sign);
        out.l = 0.0f;
        return true;
    }
    // h: x rounded to 24 significant bits (half up at stored bit 28; a carry
    // runs into the exponent), rebiased to single precision
    const uint64_t rb = bits + (uint64_t(1) << 28);
    const uint32_t rhw = (uint32_t)(rb >> 32);
    const uint32_t eh = (rhw >> 20) & 0x7FFu;
    out.h = bits_to_float(sign | ((eh - 896u) << 23) | ((rhw & 0xFFFFFu) << 3) | ((uint32_t)rb >> 29));
    // l = x - h: the low 29 stored bits, less 2^29 when h was rounded up, in
    // units of 2^(e - 1075) (a normal scale for e >= 949); |l| <= ulp(h) / 2
    if (e < 949u) {
        out.l = 0.0f;
        return true;
    }
    // the low 29 bits as a two's-complement number: minus 2^29 when bit 28
    // (the rounding bit) is set
    const int32_t r = (int32_t)(lw << 3) >> 3;
    out.l = f_mul((float)r, bits_to_float(sign | ((e - 948u) << 23)));
    return true;
}

// True when 2^-74 <= |x| < 2^127 (biased exponent 949..1150): split_fast
// applies.
__host__ __device__ __forceinline__ bool split_fast_ok(uint64_t bits)
{
    return ((uint32_t)(bits >> 32) & 0x7FFFFFFFu) - (949u << 20) < (202u << 20);
}

// split_f64 for |x| in split_fast_ok's range, in fewer operations: h's
// exponent and significand come from the rounded bit pattern shifted by 29
// (the exponent rebiased in place: its low 9 bits suffice since the result
// fits in 8), l's scale from x's own exponent.
__host__ __device__ __forceinline__ DF split_fast(uint64_t bits)
{
    const uint32_t hw = (uint32_t)(bits >> 32), lw = (uint32_t)bits;
    const uint32_t sign = hw & 0x80000000u;
    const uint32_t t = (uint32_t)((bits + (uint64_t(1) << 28)) >> 29);
    const float h = bits_to_float((t - (896u << 23)) | sign);
    const int32_t r = (int32_t)(lw << 3) >> 3;
    const float l = f_mul((float)r, bits_to_float((((hw << 3) & 0xFF800000u) - (948u << 23)) | sign));
    return DF{h, l};
}

// h + l, a pair normalised so that |l| <= ulp(h) / 2, as IEEE double bits.
// h's double encoding has its low 29 significand bits clear; l, rounded to
// units of h's double ulp, is added to the encoding as an integer, so a
// borrow below a power of two runs into the exponent (l is then measured in
// the halved ulp of the binade below).  |h| < 2^-126 gives a signed zero;
// for |h| < 2^-74 l is dropped.
__host__ __device__ __forceinline__ uint64_t join_f64(DF v)
{
    const uint32_t hb = float_to_bits(v.h), lb = float_to_bits(v.l);
    const uint32_t sign = hb & 0x80000000u;
    const uint32_t eh = (hb >> 23) & 0xFFu;
    if (eh == 0) return (uint64_t)sign << 32;
    const uint32_t mh = hb & 0x7FFFFFu;
    uint64_t mag = ((uint64_t)(((eh + 896u) << 20) | (mh >> 3)) << 32) | ((uint64_t)(mh & 7u) << 29);
    if (eh >= 53u && (lb & 0x7FFFFFFFu) != 0) {
        const bool opposite = ((lb ^ hb) & 0x80000000u) != 0;
        const uint32_t down = (mh == 0 && opposite) ? 1u : 0u;   // h a power of two, result below it
        // |l| in units of 2^(e_h - 52 - down), e_h = eh - 127
        const int lm = f_to_int_rn(f_mul(bits_to_float(lb & 0x7FFFFFFFu), bits_to_float((306u - eh + down) << 23)));
        mag = opposite ? mag - (uint64_t)lm : mag + (uint64_t)lm;
    }
    return ((uint64_t)sign << 32) | mag;
}

// A matrix coefficient as a double-float pair on the host (split_f64; a
// value outside the split's range becomes the nearest float pair).
inline DF host_split(double v)
{
    uint64_t b;
    std::memcpy(&b, &v, 8);
    DF d{0.0f, 0.0f};
    if (!split_f64(b, d)) {
        d.h = (float)v;
        d.l = (float)(v - (double)d.h);
    }
    return d;
}

// sum_k a[k] * b[k] over N double-float terms, normalised (|l| <= ulp(h)/2).
template <int N>
__host__ __device__ __forceinline__ DF dot(const DF* a, const DF* b)
{
    float p[N], lo = 0.0f;
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int k = 0; k < N; ++k) {
        p[k] = f_mul(a[k].h, b[k].h);
        // exact error of the leading product, then the two cross terms
        const float e = f_fma(a[k].h, b[k].h, -p[k]);
        lo = f_add(lo, f_fma(a[k].l, b[k].h, f_fma(a[k].h, b[k].l, e)));
    }
    // TwoSum chain over the leading products
    float s = p[0];
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
    for (int k = 1; k < N; ++k) {
        const float t = f_add(s, p[k]);
        const float bv = f_sub(t, s);
        const float av = f_sub(t, bv);
        lo = f_add(lo, f_add(f_sub(s, av), f_sub(p[k], bv)));
        s = t;
    }
    // TwoSum (s may be smaller than lo after cancellation): normalise
    const float h = f_add(s, lo);
    const float bv = f_sub(h, s);
    const float av = f_sub(h, bv);
    return DF{h, f_add(f_sub(s, av), f_sub(lo, bv))};
}

__host__ __device__ __forceinline__ DF dot4(const DF* a, const DF* b) { return dot<4>(a, b); }

#ifdef __CUDACC__
// Two N-term double-float dot products at once, one per lane of packed
// FP32x2 instructions (sm_100+): a[k] = (ah[k], al[k]) times b[k] = (bh[k],
// bl[k]) summed as in dot<N>; lane 0 and lane 1 are independent.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

template <int N>
__device__ __forceinline__ void dot_x2(const float2* ah, const float2* al, const float2* bh, const float2* bl,
                                       float2& h, float2& l)
{
    float2 p[N], lo = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int k = 0; k < N; ++k) {
        p[k] = __fmul2_rn(ah[k], bh[k]);
        const float2 e = __ffma2_rn(ah[k], bh[k], neg2(p[k]));
        lo = __fadd2_rn(lo, __ffma2_rn(al[k], bh[k], __ffma2_rn(ah[k], bl[k], e)));
    }
    float2 s = p[0];
#pragma unroll
    for (int k = 1; k < N; ++k) {
        const float2 t = __fadd2_rn(s, p[k]);
        const float2 bv = __fadd2_rn(t, neg2(s));
        const float2 av = __fadd2_rn(t, neg2(bv));
        lo = __fadd2_rn(lo, __fadd2_rn(__fadd2_rn(s, neg2(av)), __fadd2_rn(p[k], neg2(bv))));
        s = t;
    }
    h = __fadd2_rn(s, lo);
    const float2 bv = __fadd2_rn(h, neg2(s));
    const float2 av = __fadd2_rn(h, neg2(bv));
    l = __fadd2_rn(__fadd2_rn(s, neg2(av)), __fadd2_rn(lo, neg2(bv)));
}
#endif

}  // namespace q1g
