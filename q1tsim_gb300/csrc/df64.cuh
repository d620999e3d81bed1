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
// The fast range is 2^-74 <= |x| < 2^126 (and x = 0); split_f64 reports any
// other value, and callers then use FP64 arithmetic for that element.
#pragma once
#include <cstdint>
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

// x (IEEE double bits) -> h + l.  False when x is outside the fast range.
__host__ __device__ __forceinline__ bool split_f64(uint64_t bits, DF& out)
{
    const uint32_t hw = (uint32_t)(bits >> 32), lw = (uint32_t)bits;
    const uint32_t e = (hw >> 20) & 0x7FFu;
    const uint32_t sign = hw & 0x80000000u;
    if (e == 0 && (hw & 0xFFFFFu) == 0 && lw == 0) {   // +-0
        out.h = bits_to_float(sign);
        out.l = 0.0f;
        return true;
    }
    if (e < 949u || e > 1149u) return false;
    // h: x rounded to 24 significant bits (half up at stored bit 28; a carry
    // runs into the exponent), rebiased to single precision
    const uint64_t rb = bits + (uint64_t(1) << 28);
    const uint32_t rhw = (uint32_t)(rb >> 32);
    const uint32_t eh = (rhw >> 20) & 0x7FFu;
    out.h = bits_to_float(sign | ((eh - 896u) << 23) | ((rhw & 0xFFFFFu) << 3) | ((uint32_t)rb >> 29));
    // l = x - h: the low 29 stored bits, less 2^29 when h was rounded up, in
    // units of 2^(e - 1075) (e >= 949: a normal scale); |l| <= ulp(h) / 2
    const int32_t r = (int32_t)(lw & 0x1FFFFFFFu) - ((lw & 0x10000000u) ? 0x20000000 : 0);
    const float l = f_mul((float)r, bits_to_float((e - 948u) << 23));
    out.l = sign ? -l : l;
    return true;
}

// h + l, a pair normalised so that |l| <= ulp(h) / 2, as IEEE double bits
// (truncated: error below one unit in the last place).  |h| < 2^-126 is
// returned as a signed zero.
__host__ __device__ __forceinline__ uint64_t join_f64(DF v)
{
    const uint32_t hb = float_to_bits(v.h), lb = float_to_bits(v.l);
    const uint64_t sign = (uint64_t)(hb >> 31) << 63;
    const uint32_t eh = (hb >> 23) & 0xFFu;
    if (eh == 0) return sign;
    uint64_t m = (uint64_t)((hb & 0x7FFFFFu) | 0x800000u) << 29;   // 53-bit significand
    int ed = (int)eh + 896;
    const uint32_t el = (lb >> 23) & 0xFFu;
    if (el != 0) {
        const uint64_t ml = (lb & 0x7FFFFFu) | 0x800000u;
        const int sh = (int)el - (int)eh + 29;   // <= 5 for a normalised pair
        const uint64_t lm = sh >= 0 ? (ml << sh) : (sh > -32 ? (ml >> -sh) : 0);
        if ((lb >> 31) == (hb >> 31)) m += lm;
        else m -= lm;
        if (m >= (uint64_t(1) << 53)) {
            m >>= 1;
            ++ed;
        } else if (m < (uint64_t(1) << 52)) {   // h a power of two, l of the other sign
            m <<= 1;
            --ed;
        }
    }
    return sign | ((uint64_t)ed << 52) | (m & ((uint64_t(1) << 52) - 1));
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

}  // namespace q1g
