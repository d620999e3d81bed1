// IEEE 754 binary16 rounding on the host (round to nearest, ties to even),
// for the f16 operand images of the tensor-core block kernel.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace q1g {

// The binary16 value nearest to v: its bits, and the value itself in
// *rounded.  |v| must stay below 65520 (no overflow handling: the callers'
// operands are scaled below 2^15).  Integer rounding on the bits of the
// double: an image of 8192 values is built for every tensor-core pass, and
// at small states the host builds them while the device runs passes of a
// few microseconds.
inline uint16_t host_f16_bits(double v, double* rounded)
{
    uint64_t b;
    std::memcpy(&b, &v, sizeof b);
    const uint64_t sign = b & 0x8000000000000000ull;
    const uint64_t a = b ^ sign;                        // |v|
    const int e = (int)(a >> 52) - 1023;                // unbiased exponent
    uint64_t out;
    uint16_t h;
    if (e >= -14) {
        // normal binary16: keep 11 significant bits of the 53
        const uint64_t m = (a & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        uint64_t q = m >> 42;                           // [1024, 2047]
        const uint64_t rem = m & ((1ull << 42) - 1), half = 1ull << 41;
        if (rem > half || (rem == half && (q & 1))) ++q;
        int E = e;
        if (q == 2048) {
            q = 1024;
            ++E;
        }
        h = (uint16_t)(((E + 15) << 10) | (int)(q - 1024));
        out = sign | ((uint64_t)(E + 1023) << 52) | ((q - 1024) << 42);
    } else {
        // zero and subnormals: multiples of 2^-24, the integer rounded to
        // nearest even by adding and subtracting 2^52 (the count is below
        // 2^11, so the sum is exact up to that one rounding); 1024 * 2^-24
        // is the smallest normal, whose bits 0x400 the same count gives
        double x;
        std::memcpy(&x, &a, sizeof x);
        const double q = (x * 16777216.0 + 4503599627370496.0) - 4503599627370496.0;
        h = (uint16_t)q;
        const double r = q * (1.0 / 16777216.0);
        std::memcpy(&out, &r, sizeof out);
        out |= sign;
    }
    std::memcpy(rounded, &out, sizeof *rounded);
    return (uint16_t)((sign >> 48) | h);
}

}  // namespace q1g
