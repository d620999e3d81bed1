// IEEE 754 binary16 rounding on the host (round to nearest, ties to even),
// for the f16 operand images of the tensor-core block kernel.
#pragma once
#include <cmath>
#include <cstdint>

namespace q1g {

// The binary16 value nearest to v: its bits, and the value itself in
// *rounded.  |v| must stay below 65520 (no overflow handling: the callers'
// operands are scaled below 2^15).
inline uint16_t host_f16_bits(double v, double* rounded)
{
    const uint16_t sign = std::signbit(v) ? 0x8000u : 0u;
    const double a = std::fabs(v);
    if (a < std::ldexp(1.0, -14)) {
        // zero and subnormals: multiples of 2^-24 (1024 * 2^-24 is the
        // smallest normal, whose bits 0x400 the same formula gives)
        const double q = std::nearbyint(std::ldexp(a, 24));
        *rounded = std::copysign(std::ldexp(q, -24), v);
        return (uint16_t)(sign | (uint16_t)q);
    }
    int e = 0;
    std::frexp(a, &e);              // a in [2^(e-1), 2^e)
    int E = e - 1;
    double q = std::nearbyint(std::ldexp(a, 10 - E));   // 11 significant bits: [1024, 2048]
    if (q == 2048.0) {
        q = 1024.0;
        ++E;
    }
    *rounded = std::copysign(std::ldexp(q, E - 10), v);
    return (uint16_t)(sign | (uint16_t)((E + 15) << 10) | (uint16_t)(q - 1024.0));
}

}  // namespace q1g
