// CPU check of the f16 operands of the tensor-core pass (libq1gpu.so, built
// by tests/test_host_logic.py):
//   - host_f16_bits: the doubles of argv[1] (raw float64) rounded to binary16,
//     their bits printed one per line (hex) for the test to compare with
//     numpy's float16 conversion;
//   - build_tc_image: the image of a random unitary 32x32 matrix, read back
//     through the SWIZZLE_128B layout, gives hi + 2^-11 lo = 2^s R to 2^-22
//     of the largest entry, at the scales s = 14 and 0 of a pass's last and
//     first block;
//   - tc_operand_scales and tc_block_bounded on known cases.
// The first output line is "bad <n>"; exit status 1 on any failure.
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "../../q1tsim_gb300/csrc/common.cuh"
#include "../../q1tsim_gb300/csrc/f16_host.h"
#include "../../q1tsim_gb300/csrc/kernels.h"

using namespace q1g;
typedef std::complex<double> cd;

static double f16_value(uint16_t b)
{
    const int sign = b >> 15, e = (b >> 10) & 31, m = b & 1023;
    const double v = e == 0 ? std::ldexp((double)m, -24) : std::ldexp((double)(1024 + m), e - 25);
    return sign ? -v : v;
}

static std::vector<cd> random_unitary(int n, std::mt19937_64& rng)
{
    std::normal_distribution<double> nd;
    std::vector<cd> a((size_t)n * n);
    for (auto& x : a) x = cd(nd(rng), nd(rng));
    // Gram-Schmidt on the rows
    for (int r = 0; r < n; ++r) {
        for (int p = 0; p < r; ++p) {
            cd dot = 0;
            for (int c = 0; c < n; ++c) dot += std::conj(a[(size_t)p * n + c]) * a[(size_t)r * n + c];
            for (int c = 0; c < n; ++c) a[(size_t)r * n + c] -= dot * a[(size_t)p * n + c];
        }
        double nn = 0;
        for (int c = 0; c < n; ++c) nn += std::norm(a[(size_t)r * n + c]);
        for (int c = 0; c < n; ++c) a[(size_t)r * n + c] /= std::sqrt(nn);
    }
    return a;
}

int main(int argc, char** argv)
{
    int bad = 0;
    std::vector<uint16_t> bits;
    if (argc > 1) {
        FILE* f = std::fopen(argv[1], "rb");
        if (!f) return 2;
        double v;
        while (std::fread(&v, sizeof(double), 1, f) == 1) {
            double r = 0.0;
            const uint16_t b = host_f16_bits(v, &r);
            if (r != f16_value(b)) ++bad;      // the rounded value is the one the bits encode
            bits.push_back(b);
        }
        std::fclose(f);
    }

    std::mt19937_64 rng(7);
    double worst = 0.0;
    for (int trial = 0; trial < 20; ++trial) {
        const auto u = random_unitary(32, rng);
        std::vector<double> m(2 * 32 * 32);
        for (int e = 0; e < 32 * 32; ++e) {
            m[2 * e] = u[e].real();
            m[2 * e + 1] = u[e].imag();
        }
        const int sl = trial % 2 ? kTcLastBScaleLog2 : 0;
        std::vector<uint16_t> img(kTcImageHalves);
        build_tc_image(m.data(), img.data(), sl);
        for (int gp = 0; gp < 32; ++gp)
            for (int g = 0; g < 32; ++g) {
                const double re = m[2 * (gp * 32 + g)], im = m[2 * (gp * 32 + g) + 1];
                const double rv[2][2] = {{re, -im}, {im, re}};
                for (int cp = 0; cp < 2; ++cp)
                    for (int c = 0; c < 2; ++c) {
                        const int n = 2 * gp + cp, k = 2 * g + c;
                        auto at = [&](int row) {
                            const size_t off = (size_t)(row >> 3) * 1024 + (size_t)(row & 7) * 128 +
                                               (size_t)(((k >> 3) ^ (row & 7)) << 4) + (size_t)(k & 7) * 2;
                            return f16_value(img[off / 2]);
                        };
                        const double got = at(n) + std::ldexp(at(n + 64), -11);
                        const double want = std::ldexp(rv[cp][c], sl);
                        worst = std::max(worst, std::fabs(got - want) / std::ldexp(1.0, sl));
                    }
            }
        if (!tc_block_bounded(u.data(), 32)) ++bad;
        std::vector<cd> big(u);
        for (auto& x : big) x *= 1.001;
        if (tc_block_bounded(big.data(), 32)) ++bad;
    }
    if (!(worst <= std::ldexp(1.0, -22))) ++bad;

    TcOffsets o{};
    tc_operand_scales(1.0, o);
    if (o.ascale != 16384.0f || o.unscale != std::ldexp(1.0f, -28)) ++bad;
    tc_operand_scales(3.9, o);        // sqrt(3.9) < 2: amplitudes times 2^13
    if (o.ascale != 8192.0f || o.unscale != std::ldexp(1.0f, -27)) ++bad;
    tc_operand_scales(0.0, o);
    if (o.ascale != 16384.0f) ++bad;

    std::printf("bad %d worst %.3e\n", bad, worst);
    for (uint16_t b : bits) std::printf("%04x\n", (unsigned)b);
    return bad ? 1 : 0;
}
