// CPU check of miccai2016_gb300/csrc/ffsincos.cuh (the double-float sin/cos of
// the ridge and direction kernels), built with g++ -ffp-contract=off so every
// float operation rounds as the device intrinsics do.  For every stride-th
// float in [-limit, limit] it compares against long double sinl/cosl:
//   * the double-float values' relative error (max reported; must stay below
//     the header's bound kRelErr),
//   * every result the header calls certain must equal the float rounding of
//     the long double value.
// Prints: values checked, certain, mismatches, max relative error of sin and cos.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../miccai2016_gb300/csrc/ffsincos.cuh"

int main(int argc, char **argv)
{
    const long stride = argc > 1 ? atol(argv[1]) : 1;
    const float limit = argc > 2 ? (float)atof(argv[2]) : 4.0f;
    uint32_t top;
    std::memcpy(&top, &limit, 4);
    long checked = 0, certain = 0, mismatches = 0;
    double max_es = 0, max_ec = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : checked, certain, mismatches) reduction(max : max_es, max_ec)
    for (long chunk = 0; chunk <= (long)(top >> 16); ++chunk) {
        for (uint32_t u = (uint32_t)chunk << 16; u < ((uint32_t)chunk + 1) << 16 && u <= top; u += (uint32_t)stride) {
            for (int sign = 0; sign < 2; ++sign) {
                float x;
                const uint32_t b = u | (sign ? 0x80000000u : 0u);
                std::memcpy(&x, &b, 4);
                m16::ff::F2 s, c;
                if (!m16::ff::sincos_f2(x, &s, &c)) continue;
                ++checked;
                const long double S = sinl((long double)x), C = cosl((long double)x);
                if (S != 0) {
                    const double e = (double)fabsl(((long double)s.h + (long double)s.l - S) / S);
                    if (e > max_es) max_es = e;
                }
                if (C != 0) {
                    const double e = (double)fabsl(((long double)c.h + (long double)c.l - C) / C);
                    if (e > max_ec) max_ec = e;
                }
                float sr, cr;
                if (m16::ff::sincos_rn(x, &sr, &cr)) {
                    ++certain;
                    if (sr != (float)S || cr != (float)C) ++mismatches;
                }
            }
        }
    }
    printf("%ld %ld %ld %.6e %.6e\n", checked, certain, mismatches, max_es, max_ec);
    return mismatches != 0;
}
