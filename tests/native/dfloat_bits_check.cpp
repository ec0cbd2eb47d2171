// Host check of the integer FP64 <-> FP32-pair conversions used by the element kernel
// (edelweissfe_gb300/csrc/dfloat_bits.h) against the exact conversions of the C++ compiler.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>

#include "../../edelweissfe_gb300/csrc/dfloat_bits.h"

static float as_float(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}
static uint64_t bits(double d) {
    uint64_t b;
    std::memcpy(&b, &d, 8);
    return b;
}
static double as_double(uint64_t b) {
    double d;
    std::memcpy(&d, &b, 8);
    return d;
}

int main() {
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> ue(-125.0, 127.0), um(-1.0, 1.0);
    long bad = 0, n = 0;
    double worst = 0.0;
    for (int t = 0; t < 2000000; ++t) {
        double d = um(g) * std::exp2(ue(g));
        if (t % 7 == 0) d = std::ldexp((double)(g() >> 11), (int)(g() % 200) - 150);  // random 53-bit significands
        uint32_t hb, lb;
        ef::split_bits(bits(d), &hb, &lb);
        const float hi = as_float(hb), lo = as_float(lb);
        const double ad = std::fabs(d);
        if (ad < std::ldexp(1.0, -126)) {
            bad += (hi != 0.0f || lo != 0.0f);
            continue;
        }
        ++n;
        // hi: d truncated to 24 significant bits
        const double trunc = std::ldexp(std::trunc(std::ldexp(d, 23 - std::ilogb(d))), std::ilogb(d) - 23);
        bad += ((double)hi != trunc);
        const double aerr = std::fabs(d - ((double)hi + (double)lo));
        if (!(aerr <= std::fmax(std::ldexp(ad, -47), std::ldexp(1.0, -149)))) ++bad;
        if (ad >= std::ldexp(1.0, -97) && aerr / ad > worst) worst = aerr / ad;
        // widening is exact (subnormals included)
        bad += (as_double(ef::widen_bits(hb)) != (double)hi);
        bad += (as_double(ef::widen_bits(lb)) != (double)lo);
    }
    // special values
    const double sp[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, 1.0, -1.0, 1e300, -1e-300, 3.0e38, 3.5e38};
    for (double d : sp) {
        uint32_t hb, lb;
        ef::split_bits(bits(d), &hb, &lb);
        const float hi = as_float(hb), lo = as_float(lb);
        if (std::isnan(d)) bad += !std::isnan(hi);
        else if (std::fabs(d) > 3.4028234663852886e38) bad += !(std::isinf(hi) && std::signbit(hi) == std::signbit(d));
        else if (std::fabs(d) < std::ldexp(1.0, -126)) bad += (hi != 0.0f || lo != 0.0f);
        else bad += (std::fabs(d - ((double)hi + (double)lo)) > std::ldexp(std::fabs(d), -47));
    }
    bad += !std::isnan(as_double(ef::widen_bits(0x7FC00000u)));
    bad += !std::isinf(as_double(ef::widen_bits(0xFF800000u)));
    bad += (as_double(ef::widen_bits(0x00000001u)) != std::ldexp(1.0, -149));  // smallest subnormal
    bad += (as_double(ef::widen_bits(0x80400000u)) != -std::ldexp(1.0, -127));
    std::printf("checked %ld values, worst relative error (|d| >= 2^-97) %.3e, failures %ld\n", n, worst, bad);
    return bad == 0 ? 0 : 1;
}
