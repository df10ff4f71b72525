// Host check of the integer-pipe FP64 <-> FP32 conversions of dg_convert.cuh against the host's own
// conversions (IEEE round to nearest even), bit for bit: random bit patterns over every exponent,
// random values in the working range, exact ties between adjacent binary32 values and their
// neighbours, and the edges of the binary32 range.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <random>

#include "../../horses3d_gb300/csrc/cuda/dg_convert.cuh"

static uint32_t fbits(float f) { uint32_t b; std::memcpy(&b, &f, 4); return b; }
static uint64_t dbits(double d) { uint64_t b; std::memcpy(&b, &d, 8); return b; }
static double dfrom(uint64_t b) { double d; std::memcpy(&d, &b, 8); return d; }
static float ffrom(uint32_t b) { float f; std::memcpy(&f, &b, 4); return f; }

static long n_narrow = 0, n_widen = 0, n_fallback = 0, n_bad = 0;

static void check(double x) {
    const uint64_t u = dbits(x);
    uint32_t out;
    if (dg::f32_bits_from_f64(static_cast<uint32_t>(u >> 32), static_cast<uint32_t>(u), out)) {
        ++n_narrow;
        const float ref = static_cast<float>(x);
        if (out != fbits(ref)) {
            if (n_bad < 10) std::printf("narrow mismatch %a -> %a (host %a)\n", x, ffrom(out), ref);
            ++n_bad;
        }
    } else {
        ++n_fallback;
    }
    const float f = static_cast<float>(x);
    uint32_t hi, lo;
    if (dg::f64_bits_from_f32(fbits(f), hi, lo)) {
        ++n_widen;
        const uint64_t w = (static_cast<uint64_t>(hi) << 32) | lo;
        if (w != dbits(static_cast<double>(f))) {
            if (n_bad < 10) std::printf("widen mismatch %a\n", f);
            ++n_bad;
        }
    }
}

int main() {
    std::mt19937_64 rng(20261204);
    for (long i = 0; i < 4000000; ++i) check(dfrom(rng()));  // every exponent, NaN and inf included
    std::uniform_real_distribution<double> ex(-130.0, 130.0), mant(1.0, 2.0);
    for (long i = 0; i < 4000000; ++i) {
        const double x = std::ldexp(mant(rng), static_cast<int>(std::floor(ex(rng))));
        check((rng() & 1) ? x : -x);
    }
    for (long i = 0; i < 2000000; ++i) {  // ties between adjacent floats and their double neighbours
        const float a = ffrom(static_cast<uint32_t>(rng()) & 0x7F7FFFFFu);
        const float b = std::nextafter(a, std::numeric_limits<float>::infinity());
        const double mid = 0.5 * (static_cast<double>(a) + static_cast<double>(b));
        check(mid);
        check(-mid);
        check(std::nextafter(mid, 0.0));
        check(std::nextafter(mid, 1e300));
    }
    const double edges[] = {0.0, -0.0, 1.0, -1.0, std::ldexp(1.0, -126), std::nextafter(std::ldexp(1.0, -126), 0.0),
                            std::ldexp(1.0, -149), static_cast<double>(std::numeric_limits<float>::max()),
                            std::nextafter(static_cast<double>(std::numeric_limits<float>::max()), 1e300),
                            std::ldexp(1.0, 128) - std::ldexp(1.0, 103), std::ldexp(1.0, 128), 1e300, -1e300,
                            std::numeric_limits<double>::infinity(), std::numeric_limits<double>::quiet_NaN(),
                            std::numeric_limits<double>::denorm_min()};
    for (double x : edges) {
        check(x);
        check(-x);
    }
    std::printf("narrowed %ld widened %ld fallback %ld mismatches %ld\n", n_narrow, n_widen, n_fallback, n_bad);
    return n_bad == 0 ? 0 : 1;
}
