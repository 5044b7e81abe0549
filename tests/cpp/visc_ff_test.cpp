// Host check of the float-float viscosity (nextsimdg_gb300/csrc/nsdg_visc_ff.hpp):
// the float-float form and the FP64 Newton form against each other and
// against P / sqrt(inv + DeltaMin^2) correctly rounded to float (evaluated in
// long double), over seeded samples of the strain invariant, the pressure
// term and DeltaMin, and seeds up to 3 ulps away from the nearest float of
// 1/sqrt(t) (the device seed, rsqrtf, is within 2 ulps); and the checked
// float-float form: wherever it reports its result exact, bitwise the FP64
// form's.
// Build with -ffp-contract=off.  Prints "key value" lines.
#include "nsdg_visc_ff.hpp"

#include <cinttypes>
#include <cmath>
#include <cstdint>
#include <cstdio>

namespace {

uint64_t state = 0x9e3779b97f4a7c15ull;
uint64_t next()
{
    // splitmix64
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
double uniform() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }
double logUniform(double lo, double hi) { return std::exp(std::log(lo) + uniform() * (std::log(hi) - std::log(lo))); }

uint32_t ulps(float a, float b)
{
    const uint32_t x = nsdg_ff::bitsOf(a), y = nsdg_ff::bitsOf(b);
    return x > y ? x - y : y - x;
}

} // namespace

int main()
{
    const double dmins[] = { 2e-9, 1e-10, 5e-9, 3.3e-8 };
    const int perSet = 250000;
    uint64_t samples = 0, mismatchAB = 0, nonfinite = 0, seedsNormal = 0;
    uint64_t checkedWrong = 0, checkedFallback = 0;
    uint32_t maxAB = 0, maxARef = 0, maxBRef = 0;
    for (double dmin : dmins) {
        float d2h, d2l;
        nsdg_ff::splitSquare(dmin, d2h, d2l);
        const long double d2 = static_cast<long double>(dmin) * static_cast<long double>(dmin);
        for (int i = 0; i < perSet; ++i) {
            const double c = uniform();
            float inv;
            if (c < 0.1)
                inv = 0.f;
            else if (c < 0.2)
                inv = static_cast<float>(dmin * dmin * logUniform(0.25, 4.0));
            else if (c < 0.25)
                inv = static_cast<float>(uniform() * 1e-39);
            else
                inv = static_cast<float>(logUniform(1e-30, 1e-4));
            const double cp = uniform();
            double Pa;
            if (cp < 0.05)
                Pa = 0.0;
            else if (cp < 0.06)
                Pa = uniform() * 1e-310; // FP64 subnormal
            else if (cp < 0.1)
                Pa = logUniform(1e-300, 1e-28);
            else if (cp < 0.15)
                Pa = logUniform(1e-28, 1e-12);
            else
                Pa = logUniform(1e-6, 1e6);
            const float th = inv + d2h;
            const float yc = static_cast<float>(1.0 / std::sqrt(static_cast<double>(th)));
            const long double zl = static_cast<long double>(Pa)
                / std::sqrt(static_cast<long double>(inv) + d2);
            const float ref = static_cast<float>(zl);
            for (int k = -3; k <= 3; ++k) {
                const float y0 = nsdg_ff::floatOf(nsdg_ff::bitsOf(yc) + static_cast<uint32_t>(k));
                if (!(y0 > 0.f) || !std::isnormal(y0))
                    continue;
                ++seedsNormal;
                const float a = nsdg_ff::viscNewton64(inv, Pa, dmin, y0);
                const float b = nsdg_ff::viscFloatFloat(inv, Pa, d2h, d2l, y0);
                ++samples;
                // the checked form: where it says exact, bitwise the FP64 form
                bool exact = false;
                const float c = nsdg_ff::viscFloatFloatChecked(inv, Pa, d2h, d2l, y0, exact);
                if (!exact)
                    ++checkedFallback;
                else if (nsdg_ff::bitsOf(c) != nsdg_ff::bitsOf(a))
                    ++checkedWrong;
                if (!std::isfinite(a) || !std::isfinite(b)) {
                    ++nonfinite;
                    continue;
                }
                const uint32_t ab = ulps(a, b);
                if (ab)
                    ++mismatchAB;
                if (ab > maxAB)
                    maxAB = ab;
                // the FP64 form flushes results below the smallest normal
                // float to zero: compare with the reference only above it
                if (ref >= 0x1p-126f) {
                    const uint32_t ar = ulps(a, ref), br = ulps(b, ref);
                    if (ar > maxARef)
                        maxARef = ar;
                    if (br > maxBRef)
                        maxBRef = br;
                }
            }
        }
    }
    // Adversarial cases for the checked form: Pa chosen so that the exact
    // Newton value lies at a float rounding midpoint, or 2^-60 to 2^-36 of it
    // away on either side (the check's margin is 2^-39).
    uint64_t advSamples = 0, advWrong = 0, advFallback = 0, physSamples = 0, physFallback = 0;
    for (int i = 0; i < 200000; ++i) {
        const double dmin = dmins[i % 4];
        float d2h, d2l;
        nsdg_ff::splitSquare(dmin, d2h, d2l);
        const long double d2 = static_cast<long double>(dmin) * static_cast<long double>(dmin);
        const float inv = uniform() < 0.2 ? 0.f : static_cast<float>(logUniform(1e-22, 1e-4));
        const float th = inv + d2h;
        const float y0 = static_cast<float>(1.0 / std::sqrt(static_cast<double>(th)));
        const long double t = static_cast<long double>(inv) + d2;
        const long double y1 = static_cast<long double>(y0) * (1.5L - 0.5L * t * y0 * y0);
        // a float z0 in [1e-3, 1e3] and the midpoint above it
        const float z0 = static_cast<float>(logUniform(1e-3, 1e3));
        const long double mid = (static_cast<long double>(z0)
            + static_cast<long double>(std::nextafter(z0, 2.f * z0))) / 2.0L;
        for (int j = -7; j <= 7; ++j) {
            const long double off = j == 0 ? 0.0L : (j > 0 ? 1.0L : -1.0L) * std::ldexp(1.0L, -60 + 4 * (j < 0 ? -j : j));
            const double Pa = static_cast<double>(mid * (1.0L + off) / y1);
            bool exact = false;
            const float c = nsdg_ff::viscFloatFloatChecked(inv, Pa, d2h, d2l, y0, exact);
            const float a = nsdg_ff::viscNewton64(inv, Pa, dmin, y0);
            ++advSamples;
            if (!exact)
                ++advFallback;
            else if (nsdg_ff::bitsOf(c) != nsdg_ff::bitsOf(a))
                ++advWrong;
        }
        // the physical range: pressure terms 1e-3 to 1e4, random strain
        const double Pp = logUniform(1e-3, 1e4);
        bool ex2 = false;
        nsdg_ff::viscFloatFloatChecked(inv, Pp, d2h, d2l, y0, ex2);
        ++physSamples;
        if (!ex2)
            ++physFallback;
    }

    std::printf("samples %" PRIu64 "\n", samples);
    std::printf("seeds %" PRIu64 "\n", seedsNormal);
    std::printf("mismatch_ab %" PRIu64 "\n", mismatchAB);
    std::printf("max_ulp_ab %u\n", maxAB);
    std::printf("max_ulp_fp64_ref %u\n", maxARef);
    std::printf("max_ulp_ff_ref %u\n", maxBRef);
    std::printf("nonfinite %" PRIu64 "\n", nonfinite);
    std::printf("checked_wrong %" PRIu64 "\n", checkedWrong);
    std::printf("checked_fallback %" PRIu64 "\n", checkedFallback);
    std::printf("adv_samples %" PRIu64 "\n", advSamples);
    std::printf("adv_wrong %" PRIu64 "\n", advWrong);
    std::printf("adv_fallback %" PRIu64 "\n", advFallback);
    std::printf("phys_samples %" PRIu64 "\n", physSamples);
    std::printf("phys_fallback %" PRIu64 "\n", physFallback);
    return 0;
}
