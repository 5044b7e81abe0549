// Column thermodynamics on the GPU: IceGrowth::update (physics/src/IceGrowth.cpp:148-182)
// with ThermoIce0 (physics/src/modules/IceThermodynamicsModule/ThermoIce0.cpp:85-172) or
// ThermoWinton (.../ThermoWinton.cpp:102-342),
// HiblerSpread (physics/src/modules/LateralIceSpreadModule/HiblerSpread.cpp:53-66) and
// ConstantHealing (physics/src/modules/DamageHealingModule/ConstantHealing.cpp:53-73).
//
// One thread per element, all in FP64 in the reference's operation order.
// This file is compiled with --fmad=false: no multiply-add is fused, so every
// value is rounded exactly where the reference's (and the CPU oracle's)
// arithmetic rounds it, and the results are bit-identical to them.  The
// update is element-local and memory-bound (25 slots read and 21 written
// per ocean element).
#include "nsdg_ice_growth.hpp"

namespace nsdg {
namespace {

constexpr int kIgBlock = 256;

// core/src/include/constants.hpp:46-69 (Ice), 105-120 (Water)
constexpr double kIceKappa = 2.0334;
constexpr double kIceCp = 2100.;
constexpr double kLf = 333.55e3;
constexpr double kRhoIce = 917;
constexpr double kRhoSnow = 330.;
constexpr double kIceS = 5;
constexpr double kTm = 273.15;
constexpr double kMu = 0.055;
constexpr double kRhoOcean = 1025;

// std::min(a, b) / std::max(a, b) as the reference calls them (NaN-ordered)
__device__ __forceinline__ double refMin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double refMax(double a, double b) { return (a < b) ? b : a; }

struct IgParams {
    nsdg_ice_growth_params p;
    double dt;
};

// ThermoIce0::calculateElement on registers (f: the element's slots)
__device__ __forceinline__ void thermoIce0(double* f, const nsdg_ice_growth_params& p, double dt)
{
    if (f[NSDG_IG_HICE] == 0. || f[NSDG_IG_CICE] == 0.) {
        f[NSDG_IG_DELTA_HICE] = 0.;
        f[NSDG_IG_SNOW_TO_ICE] = 0.;
        return;
    }
    const double bulkLHFusionSnow = kLf * kRhoSnow;
    const double bulkLHFusionIce = kLf * kRhoIce;
    constexpr double beta = 0.4;  // Semtner's factors for the zero-layer model
    constexpr double gamma = 1.065;
    const double freezingPointIce = -kMu * kIceS;
    const double tice0 = f[NSDG_IG_TICE0];
    const double kSlab = p.ks * kIceKappa / (p.ks * f[NSDG_IG_HICE] + kIceKappa * f[NSDG_IG_HSNOW]) * gamma;
    const double qic = kSlab * (f[NSDG_IG_TF] - tice0);
    f[NSDG_IG_QIC] = qic;
    const double remaining = qic - (f[NSDG_IG_QIA] + (1. - beta) * f[NSDG_IG_PENSW]);
    double tice = tice0 + remaining / (kSlab + f[NSDG_IG_DQIA_DT]);
    tice = refMin((f[NSDG_IG_HSNOW] > 0) ? 0 : freezingPointIce, tice);
    // top melt (non-positive rates), sublimation, excess flux melting ice
    const double snowMeltRate = refMin(-remaining, 0.) / bulkLHFusionSnow;
    f[NSDG_IG_SNOW_MELT] = snowMeltRate * dt;
    const double nowSnow = f[NSDG_IG_HSNOW] + (snowMeltRate - f[NSDG_IG_SUBLIM] / kRhoSnow) * dt;
    const double excessIceMelt = refMin(nowSnow, 0.) * bulkLHFusionSnow / bulkLHFusionIce;
    double hsnow = refMax(nowSnow, 0.);
    // bottom growth or melt
    const double bottom = (qic - f[NSDG_IG_QIO]) * dt / bulkLHFusionIce;
    double deltaHi = excessIceMelt + bottom;
    double hice = f[NSDG_IG_HICE] + deltaHi;
    if (hice > 0.)
        hsnow += f[NSDG_IG_SNOWFALL] * dt / kRhoSnow;
    double topMelt = refMin(excessIceMelt, 0.);
    double botMelt = refMin(bottom, 0.);
    // flooding: snow below the waterline becomes ice
    const double draught = (hice * kRhoIce + hsnow * kRhoSnow) / kRhoOcean;
    double snowToIce = 0;
    if (p.flooding && draught > hice) {
        snowToIce = draught - hice;
        hsnow -= snowToIce * kRhoIce / kRhoSnow;
        hice = draught;
    }
    double cice = f[NSDG_IG_CICE];
    if (hice < p.h_min) { // all the ice melts
        const double oldHi = f[NSDG_IG_HICE0];
        if (deltaHi < 0) {
            const double scaling = oldHi / deltaHi;
            topMelt *= scaling;
            botMelt *= scaling;
        }
        snowToIce = 0.;
        deltaHi = -oldHi;
        f[NSDG_IG_QIO] += hice * bulkLHFusionIce / dt + hsnow * bulkLHFusionSnow / dt;
        cice = 0.;
        hice = 0.;
        hsnow = 0.;
        tice = kTm - kTm; // the melting point of ice in C
    }
    f[NSDG_IG_TICE] = tice;
    f[NSDG_IG_HSNOW] = hsnow;
    f[NSDG_IG_DELTA_HICE] = deltaHi;
    f[NSDG_IG_HICE] = hice;
    f[NSDG_IG_TOP_MELT] = topMelt;
    f[NSDG_IG_BOT_MELT] = botMelt;
    f[NSDG_IG_SNOW_TO_ICE] = snowToIce;
    f[NSDG_IG_CICE] = cice;
}

// ThermoWinton::calculateTemps (ThermoWinton.cpp:298-342): Winton (2000)
// eqs. (5)-(22), surface and layer temperatures
__device__ __forceinline__ void wintonTemps(const double* f, const nsdg_ice_growth_params& p, double& tSurf,
    double& tUppr, double& tLowr, double& mSurf, double dt)
{
    const double cVol = kIceCp * kRhoIce;
    const double seaIceTf = -kMu * kIceS;
    const double hi = f[NSDG_IG_HICE];
    const double hsnow = f[NSDG_IG_HSNOW];
    const double tBase = f[NSDG_IG_TF];
    const double tMelt = (hsnow > 0) ? 0 : seaIceTf;
    const double k12 = 4 * kIceKappa * p.ks / (p.ks * hi + 4 * kIceKappa * hsnow);
    const double a = f[NSDG_IG_QIA] - tSurf * f[NSDG_IG_DQIA_DT];
    const double b = f[NSDG_IG_DQIA_DT];
    const double k32 = 2 * kIceKappa / hi;
    double a1 = hi * cVol / (2 * dt) + k32 * (4 * dt * k32 + hi * cVol) / (6 * dt * k32 + hi * cVol)
        + b * k12 / (k12 + b);
    double b1 = -hi * (cVol * tUppr + kLf * kRhoIce * seaIceTf / tUppr) / (2 * dt) - f[NSDG_IG_PENSW]
        - k32 * (4 * dt * k32 * tBase + hi * cVol * tLowr) / (6 * dt * k32 + hi * cVol)
        + a * k12 / (k12 + b);
    const double c1 = hi * kLf * kRhoIce * seaIceTf / (2 * dt);
    tUppr = -(b1 + sqrt(b1 * b1 - 4 * a1 * c1)) / (2 * a1);
    tSurf = (k12 * tUppr - a) / (k12 + b);
    if (tSurf > tMelt) { // the surface melts: recompute with the surface at the melting point
        tSurf = tMelt;
        a1 += k12 - k12 * b / (k12 + b);
        b1 -= k12 * tSurf + a * k12 / (k12 + b);
        tUppr = -(b1 + sqrt(b1 * b1 - 4 * a1 * c1)) / (2 * a1);
        mSurf = k12 * (tUppr - tSurf) - (a + b * tSurf);
    }
    tLowr = (2 * dt * k32 * (tUppr + 2 * f[NSDG_IG_TF]) + hi * cVol * tLowr) / (6 * dt * k32 + hi * cVol);
}

// ThermoWinton::calculateElement (ThermoWinton.cpp:102-296); bottom_melt and
// snow_to_ice accumulate onto their previous values, as in the reference
__device__ __forceinline__ void thermoWinton(double* f, const nsdg_ice_growth_params& p, double dt)
{
    const double cVol = kIceCp * kRhoIce;
    const double seaIceTf = -kMu * kIceS;
    if (f[NSDG_IG_CICE] <= 0 || f[NSDG_IG_HICE] <= 0) {
        f[NSDG_IG_SNOW_TO_ICE] = 0;
        f[NSDG_IG_DELTA_HICE] = 0;
        f[NSDG_IG_HICE] = 0;
        f[NSDG_IG_HSNOW] = 0;
        f[NSDG_IG_TICE] = seaIceTf;
        f[NSDG_IG_TICE_1] = seaIceTf;
        f[NSDG_IG_TICE_2] = seaIceTf;
        return;
    }
    const double bulkLHFusionSnow = kLf * kRhoSnow;
    const double bulkLHFusionIce = kLf * kRhoIce;
    const double hice = f[NSDG_IG_HICE];
    double tSurf = f[NSDG_IG_TICE0], tUppr = f[NSDG_IG_TICE0_1], tLowr = f[NSDG_IG_TICE0_2];
    const double tBott = f[NSDG_IG_TF];
    double surfMelt = 0;
    wintonTemps(f, p, tSurf, tUppr, tLowr, surfMelt, dt);
    const double dHfTf_cp = kLf * seaIceTf / kIceCp;
    double h1 = hice / 2, h2 = hice / 2;
    const double e1 = cVol * (tUppr - seaIceTf) - bulkLHFusionIce * (1 - seaIceTf / tUppr);
    const double e2 = cVol * (tLowr - seaIceTf) - bulkLHFusionIce;
    double hs = f[NSDG_IG_HSNOW] + f[NSDG_IG_SNOWFALL] / kRhoSnow * dt;
    // sublimation: of snow, of the upper, of the lower half, of all
    const double deltaSnow = f[NSDG_IG_SUBLIM] * dt / kRhoSnow;
    double deltaIce1 = (deltaSnow - hs) * kRhoSnow / kRhoIce;
    double deltaIce2 = deltaIce1 - h1;
    if (deltaSnow <= hs) {
        hs -= deltaSnow;
    } else if (deltaIce1 <= h1) {
        h1 -= deltaIce1;
        hs = 0;
    } else if (deltaIce2 <= h2) {
        h2 -= deltaIce2;
        h1 = 0;
        hs = 0;
    } else {
        h2 = 0;
        h1 = 0;
        hs = 0;
    }
    double topMelt = refMax(0., h1 + h2 - hice);
    double botMelt = f[NSDG_IG_BOT_MELT];
    double qio = f[NSDG_IG_QIO];
    const double meltBottom = (qio - 4 * kIceKappa * (tBott - tLowr) / hice) * dt;
    double snowMelt = 0;
    if (meltBottom <= 0.) { // bottom freezing
        const double eBot = cVol * (tBott - seaIceTf) - bulkLHFusionIce;
        deltaIce2 = meltBottom / eBot;
        tLowr = (deltaIce2 * tBott + h2 * tLowr) / (deltaIce2 + h2);
        h2 += deltaIce2;
    } else { // bottom melting
        deltaIce2 = -refMin(-meltBottom / e2, h2);
        deltaIce1 = -refMin(refMax(-(meltBottom + e2 * h2) / e1, 0.), h1);
        snowMelt = -refMin(refMax((meltBottom + e2 * h2 + e1 * h1) / bulkLHFusionSnow, 0.), hs);
        if (h2 + h1 + hs - deltaIce2 - deltaIce1 - snowMelt <= 0.)
            qio -= refMax(meltBottom - bulkLHFusionSnow * hs + e1 * h1 + e2 * h2, 0.) / dt;
        hs += snowMelt;
        h1 += deltaIce1;
        h2 += deltaIce2;
        botMelt += deltaIce1 + deltaIce2;
    }
    // surface melt
    snowMelt -= refMin(surfMelt * dt / bulkLHFusionSnow, hs);
    deltaIce1 = -refMin(refMax(-(surfMelt * dt - bulkLHFusionSnow * hs) / e1, 0.), h1);
    deltaIce2 = -refMin(refMax(-(surfMelt * dt - bulkLHFusionSnow * hs + e1 * h1) / e2, 0.), h2);
    if (h2 + h1 + hs - deltaIce2 - deltaIce1 - snowMelt <= 0.)
        qio -= refMax(surfMelt * dt - bulkLHFusionSnow * hs + e1 * h1 + e2 * h2, 0.) / dt;
    hs += snowMelt;
    h1 += deltaIce1;
    h2 += deltaIce2;
    topMelt += deltaIce1 + deltaIce2;
    // snow to ice
    double snowToIce = f[NSDG_IG_SNOW_TO_ICE];
    const double freeboard = (hice * (kRhoOcean - kRhoIce) - hs * kRhoSnow) / kRhoOcean;
    if (p.flooding && freeboard < 0.) {
        hs += refMin(freeboard * kRhoIce / kRhoSnow, 0.);
        deltaIce1 = refMax(-freeboard, 0.);
        const double f1 = 1 - deltaIce1 / (deltaIce1 + h1);
        const double tBar = f1 * (tUppr + dHfTf_cp / tUppr) + (1 - f1) * seaIceTf;
        tUppr = (tBar - sqrt(tBar * tBar - 4 * dHfTf_cp)) / 2;
        h1 += deltaIce1;
        snowToIce += deltaIce1;
    }
    double hi = h1 + h2;
    // equal layers again
    if (h2 > h1) {
        const double f1 = h1 / hi * 2;
        const double tBar = f1 * (tUppr + dHfTf_cp / tUppr) + (1 - f1) * tLowr;
        tUppr = (tBar - sqrt(tBar * tBar - 4 * dHfTf_cp)) / 2;
    } else {
        const double f1 = (2 * h1 - hi) / hi;
        tLowr = f1 * (tUppr + dHfTf_cp / tUppr) + (1 - f1) * tLowr;
        if (tLowr > seaIceTf) {
            const double deltaMelt = hi / 4 * kIceCp * (tLowr - seaIceTf) * tUppr
                / (kLf * tUppr + (kIceCp * tUppr - kLf) * (seaIceTf - tUppr));
            topMelt -= deltaMelt;
            botMelt -= deltaMelt;
            hi -= 2 * deltaMelt;
            tLowr = seaIceTf;
        }
    }
    const double oldHi = f[NSDG_IG_HICE0];
    double deltaHi = hi - oldHi;
    if (hi < p.h_min) { // remove very thin ice
        qio -= (-bulkLHFusionSnow * hs + (e1 + e2) * hi / 2) / dt;
        if (deltaHi < 0) {
            topMelt *= oldHi / deltaHi;
            botMelt *= oldHi / deltaHi;
        }
        snowToIce = 0;
        deltaHi = -oldHi;
        hi = 0;
        hs = 0;
        tSurf = seaIceTf;
        tUppr = seaIceTf;
        tLowr = seaIceTf;
    }
    f[NSDG_IG_HICE] = hi;
    f[NSDG_IG_HSNOW] = hs;
    f[NSDG_IG_QIO] = qio;
    f[NSDG_IG_TOP_MELT] = topMelt;
    f[NSDG_IG_BOT_MELT] = botMelt;
    f[NSDG_IG_SNOW_MELT] = snowMelt;
    f[NSDG_IG_SNOW_TO_ICE] = snowToIce;
    f[NSDG_IG_DELTA_HICE] = deltaHi;
    f[NSDG_IG_TICE] = tSurf;
    f[NSDG_IG_TICE_1] = tUppr;
    f[NSDG_IG_TICE_2] = tLowr;
}

// IceGrowth::applyLimits (IceGrowth.cpp:260-268)
__device__ __forceinline__ void applyLimits(double* f, const nsdg_ice_growth_params& p, double dt)
{
    const double cice = f[NSDG_IG_CICE], hice = f[NSDG_IG_HICE];
    if ((0. < cice && cice < p.c_min) || (0. < hice && hice < p.h_min)) {
        f[NSDG_IG_QOW] += cice * kLf * (hice * kRhoIce + f[NSDG_IG_HSNOW] * kRhoSnow) / dt;
        f[NSDG_IG_HICE] = 0;
        f[NSDG_IG_CICE] = 0;
        f[NSDG_IG_HSNOW] = 0;
    }
}

// the slots an ocean element reads before writing them
__device__ __forceinline__ bool readSlot(int k)
{
    return !(k == NSDG_IG_HICE || k == NSDG_IG_CICE || k == NSDG_IG_HSNOW || k == NSDG_IG_HICE0
        || k == NSDG_IG_HSNOW0 || k == NSDG_IG_NEWICE || k == NSDG_IG_DELTA_CICE || k == NSDG_IG_TICE
        || k == NSDG_IG_TICE_1 || k == NSDG_IG_TICE_2);
}
// the slots an update may change
__device__ __forceinline__ bool writeSlot(int k)
{
    return (k >= NSDG_IG_HICE && k != NSDG_IG_TICE0_1 && k != NSDG_IG_TICE0_2) || k == NSDG_IG_QOW
        || k == NSDG_IG_QIO || k == NSDG_IG_DAMAGE;
}

__global__ void __launch_bounds__(kIgBlock) kIceGrowth(size_t n, const uint8_t* __restrict__ ocean, IgParams a,
    double* __restrict__ F)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const nsdg_ice_growth_params& p = a.p;
    const double dt = a.dt;
    // initializeThicknesses: cice = cice0 and tice = tice0 on every element
    if (!ocean[i]) {
        F[size_t(NSDG_IG_CICE) * n + i] = F[size_t(NSDG_IG_CICE0) * n + i];
        F[size_t(NSDG_IG_TICE) * n + i] = F[size_t(NSDG_IG_TICE0) * n + i];
        F[size_t(NSDG_IG_TICE_1) * n + i] = F[size_t(NSDG_IG_TICE0_1) * n + i];
        F[size_t(NSDG_IG_TICE_2) * n + i] = F[size_t(NSDG_IG_TICE0_2) * n + i];
        return;
    }
    double f[NSDG_IG_NFIELDS];
#pragma unroll
    for (int k = 0; k < NSDG_IG_NFIELDS; ++k)
        f[k] = readSlot(k) ? F[size_t(k) * n + i] : 0.0;
    // IceGrowth::initializeThicknessesElement (IceGrowth.cpp:184-199)
    f[NSDG_IG_CICE] = f[NSDG_IG_CICE0];
    f[NSDG_IG_DELTA_CICE] = 0;
    if (f[NSDG_IG_CICE0] > 0 && f[NSDG_IG_HICE_CELL] > 0) {
        f[NSDG_IG_HICE] = f[NSDG_IG_HICE0] = f[NSDG_IG_HICE_CELL] / f[NSDG_IG_CICE0];
        f[NSDG_IG_HSNOW] = f[NSDG_IG_HSNOW0] = f[NSDG_IG_HSNOW_CELL] / f[NSDG_IG_CICE0];
    } else {
        f[NSDG_IG_HICE] = f[NSDG_IG_HICE0] = 0.;
        f[NSDG_IG_HSNOW] = f[NSDG_IG_HSNOW0] = 0.;
        f[NSDG_IG_CICE] = 0.;
    }
    f[NSDG_IG_NEWICE] = 0;
    f[NSDG_IG_TICE] = f[NSDG_IG_TICE0]; // IIceThermodynamics::initialiseTice, every level
    f[NSDG_IG_TICE_1] = f[NSDG_IG_TICE0_1];
    f[NSDG_IG_TICE_2] = f[NSDG_IG_TICE0_2];
    applyLimits(f, p, dt);
    if (p.use_thermo) {
        if (p.thermo_model == 0)
            thermoIce0(f, p, dt);
        else if (p.thermo_model == 2)
            thermoWinton(f, p, dt);
        // IceGrowth::newIceFormation (IceGrowth.cpp:201-227)
        {
            const double cooling = f[NSDG_IG_QOW];
            const double deltaTml = -cooling / f[NSDG_IG_MLBHC] * dt;
            const double t0 = f[NSDG_IG_SST], tf0 = f[NSDG_IG_TF];
            if (t0 + deltaTml < tf0) {
                const double sensible = (tf0 - t0) / deltaTml * cooling;
                const double latent = cooling - sensible;
                f[NSDG_IG_QOW] = sensible;
                f[NSDG_IG_NEWICE] = latent * dt * (1 - f[NSDG_IG_CICE]) / (kLf * kRhoIce);
            } else {
                f[NSDG_IG_NEWICE] = 0;
            }
        }
        // IceGrowth::lateralIceSpread (IceGrowth.cpp:235-258), HiblerSpread or DummyIceSpread
        {
            double dcMelt = 0, dcFreeze = 0;
            if (p.lateral_model == 0)
                dcFreeze = f[NSDG_IG_NEWICE] * (1. / p.h0);
            if (f[NSDG_IG_DELTA_HICE] < 0 && p.lateral_model == 0 && f[NSDG_IG_CICE] < 1)
                dcMelt = f[NSDG_IG_DELTA_HICE] * f[NSDG_IG_CICE] * p.phi_m / f[NSDG_IG_HICE0];
            const double dc = dcFreeze + dcMelt;
            f[NSDG_IG_DELTA_CFREEZE] = dcFreeze;
            f[NSDG_IG_DELTA_CMELT] = dcMelt;
            f[NSDG_IG_DELTA_CICE] = dc;
            const double cice = (f[NSDG_IG_HICE] > 0 || f[NSDG_IG_NEWICE] > 0) ? f[NSDG_IG_CICE] + dc : 0;
            f[NSDG_IG_CICE] = cice;
            if (cice >= p.c_min) {
                f[NSDG_IG_HICE] += (f[NSDG_IG_NEWICE] - f[NSDG_IG_HICE] * dc) / cice;
                if (dc < 0)
                    f[NSDG_IG_QOW] -= dc * f[NSDG_IG_HSNOW] * kLf * kRhoSnow / dt;
                else
                    f[NSDG_IG_HSNOW] += (0 - f[NSDG_IG_HSNOW] * dc) / cice;
            }
        }
        applyLimits(f, p, dt);
    }
    // ConstantHealing::updateElement (ConstantHealing.cpp:53-73)
    if (p.healing_model == 0) {
        const double growth = refMax(0., f[NSDG_IG_DELTA_CICE]);
        double d = (f[NSDG_IG_DAMAGE] * (f[NSDG_IG_CICE] - growth) + growth) / f[NSDG_IG_CICE];
        d += dt / p.healing_time;
        f[NSDG_IG_DAMAGE] = refMin(1., d);
    }
#pragma unroll
    for (int k = 0; k < NSDG_IG_NFIELDS; ++k)
        if (writeSlot(k))
            F[size_t(k) * n + i] = f[k];
}

__global__ void __launch_bounds__(kIgBlock) kIceGrowthFromDynamics(size_t n, const double* __restrict__ h,
    const double* __restrict__ c, const double* __restrict__ d, double* __restrict__ F)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    F[size_t(NSDG_IG_HICE_CELL) * n + i] = h[i];
    F[size_t(NSDG_IG_CICE0) * n + i] = c[i];
    if (d)
        F[size_t(NSDG_IG_DAMAGE) * n + i] = d[i];
}

__global__ void __launch_bounds__(kIgBlock) kIceGrowthToDynamics(size_t n, int dg, const double* __restrict__ F,
    double* __restrict__ h, double* __restrict__ c, double* __restrict__ d)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    // PrognosticData::updatePrognosticFields: the cell average hice_true x cice
    const double cice = F[size_t(NSDG_IG_CICE) * n + i];
    h[i] = F[size_t(NSDG_IG_HICE) * n + i] * cice;
    c[i] = cice;
    if (d)
        d[i] = F[size_t(NSDG_IG_DAMAGE) * n + i];
    for (int k = 1; k < dg; ++k) {
        h[size_t(k) * n + i] = 0.0;
        c[size_t(k) * n + i] = 0.0;
        if (d)
            d[size_t(k) * n + i] = 0.0;
    }
}

unsigned gridFor(size_t n) { return static_cast<unsigned>((n + kIgBlock - 1) / kIgBlock); }

} // namespace

cudaError_t launchIceGrowth(cudaStream_t s, size_t n, const uint8_t* ocean, const nsdg_ice_growth_params& p,
    double dt, double* fields)
{
    if (n == 0)
        return cudaSuccess;
    kIceGrowth<<<gridFor(n), kIgBlock, 0, s>>>(n, ocean, IgParams { p, dt }, fields);
    return cudaGetLastError();
}

cudaError_t launchIceGrowthFromDynamics(cudaStream_t s, size_t n, const double* hiceDG, const double* ciceDG,
    const double* damageDG, double* fields)
{
    if (n == 0)
        return cudaSuccess;
    kIceGrowthFromDynamics<<<gridFor(n), kIgBlock, 0, s>>>(n, hiceDG, ciceDG, damageDG, fields);
    return cudaGetLastError();
}

cudaError_t launchIceGrowthToDynamics(cudaStream_t s, size_t n, int dg, const double* fields, double* hiceDG,
    double* ciceDG, double* damageDG)
{
    if (n == 0)
        return cudaSuccess;
    kIceGrowthToDynamics<<<gridFor(n), kIgBlock, 0, s>>>(n, dg, fields, hiceDG, ciceDG, damageDG);
    return cudaGetLastError();
}

} // namespace nsdg
