// Column thermodynamics on the GPU: IceGrowth::update (physics/src/IceGrowth.cpp:148-182)
// with ThermoIce0 (physics/src/modules/IceThermodynamicsModule/ThermoIce0.cpp:85-172),
// HiblerSpread (physics/src/modules/LateralIceSpreadModule/HiblerSpread.cpp:53-66) and
// ConstantHealing (physics/src/modules/DamageHealingModule/ConstantHealing.cpp:53-73).
//
// One thread per element, all in FP64 in the reference's operation order.
// This file is compiled with --fmad=false: no multiply-add is fused, so every
// value is rounded exactly where the reference's (and the CPU oracle's)
// arithmetic rounds it, and the results are bit-identical to them.  The
// update is element-local and memory-bound (about 23 slots read and 19
// written per ocean element).
#include "nsdg_ice_growth.hpp"

namespace nsdg {
namespace {

constexpr int kIgBlock = 256;

// core/src/include/constants.hpp:46-69 (Ice), 105-120 (Water)
constexpr double kIceKappa = 2.0334;
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
        || k == NSDG_IG_HSNOW0 || k == NSDG_IG_NEWICE || k == NSDG_IG_DELTA_CICE || k == NSDG_IG_TICE);
}
// the slots an update may change
__device__ __forceinline__ bool writeSlot(int k) { return k >= NSDG_IG_HICE || k == NSDG_IG_QOW
        || k == NSDG_IG_QIO || k == NSDG_IG_DAMAGE; }

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
    f[NSDG_IG_TICE] = f[NSDG_IG_TICE0];
    applyLimits(f, p, dt);
    if (p.use_thermo) {
        if (p.thermo_model == 0)
            thermoIce0(f, p, dt);
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
