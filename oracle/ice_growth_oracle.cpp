// CPU oracle of the column thermodynamics step (IceGrowth with ThermoIce0 or
// ThermoWinton, HiblerSpread, ConstantHealing, IceMinima, and the Dummy / NoHealing
// alternatives).  TEST INFRASTRUCTURE ONLY: the checker of the GPU ice-growth
// path, never linked into the product.  A plain C++17 restatement of the
// reference's per-element arithmetic in its operation order, each function
// citing the reference lines it follows; built with -ffp-contract=off.
//
// Pinned against the reference's own known-answer tests that its build runs
// (physics/test/IceGrowth_test.cpp, ThermoIce0_test.cpp, ThermoWintonTemperature_test.cpp,
// DamageHealing_test.cpp; physics/test/CMakeLists.txt:51-117) in tests/test_oracle_ice_growth.py.
// physics/test/ThermoIce0Temperature_test.cpp is not built there (it uses a
// retired array-store API) and its expected conductive flux predates the
// Semtner factor gamma = 1.065 (its 44.4839 W m^-2 is 47.375 / 1.065).
#include "nsdg.h"

#include <cmath>
#include <cstddef>
#include <vector>

namespace {

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
constexpr double kWaterTf = kTm;

// std::min / std::max as the reference calls them: min(a, b) = (b < a) ? b : a
inline double stdMin(double a, double b) { return (b < a) ? b : a; }
inline double stdMax(double a, double b) { return (a < b) ? b : a; }

struct Elem {
    double* f;   // fields base
    size_t n, i; // count, element
    double& operator[](int slot) const { return f[size_t(slot) * n + i]; }
};

// IceGrowth::initializeThicknessesElement (physics/src/IceGrowth.cpp:184-199)
void initializeThicknessesElement(const Elem& x)
{
    x[NSDG_IG_DELTA_CICE] = 0;
    if (x[NSDG_IG_CICE0] > 0 && x[NSDG_IG_HICE_CELL] > 0) {
        x[NSDG_IG_HICE] = x[NSDG_IG_HICE0] = x[NSDG_IG_HICE_CELL] / x[NSDG_IG_CICE0];
        x[NSDG_IG_HSNOW] = x[NSDG_IG_HSNOW0] = x[NSDG_IG_HSNOW_CELL] / x[NSDG_IG_CICE0];
    } else {
        x[NSDG_IG_HICE] = x[NSDG_IG_HICE0] = 0.;
        x[NSDG_IG_HSNOW] = x[NSDG_IG_HSNOW0] = 0.;
        x[NSDG_IG_CICE] = 0.;
    }
    x[NSDG_IG_NEWICE] = 0;
}

// IceGrowth::applyLimits (physics/src/IceGrowth.cpp:260-268)
void applyLimits(const Elem& x, const nsdg_ice_growth_params& p, double dt)
{
    double& cice = x[NSDG_IG_CICE];
    double& hice = x[NSDG_IG_HICE];
    if ((0. < cice && cice < p.c_min) || (0. < hice && hice < p.h_min)) {
        x[NSDG_IG_QOW] += cice * kLf * (hice * kRhoIce + x[NSDG_IG_HSNOW] * kRhoSnow) / dt;
        hice = 0;
        cice = 0;
        x[NSDG_IG_HSNOW] = 0;
    }
}

// ThermoIce0::calculateElement (physics/src/modules/IceThermodynamicsModule/ThermoIce0.cpp:85-172)
void thermoIce0(const Elem& x, const nsdg_ice_growth_params& p, double dt)
{
    double& hice = x[NSDG_IG_HICE];
    double& cice = x[NSDG_IG_CICE];
    double& hsnow = x[NSDG_IG_HSNOW];
    if (hice == 0. || cice == 0.) {
        x[NSDG_IG_DELTA_HICE] = 0.;
        x[NSDG_IG_SNOW_TO_ICE] = 0.;
        return;
    }
    const double bulkLHFusionSnow = kLf * kRhoSnow;
    const double bulkLHFusionIce = kLf * kRhoIce;
    constexpr double beta = 0.4;
    constexpr double gamma = 1.065;
    const double freezingPointIce = -kMu * kIceS; // ThermoIce0.cpp:23
    double& tice = x[NSDG_IG_TICE];
    const double tice0 = x[NSDG_IG_TICE0];
    const double kLSlab = p.ks * kIceKappa / (p.ks * hice + kIceKappa * hsnow) * gamma;
    double& qic = x[NSDG_IG_QIC];
    qic = kLSlab * (x[NSDG_IG_TF] - tice0);
    const double remainingFlux = qic - (x[NSDG_IG_QIA] + (1. - beta) * x[NSDG_IG_PENSW]);
    tice = tice0 + remainingFlux / (kLSlab + x[NSDG_IG_DQIA_DT]);
    const double meltingLimit = (hsnow > 0) ? 0 : freezingPointIce;
    tice = stdMin(meltingLimit, tice);
    const double snowMeltRate = stdMin(-remainingFlux, 0.) / bulkLHFusionSnow;
    x[NSDG_IG_SNOW_MELT] = snowMeltRate * dt;
    const double snowSublRate = x[NSDG_IG_SUBLIM] / kRhoSnow;
    const double nowSnow = hsnow + (snowMeltRate - snowSublRate) * dt;
    const double excessIceMelt = stdMin(nowSnow, 0.) * bulkLHFusionSnow / bulkLHFusionIce;
    hsnow = stdMax(nowSnow, 0.);
    const double iceBottomChange = (qic - x[NSDG_IG_QIO]) * dt / bulkLHFusionIce;
    double& deltaHi = x[NSDG_IG_DELTA_HICE];
    deltaHi = excessIceMelt + iceBottomChange;
    hice += deltaHi;
    if (hice > 0.)
        hsnow += x[NSDG_IG_SNOWFALL] * dt / kRhoSnow;
    double& topMelt = x[NSDG_IG_TOP_MELT];
    double& botMelt = x[NSDG_IG_BOT_MELT];
    topMelt = stdMin(excessIceMelt, 0.);
    botMelt = stdMin(iceBottomChange, 0.);
    const double iceDraught = (hice * kRhoIce + hsnow * kRhoSnow) / kRhoOcean;
    if (p.flooding && iceDraught > hice) {
        const double snowDraught = iceDraught - hice;
        x[NSDG_IG_SNOW_TO_ICE] = snowDraught;
        hsnow -= snowDraught * kRhoIce / kRhoSnow;
        hice = iceDraught;
    } else {
        x[NSDG_IG_SNOW_TO_ICE] = 0;
    }
    if (hice < p.h_min) {
        const double oldHi = x[NSDG_IG_HICE0];
        if (deltaHi < 0) {
            const double scaling = oldHi / deltaHi;
            topMelt *= scaling;
            botMelt *= scaling;
        }
        x[NSDG_IG_SNOW_TO_ICE] = 0.;
        deltaHi = -oldHi;
        x[NSDG_IG_QIO] += hice * bulkLHFusionIce / dt + hsnow * bulkLHFusionSnow / dt;
        cice = 0.;
        hice = 0.;
        hsnow = 0.;
        tice = kTm - kWaterTf; // celsius(Ice::Tm), constants.hpp:131
    }
}

// ThermoWinton::calculateTemps (physics/src/modules/IceThermodynamicsModule/ThermoWinton.cpp:298-342):
// Winton (2000) eqs. (5)-(22) for the surface and the two layer temperatures
void wintonTemps(const Elem& x, const nsdg_ice_growth_params& p, double& tSurf, double& tUppr, double& tLowr,
    double& mSurf, double dt)
{
    const double cVol = kIceCp * kRhoIce;
    const double seaIceTf = -kMu * kIceS;
    const double hi = x[NSDG_IG_HICE];
    const double hsnow = x[NSDG_IG_HSNOW];
    const double tBase = x[NSDG_IG_TF];
    const double tMelt = (hsnow > 0) ? 0 : seaIceTf;
    const double k12 = 4 * kIceKappa * p.ks / (p.ks * hi + 4 * kIceKappa * hsnow); // (5)
    const double a = x[NSDG_IG_QIA] - tSurf * x[NSDG_IG_DQIA_DT];                    // (7)
    const double b = x[NSDG_IG_DQIA_DT];                                             // (8)
    const double k32 = 2 * kIceKappa / hi;                                           // (10)
    double a1 = hi * cVol / (2 * dt) + k32 * (4 * dt * k32 + hi * cVol) / (6 * dt * k32 + hi * cVol)
        + b * k12 / (k12 + b); // (16)
    double b1 = -hi * (cVol * tUppr + kLf * kRhoIce * seaIceTf / tUppr) / (2 * dt) - x[NSDG_IG_PENSW]
        - k32 * (4 * dt * k32 * tBase + hi * cVol * tLowr) / (6 * dt * k32 + hi * cVol)
        + a * k12 / (k12 + b); // (17)
    const double c1 = hi * kLf * kRhoIce * seaIceTf / (2 * dt); // (18)
    tUppr = -(b1 + std::sqrt(b1 * b1 - 4 * a1 * c1)) / (2 * a1); // (21)
    tSurf = (k12 * tUppr - a) / (k12 + b);                         // (6)
    if (tSurf > tMelt) {
        tSurf = tMelt;
        a1 += k12 - k12 * b / (k12 + b);                           // (19)
        b1 -= k12 * tSurf + a * k12 / (k12 + b);                   // (20)
        tUppr = -(b1 + std::sqrt(b1 * b1 - 4 * a1 * c1)) / (2 * a1); // (21)
        mSurf = k12 * (tUppr - tSurf) - (a + b * tSurf);           // (22)
    }
    tLowr = (2 * dt * k32 * (tUppr + 2 * x[NSDG_IG_TF]) + hi * cVol * tLowr) / (6 * dt * k32 + hi * cVol); // (15)
}

// ThermoWinton::calculateElement (ThermoWinton.cpp:102-296).  As in the
// reference, bottom_melt and snow_to_ice accumulate onto their previous values.
void thermoWinton(const Elem& x, const nsdg_ice_growth_params& p, double dt)
{
    const double cVol = kIceCp * kRhoIce;
    const double seaIceTf = -kMu * kIceS;
    double& hice = x[NSDG_IG_HICE];
    if (x[NSDG_IG_CICE] <= 0 || hice <= 0) {
        x[NSDG_IG_SNOW_TO_ICE] = 0;
        x[NSDG_IG_DELTA_HICE] = 0;
        hice = 0;
        x[NSDG_IG_HSNOW] = 0;
        x[NSDG_IG_TICE] = seaIceTf;
        x[NSDG_IG_TICE_1] = seaIceTf;
        x[NSDG_IG_TICE_2] = seaIceTf;
        return;
    }
    const double bulkLHFusionSnow = kLf * kRhoSnow;
    const double bulkLHFusionIce = kLf * kRhoIce;
    double tSurf = x[NSDG_IG_TICE0];
    double tUppr = x[NSDG_IG_TICE0_1];
    double tLowr = x[NSDG_IG_TICE0_2];
    const double tBott = x[NSDG_IG_TF];
    double surfMelt = 0;
    wintonTemps(x, p, tSurf, tUppr, tLowr, surfMelt, dt);
    const double dHfTf_cp = kLf * seaIceTf / kIceCp;
    double h1 = hice / 2;
    double h2 = hice / 2;
    const double e1 = cVol * (tUppr - seaIceTf) - bulkLHFusionIce * (1 - seaIceTf / tUppr);
    const double e2 = cVol * (tLowr - seaIceTf) - bulkLHFusionIce;
    double& hs = x[NSDG_IG_HSNOW];
    hs += x[NSDG_IG_SNOWFALL] / kRhoSnow * dt;
    // sublimation, four cases
    const double deltaSnow = x[NSDG_IG_SUBLIM] * dt / kRhoSnow;
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
    double& topMelt = x[NSDG_IG_TOP_MELT];
    double& botMelt = x[NSDG_IG_BOT_MELT];
    double& snowMelt = x[NSDG_IG_SNOW_MELT];
    double& qio = x[NSDG_IG_QIO];
    topMelt = stdMax(0., h1 + h2 - hice); // (23)
    // bottom melt / freezing
    const double meltBottom = (qio - 4 * kIceKappa * (tBott - tLowr) / hice) * dt;
    snowMelt = 0;
    if (meltBottom <= 0.) {
        const double eBot = cVol * (tBott - seaIceTf) - bulkLHFusionIce;
        deltaIce2 = meltBottom / eBot;                                 // (24)
        tLowr = (deltaIce2 * tBott + h2 * tLowr) / (deltaIce2 + h2);   // (26)
        h2 += deltaIce2;
    } else {
        deltaIce2 = -stdMin(-meltBottom / e2, h2);
        deltaIce1 = -stdMin(stdMax(-(meltBottom + e2 * h2) / e1, 0.), h1);
        snowMelt = -stdMin(stdMax((meltBottom + e2 * h2 + e1 * h1) / bulkLHFusionSnow, 0.), hs);
        if (h2 + h1 + hs - deltaIce2 - deltaIce1 - snowMelt <= 0.)
            qio -= stdMax(meltBottom - bulkLHFusionSnow * hs + e1 * h1 + e2 * h2, 0.) / dt; // (34)
        hs += snowMelt;
        h1 += deltaIce1;
        h2 += deltaIce2;
        botMelt += deltaIce1 + deltaIce2;
    }
    // surface melt (27)-(29)
    snowMelt -= stdMin(surfMelt * dt / bulkLHFusionSnow, hs);
    deltaIce1 = -stdMin(stdMax(-(surfMelt * dt - bulkLHFusionSnow * hs) / e1, 0.), h1);
    deltaIce2 = -stdMin(stdMax(-(surfMelt * dt - bulkLHFusionSnow * hs + e1 * h1) / e2, 0.), h2);
    if (h2 + h1 + hs - deltaIce2 - deltaIce1 - snowMelt <= 0.)
        qio -= stdMax(surfMelt * dt - bulkLHFusionSnow * hs + e1 * h1 + e2 * h2, 0.) / dt; // (30)
    hs += snowMelt;
    h1 += deltaIce1;
    h2 += deltaIce2;
    topMelt += deltaIce1 + deltaIce2;
    // snow to ice (35)-(39)
    const double freeboard = (hice * (kRhoOcean - kRhoIce) - hs * kRhoSnow) / kRhoOcean;
    if (p.flooding && freeboard < 0.) {
        hs += stdMin(freeboard * kRhoIce / kRhoSnow, 0.);
        deltaIce1 = stdMax(-freeboard, 0.);
        const double f1 = 1 - deltaIce1 / (deltaIce1 + h1);
        const double tBar = f1 * (tUppr + dHfTf_cp / tUppr) + (1 - f1) * seaIceTf;
        tUppr = (tBar - std::sqrt(tBar * tBar - 4 * dHfTf_cp)) / 2;
        h1 += deltaIce1;
        x[NSDG_IG_SNOW_TO_ICE] += deltaIce1;
    }
    double& hi = hice;
    hi = h1 + h2;
    // even layers (38)-(40)
    if (h2 > h1) {
        const double f1 = h1 / hi * 2;
        const double tBar = f1 * (tUppr + dHfTf_cp / tUppr) + (1 - f1) * tLowr;
        tUppr = (tBar - std::sqrt(tBar * tBar - 4 * dHfTf_cp)) / 2;
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
    double& deltaHi = x[NSDG_IG_DELTA_HICE];
    const double oldHi = x[NSDG_IG_HICE0];
    deltaHi = hi - oldHi;
    if (hi < p.h_min) {
        qio -= (-bulkLHFusionSnow * hs + (e1 + e2) * hi / 2) / dt;
        if (deltaHi < 0) {
            topMelt *= oldHi / deltaHi;
            botMelt *= oldHi / deltaHi;
        }
        x[NSDG_IG_SNOW_TO_ICE] = 0;
        deltaHi = -oldHi;
        hi = 0;
        hs = 0;
        tSurf = seaIceTf;
        tUppr = seaIceTf;
        tLowr = seaIceTf;
    }
    x[NSDG_IG_TICE] = tSurf;
    x[NSDG_IG_TICE_1] = tUppr;
    x[NSDG_IG_TICE_2] = tLowr;
}

// IceGrowth::newIceFormation (physics/src/IceGrowth.cpp:201-227)
void newIceFormation(const Elem& x, double dt)
{
    const double coolingFlux = x[NSDG_IG_QOW];
    const double deltaTml = -coolingFlux / x[NSDG_IG_MLBHC] * dt;
    const double t0 = x[NSDG_IG_SST];
    const double tf0 = x[NSDG_IG_TF];
    const double t1 = t0 + deltaTml;
    if (t1 < tf0) {
        const double sensibleFlux = (tf0 - t0) / deltaTml * coolingFlux;
        const double latentFlux = coolingFlux - sensibleFlux;
        x[NSDG_IG_QOW] = sensibleFlux;
        x[NSDG_IG_NEWICE] = latentFlux * dt * (1 - x[NSDG_IG_CICE]) / (kLf * kRhoIce);
    } else {
        x[NSDG_IG_NEWICE] = 0;
    }
}

// updateThickness (physics/src/IceGrowth.cpp:230-233)
void updateThickness(double& thick, double newConc, double deltaC, double deltaV)
{
    thick += (deltaV - thick * deltaC) / newConc;
}

// IceGrowth::lateralIceSpread (physics/src/IceGrowth.cpp:235-258) with
// HiblerSpread::freeze / melt (HiblerSpread.cpp:53-66) or DummyIceSpread
void lateralIceSpread(const Elem& x, const nsdg_ice_growth_params& p, double dt)
{
    double& dcMelt = x[NSDG_IG_DELTA_CMELT];
    double& dcFreeze = x[NSDG_IG_DELTA_CFREEZE];
    double& cice = x[NSDG_IG_CICE];
    dcMelt = 0;
    dcFreeze = 0;
    if (p.lateral_model == 0) {
        const double ooh0 = 1. / p.h0;
        dcFreeze = x[NSDG_IG_NEWICE] * ooh0;
    } else {
        dcFreeze = 0.;
    }
    if (x[NSDG_IG_DELTA_HICE] < 0) {
        if (p.lateral_model == 0) {
            if (cice < 1)
                dcMelt = x[NSDG_IG_DELTA_HICE] * cice * p.phi_m / x[NSDG_IG_HICE0];
        } else {
            dcMelt = 0.;
        }
    }
    double& dc = x[NSDG_IG_DELTA_CICE];
    dc = dcFreeze + dcMelt;
    cice = (x[NSDG_IG_HICE] > 0 || x[NSDG_IG_NEWICE] > 0) ? cice + dc : 0;
    if (cice >= p.c_min) {
        updateThickness(x[NSDG_IG_HICE], cice, dc, x[NSDG_IG_NEWICE]);
        if (dc < 0) {
            x[NSDG_IG_QOW] -= dc * x[NSDG_IG_HSNOW] * kLf * kRhoSnow / dt;
        } else {
            updateThickness(x[NSDG_IG_HSNOW], cice, dc, 0);
        }
    }
}

// ConstantHealing::updateElement (physics/src/modules/DamageHealingModule/ConstantHealing.cpp:53-73)
void constantHealing(const Elem& x, const nsdg_ice_growth_params& p, double dt)
{
    const double lateralGrowth = stdMax(0., x[NSDG_IG_DELTA_CICE]);
    double& damage = x[NSDG_IG_DAMAGE];
    const double cice = x[NSDG_IG_CICE];
    damage = (damage * (cice - lateralGrowth) + lateralGrowth) / cice;
    damage += dt / p.healing_time;
    damage = stdMin(1., damage);
}

} // namespace

extern "C" {

// Defaults of IceGrowth::configure, ThermoIce0::configure, HiblerSpread::configure,
// ConstantHealing::configure (IceGrowth.cpp:119-136, ThermoIce0.cpp:22,47-51,
// HiblerSpread.cpp:15-27, ConstantHealing.cpp:13-23, IceMinima.cpp:12-13)
void oracle_ice_growth_default_params(nsdg_ice_growth_params* p)
{
    p->ks = 0.3096;
    p->h_min = 0.01;
    p->c_min = 1e-12;
    p->h0 = 0.25;
    p->phi_m = 0.5;
    p->healing_time = 15. * 86400.;
    p->use_thermo = 1;
    p->thermo_model = 0;
    p->lateral_model = 0;
    p->healing_model = 0;
    p->flooding = 1;
}

// IceGrowth::update (physics/src/IceGrowth.cpp:148-182): fields is
// double[NSDG_IG_NFIELDS][n] in the slot order of include/nsdg.h.
void oracle_ice_growth_update(size_t n, const double* mask, const nsdg_ice_growth_params* p, double dt,
    double* fields)
{
    std::vector<size_t> ocean; // ModelComponent::overElements runs over the ocean points
    for (size_t i = 0; i < n; ++i)
        if (!mask || mask[i] > 0)
            ocean.push_back(i);
    // initializeThicknesses (IceGrowth.cpp:173-182): cice = cice0 everywhere,
    // the per-element part over the ocean, then tice = tice0 everywhere
    for (size_t i = 0; i < n; ++i)
        fields[size_t(NSDG_IG_CICE) * n + i] = fields[size_t(NSDG_IG_CICE0) * n + i];
    for (size_t i : ocean)
        initializeThicknessesElement(Elem { fields, n, i });
    for (size_t i = 0; i < n; ++i) { // IIceThermodynamics::initialiseTice: all levels
        fields[size_t(NSDG_IG_TICE) * n + i] = fields[size_t(NSDG_IG_TICE0) * n + i];
        fields[size_t(NSDG_IG_TICE_1) * n + i] = fields[size_t(NSDG_IG_TICE0_1) * n + i];
        fields[size_t(NSDG_IG_TICE_2) * n + i] = fields[size_t(NSDG_IG_TICE0_2) * n + i];
    }
    for (size_t i : ocean)
        applyLimits(Elem { fields, n, i }, *p, dt);
    if (p->use_thermo) {
        if (p->thermo_model == 0)
            for (size_t i : ocean)
                thermoIce0(Elem { fields, n, i }, *p, dt);
        else if (p->thermo_model == 2)
            for (size_t i : ocean)
                thermoWinton(Elem { fields, n, i }, *p, dt);
        for (size_t i : ocean) { // updateWrapper (IceGrowth.hpp)
            const Elem x { fields, n, i };
            newIceFormation(x, dt);
            lateralIceSpread(x, *p, dt);
            applyLimits(x, *p, dt);
        }
    }
    if (p->healing_model == 0)
        for (size_t i : ocean)
            constantHealing(Elem { fields, n, i }, *p, dt);
}

// The vertical thermodynamics alone (ThermoIce0, or ThermoWinton when
// thermo_model is 2) on the true thickness slots (hice_updated,
// cice_updated, hsnow_updated, hice_initial) with tice = tice0 first, as the
// known-answer test physics/test/ThermoIce0_test.cpp:30-160 drives it.
void oracle_thermo_ice0(size_t n, const nsdg_ice_growth_params* p, double dt, double* fields)
{
    for (size_t i = 0; i < n; ++i) {
        fields[size_t(NSDG_IG_TICE) * n + i] = fields[size_t(NSDG_IG_TICE0) * n + i];
        fields[size_t(NSDG_IG_TICE_1) * n + i] = fields[size_t(NSDG_IG_TICE0_1) * n + i];
        fields[size_t(NSDG_IG_TICE_2) * n + i] = fields[size_t(NSDG_IG_TICE0_2) * n + i];
        if (p->thermo_model == 2)
            thermoWinton(Elem { fields, n, i }, *p, dt);
        else
            thermoIce0(Elem { fields, n, i }, *p, dt);
    }
}

// ConstantHealing::updateElement for one element (the known-answer tests of
// physics/test/DamageHealing_test.cpp drive it with given cice, deltaCi)
double oracle_constant_healing(double damage, double cice, double deltaCi, double dt, double tD)
{
    double f[NSDG_IG_NFIELDS] = {};
    f[NSDG_IG_DAMAGE] = damage;
    f[NSDG_IG_CICE] = cice;
    f[NSDG_IG_DELTA_CICE] = deltaCi;
    nsdg_ice_growth_params p;
    oracle_ice_growth_default_params(&p);
    p.healing_time = tD;
    constantHealing(Elem { f, 1, 0 }, p, dt);
    return f[NSDG_IG_DAMAGE];
}

// UnescoFreezing (core/src/modules/FreezingPointModule/include/UnescoFreezing.hpp:29-39):
// Fofonoff and Millard (1983), at zero pressure
double oracle_unesco_freezing(double sss)
{
    const double a0 = -0.0575;
    const double a1 = +1.710523e-3;
    const double a2 = -2.154996e-4;
    const double b = -7.53e-4;
    const double p0 = 0;
    return sss * (a0 + a1 * std::sqrt(sss) + a2 * sss) + b * p0;
}

} // extern "C"
