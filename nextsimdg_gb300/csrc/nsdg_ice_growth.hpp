// Column thermodynamics (IceGrowth with ThermoIce0, HiblerSpread,
// ConstantHealing) on the GPU: handle layout and launchers.
#pragma once

#include "nsdg.h"

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>

struct nsdg_ice_growth {
    size_t n = 0;
    nsdg_ice_growth_params p {};
    cudaStream_t stream = nullptr;
    double* fields = nullptr;   // [NSDG_IG_NFIELDS][n] on the device
    uint8_t* ocean = nullptr;   // n, 1 = ocean element
    double* staging = nullptr;  // pinned host buffer of n doubles
    std::string err;
    int fail(int code, const std::string& m)
    {
        err = m;
        return code;
    }
};

namespace nsdg {
// One IceGrowth::update of dt seconds over the ocean elements.
cudaError_t launchIceGrowth(cudaStream_t s, size_t n, const uint8_t* ocean, const nsdg_ice_growth_params& p,
    double dt, double* fields);
// DG0 components of the dynamics' h, A, damage -> growth inputs "hice",
// "cice", "damage" (damage may be null: left as it is).
cudaError_t launchIceGrowthFromDynamics(cudaStream_t s, size_t n, const double* hiceDG, const double* ciceDG,
    const double* damageDG, double* fields);
// hice_updated x cice_updated, cice_updated, damage -> the dynamics' DG
// fields (component 0; components 1 .. dg-1 zeroed); damageDG may be null.
cudaError_t launchIceGrowthToDynamics(cudaStream_t s, size_t n, int dg, const double* fields, double* hiceDG,
    double* ciceDG, double* damageDG);
} // namespace nsdg
