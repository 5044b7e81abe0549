// C ABI of the GPU column thermodynamics (IceGrowth::update with ThermoIce0,
// HiblerSpread, ConstantHealing): create / set_field / update / get_field.
// The coupling with a dynamics handle (nsdg_ice_growth_exchange) lives with
// the dynamics handle in nsdg_capi.cpp.
#include "nsdg_ice_growth.hpp"

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

using namespace nsdg;

namespace {

// the names of the slots, in NSDG_IG_* order (IceGrowth::getState names for
// the updated and initial thicknesses, IceGrowth.cpp:72-84)
const char* const kSlotNames[NSDG_IG_NFIELDS] = { "hice", "cice", "hsnow", "tice", "qia", "dqia_dt", "qow", "qio",
    "sublim", "snowfall", "penSW", "sst", "tf", "mlbhc", "damage", "hice_updated", "cice_updated", "hsnow_updated",
    "hice_initial", "hsnow_initial", "newice", "delta_cice", "delta_hice", "tice_updated", "qic", "snow_to_ice",
    "top_melt", "bottom_melt", "snow_melt", "delta_cfreeze", "delta_cmelt", "tice_1", "tice_2", "tice_updated_1",
    "tice_updated_2" };

int slotOf(const char* name)
{
    for (int k = 0; k < NSDG_IG_NFIELDS; ++k)
        if (std::strcmp(name, kSlotNames[k]) == 0)
            return k;
    return -1;
}

bool validParams(const nsdg_ice_growth_params& p)
{
    return std::isfinite(p.ks) && p.ks > 0 && std::isfinite(p.h_min) && p.h_min >= 0 && std::isfinite(p.c_min)
        && p.c_min >= 0 && std::isfinite(p.h0) && p.h0 > 0 && std::isfinite(p.phi_m)
        && std::isfinite(p.healing_time) && p.healing_time > 0 && (p.thermo_model >= 0 && p.thermo_model <= 2)
        && (p.lateral_model == 0 || p.lateral_model == 1) && (p.healing_model == 0 || p.healing_model == 1);
}

} // namespace

extern "C" {

void nsdg_ice_growth_default_params(nsdg_ice_growth_params* p)
{
    if (!p)
        return;
    // IceGrowth / ThermoIce0 / HiblerSpread / ConstantHealing / IceMinima
    // configuration defaults (IceGrowth.cpp:119-136, ThermoIce0.cpp:22,
    // HiblerSpread.cpp:15-16, ConstantHealing.cpp:13-23, IceMinima.cpp:12-13)
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

int nsdg_ice_growth_create(size_t n_elements, const double* mask, const nsdg_ice_growth_params* p,
    nsdg_ice_growth** out)
{
    if (!out || n_elements == 0 || n_elements > (size_t(1) << 31))
        return NSDG_ERR_BAD_ARG;
    *out = nullptr;
    nsdg_ice_growth_params prm;
    nsdg_ice_growth_default_params(&prm);
    if (p)
        prm = *p;
    if (!validParams(prm))
        return NSDG_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return NSDG_ERR_NO_DEVICE;
    auto* g = new (std::nothrow) nsdg_ice_growth;
    if (!g)
        return NSDG_ERR_CUDA;
    g->n = n_elements;
    g->p = prm;
    std::vector<uint8_t> ocean(n_elements, 1);
    if (mask)
        for (size_t i = 0; i < n_elements; ++i)
            ocean[i] = mask[i] > 0 ? 1 : 0;
    const size_t bytes = size_t(NSDG_IG_NFIELDS) * n_elements * sizeof(double);
    cudaError_t e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&g->fields, bytes);
    if (e == cudaSuccess) e = cudaMalloc(&g->ocean, n_elements);
    if (e == cudaSuccess) e = cudaMallocHost(&g->staging, n_elements * sizeof(double));
    if (e == cudaSuccess) e = cudaMemsetAsync(g->fields, 0, bytes, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(g->ocean, ocean.data(), n_elements, cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) {
        nsdg_ice_growth_destroy(g);
        return NSDG_ERR_CUDA;
    }
    *out = g;
    return NSDG_OK;
}

int nsdg_ice_growth_destroy(nsdg_ice_growth* g)
{
    if (!g)
        return NSDG_OK;
    if (g->stream)
        cudaStreamSynchronize(g->stream);
    cudaFree(g->fields);
    cudaFree(g->ocean);
    cudaFreeHost(g->staging);
    if (g->stream)
        cudaStreamDestroy(g->stream);
    delete g;
    return NSDG_OK;
}

const char* nsdg_ice_growth_last_error(nsdg_ice_growth* g)
{
    return g ? g->err.c_str() : "null handle";
}

int nsdg_ice_growth_set_field(nsdg_ice_growth* g, const char* name, const double* data, size_t n)
{
    if (!g || !name || !data)
        return NSDG_ERR_BAD_ARG;
    const int k = slotOf(name);
    if (k < 0)
        return g->fail(NSDG_ERR_UNKNOWN_FIELD, std::string("set_field: unknown field ") + name);
    if (n != g->n)
        return g->fail(NSDG_ERR_SIZE_MISMATCH, "set_field: expected one value per element");
    cudaError_t e = cudaStreamSynchronize(g->stream); // the staging buffer is free
    if (e == cudaSuccess) {
        std::memcpy(g->staging, data, n * sizeof(double));
        e = cudaMemcpyAsync(g->fields + size_t(k) * g->n, g->staging, n * sizeof(double), cudaMemcpyHostToDevice,
            g->stream);
    }
    if (e != cudaSuccess)
        return g->fail(NSDG_ERR_CUDA, std::string("set_field: ") + cudaGetErrorString(e));
    g->err.clear();
    return NSDG_OK;
}

int nsdg_ice_growth_get_field(nsdg_ice_growth* g, const char* name, double* out, size_t n)
{
    if (!g || !name || !out)
        return NSDG_ERR_BAD_ARG;
    const int k = slotOf(name);
    if (k < 0)
        return g->fail(NSDG_ERR_UNKNOWN_FIELD, std::string("get_field: unknown field ") + name);
    if (n != g->n)
        return g->fail(NSDG_ERR_SIZE_MISMATCH, "get_field: expected one value per element");
    cudaError_t e = cudaMemcpyAsync(g->staging, g->fields + size_t(k) * g->n, n * sizeof(double),
        cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess)
        return g->fail(NSDG_ERR_CUDA, std::string("get_field: ") + cudaGetErrorString(e));
    std::memcpy(out, g->staging, n * sizeof(double));
    g->err.clear();
    return NSDG_OK;
}

int nsdg_ice_growth_update(nsdg_ice_growth* g, double dt)
{
    if (!g)
        return NSDG_ERR_BAD_ARG;
    if (!(dt > 0) || !std::isfinite(dt))
        return g->fail(NSDG_ERR_BAD_ARG, "update: dt must be positive");
    const cudaError_t e = launchIceGrowth(g->stream, g->n, g->ocean, g->p, dt, g->fields);
    if (e != cudaSuccess)
        return g->fail(NSDG_ERR_CUDA, std::string("update: ") + cudaGetErrorString(e));
    g->err.clear();
    return NSDG_OK;
}

int nsdg_ice_growth_time_updates(nsdg_ice_growth* g, double dt, int reps, float* ms)
{
    if (!g || !ms || reps < 1 || !(dt > 0))
        return NSDG_ERR_BAD_ARG;
    cudaEvent_t a = nullptr, b = nullptr;
    cudaError_t e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    if (e == cudaSuccess) e = launchIceGrowth(g->stream, g->n, g->ocean, g->p, dt, g->fields); // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(a, g->stream);
    for (int r = 0; r < reps && e == cudaSuccess; ++r)
        e = launchIceGrowth(g->stream, g->n, g->ocean, g->p, dt, g->fields);
    if (e == cudaSuccess) e = cudaEventRecord(b, g->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (e != cudaSuccess)
        return g->fail(NSDG_ERR_CUDA, std::string("time_updates: ") + cudaGetErrorString(e));
    return NSDG_OK;
}

} // extern "C"
