// C ABI over neXtSIM_DG dynamics modules, for the module-level tests.
//
// TEST INFRASTRUCTURE ONLY.  Built by `make -C oracle module` where the
// reference sources are: the reference's own module framework (IDynamics,
// ModelComponent, the configuration layer against oracle/boost_min) and its
// MEVPDynamics and BBMDynamics modules
// (core/src/modules/DynamicsModule/{MEVPDynamics,BBMDynamics}.cpp), compiled
// unmodified, next to the product's adapters GPUMEVPDynamics and
// GPUBBMDynamics (nextsimdg_gb300/module/), which call the GB300 kernel
// through its C ABI.  The harness plays the rest of the model: it owns the
// arrays the dynamics module reads and writes through the shared store
// (ModelArrayReferenceStore: h, A, snow, damage, winds, ocean, ssh;
// PrognosticData.cpp:87-95 fills them the same way), calls setData with an
// initial ModelState and update with a TimestepTime per step, and reads the
// results back from the store.
#include "include/BBMDynamics.hpp"
#include "include/MEVPDynamics.hpp"

#include "GPUDynamicsModule.hpp"

#include "include/gridNames.hpp"

#include <cstring>
#include <exception>
#include <memory>
#include <sstream>
#include <string>

double nsdg_ref_alpha = 1500.0;
double nsdg_ref_beta = 1500.0;

using namespace Nextsim;

namespace {
struct Harness {
    size_t nx = 0, ny = 0;
    HField hice { ModelArray::Type::H }, cice { ModelArray::Type::H }, hsnow { ModelArray::Type::H };
    HField damage0 { ModelArray::Type::H };
    HField uwind { ModelArray::Type::H }, vwind { ModelArray::Type::H };
    HField uocean { ModelArray::Type::H }, vocean { ModelArray::Type::H }, ssh { ModelArray::Type::H };
    std::unique_ptr<IDynamics> dyn;
    std::string err;
};
std::string g_err;

int fail(Harness* h, const std::string& msg, int code = 1)
{
    (h ? h->err : g_err) = msg;
    return code;
}

void fill(ModelArray& a, const double* src)
{
    a.resize();
    a.setData(src);
}
} // namespace

extern "C" {

const char* mod_last_error(void* hp) { return hp ? static_cast<Harness*>(hp)->err.c_str() : g_err.c_str(); }

// kind: MEVPDynamics, BBMDynamics (the reference's), GPUMEVPDynamics,
// GPUBBMDynamics (the product's); precision (GPU modules): 0 FP64, 1 mixed.
void* mod_create(const char* kind, size_t nx, size_t ny, int precision)
{
    try {
        ModelArray::setDimension(ModelArray::Dimension::X, nx);
        ModelArray::setDimension(ModelArray::Dimension::Y, ny);
        ModelArray::setDimension(ModelArray::Dimension::XVERTEX, nx + 1);
        ModelArray::setDimension(ModelArray::Dimension::YVERTEX, ny + 1);
        ModelArray::setDimension(ModelArray::Dimension::XCG, CGdegree * nx + 1);
        ModelArray::setDimension(ModelArray::Dimension::YCG, CGdegree * ny + 1);
        ModelArray::setNComponents(ModelArray::Type::DG, size_t(DGCOMP));
        ModelArray::setNComponents(ModelArray::Type::DGSTRESS, size_t(DGSTRESSCOMP));
        auto h = std::make_unique<Harness>();
        h->nx = nx;
        h->ny = ny;
        for (HField* a : { &h->hice, &h->cice, &h->hsnow, &h->damage0, &h->uwind, &h->vwind, &h->uocean,
                 &h->vocean, &h->ssh }) {
            a->resize();
            *a = 0.0;
        }
        auto& store = ModelComponent::getStore();
        store.registerArray(Shared::H_ICE, &h->hice, RW);
        store.registerArray(Shared::C_ICE, &h->cice, RW);
        store.registerArray(Shared::H_SNOW, &h->hsnow, RW);
        store.registerArray(Protected::DAMAGE, &h->damage0, RO);
        store.registerArray(Protected::WIND_U, &h->uwind, RO);
        store.registerArray(Protected::WIND_V, &h->vwind, RO);
        store.registerArray(Protected::OCEAN_U, &h->uocean, RO);
        store.registerArray(Protected::OCEAN_V, &h->vocean, RO);
        store.registerArray(Protected::SSH, &h->ssh, RO);
        const std::string k(kind);
        if (k == "MEVPDynamics") {
            h->dyn = std::make_unique<MEVPDynamics>();
        } else if (k == "BBMDynamics") {
            h->dyn = std::make_unique<BBMDynamics>();
        } else if (k == "GPUMEVPDynamics" || k == "GPUBBMDynamics") {
            std::unique_ptr<GPUDynamicsBase> g;
            if (k == "GPUMEVPDynamics")
                g = std::make_unique<GPUMEVPDynamics>();
            else
                g = std::make_unique<GPUBBMDynamics>();
            g->parameters().precision = precision;
            h->dyn = std::move(g);
        } else {
            fail(nullptr, "unknown module " + k);
            return nullptr;
        }
        return h.release();
    } catch (const std::exception& e) {
        fail(nullptr, e.what());
        return nullptr;
    }
}

void mod_destroy(void* hp) { delete static_cast<Harness*>(hp); }

// Configuration text in the reference's format ("[section]", "key = value")
// as the only configuration source, then the module's configure().
int mod_configure(void* hp, const char* text)
{
    Harness* h = static_cast<Harness*>(hp);
    try {
        Configurator::clear();
        std::stringstream ss(text ? text : "");
        Configurator::addSStream(ss);
        if (auto* c = dynamic_cast<Configured<GPUMEVPDynamics>*>(h->dyn.get()))
            c->configure();
        else if (auto* c = dynamic_cast<Configured<GPUBBMDynamics>*>(h->dyn.get()))
            c->configure();
        else if (auto* c = dynamic_cast<Configured<MEVPDynamics>*>(h->dyn.get()))
            c->configure();
        Configurator::clear();
        return 0;
    } catch (const std::exception& e) {
        Configurator::clear();
        return fail(h, e.what());
    }
}

// The precision a GPU module will create its kernel with (-1: not a GPU module).
int mod_precision(void* hp)
{
    auto* g = dynamic_cast<GPUDynamicsBase*>(static_cast<Harness*>(hp)->dyn.get());
    return g ? g->parameters().precision : -1;
}

// coords: (nx+1)(ny+1) x 2 (x, y in metres, or lon, lat in degrees);
// mask, hice, cice, u, v: nx*ny; damage: nx*ny or null (the module's default)
int mod_set_state(void* hp, const double* coords, int spherical, const double* mask, const double* hice,
    const double* cice, const double* u, const double* v, const double* damage)
{
    Harness* h = static_cast<Harness*>(hp);
    try {
        ModelArray c(ModelArray::Type::VERTEX);
        fill(c, coords);
        HField m(ModelArray::Type::H), hi(ModelArray::Type::H), ci(ModelArray::Type::H);
        HField uu(ModelArray::Type::H), vv(ModelArray::Type::H), axis(ModelArray::Type::H);
        fill(m, mask);
        fill(hi, hice);
        fill(ci, cice);
        fill(uu, u);
        fill(vv, v);
        axis.resize();
        axis = 0.0;
        ModelState::DataMap ms = {
            { coordsName, c },
            { maskName, m },
            { hiceName, hi },
            { ciceName, ci },
            { uName, uu },
            { vName, vv },
            { spherical ? longitudeName : xName, axis },
            { spherical ? latitudeName : yName, axis },
        };
        if (damage) {
            HField d(ModelArray::Type::H);
            fill(d, damage);
            ms.insert({ damageName, d });
        }
        h->hice.setData(hice);
        h->cice.setData(cice);
        if (damage)
            h->damage0.setData(damage);
        else
            h->damage0 = 1.0;
        h->dyn->setData(ms);
        return 0;
    } catch (const std::exception& e) {
        return fail(h, e.what());
    }
}

// One model step: the forcing arrays (nx*ny each; null leaves the previous
// value) are put into the store, then update, then the updated damage is
// copied to the damage the next step starts from.
int mod_step(void* hp, double t_start, double dt, const double* uwind, const double* vwind, const double* uocean,
    const double* vocean, const double* ssh)
{
    Harness* h = static_cast<Harness*>(hp);
    try {
        if (uwind)
            h->uwind.setData(uwind);
        if (vwind)
            h->vwind.setData(vwind);
        if (uocean)
            h->uocean.setData(uocean);
        if (vocean)
            h->vocean.setData(vocean);
        if (ssh)
            h->ssh.setData(ssh);
        TimestepTime tst { TimePoint() + Duration(t_start), Duration(dt) };
        h->dyn->update(tst);
        // PrognosticData.cpp:108-118: the updated damage is the next step's
        // damage
        ModelArrayRef<Shared::DAMAGE> upd(ModelComponent::getStore());
        h->damage0.setData(upd.data());
        return 0;
    } catch (const std::exception& e) {
        return fail(h, e.what());
    }
}

// The fields the model sees after a step: hice, cice (the shared arrays the
// module wrote), u, v (the module's velocity arrays), damage (the updated
// shared damage), taux, tauy (the ice-ocean stress for the coupler).
int mod_get(void* hp, const char* name, double* out, size_t n)
{
    Harness* h = static_cast<Harness*>(hp);
    try {
        const std::string f(name);
        const ModelArray* a = nullptr;
        ModelArrayRef<Protected::ICE_U> u(ModelComponent::getStore());
        ModelArrayRef<Protected::ICE_V> v(ModelComponent::getStore());
        ModelArrayRef<Shared::DAMAGE> d(ModelComponent::getStore());
        ModelArrayRef<Protected::IO_STRESS_U> tx(ModelComponent::getStore());
        ModelArrayRef<Protected::IO_STRESS_V> ty(ModelComponent::getStore());
        if (f == "hice")
            a = &h->hice;
        else if (f == "cice")
            a = &h->cice;
        else if (f == "u")
            a = &u.data();
        else if (f == "v")
            a = &v.data();
        else if (f == "damage")
            a = &d.data();
        else if (f == "taux")
            a = &tx.data();
        else if (f == "tauy")
            a = &ty.data();
        else
            return fail(h, "unknown read-out " + f, 2);
        if (a->trueSize() != n)
            return fail(h, f + ": " + std::to_string(a->trueSize()) + " values, asked for " + std::to_string(n), 3);
        std::memcpy(out, a->getData(), n * sizeof(double));
        return 0;
    } catch (const std::exception& e) {
        return fail(h, e.what());
    }
}

} // extern "C"
