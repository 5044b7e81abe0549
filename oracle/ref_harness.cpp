/*
 * ref_harness.cpp — C ABI around the reference's own dynamics kernels, built
 * from the unmodified reference sources (plus the project's Eigen subset,
 * oracle/eigen_min) into oracle/_ref/libnsdg_ref.so by `make -C oracle ref`.
 *
 * TEST INFRASTRUCTURE ONLY: this is the reference implementation the tests
 * pin the CPU restatement (oracle/nsdg_oracle.cpp) and the GPU path against.
 * It is built only where the reference sources are present and is never
 * linked into the product.
 *
 * It drives the reference classes through their public API, the way the
 * model's dynamics modules do (core/src/modules/DynamicsModule/
 * MEVPDynamics.cpp:29-101, BBMDynamics.cpp:19-134):
 *   MEVPDynamicsKernel<DG>(VPParameters)        MEVPDynamicsKernel.hpp:22-26
 *   BBMDynamicsKernel<DG>(MEBParameters)        BBMDynamicsKernel.hpp:26-29
 *   initialise(coords, isSpherical, mask)       DynamicsKernel.hpp:44-75
 *   setData / getDG0Data / getDGData            DynamicsKernel.hpp:93-156,
 *                                               CGDynamicsKernel.cpp:54-118
 *   update(TimestepTime)                        VPCGDynamicsKernel.hpp:63-94,
 *                                               BrittleCGDynamicsKernel.hpp:91-136
 * and sets the ModelArray dimensions (ModelArray::setDimension,
 * setNComponents; core/src/ModelArray.cpp:187-213) for the handle's grid
 * before every call, since ModelArray keeps them in static storage.
 *
 * It also replays the procedure of the reference's transport tests
 * (dynamics/test/Advection_test.cpp:136-301,
 * dynamics/test/AdvectionPeriodicBC_test.cpp:117-297) on the reference's
 * DGTransport, Interpolations, Tools and dgLimit code, so that its results
 * can be checked against the golden values those tests hold.
 */
#include "include/BBMDynamicsKernel.hpp"
#include "MEVPDynamicsKernel.hpp" // the copy in oracle/_ref/gen (alpha, beta from ref_params.h)

#include "include/DGTransport.hpp"
#include "include/Interpolations.hpp"
#include "include/Tools.hpp"
#include "include/dgLimit.hpp"

#include "include/ModelArray.hpp"
#include "include/Time.hpp"

#include <cstring>
#include <memory>
#include <string>

double nsdg_ref_alpha = 1500.0;
double nsdg_ref_beta = 1500.0;

using namespace Nextsim;

namespace {

// The reference's kernels keep the sub-cycle count in a protected member
// (DynamicsKernel.hpp:187); these subclasses only expose a setter.
template <int DG> struct RefMEVP : public MEVPDynamicsKernel<DG> {
    explicit RefMEVP(const DynamicsParameters& p)
        : MEVPDynamicsKernel<DG>(p)
    {
    }
    void setSubSteps(size_t n) { this->nSteps = n; }
    CGVector<CGdegree> cg(const std::string& name) const
    {
        if (name == "u")
            return this->u;
        if (name == "v")
            return this->v;
        return this->getIceOceanStress(name);
    }
    const DGVector<DGstressComp>& stress(int k) const { return k == 0 ? this->s11 : (k == 1 ? this->s12 : this->s22); }
};
template <int DG> struct RefBBM : public BBMDynamicsKernel<DG> {
    explicit RefBBM(const DynamicsParameters& p)
        : BBMDynamicsKernel<DG>(p)
    {
    }
    void setSubSteps(size_t n) { this->nSteps = n; }
    CGVector<CGdegree> cg(const std::string& name) const
    {
        if (name == "u")
            return this->u;
        if (name == "v")
            return this->v;
        return this->getIceOceanStress(name);
    }
    const DGVector<DGstressComp>& stress(int k) const { return k == 0 ? this->s11 : (k == 1 ? this->s12 : this->s22); }
};

struct Base {
    virtual ~Base() = default;
    virtual DynamicsKernel<1, DGstressComp>* k1() { return nullptr; }
    virtual DynamicsKernel<3, DGstressComp>* k3() { return nullptr; }
    virtual DynamicsKernel<6, DGstressComp>* k6() { return nullptr; }
    virtual void setSubSteps(size_t) = 0;
    virtual CGVector<CGdegree> cg(const std::string& name) const = 0;
    virtual const DGVector<DGstressComp>& stress(int k) const = 0;
};

template <int DG, class K> struct Holder : Base {
    std::unique_ptr<VPParameters> vp;
    std::unique_ptr<MEBParameters> meb;
    std::unique_ptr<K> k;
    void setSubSteps(size_t n) override { k->setSubSteps(n); }
    CGVector<CGdegree> cg(const std::string& name) const override { return k->cg(name); }
    const DGVector<DGstressComp>& stress(int i) const override { return k->stress(i); }
    DynamicsKernel<1, DGstressComp>* k1() override
    {
        if constexpr (DG == 1)
            return k.get();
        return nullptr;
    }
    DynamicsKernel<3, DGstressComp>* k3() override
    {
        if constexpr (DG == 3)
            return k.get();
        return nullptr;
    }
    DynamicsKernel<6, DGstressComp>* k6() override
    {
        if constexpr (DG == 6)
            return k.get();
        return nullptr;
    }
};

struct Handle {
    int rheology = 0, dg = 6;
    size_t nx = 0, ny = 0;
    std::unique_ptr<Base> impl;
    std::string err;
};

template <int DG> Base* makeKernel(int rheology, double alpha, double beta)
{
    nsdg_ref_alpha = alpha;
    nsdg_ref_beta = beta;
    if (rheology == 0) {
        auto* h = new Holder<DG, RefMEVP<DG>>();
        h->vp = std::make_unique<VPParameters>();
        h->k = std::make_unique<RefMEVP<DG>>(*h->vp);
        return h;
    }
    auto* h = new Holder<DG, RefBBM<DG>>();
    h->meb = std::make_unique<MEBParameters>();
    h->k = std::make_unique<RefBBM<DG>>(*h->meb);
    return h;
}

void setDims(const Handle* h)
{
    ModelArray::setDimension(ModelArray::Dimension::X, h->nx);
    ModelArray::setDimension(ModelArray::Dimension::Y, h->ny);
    ModelArray::setDimension(ModelArray::Dimension::XVERTEX, h->nx + 1);
    ModelArray::setDimension(ModelArray::Dimension::YVERTEX, h->ny + 1);
    ModelArray::setDimension(ModelArray::Dimension::XCG, CGdegree * h->nx + 1);
    ModelArray::setDimension(ModelArray::Dimension::YCG, CGdegree * h->ny + 1);
    ModelArray::setNComponents(ModelArray::Type::DG, size_t(h->dg));
    ModelArray::setNComponents(ModelArray::Type::DGSTRESS, size_t(DGstressComp));
}

// Calls f(kernel) on the handle's DynamicsKernel<DG, 8>.
template <class F> int withKernel(Handle* h, F f)
{
    try {
        setDims(h);
        if (h->dg == 1)
            f(*h->impl->k1());
        else if (h->dg == 3)
            f(*h->impl->k3());
        else
            f(*h->impl->k6());
        return 0;
    } catch (const std::out_of_range& e) {
        h->err = e.what();
        return 2;
    } catch (const std::exception& e) {
        h->err = e.what();
        return 7;
    }
}

} // namespace

extern "C" {

void* ref_kernel_create(int rheology, int dg, double alpha, double beta, int n_steps)
{
    if ((rheology != 0 && rheology != 1) || (dg != 1 && dg != 3 && dg != 6))
        return nullptr;
    auto* h = new Handle();
    h->rheology = rheology;
    h->dg = dg;
    h->impl.reset(dg == 1 ? makeKernel<1>(rheology, alpha, beta)
                          : (dg == 3 ? makeKernel<3>(rheology, alpha, beta) : makeKernel<6>(rheology, alpha, beta)));
    if (n_steps > 0)
        h->impl->setSubSteps(size_t(n_steps));
    return h;
}

void ref_kernel_destroy(void* p) { delete static_cast<Handle*>(p); }

const char* ref_kernel_last_error(void* p) { return static_cast<Handle*>(p)->err.c_str(); }

int ref_kernel_initialise(void* p, size_t nx, size_t ny, const double* coords, int is_spherical, const double* mask)
{
    Handle* h = static_cast<Handle*>(p);
    h->nx = nx;
    h->ny = ny;
    return withKernel(h, [&](auto& k) {
        ModelArray c(ModelArray::Type::VERTEX);
        c.resize();
        c.setData(coords);
        ModelArray m(ModelArray::Type::H);
        m.resize();
        m.setData(mask);
        k.initialise(c, is_spherical != 0, m);
    });
}

// data: n_elements * n_comp doubles, element-major.  n_comp == the DG count
// makes a DG field, 8 a DGSTRESS field, anything else an H field of
// component 0 (the module's HField inputs).
int ref_kernel_set_data(void* p, const char* name, const double* data, size_t n, size_t ncomp)
{
    Handle* h = static_cast<Handle*>(p);
    if (n != h->nx * h->ny) {
        h->err = "set_data: size mismatch";
        return 3;
    }
    return withKernel(h, [&](auto& k) {
        const ModelArray::Type t = ncomp == size_t(h->dg) && ncomp > 1 ? ModelArray::Type::DG
            : (ncomp == size_t(DGstressComp) ? ModelArray::Type::DGSTRESS : ModelArray::Type::H);
        ModelArray a(t);
        a.resize();
        if (t == ModelArray::Type::H && ncomp > 1) {
            for (size_t i = 0; i < n; ++i)
                a[i] = data[i * ncomp];
        } else {
            a.setData(data);
        }
        k.setData(name, a);
    });
}

int ref_kernel_get_dg0(void* p, const char* name, double* out, size_t n)
{
    Handle* h = static_cast<Handle*>(p);
    return withKernel(h, [&](auto& k) {
        ModelArray a = k.getDG0Data(name);
        if (a.trueSize() != n)
            throw std::logic_error("get_dg0: size mismatch");
        for (size_t i = 0; i < n; ++i)
            out[i] = a[i];
    });
}

int ref_kernel_get_dg(void* p, const char* name, double* out, size_t n, size_t ncomp)
{
    Handle* h = static_cast<Handle*>(p);
    return withKernel(h, [&](auto& k) {
        ModelArray a = k.getDGData(name);
        if (a.trueSize() != n || a.nComponents() != ncomp)
            throw std::logic_error("get_dg: size mismatch");
        std::memcpy(out, a.getData(), n * ncomp * sizeof(double));
    });
}

int ref_kernel_update(void* p, double start, double dt)
{
    Handle* h = static_cast<Handle*>(p);
    (void)start;
    return withKernel(h, [&](auto& k) {
        TimestepTime tst { TimePoint(), Duration(dt) };
        k.update(tst);
    });
}

// The CG2 velocity (u, v) or ice-ocean stress (uiostress, viostress) node
// values, (2nx+1)(2ny+1) doubles.
int ref_kernel_get_cg(void* p, const char* name, double* out, size_t n)
{
    Handle* h = static_cast<Handle*>(p);
    try {
        setDims(h);
        CGVector<CGdegree> v = h->impl->cg(name);
        if (size_t(v.rows()) != n) {
            h->err = "get_cg: size mismatch";
            return 3;
        }
        for (size_t i = 0; i < n; ++i)
            out[i] = v(i);
        return 0;
    } catch (const std::exception& e) {
        h->err = e.what();
        return 7;
    }
}

// s11, s12 or s22: n_elements x 8 doubles.
int ref_kernel_get_stress(void* p, const char* name, double* out, size_t n)
{
    Handle* h = static_cast<Handle*>(p);
    const std::string s(name);
    const int k = s == "s11" ? 0 : (s == "s12" ? 1 : (s == "s22" ? 2 : -1));
    if (k < 0) {
        h->err = "get_stress: s11, s12 or s22";
        return 2;
    }
    const DGVector<DGstressComp>& v = h->impl->stress(k);
    if (size_t(v.rows()) * DGstressComp != n) {
        h->err = "get_stress: size mismatch";
        return 3;
    }
    for (size_t e = 0; e < size_t(v.rows()); ++e)
        for (int c = 0; c < DGstressComp; ++c)
            out[e * DGstressComp + c] = v(e, c);
    return 0;
}


} // extern "C"

// ---- the transport tests -------------------------------------------------
// The analytic fields and meshes below are the test cases' definitions
// (Advection_test.cpp:56-100,198-241; AdvectionPeriodicBC_test.cpp:68-116,
// 207-255), written here as Interpolations::Function objects.

namespace {
struct Bump : Nextsim::Interpolations::Function {
    double L;
    explicit Bump(double l)
        : L(l)
    {
    }
    double operator()(double x, double y) const override
    {
        const double X = x / L, Y = y / L;
        const double r = ((X - 0.25) * (X - 0.25) + (Y - 0.5) * (Y - 0.5)) / 0.025;
        return r < 1 ? std::exp(-1.0 / (1.0 - r)) : 0.0;
    }
};
struct RotX : Nextsim::Interpolations::Function {
    double L;
    explicit RotX(double l)
        : L(l)
    {
    }
    double operator()(double, double y) const override { return (y - 0.5 * L) * 2.0 * M_PI / L; }
};
struct RotY : Nextsim::Interpolations::Function {
    double L;
    explicit RotY(double l)
        : L(l)
    {
    }
    double operator()(double x, double) const override { return (0.5 * L - x) * 2.0 * M_PI / L; }
};
struct RingX : Nextsim::Interpolations::Function {
    double R1;
    explicit RingX(double r)
        : R1(r)
    {
    }
    double operator()(double, double y) const override { return y * 2.0 * M_PI / R1; }
};
struct RingY : Nextsim::Interpolations::Function {
    double R1;
    explicit RingY(double r)
        : R1(r)
    {
    }
    double operator()(double x, double) const override { return -x * 2.0 * M_PI / R1; }
};
// four shapes on the ring: a smooth bump, a slotted disc, a cone, a disc
struct Shapes : Nextsim::Interpolations::Function {
    double operator()(double x, double y) const override
    {
        const double a = 50000.0, c = 175000.0;
        double r = ((x + c) / a) * ((x + c) / a) + (y / a) * (y / a);
        if (r < 1.0)
            return std::exp(1.0) * std::exp(-1.0 / (1.0 - r));
        r = (x / a) * (x / a) + ((y - c) / a) * ((y - c) / a);
        if (r < 1.0)
            return (y > c || std::fabs(x) > 15000.0) ? 1.0 : 0.0;
        r = std::sqrt(((x - c) / a) * ((x - c) / a) + (y / a) * (y / a));
        if (r < 1.0)
            return 1.0 - r;
        r = std::sqrt((x / a) * (x / a) + ((y + c) / a) * ((y + c) / a));
        return r < 1.0 ? 1.0 : 0.0;
    }
};

void boxMesh(ParametricMesh& m, double Lx, double Ly, size_t Nx, size_t Ny, double distort)
{
    m.reset();
    m.nx = Nx;
    m.ny = Ny;
    m.nnodes = (Nx + 1) * (Ny + 1);
    m.nelements = Nx * Ny;
    m.vertices.resize(m.nnodes, 2);
    for (size_t iy = 0, k = 0; iy <= Ny; ++iy)
        for (size_t ix = 0; ix <= Nx; ++ix, ++k) {
            m.vertices(k, 0) = Lx * ix / Nx + Lx * distort * std::sin(M_PI * ix / Nx * 3.0) * std::sin(M_PI * iy / Ny);
            m.vertices(k, 1)
                = Ly * iy / Ny + Ly * distort * std::sin(M_PI * iy / Ny * 2.0) * std::sin(M_PI * ix / Nx * 2.0);
        }
    m.landmask.resize(m.nelements, 1);
    for (size_t i = 0; i < Nx; ++i) {
        m.dirichlet[0].push_back(i);
        m.dirichlet[2].push_back(Nx * (Ny - 1) + i);
    }
    for (size_t j = 0; j < Ny; ++j) {
        m.dirichlet[1].push_back(j * Nx + Nx - 1);
        m.dirichlet[3].push_back(j * Nx);
    }
}

void ringMesh(ParametricMesh& m, double R0, double R1, size_t Nx, size_t Ny)
{
    m.reset();
    m.nx = Nx;
    m.ny = Ny;
    m.nnodes = (Nx + 1) * (Ny + 1);
    m.nelements = Nx * Ny;
    m.vertices.resize(m.nnodes, 2);
    for (size_t iy = 0, k = 0; iy <= Ny; ++iy)
        for (size_t ix = 0; ix <= Nx; ++ix, ++k) {
            const double r = R0 + (R1 - R0) * iy / Ny, p = -2.0 * M_PI * ix / Nx;
            m.vertices(k, 0) = r * std::cos(p);
            m.vertices(k, 1) = r * std::sin(p);
        }
    m.landmask.resize(m.nelements, 1);
    for (size_t i = 0; i < Nx; ++i) {
        m.dirichlet[0].push_back(i);
        m.dirichlet[2].push_back(Nx * (Ny - 1) + i);
    }
    m.periodic.resize(1);
    m.periodic[0].resize(Ny);
    for (size_t j = 0; j < Ny; ++j)
        m.periodic[0][j] = { 1, (j + 1) * Nx - 1, j * Nx, j * (Nx + 1) + j };
}

template <int DG> double advection(double distort, int it, double* massloss)
{
    const double Lx = 409600.0, Ly = 512000.0;
    const size_t Nx = size_t(12) << it, Ny = size_t(13) << it;
    const int deg = DG == 1 ? 0 : (DG == 3 ? 1 : 2);
    const size_t NT = size_t(100 * (deg + 1) * (deg + 1)) << it;
    ParametricMesh m(CARTESIAN);
    boxMesh(m, Lx, Ly, Nx, Ny, distort);
    DGTransport<DG> tr(m);
    tr.settimesteppingscheme(DG < 3 ? "rk2" : "rk3");
    const double dt = Lx / NT;
    DGVector<DG> phi;
    phi.resize_by_mesh(m);
    Interpolations::Function2DG(m, phi, Bump(Lx));
    const double initial = Tools::MeanValue(m, phi);
    Interpolations::Function2DG(m, tr.GetVx(), RotX(Lx));
    Interpolations::Function2DG(m, tr.GetVy(), RotY(Lx));
    for (size_t i = 1; i <= NT; ++i) {
        tr.reinitnormalvelocity();
        tr.step(dt, phi);
    }
    if (massloss)
        *massloss = (initial - Tools::MeanValue(m, phi)) / initial;
    return std::sqrt(Interpolations::L2ErrorFunctionDG(m, phi, Bump(Lx))) / Lx;
}

template <int DG> double periodic(int it, double* massloss)
{
    const double R0 = 100000.0, R1 = 250000.0;
    const size_t Nx = size_t(32) << it, Ny = size_t(4) << it;
    const int deg = DG == 1 ? 0 : (DG == 3 ? 1 : 2);
    const size_t NT = size_t(50 * (deg + 1) * (deg + 1)) << it;
    ParametricMesh m(CARTESIAN);
    ringMesh(m, R0, R1, Nx, Ny);
    DGTransport<DG> tr(m);
    tr.settimesteppingscheme(DG < 3 ? "rk2" : "rk3");
    const double dt = R1 / NT;
    DGVector<DG> phi;
    phi.resize_by_mesh(m);
    Interpolations::Function2DG(m, phi, Shapes());
    LimitMax(phi, 1.0);
    const double initial = Tools::MeanValue(m, phi);
    Interpolations::Function2DG(m, tr.GetVx(), RingX(R1));
    Interpolations::Function2DG(m, tr.GetVy(), RingY(R1));
    for (size_t i = 1; i <= NT; ++i) {
        tr.reinitnormalvelocity();
        tr.step(dt, phi);
        LimitMax(phi, 1.0);
        LimitMin(phi, 0.0);
    }
    if (massloss)
        *massloss = (initial - Tools::MeanValue(m, phi)) / initial;
    return std::sqrt(Interpolations::L2ErrorFunctionDG(m, phi, Shapes())) / R0;
}
} // namespace

extern "C" {

// L2 error of the rotating-bump test (Advection_test.cpp:136-196,244-268)
double ref_advection_golden(int dg, double distort, int it, double* massloss)
{
    return dg == 1 ? advection<1>(distort, it, massloss)
                   : (dg == 3 ? advection<3>(distort, it, massloss) : advection<6>(distort, it, massloss));
}

// L2 error of the periodic ring test (AdvectionPeriodicBC_test.cpp:117-276)
double ref_periodic_golden(int dg, int it, double* massloss)
{
    return dg == 1 ? periodic<1>(it, massloss) : (dg == 3 ? periodic<3>(it, massloss) : periodic<6>(it, massloss));
}

} // extern "C"
