/*!
 * @file GPUDynamicsModule.cpp
 *
 * GPUMEVPDynamics and GPUBBMDynamics: the module step of the reference's
 * MEVPDynamics (core/src/modules/DynamicsModule/MEVPDynamics.cpp:36-95) and
 * BBMDynamics (BBMDynamics.cpp:19-104) with the calls going to the GB300
 * kernel through the C ABI.  ModelArray data is element-major with the
 * components contiguous (ModelArray.hpp:253-258), which is the layout the C
 * ABI takes, so a field is passed as a view of its storage without a copy.
 */

#include "GPUDynamicsModule.hpp"

#include "include/gridNames.hpp"

#include <stdexcept>
#include <string>
#include <vector>

namespace Nextsim {

namespace {
    // Degrees to radians (MEVPDynamics.cpp:20)
    const double radiansPerDegree = 0x1.1df46a2529d39p-6;

    GB300::FieldView view(const ModelArray& ma)
    {
        return { ma.getData(), ma.trueSize(), ma.nComponents() };
    }

    void assign(ModelArray& target, const std::vector<double>& values)
    {
        target.resize();
        if (values.size() != target.trueSize())
            throw std::length_error("the kernel returned " + std::to_string(values.size())
                + " values for a field of " + std::to_string(target.trueSize()) + " elements");
        target.setData(values.data());
    }

    const std::vector<std::string> namedFields = { hiceName, ciceName, uName, vName };
}

GPUDynamicsBase::GPUDynamicsBase(GB300::Rheology rheology, bool usesDamage)
    : IDynamics(usesDamage)
    , m_rheology(rheology)
    , m_params(GB300::defaultParameters())
{
    getStore().registerArray(Protected::ICE_U, &uice, RO);
    getStore().registerArray(Protected::ICE_V, &vice, RO);
}

GB300::GPUDynamicsKernel<DGCOMP>& GPUDynamicsBase::kernel() const
{
    if (!m_kernel)
        throw std::logic_error(getName() + ": setData must run before the kernel is used");
    return *m_kernel;
}

void GPUDynamicsBase::setData(const ModelState::DataMap& ms)
{
    IDynamics::setData(ms);

    const bool isSpherical = checkSpherical(ms);
    ModelArray coords = ms.at(coordsName);
    if (isSpherical)
        coords *= radiansPerDegree;

    m_kernel = std::make_unique<GB300::GPUDynamicsKernel<DGCOMP>>(m_rheology, m_params);
    const size_t nx = ModelArray::size(ModelArray::Dimension::X);
    const size_t ny = ModelArray::size(ModelArray::Dimension::Y);
    m_kernel->initialise(nx, ny, view(coords), isSpherical, view(ms.at(maskName)));

    uice = ms.at(uName);
    vice = ms.at(vName);
    for (const auto& name : namedFields)
        m_kernel->setData(name, view(ms.at(name)));

    if (m_rheology == GB300::Rheology::BBM) {
        // BBMDynamics.cpp:46-61: damage from the state, else 1 where there is ice
        if (ms.count(damageName) > 0) {
            m_kernel->setData(damageName, view(ms.at(damageName)));
        } else {
            ModelArray d(ModelArray::Type::H);
            d.resize();
            d = 1.0;
            m_kernel->setData(damageName, view(mask(d)));
        }
    }
}

void GPUDynamicsBase::update(const TimestepTime& tst)
{
    GB300::GPUDynamicsKernel<DGCOMP>& k = kernel();
    const bool bbm = m_rheology == GB300::Rheology::BBM;
    if (bbm)
        damage = damage0.data();

    // the module step of MEVPDynamics.cpp:59-87 / BBMDynamics.cpp:63-104 as
    // one library call: the same inputs and read-outs, one wait
    std::vector<std::pair<std::string, GB300::FieldView>> inputs = {
        { hiceName, view(hice.data()) },
        { ciceName, view(cice.data()) },
    };
    if (bbm)
        inputs.push_back({ damageName, view(damage) });
    inputs.insert(inputs.end(),
        { { uWindName, view(uwind.data()) }, { vWindName, view(vwind.data()) },
            { uOceanName, view(uocean.data()) }, { vOceanName, view(vocean.data()) }, { sshName, view(ssh.data()) } });
    const size_t n = k.nelements();
    std::vector<double> hOut(n), cOut(n), dOut(n), uOut(n), vOut(n), txOut(n), tyOut(n);
    std::vector<std::pair<std::string, double*>> outputs = { { hiceName, hOut.data() }, { ciceName, cOut.data() } };
    if (bbm)
        outputs.push_back({ damageName, dOut.data() });
    outputs.insert(outputs.end(),
        { { uName, uOut.data() }, { vName, vOut.data() }, { uIOStressName, txOut.data() },
            { vIOStressName, tyOut.data() } });

    k.moduleStep(inputs, { (tst.start - TimePoint()).seconds(), tst.step.seconds() }, outputs);

    assign(hice.data(), hOut);
    assign(cice.data(), cOut);
    if (bbm)
        assign(damage, dOut);
    assign(uice, uOut);
    assign(vice, vOut);
    assign(taux, txOut);
    assign(tauy, tyOut);
}

ModelState GPUDynamicsBase::getStateRecursive(const OutputSpec& os) const
{
    ModelState state(IDynamics::getStateRecursive(os));
    if (os.allComponents()) {
        ModelArray h(ModelArray::Type::DG), c(ModelArray::Type::DG);
        assign(h, kernel().getDGData(hiceName));
        assign(c, kernel().getDGData(ciceName));
        state.merge({ { hiceName, h }, { ciceName, c } });
        if (m_rheology == GB300::Rheology::BBM) {
            ModelArray d(ModelArray::Type::DG);
            assign(d, kernel().getDGData(damageName));
            state.merge({ { damageName, d } });
        }
    }
    return state;
}

namespace {
    int precisionOf(const std::string& s)
    {
        if (s == "fp64")
            return NSDG_PRECISION_FP64;
        if (s == "mixed")
            return NSDG_PRECISION_MIXED;
        throw std::invalid_argument("GPUDynamics.precision must be fp64 or mixed, not '" + s + "'");
    }
}

GPUMEVPDynamics::GPUMEVPDynamics()
    : GPUDynamicsBase(GB300::Rheology::MEVP, false)
{
}

void GPUMEVPDynamics::configure()
{
    m_params.precision = precisionOf(Configured::getConfiguration(std::string("GPUDynamics.precision"),
        std::string("fp64")));
}

GPUBBMDynamics::GPUBBMDynamics()
    : GPUDynamicsBase(GB300::Rheology::BBM, true)
{
}

void GPUBBMDynamics::configure()
{
    m_params.precision = precisionOf(Configured::getConfiguration(std::string("GPUDynamics.precision"),
        std::string("fp64")));
}

// BBMDynamics.cpp:107-120: the velocities and the DG data of h, A and damage
ModelState GPUBBMDynamics::getState() const
{
    ModelState state(IDynamics::getState());
    ModelArray h(ModelArray::Type::DG), c(ModelArray::Type::DG), d(ModelArray::Type::DG);
    assign(h, kernel().getDGData(hiceName));
    assign(c, kernel().getDGData(ciceName));
    assign(d, kernel().getDGData(damageName));
    state.merge({ { hiceName, h }, { ciceName, c }, { damageName, d } });
    return state;
}

} /* namespace Nextsim */
