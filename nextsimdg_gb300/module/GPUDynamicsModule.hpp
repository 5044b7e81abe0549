/*!
 * @file GPUDynamicsModule.hpp
 *
 * The GB300 dynamics kernel as neXtSIM_DG dynamics modules: GPUMEVPDynamics
 * and GPUBBMDynamics are the reference's MEVPDynamics and BBMDynamics
 * (core/src/modules/DynamicsModule/include/MEVPDynamics.hpp:28-44,
 * include/BBMDynamics.hpp:23-41) with Nextsim::GB300::GPUDynamicsKernel in
 * place of MEVPDynamicsKernel<DGCOMP> / BBMDynamicsKernel<DGCOMP>.  They
 * derive from the reference's IDynamics (core/src/modules/include/IDynamics.hpp)
 * and are compiled against the reference's own headers: in the reference's
 * build they sit in core/src/modules/DynamicsModule/ with one module.cfg
 * section each.
 *
 * Configuration (Configured, the reference's configuration layer):
 *   GPUDynamics.precision   "fp64" (default: the reference's arithmetic) or
 *                           "mixed" (FP32 bulk, FP64 Delta/viscosity,
 *                           inverse mass matrices and conservation sums)
 * The kernel is created on the first setData, after configure().
 */

#ifndef GPUDYNAMICSMODULE_HPP
#define GPUDYNAMICSMODULE_HPP

#include "include/Configured.hpp"
#include "include/IDynamics.hpp"

#include "nsdg_dynamics_kernel.hpp"

#include <memory>

#ifndef DGCOMP
#error "Number of DG components (DGCOMP) not defined"
#endif

namespace Nextsim {

class GPUDynamicsBase : public IDynamics {
public:
    GPUDynamicsBase(GB300::Rheology rheology, bool usesDamage);

    void setData(const ModelState::DataMap&) override;
    void update(const TimestepTime& tst) override;
    ModelState getStateRecursive(const OutputSpec& os) const override;

    //! The kernel's parameters (nsdg_params), set before the first setData.
    nsdg_params& parameters() { return m_params; }

protected:
    GB300::Rheology m_rheology;
    nsdg_params m_params;
    std::unique_ptr<GB300::GPUDynamicsKernel<DGCOMP>> m_kernel;

    GB300::GPUDynamicsKernel<DGCOMP>& kernel() const;
};

class GPUMEVPDynamics : public GPUDynamicsBase, public Configured<GPUMEVPDynamics> {
public:
    GPUMEVPDynamics();
    std::string getName() const override { return "GPUMEVPDynamics"; }
    void configure() override;
};

class GPUBBMDynamics : public GPUDynamicsBase, public Configured<GPUBBMDynamics> {
public:
    GPUBBMDynamics();
    std::string getName() const override { return "GPUBBMDynamics"; }
    void configure() override;
    ModelState getState() const override;
};

} /* namespace Nextsim */

#endif /* GPUDYNAMICSMODULE_HPP */
