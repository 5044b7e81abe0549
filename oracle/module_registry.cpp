// Stand-ins for the parts of the reference's module framework that its CMake
// build generates or that need libraries absent here (Boost.Log).
//
// TEST INFRASTRUCTURE ONLY (the module build, oracle/Makefile `module`).
//
// * The damage-healing module registry.  The reference generates it from
//   physics/src/modules/DamageHealingModule/module.cfg with
//   core/src/modules/module_maker.py: Module<IDamageHealing>'s name, its
//   default implementation and the map from implementation names to
//   generators, plus the explicit instantiation that MEVPDynamics.hpp:25
//   declares extern.  This registry holds NoHealing only, the implementation
//   MEVPDynamics::configure selects (MEVPDynamics.cpp:22-25), and makes it the
//   default.
// * Logged::log (core/src/Logged.cpp:83-86 sends messages through Boost.Log):
//   here to standard error.
#include "include/IDamageHealing.hpp"
#include "include/Logged.hpp"
#include "include/NextsimModule.hpp"
#include "DamageHealingModule/include/NoHealing.hpp"

#include <iostream>

namespace Module {

template <> std::string Module<Nextsim::IDamageHealing>::moduleName() { return "Nextsim::IDamageHealing"; }

template <> std::string Module<Nextsim::IDamageHealing>::getDefaultImplementationName()
{
    return "Nextsim::NoHealing";
}

template <> const Module<Nextsim::IDamageHealing>::Map& Module<Nextsim::IDamageHealing>::functionMap()
{
    static const Map map = {
        { "Nextsim::NoHealing", newImpl<Nextsim::IDamageHealing, Nextsim::NoHealing> },
    };
    return map;
}

template class Module<Nextsim::IDamageHealing>;

} // namespace Module

namespace Nextsim {
void Logged::log(const std::string& message, Logged::level) { std::cerr << message << std::endl; }
}
