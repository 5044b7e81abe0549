/*
 * nsdg_dynamics_kernel.hpp — C++17 host class over the C ABI (nsdg.h).
 *
 * GPUDynamicsKernel has the public interface of the reference's dynamics
 * kernels (dynamics/src/include/DynamicsKernel.hpp:37-229 and its
 * CGDynamicsKernel / MEVPDynamicsKernel / BBMDynamicsKernel subclasses):
 *
 *   initialise(coords, isSpherical, mask)   DynamicsKernel.hpp:44-75
 *   setData(name, data)                     DynamicsKernel.hpp:93-110, CGDynamicsKernel.cpp:54-90
 *   getDG0Data(name)                        DynamicsKernel.hpp:119-130, CGDynamicsKernel.cpp:93-118
 *   getDGData(name)                         DynamicsKernel.hpp:138-156
 *   update(tst)                             VPCGDynamicsKernel.hpp:63-94, BrittleCGDynamicsKernel.hpp:91-136
 *
 * so a module such as MEVPDynamics (core/src/modules/DynamicsModule/MEVPDynamics.cpp)
 * can hold it in place of MEVPDynamicsKernel<DGCOMP>.  Fields cross the
 * boundary as FieldView (pointer + element count + component count, the
 * memory layout of the reference's ModelArray: element-major, component
 * fastest).  Errors are thrown as the reference's exception types:
 * std::out_of_range for unknown field names (the reference's .at()),
 * std::logic_error for unsupported requests, std::runtime_error otherwise.
 *
 * Header-only; link against libnsdg_gb300.so.
 */
#ifndef NSDG_DYNAMICS_KERNEL_HPP
#define NSDG_DYNAMICS_KERNEL_HPP

#include "nsdg.h"

#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace Nextsim {
namespace GB300 {

    //! A read-only view of ModelArray-shaped data.
    struct FieldView {
        const double* data = nullptr;
        size_t nElements = 0;
        size_t nComponents = 1;
    };

    //! core/src/include/Time.hpp:265-268, in seconds.
    struct TimestepTime {
        double start = 0.0;
        double step = 0.0;
    };

    enum class Rheology { MEVP = NSDG_RHEOLOGY_MEVP, BBM = NSDG_RHEOLOGY_BBM };

    inline nsdg_params defaultParameters()
    {
        nsdg_params p;
        nsdg_default_params(&p);
        return p;
    }

    template <int DGadvection> class GPUDynamicsKernel {
        static_assert(DGadvection == 1 || DGadvection == 3 || DGadvection == 6,
            "DGadvection must be 1, 3 or 6 (DGCOMP)");

    public:
        explicit GPUDynamicsKernel(Rheology r = Rheology::MEVP,
            const nsdg_params& params = defaultParameters())
        {
            check(nsdg_kernel_create(static_cast<int>(r), DGadvection, &params, &handle), "create");
        }
        ~GPUDynamicsKernel()
        {
            if (handle)
                nsdg_kernel_destroy(handle);
        }
        GPUDynamicsKernel(const GPUDynamicsKernel&) = delete;
        GPUDynamicsKernel& operator=(const GPUDynamicsKernel&) = delete;

        //! coords: (nx+1)*(ny+1) vertices with 2 components; mask: nx*ny, 1.0 = ice.
        void initialise(size_t nx, size_t ny, const FieldView& coords, bool isSpherical,
            const FieldView& mask)
        {
            if (coords.nElements != (nx + 1) * (ny + 1) || coords.nComponents != 2
                || mask.nElements != nx * ny)
                throw std::invalid_argument("initialise: coordinate or mask size does not match nx, ny");
            check(nsdg_kernel_initialise(handle, nx, ny, coords.data, isSpherical ? 1 : 0, mask.data),
                "initialise");
            nElements = nx * ny;
        }

        void setData(const std::string& name, const FieldView& data)
        {
            check(nsdg_kernel_set_data(handle, name.c_str(), data.data, data.nElements, data.nComponents),
                "setData");
        }

        //! Component 0 (the cell average) of the named field, one value per element.
        std::vector<double> getDG0Data(const std::string& name) const
        {
            std::vector<double> out(nElements);
            check(nsdg_kernel_get_dg0(handle, name.c_str(), out.data(), nElements), "getDG0Data");
            return out;
        }

        //! All DGadvection components of the named field, element-major.
        std::vector<double> getDGData(const std::string& name, size_t nComponents = DGadvection) const
        {
            std::vector<double> out(nElements * nComponents);
            check(nsdg_kernel_get_dg(handle, name.c_str(), out.data(), nElements, nComponents), "getDGData");
            return out;
        }

        void update(const TimestepTime& tst) { check(nsdg_kernel_update(handle, tst.start, tst.step), "update"); }

        //! One module step in one call (nsdg_kernel_module_step): setData of
        //! every input in order, update, then the cell averages of every
        //! output into its buffer (nelements() doubles each).
        void moduleStep(const std::vector<std::pair<std::string, FieldView>>& inputs, const TimestepTime& tst,
            const std::vector<std::pair<std::string, double*>>& outputs)
        {
            std::vector<nsdg_field_in> in;
            in.reserve(inputs.size());
            for (const auto& f : inputs) {
                if (f.second.nElements != nElements)
                    throw std::invalid_argument("moduleStep: size mismatch for " + f.first);
                in.push_back({ f.first.c_str(), f.second.data, f.second.nComponents });
            }
            std::vector<nsdg_field_out> out;
            out.reserve(outputs.size());
            for (const auto& f : outputs)
                out.push_back({ f.first.c_str(), f.second });
            check(nsdg_kernel_module_step(handle, in.data(), in.size(), tst.start, tst.step, out.data(), out.size()),
                "moduleStep");
        }

        //! Waits for the device and reports numeric faults of the last steps.
        void synchronize() { check(nsdg_kernel_synchronize(handle), "synchronize"); }

        std::vector<unsigned char> snapshot() const
        {
            size_t n = 0;
            check(nsdg_kernel_snapshot_size(handle, &n), "snapshot");
            std::vector<unsigned char> buf(n);
            check(nsdg_kernel_snapshot_save(handle, buf.data(), n), "snapshot");
            return buf;
        }
        void restore(const std::vector<unsigned char>& buf)
        {
            check(nsdg_kernel_snapshot_load(handle, buf.data(), buf.size()), "restore");
        }

        size_t nelements() const { return nElements; }

    private:
        nsdg_kernel* handle = nullptr;
        size_t nElements = 0;

        void check(int status, const char* what) const
        {
            if (status == NSDG_OK)
                return;
            const std::string msg = std::string(what) + ": "
                + (handle ? nsdg_kernel_last_error(handle) : nsdg_status_string(status));
            switch (status) {
            case NSDG_ERR_UNKNOWN_FIELD: throw std::out_of_range(msg);
            case NSDG_ERR_UNSUPPORTED:
            case NSDG_ERR_LOGIC: throw std::logic_error(msg);
            case NSDG_ERR_BAD_ARG:
            case NSDG_ERR_SIZE_MISMATCH: throw std::invalid_argument(msg);
            default: throw std::runtime_error(msg);
            }
        }
    };

} // namespace GB300
} // namespace Nextsim

#endif /* NSDG_DYNAMICS_KERNEL_HPP */
