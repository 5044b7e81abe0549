// nsdg_paragrid_io.hpp — C++17 host wrapper of the restart-file entry points
// (nsdg_restart_*, nsdg_diagnostic_writer_* in nsdg.h), shaped like the
// reference's ParaGridIO (core/src/include/ParaGridIO.hpp):
//   getModelState(path)                     ParaGridIO::getModelState (ParaGridIO.cpp:87-208)
//   readForcingTimeStatic(fields, t, path)  ParaGridIO::readForcingTimeStatic (:210-270)
//   dumpModelState(state, meta, path)       ParaGridIO::dumpModelState (:272-348)
// (diagnostic files, ParaGridIO::writeDiagnosticTime, go through
// nsdg_diagnostic_writer_* directly)
// A state maps field names to a ModelArray type (NSDG_MA_*) and its values
// in ModelArray order.  Errors throw the exception types the reference's
// netCDF path ends in: std::out_of_range for a missing field or an unknown
// dimension key, std::runtime_error for files that cannot be read or
// written.  Host code only; header-only.
#pragma once

#include "nsdg.h"

#include <algorithm>
#include <cstdint>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

namespace Nextsim::GB300 {

struct Field {
    int type = NSDG_MA_H;
    std::vector<double> data;
};
using ModelState = std::map<std::string, Field>;

// what CommonRestartMetadata writes for the grid and the time
struct RestartMetadata {
    size_t nx = 0, ny = 0, nz = 1;
    int dgComp = 6, dgStressComp = 8, cgDegree = 2;
    std::string structure = "parametric_rectangular";
    long long timeSeconds = 0;
    std::string timeFormatted = "1970-01-01T00:00:00Z";
};

class ParaGridIO {
public:
    static ModelState getModelState(const std::string& path)
    {
        File f(path);
        ModelState state;
        for (size_t i = 0, n = f.count("data"); i < n; ++i) {
            const auto v = f.info("data", i);
            if (v.type == NSDG_MA_NONE)
                throw std::out_of_range("No ModelArray::Type corresponds to the dimensions of " + v.name);
            state[v.name] = Field { v.type, f.read("data/" + v.name, 0, v.values) };
        }
        return state;
    }

    static ModelState readForcingTimeStatic(
        const std::set<std::string>& fields, double timeSeconds, const std::string& path)
    {
        File f(path);
        const auto tv = f.info("data", f.index("data", "time"));
        const auto times = f.read("data/time", 0, tv.values);
        size_t rec = std::find_if(times.begin(), times.end(), [&](double t) { return t > timeSeconds; })
            - times.begin();
        if (rec > 0)
            --rec;
        ModelState state;
        for (const auto& name : fields) {
            const size_t i = f.index("data", name);
            if (i == SIZE_MAX)
                continue; // absent forcings are skipped, as in the reference
            const auto v = f.info("data", i);
            state[name] = Field { NSDG_MA_H, f.read("data/" + name, rec, v.values) };
        }
        return state;
    }

    static void dumpModelState(const ModelState& state, const RestartMetadata& m, const std::string& path)
    {
        static const std::set<std::string> restartFields = { "hice", "cice", "hsnow", "tice", "sst", "sss",
            "mask", "coords", "x", "y", "longitude", "latitude", "grid_azimuth", "u", "v", "damage" };
        nsdg_restart_writer* w = nullptr;
        check(nsdg_restart_writer_create(m.nx, m.ny, m.nz, m.dgComp, m.dgStressComp, m.cgDegree,
                  m.structure.c_str(), m.timeSeconds, m.timeFormatted.c_str(), &w),
            "create " + path);
        try {
            for (const auto& [name, field] : state)
                if (restartFields.count(name))
                    check(nsdg_restart_writer_add(w, name.c_str(), field.type, field.data.data(), field.data.size()),
                        "field " + name);
            check(nsdg_restart_writer_save(w, path.c_str()), "write " + path);
        } catch (...) {
            nsdg_restart_writer_destroy(w);
            throw;
        }
        nsdg_restart_writer_destroy(w);
    }

private:
    static void check(int st, const std::string& what)
    {
        if (st == NSDG_ERR_UNKNOWN_FIELD)
            throw std::out_of_range(what);
        if (st != NSDG_OK)
            throw std::runtime_error(what + ": " + nsdg_status_string(st));
    }

    struct VarInfo {
        std::string name;
        int type;
        size_t records, values;
    };

    class File {
    public:
        explicit File(const std::string& path)
        {
            if (nsdg_restart_open(path.c_str(), &r_) != NSDG_OK)
                throw std::runtime_error(path + ": " + nsdg_restart_last_error(nullptr));
        }
        ~File() { nsdg_restart_close(r_); }
        File(const File&) = delete;
        File& operator=(const File&) = delete;
        size_t count(const char* group)
        {
            size_t n = 0;
            check(nsdg_restart_num_vars(r_, group, &n), group);
            return n;
        }
        VarInfo info(const char* group, size_t i)
        {
            char name[1024];
            VarInfo v {};
            size_t nc = 0;
            check(nsdg_restart_var_info(r_, group, i, name, sizeof name, &v.type, &nc, &v.records, &v.values), group);
            v.name = name;
            return v;
        }
        size_t index(const char* group, const std::string& name)
        {
            for (size_t i = 0, n = count(group); i < n; ++i)
                if (info(group, i).name == name)
                    return i;
            return SIZE_MAX;
        }
        std::vector<double> read(const std::string& path, size_t record, size_t n)
        {
            std::vector<double> v(n);
            check(nsdg_restart_read(r_, path.c_str(), record, v.data(), n), path);
            return v;
        }

    private:
        nsdg_restart* r_ = nullptr;
    };
};

} // namespace Nextsim::GB300
