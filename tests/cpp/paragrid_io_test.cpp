// Nextsim::GB300::ParaGridIO (include/nsdg_paragrid_io.hpp) from C++17, no
// GPU: dumpModelState then getModelState returns the restart fields bit for
// bit and skips the others; readForcingTimeStatic picks the record at or
// before the requested time and skips absent fields; a CG field (no
// dimension key in the reference) and a missing file throw the reference's
// exception types.  Prints "ok" on success.
#include "nsdg_paragrid_io.hpp"

#include <cstdio>
#include <string>

using namespace Nextsim::GB300;

#define CHECK(c)                                                          \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::fprintf(stderr, "failed at line %d: %s\n", __LINE__, #c); \
            return 1;                                                     \
        }                                                                 \
    } while (0)

int main(int argc, char** argv)
{
    const std::string dir = argc > 1 ? argv[1] : ".";
    RestartMetadata m;
    m.nx = 7;
    m.ny = 3;
    const size_t n = m.nx * m.ny;
    ModelState s;
    s["hice"] = Field { NSDG_MA_DG, std::vector<double>(n * 6) };
    s["mask"] = Field { NSDG_MA_H, std::vector<double>(n, 1.0) };
    s["uwind"] = Field { NSDG_MA_H, std::vector<double>(n, 5.0) }; // not a restart field
    for (size_t i = 0; i < n * 6; ++i)
        s["hice"].data[i] = 0.25 + 1e-3 * static_cast<double>(i);
    ParaGridIO::dumpModelState(s, m, dir + "/restart.nc");
    const ModelState back = ParaGridIO::getModelState(dir + "/restart.nc");
    CHECK(back.size() == 2 && back.count("uwind") == 0);
    CHECK(back.at("hice").type == NSDG_MA_DG && back.at("hice").data == s["hice"].data);
    CHECK(back.at("mask").type == NSDG_MA_H && back.at("mask").data == s["mask"].data);

    // a diagnostic file with three records as forcing input
    nsdg_restart_writer* w = nullptr;
    CHECK(nsdg_diagnostic_writer_create(m.nx, m.ny, 1, 6, 8, 2, "parametric_rectangular", 0,
              "1970-01-01T00:00:00Z", &w) == NSDG_OK);
    std::vector<double> wind(n);
    for (int rec = 0; rec < 3; ++rec) {
        for (size_t i = 0; i < n; ++i)
            wind[i] = 10.0 * rec + static_cast<double>(i);
        const char* names[1] = { "uwind" };
        const int types[1] = { NSDG_MA_H };
        const double* data[1] = { wind.data() };
        const size_t counts[1] = { n };
        CHECK(nsdg_diagnostic_writer_record(w, 3600.0 * rec, 1, names, types, data, counts) == NSDG_OK);
    }
    CHECK(nsdg_restart_writer_save(w, (dir + "/forcing.nc").c_str()) == NSDG_OK);
    nsdg_restart_writer_destroy(w);
    const ModelState f = ParaGridIO::readForcingTimeStatic({ "uwind", "vwind" }, 5400.0, dir + "/forcing.nc");
    CHECK(f.size() == 1 && f.at("uwind").data[3] == 13.0);
    CHECK(ParaGridIO::readForcingTimeStatic({ "uwind" }, -1.0, dir + "/forcing.nc").at("uwind").data[0] == 0.0);

    s["grid_azimuth"] = Field { NSDG_MA_CG, std::vector<double>((2 * m.nx + 1) * (2 * m.ny + 1)) };
    ParaGridIO::dumpModelState(s, m, dir + "/restart_cg.nc");
    bool threw = false;
    try {
        ParaGridIO::getModelState(dir + "/restart_cg.nc");
    } catch (const std::out_of_range&) {
        threw = true;
    }
    CHECK(threw);
    threw = false;
    try {
        ParaGridIO::getModelState(dir + "/a44f5cc1f7934a8ae8dd03a95308745d.nc");
    } catch (const std::runtime_error&) {
        threw = true;
    }
    CHECK(threw);
    std::printf("ok\n");
    return 0;
}
