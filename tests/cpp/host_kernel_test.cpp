// Drives the C++17 host class (include/nsdg_dynamics_kernel.hpp) the way the
// reference's MEVPDynamics module drives MEVPDynamicsKernel: initialise, the
// setData calls, update, getDG0Data; then the same steps through moduleStep
// (one call per step), which must give the same results.  Inputs are raw FP64
// files written by the pytest that runs this program; outputs are written
// next to them.
#include "nsdg_dynamics_kernel.hpp"

#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

static std::vector<double> readRaw(const std::string& path, size_t n)
{
    std::vector<double> v(n);
    std::ifstream f(path, std::ios::binary);
    f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * sizeof(double)));
    if (!f)
        throw std::runtime_error("cannot read " + path);
    return v;
}

int main(int argc, char** argv)
{
    if (argc < 4) {
        std::cerr << "usage: host_kernel_test <dir> <n> <steps>\n";
        return 2;
    }
    const std::string dir = argv[1];
    const size_t n = std::stoul(argv[2]);
    const int steps = std::stoi(argv[3]);
    const size_t N = n * n, nn = (n + 1) * (n + 1);
    using namespace Nextsim::GB300;
    nsdg_params p = defaultParameters();
    p.alpha = 300.0;
    p.beta = 300.0;
    GPUDynamicsKernel<6> kernel(Rheology::MEVP, p);
    const auto coords = readRaw(dir + "/coords.bin", 2 * nn);
    const auto mask = readRaw(dir + "/mask.bin", N);
    kernel.initialise(n, n, { coords.data(), nn, 2 }, false, { mask.data(), N, 1 });
    for (const char* name : { "hice", "cice", "u", "v", "uocean", "vocean", "ssh" }) {
        const auto f = readRaw(dir + "/" + name + ".bin", N);
        kernel.setData(name, { f.data(), N, 1 });
    }
    for (int s = 0; s < steps; ++s) {
        const auto uw = readRaw(dir + "/uwind_" + std::to_string(s) + ".bin", N);
        const auto vw = readRaw(dir + "/vwind_" + std::to_string(s) + ".bin", N);
        kernel.setData("uwind", { uw.data(), N, 1 });
        kernel.setData("vwind", { vw.data(), N, 1 });
        kernel.update({ s * 120.0, 120.0 });
    }
    for (const char* name : { "hice", "cice", "u", "v", "uiostress", "viostress" }) {
        const auto out = kernel.getDG0Data(name);
        std::ofstream f(dir + "/out_" + name + ".bin", std::ios::binary);
        f.write(reinterpret_cast<const char*>(out.data()), static_cast<std::streamsize>(out.size() * sizeof(double)));
    }
    try {
        kernel.getDG0Data("not_a_field");
        std::cerr << "missing std::out_of_range\n";
        return 1;
    } catch (const std::out_of_range&) {
    }
    // the same steps as one moduleStep call each (the winds as inputs, the
    // read-outs of the last step as outputs): the same results
    GPUDynamicsKernel<6> batched(Rheology::MEVP, p);
    batched.initialise(n, n, { coords.data(), nn, 2 }, false, { mask.data(), N, 1 });
    for (const char* name : { "hice", "cice", "u", "v", "uocean", "vocean", "ssh" }) {
        const auto f = readRaw(dir + "/" + name + ".bin", N);
        batched.setData(name, { f.data(), N, 1 });
    }
    const char* outNames[] = { "hice", "cice", "u", "v", "uiostress", "viostress" };
    std::vector<std::vector<double>> outs(6, std::vector<double>(N));
    for (int s = 0; s < steps; ++s) {
        const auto uw = readRaw(dir + "/uwind_" + std::to_string(s) + ".bin", N);
        const auto vw = readRaw(dir + "/vwind_" + std::to_string(s) + ".bin", N);
        std::vector<std::pair<std::string, double*>> o;
        for (int i = 0; i < 6; ++i)
            o.push_back({ outNames[i], outs[i].data() });
        batched.moduleStep({ { "uwind", { uw.data(), N, 1 } }, { "vwind", { vw.data(), N, 1 } } },
            { s * 120.0, 120.0 }, o);
    }
    for (int i = 0; i < 6; ++i)
        if (outs[i] != kernel.getDG0Data(outNames[i])) {
            std::cerr << "moduleStep differs from the separate calls for " << outNames[i] << "\n";
            return 1;
        }
    try {
        double dummy = 0.0;
        batched.moduleStep({}, { 0.0, 120.0 }, { { "not_a_field", &dummy } });
        std::cerr << "missing std::out_of_range from moduleStep\n";
        return 1;
    } catch (const std::out_of_range&) {
    }
    std::cout << "ok" << std::endl;
    return 0;
}
