// nsdg_forcing.cu — the benchmark forcing on the device (sm_103a).
//
// In the reference the atmosphere and ocean boundary modules update their
// fields right before the dynamics (PrognosticData.cpp:87-95), and the
// dynamics module copies them into its kernel with setData.  For the
// benchmark case both are closed-form fields on the cell centres of the
// box (BenchmarkCoordinates.cpp:21-40: x = i dx, y = j dy):
//   ocean  (BenchmarkOcean.cpp:15-39): u = vmax (2 fy - 1), v = vmax (1 - 2 fx),
//          fx = x / (nx dx), fy = y / (ny dy);
//   wind   (BenchmarkAtmosphere.cpp:29-77): a cyclone centred at (x0, y0),
//          x' = x - x0, y' = y - y0, scale = A exp(-k hypot(x', y')),
//          u = -scale vmax (cos a x' + sin a y'), v = -scale vmax (-sin a x' + cos a y').
// These kernels write them straight into device memory, so that a model step
// needs no host copy of its forcing.  The file is compiled without
// contraction (--fmad=false) so that each product and sum rounds as in the
// CPU formula.
#include "nsdg_kernels.hpp"

namespace nsdg {

namespace {

__global__ void kBenchmarkWind(size_t nx, size_t n, BenchmarkWindArgs a, double* __restrict__ uw,
    double* __restrict__ vw)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= n)
        return;
    const size_t i = e % nx, j = e / nx;
    const double xp = double(i) * a.dx - a.x0;
    const double yp = double(j) * a.dy - a.y0;
    const double scale = a.A * exp(-a.k * hypot(xp, yp));
    uw[e] = -scale * a.vmax * (a.cosa * xp + a.sina * yp);
    vw[e] = -scale * a.vmax * (-a.sina * xp + a.cosa * yp);
}

__global__ void kBenchmarkOcean(size_t nx, size_t ny, double dx, double dy, double vmax, double* __restrict__ uo,
    double* __restrict__ vo)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= nx * ny)
        return;
    const size_t i = e % nx, j = e / nx;
    const double fx = (double(i) * dx) / (double(nx) * dx);
    const double fy = (double(j) * dy) / (double(ny) * dy);
    uo[e] = vmax * (2.0 * fy - 1.0);
    vo[e] = vmax * (1.0 - 2.0 * fx);
}

} // namespace

cudaError_t launchBenchmarkWind(cudaStream_t s, size_t nx, size_t ny, const BenchmarkWindArgs& a, double* uw,
    double* vw)
{
    const size_t n = nx * ny;
    kBenchmarkWind<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(nx, n, a, uw, vw);
    return cudaGetLastError();
}

cudaError_t launchBenchmarkOcean(cudaStream_t s, size_t nx, size_t ny, double dx, double dy, double vmax,
    double* uo, double* vo)
{
    const size_t n = nx * ny;
    kBenchmarkOcean<<<static_cast<unsigned>((n + 255) / 256), 256, 0, s>>>(nx, ny, dx, dy, vmax, uo, vo);
    return cudaGetLastError();
}

} // namespace nsdg
