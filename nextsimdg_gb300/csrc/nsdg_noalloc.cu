// nsdg_noalloc.cu — Tools::MeanValue for callers that cannot allocate device memory.
//
// The regular entry points keep their reduction scratch (the per-block
// partial sums) in memory the handle allocated with cudaMalloc.  Some callers
// cannot allocate: a host model that hands the whole GPU memory to its own
// pool allocator at start-up (a cudaMalloc from a library would then fail, or
// fragment the pool behind the allocator's back), and code in a time-critical
// loop that may not pay cudaMalloc's implicit device-wide synchronisation.
// For them, nsdg_mean_value_noalloc takes device pointers to the field and the
// quadrature weights and writes the integral to a device pointer; its scratch
// is the file-scope array below, reserved once per process on every GPU that
// loads the library, of NSDG_NOALLOC_MAX_ELEMENTS / 256 doubles (512 KiB).
//
// Rules of the shared scratch: every call overwrites all the partial sums it
// reads (one per block of 256 elements), so nothing in it has to start at
// zero, and the last call's partial sums stay there afterwards.  All calls
// share the one array: two calls that overlap on the GPU (different streams
// or threads without ordering between them) race on it and give undefined
// results.  The first call on a device looks up the array's device address
// (cudaGetSymbolAddress) with that device current; make that first call before
// any stream capture that would record a later one.
#include "nsdg.h"

#include <cmath>
#include <cuda_runtime.h>
#include <mutex>

namespace {

static_assert(NSDG_NOALLOC_MAX_ELEMENTS % 256 == 0, "the maximum must be a multiple of the block size");
constexpr int kBlock = 256;
constexpr size_t kMaxPartials = NSDG_NOALLOC_MAX_ELEMENTS / kBlock;

// The scratch: one FP64 partial sum per block of 256 elements.
static __device__ __align__(256) double g_noallocPartials[kMaxPartials];

struct GaussPoints3 {
    double x[3];
};

// DG basis function j at (x, y) of the unit square (the Legendre-type modal
// basis of the reference: 1, x~, y~, x~^2-1/12, y~^2-1/12, x~y~, y~(x~^2-1/12),
// x~(y~^2-1/12), x~ = x - 1/2).
__device__ __forceinline__ double basis(int j, double x, double y)
{
    const double xs = x - 0.5, ys = y - 0.5;
    switch (j) {
    case 0: return 1.0;
    case 1: return xs;
    case 2: return ys;
    case 3: return xs * xs - 1.0 / 12.0;
    case 4: return ys * ys - 1.0 / 12.0;
    case 5: return xs * ys;
    case 6: return ys * (xs * xs - 1.0 / 12.0);
    default: return xs * (ys * ys - 1.0 / 12.0);
    }
}

// Per-block partial sums of sum_e sum_q phi_e(q) (J w)_e(q), written to the
// scratch (one value per block).
__global__ void __launch_bounds__(kBlock) kMeanValueNoAllocPartial(size_t N, int dg,
    const double* __restrict__ phi, const double* __restrict__ jw, GaussPoints3 gp, double* __restrict__ partials)
{
    __shared__ double ws[kBlock / 32];
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    double s = 0.0;
    if (e < N) {
        for (int q = 0; q < 9; ++q) {
            const double x = gp.x[q % 3], y = gp.x[q / 3];
            double v = 0.0;
            for (int j = 0; j < dg; ++j)
                v += phi[j * N + e] * basis(j, x, y);
            s += v * jw[q * N + e];
        }
    }
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < kBlock / 32 ? ws[threadIdx.x] : 0.0;
        for (int off = 16; off > 0; off >>= 1)
            t += __shfl_down_sync(0xffffffffu, t, off);
        if (threadIdx.x == 0)
            partials[blockIdx.x] = t;
    }
}

// Sum of the first n partials into *out (one block).
__global__ void __launch_bounds__(1024) kMeanValueNoAllocFinal(size_t n, const double* __restrict__ partials,
    double* __restrict__ out)
{
    __shared__ double ws[32];
    double s = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x)
        s += partials[i];
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = ws[threadIdx.x];
        for (int off = 16; off > 0; off >>= 1)
            t += __shfl_down_sync(0xffffffffu, t, off);
        if (threadIdx.x == 0)
            *out = t;
    }
}

// Device address of the scratch, looked up once per device.
constexpr int kMaxDevices = 64;
std::mutex g_setupMutex;
double* g_scratch[kMaxDevices] = {};

int scratchForCurrentDevice(double** out)
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return NSDG_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_setupMutex);
    if (!g_scratch[dev]) {
        double* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noallocPartials);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return NSDG_ERR_CUDA;
        }
        g_scratch[dev] = p;
    }
    *out = g_scratch[dev];
    return NSDG_OK;
}

} // namespace

extern "C" int nsdg_mean_value_noalloc(int dg, size_t n_elements, const double* phi, const double* jw,
    double* out, void* stream)
{
    if (dg != 1 && dg != 3 && dg != 6 && dg != 8)
        return NSDG_ERR_BAD_ARG;
    if (!phi || !jw || !out || n_elements == 0)
        return NSDG_ERR_BAD_ARG;
    if (n_elements > NSDG_NOALLOC_MAX_ELEMENTS)
        return NSDG_ERR_SIZE_MISMATCH; // larger than the static scratch holds
    double* partials = nullptr;
    const int st = scratchForCurrentDevice(&partials);
    if (st != NSDG_OK)
        return st;
    GaussPoints3 gp;
    const double a = std::sqrt(3. / 20.);
    gp.x[0] = 0.5 - a;
    gp.x[1] = 0.5;
    gp.x[2] = 0.5 + a;
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const unsigned blocks = static_cast<unsigned>((n_elements + kBlock - 1) / kBlock);
    kMeanValueNoAllocPartial<<<blocks, kBlock, 0, s>>>(n_elements, dg, phi, jw, gp, partials);
    kMeanValueNoAllocFinal<<<1, 1024, 0, s>>>(blocks, partials, out);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSDG_OK : NSDG_ERR_CUDA;
}
