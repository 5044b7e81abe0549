// nsdg_common.cuh — device-side constants and helpers shared by the kernels.
//
// Layout conventions on the device (HBM):
//   DG field with C components ........ double[C][N]   (component-major SoA)
//   per-element operator with K entries  double[K][N]   (entry-major SoA)
//   CG2 node field ...................... double[(2nx+1)(2ny+1)], row-major
//   X-edge / Y-edge normal velocity ..... double[ED][nx(ny+1)] / double[ED][(nx+1)ny]
// so thread e of a warp reading entry k of element e touches base + k*N + e:
// 32 consecutive doubles per warp, one 256-byte transaction.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "nsdg_host.hpp"

namespace nsdg {

// Basis tables: defined in nsdg_kernels.cu (the only translation unit with
// device code), filled once per device by uploadConstTables().

// table access by compute type: cT (FP64) or cT32 (FP32), both defined in
// nsdg_kernels.cu
template <typename T> struct tab;
template <> struct tab<double> {
    static __device__ __forceinline__ double psi(int Q, int j, int q) { return cT.psi[Q][j][q]; }
    static __device__ __forceinline__ double psie(int G, int j, int g) { return cT.psie[G][j][g]; }
    static __device__ __forceinline__ double psiew(int G, int E, int g, int j) { return cT.psiew[G][E][g][j]; }
};
template <> struct tab<float> {
    static __device__ __forceinline__ float psi(int Q, int j, int q) { return cT32.psi[Q][j][q]; }
    static __device__ __forceinline__ float psie(int G, int j, int g) { return cT32.psie[G][j][g]; }
    static __device__ __forceinline__ float psiew(int G, int E, int g, int j) { return cT32.psiew[G][E][g][j]; }
};

template <int DG> struct DGTraits;
template <> struct DGTraits<1> { static constexpr int Q = 1, ED = 1; };
template <> struct DGTraits<3> { static constexpr int Q = 2, ED = 2; };
template <> struct DGTraits<6> { static constexpr int Q = 3, ED = 3; };
template <> struct DGTraits<8> { static constexpr int Q = 3, ED = 3; };

// Traces of a cell's DG expansion on its four edges, in the 1d edge basis
// {1, t-1/2, (t-1/2)^2-1/12} (DGTransport.cpp:31-142).  c[j] is component j.
template <int DG, typename T = double> __device__ __forceinline__ void traceLeft(const T* c, T* o)
{
    if constexpr (DG == 1) { o[0] = c[0]; }
    else if constexpr (DG == 3) { o[0] = c[0] - T(0.5) * c[1]; o[1] = c[2]; }
    else if constexpr (DG == 6) { o[0] = c[0] - T(0.5) * c[1] + T(1. / 6.) * c[3]; o[1] = c[2] - T(0.5) * c[5]; o[2] = c[4]; }
    else { o[0] = c[0] - T(0.5) * c[1] + T(1. / 6.) * c[3]; o[1] = c[2] - T(0.5) * c[5] + T(1. / 6.) * c[6]; o[2] = c[4] - T(0.5) * c[7]; }
}
template <int DG, typename T = double> __device__ __forceinline__ void traceRight(const T* c, T* o)
{
    if constexpr (DG == 1) { o[0] = c[0]; }
    else if constexpr (DG == 3) { o[0] = c[0] + T(0.5) * c[1]; o[1] = c[2]; }
    else if constexpr (DG == 6) { o[0] = c[0] + T(0.5) * c[1] + T(1. / 6.) * c[3]; o[1] = c[2] + T(0.5) * c[5]; o[2] = c[4]; }
    else { o[0] = c[0] + T(0.5) * c[1] + T(1. / 6.) * c[3]; o[1] = c[2] + T(0.5) * c[5] + T(1. / 6.) * c[6]; o[2] = c[4] + T(0.5) * c[7]; }
}
template <int DG, typename T = double> __device__ __forceinline__ void traceBottom(const T* c, T* o)
{
    if constexpr (DG == 1) { o[0] = c[0]; }
    else if constexpr (DG == 3) { o[0] = c[0] - T(0.5) * c[2]; o[1] = c[1]; }
    else if constexpr (DG == 6) { o[0] = c[0] - T(0.5) * c[2] + T(1. / 6.) * c[4]; o[1] = c[1] - T(0.5) * c[5]; o[2] = c[3]; }
    else { o[0] = c[0] - T(0.5) * c[2] + T(1. / 6.) * c[4]; o[1] = c[1] - T(0.5) * c[5] + T(1. / 6.) * c[7]; o[2] = c[3] - T(0.5) * c[6]; }
}
template <int DG, typename T = double> __device__ __forceinline__ void traceTop(const T* c, T* o)
{
    if constexpr (DG == 1) { o[0] = c[0]; }
    else if constexpr (DG == 3) { o[0] = c[0] + T(0.5) * c[2]; o[1] = c[1]; }
    else if constexpr (DG == 6) { o[0] = c[0] + T(0.5) * c[2] + T(1. / 6.) * c[4]; o[1] = c[1] + T(0.5) * c[5]; o[2] = c[3]; }
    else { o[0] = c[0] + T(0.5) * c[2] + T(1. / 6.) * c[4]; o[1] = c[1] + T(0.5) * c[5] + T(1. / 6.) * c[7]; o[2] = c[3] + T(0.5) * c[6]; }
}
// trace coefficients -> values at the ED edge Gauss points
template <int ED, typename T = double> __device__ __forceinline__ void edgeGauss(const T* t, T* g)
{
#pragma unroll
    for (int q = 0; q < ED; ++q) {
        T s = T(0);
#pragma unroll
        for (int j = 0; j < ED; ++j)
            s += t[j] * tab<T>::psie(ED, j, q);
        g[q] = s;
    }
}

} // namespace nsdg
