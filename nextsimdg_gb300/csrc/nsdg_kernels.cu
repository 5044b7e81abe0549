// nsdg_kernels.cu — sm_103a kernels of the sea-ice dynamics hot path.
//
// One thread per element (element kernels) or per CG2 node (node kernels);
// every accumulation into a node or an element is a gather in a fixed order,
// so results are bitwise reproducible from run to run (no atomics on data).
#include <algorithm>
#include <cmath>
#include <cstddef>

#include "nsdg_host.hpp"

namespace nsdg {
__constant__ ConstTables cT;
__constant__ ConstTables32 cT32;
}

#include "nsdg_common.cuh"
#include "nsdg_kernels.hpp"
#include "nsdg_visc_ff.hpp"
#include "nsdg_tma.cuh"

namespace nsdg {

cudaError_t uploadConstTables()
{
    static ConstTables host;
    static ConstTables32 host32;
    static bool filled = false;
    if (!filled) {
        fillConstTables(host);
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 8; ++b)
                for (int c = 0; c < 16; ++c)
                    host32.psi[a][b][c] = static_cast<float>(host.psi[a][b][c]);
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 3; ++b)
                for (int c = 0; c < 3; ++c)
                    host32.psie[a][b][c] = static_cast<float>(host.psie[a][b][c]);
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b)
                for (int c = 0; c < 3; ++c)
                    for (int d = 0; d < 8; ++d)
                        host32.psiew[a][b][c][d] = static_cast<float>(host.psiew[a][b][c][d]);
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 9; ++b)
                for (int c = 0; c < 16; ++c)
                    host32.phi2[a][b][c] = static_cast<float>(host.phi2[a][b][c]);
        filled = true;
    }
    const cudaError_t e = cudaMemcpyToSymbol(cT, &host, sizeof(ConstTables));
    return e != cudaSuccess ? e : cudaMemcpyToSymbol(cT32, &host32, sizeof(ConstTables32));
}

namespace {

constexpr int kBlock = 128;
inline unsigned blocksFor(size_t n, int b = kBlock) { return static_cast<unsigned>((n + b - 1) / b); }

// ===========================================================================
// CG2 -> DG projection   (Interpolations.cpp:74-122, Cartesian)
//   val(q) = sum_j PHI_j(q) cg_j ; t(q) = (J w)(q) val(q) ;
//   r_i = sum_q PSI_i(q) t(q) ;  dg = M^{-1} r
// ===========================================================================
template <int DG, int NF>
__global__ void __launch_bounds__(kBlock) kCG2DG(int nx, size_t N, const double* __restrict__ jw,
    const double* __restrict__ minv, const double* __restrict__ cg0, const double* __restrict__ cg1,
    double* __restrict__ out0, double* __restrict__ out1)
{
    constexpr int Q = DGTraits<DG>::Q, QQ = Q * Q;
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= N)
        return;
    const size_t s2 = 2 * size_t(nx) + 1;
    const size_t ix = static_cast<unsigned>(e) % static_cast<unsigned>(nx), iy = static_cast<unsigned>(e) / static_cast<unsigned>(nx);
    const size_t base = 2 * s2 * iy + 2 * ix;
    const double* cg[2] = { cg0, cg1 };
    double* out[2] = { out0, out1 };
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        double loc[9];
#pragma unroll
        for (int j = 0; j < 9; ++j)
            loc[j] = cg[f][base + (j % 3) + (j / 3) * s2];
        double t[QQ];
#pragma unroll
        for (int q = 0; q < QQ; ++q) {
            double v = 0.0;
#pragma unroll
            for (int j = 0; j < 9; ++j)
                v += cT.phi2[Q][j][q] * loc[j];
            t[q] = jw[q * N + e] * v;
        }
        double r[DG];
#pragma unroll
        for (int i = 0; i < DG; ++i) {
            double a = 0.0;
#pragma unroll
            for (int q = 0; q < QQ; ++q)
                a += cT.psi[Q][i][q] * t[q];
            r[i] = a;
        }
#pragma unroll
        for (int i = 0; i < DG; ++i) {
            double a = 0.0;
#pragma unroll
            for (int k = 0; k < DG; ++k)
                a += minv[(i * DG + k) * N + e] * r[k];
            out[f][i * N + e] = a;
        }
    }
}

// The same projection for the mixed-precision transport velocity: the CG2
// values at the Gauss points and the weighted moments against the DG basis in
// FP32 (jw32: FP32 copy of J w), the inverse mass matrix applied in FP64 (on a
// parallelogram mesh, DIAG: its diagonal, minv = [DG][N]).
template <int DG, int NF, bool DIAG>
__global__ void __launch_bounds__(kBlock) kCG2DG32(int nx, size_t N, const float* __restrict__ jw32,
    const double* __restrict__ minv, const double* __restrict__ cg0, const double* __restrict__ cg1,
    double* __restrict__ out0, double* __restrict__ out1)
{
    constexpr int Q = DGTraits<DG>::Q, QQ = Q * Q;
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= N)
        return;
    const size_t s2 = 2 * size_t(nx) + 1;
    const size_t ix = static_cast<unsigned>(e) % static_cast<unsigned>(nx);
    const size_t iy = static_cast<unsigned>(e) / static_cast<unsigned>(nx);
    const size_t base = 2 * s2 * iy + 2 * ix;
    const double* cg[2] = { cg0, cg1 };
    double* out[2] = { out0, out1 };
    float w[QQ];
#pragma unroll
    for (int q = 0; q < QQ; ++q)
        w[q] = jw32[q * N + e];
#pragma unroll
    for (int f = 0; f < NF; ++f) {
        float loc[9];
#pragma unroll
        for (int j = 0; j < 9; ++j)
            loc[j] = static_cast<float>(cg[f][base + (j % 3) + (j / 3) * s2]);
        float t[QQ];
#pragma unroll
        for (int q = 0; q < QQ; ++q) {
            float v = 0.f;
#pragma unroll
            for (int j = 0; j < 9; ++j)
                v = fmaf(cT32.phi2[Q][j][q], loc[j], v);
            t[q] = w[q] * v;
        }
        double r[DG];
#pragma unroll
        for (int i = 0; i < DG; ++i) {
            float a = 0.f;
#pragma unroll
            for (int q = 0; q < QQ; ++q)
                a = fmaf(cT32.psi[Q][i][q], t[q], a);
            r[i] = static_cast<double>(a);
        }
#pragma unroll
        for (int i = 0; i < DG; ++i) {
            if constexpr (DIAG) {
                out[f][i * N + e] = minv[i * N + e] * r[i];
            } else {
                double a = 0.0;
#pragma unroll
                for (int k = 0; k < DG; ++k)
                    a += minv[(i * DG + k) * N + e] * r[k];
                out[f][i * N + e] = a;
            }
        }
    }
}

// ===========================================================================
// Edge normal velocities  (DGTransport.cpp:158-252)
// X-edge (ix,iy), iy in [0,ny]: first the cell below contributes through its
// top trace, then the cell above through its bottom trace; Y-edge (ix,iy):
// left cell (right trace) then right cell (left trace).  Land cells are
// skipped; Dirichlet edges are doubled.
// ===========================================================================
// Longitude difference of an edge vector on a spherical mesh, with the jump
// at +-Pi removed (ParametricMesh.hpp:381-397).
__device__ __forceinline__ double wrapLon(const DevMesh& m, double d)
{
    if (m.spherical) {
        if (d > 0.5 * M_PI)
            d -= 2.0 * M_PI;
        if (d < -0.5 * M_PI)
            d += 2.0 * M_PI;
    }
    return d;
}

template <int DG>
__global__ void __launch_bounds__(kBlock) kNormalVelocity(DevMesh m, const double* __restrict__ velx,
    const double* __restrict__ vely, double* __restrict__ nvX, double* __restrict__ nvY)
{
    constexpr int ED = DGTraits<DG>::ED;
    const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    const size_t N = m.N;
    const int nx = m.nx, ny = m.ny;
    const size_t sv = size_t(nx) + 1;
    if (t < m.nXe) {
        const size_t ix = static_cast<unsigned>(t) % static_cast<unsigned>(nx), iy = static_cast<unsigned>(t) / static_cast<unsigned>(nx);
        const size_t n0 = iy * sv + ix;
        const double t0 = wrapLon(m, m.vx[n0 + 1] - m.vx[n0]), t1 = m.vy[n0 + 1] - m.vy[n0];
        double acc[ED];
#pragma unroll
        for (int k = 0; k < ED; ++k)
            acc[k] = 0.0;
        double cx[DG], cy[DG], tx[ED], ty[ED];
        if (iy >= 1) {
            const size_t c = (iy - 1) * nx + ix;
            if (m.ice[c]) {
#pragma unroll
                for (int j = 0; j < DG; ++j) {
                    cx[j] = velx[j * N + c];
                    cy[j] = vely[j * N + c];
                }
                traceTop<DG>(cx, tx);
                traceTop<DG>(cy, ty);
#pragma unroll
                for (int k = 0; k < ED; ++k)
                    acc[k] += 0.5 * (-t1 * tx[k] + t0 * ty[k]);
            }
        }
        if (iy < size_t(ny)) {
            const size_t c = iy * nx + ix;
            if (m.ice[c]) {
#pragma unroll
                for (int j = 0; j < DG; ++j) {
                    cx[j] = velx[j * N + c];
                    cy[j] = vely[j * N + c];
                }
                traceBottom<DG>(cx, tx);
                traceBottom<DG>(cy, ty);
#pragma unroll
                for (int k = 0; k < ED; ++k)
                    acc[k] += 0.5 * (-t1 * tx[k] + t0 * ty[k]);
            }
        }
        for (int r = 0; r < m.edgeXCount[t]; ++r)
#pragma unroll
            for (int k = 0; k < ED; ++k)
                acc[k] *= 2.0;
#pragma unroll
        for (int k = 0; k < ED; ++k)
            nvX[k * m.nXe + t] = acc[k];
        return;
    }
    const size_t u = t - m.nXe;
    if (u >= m.nYe)
        return;
    const size_t ix = u % sv, iy = u / sv;
    const size_t n0 = iy * sv + ix;
    const double t0 = wrapLon(m, m.vx[n0 + sv] - m.vx[n0]), t1 = m.vy[n0 + sv] - m.vy[n0];
    double acc[ED];
#pragma unroll
    for (int k = 0; k < ED; ++k)
        acc[k] = 0.0;
    double cx[DG], cy[DG], tx[ED], ty[ED];
    if (ix >= 1) {
        const size_t c = iy * nx + ix - 1;
        if (m.ice[c]) {
#pragma unroll
            for (int j = 0; j < DG; ++j) {
                cx[j] = velx[j * N + c];
                cy[j] = vely[j * N + c];
            }
            traceRight<DG>(cx, tx);
            traceRight<DG>(cy, ty);
#pragma unroll
            for (int k = 0; k < ED; ++k)
                acc[k] += 0.5 * (t1 * tx[k] - t0 * ty[k]);
        }
    }
    if (ix < size_t(nx)) {
        const size_t c = iy * nx + ix;
        if (m.ice[c]) {
#pragma unroll
            for (int j = 0; j < DG; ++j) {
                cx[j] = velx[j * N + c];
                cy[j] = vely[j * N + c];
            }
            traceLeft<DG>(cx, tx);
            traceLeft<DG>(cy, ty);
#pragma unroll
            for (int k = 0; k < ED; ++k)
                acc[k] += 0.5 * (t1 * tx[k] - t0 * ty[k]);
        }
    }
    for (int r = 0; r < m.edgeYCount[u]; ++r)
#pragma unroll
        for (int k = 0; k < ED; ++k)
            acc[k] *= 2.0;
#pragma unroll
    for (int k = 0; k < ED; ++k)
        nvY[k * m.nYe + u] = acc[k];
}

// ===========================================================================
// float <-> double on the integer pipe (GB300 issues FP64 instructions, the
// conversions among them, at about 1/60 of its FP32 rate).  Round to nearest
// (ties away from zero); magnitudes below the smallest normal float become a
// signed zero; infinities and NaNs are kept.
// ===========================================================================
__device__ __forceinline__ float narrowAny(double d)
{
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
    const unsigned long long mag = b & 0x7fffffffffffffffull;
    const unsigned sign = static_cast<unsigned>(b >> 32) & 0x80000000u;
    if (mag < (897ull << 52))
        return __uint_as_float(sign);
    if (mag >= 0x47effffff0000000ull) // beyond the largest float (or inf / NaN)
        return __uint_as_float(sign | (mag > 0x7ff0000000000000ull ? 0x7fc00000u : 0x7f800000u));
    return __uint_as_float(sign | static_cast<unsigned>((mag - (896ull << 52) + (1ull << 28)) >> 29));
}
__device__ __forceinline__ double widenAny(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned mag = u & 0x7fffffffu;
    const unsigned long long sign = static_cast<unsigned long long>(u & 0x80000000u) << 32;
    if (mag < 0x00800000u)
        return __longlong_as_double(static_cast<long long>(sign));
    if (mag >= 0x7f800000u)
        return __longlong_as_double(static_cast<long long>(
            sign | 0x7ff0000000000000ull | (mag > 0x7f800000u ? 0x8000000000000ull : 0ull)));
    return __longlong_as_double(static_cast<long long>(sign | ((static_cast<unsigned long long>(mag) << 29)
        + (896ull << 52))));
}
// ===========================================================================
// Cell averages of the CG2 -> DG projection of two fields (what getDG0Data
// returns): the quadrature of kCG2DG (FP64) or kCG2DG32 (F32: FP32
// quadrature, conversions on the integer pipe) and only row 0 of M^{-1}.  In
// FP64 the arithmetic is kCG2DG's for component 0, operation for operation.
// ===========================================================================
template <int DG, bool F32>
__global__ void __launch_bounds__(kBlock) kCG2DG0(int nx, size_t N, const double* __restrict__ jw,
    const float* __restrict__ jw32, const double* __restrict__ minv, const double* __restrict__ cg0,
    const double* __restrict__ cg1, double* __restrict__ out0, double* __restrict__ out1)
{
    constexpr int Q = DGTraits<DG>::Q, QQ = Q * Q;
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= N)
        return;
    const size_t s2 = 2 * size_t(nx) + 1;
    const size_t ix = static_cast<unsigned>(e) % static_cast<unsigned>(nx);
    const size_t iy = static_cast<unsigned>(e) / static_cast<unsigned>(nx);
    const size_t base = 2 * s2 * iy + 2 * ix;
    const double* cg[2] = { cg0, cg1 };
    double* out[2] = { out0, out1 };
#pragma unroll
    for (int f = 0; f < 2; ++f) {
        double r[DG];
        if constexpr (F32) {
            float loc[9];
#pragma unroll
            for (int j = 0; j < 9; ++j)
                loc[j] = narrowAny(cg[f][base + (j % 3) + (j / 3) * s2]);
            float t[QQ];
#pragma unroll
            for (int q = 0; q < QQ; ++q) {
                float v = 0.f;
#pragma unroll
                for (int j = 0; j < 9; ++j)
                    v = fmaf(cT32.phi2[Q][j][q], loc[j], v);
                t[q] = jw32[q * N + e] * v;
            }
#pragma unroll
            for (int i = 0; i < DG; ++i) {
                float a = 0.f;
#pragma unroll
                for (int q = 0; q < QQ; ++q)
                    a = fmaf(cT32.psi[Q][i][q], t[q], a);
                r[i] = widenAny(a);
            }
        } else {
            double loc[9];
#pragma unroll
            for (int j = 0; j < 9; ++j)
                loc[j] = cg[f][base + (j % 3) + (j / 3) * s2];
            double t[QQ];
#pragma unroll
            for (int q = 0; q < QQ; ++q) {
                double v = 0.0;
#pragma unroll
                for (int j = 0; j < 9; ++j)
                    v += cT.phi2[Q][j][q] * loc[j];
                t[q] = jw[q * N + e] * v;
            }
#pragma unroll
            for (int i = 0; i < DG; ++i) {
                double a = 0.0;
#pragma unroll
                for (int q = 0; q < QQ; ++q)
                    a += cT.psi[Q][i][q] * t[q];
                r[i] = a;
            }
        }
        double a = 0.0;
#pragma unroll
        for (int k = 0; k < DG; ++k)
            a += minv[k * N + e] * r[k];
        out[f][e] = a;
    }
}

// The ice-ocean stress at the CG2 nodes in FP32 for the mixed path's
// read-out (its velocities are FP32 iterates), kIceOceanStress's formulas
__global__ void __launch_bounds__(kBlock) kIceOceanStress32(size_t n, int brittle, const double* __restrict__ u,
    const double* __restrict__ v, const double* __restrict__ uo, const double* __restrict__ vo,
    float Fo, float ca, float sa, double* __restrict__ tx, double* __restrict__ ty)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const float ui = narrowAny(u[i]), vi = narrowAny(v[i]), uoi = narrowAny(uo[i]), voi = narrowAny(vo[i]);
    if (!brittle) {
        const float ur = ui - uoi, vr = vi - voi;
        const float a = sqrtf(ur * ur + vr * vr);
        tx[i] = widenAny(Fo * a * ur);
        ty[i] = widenAny(Fo * a * vr);
    } else {
        const float ur = uoi - ui, vr = voi - vi;
        const float cp = Fo * hypotf(ur, vr);
        tx[i] = widenAny(cp * (ur * ca - vr * sa));
        ty[i] = widenAny(cp * (vr * ca + ur * sa));
    }
}

template <class T> __device__ __forceinline__ T toT(double x) { return x; }
template <> __device__ __forceinline__ float toT<float>(double x) { return narrowAny(x); }
template <class T> __device__ __forceinline__ double fromT(T x) { return x; }
template <> __device__ __forceinline__ double fromT<float>(float x) { return widenAny(x); }

// ===========================================================================
// DG transport operator + Runge-Kutta stage  (DGTransport.cpp:278-566)
// ===========================================================================
template <int DG> struct Cell {
    double c[DG];
};

// upwind flux at the ED edge Gauss points between trace 1 (cell 1: bottom /
// left) and trace 2 (cell 2: top / right)
template <int DG, typename T = double>
__device__ __forceinline__ void upwind(const T* nv, const T* t1, const T* t2, T* tmp)
{
    constexpr int ED = DGTraits<DG>::ED;
    T vg[ED], g1[ED], g2[ED];
    edgeGauss<ED, T>(nv, vg);
    edgeGauss<ED, T>(t1, g1);
    edgeGauss<ED, T>(t2, g2);
#pragma unroll
    for (int g = 0; g < ED; ++g)
        tmp[g] = fmax(vg[g], T(0)) * g1[g] + fmin(vg[g], T(0)) * g2[g];
}
// acc += sdt * sum_g tmp(g) PSIe_w<DG,ED,E>(g, :)
template <int DG, typename T = double>
__device__ __forceinline__ void addEdge(T* acc, T sdt, const T* tmp, int E)
{
    constexpr int ED = DGTraits<DG>::ED;
#pragma unroll
    for (int j = 0; j < DG; ++j) {
        T s = T(0);
#pragma unroll
        for (int g = 0; g < ED; ++g)
            s += tmp[g] * tab<T>::psiew(ED, E, g, j);
        acc[j] += sdt * s;
    }
}

template <int DG>
__device__ __forceinline__ void loadCell(const double* __restrict__ p, size_t N, size_t c, double* out)
{
#pragma unroll
    for (int j = 0; j < DG; ++j)
        out[j] = p[j * N + c];
}

// The DG6 limiters evaluate the Gauss-point values in T (FP32 for the mixed
// transport: the coefficients narrowed on the integer pipe); the limited
// coefficients and the scaling stay FP64.
template <int DG, class T = double> __device__ __forceinline__ void limitMax(double* r, double mx)
{
    if constexpr (DG == 1) {
        r[0] = fmin(r[0], mx);
    } else if constexpr (DG == 3) {
        r[0] = fmin(mx, r[0]);
        const double l0 = 2.0 * fmax(fabs(r[1] + r[2]), fabs(r[1] - r[2]));
        if (l0 != 0.0 && r[0] + l0 - mx > 0) {
            r[1] *= (mx - r[0]) / l0;
            r[2] *= (mx - r[0]) / l0;
        }
    } else if constexpr (DG == 6) {
        r[0] = fmin(mx, r[0]);
        T rt[6];
#pragma unroll
        for (int j = 0; j < 6; ++j)
            rt[j] = toT<T>(r[j]);
        T mv = T(-INFINITY);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            T s = T(0);
#pragma unroll
            for (int j = 0; j < 6; ++j)
                s += rt[j] * tab<T>::psi(3, j, q);
            mv = fmax(mv, s);
        }
        if (fromT<T>(mv) > mx) {
            const double f = (mx - r[0]) / (fromT<T>(mv) - r[0]);
#pragma unroll
            for (int j = 1; j < 6; ++j)
                r[j] *= f;
        }
    }
}
template <int DG, class T = double> __device__ __forceinline__ void limitMin(double* r, double mn)
{
    if constexpr (DG == 1) {
        r[0] = fmax(r[0], mn);
    } else if constexpr (DG == 3) {
        r[0] = fmax(mn, r[0]);
        const double l0 = 2.0 * fmax(fabs(r[1] + r[2]), fabs(r[1] - r[2]));
        if (l0 != 0.0 && r[0] - l0 - mn < 0) {
            r[1] *= (r[0] - mn) / l0;
            r[2] *= (r[0] - mn) / l0;
        }
    } else if constexpr (DG == 6) {
        r[0] = fmax(mn, r[0]);
        T rt[6];
#pragma unroll
        for (int j = 0; j < 6; ++j)
            rt[j] = toT<T>(r[j]);
        T mv = T(INFINITY);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            T s = T(0);
#pragma unroll
            for (int j = 0; j < 6; ++j)
                s += rt[j] * tab<T>::psi(3, j, q);
            mv = fmin(mv, s);
        }
        if (fromT<T>(mv) < mn) {
            const double f = (r[0] - mn) / (fromT<T>(mv) - r[0]);
#pragma unroll
            for (int j = 1; j < 6; ++j)
                r[j] *= f;
        }
    }
}

struct TransportArgs {
    DevMesh m;
    const double* cellX;
    const double* cellY;
    const double* minv;
    const double* velx;
    const double* vely;
    const double* nvX;
    const double* nvY;
    double dt;
    int mode;
    const float* cellX32; // FP32 copies of cellX / cellY (T = float)
    const float* cellY32;
};

// Dirichlet (closed) boundaries of cell c: outflow only (DGTransport.cpp:306-351)
template <int DG, int NF, typename T>
__device__ __forceinline__ void dirichletOutflow(const DevMesh& m, const double* __restrict__ nvX,
    const double* __restrict__ nvY, size_t c, int ix, int iy, const T (*ownT)[DG], T (*acc)[DG], T dt)
{
    constexpr int ED = DGTraits<DG>::ED;
    const int seg = m.cellSeg[c];
    if (!seg)
        return;
    const int nx = m.nx;
    T nv[ED], t1[ED], tmp[ED];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
        if (!(seg & (1 << s)))
            continue;
        const double* nvp = (s == 0 || s == 2) ? nvX : nvY;
        const size_t ne = (s == 0 || s == 2) ? m.nXe : m.nYe;
        const size_t e = s == 0 ? size_t(iy) * nx + ix
            : s == 1          ? size_t(iy) * (nx + 1) + ix + 1
            : s == 2          ? size_t(iy + 1) * nx + ix
                              : size_t(iy) * (nx + 1) + ix;
#pragma unroll
        for (int k = 0; k < ED; ++k)
            nv[k] = toT<T>(nvp[k * ne + e]);
        T vg[ED];
        edgeGauss<ED, T>(nv, vg);
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            if (s == 0) traceBottom<DG, T>(ownT[k], t1);
            else if (s == 1) traceRight<DG, T>(ownT[k], t1);
            else if (s == 2) traceTop<DG, T>(ownT[k], t1);
            else traceLeft<DG, T>(ownT[k], t1);
            T tg[ED];
            edgeGauss<ED, T>(t1, tg);
#pragma unroll
            for (int g = 0; g < ED; ++g)
                tmp[g] = tg[g] * ((s == 0 || s == 3) ? fmax(-vg[g], T(0)) : fmax(vg[g], T(0)));
            addEdge<DG, T>(acc[k], -dt, tmp, s);
        }
    }
}

// The Runge-Kutta combination (FP64) of field k of cell c from its
// M^{-1}-scaled right-hand side r, the limiters, the store
// (DGTransport.cpp:498-566)
template <int DG, typename T>
__device__ __forceinline__ void finishStage(int mode, const StageFields& f, int k, size_t N, size_t c,
    const double* own, const double* r)
{
    double out[DG];
    switch (mode) {
    case STAGE_RK1:
#pragma unroll
        for (int i = 0; i < DG; ++i)
            out[i] = own[i] + r[i];
        break;
    case STAGE_RK2_A:
#pragma unroll
        for (int i = 0; i < DG; ++i) {
            f.k1[k][i * N + c] = r[i];
            out[i] = f.phi[k][i * N + c] + r[i];
        }
        break;
    case STAGE_RK2_B:
#pragma unroll
        for (int i = 0; i < DG; ++i)
            out[i] = own[i] + 0.5 * (r[i] - f.k1[k][i * N + c]);
        break;
    case STAGE_RK3_A:
#pragma unroll
        for (int i = 0; i < DG; ++i)
            out[i] = r[i] + f.phi[k][i * N + c];
        break;
    case STAGE_RK3_B:
#pragma unroll
        for (int i = 0; i < DG; ++i)
            out[i] = (r[i] + own[i]) * 0.25 + 0.75 * f.phi[k][i * N + c];
        break;
    default: // STAGE_RK3_C
#pragma unroll
        for (int i = 0; i < DG; ++i)
            out[i] = f.phi[k][i * N + c] * (1.0 / 3.0) + 2.0 / 3.0 * (r[i] + own[i]);
        break;
    }
    if (f.lmax[k])
        limitMax<DG, T>(out, f.vmax[k]);
    if (f.lmin[k])
        limitMin<DG, T>(out, f.vmin[k]);
#pragma unroll
    for (int i = 0; i < DG; ++i)
        f.dst[k][i * N + c] = out[i];
}

// One Runge-Kutta stage of DGTransport for NF fields.  T is the type of the
// flux arithmetic (cell term, edge traces, upwind fluxes, the accumulated
// right-hand side): double reproduces the reference's arithmetic; float is
// the mixed-precision transport, whose fields, inverse mass matrices and
// Runge-Kutta combination stay FP64.
template <int DG, int NF, typename T>
__global__ void __launch_bounds__(kBlock) kTransportStage(TransportArgs a, StageFields f)
{
    constexpr int Q = DGTraits<DG>::Q, QQ = Q * Q, ED = DGTraits<DG>::ED;
    const size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    const DevMesh& m = a.m;
    const size_t N = m.N;
    if (c >= N)
        return;
    const int nx = m.nx, ny = m.ny;
    const int ix = static_cast<int>(static_cast<unsigned>(c) % static_cast<unsigned>(nx)), iy = static_cast<int>(static_cast<unsigned>(c) / static_cast<unsigned>(nx));
    const T dt = static_cast<T>(a.dt);
    const bool ice = m.ice[c] != 0;
    const T* cellX;
    const T* cellY;
    if constexpr (sizeof(T) == 4) {
        cellX = a.cellX32;
        cellY = a.cellY32;
    } else {
        cellX = a.cellX;
        cellY = a.cellY;
    }

    double own[NF][DG];
    T ownT[NF][DG], acc[NF][DG];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        loadCell<DG>(f.src[k], N, c, own[k]);
#pragma unroll
        for (int j = 0; j < DG; ++j) {
            ownT[k][j] = toT<T>(own[k][j]);
            acc[k][j] = T(0);
        }
    }

    // cell term: dt * sum_q (cellX_iq vx(q) + cellY_iq vy(q)) phi(q)
    if constexpr (DG > 1) {
        if (ice) {
            T vxg[QQ], vyg[QQ], pg[NF][QQ];
            T vx[DG], vy[DG];
#pragma unroll
            for (int j = 0; j < DG; ++j) {
                vx[j] = toT<T>(a.velx[j * N + c]);
                vy[j] = toT<T>(a.vely[j * N + c]);
            }
#pragma unroll
            for (int q = 0; q < QQ; ++q) {
                T sx = T(0), sy = T(0);
#pragma unroll
                for (int j = 0; j < DG; ++j) {
                    sx += vx[j] * tab<T>::psi(Q, j, q);
                    sy += vy[j] * tab<T>::psi(Q, j, q);
                }
                vxg[q] = sx;
                vyg[q] = sy;
#pragma unroll
                for (int k = 0; k < NF; ++k) {
                    T sp = T(0);
#pragma unroll
                    for (int j = 0; j < DG; ++j)
                        sp += ownT[k][j] * tab<T>::psi(Q, j, q);
                    pg[k][q] = sp;
                }
            }
#pragma unroll
            for (int i = 0; i < DG; ++i) {
                T t[NF];
#pragma unroll
                for (int k = 0; k < NF; ++k)
                    t[k] = T(0);
#pragma unroll
                for (int q = 0; q < QQ; ++q) {
                    const T mq = cellX[(i * QQ + q) * N + c] * vxg[q] + cellY[(i * QQ + q) * N + c] * vyg[q];
#pragma unroll
                    for (int k = 0; k < NF; ++k)
                        t[k] += mq * pg[k][q];
                }
#pragma unroll
                for (int k = 0; k < NF; ++k)
                    acc[k][i] += dt * t[k];
            }
        }
    }

    T nv[ED], t1[ED], t2[ED], tmp[ED], nb[DG];
    auto loadNb = [&](const double* src, size_t cc) {
#pragma unroll
        for (int j = 0; j < DG; ++j)
            nb[j] = toT<T>(src[j * N + cc]);
    };
    auto loadNv = [&](const double* nvp, size_t ne, size_t e) {
#pragma unroll
        for (int k = 0; k < ED; ++k)
            nv[k] = toT<T>(nvp[k * ne + e]);
    };
    // left Y-edge (this cell is "cell 2"), interior edges only
    if (ix >= 1) {
        const size_t c1 = c - 1;
        if (ice && m.ice[c1]) {
            loadNv(a.nvY, m.nYe, size_t(iy) * (nx + 1) + ix);
#pragma unroll
            for (int k = 0; k < NF; ++k) {
                loadNb(f.src[k], c1);
                traceRight<DG, T>(nb, t1);
                traceLeft<DG, T>(ownT[k], t2);
                upwind<DG, T>(nv, t1, t2, tmp);
                addEdge<DG, T>(acc[k], dt, tmp, 3);
            }
        }
    }
    // right Y-edge (this cell is "cell 1")
    if (ix + 1 <= nx - 1) {
        const size_t c2 = c + 1;
        if (ice && m.ice[c2]) {
            loadNv(a.nvY, m.nYe, size_t(iy) * (nx + 1) + ix + 1);
#pragma unroll
            for (int k = 0; k < NF; ++k) {
                loadNb(f.src[k], c2);
                traceRight<DG, T>(ownT[k], t1);
                traceLeft<DG, T>(nb, t2);
                upwind<DG, T>(nv, t1, t2, tmp);
                addEdge<DG, T>(acc[k], -dt, tmp, 1);
            }
        }
    }
    // bottom X-edge (this cell is "cell 2")
    if (iy >= 1) {
        const size_t c1 = c - nx;
        if (ice && m.ice[c1]) {
            loadNv(a.nvX, m.nXe, size_t(iy) * nx + ix);
#pragma unroll
            for (int k = 0; k < NF; ++k) {
                loadNb(f.src[k], c1);
                traceTop<DG, T>(nb, t1);
                traceBottom<DG, T>(ownT[k], t2);
                upwind<DG, T>(nv, t1, t2, tmp);
                addEdge<DG, T>(acc[k], dt, tmp, 0);
            }
        }
    }
    // top X-edge (this cell is "cell 1")
    if (iy + 1 <= ny - 1) {
        const size_t c2 = c + nx;
        if (ice && m.ice[c2]) {
            loadNv(a.nvX, m.nXe, size_t(iy + 1) * nx + ix);
#pragma unroll
            for (int k = 0; k < NF; ++k) {
                loadNb(f.src[k], c2);
                traceTop<DG, T>(ownT[k], t1);
                traceBottom<DG, T>(nb, t2);
                upwind<DG, T>(nv, t1, t2, tmp);
                addEdge<DG, T>(acc[k], -dt, tmp, 2);
            }
        }
    }
    // periodic edges touching this cell, in list order
    for (int p = m.perPtr[c]; p < m.perPtr[c + 1]; ++p) {
        const int type = m.perEntry[4 * p], p1 = m.perEntry[4 * p + 1], p2 = m.perEntry[4 * p + 2];
        const size_t e = static_cast<size_t>(m.perEntry[4 * p + 3]);
        if (!m.ice[p1] || !m.ice[p2])
            continue;
        loadNv(type == 0 ? a.nvX : a.nvY, type == 0 ? m.nXe : m.nYe, e);
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            T b1[DG], b2[DG];
#pragma unroll
            for (int j = 0; j < DG; ++j) {
                b1[j] = toT<T>(f.src[k][j * N + p1]);
                b2[j] = toT<T>(f.src[k][j * N + p2]);
            }
            if (type == 0) {
                traceTop<DG, T>(b1, t1);
                traceBottom<DG, T>(b2, t2);
            } else {
                traceRight<DG, T>(b1, t1);
                traceLeft<DG, T>(b2, t2);
            }
            upwind<DG, T>(nv, t1, t2, tmp);
            if (size_t(p1) == c)
                addEdge<DG, T>(acc[k], -dt, tmp, type == 0 ? 2 : 1);
            if (size_t(p2) == c)
                addEdge<DG, T>(acc[k], dt, tmp, type == 0 ? 0 : 3);
        }
    }
    dirichletOutflow<DG, NF, T>(m, a.nvX, a.nvY, c, ix, iy, ownT, acc, dt);
    // inverse mass (FP64) and the Runge-Kutta combination (FP64)
    double Mi[DG * DG];
#pragma unroll
    for (int i = 0; i < DG * DG; ++i)
        Mi[i] = a.minv[i * N + c];
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        double r[DG];
#pragma unroll
        for (int i = 0; i < DG; ++i) {
            double s = 0.0;
#pragma unroll
            for (int j = 0; j < DG; ++j)
                s += Mi[i * DG + j] * fromT<T>(acc[k][j]);
            r[i] = s;
        }
        finishStage<DG, T>(a.mode, f, k, N, c, own[k], r);
    }
}

// ---------------------------------------------------------------------------
// The same stage on a mesh of parallelograms, FP32 fluxes (mixed precision),
// by tiles of kTrX x kTrY elements.
//
// * The tile's coefficients and a one-cell halo (narrowed to FP32) and the
//   ice flags are staged in shared memory; each interior edge's upwind flux
//   at its Gauss points is evaluated once, by one thread, into shared memory,
//   and read by the two cells it separates (the per-element kernel evaluates
//   every interior edge twice, once from each side).  Edges on the tile's
//   border are evaluated by both tiles.
// * The cell term takes the element's four Jacobian coefficients c0..c3
//   instead of its 2 x DG x Q^2 operator entries:
//   sum_q (cellX_iq vx_q + cellY_iq vy_q) phi_q
//     = sum_q (U_xi,iq (c0 vx_q + c2 vy_q) + U_eta,iq (c1 vx_q + c3 vy_q)) phi_q
//   with the unit square's U in constant memory.
// * M^{-1} is diagonal (J M_ref with the Legendre basis): DG FP64 products
//   per field instead of DG^2.
// Each cell adds its terms in the per-element kernel's order (cell term,
// left, right, bottom, top edge, Dirichlet outflow).  Meshes with periodic
// edges keep the per-element kernel.
// ---------------------------------------------------------------------------
constexpr int kTrX = 32, kTrY = 8;

struct AffTransportTables {
    float u6[2][6][9]; // U_xi, U_eta [i][q] for DG 6 (3 x 3 Gauss points)
    float u3[2][3][4]; // for DG 3 (2 x 2 Gauss points)
};
__constant__ AffTransportTables cTrAff;

template <int DG> __device__ __forceinline__ float trU(int b, int i, int q)
{
    if constexpr (DG == 6)
        return cTrAff.u6[b][i][q];
    else
        return cTrAff.u3[b][i][q];
}

struct TransportAffArgs {
    DevMesh m;
    const float* coef; // [5][ld] c0 .. c4
    size_t ld;
    const double* minvDiag; // [DG][N]
    const double* velx;
    const double* vely;
    const double* nvX;
    const double* nvY;
    double dt;
    int mode;
};

template <int DG, int NF>
__global__ void __launch_bounds__(kTrX * kTrY, 4) kTransportStageAffine(TransportAffArgs a, StageFields f)
{
    constexpr int Q = DGTraits<DG>::Q, QQ = Q * Q, ED = DGTraits<DG>::ED;
    constexpr int SX = kTrX + 2, SY = kTrY + 2;
    __shared__ float sc[NF][DG][SY][SX];        // coefficients, tile + halo
    __shared__ uint8_t sIce[SY][SX];            // ice flags (0 outside the grid)
    __shared__ float fy[NF][ED][kTrY][kTrX + 1]; // upwind Gauss values of the Y-edges (x = x0 .. x0 + kTrX)
    __shared__ float fx[NF][ED][kTrY + 1][kTrX]; // of the X-edges (y = y0 .. y0 + kTrY)
    const DevMesh& m = a.m;
    const size_t N = m.N;
    const int nx = m.nx, ny = m.ny;
    const int lx = threadIdx.x, ly = threadIdx.y;
    const int x0 = blockIdx.x * kTrX, y0 = blockIdx.y * kTrY;
    const int ix = x0 + lx, iy = y0 + ly;
    const bool in = ix < nx && iy < ny;
    const size_t c = in ? size_t(iy) * nx + ix : 0;
    const float dt = static_cast<float>(a.dt);

    // the cell's own coefficients live in shared memory (FP32) and are
    // reloaded in FP64 for the Runge-Kutta combination: fewer registers,
    // more resident blocks
    bool ice = false;
    if (in) {
        ice = m.ice[c] != 0;
#pragma unroll
        for (int k = 0; k < NF; ++k)
#pragma unroll
            for (int j = 0; j < DG; ++j)
                sc[k][j][ly + 1][lx + 1] = toT<float>(f.src[k][j * N + c]);
    }
    sIce[ly + 1][lx + 1] = ice ? 1 : 0;
    // the halo: bottom and top rows, left and right columns (no corners)
    const int t = ly * kTrX + lx;
    if (t < 2 * (kTrX + kTrY)) {
        int hx, hy;
        if (t < kTrX) { hx = t + 1; hy = 0; }
        else if (t < 2 * kTrX) { hx = t - kTrX + 1; hy = SY - 1; }
        else if (t < 2 * kTrX + kTrY) { hx = 0; hy = t - 2 * kTrX + 1; }
        else { hx = SX - 1; hy = t - 2 * kTrX - kTrY + 1; }
        const int gx = x0 - 1 + hx, gy = y0 - 1 + hy;
        uint8_t hi = 0;
        if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) {
            const size_t cc = size_t(gy) * nx + gx;
            hi = m.ice[cc] != 0 ? 1 : 0;
            if (hi) {
#pragma unroll
                for (int k = 0; k < NF; ++k)
#pragma unroll
                    for (int j = 0; j < DG; ++j)
                        sc[k][j][hy][hx] = toT<float>(f.src[k][j * N + cc]);
            }
        }
        sIce[hy][hx] = hi;
    }
    __syncthreads();

    // upwind fluxes: Y-edge e of tile row r lies between smem cells (r+1, e)
    // (cell 1, left) and (r+1, e+1) (cell 2, right); X-edge r of tile column
    // e between (r, e+1) (cell 1, below) and (r+1, e+1) (cell 2, above).  An
    // edge carries a flux only if both cells are ice, which also excludes the
    // grid's outer boundary (cells outside the grid are flagged land).
    auto yEdge = [&](int r, int e) {
        if (!(sIce[r + 1][e] && sIce[r + 1][e + 1]))
            return;
        const size_t ei = size_t(y0 + r) * (nx + 1) + x0 + e;
        float nv[ED], t1[ED], t2[ED], tmp[ED], cb[DG];
#pragma unroll
        for (int g = 0; g < ED; ++g)
            nv[g] = toT<float>(a.nvY[g * m.nYe + ei]);
#pragma unroll
        for (int k = 0; k < NF; ++k) {
#pragma unroll
            for (int j = 0; j < DG; ++j)
                cb[j] = sc[k][j][r + 1][e];
            traceRight<DG, float>(cb, t1);
#pragma unroll
            for (int j = 0; j < DG; ++j)
                cb[j] = sc[k][j][r + 1][e + 1];
            traceLeft<DG, float>(cb, t2);
            upwind<DG, float>(nv, t1, t2, tmp);
#pragma unroll
            for (int g = 0; g < ED; ++g)
                fy[k][g][r][e] = tmp[g];
        }
    };
    auto xEdge = [&](int r, int e) {
        if (!(sIce[r][e + 1] && sIce[r + 1][e + 1]))
            return;
        const size_t ei = size_t(y0 + r) * nx + x0 + e;
        float nv[ED], t1[ED], t2[ED], tmp[ED], cb[DG];
#pragma unroll
        for (int g = 0; g < ED; ++g)
            nv[g] = toT<float>(a.nvX[g * m.nXe + ei]);
#pragma unroll
        for (int k = 0; k < NF; ++k) {
#pragma unroll
            for (int j = 0; j < DG; ++j)
                cb[j] = sc[k][j][r][e + 1];
            traceTop<DG, float>(cb, t1);
#pragma unroll
            for (int j = 0; j < DG; ++j)
                cb[j] = sc[k][j][r + 1][e + 1];
            traceBottom<DG, float>(cb, t2);
            upwind<DG, float>(nv, t1, t2, tmp);
#pragma unroll
            for (int g = 0; g < ED; ++g)
                fx[k][g][r][e] = tmp[g];
        }
    };
    yEdge(ly, lx); // the edge left of this thread's cell
    xEdge(ly, lx); // the edge below it
    if (t < kTrY)
        yEdge(t, kTrX); // the tile's right border
    else if (t < kTrY + kTrX)
        xEdge(kTrY, t - kTrY); // the tile's top border
    __syncthreads();
    if (!in)
        return;

    float acc[NF][DG];
#pragma unroll
    for (int k = 0; k < NF; ++k)
#pragma unroll
        for (int j = 0; j < DG; ++j)
            acc[k][j] = 0.f;

    if constexpr (DG > 1) {
        if (ice) {
            float vx[DG], vy[DG], ag[QQ], bg[QQ], pg[NF][QQ];
#pragma unroll
            for (int j = 0; j < DG; ++j) {
                vx[j] = toT<float>(a.velx[j * N + c]);
                vy[j] = toT<float>(a.vely[j * N + c]);
            }
            const float c0 = a.coef[c], c1 = a.coef[a.ld + c], c2 = a.coef[2 * a.ld + c],
                        c3 = a.coef[3 * a.ld + c];
#pragma unroll
            for (int q = 0; q < QQ; ++q) {
                float sx = 0.f, sy = 0.f;
#pragma unroll
                for (int j = 0; j < DG; ++j) {
                    sx += vx[j] * tab<float>::psi(Q, j, q);
                    sy += vy[j] * tab<float>::psi(Q, j, q);
                }
                ag[q] = c0 * sx + c2 * sy;
                bg[q] = c1 * sx + c3 * sy;
#pragma unroll
                for (int k = 0; k < NF; ++k) {
                    float sp = 0.f;
#pragma unroll
                    for (int j = 0; j < DG; ++j)
                        sp += sc[k][j][ly + 1][lx + 1] * tab<float>::psi(Q, j, q);
                    pg[k][q] = sp;
                }
            }
#pragma unroll
            for (int i = 0; i < DG; ++i) {
                float tt[NF];
#pragma unroll
                for (int k = 0; k < NF; ++k)
                    tt[k] = 0.f;
#pragma unroll
                for (int q = 0; q < QQ; ++q) {
                    const float mq = trU<DG>(0, i, q) * ag[q] + trU<DG>(1, i, q) * bg[q];
#pragma unroll
                    for (int k = 0; k < NF; ++k)
                        tt[k] += mq * pg[k][q];
                }
#pragma unroll
                for (int k = 0; k < NF; ++k)
                    acc[k][i] += dt * tt[k];
            }
        }
    }

    if (ice) {
        float tmp[ED];
        const bool left = sIce[ly + 1][lx], right = sIce[ly + 1][lx + 2];
        const bool below = sIce[ly][lx + 1], above = sIce[ly + 2][lx + 1];
#pragma unroll
        for (int k = 0; k < NF; ++k) {
            if (left) {
#pragma unroll
                for (int g = 0; g < ED; ++g)
                    tmp[g] = fy[k][g][ly][lx];
                addEdge<DG, float>(acc[k], dt, tmp, 3);
            }
            if (right) {
#pragma unroll
                for (int g = 0; g < ED; ++g)
                    tmp[g] = fy[k][g][ly][lx + 1];
                addEdge<DG, float>(acc[k], -dt, tmp, 1);
            }
            if (below) {
#pragma unroll
                for (int g = 0; g < ED; ++g)
                    tmp[g] = fx[k][g][ly][lx];
                addEdge<DG, float>(acc[k], dt, tmp, 0);
            }
            if (above) {
#pragma unroll
                for (int g = 0; g < ED; ++g)
                    tmp[g] = fx[k][g][ly + 1][lx];
                addEdge<DG, float>(acc[k], -dt, tmp, 2);
            }
        }
    }
    if (m.cellSeg[c]) {
        float ownT[NF][DG];
#pragma unroll
        for (int k = 0; k < NF; ++k)
#pragma unroll
            for (int j = 0; j < DG; ++j)
                ownT[k][j] = sc[k][j][ly + 1][lx + 1];
        dirichletOutflow<DG, NF, float>(m, a.nvX, a.nvY, c, ix, iy, ownT, acc, dt);
    }

    // diagonal inverse mass (FP64) and the Runge-Kutta combination (FP64)
#pragma unroll
    for (int k = 0; k < NF; ++k) {
        double r[DG], own[DG];
        loadCell<DG>(f.src[k], N, c, own);
#pragma unroll
        for (int i = 0; i < DG; ++i)
            r[i] = a.minvDiag[i * N + c] * fromT<float>(acc[k][i]);
        finishStage<DG, float>(a.mode, f, k, N, c, own, r);
    }
}

// ===========================================================================
// DG -> CG2 (Interpolations.cpp:144-204): per node, contributions of the (up
// to four) cells around it, odd cell rows first then even rows (the
// reference's reversed-parity stripes), cells in ascending x; then the
// boundary rows and columns are doubled.
// ===========================================================================
// The cells along one direction touching CG2 index i2 (0..2n) and the node's
// local index in each (0, 1, 2), ascending; kept in registers (no local
// arrays): n of them
struct NodeCand {
    int n, c0, l0, c1, l1;
};
__device__ __forceinline__ NodeCand nodeCand(int i2, int n)
{
    NodeCand r { 1, 0, 0, 0, 0 };
    if (i2 & 1) {
        r.c0 = (i2 - 1) / 2;
        r.l0 = 1;
    } else if (i2 >= 2 && i2 / 2 < n) {
        r.n = 2;
        r.c0 = i2 / 2 - 1;
        r.l0 = 2;
        r.c1 = i2 / 2;
        r.l1 = 0;
    } else if (i2 >= 2) {
        r.c0 = i2 / 2 - 1;
        r.l0 = 2;
    } else {
        r.c0 = i2 / 2;
        r.l0 = 0;
    }
    return r;
}

template <int DG, int NF>
__global__ void __launch_bounds__(kBlock) kDG2CG(DevMesh m, const double* __restrict__ in0,
    const double* __restrict__ in1, double* __restrict__ out0, double* __restrict__ out1)
{
    const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (t >= m.Ncg)
        return;
    const int s2 = 2 * m.nx + 1;
    const int i2 = static_cast<int>(static_cast<unsigned>(t) % static_cast<unsigned>(s2)), j2 = static_cast<int>(static_cast<unsigned>(t) / static_cast<unsigned>(s2));
    const NodeCand X = nodeCand(i2, m.nx);
    NodeCand Y = nodeCand(j2, m.ny);
    if (Y.n == 2 && !(Y.c0 & 1)) { // odd cell rows first
        const int c = Y.c0, l = Y.l0;
        Y.c0 = Y.c1;
        Y.l0 = Y.l1;
        Y.c1 = c;
        Y.l1 = l;
    }
    const double* in[2] = { in0, in1 };
    double acc[NF];
#pragma unroll
    for (int f = 0; f < NF; ++f)
        acc[f] = 0.0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        if (r >= Y.n)
            continue;
        const int cy = r ? Y.c1 : Y.c0, ly = r ? Y.l1 : Y.l0;
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            if (k >= X.n)
                continue;
            const int cx = k ? X.c1 : X.c0, lx = k ? X.l1 : X.l0;
            const size_t c = size_t(cy) * m.nx + cx;
            const int q = lx + 3 * ly;
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                double at = 0.0;
#pragma unroll
                for (int j = 0; j < DG; ++j)
                    at += in[f][j * m.N + c] * cT.psiLag3[j][q];
                if (q == 4)
                    acc[f] += at;
                else if (q == 1 || q == 3 || q == 5 || q == 7)
                    acc[f] += 0.5 * at;
                else
                    acc[f] += 0.25 * at;
            }
        }
    }
    double scale = 1.0;
    if (j2 == 0 || j2 == 2 * m.ny)
        scale *= 2.0;
    if (i2 == 0 || i2 == 2 * m.nx)
        scale *= 2.0;
    out0[t] = acc[0] * scale;
    if constexpr (NF > 1)
        out1[t] = acc[1] * scale;
}

// ===========================================================================
// Sea-surface-height gradient (CGDynamicsKernel.cpp:126-258)
// ===========================================================================
// CG1 Lagrange average of the DG0 ssh (reversed parity: odd rows first)
__global__ void __launch_bounds__(kBlock) kSSHToCG1(DevMesh m, const double* __restrict__ ssh, double* __restrict__ cg1)
{
    const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (t >= m.Ncg1)
        return;
    const unsigned s1 = static_cast<unsigned>(m.nx) + 1u;
    const int i1 = static_cast<int>(static_cast<unsigned>(t) % s1), j1 = static_cast<int>(static_cast<unsigned>(t) / s1);
    // the cell rows touching the node, odd rows first (registers, no local arrays)
    const bool below = j1 >= 1, above = j1 < m.ny;
    const int nr = int(below) + int(above);
    int row0 = below ? j1 - 1 : j1, row1 = j1;
    if (nr == 2 && (row0 % 2) == 0) {
        row0 = j1;
        row1 = j1 - 1;
    }
    double acc = 0.0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        if (r >= nr)
            continue;
        const int row = r ? row1 : row0;
        for (int cx = i1 - 1; cx <= i1; ++cx) {
            if (cx < 0 || cx >= m.nx)
                continue;
            acc += 0.25 * ssh[size_t(row) * m.nx + cx];
        }
    }
    double scale = 1.0;
    if (j1 == 0 || j1 == m.ny)
        scale *= 2.0;
    if (i1 == 0 || i1 == m.nx)
        scale *= 2.0;
    cg1[t] = acc * scale;
}
// CG1 gradient by element gather (even rows first), divided by the lumped mass
__global__ void __launch_bounds__(kBlock) kSSHGrad1(DevMesh m, DevOps o, const double* __restrict__ cg1,
    double* __restrict__ ug, double* __restrict__ vg)
{
    const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (t >= m.Ncg1)
        return;
    const unsigned s1 = static_cast<unsigned>(m.nx) + 1u;
    const int i1 = static_cast<int>(static_cast<unsigned>(t) % s1), j1 = static_cast<int>(static_cast<unsigned>(t) / s1);
    // the cell rows touching the node with the node's local row in each, even
    // rows first (registers, no local arrays)
    const bool below = j1 >= 1, above = j1 < m.ny;
    const int nr = int(below) + int(above);
    int row0 = below ? j1 - 1 : j1, ly0 = below ? 1 : 0, row1 = j1, ly1 = 0;
    if (nr == 2 && (row0 % 2) == 1) {
        row0 = j1;
        ly0 = 0;
        row1 = j1 - 1;
        ly1 = 1;
    }
    double au = 0.0, av = 0.0;
    const size_t N = m.N;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        if (r >= nr)
            continue;
        for (int lx = 1; lx >= 0; --lx) {
            const int cx = i1 - lx;
            if (cx < 0 || cx >= m.nx)
                continue;
            const int cy = r ? row1 : row0, ly = r ? ly1 : ly0;
            const size_t e = size_t(cy) * m.nx + cx;
            const size_t n0 = size_t(cy) * s1 + cx;
            const double loc[4] = { cg1[n0], cg1[n0 + 1], cg1[n0 + s1], cg1[n0 + s1 + 1] };
            const int k = lx + 2 * ly;
            double tx = 0.0, ty = 0.0;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                tx += o.dxssh[(k * 4 + j) * N + e] * loc[j];
                ty += o.dyssh[(k * 4 + j) * N + e] * loc[j];
            }
            au -= tx;
            av -= ty;
        }
    }
    ug[t] = au / o.lumped1[t];
    vg[t] = av / o.lumped1[t];
}
// boundary extension of the CG1 gradient (the value a boundary node copies
// from the neighbouring interior node) followed by CG1 -> CG2 interpolation
__device__ __forceinline__ size_t sshSource(int i1, int j1, int nx, int ny)
{
    int si = i1, sj = j1;
    if (i1 == 0) si = 1;
    if (i1 == nx) si = nx - 1;
    if (j1 == 0) sj = 1;
    if (j1 == ny) sj = ny - 1;
    return size_t(sj) * (nx + 1) + si;
}
__global__ void __launch_bounds__(kBlock) kSSHToCG2(DevMesh m, const double* __restrict__ ug,
    const double* __restrict__ vg, double* __restrict__ uGrad, double* __restrict__ vGrad)
{
    const size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (t >= m.Ncg)
        return;
    const int s2 = 2 * m.nx + 1;
    const int i2 = static_cast<int>(static_cast<unsigned>(t) % static_cast<unsigned>(s2)), j2 = static_cast<int>(static_cast<unsigned>(t) / static_cast<unsigned>(s2));
    const int nx = m.nx, ny = m.ny;
    const int ix = i2 / 2, iy = j2 / 2;
    double u, v;
    if (!(i2 & 1) && !(j2 & 1)) {
        const size_t a = sshSource(ix, iy, nx, ny);
        u = ug[a];
        v = vg[a];
    } else if ((i2 & 1) && !(j2 & 1)) {
        const size_t a = sshSource(ix, iy, nx, ny), b = sshSource(ix + 1, iy, nx, ny);
        u = 0.5 * (ug[a] + ug[b]);
        v = 0.5 * (vg[a] + vg[b]);
    } else if (!(i2 & 1) && (j2 & 1)) {
        const size_t a = sshSource(ix, iy, nx, ny), b = sshSource(ix, iy + 1, nx, ny);
        u = 0.5 * (ug[a] + ug[b]);
        v = 0.5 * (vg[a] + vg[b]);
    } else {
        const size_t a = sshSource(ix, iy, nx, ny), b = sshSource(ix + 1, iy, nx, ny);
        const size_t c = sshSource(ix, iy + 1, nx, ny), d = sshSource(ix + 1, iy + 1, nx, ny);
        u = 0.25 * (ug[a] + ug[b] + ug[c] + ug[d]);
        v = 0.25 * (vg[a] + vg[b] + vg[c] + vg[d]);
    }
    uGrad[t] = u;
    vGrad[t] = v;
}

// ===========================================================================
// mEVP
// ===========================================================================
__global__ void __launch_bounds__(kBlock) kMevpPrepNodes(size_t n, MevpNodeState st, MevpParams p)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    // clamps of prepareIteration (CGDynamicsKernel.cpp:273-275)
    const double A = fmax(fmin(st.cgA[i], 1.0), 1.e-4);
    const double H = fmax(st.cgH[i], 1.e-4);
    st.cgA[i] = A;
    st.cgH[i] = H;
    st.u0[i] = st.u[i];
    st.v0[i] = st.v[i];
    const double rhoH = p.rho_ice * H;
    const double c1 = rhoH / p.dt;
    st.c1[i] = c1;
    st.c1b[i] = c1 * (1.0 + p.beta);
    const double ua = st.ua[i], va = st.va[i];
    const double absatm = sqrt(ua * ua + va * va);
    st.fau[i] = p.F_atm * absatm * ua;
    st.fav[i] = p.F_atm * absatm * va;
    st.rhfc[i] = rhoH * p.fc;
    st.gu[i] = rhoH * p.gravity * st.uGrad[i];
    st.gv[i] = rhoH * p.gravity * st.vGrad[i];
}

template <int DG>
__global__ void __launch_bounds__(kBlock) kMevpPrepElements(size_t N, const double* __restrict__ h,
    const double* __restrict__ a, double* __restrict__ Pg, double Pstar, double invAlpha, float* __restrict__ hP32,
    const float* __restrict__ tdiv32, float* __restrict__ tdivLast)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= N)
        return;
    if (tdivLast) // the divergence at the start of this sub-cycle (warm-start features)
#pragma unroll
        for (int k = 0; k < 18; ++k)
            tdivLast[k * N + e] = tdiv32[k * N + e];
    double hc[DG], ac[DG];
    loadCell<DG>(h, N, e, hc);
    loadCell<DG>(a, N, e, ac);
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        double hs = 0.0, as = 0.0;
#pragma unroll
        for (int j = 0; j < DG; ++j) {
            hs += hc[j] * cT.psi[3][j][q];
            as += ac[j] * cT.psi[3][j][q];
        }
        const double hq = fmax(hs, 0.0);
        const double aq = fmin(fmax(as, 0.0), 1.0);
        const double pa = Pstar * hq * exp(-20.0 * (1.0 - aq)) * invAlpha;
        if (hP32) {
            Pg[q * N + e] = 0.125 * pa;
            hP32[q * N + e] = static_cast<float>(0.5 * pa);
        } else {
            Pg[q * N + e] = pa;
        }
    }
}

// One mEVP iteration, element part, carried in divergence space.
//
// The reference updates the stress coefficients s (8 per component,
// MEVPStressUpdateStep.hpp:80-116) and then forms the element's share of the
// stress divergence at its 9 CG2 nodes, divS1 s11 + divS2 s12 and
// divS1 s12 + divS2 s22 (CGDynamicsKernel.cpp:340-363).  In the mEVP solver s
// is observed only through that divergence, and the update is linear in s:
//   s' = (1 - 1/alpha) s + iMJwPSI f    =>   divS s' = (1 - 1/alpha) divS s + (divS iMJwPSI) f
// so each element keeps its 18 divergence coefficients tdiv instead of the 24
// stress coefficients and applies the 9 x 9 operators A = divS iMJwPSI,
// precomputed in FP64 on the host.  This drops the separate projection and
// divergence products (216 + 288 FMA) for 324 FMA on an FP64-issue-bound
// kernel.  The strain at the Gauss points comes straight from the 9 velocity
// nodes through G = psi^T iMgrad (9 x 9), so the strain coefficients are not
// formed either.  Land cells keep tdiv = 0 (the reference's divergence skips
// them).  Pg holds P/alpha at the 9 Gauss points.
//
// Thread layout: three threads per element (kStressParts), 64 elements per
// block.  Phase 1: thread `part` computes the strain, Delta and the stress
// increments at Gauss points 3*part .. 3*part+2 and leaves them in shared
// memory.  Phase 2: the same thread updates the divergence coefficients of
// nodes 3*part .. 3*part+2.  Same FP64 work as one thread per element, three
// times the warps to hide the operator loads.
constexpr int kStressElems = 64;
constexpr int kStressParts = 3;

// SPH: spherical metric terms (CGDynamicsKernel.cpp:331-334, 348-351): the
// strain gains e11 -= iMM v, e12 += iMM u / 2 (through the composite G_m),
// the divergence gains +divM s12 (x) and -divM s11 (y) (through A_3).
template <bool SPH>
__global__ void __launch_bounds__(kStressElems * kStressParts) kMevpStress(DevMesh m, DevOps o,
    const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ Pg,
    double* __restrict__ tdiv, MevpParams p)
{
    __shared__ double fs[3][9][kStressElems];
    const int le = threadIdx.x % kStressElems;
    const int part = threadIdx.x / kStressElems; // warp-uniform
    const size_t N = m.N;
    const size_t e = blockIdx.x * size_t(kStressElems) + le;
    const bool active = e < N && m.ice[e];
    if (active) {
        const size_t s2 = 2 * size_t(m.nx) + 1;
        const size_t ix = static_cast<unsigned>(e) % static_cast<unsigned>(m.nx), iy = static_cast<unsigned>(e) / static_cast<unsigned>(m.nx);
        const size_t base = 2 * s2 * iy + 2 * ix;
        double ul[9], vl[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const size_t nd = base + (j % 3) + (j / 3) * s2;
            ul[j] = u[nd];
            vl[j] = v[nd];
        }
        const double dmin2 = p.DeltaMin * p.DeltaMin;
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) {
            const int q = 3 * part + qq;
            double ex = 0.0, ey = 0.0, exv = 0.0, eyu = 0.0;
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const double gxq = o.gx[(q * 9 + j) * N + e];
                const double gyq = o.gy[(q * 9 + j) * N + e];
                ex = fma(gxq, ul[j], ex);
                ey = fma(gyq, vl[j], ey);
                exv = fma(gxq, vl[j], exv);
                eyu = fma(gyq, ul[j], eyu);
            }
            if constexpr (SPH) {
                double mu = 0.0, mv = 0.0;
#pragma unroll
                for (int j = 0; j < 9; ++j) {
                    const double gmq = o.gm[(q * 9 + j) * N + e];
                    mu = fma(gmq, ul[j], mu);
                    mv = fma(gmq, vl[j], mv);
                }
                ex -= mv;
                eyu += mu;
            }
            // e11 = ex, e22 = ey, e12 = (exv + eyu) / 2
            const double sxy = exv + eyu;
            const double d2 = dmin2 + 1.25 * (ex * ex + ey * ey) + 1.50 * ex * ey + 0.25 * sxy * sxy;
            const double Pa = Pg[q * N + e];
            const double z8 = 0.125 * Pa * rsqrt(d2); // P / (8 alpha Delta)
            const double hP = 0.5 * Pa;
            fs[0][q][le] = fma(z8, fma(5.0, ex, 3.0 * ey), -hP);
            fs[1][q][le] = z8 * sxy; // P / (4 alpha Delta) e12
            fs[2][q][le] = fma(z8, fma(5.0, ey, 3.0 * ex), -hP);
        }
    }
    __syncthreads();
    if (!active)
        return;
    const double keep = p.keepd;
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
        const int j = 3 * part + jj;
        double ax = 0.0, ay = 0.0;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const double a1 = o.a1[(j * 9 + q) * N + e];
            const double a2 = o.a2[(j * 9 + q) * N + e];
            const double f11 = fs[0][q][le], f12 = fs[1][q][le], f22 = fs[2][q][le];
            ax = fma(a1, f11, fma(a2, f12, ax));
            ay = fma(a1, f12, fma(a2, f22, ay));
            if constexpr (SPH) {
                const double a3 = o.a3[(j * 9 + q) * N + e];
                ax = fma(a3, f12, ax);
                ay = fma(-a3, f11, ay);
            }
        }
        tdiv[j * N + e] = fma(tdiv[j * N + e], keep, ax);
        tdiv[(9 + j) * N + e] = fma(tdiv[(9 + j) * N + e], keep, ay);
    }
}

// Gathers the divergence contributions of the (up to four) ice cells around
// a CG2 node in the reference's scatter order (even cell rows first, then
// odd; ascending x) and returns -sum.
__device__ __forceinline__ void gatherDivergence(const DevMesh& m, int i2, int j2,
    const double* __restrict__ contrib, double& dx, double& dy)
{
    const NodeCand X = nodeCand(i2, m.nx);
    NodeCand Y = nodeCand(j2, m.ny);
    if (Y.n == 2 && (Y.c0 & 1)) { // even cell rows first
        const int c = Y.c0, l = Y.l0;
        Y.c0 = Y.c1;
        Y.l0 = Y.l1;
        Y.c1 = c;
        Y.l1 = l;
    }
    const size_t N = m.N;
    double ax = 0.0, ay = 0.0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
        if (r < Y.n) {
            const int cy = r ? Y.c1 : Y.c0, ly = r ? Y.l1 : Y.l0;
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (k < X.n) {
                    const size_t c = size_t(cy) * m.nx + (k ? X.c1 : X.c0);
                    const int j = (k ? X.l1 : X.l0) + 3 * ly;
                    ax -= contrib[j * N + c];
                    ay -= contrib[(9 + j) * N + c];
                }
            }
        }
    }
    dx = ax;
    dy = ay;
}

__global__ void __launch_bounds__(kBlock) kMevpMomentum(DevMesh m, DevOps o, MevpNodeState st,
    const double* __restrict__ contrib, MevpParams p, int* __restrict__ err)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= m.Ncg)
        return;
    const int s2 = 2 * m.nx + 1;
    const int i2 = static_cast<int>(static_cast<unsigned>(i) % static_cast<unsigned>(s2)), j2 = static_cast<int>(static_cast<unsigned>(i) / static_cast<unsigned>(s2));
    const bool dir = m.cg2Dir[i] != 0;
    double dSx = 0.0, dSy = 0.0;
    if (!dir)
        gatherDivergence(m, i2, j2, contrib, dSx, dSy);
    const double u = st.u[i], v = st.v[i];
    const double uo = st.uo[i], vo = st.vo[i];
    const double uOcnRel = uo - u, vOcnRel = v - vo;
    const double absocn = sqrt(uOcnRel * uOcnRel + vOcnRel * vOcnRel);
    const double A = st.cgA[i];
    const double c1 = st.c1[i];
    const double invm = o.invm2[i];
    const double rden = 1.0 / (st.c1b[i] + A * p.F_ocean * absocn);
    const double focn = p.F_ocean * absocn;
    double un = rden * (c1 * (p.beta * u + st.u0[i]) + A * (st.fau[i] + focn * uo) - st.rhfc[i] * u
        - st.gu[i] + dSx * invm);
    double vn = rden * (c1 * (p.beta * v + st.v0[i]) + A * (st.fav[i] + focn * vo) + st.rhfc[i] * v
        - st.gv[i] + dSy * invm);
    if (!isfinite(un) || !isfinite(vn))
        atomicOr(err, DEV_ERR_NONFINITE_VELOCITY);
    if (dir) {
        un = 0.0;
        vn = 0.0;
    }
    st.u[i] = un;
    st.v[i] = vn;
}

// ===========================================================================
// mEVP, mixed precision
// ===========================================================================
__global__ void __launch_bounds__(kBlock) kMevpPrepNodes32(size_t n, MevpNodeState st, MevpNodeState32 f,
    const double* __restrict__ invm2, const uint8_t* __restrict__ dir, MevpParams p, float* __restrict__ uLast,
    float* __restrict__ vLast)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    // clamps of prepareIteration (CGDynamicsKernel.cpp:273-275)
    const double A = fmax(fmin(st.cgA[i], 1.0), 1.e-4);
    const double H = fmax(st.cgH[i], 1.e-4);
    st.cgA[i] = A;
    st.cgH[i] = H;
    const double u = st.u[i], v = st.v[i];
    st.u0[i] = u;
    st.v0[i] = v;
    // c1 = rho H / dt and its reciprocal: one FP64 division per node
    const double rhoH = p.rho_ice * H;
    const double rc1 = p.dt / rhoH;
    const double ua = st.ua[i], va = st.va[i];
    const double fatm = p.F_atm * sqrt(ua * ua + va * va);
    const float uf = static_cast<float>(u), vf = static_cast<float>(v);
    f.u[i] = uf;
    f.v[i] = vf;
    f.u0[i] = uf;
    f.v0[i] = vf;
    if (uLast) { // the velocity at the start of this sub-cycle (warm-start features)
        uLast[i] = uf;
        vLast[i] = vf;
    }
    // u0 + (A F_atm |wind| uwind - rho H g dxSSH) / c1, in FP64
    const double ku = u + (A * (fatm * ua) - rhoH * p.gravity * st.uGrad[i]) * rc1;
    const double kv = v + (A * (fatm * va) - rhoH * p.gravity * st.vGrad[i]) * rc1;
    const double im = invm2[i] * rc1;
    const float hi = static_cast<float>(im);
    f.k0[i] = make_float4(static_cast<float>(A * rc1), static_cast<float>(ku), static_cast<float>(kv),
        static_cast<float>(st.uo[i]));
    f.k1[i] = make_float4(static_cast<float>(st.vo[i]), hi, static_cast<float>(im - static_cast<double>(hi)),
        dir[i] ? 1.f : 0.f);
}

// The FP64 kernel kMevpStress with FP32 operators and state.  The strain
// invariant 1.25(e11^2+e22^2) + 1.5 e11 e22 + e12^2 is formed in FP32 from the
// FP32 strain (it is a positive-definite quadratic form: no cancellation);
// Delta = sqrt(invariant + DeltaMin^2) and the viscosity P/(8 alpha Delta) are
// evaluated in FP64 (Pg holds P/(8 alpha), hP = P/(2 alpha) in FP32); the
// stress increments and the divergence update are FP32.
// Body of the mixed-precision element kernel for element e handled by thread
// (le, part) of a block of kStressElems x kStressParts threads; shared by the
// single-grid and the batched (ensemble) kernels.
__device__ __forceinline__ void mevpStress32Element(int nx, size_t N, bool active, size_t e, int le, int part,
    const DevOps32& o, const float* __restrict__ u, const float* __restrict__ v, const double* __restrict__ Pg,
    const float* __restrict__ hPg, float* __restrict__ tdiv, const MevpParams& p, float (*fs)[9][kStressElems])
{
    if (active) {
        const size_t s2 = 2 * size_t(nx) + 1;
        const size_t ix = static_cast<unsigned>(e) % static_cast<unsigned>(nx);
        const size_t iy = static_cast<unsigned>(e) / static_cast<unsigned>(nx);
        const size_t base = 2 * s2 * iy + 2 * ix;
        float ul[9], vl[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const size_t nd = base + (j % 3) + (j / 3) * s2;
            ul[j] = u[nd];
            vl[j] = v[nd];
        }
        const double dmin = p.DeltaMin; // Delta^2 = inv + DeltaMin^2 with one rounding (FMA)
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) {
            const int q = 3 * part + qq;
            float ex = 0.f, ey = 0.f, exv = 0.f, eyu = 0.f;
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const float gxq = o.gx[(q * 9 + j) * o.ld + e];
                const float gyq = o.gy[(q * 9 + j) * o.ld + e];
                ex = fmaf(gxq, ul[j], ex);
                ey = fmaf(gyq, vl[j], ey);
                exv = fmaf(gxq, vl[j], exv);
                eyu = fmaf(gyq, ul[j], eyu);
            }
            if (o.gm) { // spherical metric term
                float mu = 0.f, mv = 0.f;
#pragma unroll
                for (int j = 0; j < 9; ++j) {
                    const float gmq = o.gm[(q * 9 + j) * o.ld + e];
                    mu = fmaf(gmq, ul[j], mu);
                    mv = fmaf(gmq, vl[j], mv);
                }
                ex -= mv;
                eyu += mu;
            }
            const float sxy = exv + eyu;
            const float inv = 1.25f * (ex * ex + ey * ey) + 1.50f * ex * ey + 0.25f * sxy * sxy;
            const float z8 = static_cast<float>(Pg[q * N + e] * rsqrt(fma(dmin, dmin, static_cast<double>(inv))));
            const float hP = hPg[q * N + e];
            fs[0][q][le] = fmaf(z8, fmaf(5.f, ex, 3.f * ey), -hP);
            fs[1][q][le] = z8 * sxy;
            fs[2][q][le] = fmaf(z8, fmaf(5.f, ey, 3.f * ex), -hP);
        }
    }
    __syncthreads();
    if (!active)
        return;
    const float keep = p.keep;
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
        const int j = 3 * part + jj;
        float ax = 0.f, ay = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float a1 = o.a1[(j * 9 + q) * o.ld + e];
            const float a2 = o.a2[(j * 9 + q) * o.ld + e];
            const float f11 = fs[0][q][le], f12 = fs[1][q][le], f22 = fs[2][q][le];
            ax = fmaf(a1, f11, fmaf(a2, f12, ax));
            ay = fmaf(a1, f12, fmaf(a2, f22, ay));
            if (o.a3) {
                const float a3 = o.a3[(j * 9 + q) * o.ld + e];
                ax = fmaf(a3, f12, ax);
                ay = fmaf(-a3, f11, ay);
            }
        }
        tdiv[j * N + e] = fmaf(tdiv[j * N + e], keep, ax);
        tdiv[(9 + j) * N + e] = fmaf(tdiv[(9 + j) * N + e], keep, ay);
    }
}

// The FP64 kernel kMevpStress with FP32 operators and state.  The strain
// invariant 1.25(e11^2+e22^2) + 1.5 e11 e22 + e12^2 is formed in FP32 from the
// FP32 strain (it is a positive-definite quadratic form: no cancellation);
// Delta = sqrt(invariant + DeltaMin^2) and the viscosity P/(8 alpha Delta) are
// evaluated in FP64; the stress increments and the divergence update are FP32.
__global__ void __launch_bounds__(kStressElems * kStressParts) kMevpStress32(DevMesh m, DevOps32 o,
    const float* __restrict__ u, const float* __restrict__ v, const double* __restrict__ Pg,
    const float* __restrict__ hP, float* __restrict__ tdiv, MevpParams p)
{
    __shared__ float fs[3][9][kStressElems];
    const int le = threadIdx.x % kStressElems;
    const int part = threadIdx.x / kStressElems;
    const size_t e = blockIdx.x * size_t(kStressElems) + le;
    const bool active = e < m.N && m.ice[e];
    mevpStress32Element(m.nx, m.N, active, e, le, part, o, u, v, Pg, hP, tdiv, p, fs);
}

// ---------------------------------------------------------------------------
// TMA-staged FP32 stress kernel
// ---------------------------------------------------------------------------
// The arithmetic of mevpStress32Element, with the operator entries of a
// block's 32 elements brought into shared memory by 2-D TMA copies that
// complete on mbarriers: first the strain rows (G_x, G_y: box {32 elements,
// 162 rows}, 20.7 KB), then, into the same buffer once the strain phase has
// read it, the divergence rows (A_1, A_2).  One 24 KB buffer per block keeps
// nine blocks (27 warps) resident per SM, each with a 20.7 KB copy in
// flight; the velocity gathers and P/alpha loads are issued while the first
// copy lands.  Waits are bounded in time (kWaitNs of the GPU's global timer,
// and at most kTmaSpin polls): a copy that has not landed by then sets
// DEV_ERR_TIMEOUT and the block returns after a second bounded wait for the
// copy it issued.
namespace {
constexpr int kTmaRows = 162;                           // G_x | G_y  (A_1 | A_2)
constexpr int kTmaRowsSph = 243;                        // G_x | G_y | G_m  (A_1 | A_2 | A_3)
template <bool SPH> __host__ __device__ constexpr int tmaRows() { return SPH ? kTmaRowsSph : kTmaRows; }
template <bool SPH> __host__ __device__ constexpr unsigned tmaTileBytes() { return tmaRows<SPH>() * kTmaElems * 4; }
} // namespace

// One block of the TMA-staged stress kernel: elements x0 .. x0+31 of a grid
// (shared by the single-grid and the batched ensemble kernels).
template <bool SPH>
__device__ __forceinline__ void stress32TmaBlock(const CUtensorMap* mapG, const CUtensorMap* mapA, int nx, size_t N,
    const uint8_t* __restrict__ ice, const float* __restrict__ u, const float* __restrict__ v,
    const double* __restrict__ Pg, const float* __restrict__ hPg, float* __restrict__ tdiv, const MevpParams& p,
    int* __restrict__ err, int x0, unsigned char* smem)
{
    float* sT = reinterpret_cast<float*>(smem);                      // [162][32]: G_x|G_y, then A_1|A_2
    float (*fs)[9][kTmaElems] = reinterpret_cast<float (*)[9][kTmaElems]>(sT + tmaRows<SPH>() * kTmaElems);
    uint64_t* bars = reinterpret_cast<uint64_t*>(fs[3]);             // 2 mbarriers, one per copy
    const int le = threadIdx.x % kTmaElems;
    const int part = threadIdx.x / kTmaElems;
    if (threadIdx.x == 0) {
        mbarInit(&bars[0], 1);
        mbarInit(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbarExpectTx(&bars[0], tmaTileBytes<SPH>());
        tmaLoad2d(sT, mapG, x0, 0, &bars[0]);
    }
    const size_t e = size_t(x0) + le;
    const bool active = e < N && ice[e];
    // P/(8 alpha), P/(2 alpha) (fixed during the sub-cycle) are loaded while the
    // copy lands; launched as a programmatic dependent of the previous
    // kernel, everything up to here overlaps that kernel's tail, and the
    // velocities and divergence it wrote are read only after the wait
    float ul[9], vl[9];
    double Pa[3];
    float hP[3];
    if (active) {
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) {
            Pa[qq] = Pg[(3 * part + qq) * N + e];
            hP[qq] = hPg[(3 * part + qq) * N + e];
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (active) {
        const size_t s2 = 2 * size_t(nx) + 1;
        const size_t ix = static_cast<unsigned>(e) % static_cast<unsigned>(nx);
        const size_t iy = static_cast<unsigned>(e) / static_cast<unsigned>(nx);
        const size_t base = 2 * s2 * iy + 2 * ix;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const size_t nd = base + (j % 3) + (j / 3) * s2;
            ul[j] = u[nd];
            vl[j] = v[nd];
        }
    }
    __syncthreads(); // the barriers are initialised before anyone polls them
    bool ok = mbarWaitBounded(&bars[0], 0);
    if (ok && active) {
        const double dmin = p.DeltaMin; // Delta^2 = inv + DeltaMin^2 with one rounding (FMA)
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) {
            const int q = 3 * part + qq;
            float ex = 0.f, ey = 0.f, exv = 0.f, eyu = 0.f;
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const float gxq = sT[(q * 9 + j) * kTmaElems + le];
                const float gyq = sT[(81 + q * 9 + j) * kTmaElems + le];
                ex = fmaf(gxq, ul[j], ex);
                ey = fmaf(gyq, vl[j], ey);
                exv = fmaf(gxq, vl[j], exv);
                eyu = fmaf(gyq, ul[j], eyu);
            }
            if constexpr (SPH) {
                float mu = 0.f, mv = 0.f;
#pragma unroll
                for (int j = 0; j < 9; ++j) {
                    const float gmq = sT[(162 + q * 9 + j) * kTmaElems + le];
                    mu = fmaf(gmq, ul[j], mu);
                    mv = fmaf(gmq, vl[j], mv);
                }
                ex -= mv;
                eyu += mu;
            }
            const float sxy = exv + eyu;
            const float inv = 1.25f * (ex * ex + ey * ey) + 1.50f * ex * ey + 0.25f * sxy * sxy;
            const float z8 = static_cast<float>(Pa[qq] * rsqrt(fma(dmin, dmin, static_cast<double>(inv))));
            fs[0][q][le] = fmaf(z8, fmaf(5.f, ex, 3.f * ey), -hP[qq]);
            fs[1][q][le] = z8 * sxy;
            fs[2][q][le] = fmaf(z8, fmaf(5.f, ey, 3.f * ex), -hP[qq]);
        }
    }
    // every thread has finished reading the strain rows (and written its
    // stress terms): the buffer may take the divergence rows
    if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0) {
            atomicOr(err, DEV_ERR_TIMEOUT);
            mbarWaitBounded(&bars[0], 0);
        }
        __syncthreads();
        return;
    }
    if (threadIdx.x == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbarExpectTx(&bars[1], tmaTileBytes<SPH>());
        tmaLoad2d(sT, mapA, x0, 0, &bars[1]);
    }
    ok = mbarWaitBounded(&bars[1], 0);
    if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0) {
            atomicOr(err, DEV_ERR_TIMEOUT);
            mbarWaitBounded(&bars[1], 0);
        }
        __syncthreads();
        return;
    }
    if (!active)
        return;
    const float keep = p.keep;
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
        const int j = 3 * part + jj;
        float ax = 0.f, ay = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float a1 = sT[(j * 9 + q) * kTmaElems + le];
            const float a2 = sT[(81 + j * 9 + q) * kTmaElems + le];
            const float f11 = fs[0][q][le], f12 = fs[1][q][le], f22 = fs[2][q][le];
            ax = fmaf(a1, f11, fmaf(a2, f12, ax));
            ay = fmaf(a1, f12, fmaf(a2, f22, ay));
            if constexpr (SPH) {
                const float a3 = sT[(162 + j * 9 + q) * kTmaElems + le];
                ax = fmaf(a3, f12, ax);
                ay = fmaf(-a3, f11, ay);
            }
        }
        tdiv[j * N + e] = fmaf(tdiv[j * N + e], keep, ax);
        tdiv[(9 + j) * N + e] = fmaf(tdiv[(9 + j) * N + e], keep, ay);
    }
}

template <bool SPH>
__global__ void __launch_bounds__(kTmaElems * kStressParts) kMevpStress32Tma(const __grid_constant__ CUtensorMap mapG,
    const __grid_constant__ CUtensorMap mapA, DevMesh m, const float* __restrict__ u, const float* __restrict__ v,
    const double* __restrict__ Pg, const float* __restrict__ hPg, float* __restrict__ tdiv, MevpParams p,
    int* __restrict__ err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    stress32TmaBlock<SPH>(&mapG, &mapA, m.nx, m.N, m.ice, u, v, Pg, hPg, tdiv, p, err, blockIdx.x * kTmaElems, smem);
}

// ---------------------------------------------------------------------------
// FP32 stress kernel for parallelogram meshes
// ---------------------------------------------------------------------------
// On a mesh of parallelograms every element's operators are combinations of
// the unit-square ones with 5 coefficients per element (c0..c3 the Jacobian
// entries, c4 = 1/J; the host derives them and checks the rebuilt operators
// against the exact ones).  The unit-square operators sit in constant memory
// and each warp handles a fixed third of the Gauss points and nodes, so their
// entries are compile-time constant-bank operands; per element-iteration the
// kernel streams 5 coefficients, P/(8 alpha), P/(2 alpha), the divergence and
// the velocities instead of 324 operator entries.
namespace {
constexpr int kAffElems = 32;
__constant__ float cAff[4][81]; // G_xi [q][j], G_eta [q][j], A_xi [j][q], A_eta [j][q]

// float <-> double by exponent rebiasing on the integer pipe (GB300 executes
// FP64 at about 1/60 of its FP32 rate): exact for positive normal
// floats; a value below the smallest normal float maps to zero.
__device__ __forceinline__ double widenPos(float f)
{
    const unsigned long long b = (static_cast<unsigned long long>(__float_as_uint(f)) << 29) + (896ull << 52);
    return __longlong_as_double(static_cast<long long>(b));
}
// f / 2 for a positive normal float f (exact)
__device__ __forceinline__ double widenHalfPos(float f)
{
    const unsigned long long b = (static_cast<unsigned long long>(__float_as_uint(f)) << 29) + (895ull << 52);
    return __longlong_as_double(static_cast<long long>(b));
}
__device__ __forceinline__ double widenNonneg(float f)
{
    return __float_as_uint(f) >= 0x00800000u ? widenPos(f) : 0.0;
}
// d >= 0 and below 2^128: nearest float (ties away from zero); 0 below the
// smallest normal float
__device__ __forceinline__ float narrowPos(double d)
{
    const long long b = __double_as_longlong(d);
    const long long r = (b - (896ll << 52) + (1ll << 28)) >> 29;
    return b >= (897ll << 52) ? __uint_as_float(static_cast<unsigned>(r)) : 0.f;
}
} // namespace

// P/(8 alpha Delta) with Delta = sqrt(t), t = inv + DeltaMin^2 formed in FP64
// with one rounding (FMA), evaluated in FP64.  VM 0: CUDA's rsqrt(double).
// VM 1 and 2: one Newton-Raphson step for the reciprocal square root,
// y1 = y0 + y0 (1 - t y0^2) / 2, in FP64 from the FP32 seed
// y0 = rsqrtf(inv + DeltaMin^2) (relative error of y1: 1.5 e0^2 + FP64
// rounding, e0 <= 2^-21 for the seed and its FP32 argument, i.e. below
// 1e-12); VM 2 converts between float and double on the integer pipe (y0/2
// by the exponent bias).  Five FP64 instructions per Gauss point in VM 2.
// VM 3: the same Newton step from the same seed with float pairs on the FP32
// pipe (nsdg_visc_ff.hpp: one FP64 subtraction per Gauss point; dmin2lo is
// the low part of DeltaMin^2).  VM 4: VM 3's float pairs with the check of
// nsdg_ff::viscFloatFloatChecked, and VM 2's FP64 operations from the same
// seed wherever the check cannot prove the pair's rounding equal to theirs
// (near a float rounding boundary: about 1e-4 of the Gauss points): bitwise
// VM 2's result with one FP64 subtraction per Gauss point instead of five
// FP64 instructions (measured slower than VM 2 on GB300: the float-pair
// arithmetic and the check cost more issue than the FP64 pipe they free).
__device__ __forceinline__ float viscNewton64(float inv, double Pa, double dmin, float y0)
{
    const double t = fma(dmin, dmin, widenNonneg(inv));
    const double yd = widenPos(y0);
    const double h = t * yd;
    const double e2 = fma(-h, widenHalfPos(y0), 0.5); // (1 - t y0^2) / 2
    const double z = Pa * yd;
    return narrowPos(fma(z, e2, z));
}

template <int VM>
__device__ __forceinline__ float viscosity8(float inv, double Pa, double dmin, float dmin2f, float dmin2lo)
{
    if constexpr (VM == 3) {
        return nsdg_ff::viscFloatFloat(inv, Pa, dmin2f, dmin2lo, rsqrtf(inv + dmin2f));
    } else if constexpr (VM == 4) {
        const float y0 = rsqrtf(inv + dmin2f);
        bool exact;
        const float z = nsdg_ff::viscFloatFloatChecked(inv, Pa, dmin2f, dmin2lo, y0, exact);
        return exact ? z : viscNewton64(inv, Pa, dmin, y0);
    } else {
        const double td = VM == 2 ? widenNonneg(inv) : static_cast<double>(inv);
        const double t = fma(dmin, dmin, td);
        if constexpr (VM == 0) {
            return static_cast<float>(Pa * rsqrt(t));
        } else {
            const float y0 = rsqrtf(inv + dmin2f);
            const double yd = VM == 1 ? static_cast<double>(y0) : widenPos(y0);
            const double yh = VM == 1 ? 0.5 * yd : widenHalfPos(y0);
            const double h = t * yd;
            const double e2 = fma(-h, yh, 0.5); // (1 - t y0^2) / 2
            const double z = Pa * yd;
            const double z8 = fma(z, e2, z);
            return VM == 1 ? static_cast<float>(z8) : narrowPos(z8);
        }
    }
}

template <int PART, int VM>
__device__ __forceinline__ void affineStrain(const float (&ul)[9], const float (&vl)[9], const float (&c)[5],
    const double (&Pa)[3], const float (&hP)[3], double dmin, float dmin2f, float dmin2lo,
    float (*fs)[9][kAffElems], int le)
{
#pragma unroll
    for (int qq = 0; qq < 3; ++qq) {
        constexpr int q0 = 3 * PART;
        const int q = q0 + qq;
        float ux = 0.f, ue = 0.f, vx = 0.f, ve = 0.f;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const float gx = cAff[0][q * 9 + j], ge = cAff[1][q * 9 + j];
            ux = fmaf(gx, ul[j], ux);
            ue = fmaf(ge, ul[j], ue);
            vx = fmaf(gx, vl[j], vx);
            ve = fmaf(ge, vl[j], ve);
        }
        const float ex = c[4] * fmaf(c[0], ux, c[1] * ue);  // G_x u
        const float ey = c[4] * fmaf(c[2], vx, c[3] * ve);  // G_y v
        const float exv = c[4] * fmaf(c[0], vx, c[1] * ve); // G_x v
        const float eyu = c[4] * fmaf(c[2], ux, c[3] * ue); // G_y u
        const float sxy = exv + eyu;
        const float inv = 1.25f * (ex * ex + ey * ey) + 1.50f * ex * ey + 0.25f * sxy * sxy;
        const float z8 = viscosity8<VM>(inv, Pa[qq], dmin, dmin2f, dmin2lo);
        const float f11 = fmaf(z8, fmaf(5.f, ex, 3.f * ey), -hP[qq]);
        const float f12 = z8 * sxy;
        const float f22 = fmaf(z8, fmaf(5.f, ey, 3.f * ex), -hP[qq]);
        // the Gauss-point weights of A_xi and A_eta in A_1 f11 + A_2 f12 and
        // A_1 f12 + A_2 f22
        fs[0][q][le] = fmaf(c[0], f11, c[2] * f12);
        fs[1][q][le] = fmaf(c[1], f11, c[3] * f12);
        fs[2][q][le] = fmaf(c[0], f12, c[2] * f22);
        fs[3][q][le] = fmaf(c[1], f12, c[3] * f22);
    }
}

template <int PART>
__device__ __forceinline__ void affineDivergence(float (*fs)[9][kAffElems], int le, size_t e, size_t N,
    float* __restrict__ tdiv, float keep, const float (&told)[6])
{
    float w[4][9];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int q = 0; q < 9; ++q)
            w[k][q] = fs[k][q][le];
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
        const int j = 3 * PART + jj;
        float ax = 0.f, ay = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const float axi = cAff[2][j * 9 + q], aet = cAff[3][j * 9 + q];
            ax = fmaf(axi, w[0][q], fmaf(aet, w[1][q], ax));
            ay = fmaf(axi, w[2][q], fmaf(aet, w[3][q], ay));
        }
        tdiv[j * N + e] = fmaf(told[jj], keep, ax);
        tdiv[(9 + j) * N + e] = fmaf(told[3 + jj], keep, ay);
    }
}

// One block of the parallelogram stress kernel: elements x0 .. x0+31 of a
// grid (shared by the single-grid and the batched ensemble kernels).
template <int VM>
__device__ __forceinline__ void affineBlock(int nx, size_t N, const uint8_t* __restrict__ ice,
    const float* __restrict__ coef, size_t ld, const float* __restrict__ u, const float* __restrict__ v,
    const double* __restrict__ Pg, float* __restrict__ tdiv, const MevpParams& p, size_t x0,
    float (*fs)[9][kAffElems])
{
    const int le = threadIdx.x % kAffElems;
    const int part = threadIdx.x / kAffElems; // one warp per third of the Gauss points / nodes
    const size_t e = x0 + le;
    const bool active = e < N && ice[e];
    // step constants first: a programmatic dependent launch overlaps them
    // with the previous kernel's tail.  So does this element's divergence
    // from the previous iteration: no launch triggers its dependents early,
    // so this kernel starts only after the node kernel before it has exited,
    // and that kernel read the divergence only after the stress kernel that
    // wrote it had completed; the node kernel only reads it.
    float c[5], ul[9], vl[9], hP[3], told[6];
    double Pa[3];
    if (active) {
#pragma unroll
        for (int jj = 0; jj < 3; ++jj) {
            told[jj] = tdiv[(3 * part + jj) * N + e];
            told[3 + jj] = tdiv[(9 + 3 * part + jj) * N + e];
        }
#pragma unroll
        for (int k = 0; k < 5; ++k)
            c[k] = coef[k * ld + e];
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) {
            Pa[qq] = Pg[(3 * part + qq) * N + e];
            // P/(2 alpha) = 4 P/(8 alpha): an exact power-of-two scaling,
            // rounded to float on the integer pipe (the value the prep kernel
            // stores for the other element kernels)
            hP[qq] = narrowPos(__longlong_as_double(__double_as_longlong(Pa[qq]) + (2ll << 52)));
        }
    }
    asm volatile("griddepcontrol.wait;" ::: "memory");
    if (active) {
        const size_t s2 = 2 * size_t(nx) + 1;
        const size_t ix = static_cast<unsigned>(e) % static_cast<unsigned>(nx);
        const size_t iy = static_cast<unsigned>(e) / static_cast<unsigned>(nx);
        const size_t base = 2 * s2 * iy + 2 * ix;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const size_t nd = base + (j % 3) + (j / 3) * s2;
            ul[j] = u[nd];
            vl[j] = v[nd];
        }
        const double dmin = p.DeltaMin;
        const float dmin2f = p.dmin2f, dmin2lo = p.dmin2lo;
        switch (part) {
        case 0: affineStrain<0, VM>(ul, vl, c, Pa, hP, dmin, dmin2f, dmin2lo, fs, le); break;
        case 1: affineStrain<1, VM>(ul, vl, c, Pa, hP, dmin, dmin2f, dmin2lo, fs, le); break;
        default: affineStrain<2, VM>(ul, vl, c, Pa, hP, dmin, dmin2f, dmin2lo, fs, le); break;
        }
    }
    __syncthreads();
    if (!active)
        return;
    const float keep = p.keep;
    switch (part) {
    case 0: affineDivergence<0>(fs, le, e, N, tdiv, keep, told); break;
    case 1: affineDivergence<1>(fs, le, e, N, tdiv, keep, told); break;
    default: affineDivergence<2>(fs, le, e, N, tdiv, keep, told); break;
    }
}

template <int VM>
__global__ void __launch_bounds__(kAffElems * kStressParts, 12) kMevpStress32Affine(DevMesh m,
    const float* __restrict__ coef, size_t ld, const float* __restrict__ u, const float* __restrict__ v,
    const double* __restrict__ Pg, float* __restrict__ tdiv, MevpParams p)
{
    __shared__ float fs[4][9][kAffElems];
    affineBlock<VM>(m.nx, m.N, m.ice, coef, ld, u, v, Pg, tdiv, p, blockIdx.x * size_t(kAffElems), fs);
}

// Self-test of the FP64 viscosity forms: out[3 n] = P/(8 alpha Delta) for
// every VM (0, 1, 2) at each (inv, Pa).
__global__ void kViscositySelfTest(size_t n, const float* __restrict__ inv, const double* __restrict__ Pa,
    double dmin, float* __restrict__ out)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const float dmin2f = static_cast<float>(dmin * dmin);
    out[i] = viscosity8<0>(inv[i], Pa[i], dmin, dmin2f, 0.f);
    out[n + i] = viscosity8<1>(inv[i], Pa[i], dmin, dmin2f, 0.f);
    out[2 * n + i] = viscosity8<2>(inv[i], Pa[i], dmin, dmin2f, 0.f);
}

// The float-float form (VM 3) at each (inv, Pa): out[n].
__global__ void kViscositySelfTestFF(size_t n, const float* __restrict__ inv, const double* __restrict__ Pa,
    double dmin, float* __restrict__ out)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const float d2h = static_cast<float>(dmin * dmin);
    out[i] = viscosity8<3>(inv[i], Pa[i], dmin, d2h, nsdg_ff::narrowAny(fma(dmin, dmin, -nsdg_ff::widenPos(d2h))));
}

// The checked float-pair form (VM 4) at each (inv, Pa): out[n]; bitwise VM 2.
__global__ void kViscositySelfTestChecked(size_t n, const float* __restrict__ inv, const double* __restrict__ Pa,
    double dmin, float* __restrict__ out)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const float d2h = static_cast<float>(dmin * dmin);
    out[i] = viscosity8<4>(inv[i], Pa[i], dmin, d2h, nsdg_ff::narrowAny(fma(dmin, dmin, -nsdg_ff::widenPos(d2h))));
}

// Body of the mixed-precision node kernel for CG2 node i.
__device__ __forceinline__ void mevpMomentum32Node(int nx, int ny, size_t N, size_t i, const uint8_t* __restrict__ cg2Dir,
    const MevpNodeState32& st, const float* __restrict__ tdiv, const MevpParams& p, int* __restrict__ err)
{
    // 32-bit index arithmetic (node counts stay far below 2^31)
    const unsigned s2 = 2u * static_cast<unsigned>(nx) + 1u;
    const int i2 = static_cast<int>(static_cast<unsigned>(i) % s2), j2 = static_cast<int>(static_cast<unsigned>(i) / s2);
    // per-step constants first, two 16-byte loads (a programmatic dependent
    // launch overlaps them with the stress kernel's tail), then the wait for
    // its results
    const float4 c0 = st.k0[i], c1 = st.k1[i];
    const float a = c0.x, ku = c0.y, kv = c0.z, uo = c0.w, vo = c1.x;
    const float2 im = make_float2(c1.y, c1.z);
    const bool dir = c1.w != 0.f;
    asm volatile("griddepcontrol.wait;" ::: "memory");
    float dSx = 0.f, dSy = 0.f;
    if (!dir) {
        const NodeCand X = nodeCand(i2, nx);
        NodeCand Y = nodeCand(j2, ny);
        if (Y.n == 2 && (Y.c0 & 1)) { // even cell rows first (the reference's accumulation order)
            const int c = Y.c0, l = Y.l0;
            Y.c0 = Y.c1;
            Y.l0 = Y.l1;
            Y.c1 = c;
            Y.l1 = l;
        }
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            if (r < Y.n) {
                const int cy = r ? Y.c1 : Y.c0, ly = r ? Y.l1 : Y.l0;
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    if (k < X.n) {
                        const size_t c = size_t(cy) * nx + (k ? X.c1 : X.c0);
                        const int j = (k ? X.l1 : X.l0) + 3 * ly;
                        dSx -= tdiv[j * N + c];
                        dSy -= tdiv[(9 + j) * N + c];
                    }
                }
            }
        }
    }
    // the divergence over the lumped mass and c1: that factor is FP64, held
    // as the unevaluated sum hi + lo of two floats and applied with FP32 FMAs
    const float mx = fmaf(dSx, im.y, dSx * im.x);
    const float my = fmaf(dSy, im.y, dSy * im.x);
    const float u = st.u[i], v = st.v[i];
    const float uOcnRel = uo - u, vOcnRel = v - vo;
    const float afocn = a * (p.F_oceanf * sqrtf(uOcnRel * uOcnRel + vOcnRel * vOcnRel));
    const float rden = 1.0f / (p.onePlusBetaf + afocn);
    // (beta u + ku + a focn uo - fc dt u + mx) / (1 + beta + a focn), VPCGDynamicsKernel.hpp:132-172 over c1
    float un = rden * (p.betaf * u + ku + afocn * uo - p.fcdtf * u + mx);
    float vn = rden * (p.betaf * v + kv + afocn * vo + p.fcdtf * v + my);
    if (!isfinite(un) || !isfinite(vn))
        atomicOr(err, DEV_ERR_NONFINITE_VELOCITY);
    if (dir) {
        un = 0.f;
        vn = 0.f;
    }
    st.u[i] = un;
    st.v[i] = vn;
}

__global__ void __launch_bounds__(kBlock) kMevpMomentum32(DevMesh m, MevpNodeState32 st,
    const float* __restrict__ tdiv, MevpParams p, int* __restrict__ err)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= m.Ncg)
        return;
    mevpMomentum32Node(m.nx, m.ny, m.N, i, m.cg2Dir, st, tdiv, p, err);
}

// ---------------------------------------------------------------------------
// Batched ensemble: one launch covers the elements (nodes) of every member.
// Block b belongs to member blockMember[b]; within the member, stress blocks
// map to 2D tiles of tileW x tileH elements (tileW * tileH = kStressElems,
// chosen per grid size by the ensemble's autotuner) and node blocks to
// consecutive runs of kBlock CG2 nodes.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kStressElems * kStressParts) kMevpStress32Batched(
    const EnsembleMember* __restrict__ members, const uint16_t* __restrict__ blockMember, MevpParams p)
{
    __shared__ float fs[3][9][kStressElems];
    const EnsembleMember& M = members[blockMember[blockIdx.x]];
    const int b = static_cast<int>(blockIdx.x) - M.stressBlock0;
    const int le = threadIdx.x % kStressElems;
    const int part = threadIdx.x / kStressElems;
    const int tx = b % M.tilesX, ty = b / M.tilesX;
    const int ix = tx * M.tileW + le % M.tileW, iy = ty * M.tileH + le / M.tileW;
    const bool inside = ix < M.nx && iy < M.ny;
    const size_t e = inside ? size_t(iy) * M.nx + ix : 0;
    const bool active = inside && M.ice[e];
    mevpStress32Element(M.nx, M.N, active, e, le, part, M.o, M.st.u, M.st.v, M.Pg, M.hP, M.tdiv, p, fs);
}

// Self-test of the bounded wait: one thread waits on an mbarrier that nothing
// will complete (expected arrivals 1, none made), records whether the wait
// ran out, and the barrier is left behind with the block.
__global__ void kBoundedWaitSelfTest(unsigned long long limitNs, int* __restrict__ timedOut)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbarInit(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *timedOut = mbarWaitBounded(&bar, 0, limitNs) ? 0 : 1;
    }
}

__global__ void __launch_bounds__(kTmaElems * kStressParts) kMevpStress32TmaBatched(
    const EnsembleMember* __restrict__ members, const uint16_t* __restrict__ blockMember, MevpParams p,
    int* __restrict__ err)
{
    extern __shared__ __align__(128) unsigned char smem[];
    const EnsembleMember& M = members[blockMember[blockIdx.x]];
    const int x0 = (static_cast<int>(blockIdx.x) - M.tmaBlock0) * kTmaElems;
    stress32TmaBlock<false>(&M.maps.g, &M.maps.a, M.nx, M.N, M.ice, M.st.u, M.st.v, M.Pg, M.hP, M.tdiv, p, err, x0,
        smem);
}

template <int VM>
__global__ void __launch_bounds__(kAffElems * kStressParts, 12) kMevpStress32AffineBatched(
    const EnsembleMember* __restrict__ members, const uint16_t* __restrict__ blockMember, MevpParams p)
{
    __shared__ float fs[4][9][kAffElems];
    const EnsembleMember& M = members[blockMember[blockIdx.x]];
    const size_t x0 = size_t(static_cast<int>(blockIdx.x) - M.tmaBlock0) * kAffElems;
    affineBlock<VM>(M.nx, M.N, M.ice, M.affCoef, M.affLd, M.st.u, M.st.v, M.Pg, M.tdiv, p, x0, fs);
}

// ---------------------------------------------------------------------------
// Persistent sub-cycle of a parallelogram ensemble: one cooperative launch
// runs all mEVP iterations of every member, the element phase and the node
// phase as grid-stride loops over the same block maps as the per-phase
// launches, separated by grid barriers.  Each element and node is computed
// by the same arithmetic in the same order as in kMevpStress32AffineBatched
// and kMevpMomentum32Batched, so the results are bitwise the same.
//
// The grid barrier is the project's own, with a bounded wait: bar[0] counts
// arrivals, bar[1] is the generation (both zero before the launch).  A block
// whose wait runs out (1 s of the GPU's global timer, or 2^26 polls) sets
// DEV_ERR_TIMEOUT and leaves the loop; every other block then runs out at
// its next barrier, so the kernel always ends.
namespace {
__device__ bool gridBarrierBounded(unsigned* bar, int* err, int* okShared)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned* gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        bool ok = true;
        if (atomicAdd(bar, 1u) == gridDim.x - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const unsigned long long t0 = globalTimerNs();
            for (long i = 0;; ++i) {
                if (*gen != g)
                    break;
                if (i >= kTmaSpin || ((i & 63) == 63 && globalTimerNs() - t0 > kWaitNs)) {
                    ok = false;
                    atomicOr(err, DEV_ERR_TIMEOUT);
                    break;
                }
            }
        }
        __threadfence();
        *okShared = ok ? 1 : 0;
    }
    __syncthreads();
    return *okShared != 0;
}
} // namespace

template <int VM>
__global__ void __launch_bounds__(kAffElems * kStressParts) kEnsembleSubcyclePersistent(
    const EnsembleMember* __restrict__ members, const uint16_t* __restrict__ elemMap, int elemBlocks,
    const uint16_t* __restrict__ nodeMap, int nodeBlocks, MevpParams p, int iterations, unsigned* __restrict__ bar,
    int* __restrict__ err)
{
    __shared__ float fs[4][9][kAffElems];
    __shared__ int okShared;
    constexpr int kThreads = kAffElems * kStressParts;
    for (int it = 0; it < iterations; ++it) {
        for (int b = blockIdx.x; b < elemBlocks; b += gridDim.x) {
            const EnsembleMember& M = members[elemMap[b]];
            const size_t x0 = size_t(b - M.tmaBlock0) * kAffElems;
            affineBlock<VM>(M.nx, M.N, M.ice, M.affCoef, M.affLd, M.st.u, M.st.v, M.Pg, M.tdiv, p, x0, fs);
            __syncthreads(); // the next work block reuses fs
        }
        if (!gridBarrierBounded(bar, err, &okShared))
            break;
        for (int b = blockIdx.x; b < nodeBlocks; b += gridDim.x) {
            const EnsembleMember& M = members[nodeMap[b]];
            const size_t i = size_t(b - M.nodeBlockP) * kThreads + threadIdx.x;
            if (i < M.Ncg)
                mevpMomentum32Node(M.nx, M.ny, M.N, i, M.cg2Dir, M.st, M.tdiv, p, err);
        }
        if (!gridBarrierBounded(bar, err, &okShared))
            break;
    }
}

__global__ void __launch_bounds__(kBlock) kMevpMomentum32Batched(const EnsembleMember* __restrict__ members,
    const uint16_t* __restrict__ blockMember, MevpParams p, int* __restrict__ err)
{
    const EnsembleMember& M = members[blockMember[blockIdx.x]];
    const size_t i = (static_cast<size_t>(blockIdx.x) - M.nodeBlock0) * kBlock + threadIdx.x;
    if (i >= M.Ncg)
        return;
    mevpMomentum32Node(M.nx, M.ny, M.N, i, M.cg2Dir, M.st, M.tdiv, p, err);
}

__global__ void kWidenVelocity(size_t n, const float* __restrict__ u32, const float* __restrict__ v32,
    double* __restrict__ u, double* __restrict__ v)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    u[i] = u32[i];
    v[i] = v32[i];
}

// ===========================================================================
// BBM (BBMStressUpdateStep.hpp:31-195, BrittleCGDynamicsKernel.hpp:206-254)
// ===========================================================================
__global__ void __launch_bounds__(kBlock) kBbmPrepNodes(size_t n, BbmNodeState st, BbmParams p,
    BbmNodeConst32 c)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const double Ad = fmax(fmin(st.cgA[i], 1.0), 1.e-4);
    const double Hd = fmax(st.cgH[i], 1.e-4);
    st.cgA[i] = Ad;
    st.cgH[i] = Hd;
    st.avgU[i] = 0.0;
    st.avgV[i] = 0.0;
    if (c.k0) {
        // the FP32 node kernel's sub-step-invariant terms, formed as it forms them
        const float H = static_cast<float>(Hd), A = static_cast<float>(Ad);
        const float dt = static_cast<float>(p.dt), rho = static_cast<float>(p.rho_ice);
        const float ua = static_cast<float>(st.ua[i]), va = static_cast<float>(st.va[i]);
        const float dragAtm = A * static_cast<float>(p.F_atm) * hypotf(ua, va);
        const float rhoHg = rho * H * static_cast<float>(p.gravity);
        c.k0[i] = make_float4(dt / (rho * H), A * static_cast<float>(p.F_ocean), static_cast<float>(st.uo[i]),
            static_cast<float>(st.vo[i]));
        c.k1[i] = make_float4(dragAtm * ua, dragAtm * va, rhoHg * static_cast<float>(st.uGrad[i]),
            rhoHg * static_cast<float>(st.vGrad[i]));
    }
}

// The mixed-precision BBM node update from the step's FP32 node constants
// (kBbmPrepNodes): per sub-step only the velocity, the gathered divergence
// and the running averages are read.
__global__ void __launch_bounds__(kBlock) kBbmMomentum32(DevMesh m, BbmNodeState st, BbmNodeConst32 c,
    const double* __restrict__ contrib, BbmParams p, int* __restrict__ err, const float2* __restrict__ invmHL)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= m.Ncg)
        return;
    const int s2 = 2 * m.nx + 1;
    const int i2 = static_cast<int>(static_cast<unsigned>(i) % static_cast<unsigned>(s2)), j2 = static_cast<int>(static_cast<unsigned>(i) / static_cast<unsigned>(s2));
    const bool dir = m.cg2Dir[i] != 0;
    const float4 k0 = c.k0[i], k1 = c.k1[i];
    const float2 im = invmHL[i];
    double dSx = 0.0, dSy = 0.0;
    if (!dir)
        gatherDivergence(m, i2, j2, contrib, dSx, dSy);
    const float dt = narrowAny(p.dt);
    const float cosA = narrowAny(p.cosA), sinA = narrowAny(p.sinA);
    const float dteOverMass = k0.x, AFo = k0.y, uo = k0.z, vo = k0.w;
    const float uIce = narrowAny(st.u[i]), vIce = narrowAny(st.v[i]);
    const float cPrime = AFo * hypotf(uo - uIce, vo - vIce);
    const float alpha = 1.f + dteOverMass * (cPrime * cosA);
    const float beta = dt * narrowAny(p.fc) + dteOverMass * cPrime * sinA;
    const float rDenom = 1.f / (alpha * alpha + beta * beta);
    const float tauX = k1.x + cPrime * (uo * cosA - vo * sinA);
    const float tauY = k1.y + cPrime * (vo * cosA + uo * sinA);
    const float fx = narrowAny(dSx), fy = narrowAny(dSy);
    const float gradX = fmaf(fx, im.y, fx * im.x) - k1.z;
    const float gradY = fmaf(fy, im.y, fy * im.x) - k1.w;
    float un = alpha * uIce + beta * vIce + dteOverMass * (alpha * (gradX + tauX) + beta * (gradY + tauY));
    un *= rDenom;
    float vn = alpha * vIce - beta * uIce + dteOverMass * (alpha * (gradY + tauY) + beta * (gradX + tauX));
    vn *= rDenom;
    if (!isfinite(un) || !isfinite(vn))
        atomicOr(err, DEV_ERR_NONFINITE_VELOCITY);
    st.avgU[i] += widenAny(un) * p.invNSteps;
    st.avgV[i] += widenAny(vn) * p.invNSteps;
    if (dir) {
        un = 0.f;
        vn = 0.f;
    }
    st.u[i] = widenAny(un);
    st.v[i] = widenAny(vn);
}

// x^y for x >= 0: by multiplication when y is a small integer (mode 1), times
// sqrt(x) when it is a small half-integer (mode 2), else pow().  Differs from
// pow() by a few ulps.
template <typename T> __device__ __forceinline__ T powByMode(T x, T y, int mode, int k)
{
    if (mode == 0)
        return pow(x, y);
    T r = T(1);
    for (int i = 0; i < k; ++i)
        r *= x;
    return mode == 2 ? r * sqrt(x) : r;
}

// Element operators of the BBM stress kernel in the compute type T.
template <typename T> struct BbmOps {
    const T* gx;
    const T* gy;
    const T* w;
    const T* wdam;
    const T* d1;
    const T* d2;
    const double* hsize;
    const T* gm; // spherical metric terms (null on Cartesian meshes)
    const T* dm;
    const float* coef = nullptr; // [5][ld] parallelogram coefficients (AFF kernels)
    size_t ld = 0;
};

// The unit square's BBM operators for the parallelogram-mesh kernel (with
// cAff's strain operators): iMJwPSI [k][q], the damage projection [k][q],
// D_xi and D_eta [j][k] (divS1 = c0 D_xi + c1 D_eta, divS2 = c2 D_xi +
// c3 D_eta)
struct BbmAffTables {
    float w[72];
    float wdam[72];
    float dxi[72];
    float deta[72];
};
__constant__ BbmAffTables cBbmAff;

// BBM stress, damage and divergence for one element.  T = double is the
// reference's arithmetic; T = float is the mixed-precision kernel (FP32
// operators and arithmetic, including exp/pow/sqrt; the stress, damage and
// divergence are stored FP64 for the FP64 transport of the stress fields;
// the conversions stay on the conversion unit: on the integer pipe, as in the
// other mixed kernels, this kernel measured 9 % slower).
// AFF (T = float on a parallelogram mesh): the strain from the unit
// square's operators and the element's coefficients c (as the mEVP
// parallelogram kernel), iMJwPSI and the damage projection from constant
// memory, the divergence as D_xi (c0 s_a + c2 s_b) + D_eta (c1 s_a + c3 s_b):
// 5 coefficients per element instead of 2 x 81 + 72 + 9 DG + 2 x 72
// operator entries.
template <int DG, typename T, bool AFF = false>
__global__ void __launch_bounds__(kBlock) kBbmStress(DevMesh m, BbmOps<T> o, const double* __restrict__ u,
    const double* __restrict__ v, const double* __restrict__ h, const double* __restrict__ a,
    double* __restrict__ damage, double* __restrict__ s11, double* __restrict__ s12,
    double* __restrict__ s22, double* __restrict__ contrib, BbmParams p, int* __restrict__ err)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    const size_t N = m.N;
    if (e >= N)
        return;
    const bool ice = m.ice[e] != 0;
    const size_t s2 = 2 * size_t(m.nx) + 1;
    const size_t ix = static_cast<unsigned>(e) % static_cast<unsigned>(m.nx), iy = static_cast<unsigned>(e) / static_cast<unsigned>(m.nx);
    const size_t base = 2 * s2 * iy + 2 * ix;
    T ul[9], vl[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        const size_t nd = base + (j % 3) + (j / 3) * s2;
        ul[j] = ice ? static_cast<T>(u[nd]) : T(0);
        vl[j] = ice ? static_cast<T>(v[nd]) : T(0);
    }
    T hc[DG], ac[DG], dc[DG], c11[8], c12[8], c22[8];
#pragma unroll
    for (int j = 0; j < DG; ++j) {
        hc[j] = static_cast<T>(h[j * N + e]);
        ac[j] = static_cast<T>(a[j * N + e]);
        dc[j] = static_cast<T>(damage[j * N + e]);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        c11[k] = static_cast<T>(s11[k * N + e]);
        c12[k] = static_cast<T>(s12[k * N + e]);
        c22[k] = static_cast<T>(s22[k * N + e]);
    }
    float cf[5] = { 0.f, 0.f, 0.f, 0.f, 0.f };
    if constexpr (AFF) {
#pragma unroll
        for (int k = 0; k < 5; ++k)
            cf[k] = o.coef[k * o.ld + e];
    }
    const T dt = static_cast<T>(p.dt);
    const T nu0 = static_cast<T>(p.nu0);
    const T hi = static_cast<T>(o.hsize[e]);
    const T scale_coef = sqrt(T(0.1) / hi);
    const T tdScale = hi * sqrt(T(2.) * (T(1.) + nu0) * static_cast<T>(p.rho_ice));
    T n11[8], n12[8], n22[8], nd[DG];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        n11[k] = n12[k] = n22[k] = T(0);
#pragma unroll
    for (int k = 0; k < DG; ++k)
        nd[k] = T(0);
#pragma unroll 1
    for (int q = 0; q < 9; ++q) {
        T hs = T(0), as = T(0), ds = T(0);
#pragma unroll
        for (int j = 0; j < DG; ++j) {
            hs += hc[j] * tab<T>::psi(3, j, q);
            as += ac[j] * tab<T>::psi(3, j, q);
            ds += dc[j] * tab<T>::psi(3, j, q);
        }
        const T hG = fmax(hs, T(0));
        const T aG = fmin(fmax(as, T(0)), T(1));
        T dG = fmin(fmax(ds, T(1e-12)), T(1));
        T ex = T(0), ey = T(0), exv = T(0), eyu = T(0);
        if constexpr (AFF) {
            float ux = 0.f, ue = 0.f, vx = 0.f, ve = 0.f;
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const float gx = cAff[0][q * 9 + j], ge = cAff[1][q * 9 + j];
                ux = fmaf(gx, ul[j], ux);
                ue = fmaf(ge, ul[j], ue);
                vx = fmaf(gx, vl[j], vx);
                ve = fmaf(ge, vl[j], ve);
            }
            ex = cf[4] * fmaf(cf[0], ux, cf[1] * ue);
            ey = cf[4] * fmaf(cf[2], vx, cf[3] * ve);
            exv = cf[4] * fmaf(cf[0], vx, cf[1] * ve);
            eyu = cf[4] * fmaf(cf[2], ux, cf[3] * ue);
        } else {
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const T gxq = o.gx[(q * 9 + j) * N + e];
                const T gyq = o.gy[(q * 9 + j) * N + e];
                ex = fma(gxq, ul[j], ex);
                ey = fma(gyq, vl[j], ey);
                exv = fma(gxq, vl[j], exv);
                eyu = fma(gyq, ul[j], eyu);
            }
        }
        if (!AFF && o.gm) { // spherical: e11 -= iMM v, e12 += iMM u / 2 (CGDynamicsKernel.cpp:331-334)
            T mu = T(0), mv = T(0);
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const T gmq = o.gm[(q * 9 + j) * N + e];
                mu = fma(gmq, ul[j], mu);
                mv = fma(gmq, vl[j], mv);
            }
            ex -= mv;
            eyu += mu;
        }
        const T e11 = ex, e22 = ey, e12 = T(0.5) * (exv + eyu);
        T g11 = T(0), g12 = T(0), g22 = T(0);
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            g11 += c11[k] * tab<T>::psi(3, k, q);
            g12 += c12[k] * tab<T>::psi(3, k, q);
            g22 += c22[k] * tab<T>::psi(3, k, q);
        }
        T sigma_n = T(0.5) * (g11 + g22);
        const T expC = exp(static_cast<T>(p.compaction_param) * (T(1.0) - aG));
        const T Pmax = static_cast<T>(p.P0)
            * powByMode(hG, static_cast<T>(p.exponent_compression_factor) + T(1.), p.powCmode, p.powCk) * expC;
        const T tildeP = (sigma_n < T(0)) ? fmin(-Pmax / sigma_n, T(1.0)) : T(0);
        T multiplicator;
        if constexpr (sizeof(T) == 8) {
            const T powalphaexpC
                = powByMode(dG * expC, static_cast<T>(p.exponent_relaxation_sigma) - T(1), p.powRmode, p.powRk);
            const T time_viscous = static_cast<T>(p.lambda) * powalphaexpC;
            multiplicator = time_viscous / (time_viscous + (T(1.) - tildeP) * dt);
        } else {
            // lambda (d e^{C(1-A)})^(n-1) underflows FP32 in open water and
            // 0 / (0 + 0) would follow where tildeP = 1: the same quantity as
            // 1 / (1 + (1 - tildeP) dt / time_viscous) with the relaxation
            // time taken in log space
            const T logTv = log(static_cast<T>(p.lambda))
                + (static_cast<T>(p.exponent_relaxation_sigma) - T(1))
                    * (log(dG) + static_cast<T>(p.compaction_param) * (T(1.0) - aG));
            const T open = T(1.) - tildeP;
            const T ratio = open > T(0) ? open * dt * exp(-logTv) : T(0);
            multiplicator = T(1) / (T(1) + ratio);
        }
        const T elasticity = hG * static_cast<T>(p.young) * dG * expC;
        const T Dunit_factor = dt * elasticity / (T(1.) - (nu0 * nu0));
        g11 += Dunit_factor * (e11 + nu0 * e22);
        g22 += Dunit_factor * (nu0 * e11 + e22);
        g12 += Dunit_factor * e12 * (T(1.) - nu0);
        g11 *= multiplicator;
        g22 *= multiplicator;
        g12 *= multiplicator;
        sigma_n = T(0.5) * (g11 + g22);
        const T dd = g11 - g22;
        const T tau = sqrt(T(0.25) * (dd * dd) + g12 * g12);
        const T tan_phi = static_cast<T>(p.tan_phi);
        const T cohesion = static_cast<T>(p.C_lab) * scale_coef * hG;
        const T compr = static_cast<T>(p.compr_strength) * scale_coef * hG;
        T dcrit = (tau + tan_phi * sigma_n > T(0)) ? cohesion / (tau + tan_phi * sigma_n) : T(1.);
        dcrit = (sigma_n < -compr) ? -compr / sigma_n : dcrit;
        dcrit = fmin(dcrit, T(1.0));
        const T td = tdScale / sqrt(elasticity);
        const T relax = (T(1.) - dcrit) * dt / td;
        dG -= dG * relax;
        g11 -= g11 * relax;
        g12 -= g12 * relax;
        g22 -= g22 * relax;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const T wk = AFF ? T(cBbmAff.w[k * 9 + q]) : o.w[(k * 9 + q) * N + e];
            n11[k] = fma(wk, g11, n11[k]);
            n12[k] = fma(wk, g12, n12[k]);
            n22[k] = fma(wk, g22, n22[k]);
        }
#pragma unroll
        for (int k = 0; k < DG; ++k)
            nd[k] = fma(AFF ? T(cBbmAff.wdam[k * 9 + q]) : o.wdam[(k * 9 + q) * N + e], dG, nd[k]);
    }
    bool finite = true;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        s11[k * N + e] = n11[k];
        s12[k * N + e] = n12[k];
        s22[k * N + e] = n22[k];
        finite = finite && isfinite(n11[k]) && isfinite(n12[k]) && isfinite(n22[k]);
    }
#pragma unroll
    for (int k = 0; k < DG; ++k)
        damage[k * N + e] = nd[k];
    if (!finite)
        atomicOr(err, DEV_ERR_NONFINITE_STRESS);
    if constexpr (AFF) {
        // divS1 n11 + divS2 n12 = D_xi (c0 n11 + c2 n12) + D_eta (c1 n11 + c3 n12),
        // divS1 n12 + divS2 n22 likewise
        T ax[8], bx[8], ay[8], by[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            ax[k] = fmaf(cf[0], n11[k], cf[2] * n12[k]);
            bx[k] = fmaf(cf[1], n11[k], cf[3] * n12[k]);
            ay[k] = fmaf(cf[0], n12[k], cf[2] * n22[k]);
            by[k] = fmaf(cf[1], n12[k], cf[3] * n22[k]);
        }
#pragma unroll 1
        for (int j = 0; j < 9; ++j) {
            T tx = T(0), ty = T(0);
            if (ice) {
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const float dxi = cBbmAff.dxi[j * 8 + k], deta = cBbmAff.deta[j * 8 + k];
                    tx = fmaf(dxi, ax[k], fmaf(deta, bx[k], tx));
                    ty = fmaf(dxi, ay[k], fmaf(deta, by[k], ty));
                }
            }
            contrib[j * N + e] = tx;
            contrib[(9 + j) * N + e] = ty;
        }
        return;
    }
#pragma unroll 1
    for (int j = 0; j < 9; ++j) {
        T tx = T(0), ty = T(0);
        if (ice) {
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const T d1 = o.d1[(j * 8 + k) * N + e];
                const T d2v = o.d2[(j * 8 + k) * N + e];
                tx = fma(d1, n11[k], fma(d2v, n12[k], tx));
                ty = fma(d1, n12[k], fma(d2v, n22[k], ty));
                if (o.dm) { // spherical: +divM s12, -divM s11 (CGDynamicsKernel.cpp:348-351)
                    const T dmv = o.dm[(j * 8 + k) * N + e];
                    tx = fma(dmv, n12[k], tx);
                    ty = fma(-dmv, n11[k], ty);
                }
            }
        }
        contrib[j * N + e] = tx;
        contrib[(9 + j) * N + e] = ty;
    }
}

// BBM momentum per CG2 node.  T = double is the reference's arithmetic; T =
// float is the mixed-precision kernel: FP32 arithmetic on the FP64 state, the
// inverse lumped mass as a hi/lo float pair, the sub-step averages of the
// velocity accumulated in FP64.
template <typename T>
__global__ void __launch_bounds__(kBlock) kBbmMomentum(DevMesh m, DevOps o, BbmNodeState st,
    const double* __restrict__ contrib, BbmParams p, int* __restrict__ err, const float2* __restrict__ invmHL)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= m.Ncg)
        return;
    const int s2 = 2 * m.nx + 1;
    const int i2 = static_cast<int>(static_cast<unsigned>(i) % static_cast<unsigned>(s2)), j2 = static_cast<int>(static_cast<unsigned>(i) / static_cast<unsigned>(s2));
    const bool dir = m.cg2Dir[i] != 0;
    double dSx = 0.0, dSy = 0.0;
    if (!dir)
        gatherDivergence(m, i2, j2, contrib, dSx, dSy);
    const T H = static_cast<T>(st.cgH[i]), A = static_cast<T>(st.cgA[i]);
    const T dt = static_cast<T>(p.dt), rho = static_cast<T>(p.rho_ice);
    const T cosA = static_cast<T>(p.cosA), sinA = static_cast<T>(p.sinA);
    const T dteOverMass = dt / (rho * H);
    const T uIce = static_cast<T>(st.u[i]), vIce = static_cast<T>(st.v[i]);
    const T uo = static_cast<T>(st.uo[i]), vo = static_cast<T>(st.vo[i]);
    const T ua = static_cast<T>(st.ua[i]), va = static_cast<T>(st.va[i]);
    const T cPrime = A * static_cast<T>(p.F_ocean) * hypot(uo - uIce, vo - vIce);
    const T alpha = 1 + dteOverMass * (cPrime * cosA);
    const T beta = dt * static_cast<T>(p.fc) + dteOverMass * cPrime * sinA;
    const T rDenom = 1 / (alpha * alpha + beta * beta);
    const T dragAtm = A * static_cast<T>(p.F_atm) * hypot(ua, va);
    const T tauX = dragAtm * ua + cPrime * (uo * cosA - vo * sinA);
    const T tauY = dragAtm * va + cPrime * (vo * cosA + uo * sinA);
    T gradX, gradY;
    if constexpr (sizeof(T) == 8) {
        const double invm = o.invm2[i];
        gradX = dSx * invm - p.rho_ice * H * p.gravity * st.uGrad[i];
        gradY = dSy * invm - p.rho_ice * H * p.gravity * st.vGrad[i];
    } else {
        const float2 im = invmHL[i];
        const float fx = static_cast<float>(dSx), fy = static_cast<float>(dSy);
        const float rhoHg = rho * H * static_cast<float>(p.gravity);
        gradX = fmaf(fx, im.y, fx * im.x) - rhoHg * static_cast<float>(st.uGrad[i]);
        gradY = fmaf(fy, im.y, fy * im.x) - rhoHg * static_cast<float>(st.vGrad[i]);
    }
    T un = alpha * uIce + beta * vIce + dteOverMass * (alpha * (gradX + tauX) + beta * (gradY + tauY));
    un *= rDenom;
    T vn = alpha * vIce - beta * uIce + dteOverMass * (alpha * (gradY + tauY) + beta * (gradX + tauX));
    vn *= rDenom;
    if (!isfinite(un) || !isfinite(vn))
        atomicOr(err, DEV_ERR_NONFINITE_VELOCITY);
    if constexpr (sizeof(T) == 8) {
        st.avgU[i] += un / p.nSteps;
        st.avgV[i] += vn / p.nSteps;
    } else {
        const double invSteps = 1.0 / p.nSteps;
        st.avgU[i] += static_cast<double>(un) * invSteps;
        st.avgV[i] += static_cast<double>(vn) * invSteps;
    }
    if (dir) {
        un = T(0);
        vn = T(0);
    }
    st.u[i] = un;
    st.v[i] = vn;
}

// ===========================================================================
// Misc
// ===========================================================================
__global__ void kIceOceanStress(size_t n, int brittle, const double* __restrict__ u,
    const double* __restrict__ v, const double* __restrict__ uo, const double* __restrict__ vo,
    double Fo, double ca, double sa, double* __restrict__ tx, double* __restrict__ ty)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    if (!brittle) {
        const double ur = u[i] - uo[i], vr = v[i] - vo[i];
        const double a = sqrt(ur * ur + vr * vr);
        tx[i] = Fo * a * ur;
        ty[i] = Fo * a * vr;
    } else {
        const double ur = uo[i] - u[i], vr = vo[i] - v[i];
        const double cp = Fo * hypot(ur, vr);
        tx[i] = cp * (ur * ca - vr * sa);
        ty[i] = cp * (vr * ca + ur * sa);
    }
}

__global__ void kAosToSoa(size_t N, int nin, int dg, const double* __restrict__ aos, double* __restrict__ soa)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= N)
        return;
    if (nin == dg) {
        for (int j = 0; j < dg; ++j)
            soa[j * N + e] = aos[e * dg + j];
    } else {
        soa[e] = aos[e * nin];
        for (int j = 1; j < dg; ++j)
            soa[j * N + e] = 0.0;
    }
}
__global__ void kSoaToAos(size_t N, int dg, int nout, const double* __restrict__ soa, double* __restrict__ aos)
{
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (e >= N)
        return;
    for (int j = 0; j < nout; ++j)
        aos[e * nout + j] = soa[j * N + e];
}

// Per-element masses summed by a fixed-shape tree: warp shuffles, then the
// block's warps, then one block over the per-block partials.
template <int DG>
__global__ void __launch_bounds__(256) kMeanValuePartial(size_t N, const double* __restrict__ phi,
    const double* __restrict__ jw3, double* __restrict__ partials)
{
    __shared__ double ws[8];
    const size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    double s = 0.0;
    if (e < N) {
        double c[DG];
        loadCell<DG>(phi, N, e, c);
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            double v = 0.0;
#pragma unroll
            for (int j = 0; j < DG; ++j)
                v += c[j] * cT.psi[3][j][q];
            s += v * jw3[q * N + e];
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < 8 ? ws[threadIdx.x] : 0.0;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
            t += __shfl_down_sync(0xffffffffu, t, off);
        if (threadIdx.x == 0)
            partials[blockIdx.x] = t;
    }
}
__global__ void __launch_bounds__(1024) kReduceFinal(size_t n, const double* __restrict__ partials, double* __restrict__ out)
{
    __shared__ double ws[32];
    double s = 0.0;
    for (size_t i = threadIdx.x; i < n; i += blockDim.x)
        s += partials[i];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
        s += __shfl_down_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0)
        ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = ws[threadIdx.x];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1)
            t += __shfl_down_sync(0xffffffffu, t, off);
        if (threadIdx.x == 0)
            *out = t;
    }
}

} // namespace

// ===========================================================================
// Launchers
// ===========================================================================
#define NSDG_DG_SWITCH(dg, CALL)                                                                  \
    switch (dg) {                                                                                  \
    case 1: { constexpr int D = 1; CALL; } break;                                                  \
    case 3: { constexpr int D = 3; CALL; } break;                                                  \
    case 6: { constexpr int D = 6; CALL; } break;                                                  \
    case 8: { constexpr int D = 8; CALL; } break;                                                  \
    default: return cudaErrorInvalidValue;                                                         \
    }

cudaError_t launchCG2DG(cudaStream_t s, const DevMesh& m, int dg, const double* jw, const double* minv,
    int nf, const double* const* cg, double* const* out)
{
    const unsigned g = blocksFor(m.N);
    if (nf == 1) {
        NSDG_DG_SWITCH(dg, (kCG2DG<D, 1><<<g, kBlock, 0, s>>>(m.nx, m.N, jw, minv, cg[0], nullptr, out[0], nullptr)));
    } else {
        NSDG_DG_SWITCH(dg, (kCG2DG<D, 2><<<g, kBlock, 0, s>>>(m.nx, m.N, jw, minv, cg[0], cg[1], out[0], out[1])));
    }
    return cudaGetLastError();
}

cudaError_t launchCG2DG32(cudaStream_t s, const DevMesh& m, int dg, const float* jw32, const double* minv,
    const double* const* cg, double* const* out, const double* minvDiag)
{
    const unsigned g = blocksFor(m.N);
    if (minvDiag) {
        NSDG_DG_SWITCH(dg, (kCG2DG32<D, 2, true><<<g, kBlock, 0, s>>>(m.nx, m.N, jw32, minvDiag, cg[0], cg[1],
                                                                       out[0], out[1])));
    } else {
        NSDG_DG_SWITCH(dg, (kCG2DG32<D, 2, false><<<g, kBlock, 0, s>>>(m.nx, m.N, jw32, minv, cg[0], cg[1],
                                                                        out[0], out[1])));
    }
    return cudaGetLastError();
}

cudaError_t launchCG2DG0(cudaStream_t s, const DevMesh& m, int dg, const double* jw, const float* jw32,
    const double* minv, const double* const* cg, double* const* out)
{
    const unsigned g = blocksFor(m.N);
    if (jw32) {
        NSDG_DG_SWITCH(dg, (kCG2DG0<D, true><<<g, kBlock, 0, s>>>(m.nx, m.N, nullptr, jw32, minv, cg[0], cg[1],
                                                                  out[0], out[1])));
    } else {
        NSDG_DG_SWITCH(dg, (kCG2DG0<D, false><<<g, kBlock, 0, s>>>(m.nx, m.N, jw, nullptr, minv, cg[0], cg[1],
                                                                   out[0], out[1])));
    }
    return cudaGetLastError();
}

cudaError_t launchNormalVelocity(cudaStream_t s, const DevMesh& m, int dg, const double* velx,
    const double* vely, double* nvX, double* nvY)
{
    const unsigned g = blocksFor(m.nXe + m.nYe);
    NSDG_DG_SWITCH(dg, (kNormalVelocity<D><<<g, kBlock, 0, s>>>(m, velx, vely, nvX, nvY)));
    return cudaGetLastError();
}

cudaError_t launchTransportStage(cudaStream_t s, const DevMesh& m, int dg, const double* cellX,
    const double* cellY, const double* minv, const double* velx, const double* vely,
    const double* nvX, const double* nvY, int mode, double dt, const StageFields& f, const float* cellX32,
    const float* cellY32)
{
    TransportArgs a { m, cellX, cellY, minv, velx, vely, nvX, nvY, dt, mode, cellX32, cellY32 };
    const unsigned g = blocksFor(m.N);
    if (cellX32 && cellY32) {
        switch (f.nf) {
        case 1: NSDG_DG_SWITCH(dg, (kTransportStage<D, 1, float><<<g, kBlock, 0, s>>>(a, f))); break;
        case 2: NSDG_DG_SWITCH(dg, (kTransportStage<D, 2, float><<<g, kBlock, 0, s>>>(a, f))); break;
        case 3: NSDG_DG_SWITCH(dg, (kTransportStage<D, 3, float><<<g, kBlock, 0, s>>>(a, f))); break;
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    switch (f.nf) {
    case 1: NSDG_DG_SWITCH(dg, (kTransportStage<D, 1, double><<<g, kBlock, 0, s>>>(a, f))); break;
    case 2: NSDG_DG_SWITCH(dg, (kTransportStage<D, 2, double><<<g, kBlock, 0, s>>>(a, f))); break;
    case 3: NSDG_DG_SWITCH(dg, (kTransportStage<D, 3, double><<<g, kBlock, 0, s>>>(a, f))); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t uploadAffineTransportReference(int dg, const double ref[2][8 * 16])
{
    if (dg == 1)
        return cudaSuccess;
    if (dg != 3 && dg != 6)
        return cudaErrorInvalidValue;
    const int Q = dg == 6 ? 3 : 2, QQ = Q * Q;
    if (dg == 6) {
        float h[2][6][9];
        for (int b = 0; b < 2; ++b)
            for (int i = 0; i < 6; ++i)
                for (int q = 0; q < QQ; ++q)
                    h[b][i][q] = static_cast<float>(ref[b][i * QQ + q]);
        return cudaMemcpyToSymbol(cTrAff, h, sizeof(h), offsetof(AffTransportTables, u6));
    }
    float h[2][3][4];
    for (int b = 0; b < 2; ++b)
        for (int i = 0; i < 3; ++i)
            for (int q = 0; q < QQ; ++q)
                h[b][i][q] = static_cast<float>(ref[b][i * QQ + q]);
    return cudaMemcpyToSymbol(cTrAff, h, sizeof(h), offsetof(AffTransportTables, u3));
}

cudaError_t launchTransportStageAffine(cudaStream_t s, const DevMesh& m, int dg, const float* coef, size_t ld,
    const double* minvDiag, const double* velx, const double* vely, const double* nvX, const double* nvY,
    int mode, double dt, const StageFields& f)
{
    TransportAffArgs a { m, coef, ld, minvDiag, velx, vely, nvX, nvY, dt, mode };
    const dim3 g((m.nx + kTrX - 1) / kTrX, (m.ny + kTrY - 1) / kTrY), b(kTrX, kTrY);
    if (m.nx <= 0 || m.ny <= 0)
        return cudaSuccess;
#define NSDG_TR_AFF(D)                                                                     \
    switch (f.nf) {                                                                        \
    case 1: kTransportStageAffine<D, 1><<<g, b, 0, s>>>(a, f); break;                      \
    case 2: kTransportStageAffine<D, 2><<<g, b, 0, s>>>(a, f); break;                      \
    case 3: kTransportStageAffine<D, 3><<<g, b, 0, s>>>(a, f); break;                      \
    default: return cudaErrorInvalidValue;                                                 \
    }
    switch (dg) {
    case 1: NSDG_TR_AFF(1); break;
    case 3: NSDG_TR_AFF(3); break;
    case 6: NSDG_TR_AFF(6); break;
    default: return cudaErrorInvalidValue;
    }
#undef NSDG_TR_AFF
    return cudaGetLastError();
}

cudaError_t launchDG2CG(cudaStream_t s, const DevMesh& m, int dg, int nf, const double* const* dgIn,
    double* const* cgOut)
{
    const unsigned g = blocksFor(m.Ncg);
    if (nf == 1) {
        NSDG_DG_SWITCH(dg, (kDG2CG<D, 1><<<g, kBlock, 0, s>>>(m, dgIn[0], nullptr, cgOut[0], nullptr)));
    } else {
        NSDG_DG_SWITCH(dg, (kDG2CG<D, 2><<<g, kBlock, 0, s>>>(m, dgIn[0], dgIn[1], cgOut[0], cgOut[1])));
    }
    return cudaGetLastError();
}

cudaError_t launchSSHGradient(cudaStream_t s, const DevMesh& m, const DevOps& o, const double* ssh,
    double* scratch, double* uGrad, double* vGrad)
{
    double* cg1 = scratch;
    double* ug = scratch + m.Ncg1;
    double* vg = scratch + 2 * m.Ncg1;
    kSSHToCG1<<<blocksFor(m.Ncg1), kBlock, 0, s>>>(m, ssh, cg1);
    kSSHGrad1<<<blocksFor(m.Ncg1), kBlock, 0, s>>>(m, o, cg1, ug, vg);
    kSSHToCG2<<<blocksFor(m.Ncg), kBlock, 0, s>>>(m, ug, vg, uGrad, vGrad);
    return cudaGetLastError();
}

cudaError_t launchMevpPrepNodes(cudaStream_t s, const DevMesh& m, const MevpNodeState& st, const MevpParams& p)
{
    kMevpPrepNodes<<<blocksFor(m.Ncg), kBlock, 0, s>>>(m.Ncg, st, p);
    return cudaGetLastError();
}

cudaError_t launchMevpPrepElements(cudaStream_t s, const DevMesh& m, int dg, const double* h,
    const double* a, double* Pg, const MevpParams& p, float* hP32, const float* tdiv32, float* tdivLast)
{
    const unsigned g = blocksFor(m.N);
    const double ia = 1.0 / p.alpha;
    switch (dg) {
    case 1: kMevpPrepElements<1><<<g, kBlock, 0, s>>>(m.N, h, a, Pg, p.Pstar, ia, hP32, tdiv32, tdivLast); break;
    case 3: kMevpPrepElements<3><<<g, kBlock, 0, s>>>(m.N, h, a, Pg, p.Pstar, ia, hP32, tdiv32, tdivLast); break;
    case 6: kMevpPrepElements<6><<<g, kBlock, 0, s>>>(m.N, h, a, Pg, p.Pstar, ia, hP32, tdiv32, tdivLast); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launchMevpStress(cudaStream_t s, const DevMesh& m, const DevOps& o, const double* u,
    const double* v, const double* Pg, double* tdiv, const MevpParams& pIn)
{
    const MevpParams p = withDerived(pIn);
    if (o.gm)
        kMevpStress<true><<<blocksFor(m.N, kStressElems), kStressElems * kStressParts, 0, s>>>(m, o, u, v, Pg, tdiv, p);
    else
        kMevpStress<false><<<blocksFor(m.N, kStressElems), kStressElems * kStressParts, 0, s>>>(m, o, u, v, Pg, tdiv, p);
    return cudaGetLastError();
}

cudaError_t launchMevpMomentum(cudaStream_t s, const DevMesh& m, const DevOps& o, const MevpNodeState& st,
    const double* contrib, const MevpParams& p, int* err)
{
    kMevpMomentum<<<blocksFor(m.Ncg), kBlock, 0, s>>>(m, o, st, contrib, p, err);
    return cudaGetLastError();
}

cudaError_t launchMevpPrepNodes32(cudaStream_t s, const DevMesh& m, const MevpNodeState& st64,
    const MevpNodeState32& st32, const double* invm2, const MevpParams& p, float* uLast, float* vLast)
{
    kMevpPrepNodes32<<<blocksFor(m.Ncg), kBlock, 0, s>>>(m.Ncg, st64, st32, invm2, m.cg2Dir, p, uLast, vLast);
    return cudaGetLastError();
}
namespace {
template <bool SPH> constexpr size_t tmaSmem() { return size_t(tmaTileBytes<SPH>()) + 3 * 9 * kTmaElems * 4 + 2 * 8; }
constexpr size_t kTmaSmem = tmaSmem<false>();
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
    CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
} // namespace

cudaError_t launchBoundedWaitSelfTest(cudaStream_t s, double limitSeconds, int* timedOut)
{
    const double ns = limitSeconds * 1e9;
    kBoundedWaitSelfTest<<<1, 32, 0, s>>>(static_cast<unsigned long long>(ns < 0 ? 0 : ns), timedOut);
    return cudaGetLastError();
}

namespace {
EncodeTiledFn encodeTiledFn(cudaError_t& e)
{
    static EncodeTiledFn encode = nullptr;
    e = cudaSuccess;
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        e = cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q);
        if (e == cudaSuccess && (q != cudaDriverEntryPointSuccess || !fn))
            e = cudaErrorNotSupported;
        if (e == cudaSuccess)
            encode = reinterpret_cast<EncodeTiledFn>(fn);
    }
    return encode;
}
} // namespace

cudaError_t encodeTiled2d(CUtensorMap* map, CUtensorMapDataType type, const void* base, uint64_t inner,
    uint64_t outer, uint64_t rowBytes, uint32_t boxInner, uint32_t boxOuter)
{
    cudaError_t e;
    const EncodeTiledFn encode = encodeTiledFn(e);
    if (!encode)
        return e;
    const cuuint64_t dims[2] = { inner, outer };
    const cuuint64_t strides[1] = { rowBytes };
    const cuuint32_t box[2] = { boxInner, boxOuter };
    const cuuint32_t estr[2] = { 1, 1 };
    const CUresult r = encode(map, type, 2, const_cast<void*>(base), dims, strides, box, estr,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t encodeTiledNd(CUtensorMap* map, CUtensorMapDataType type, const void* base, int rank,
    const uint64_t* dims, const uint64_t* strideBytes, const uint32_t* box)
{
    cudaError_t e;
    const EncodeTiledFn encode = encodeTiledFn(e);
    if (!encode)
        return e;
    if (rank < 1 || rank > 5)
        return cudaErrorInvalidValue;
    cuuint64_t d[5], st[4];
    cuuint32_t b[5], es[5];
    for (int i = 0; i < rank; ++i) {
        d[i] = dims[i];
        b[i] = box[i];
        es[i] = 1;
        if (i + 1 < rank)
            st[i] = strideBytes[i];
    }
    const CUresult r = encode(map, type, static_cast<cuuint32_t>(rank), const_cast<void*>(base), d, st, b, es,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t makeStressMaps(const DevOps32& o, StressMaps* out)
{
    cudaError_t ee;
    const EncodeTiledFn encode = encodeTiledFn(ee);
    if (!encode)
        return ee;
    // the four operator blocks are rows of one [324][ld] array; ld * 4 bytes
    // is a multiple of 128 and the base is 256-byte aligned
    const cuuint64_t dims[2] = { o.ld, static_cast<cuuint64_t>(o.rowsG) };
    const cuuint64_t strides[1] = { o.ld * sizeof(float) };
    const cuuint32_t box[2] = { kTmaElems, static_cast<cuuint32_t>(o.rowsG) };
    const cuuint32_t estr[2] = { 1, 1 };
    const float* rows[2] = { o.gx, o.a1 };
    CUtensorMap* maps[2] = { &out->g, &out->a };
    for (int i = 0; i < 2; ++i) {
        const CUresult r = encode(maps[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(rows[i]), dims,
            strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS)
            return cudaErrorInvalidValue;
    }
    // dynamic shared memory of the kernel (24 KB: one operator tile, the
    // stress terms, two mbarriers), set once
    cudaError_t e = cudaFuncSetAttribute(kMevpStress32Tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        static_cast<int>(tmaSmem<false>()));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kMevpStress32Tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
            static_cast<int>(tmaSmem<true>()));
    return e != cudaSuccess ? e
                            : cudaFuncSetAttribute(kMevpStress32TmaBatched,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(kTmaSmem));
}

cudaError_t launchMevpStress32Tma(cudaStream_t s, const DevMesh& m, const StressMaps& maps, const float* u,
    const float* v, const double* Pg, const float* hP, float* tdiv, const MevpParams& pIn, int* err)
{
    const MevpParams p = withDerived(pIn);
    cudaLaunchConfig_t cfg {};
    cfg.gridDim = dim3(blocksFor(m.N, kTmaElems));
    cfg.blockDim = dim3(kTmaElems * kStressParts);
    cfg.dynamicSmemBytes = m.spherical ? tmaSmem<true>() : tmaSmem<false>();
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (m.spherical)
        return cudaLaunchKernelEx(&cfg, kMevpStress32Tma<true>, maps.g, maps.a, m, u, v, Pg, hP, tdiv, p, err);
    return cudaLaunchKernelEx(&cfg, kMevpStress32Tma<false>, maps.g, maps.a, m, u, v, Pg, hP, tdiv, p, err);
}

cudaError_t uploadAffineBbmReference(const double* w, const double* wdam, int dg, const double* dxi,
    const double* deta)
{
    BbmAffTables t {};
    for (int r = 0; r < 72; ++r) {
        t.w[r] = static_cast<float>(w[r]);
        t.dxi[r] = static_cast<float>(dxi[r]);
        t.deta[r] = static_cast<float>(deta[r]);
    }
    for (int r = 0; r < dg * 9 && r < 72; ++r)
        t.wdam[r] = static_cast<float>(wdam[r]);
    return cudaMemcpyToSymbol(cBbmAff, &t, sizeof(t));
}

cudaError_t uploadAffineReference(const double ref[4][81])
{
    float h[4][81];
    for (int b = 0; b < 4; ++b)
        for (int r = 0; r < 81; ++r)
            h[b][r] = static_cast<float>(ref[b][r]);
    return cudaMemcpyToSymbol(cAff, h, sizeof(h));
}

cudaError_t launchMevpStress32Affine(cudaStream_t s, const DevMesh& m, const float* coef, size_t ld, const float* u,
    const float* v, const double* Pg, float* tdiv, const MevpParams& pIn, int viscosityMode)
{
    const MevpParams p = withDerived(pIn);
    cudaLaunchConfig_t cfg {};
    cfg.gridDim = dim3(blocksFor(m.N, kAffElems));
    cfg.blockDim = dim3(kAffElems * kStressParts);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    switch (viscosityMode) {
    case 0: return cudaLaunchKernelEx(&cfg, kMevpStress32Affine<0>, m, coef, ld, u, v, Pg, tdiv, p);
    case 1: return cudaLaunchKernelEx(&cfg, kMevpStress32Affine<1>, m, coef, ld, u, v, Pg, tdiv, p);
    case 3: return cudaLaunchKernelEx(&cfg, kMevpStress32Affine<3>, m, coef, ld, u, v, Pg, tdiv, p);
    case 4: return cudaLaunchKernelEx(&cfg, kMevpStress32Affine<4>, m, coef, ld, u, v, Pg, tdiv, p);
    default: return cudaLaunchKernelEx(&cfg, kMevpStress32Affine<2>, m, coef, ld, u, v, Pg, tdiv, p);
    }
}

cudaError_t launchViscositySelfTest(cudaStream_t s, size_t n, const float* inv, const double* Pa, double dmin,
    float* out)
{
    kViscositySelfTest<<<blocksFor(n), kBlock, 0, s>>>(n, inv, Pa, dmin, out);
    return cudaGetLastError();
}

cudaError_t launchViscositySelfTestFF(cudaStream_t s, size_t n, const float* inv, const double* Pa, double dmin,
    float* out)
{
    kViscositySelfTestFF<<<blocksFor(n), kBlock, 0, s>>>(n, inv, Pa, dmin, out);
    return cudaGetLastError();
}

cudaError_t launchViscositySelfTestChecked(cudaStream_t s, size_t n, const float* inv, const double* Pa,
    double dmin, float* out)
{
    kViscositySelfTestChecked<<<blocksFor(n), kBlock, 0, s>>>(n, inv, Pa, dmin, out);
    return cudaGetLastError();
}

cudaError_t launchMevpStress32(cudaStream_t s, const DevMesh& m, const DevOps32& o, const float* u,
    const float* v, const double* Pg, const float* hP, float* tdiv, const MevpParams& pIn)
{
    const MevpParams p = withDerived(pIn);
    kMevpStress32<<<blocksFor(m.N, kStressElems), kStressElems * kStressParts, 0, s>>>(m, o, u, v, Pg, hP, tdiv, p);
    return cudaGetLastError();
}
cudaError_t launchMevpMomentum32(cudaStream_t s, const DevMesh& m, const MevpNodeState32& st,
    const float* tdiv, const MevpParams& pIn, int* err)
{
    const MevpParams p = withDerived(pIn);
    cudaLaunchConfig_t cfg {};
    cfg.gridDim = dim3(blocksFor(m.Ncg));
    cfg.blockDim = dim3(kBlock);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kMevpMomentum32, m, st, tdiv, p, err);
}
cudaError_t launchMevpStress32Batched(cudaStream_t s, const EnsembleMember* members, const uint16_t* blockMember,
    int blocks, const MevpParams& pIn)
{
    const MevpParams p = withDerived(pIn);
    kMevpStress32Batched<<<blocks, kStressElems * kStressParts, 0, s>>>(members, blockMember, p);
    return cudaGetLastError();
}
cudaError_t launchMevpMomentum32Batched(cudaStream_t s, const EnsembleMember* members, const uint16_t* blockMember,
    int blocks, const MevpParams& pIn, int* err)
{
    const MevpParams p = withDerived(pIn);
    cudaLaunchConfig_t cfg {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kBlock);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kMevpMomentum32Batched, members, blockMember, p, err);
}
cudaError_t launchMevpStress32TmaBatched(cudaStream_t s, const EnsembleMember* members, const uint16_t* blockMember,
    int blocks, const MevpParams& pIn, int* err)
{
    const MevpParams p = withDerived(pIn);
    cudaLaunchConfig_t cfg {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kTmaElems * kStressParts);
    cfg.dynamicSmemBytes = kTmaSmem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kMevpStress32TmaBatched, members, blockMember, p, err);
}
cudaError_t launchMevpStress32AffineBatched(cudaStream_t s, const EnsembleMember* members,
    const uint16_t* blockMember, int blocks, const MevpParams& pIn, int viscosityMode)
{
    const MevpParams p = withDerived(pIn);
    static_assert(kAffElems == kTmaElems, "the parallelogram and TMA kernels share the block map");
    cudaLaunchConfig_t cfg {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(kAffElems * kStressParts);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    switch (viscosityMode) {
    case 0: return cudaLaunchKernelEx(&cfg, kMevpStress32AffineBatched<0>, members, blockMember, p);
    case 1: return cudaLaunchKernelEx(&cfg, kMevpStress32AffineBatched<1>, members, blockMember, p);
    case 4: return cudaLaunchKernelEx(&cfg, kMevpStress32AffineBatched<4>, members, blockMember, p);
    default: return cudaLaunchKernelEx(&cfg, kMevpStress32AffineBatched<2>, members, blockMember, p);
    }
}
int persistentNodesPerBlock() { return kAffElems * kStressParts; }

cudaError_t launchEnsembleSubcyclePersistent(cudaStream_t s, const EnsembleMember* members, const uint16_t* elemMap,
    int elemBlocks, const uint16_t* nodeMap, int nodeBlocks, const MevpParams& pIn, int viscosityMode,
    int iterations, unsigned* bar, int* err)
{
    const MevpParams p = withDerived(pIn);
    int dev = 0, sms = 0, perSm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto kern = viscosityMode == 0 ? kEnsembleSubcyclePersistent<0>
        : viscosityMode == 1 ? kEnsembleSubcyclePersistent<1>
        : viscosityMode == 4 ? kEnsembleSubcyclePersistent<4> : kEnsembleSubcyclePersistent<2>;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, kern, kAffElems * kStressParts, 0);
    if (e != cudaSuccess)
        return e;
    if (perSm < 1)
        return cudaErrorInvalidConfiguration;
    // every block resident at once (the cooperative launch enforces it), and
    // no more blocks than the larger phase has work blocks
    const int grid = std::max(1, std::min(perSm * sms, std::max(elemBlocks, nodeBlocks)));
    e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned), s);
    if (e != cudaSuccess)
        return e;
    cudaLaunchConfig_t cfg {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kAffElems * kStressParts);
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, members, elemMap, elemBlocks, nodeMap, nodeBlocks, p, iterations, bar, err);
}

int stressElementsPerBlock() { return kStressElems; }
int nodesPerBlock() { return kBlock; }

cudaError_t launchWidenVelocity(cudaStream_t s, size_t n, const float* u32, const float* v32, double* u, double* v)
{
    kWidenVelocity<<<blocksFor(n), kBlock, 0, s>>>(n, u32, v32, u, v);
    return cudaGetLastError();
}

cudaError_t launchIceOceanStress(cudaStream_t s, size_t n, int brittle, const double* u, const double* v,
    const double* uo, const double* vo, double F_ocean, double cosA, double sinA, double* tx, double* ty,
    bool fp32)
{
    if (fp32)
        kIceOceanStress32<<<blocksFor(n), kBlock, 0, s>>>(n, brittle, u, v, uo, vo, static_cast<float>(F_ocean),
            static_cast<float>(cosA), static_cast<float>(sinA), tx, ty);
    else
        kIceOceanStress<<<blocksFor(n), kBlock, 0, s>>>(n, brittle, u, v, uo, vo, F_ocean, cosA, sinA, tx, ty);
    return cudaGetLastError();
}

cudaError_t launchBbmPrepNodes(cudaStream_t s, const DevMesh& m, const BbmNodeState& st, const BbmParams* p,
    const BbmNodeConst32* c)
{
    const BbmNodeConst32 none { nullptr, nullptr };
    kBbmPrepNodes<<<blocksFor(m.Ncg), kBlock, 0, s>>>(m.Ncg, st, p ? *p : BbmParams {}, (c && p) ? *c : none);
    return cudaGetLastError();
}

cudaError_t launchBbmStress(cudaStream_t s, const DevMesh& m, const DevOps& o, int dg, const double* u,
    const double* v, const double* h, const double* a, double* damage, double* s11, double* s12,
    double* s22, double* contrib, const BbmParams& p, int* err, const BbmOps32* o32)
{
    const unsigned g = blocksFor(m.N);
    if (o32 && o32->coef) {
        BbmOps<float> of { o32->gx, o32->gy, o32->w, o32->wdam, o32->d1, o32->d2, o.hsize, o32->gm, o32->dm };
        of.coef = o32->coef;
        of.ld = o32->ld;
        switch (dg) {
        case 1: kBbmStress<1, float, true><<<g, kBlock, 0, s>>>(m, of, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
        case 3: kBbmStress<3, float, true><<<g, kBlock, 0, s>>>(m, of, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
        case 6: kBbmStress<6, float, true><<<g, kBlock, 0, s>>>(m, of, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    if (o32) {
        const BbmOps<float> of { o32->gx, o32->gy, o32->w, o32->wdam, o32->d1, o32->d2, o.hsize, o32->gm, o32->dm };
        switch (dg) {
        case 1: kBbmStress<1, float><<<g, kBlock, 0, s>>>(m, of, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
        case 3: kBbmStress<3, float><<<g, kBlock, 0, s>>>(m, of, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
        case 6: kBbmStress<6, float><<<g, kBlock, 0, s>>>(m, of, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
        default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }
    const BbmOps<double> od { o.gx, o.gy, o.w, o.wdam, o.d1, o.d2, o.hsize, o.gm, o.dm };
    switch (dg) {
    case 1: kBbmStress<1, double><<<g, kBlock, 0, s>>>(m, od, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
    case 3: kBbmStress<3, double><<<g, kBlock, 0, s>>>(m, od, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
    case 6: kBbmStress<6, double><<<g, kBlock, 0, s>>>(m, od, u, v, h, a, damage, s11, s12, s22, contrib, p, err); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launchBbmMomentum(cudaStream_t s, const DevMesh& m, const DevOps& o, const BbmNodeState& st,
    const double* contrib, const BbmParams& p, int* err, const float2* invmHL, const BbmNodeConst32* c)
{
    if (invmHL && c && c->k0)
        kBbmMomentum32<<<blocksFor(m.Ncg), kBlock, 0, s>>>(m, st, *c, contrib, p, err, invmHL);
    else if (invmHL)
        kBbmMomentum<float><<<blocksFor(m.Ncg), kBlock, 0, s>>>(m, o, st, contrib, p, err, invmHL);
    else
        kBbmMomentum<double><<<blocksFor(m.Ncg), kBlock, 0, s>>>(m, o, st, contrib, p, err, nullptr);
    return cudaGetLastError();
}

// Up to kHostMoves arrays moved by one grid-stride kernel: on a GPU that
// reads and writes pageable host memory directly (Grace: address translation
// over the CPU-GPU link), one kernel over all of a call's host arrays moves
// them at the link's rate, where a copy from or to pageable memory is staged
// through a driver buffer.
__global__ void __launch_bounds__(256) kHostMove(HostMoves m)
{
    unsigned long long total = 0;
    for (int f = 0; f < m.count; ++f)
        total += m.n[f];
    for (unsigned long long i = blockIdx.x * 256ull + threadIdx.x; i < total; i += gridDim.x * 256ull) {
        unsigned long long off = i;
        int f = 0;
        while (f < m.count - 1 && off >= m.n[f]) {
            off -= m.n[f];
            ++f;
        }
        m.dst[f][off] = m.src[f][off];
    }
}

cudaError_t launchHostMove(cudaStream_t s, const HostMoves& m)
{
    if (m.count <= 0)
        return cudaSuccess;
    if (m.count > kHostMoves)
        return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess)
        return e;
    kHostMove<<<static_cast<unsigned>(4 * sms), 256, 0, s>>>(m);
    return cudaGetLastError();
}

cudaError_t launchAosToSoa(cudaStream_t s, size_t N, int nin, int dg, const double* aos, double* soa)
{
    kAosToSoa<<<blocksFor(N), kBlock, 0, s>>>(N, nin, dg, aos, soa);
    return cudaGetLastError();
}
cudaError_t launchSoaToAos(cudaStream_t s, size_t N, int dg, int nout, const double* soa, double* aos)
{
    kSoaToAos<<<blocksFor(N), kBlock, 0, s>>>(N, dg, nout, soa, aos);
    return cudaGetLastError();
}

cudaError_t launchMeanValue(cudaStream_t s, size_t N, int dg, const double* phi, const double* jw3,
    double* partials, double* out)
{
    const unsigned g = blocksFor(N, 256);
    NSDG_DG_SWITCH(dg, (kMeanValuePartial<D><<<g, 256, 0, s>>>(N, phi, jw3, partials)));
    kReduceFinal<<<1, 1024, 0, s>>>(g, partials, out);
    return cudaGetLastError();
}

} // namespace nsdg
