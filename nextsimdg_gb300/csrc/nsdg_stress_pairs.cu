// nsdg_stress_pairs.cu — the FP64 path's element stress kernel with its
// operator products in float-pair arithmetic (sm_103a).
//
// The same mEVP element step as kMevpStress (nsdg_kernels.cu): the strain at
// the 9 Gauss points from the 9 CG2 velocity nodes through G = psi^T iMgrad
// (CGDynamicsKernel.cpp:300-337), Delta, the ice strength term and the
// relaxed stress increments (MEVPStressUpdateStep.hpp:54-116), and the
// element's stress divergence coefficients tdiv = divS s at its 9 nodes
// (CGDynamicsKernel.cpp:340-363), carried in divergence space.
//
// In FP64 that is 648 FMA of operator products per element, and GB300 issues
// FP64 at about 2 FMA per SM per clock: kMevpStress is FP64-issue bound at
// about 0.3 of the HBM roofline.  Here the four 9 x 9 products, Delta^2 and
// the stress increments are formed in float pairs (nsdg_pairs.cuh: about 48
// significant bits, error-free products and sums on the FP32 pipe), and the
// FP64 pipe keeps what sets the accuracy of the nonlinear step: 1/Delta by two
// Newton steps in FP64 from an FP32 seed, P / (8 alpha Delta), and the
// divergence update tdiv <- (1 - 1/alpha) tdiv + A f, 18 FMA per element.
// Operators are stored as float pairs (hi = RN(x), lo = RN(x - hi)): the same
// 8 bytes per entry as FP64.  State, inputs and outputs stay FP64.
#include "nsdg_kernels.hpp"
#include "nsdg_pairs.cuh"

namespace nsdg {

namespace {

constexpr int kPairElems = 64;
constexpr int kPairParts = 3;

inline unsigned blocksOf(size_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

__global__ void kSplitPairs(size_t n, const double* __restrict__ src, float2* __restrict__ dst)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const double x = src[i];
    const float hi = __double2float_rn(x);
    dst[i] = make_float2(hi, __double2float_rn(x - static_cast<double>(hi)));
}

// Thread layout as kMevpStress: three threads per element, 64 elements per
// block; thread `part` forms the Gauss points 3 part .. 3 part + 2, then the
// divergence coefficients of nodes 3 part .. 3 part + 2.
__global__ void __launch_bounds__(kPairElems * kPairParts) kMevpStressPairs(DevMesh m,
    const float2* __restrict__ ops, const double* __restrict__ u, const double* __restrict__ v,
    const double* __restrict__ Pg, double* __restrict__ tdiv, MevpParams p)
{
    using namespace pairs;
    __shared__ float2 fs[3][9][kPairElems];
    const int le = threadIdx.x % kPairElems;
    const int part = threadIdx.x / kPairElems; // warp-uniform
    const size_t N = m.N;
    const size_t e = blockIdx.x * size_t(kPairElems) + le;
    const bool active = e < N && m.ice[e];
    const float2* __restrict__ gxo = ops;
    const float2* __restrict__ gyo = ops + 81 * N;
    const float2* __restrict__ a1o = ops + 162 * N;
    const float2* __restrict__ a2o = ops + 243 * N;
    if (active) {
        const unsigned s2 = 2u * static_cast<unsigned>(m.nx) + 1u;
        const unsigned ix = static_cast<unsigned>(e) % static_cast<unsigned>(m.nx);
        const unsigned iy = static_cast<unsigned>(e) / static_cast<unsigned>(m.nx);
        const unsigned base = 2u * s2 * iy + 2u * ix;
        F2 ul[9], vl[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const unsigned nd = base + unsigned(j % 3) + unsigned(j / 3) * s2;
            ul[j] = split(u[nd]);
            vl[j] = split(v[nd]);
        }
        const F2 dmin2 { p.dmin2f, p.dmin2lo };
#pragma unroll
        for (int qq = 0; qq < 3; ++qq) {
            const int q = 3 * part + qq;
            Acc ax, ay, axv, ayu;
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const F2 gx = pairOf(gxo[(q * 9 + j) * N + e]);
                const F2 gy = pairOf(gyo[(q * 9 + j) * N + e]);
                madd(ax, gx, ul[j]);
                madd(ay, gy, vl[j]);
                madd(axv, gx, vl[j]);
                madd(ayu, gy, ul[j]);
            }
            // e11 = ex, e22 = ey, e12 = sxy / 2
            const F2 ex = result(ax), ey = result(ay);
            const F2 sxy = add(result(axv), result(ayu));
            // Delta^2 = DeltaMin^2 + 1.25 (ex^2 + ey^2) + 1.5 ex ey + 0.25 sxy^2
            F2 d2 = mul(add(mul(ex, ex), mul(ey, ey)), 1.25f);
            d2 = add(d2, mul(mul(ex, ey), 1.5f));
            d2 = add(d2, scale2(mul(sxy, sxy), 0.25f));
            d2 = add(d2, dmin2);
            // 1/Delta: FP32 seed, two Newton steps in FP64 (y <- y (3 - t y^2) / 2)
            const double t = value(d2);
            double y = widen(rsqrtf(d2.hi));
            y = fma(y, fma(-0.5 * t * y, y, 0.5), y);
            y = fma(y, fma(-0.5 * t * y, y, 0.5), y);
            const double Pa = Pg[q * N + e];
            const F2 z8 = split(0.125 * Pa * y); // P / (8 alpha Delta)
            const F2 hP = scale2(split(Pa), 0.5f); // P / (2 alpha)
            // stress increments at the Gauss point (MEVPStressUpdateStep.hpp:92-116)
            const F2 r11 = add(mul(z8, add(mul(ex, 5.0f), mul(ey, 3.0f))), F2 { -hP.hi, -hP.lo });
            const F2 r12 = mul(z8, sxy);
            const F2 r22 = add(mul(z8, add(mul(ey, 5.0f), mul(ex, 3.0f))), F2 { -hP.hi, -hP.lo });
            fs[0][q][le] = make_float2(r11.hi, r11.lo);
            fs[1][q][le] = make_float2(r12.hi, r12.lo);
            fs[2][q][le] = make_float2(r22.hi, r22.lo);
        }
    }
    __syncthreads();
    if (!active)
        return;
    const double keep = p.keepd;
#pragma unroll
    for (int jj = 0; jj < 3; ++jj) {
        const int j = 3 * part + jj;
        Acc dx, dy;
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            const F2 a1 = pairOf(a1o[(j * 9 + q) * N + e]);
            const F2 a2 = pairOf(a2o[(j * 9 + q) * N + e]);
            const F2 f11 = pairOf(fs[0][q][le]), f12 = pairOf(fs[1][q][le]), f22 = pairOf(fs[2][q][le]);
            madd(dx, a1, f11);
            madd(dx, a2, f12);
            madd(dy, a1, f12);
            madd(dy, a2, f22);
        }
        tdiv[j * N + e] = fma(tdiv[j * N + e], keep, value(result(dx)));
        tdiv[(9 + j) * N + e] = fma(tdiv[(9 + j) * N + e], keep, value(result(dy)));
    }
}

// Checks of the pair arithmetic against FP64 on given inputs: for each i,
// out[4 i + 0..3] = value(split(x)) - x, widen of the float x rounded,
// value(a x) for the pairs of a and x, value(sum) of a 9-term dot product.
__global__ void kPairsSelfTest(size_t n, const double* __restrict__ a, const double* __restrict__ x,
    double* __restrict__ out)
{
    using namespace pairs;
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= n)
        return;
    const F2 sa = split(a[i]), sx = split(x[i]);
    out[4 * i + 0] = value(sa) - a[i];
    out[4 * i + 1] = widen(__double2float_rn(x[i]));
    out[4 * i + 2] = value(mul(sa, sx));
    Acc s;
    for (int k = 0; k < 9; ++k) {
        const size_t j = (i + 7 * size_t(k)) % n;
        madd(s, split(a[j]), split(x[j]));
    }
    out[4 * i + 3] = value(result(s));
}

} // namespace

cudaError_t launchSplitPairs(cudaStream_t s, size_t n, const double* src, float2* dst)
{
    if (n == 0)
        return cudaSuccess;
    kSplitPairs<<<blocksOf(n, 256), 256, 0, s>>>(n, src, dst);
    return cudaGetLastError();
}

cudaError_t launchMevpStressPairs(cudaStream_t s, const DevMesh& m, const float2* ops, const double* u,
    const double* v, const double* Pg, double* tdiv, const MevpParams& pIn)
{
    const MevpParams p = withDerived(pIn);
    kMevpStressPairs<<<blocksOf(m.N, kPairElems), kPairElems * kPairParts, 0, s>>>(m, ops, u, v, Pg, tdiv, p);
    return cudaGetLastError();
}

cudaError_t launchPairsSelfTest(cudaStream_t s, size_t n, const double* a, const double* x, double* out)
{
    kPairsSelfTest<<<blocksOf(n, 128), 128, 0, s>>>(n, a, x, out);
    return cudaGetLastError();
}

} // namespace nsdg
