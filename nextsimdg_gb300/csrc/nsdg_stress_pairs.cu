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
// 8 bytes per entry as FP64, in one [324][ld] array (rows G_x | G_y | A_1 |
// A_2, ld = N rounded up to 32).  State, inputs and outputs stay FP64.
//
// kMevpStressPairs reads the operators straight from global memory, and
// waits on memory latency: a warp has only a few loads outstanding.
// kMevpStressPairsTma stages each phase's operator rows for 32 elements
// (162 rows x 32 pairs = 41.5 KB) into shared memory with one TMA copy, so
// that four blocks per SM keep 166 KB of operator loads in flight; nine
// threads per element (one per Gauss point, then one per node) give those
// four blocks 36 warps, enough to keep the FP32 pipe issuing the long chains
// of dependent float-pair instructions.
#include "nsdg_kernels.hpp"
#include "nsdg_pairs.cuh"
#include "nsdg_tma.cuh"

namespace nsdg {

namespace {

constexpr int kPairElems = 64;
constexpr int kPairParts = 3;

inline unsigned blocksOf(size_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

// rows x n FP64 entries (rows n apart) -> float pairs (rows ld apart)
__global__ void kSplitPairs(size_t rows, size_t n, size_t ld, const double* __restrict__ src, float2* __restrict__ dst)
{
    const size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
    if (i >= rows * n)
        return;
    const size_t r = i / n, c = i % n;
    const double x = src[i];
    const float hi = __double2float_rn(x);
    dst[r * ld + c] = make_float2(hi, __double2float_rn(x - static_cast<double>(hi)));
}

// The stress increments at one Gauss point from its strain sums
// (MEVPStressUpdateStep.hpp:54-116): e11 = ex, e22 = ey, e12 = sxy / 2,
// Delta^2 = DeltaMin^2 + 1.25 (ex^2 + ey^2) + 1.5 ex ey + 0.25 sxy^2 in float
// pairs, 1/Delta from an FP32 seed by two Newton steps in FP64
// (y <- y (3 - t y^2) / 2), z8 = P / (8 alpha Delta) in FP64, the increments
// z8 (5 ex + 3 ey) - P / (2 alpha), z8 sxy, z8 (5 ey + 3 ex) - P / (2 alpha)
// in float pairs.  Pa = P / alpha.
__device__ __forceinline__ void gaussPoint(const pairs::Acc& ax, const pairs::Acc& ay, const pairs::Acc& axv,
    const pairs::Acc& ayu, pairs::F2 dmin2, double Pa, float2& f11, float2& f12, float2& f22)
{
    using namespace pairs;
    const F2 ex = result(ax), ey = result(ay);
    const F2 sxy = add(result(axv), result(ayu));
    F2 d2 = mul(add(mul(ex, ex), mul(ey, ey)), 1.25f);
    d2 = add(d2, mul(mul(ex, ey), 1.5f));
    d2 = add(d2, scale2(mul(sxy, sxy), 0.25f));
    d2 = add(d2, dmin2);
    const double t = value(d2);
    const double th = -0.5 * t;
    double y = widen(rsqrtf(d2.hi));
    y = fma(y, fma(th * y, y, 0.5), y);
    y = fma(y, fma(th * y, y, 0.5), y);
    const F2 z8 = split(0.125 * Pa * y);
    const F2 hP = scale2(split(Pa), 0.5f);
    const F2 mhP { -hP.hi, -hP.lo };
    const F2 r11 = add(mul(z8, add(mul(ex, 5.0f), mul(ey, 3.0f))), mhP);
    const F2 r12 = mul(z8, sxy);
    const F2 r22 = add(mul(z8, add(mul(ey, 5.0f), mul(ex, 3.0f))), mhP);
    f11 = make_float2(r11.hi, r11.lo);
    f12 = make_float2(r12.hi, r12.lo);
    f22 = make_float2(r22.hi, r22.lo);
}

// Thread layout as kMevpStress: three threads per element, 64 elements per
// block; thread `part` forms the Gauss points 3 part .. 3 part + 2, then the
// divergence coefficients of nodes 3 part .. 3 part + 2.
__global__ void __launch_bounds__(kPairElems * kPairParts) kMevpStressPairs(DevMesh m,
    const float2* __restrict__ ops, size_t ld, const double* __restrict__ u, const double* __restrict__ v,
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
    const float2* __restrict__ gyo = ops + 81 * ld;
    const float2* __restrict__ a1o = ops + 162 * ld;
    const float2* __restrict__ a2o = ops + 243 * ld;
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
                const F2 gx = pairOf(gxo[(q * 9 + j) * ld + e]);
                const F2 gy = pairOf(gyo[(q * 9 + j) * ld + e]);
                madd(ax, gx, ul[j]);
                madd(ay, gy, vl[j]);
                madd(axv, gx, vl[j]);
                madd(ayu, gy, ul[j]);
            }
            gaussPoint(ax, ay, axv, ayu, dmin2, Pg[q * N + e], fs[0][q][le], fs[1][q][le], fs[2][q][le]);
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
            const F2 a1 = pairOf(a1o[(j * 9 + q) * ld + e]);
            const F2 a2 = pairOf(a2o[(j * 9 + q) * ld + e]);
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

constexpr int kPairTmaElems = 32;
constexpr int kPairTmaParts = 9; // one thread per Gauss point (strain) and per node (divergence)
constexpr int kPairRows = 162;   // G_x | G_y, then A_1 | A_2
constexpr unsigned kPairTileBytes = kPairRows * kPairTmaElems * 8;
constexpr size_t kPairTmaSmem = size_t(kPairTileBytes) + 3 * 9 * kPairTmaElems * 8 + 2 * 8;

// Elements x0 .. x0 + 31 with their operator rows staged by TMA: the strain
// rows first, then (after every thread has read them) the divergence rows
// into the same buffer.  Warp g of the block owns Gauss point g, then node g.
// Bounded waits: a copy that has not landed in time sets DEV_ERR_TIMEOUT and
// the block returns after a second bounded wait for the copy it issued.
__global__ void __launch_bounds__(kPairTmaElems * kPairTmaParts, 4) kMevpStressPairsTma(
    const __grid_constant__ CUtensorMap mapG, const __grid_constant__ CUtensorMap mapA, DevMesh m,
    const double* __restrict__ u, const double* __restrict__ v, const double* __restrict__ Pg,
    double* __restrict__ tdiv, MevpParams p, int* __restrict__ err)
{
    using namespace pairs;
    extern __shared__ __align__(128) unsigned char smem[];
    float2* sT = reinterpret_cast<float2*>(smem);                         // [162][32]
    float2 (*fs)[9][kPairTmaElems] = reinterpret_cast<float2 (*)[9][kPairTmaElems]>(sT + kPairRows * kPairTmaElems);
    uint64_t* bars = reinterpret_cast<uint64_t*>(fs[3]);
    const int le = threadIdx.x % kPairTmaElems;
    const int g = threadIdx.x / kPairTmaElems; // warp-uniform: the Gauss point, then the node
    const int x0 = static_cast<int>(blockIdx.x) * kPairTmaElems;
    if (threadIdx.x == 0) {
        mbarInit(&bars[0], 1);
        mbarInit(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        mbarExpectTx(&bars[0], kPairTileBytes);
        tmaLoad2d(sT, &mapG, x0, 0, &bars[0]);
    }
    const size_t N = m.N;
    const size_t e = size_t(x0) + le;
    const bool active = e < N && m.ice[e];
    // the velocities, P/alpha and this thread's divergence coefficients are
    // loaded while the copy lands
    F2 ul[9], vl[9];
    double Pa = 0.0, t0 = 0.0, t1 = 0.0;
    if (active) {
        Pa = Pg[g * N + e];
        t0 = tdiv[g * N + e];
        t1 = tdiv[(9 + g) * N + e];
        const unsigned s2 = 2u * static_cast<unsigned>(m.nx) + 1u;
        const unsigned ix = static_cast<unsigned>(e) % static_cast<unsigned>(m.nx);
        const unsigned iy = static_cast<unsigned>(e) / static_cast<unsigned>(m.nx);
        const unsigned base = 2u * s2 * iy + 2u * ix;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const unsigned nd = base + unsigned(j % 3) + unsigned(j / 3) * s2;
            ul[j] = split(u[nd]);
            vl[j] = split(v[nd]);
        }
    }
    __syncthreads(); // the barriers are initialised before anyone polls them
    bool ok = mbarWaitBounded(&bars[0], 0);
    if (ok && active) {
        const F2 dmin2 { p.dmin2f, p.dmin2lo };
        Acc ax, ay, axv, ayu;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const F2 gx = pairOf(sT[(g * 9 + j) * kPairTmaElems + le]);
            const F2 gy = pairOf(sT[(81 + g * 9 + j) * kPairTmaElems + le]);
            madd(ax, gx, ul[j]);
            madd(ay, gy, vl[j]);
            madd(axv, gx, vl[j]);
            madd(ayu, gy, ul[j]);
        }
        gaussPoint(ax, ay, axv, ayu, dmin2, Pa, fs[0][g][le], fs[1][g][le], fs[2][g][le]);
    }
    // every thread has read the strain rows: the buffer may take the
    // divergence rows
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
        mbarExpectTx(&bars[1], kPairTileBytes);
        tmaLoad2d(sT, &mapA, x0, 0, &bars[1]);
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
    const int j = g;
    Acc dx, dy;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const F2 a1 = pairOf(sT[(j * 9 + q) * kPairTmaElems + le]);
        const F2 a2 = pairOf(sT[(81 + j * 9 + q) * kPairTmaElems + le]);
        const F2 f11 = pairOf(fs[0][q][le]), f12 = pairOf(fs[1][q][le]), f22 = pairOf(fs[2][q][le]);
        madd(dx, a1, f11);
        madd(dx, a2, f12);
        madd(dy, a1, f12);
        madd(dy, a2, f22);
    }
    tdiv[j * N + e] = fma(t0, p.keepd, value(result(dx)));
    tdiv[(9 + j) * N + e] = fma(t1, p.keepd, value(result(dy)));
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

cudaError_t launchSplitPairs(cudaStream_t s, size_t rows, size_t n, size_t ld, const double* src, float2* dst)
{
    if (rows * n == 0)
        return cudaSuccess;
    kSplitPairs<<<blocksOf(rows * n, 256), 256, 0, s>>>(rows, n, ld, src, dst);
    return cudaGetLastError();
}

size_t pairsLd(size_t N) { return (N + kPairTmaElems - 1) / kPairTmaElems * kPairTmaElems; }

cudaError_t makePairsMaps(const float2* ops, size_t ld, PairsMaps* out)
{
    // rows 0..161 (G_x | G_y) and 162..323 (A_1 | A_2) of the [324][ld]
    // array of 8-byte pairs; ld * 8 bytes is a multiple of 256 and the base
    // 256-byte aligned, so every box starts on a 256-byte boundary
    cudaError_t e = encodeTiled2d(&out->g, CU_TENSOR_MAP_DATA_TYPE_UINT64, ops, ld, kPairRows, ld * 8,
        kPairTmaElems, kPairRows);
    if (e == cudaSuccess)
        e = encodeTiled2d(&out->a, CU_TENSOR_MAP_DATA_TYPE_UINT64, ops + kPairRows * ld, ld, kPairRows, ld * 8,
            kPairTmaElems, kPairRows);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(kMevpStressPairsTma, cudaFuncAttributeMaxDynamicSharedMemorySize,
            static_cast<int>(kPairTmaSmem));
    return e;
}

cudaError_t launchMevpStressPairs(cudaStream_t s, const DevMesh& m, const float2* ops, size_t ld, const double* u,
    const double* v, const double* Pg, double* tdiv, const MevpParams& pIn)
{
    const MevpParams p = withDerived(pIn);
    kMevpStressPairs<<<blocksOf(m.N, kPairElems), kPairElems * kPairParts, 0, s>>>(m, ops, ld, u, v, Pg, tdiv, p);
    return cudaGetLastError();
}

cudaError_t launchMevpStressPairsTma(cudaStream_t s, const DevMesh& m, const PairsMaps& maps, const double* u,
    const double* v, const double* Pg, double* tdiv, const MevpParams& pIn, int* err)
{
    const MevpParams p = withDerived(pIn);
    kMevpStressPairsTma<<<blocksOf(m.N, kPairTmaElems), kPairTmaElems * kPairTmaParts, kPairTmaSmem, s>>>(
        maps.g, maps.a, m, u, v, Pg, tdiv, p, err);
    return cudaGetLastError();
}

cudaError_t launchPairsSelfTest(cudaStream_t s, size_t n, const double* a, const double* x, double* out)
{
    kPairsSelfTest<<<blocksOf(n, 128), 128, 0, s>>>(n, a, x, out);
    return cudaGetLastError();
}

} // namespace nsdg
