// nsdg_kernels.hpp — host-callable launchers for the sm_103a kernels.
//
// Pure C++ declarations (no CUDA syntax) so the C-ABI layer can be compiled
// by the host compiler.  Every launcher enqueues on `stream` and returns the
// cudaError_t of the launch.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

#include "nsdg_host.hpp"

namespace nsdg {

// Device copy of the mesh connectivity and boundary flags.
struct DevMesh {
    int nx = 0, ny = 0;
    int spherical = 0; // x = lon, y = lat (radians): edge tangents wrap in longitude
    size_t N = 0;      // elements
    size_t Ncg = 0;    // CG2 nodes (2nx+1)(2ny+1)
    size_t Ncg1 = 0;   // CG1 nodes (nx+1)(ny+1)
    size_t nXe = 0;    // X-edges nx(ny+1)
    size_t nYe = 0;    // Y-edges (nx+1)ny
    const double* vx = nullptr;
    const double* vy = nullptr;
    const uint8_t* ice = nullptr;
    const uint8_t* cellSeg = nullptr;
    const uint8_t* edgeXCount = nullptr;
    const uint8_t* edgeYCount = nullptr;
    const uint8_t* cg2Dir = nullptr;
    const int* perPtr = nullptr;
    const int* perEntry = nullptr;
};

// Device copy of the element operators (entry-major SoA, see nsdg_host.hpp).
struct DevOps {
    const double* cellX = nullptr;
    const double* cellY = nullptr;
    const double* minv = nullptr;
    const double* jwA = nullptr;
    const double* jw3 = nullptr;
    const double* cellX8 = nullptr;
    const double* cellY8 = nullptr;
    const double* minv8 = nullptr;
    const double* gx = nullptr;
    const double* gy = nullptr;
    const double* w = nullptr;
    const double* a1 = nullptr;
    const double* a2 = nullptr;
    const double* d1 = nullptr;
    const double* d2 = nullptr;
    const double* wdam = nullptr;
    const double* dxssh = nullptr;
    const double* dyssh = nullptr;
    const double* hsize = nullptr;
    const double* invm2 = nullptr;   // 1 / lumped CG2 mass
    const double* lumped1 = nullptr; // lumped CG1 mass
    // spherical metric terms (null on Cartesian meshes)
    const double* gm = nullptr;      // strain term iMM at the Gauss points [q][j]
    const double* minvP = nullptr;   // CG2DG inverse mass (the transport's minv carries 1 / R)
    const double* minv8P = nullptr;
    const double* a3 = nullptr;      // divM iMJwPSI [j][q]
    const double* dm = nullptr;      // divM [j][k] (BBM)
};

// Status bits written by kernels into the handle's device error word.
enum DeviceError : int {
    DEV_ERR_NONFINITE_VELOCITY = 1,
    DEV_ERR_NONFINITE_STRESS = 2,
    DEV_ERR_TIMEOUT = 4,            // a bounded wait on an asynchronous copy ran out
};

cudaError_t uploadConstTables();

// --- transport ---------------------------------------------------------
enum StageMode { STAGE_RK1 = 0, STAGE_RK2_A, STAGE_RK2_B, STAGE_RK3_A, STAGE_RK3_B, STAGE_RK3_C };
struct StageFields {
    int nf = 1;
    const double* src[3] = {};
    const double* phi[3] = {};
    double* k1[3] = {};
    double* dst[3] = {};
    int lmax[3] = {};
    int lmin[3] = {};
    double vmax[3] = {};
    double vmin[3] = {};
};
// CG2 -> DG projection of nf (<=2) node fields (Interpolations.cpp:74-122).
// Uses jw/minv for `dg` components (jwA/minv, or jw3/minv8 for dg == 8).
cudaError_t launchCG2DG(cudaStream_t s, const DevMesh& m, int dg, const double* jw,
    const double* minv, int nf, const double* const* cg, double* const* out);
// CG2DG of two fields with FP32 quadrature (jw32: J w at the advection Gauss
// points in FP32) and the FP64 inverse mass matrix (the mixed-precision
// transport velocity); with minvDiag ([dg][N], parallelogram meshes) only
// the diagonal of M^{-1} is applied.
cudaError_t launchCG2DG32(cudaStream_t s, const DevMesh& m, int dg, const float* jw32, const double* minv,
    const double* const* cg, double* const* out, const double* minvDiag = nullptr);
// Cell averages (component 0) of the CG2DG projection of two fields, written
// to out[0][0..N) and out[1][0..N): FP32 quadrature when jw32 is given (the
// mixed path), else kCG2DG's FP64 arithmetic.  Row 0 of minv only.
cudaError_t launchCG2DG0(cudaStream_t s, const DevMesh& m, int dg, const double* jw, const float* jw32,
    const double* minv, const double* const* cg, double* const* out);
// Edge normal velocities (DGTransport.cpp:158-252).
cudaError_t launchNormalVelocity(cudaStream_t s, const DevMesh& m, int dg, const double* velx,
    const double* vely, double* nvX, double* nvY);
// One Runge-Kutta stage of the DG transport operator for nf fields sharing a
// velocity (DGTransport.cpp:435-566).  With FP32 copies of the cell
// operators (cellX32, cellY32) the flux arithmetic is FP32; the fields, the
// inverse mass matrices and the stage combination stay FP64.
cudaError_t launchTransportStage(cudaStream_t s, const DevMesh& m, int dg, const double* cellX,
    const double* cellY, const double* minv, const double* velx, const double* vely,
    const double* nvX, const double* nvY, int mode, double dt, const StageFields& f,
    const float* cellX32 = nullptr, const float* cellY32 = nullptr);
// The same stage on a mesh of parallelograms with FP32 fluxes: tiles of
// 32 x 8 elements with the edge fluxes staged in shared memory, the cell term
// from the Jacobian coefficients coef ([5][ld], c0 .. c3 used) and the
// unit-square operators uploaded by uploadAffineTransportReference, and the
// diagonal of M^{-1} (minvDiag, [dg][N]).  dg in {1, 3, 6}; no periodic edges.
cudaError_t uploadAffineTransportReference(int dg, const double ref[2][8 * 16]);
cudaError_t launchTransportStageAffine(cudaStream_t s, const DevMesh& m, int dg, const float* coef, size_t ld,
    const double* minvDiag, const double* velx, const double* vely, const double* nvX, const double* nvY,
    int mode, double dt, const StageFields& f);

// --- interpolation / preparation ----------------------------------------
// DG -> CG2 Lagrange averaging of nf (<=2) DG fields (Interpolations.cpp:144-204).
cudaError_t launchDG2CG(cudaStream_t s, const DevMesh& m, int dg, int nf,
    const double* const* dgIn, double* const* cgOut);
// Gradient of the sea-surface height on CG2 (CGDynamicsKernel.cpp:126-258);
// scratch needs 3*Ncg1 doubles.
cudaError_t launchSSHGradient(cudaStream_t s, const DevMesh& m, const DevOps& o, const double* ssh,
    double* scratch, double* uGrad, double* vGrad);

// mEVP per-step node constants (CGDynamicsKernel.cpp:260-276 clamps plus the
// loop-invariant parts of VPCGDynamicsKernel.hpp:132-172).
struct MevpNodeState {
    double* u;
    double* v;
    double* u0;
    double* v0;
    double* cgH;     // in: DG2CG(h) ; out: clamped
    double* cgA;     // in: DG2CG(A) ; out: clamped
    const double* uo;
    const double* vo;
    const double* ua;
    const double* va;
    const double* uGrad;
    const double* vGrad;
    double* c1;      // rho H / dt
    double* c1b;     // rho H / dt * (1 + beta)
    double* fau;     // F_atm |wind| uwind
    double* fav;
    double* rhfc;    // rho H fc
    double* gu;      // rho H g dxSSH
    double* gv;
};
struct MevpParams {
    double rho_ice, F_atm, F_ocean, fc, gravity, Pstar, DeltaMin, alpha, beta, dt;
    // derived on the host by withDerived() in every stress launcher, so that
    // no thread spends FP64 instructions (about 1/60 of the FP32 rate on
    // GB300) on a division or a square of the parameters
    double keepd = 0;                          // 1 - 1/alpha
    float keep = 0, dmin2f = 0, F_oceanf = 0;  // FP32 copies (dmin2f: DeltaMin^2)
    float dmin2lo = 0;                         // DeltaMin^2 - dmin2f (its float-pair low part)
    float betaf = 0, onePlusBetaf = 0, fcdtf = 0; // beta, 1 + beta, fc dt
};
inline MevpParams withDerived(MevpParams p)
{
    p.keepd = 1.0 - 1.0 / p.alpha;
    p.keep = static_cast<float>(p.keepd);
    p.dmin2f = static_cast<float>(p.DeltaMin * p.DeltaMin);
    p.dmin2lo = static_cast<float>(std::fma(p.DeltaMin, p.DeltaMin, -static_cast<double>(p.dmin2f)));
    p.F_oceanf = static_cast<float>(p.F_ocean);
    p.betaf = static_cast<float>(p.beta);
    p.onePlusBetaf = static_cast<float>(1.0 + p.beta);
    p.fcdtf = static_cast<float>(p.fc * p.dt);
    return p;
}
cudaError_t launchMevpPrepNodes(cudaStream_t s, const DevMesh& m, const MevpNodeState& st,
    const MevpParams& p);
// P at the 3x3 Gauss points from h and A (MEVPStressUpdateStep.hpp:54-57,75-77):
// Pg = P/alpha, or, for the mixed-precision kernels (hP32 given),
// Pg = P/(8 alpha) (FP64, the viscosity numerator) and hP32 = P/(2 alpha).
// tdivLast (mixed precision, optional): also copies tdiv32 there (the
// sub-cycle's starting divergence, a warm-start feature).
cudaError_t launchMevpPrepElements(cudaStream_t s, const DevMesh& m, int dg, const double* h,
    const double* a, double* Pg, const MevpParams& p, float* hP32 = nullptr, const float* tdiv32 = nullptr,
    float* tdivLast = nullptr);
// One mEVP iteration, element part, carried in divergence space: the strain at
// the Gauss points, Delta, and the relaxed update of the element's stress
// divergence contributions tdiv[18][N] = (divS1 s11 + divS2 s12, divS1 s12 +
// divS2 s22) at its 9 CG2 nodes (CGDynamicsKernel.cpp:300-398,
// MEVPStressUpdateStep.hpp:30-118).  Pg holds P/alpha at the Gauss points.
cudaError_t launchMevpStress(cudaStream_t s, const DevMesh& m, const DevOps& o, const double* u,
    const double* v, const double* Pg, double* tdiv, const MevpParams& p);
// The benchmark forcing on the cell centres (nsdg_forcing.cu):
// BenchmarkAtmosphere.cpp:29-77 and BenchmarkOcean.cpp:15-39.
struct BenchmarkWindArgs {
    double dx, dy, x0, y0, A, k, vmax, cosa, sina;
};
cudaError_t launchBenchmarkWind(cudaStream_t s, size_t nx, size_t ny, const BenchmarkWindArgs& a, double* uw,
    double* vw);
cudaError_t launchBenchmarkOcean(cudaStream_t s, size_t nx, size_t ny, double dx, double dy, double vmax,
    double* uo, double* vo);
// FP64 operator entries as float pairs {RN(x), RN(x - RN(x))}: rows x n
// entries, rows n apart in src and ld apart in dst.
cudaError_t launchSplitPairs(cudaStream_t s, size_t rows, size_t n, size_t ld, const double* src, float2* dst);
// launchMevpStress with the operator products, Delta^2 and the stress
// increments in float-pair arithmetic (nsdg_stress_pairs.cu); 1/Delta,
// P / (8 alpha Delta) and the divergence update in FP64.  ops: [4][81][N]
// float pairs of G_x, G_y, A_1, A_2 (Cartesian meshes).
// ops: [324][ld] float pairs, rows G_x | G_y | A_1 | A_2, ld = pairsLd(N).
size_t pairsLd(size_t N);
cudaError_t launchMevpStressPairs(cudaStream_t s, const DevMesh& m, const float2* ops, size_t ld, const double* u,
    const double* v, const double* Pg, double* tdiv, const MevpParams& p);
// The same kernel with each phase's operator rows staged in shared memory by
// one TMA copy per 32 elements (descriptors from makePairsMaps).
struct alignas(64) PairsMaps {
    CUtensorMap g;
    CUtensorMap a;
};
cudaError_t makePairsMaps(const float2* ops, size_t ld, PairsMaps* out);
cudaError_t launchMevpStressPairsTma(cudaStream_t s, const DevMesh& m, const PairsMaps& maps, const double* u,
    const double* v, const double* Pg, double* tdiv, const MevpParams& p, int* err);
// out[4 i + 0..3]: split(a) - a, widen(RN(x)), a x and a 9-term dot product,
// each formed in float pairs and returned in FP64 (checks of nsdg_pairs.cuh).
cudaError_t launchPairsSelfTest(cudaStream_t s, size_t n, const double* a, const double* x, double* out);
// Node gather of the divergence, Dirichlet zero, implicit velocity update and
// boundary zero (CGDynamicsKernel.cpp:365-444, VPCGDynamicsKernel.hpp:132-172).
cudaError_t launchMevpMomentum(cudaStream_t s, const DevMesh& m, const DevOps& o,
    const MevpNodeState& st, const double* contrib, const MevpParams& p, int* err);

// --- mEVP, mixed precision (NSDG_PRECISION_MIXED) ----------------------
// FP32 operators, velocities, divergence coefficients and momentum
// arithmetic; FP64 for Delta = sqrt(strain invariant + DeltaMin^2), the
// viscosity P/(2 Delta), and the lumped-mass inverse.
// FP32 element operators, one [rows][ld] block: G_x, G_y (and G_m on a
// sphere), then A_1, A_2 (and A_3), 81 rows each; ld = N rounded up to
// kTmaElems (padding zero).
struct DevOps32 {
    const float* gx = nullptr;
    const float* gy = nullptr;
    const float* a1 = nullptr;
    const float* a2 = nullptr;
    const float* gm = nullptr; // spherical only
    const float* a3 = nullptr; // spherical only
    size_t ld = 0;
    int rowsG = 162;           // rows of the strain (and of the divergence) part: 162, or 243 on a sphere
};
constexpr int kTmaElems = 32;   // elements per block of the TMA-staged stress kernel
inline size_t ops32Ld(size_t N) { return (N + kTmaElems - 1) / kTmaElems * kTmaElems; }
// TMA descriptors of the strain rows (G_x, G_y) and the divergence rows
// (A_1, A_2) of a DevOps32 block: 2-D, inner dimension the element index.
struct alignas(64) StressMaps {
    CUtensorMap g;
    CUtensorMap a;
};
cudaError_t makeStressMaps(const DevOps32& o, StressMaps* out);
// A 2-D tiled TMA descriptor (cuTensorMapEncodeTiled through the runtime's
// driver entry point): inner x outer elements of `type`, rows rowBytes apart
// (a multiple of 16), boxes of boxInner x boxOuter, no swizzle, zero fill.
cudaError_t encodeTiled2d(CUtensorMap* map, CUtensorMapDataType type, const void* base, uint64_t inner,
    uint64_t outer, uint64_t rowBytes, uint32_t boxInner, uint32_t boxOuter);
// A tensor map of rank 1..5 without swizzle, out-of-bounds elements read as
// zero: dims[0] innermost, strideBytes[i] the byte stride of dimension i + 1
// (multiples of 16), box the tile copied per load (box[0] * element size a
// multiple of 16 bytes).
cudaError_t encodeTiledNd(CUtensorMap* map, CUtensorMapDataType type, const void* base, int rank,
    const uint64_t* dims, const uint64_t* strideBytes, const uint32_t* box);
// One block waits (bounded) on an mbarrier nothing completes; *timedOut = 1
// when the wait ran out as it must.
cudaError_t launchBoundedWaitSelfTest(cudaStream_t s, double limitSeconds, int* timedOut);
// kMevpStress32 with the operator tiles staged in shared memory by TMA.
cudaError_t launchMevpStress32Tma(cudaStream_t s, const DevMesh& m, const StressMaps& maps, const float* u,
    const float* v, const double* Pg, const float* hP, float* tdiv, const MevpParams& p, int* err);
// The mixed-precision node state.  The momentum update is divided through by
// c1 = rho H / dt, so that per node it needs only
//   u_new = (beta u + ku + a F_ocean |u_o - u| u_o - fc dt u + im dSx)
//           / (1 + beta + a F_ocean |u_o - u|)
// (and likewise v with +fc dt v), with the per-step constants
//   a = A / c1,  ku = u0 + (A F_atm |wind| uwind - rho H g dxSSH) / c1,
//   im = (1 / lumped mass) / c1
// formed in FP64 (im kept as the unevaluated sum hi + lo of two floats).
struct MevpNodeState32 {
    float* u;
    float* v;
    float* u0;
    float* v0;
    float4* k0; // (a, ku, kv, u_ocean)
    float4* k1; // (v_ocean, im hi, im lo, 1 on a Dirichlet node else 0)
};
// The per-step node preparation of the mixed path (prepareIteration's clamps,
// CGDynamicsKernel.cpp:260-276, and the constants of updateMomentum,
// VPCGDynamicsKernel.hpp:132-172): FP64 inputs, the FP32 state above; the
// clamped cgA, cgH and u0, v0 are written back in FP64.  invm2: the FP64
// inverse lumped CG2 mass.
cudaError_t launchMevpPrepNodes32(cudaStream_t s, const DevMesh& m, const MevpNodeState& st64,
    const MevpNodeState32& st32, const double* invm2, const MevpParams& p,
    float* uLast = nullptr, float* vLast = nullptr);
// (the Dirichlet flags of the nodes come from m.cg2Dir)
// kMevpStress32 for parallelogram meshes: the unit-square operators
// (G_xi, G_eta [q][j], A_xi, A_eta [j][q]) in constant memory, uploaded once
// per device (they depend only on the basis), and 5 coefficients per element
// ([5][ld]).  viscosityMode selects the FP64 evaluation of P/(8 alpha Delta):
// 0 CUDA's rsqrt(double), 1 a Newton step from an FP32 seed, 2 the same with
// float/double conversions on the integer pipe; 3 the same Newton step with
// float pairs on the FP32 pipe (nsdg_visc_ff.hpp); 4 form 3 checked against
// form 2's rounding, with form 2 where the check fails (bitwise form 2).
cudaError_t uploadAffineReference(const double ref[4][81]);
cudaError_t launchMevpStress32Affine(cudaStream_t s, const DevMesh& m, const float* coef, size_t ld, const float* u,
    const float* v, const double* Pg, float* tdiv, const MevpParams& p, int viscosityMode);
// out[k n + i] = P/(8 alpha Delta) of (inv[i], Pa[i]) by viscosity mode k = 0, 1, 2.
cudaError_t launchViscositySelfTest(cudaStream_t s, size_t n, const float* inv, const double* Pa, double dmin,
    float* out);
// out[i] = P/(8 alpha Delta) of (inv[i], Pa[i]) by viscosity mode 3.
cudaError_t launchViscositySelfTestFF(cudaStream_t s, size_t n, const float* inv, const double* Pa, double dmin,
    float* out);
// out[i] = P/(8 alpha Delta) of (inv[i], Pa[i]) by viscosity mode 4.
cudaError_t launchViscositySelfTestChecked(cudaStream_t s, size_t n, const float* inv, const double* Pa,
    double dmin, float* out);
cudaError_t launchMevpStress32(cudaStream_t s, const DevMesh& m, const DevOps32& o, const float* u,
    const float* v, const double* Pg, const float* hP, float* tdiv, const MevpParams& p);
cudaError_t launchMevpMomentum32(cudaStream_t s, const DevMesh& m,
    const MevpNodeState32& st, const float* tdiv, const MevpParams& p, int* err);
// One member of a batched ensemble (device-resident table entry).
struct EnsembleMember {
    int nx, ny;
    size_t N, Ncg;
    const uint8_t* ice;
    const uint8_t* cg2Dir;
    const double* invm2;
    DevOps32 o;
    MevpNodeState32 st;
    const double* Pg;
    const float* hP;
    float* tdiv;
    int tileW, tileH, tilesX;
    int stressBlock0, nodeBlock0;
    int tmaBlock0;   // first block of this member in the TMA-staged / parallelogram batched launch
    int nodeBlockP;  // first block of this member in the persistent sub-cycle's node phase
    StressMaps maps; // the member's tensor maps (64-byte aligned inside the device table)
    const float* affCoef; // [5][affLd] parallelogram coefficients (null: not a parallelogram mesh)
    size_t affLd;
};
// The whole mEVP sub-cycle of a parallelogram ensemble (every member has
// coefficients) as one cooperative, persistent launch: `iterations` times the
// element phase (the parallelogram kernel, blocks of elemMap as in the batched
// launch) and the node phase (nodeMap: blocks of persistentNodesPerBlock()
// nodes), separated by bounded grid barriers on bar[2] (set to zero here
// first).  Bitwise the same results as the per-phase launches.
int persistentNodesPerBlock();
cudaError_t launchEnsembleSubcyclePersistent(cudaStream_t s, const EnsembleMember* members, const uint16_t* elemMap,
    int elemBlocks, const uint16_t* nodeMap, int nodeBlocks, const MevpParams& p, int viscosityMode,
    int iterations, unsigned* bar, int* err);
// One launch each for the element and the node phase of every member.
cudaError_t launchMevpStress32Batched(cudaStream_t s, const EnsembleMember* members, const uint16_t* blockMember,
    int blocks, const MevpParams& p);
cudaError_t launchMevpMomentum32Batched(cudaStream_t s, const EnsembleMember* members, const uint16_t* blockMember,
    int blocks, const MevpParams& p, int* err);
// The element phase of every member with the TMA-staged kernel: blocks of
// kTmaElems consecutive elements, tensor maps read from the member table.
cudaError_t launchMevpStress32TmaBatched(cudaStream_t s, const EnsembleMember* members,
    const uint16_t* blockMember, int blocks, const MevpParams& p, int* err);
// The element phase of every member with the parallelogram kernel (every
// member must have coefficients); blocks as for the TMA-staged launch.
cudaError_t launchMevpStress32AffineBatched(cudaStream_t s, const EnsembleMember* members,
    const uint16_t* blockMember, int blocks, const MevpParams& p, int viscosityMode);
int stressElementsPerBlock();
int nodesPerBlock();

// u, v (FP64) from the FP32 iterate at the end of the sub-cycle
cudaError_t launchWidenVelocity(cudaStream_t s, size_t n, const float* u32, const float* v32, double* u,
    double* v);

// Ice-ocean stress on CG2 nodes (VPCGDynamicsKernel.hpp:96-120 / BrittleCGDynamicsKernel.hpp:168-192);
// fp32: the same formulas in FP32 (the mixed path's read-out).
cudaError_t launchIceOceanStress(cudaStream_t s, size_t n, int brittle, const double* u,
    const double* v, const double* uo, const double* vo, double F_ocean, double cosA, double sinA,
    double* tx, double* ty, bool fp32 = false);

// --- BBM -----------------------------------------------------------------
struct BbmParams {
    double rho_ice, F_atm, F_ocean, fc, gravity, dt, nSteps, cosA, sinA;
    double compaction_param, nu0, young, P0, lambda, exponent_relaxation_sigma,
        exponent_compression_factor, tan_phi, compr_strength, C_lab;
    // how the kernels evaluate d^(n-1) (relaxation) and h^(m+1) (compression):
    // mode 1 = integer power k by multiplication, 2 = x^k sqrt(x), 0 = pow()
    int powRmode = 0, powRk = 0, powCmode = 0, powCk = 0;
    double invNSteps = 0; // 1 / nSteps (set by bbmPowModes)
};
// Sets the power modes of p from its exponents (integers and half-integers up to 8).
inline void bbmPowModes(BbmParams& p)
{
    p.invNSteps = 1.0 / p.nSteps;
    auto classify = [](double y, int& mode, int& k) {
        mode = 0;
        k = 0;
        for (int n = 0; n <= 8; ++n) {
            if (y == n) {
                mode = 1;
                k = n;
                return;
            }
            if (y == n + 0.5) {
                mode = 2;
                k = n;
                return;
            }
        }
    };
    classify(p.exponent_relaxation_sigma - 1, p.powRmode, p.powRk);
    classify(p.exponent_compression_factor + 1., p.powCmode, p.powCk);
}
struct BbmNodeState {
    double* u;
    double* v;
    double* avgU;
    double* avgV;
    double* cgH;
    double* cgA;
    const double* uo;
    const double* vo;
    const double* ua;
    const double* va;
    const double* uGrad;
    const double* vGrad;
};
// Mixed-precision BBM: the node terms that stay fixed through the elastic
// sub-steps, in FP32, formed once per step by the preparation kernel:
// k0 = (dt_sub / (rho H), A F_ocean, u_ocean, v_ocean), k1 = (the wind
// stress tau_atm,x, tau_atm,y, rho H g dX_ssh, rho H g dY_ssh).
struct BbmNodeConst32 {
    float4* k0;
    float4* k1;
};
// c (mixed precision, with p): also forms the FP32 node constants.
cudaError_t launchBbmPrepNodes(cudaStream_t s, const DevMesh& m, const BbmNodeState& st,
    const BbmParams* p = nullptr, const BbmNodeConst32* c = nullptr);
// Per-step Gauss-point constants of the BBM update from h and A:
// 0 hG, 1 expC, 2 Pmax, 3 elasticity, 4 Dunit_factor / dt ... (9 x 5 per element)
// FP32 copies of the BBM element operators (mixed precision)
struct BbmOps32 {
    const float* gx;
    const float* gy;
    const float* w;
    const float* wdam;
    const float* d1;
    const float* d2;
    const float* gm; // spherical only
    const float* dm; // spherical only
    // parallelogram meshes: [5][ld] coefficients; the stress kernel then takes
    // the unit square's operators (uploadAffineReference,
    // uploadAffineBbmReference) instead of the per-element ones above
    const float* coef = nullptr;
    size_t ld = 0;
};
cudaError_t uploadAffineBbmReference(const double* w, const double* wdam, int dg, const double* dxi,
    const double* deta);
cudaError_t launchBbmStress(cudaStream_t s, const DevMesh& m, const DevOps& o, int dg, const double* u,
    const double* v, const double* h, const double* a, double* damage, double* s11, double* s12,
    double* s22, double* contrib, const BbmParams& p, int* err, const BbmOps32* o32 = nullptr);
cudaError_t launchBbmMomentum(cudaStream_t s, const DevMesh& m, const DevOps& o,
    const BbmNodeState& st, const double* contrib, const BbmParams& p, int* err,
    const float2* invmHL = nullptr, const BbmNodeConst32* c = nullptr);

// --- layout conversion, reductions ---------------------------------------
// host ModelArray layout (AoS, nin comps) -> device SoA with `dg` comps,
// following DGModelArray::ma2dg (zero, then all or component 0 only).
cudaError_t launchAosToSoa(cudaStream_t s, size_t N, int nin, int dg, const double* aos, double* soa);
// Moves of whole arrays (dst[i][0 .. n[i]) = src[i][0 .. n[i])) in one kernel,
// for host arrays on a GPU that accesses pageable host memory directly.
constexpr int kHostMoves = 8;
struct HostMoves {
    const double* src[kHostMoves] = {};
    double* dst[kHostMoves] = {};
    unsigned long long n[kHostMoves] = {};
    int count = 0;
};
cudaError_t launchHostMove(cudaStream_t s, const HostMoves& m);
// device SoA -> AoS with `nout` comps (all, or component 0 only)
cudaError_t launchSoaToAos(cudaStream_t s, size_t N, int dg, int nout, const double* soa, double* aos);
// Tools::MeanValue: writes partial sums per block into `partials` and the
// final FP64 sum into *out (device).  partials needs ceil(N/256) doubles.
cudaError_t launchMeanValue(cudaStream_t s, size_t N, int dg, const double* phi, const double* jw3,
    double* partials, double* out);

} // namespace nsdg
