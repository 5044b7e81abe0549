// nsdg_capi.cpp — the C ABI (include/nsdg.h): handles, device memory, the
// CUDA-graph capture of one model step, and the field exchange with the
// reference's ModelArray layout.
//
// No exception crosses the ABI; every entry point returns a status code and
// keeps a message in the handle.
#include "nsdg.h"

#include "nsdg_host.hpp"
#include "nsdg_ice_growth.hpp"
#include "nsdg_kernels.hpp"
#include "nsdg_surrogate.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <exception>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

using namespace nsdg;

namespace {

const char* kVersion = "nsdg-gb300 0.1 sm_103a";

// Bump allocator over one device allocation (256-byte aligned sub-buffers).
struct Arena {
    char* base = nullptr;
    size_t cap = 0, used = 0;
    cudaError_t reserve(size_t bytes)
    {
        cap = bytes;
        used = 0;
        return cudaMalloc(&base, bytes);
    }
    template <class T> T* take(size_t n)
    {
        const size_t bytes = ((n * sizeof(T) + 255) / 256) * 256;
        if (used + bytes > cap)
            return nullptr;
        T* p = reinterpret_cast<T*>(base + used);
        used += bytes;
        return p;
    }
    void release()
    {
        if (base)
            cudaFree(base);
        base = nullptr;
        cap = used = 0;
    }
};
inline size_t al(size_t bytes) { return ((bytes + 255) / 256) * 256; }

struct Status {
    int code = NSDG_OK;
    std::string msg;
};

#define CUDA_TRY(expr)                                                                             \
    do {                                                                                           \
        cudaError_t e_ = (expr);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            return fail(NSDG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));       \
        }                                                                                          \
    } while (0)

int deviceCheck(std::string& msg)
{
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        msg = std::string("no CUDA device: ") + (e != cudaSuccess ? cudaGetErrorString(e) : "count 0");
        cudaGetLastError();
        return NSDG_ERR_NO_DEVICE;
    }
    return NSDG_OK;
}

} // namespace

// ===========================================================================
// Dynamics kernel handle
// ===========================================================================
struct nsdg_kernel {
    int rheology = NSDG_RHEOLOGY_MEVP;
    int dg = 6;
    nsdg_params P {};
    std::string err;
    bool ready = false;
    cudaStream_t stream = nullptr;
    Arena arena;
    HostMesh mesh;
    BoundaryFlags flags;
    DevMesh dm;
    DevOps dops;
    size_t N = 0, Ncg = 0, Ncg1 = 0;
    // state
    double *hice = nullptr, *cice = nullptr, *ssh = nullptr, *damage = nullptr;
    double *s11 = nullptr, *s12 = nullptr, *s22 = nullptr;
    double *u = nullptr, *v = nullptr, *uo = nullptr, *vo = nullptr, *ua = nullptr, *va = nullptr;
    double *avgU = nullptr, *avgV = nullptr;
    // per-step work
    double *u0 = nullptr, *v0 = nullptr, *cgH = nullptr, *cgA = nullptr, *uGrad = nullptr, *vGrad = nullptr;
    double *c1 = nullptr, *c1b = nullptr, *fau = nullptr, *fav = nullptr, *rhfc = nullptr, *gu = nullptr, *gv = nullptr;
    double *Pg = nullptr, *contrib = nullptr;
    double *velx = nullptr, *vely = nullptr, *nvX = nullptr, *nvY = nullptr;
    double *phiA = nullptr, *k1 = nullptr; // 3 fields x dg x N
    double *velx8 = nullptr, *vely8 = nullptr, *nvX8 = nullptr, *nvY8 = nullptr;
    double *sA = nullptr, *sK1 = nullptr;  // 3 x 8 x N
    double *sshScratch = nullptr, *staging = nullptr, *dgTmp = nullptr, *cgTmp = nullptr;
    // mixed precision (NSDG_PRECISION_MIXED)
    DevOps32 dops32;
    StressMaps maps32 {};
    float* hP32 = nullptr; // P/(2 alpha) at the Gauss points (mixed precision)
    float *cellX32 = nullptr, *cellY32 = nullptr; // FP32 transport cell operators (mixed precision)
    float* jwA32 = nullptr; // FP32 J w at the advection Gauss points (mixed-precision CG2DG)
    float2* invmHL = nullptr; // inverse lumped CG2 mass as {hi, lo} floats (mixed precision)
    BbmOps32 bbm32 {};        // FP32 BBM operators (mixed precision BBM)
    // mixed BBM: the node terms fixed through the elastic sub-steps (FP32,
    // formed by the step's node preparation)
    BbmNodeConst32 bbmConst { nullptr, nullptr };
    bool bbmK0 = false;
    float *cellX8_32 = nullptr, *cellY8_32 = nullptr; // FP32 DG8 stress-transport operators
    // which FP32 stress kernel the updates use (chosen by timing at
    // initialise): 0 operators by global loads, 1 operator tiles by TMA,
    // 2 parallelogram coefficients (when the mesh allows it)
    int stressKind = 1;
    int viscMode = 2;                // FP64 viscosity form of the parallelogram kernel
    // FP64 path: the element stress kernel, 0 = FP64 FMA (kMevpStress, the
    // default), 1 = float-pair products (kMevpStressPairs), 2 = the same with
    // TMA-staged operators (kMevpStressPairsTma); Cartesian mEVP.  The
    // operators as float pairs [324][pairsLd(N)] and their TMA descriptors.
    int fp64Stress = 0;
    float2* opsPairs = nullptr;
    size_t pairsLdN = 0;
    PairsMaps pairsMaps {};
    // mixed path: transport velocity (CG2DG) and fluxes in FP32 (the
    // default); NSDG_MIXED_TRANSPORT=fp64 keeps them in FP64 (to measure what
    // the FP32 transport contributes to the mixed path's error)
    bool transport32 = true;
    float* affCoef = nullptr;        // [5][ld] parallelogram coefficients (null: not a parallelogram mesh)
    size_t affLd = 0;
    double affWorst = -1;            // largest relative mismatch of the rebuilt operators (FP64)
    // mixed path on a parallelogram mesh without periodic edges: the tiled
    // transport stage (edge fluxes staged in shared memory, cell term from
    // affCoef, diagonal M^{-1}); NSDG_TRANSPORT_KERNEL=element keeps the
    // per-element kernel
    double* minvDiag = nullptr;      // [dg][N]
    bool trAffine = false;
    double trAffWorst[2] = { -1, -1 }; // cell-operator mismatch, relative off-diagonal of M^{-1}
    cudaError_t launchTransport(cudaStream_t s, int mode, double dt, const StageFields& f, bool forceElement = false)
    {
        if (trAffine && !forceElement)
            return launchTransportStageAffine(s, dm, dg, affCoef, affLd, minvDiag, velx, vely, nvX, nvY, mode, dt, f);
        const bool t32 = mixed() && transport32;
        return launchTransportStage(s, dm, dg, dops.cellX, dops.cellY, dops.minv, velx, vely, nvX, nvY, mode, dt, f,
            t32 ? cellX32 : nullptr, t32 ? cellY32 : nullptr);
    }
    cudaError_t launchStress32(cudaStream_t s, const MevpParams& mp, int* errWord, int variant = -1,
        int vm = -1)
    {
        const int kind = variant < 0 ? stressKind : variant;
        if (kind == 2 && affCoef)
            return launchMevpStress32Affine(s, dm, affCoef, affLd, st32.u, st32.v, Pg, tdiv32, mp,
                vm < 0 ? viscMode : vm);
        return kind == 1 ? launchMevpStress32Tma(s, dm, maps32, st32.u, st32.v, Pg, hP32, tdiv32, mp, errWord)
                         : launchMevpStress32(s, dm, dops32, st32.u, st32.v, Pg, hP32, tdiv32, mp);
    }
    int chooseStress32();
    float* tdiv32 = nullptr;
    MevpNodeState32 st32 {};
    // FP32 u, v and divergence at the start of the previous sub-cycle (the
    // warm-start features), refreshed by every mixed-precision mEVP update
    float *uLast = nullptr, *vLast = nullptr, *tdivLast = nullptr;
    bool mixed() const { return P.precision == NSDG_PRECISION_MIXED; }
    double *partials = nullptr, *dsum = nullptr;
    int* derr = nullptr;
    // pinned host copy of derr (a pageable target would make the read a
    // staged, synchronous copy) and the event set_data waits on
    int* hErr = nullptr;
    cudaEvent_t copied = nullptr;
    // set_data's host copies run on copyStream into two staging buffers in
    // turn, so that a copy overlaps the conversion of the one before it;
    // converted[i]: the last conversion that read staging buffer i
    cudaStream_t copyStream = nullptr;
    cudaEvent_t converted[2] = { nullptr, nullptr };
    double* stage2 = nullptr;
    int stageSlot = 0;
    // nsdg_kernel_module_step's staging for all of a step's inputs at once
    double* moduleStage = nullptr;
    size_t moduleStageDoubles = 0;
    // graph of one update
    cudaGraphExec_t graph = nullptr;
    double graphDt = -1.0;
    int launchesPerUpdate = 0;
    // fields stored but not advected (DynamicsKernel::advectedFields)
    std::unordered_map<std::string, std::vector<double>> bucket;
    std::unordered_map<std::string, int> bucketComps;
    size_t stepNumber = 0;
    // read-out projections kept until the state changes: bit 1 = u, v in
    // (velx, vely), bit 2 = the ice-ocean stress in phiA (work arrays that are
    // free outside an update)
    int readCache = 0;
    // learned warm start (mixed-precision mEVP): the attached network, the
    // iteration count after it, the acceptance bound, the audit schedule,
    // backups of the sub-cycle's starting state, the previous sub-cycle's
    // starting state (features) and the device-side decision record
    NetImpl* warmNet = nullptr;
    int warmK = 0;
    double warmKappa = 0.0;
    int auditEvery = 0;
    double auditTol = 0.0;
    long long warmSteps = 0;   // updates since attaching
    void* warmMem = nullptr;
    float *bu = nullptr, *bv = nullptr, *btdiv = nullptr, *uPrev = nullptr, *vPrev = nullptr;
    float* wbase = nullptr;
    double *wPart = nullptr, *wRes = nullptr;
    WarmRecord rec {};
    cudaGraphExec_t auditGraph = nullptr;
    int auditLaunches = 0;
    int warmBodyLaunches = 0;

    int fail(int code, const std::string& m)
    {
        err = m;
        return code;
    }
    int ok()
    {
        err.clear();
        return NSDG_OK;
    }
    void dropGraphs()
    {
        if (graph)
            cudaGraphExecDestroy(graph);
        if (auditGraph)
            cudaGraphExecDestroy(auditGraph);
        graph = auditGraph = nullptr;
        graphDt = -1.0;
        launchesPerUpdate = 0;
    }
    void releaseWarm()
    {
        if (warmMem)
            cudaFree(warmMem);
        warmMem = nullptr;
        warmNet = nullptr;
        warmK = 0;
    }
    void releaseDevice()
    {
        releaseWarm();
        if (auditGraph)
            cudaGraphExecDestroy(auditGraph);
        auditGraph = nullptr;
        if (graph)
            cudaGraphExecDestroy(graph);
        graph = nullptr;
        graphDt = -1.0;
        if (copyStream)
            cudaStreamSynchronize(copyStream);
        arena.release();
        if (copied)
            cudaEventDestroy(copied);
        copied = nullptr;
        for (auto& c : converted) {
            if (c)
                cudaEventDestroy(c);
            c = nullptr;
        }
        if (copyStream)
            cudaStreamDestroy(copyStream);
        copyStream = nullptr;
        stageSlot = 0;
        if (moduleStage)
            cudaFree(moduleStage);
        moduleStage = nullptr;
        moduleStageDoubles = 0;
        if (hErr)
            cudaFreeHost(hErr);
        hErr = nullptr;
        if (stream)
            cudaStreamDestroy(stream);
        stream = nullptr;
        ready = false;
    }
    int initialise(size_t nx, size_t ny, const double* coords, int spherical, const double* mask);
    // Phases of one model step: everything before the sub-cycle, the
    // sub-cycle, and what follows it (the ensemble runs the sub-cycle of all
    // its members as batched launches between the other two).
    enum Phase { PHASE_PREP = 1, PHASE_LOOP = 2, PHASE_FINISH = 4, PHASE_ALL = 7 };
    int enqueuePhases(cudaStream_t s, double dt, int phases, int& launches);
    int enqueueUpdate(double dt, int& launches) { return enqueuePhases(stream, dt, PHASE_ALL, launches); }
    int ensureGraph(double dt);
    MevpParams mevpParams(double dt) const
    {
        return MevpParams { P.rho_ice, P.F_atm, P.F_ocean, P.fc, P.gravity, P.Pstar, P.DeltaMin, P.alpha, P.beta, dt };
    }
    // `count` mixed-precision mEVP iterations, numeric faults to `errWord`
    int mixedIterations(cudaStream_t s, double dt, int count, int* errWord, int& launches);
    WarmState warmState() const;
    int allocWarm();
    int saveLast(cudaStream_t s, float* bu_, float* bv_, float* btdiv_);
    int enqueueWarmFront(cudaStream_t s, double dt, int& launches);
    int captureWarmGraph(double dt, cudaGraph_t& g, int& launches);
    int captureAuditGraph(double dt, cudaGraph_t& g, int& launches);
    int launchStep(double dt);
    int checkDeviceError();
    // setData's device target for a field name: CG2 node values (cg, by the
    // DG -> CG2 interpolation) or DG components (dg, comps of them); neither
    // for a field that is only stored (DynamicsKernel.hpp:104-109)
    struct SetTarget {
        double* cg = nullptr;
        double* dg = nullptr;
        int comps = 0;
    };
    SetTarget setTarget(const std::string& s);
    void storeField(const std::string& s, const double* data, size_t nComp);
    // the conversion of a field copied to `staging` into its target, on `stream`
    int enqueueConversion(const SetTarget& t, const double* staging, size_t nComp);
    // the cell averages of a field into host memory `out`: projections and
    // the copy enqueued on `stream` (a stored field is copied at once)
    int enqueueReadout(const std::string& s, double* out, HostMoves* batch = nullptr);
    // the GPU reads and writes pageable host memory directly (Grace: address
    // translation over the CPU-GPU link; NSDG_HOST_DIRECT=0 turns it off):
    // host arrays that are not page-locked then move by a kernel, which runs
    // at the link's rate, instead of a copy staged through a driver buffer
    bool hostDirect = false;
    static bool isPageable(const void* p)
    {
        cudaPointerAttributes a {};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return a.type == cudaMemoryTypeUnregistered;
    }
    bool moveByKernel(const void* p) const { return hostDirect && isPageable(p); }
};

int nsdg_kernel::checkDeviceError()
{
    CUDA_TRY(cudaMemcpyAsync(hErr, derr, sizeof(int), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaStreamSynchronize(stream));
    const int h = *hErr;
    if (h) {
        CUDA_TRY(cudaMemsetAsync(derr, 0, sizeof(int), stream));
        std::string m = "non-finite values detected on the device:";
        if (h & DEV_ERR_NONFINITE_VELOCITY)
            m += " velocity";
        if (h & DEV_ERR_NONFINITE_STRESS)
            m += " stress";
        if (h & DEV_ERR_TIMEOUT)
            return fail(NSDG_ERR_CUDA, "a bounded wait for an asynchronous copy ran out on the device");
        return fail(NSDG_ERR_NUMERIC, m);
    }
    return NSDG_OK;
}

int nsdg_kernel::initialise(size_t nx, size_t ny, const double* coords, int spherical, const double* mask)
{
    if (!coords || !mask)
        return fail(NSDG_ERR_BAD_ARG, "initialise: null coords or mask");
    if (spherical && rheology == NSDG_RHEOLOGY_BBM)
        // the BBM's element size is sqrt(area) of the raw vertex coordinates
        // (ParametricMesh.hpp:276-299, BBMStressUpdateStep.hpp:134,158): in
        // radians on a sphere, which makes its relaxation times meaningless
        return fail(NSDG_ERR_UNSUPPORTED, "initialise: BBM on spherical coordinates is not supported "
                                          "(its element size would be in radians)");
    if (nx < 2 || ny < 2)
        return fail(NSDG_ERR_BAD_ARG, "initialise: the mesh needs nx >= 2 and ny >= 2");
    {
        std::string m;
        const int st = deviceCheck(m);
        if (st != NSDG_OK)
            return fail(st, m);
    }
    releaseDevice();
    bucket.clear();
    bucketComps.clear();
    stepNumber = 0;
    readCache = 0;

    // --- host mesh (DynamicsKernel.hpp:44-75) ---
    mesh = HostMesh();
    mesh.spherical = spherical != 0;
    mesh.nx = nx;
    mesh.ny = ny;
    const size_t nn = (nx + 1) * (ny + 1);
    mesh.vx.resize(nn);
    mesh.vy.resize(nn);
    for (size_t i = 0; i < nn; ++i) {
        mesh.vx[i] = coords[2 * i];
        mesh.vy[i] = coords[2 * i + 1];
        if (!std::isfinite(mesh.vx[i]) || !std::isfinite(mesh.vy[i]))
            return fail(NSDG_ERR_BAD_ARG, "initialise: non-finite coordinate");
    }
    // spherical meshes: (lon, lat) in radians, poles moved to Greenland /
    // Antarctica as DynamicsKernel::initialise does (DynamicsKernel.hpp:49-51)
    if (mesh.spherical)
        mesh.rotatePoleToGreenland();
    N = nx * ny;
    mesh.ice.resize(N);
    for (size_t i = 0; i < N; ++i)
        mesh.ice[i] = (mask[i] == 1.0) ? 1 : 0;
    mesh.dirichletFromMaskAndEdges();
    const std::string fm = buildBoundaryFlags(mesh, flags);
    if (!fm.empty())
        return fail(NSDG_ERR_BAD_ARG, "initialise: " + fm);
    ElementOps ops;
    const bool bbm = rheology == NSDG_RHEOLOGY_BBM;
    buildElementOps(mesh, dg, bbm, ops);
    for (size_t i = 0; i < N; ++i) {
        const size_t e = i;
        for (int q = 0; q < 9; ++q)
            if (!(ops.jw3[q * N + e] > 0.0))
                return fail(NSDG_ERR_BAD_ARG, "initialise: element " + std::to_string(e) + " is degenerate or inverted");
    }

    Ncg = (2 * nx + 1) * (2 * ny + 1);
    Ncg1 = (nx + 1) * (ny + 1);
    const int Qa = gaussPoints1d(dg);
    const size_t nXe = nx * (ny + 1), nYe = (nx + 1) * ny;
    const int ED = edgeDofs(dg);

    // --- size the arena ---
    size_t bytes = 0;
    auto add = [&](size_t n, size_t sz = sizeof(double)) { bytes += al(n * sz); };
    // mesh
    add(nn, 8); add(nn, 8);
    add(N, 1); add(N, 1); add(nXe, 1); add(nYe, 1); add(Ncg, 1);
    add(N + 1, 4); add(std::max<size_t>(flags.perEntry.size(), 1), 4);
    // ops
    add(ops.cellX.size()); add(ops.cellY.size()); add(ops.minv.size()); add(ops.jwA.size()); add(ops.jw3.size());
    add(ops.gx.size()); add(ops.gy.size()); add(ops.a1.size()); add(ops.a2.size());
    if (bbm) {
        add(ops.w.size()); add(ops.d1.size()); add(ops.d2.size());
    }
    add(ops.dxssh.size()); add(ops.dyssh.size()); add(Ncg); add(Ncg1);
    if (mesh.spherical) {
        add(ops.gm.size()); add(ops.a3.size() + 1); add(ops.dm.size() + 1);
        add(ops.minvP.size()); add(ops.minv8P.size() + 1);
    }
    if (bbm) {
        add(ops.cellX8.size()); add(ops.cellY8.size()); add(ops.minv8.size()); add(ops.wdam.size()); add(ops.hsize.size());
    }
    // state and work
    add(size_t(dg) * N); add(size_t(dg) * N); add(N); add(size_t(dg) * N);
    add(8 * N); add(8 * N); add(8 * N);
    for (int i = 0; i < 25; ++i) add(Ncg);
    add(9 * N); add(18 * N);
    add(size_t(dg) * N); add(size_t(dg) * N); add(ED * nXe); add(ED * nYe);
    add(3 * size_t(dg) * N); add(3 * size_t(dg) * N);
    if (bbm) {
        add(8 * N); add(8 * N); add(3 * nXe); add(3 * nYe); add(24 * N); add(24 * N);
    }
    add(3 * Ncg1); add(8 * N); add(8 * N); add(8 * N); add(Ncg);
    if (P.precision == NSDG_PRECISION_FP64 && !bbm && !mesh.spherical)
        add(324 * pairsLd(N), 8);                 // float-pair stress operators
    if (P.precision == NSDG_PRECISION_MIXED && !bbm) {
        add((mesh.spherical ? 486 : 324) * ops32Ld(N), 4);
        add(5 * ops32Ld(N), 4);                   // parallelogram coefficients
        add(18 * N, 4);
        for (int i = 0; i < 4; ++i) add(Ncg, 4);  // FP32 u, v, u0, v0
        add(8 * Ncg, 4);                          // the packed per-step node constants
        add(18 * N, 4); add(Ncg, 4); add(Ncg, 4); // start of the previous sub-cycle
        add(9 * N, 4);                            // P/(2 alpha)
        add(size_t(dg) * N);                      // diagonal of M^{-1} (parallelogram transport)
    }
    if (P.precision == NSDG_PRECISION_MIXED) {
        add(ops.cellX.size(), 4); add(ops.cellY.size(), 4); // FP32 transport operators
        add(ops.jwA.size(), 4);                             // FP32 J w of the CG2DG quadrature
        add(Ncg, 8);                                        // inverse lumped mass {hi, lo}
    }
    if (P.precision == NSDG_PRECISION_MIXED && bbm) {
        add(5 * ops32Ld(N), 4);                   // parallelogram coefficients
        add(4 * Ncg, 4); add(4 * Ncg, 4);         // the node constants of the sub-steps
        add(ops.gx.size(), 4); add(ops.gy.size(), 4); add(ops.w.size(), 4); add(ops.wdam.size(), 4);
        add(ops.d1.size(), 4); add(ops.d2.size(), 4); add(ops.cellX8.size(), 4); add(ops.cellY8.size(), 4);
        if (mesh.spherical) {
            add(ops.gm.size(), 4); add(ops.dm.size(), 4);
        }
    }
    add((N + 255) / 256 + 1); add(1); add(1, 4);
    bytes += 4096;

    CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    CUDA_TRY(cudaStreamCreateWithFlags(&copyStream, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&copied, cudaEventDisableTiming));
    for (auto& c : converted)
        CUDA_TRY(cudaEventCreateWithFlags(&c, cudaEventDisableTiming));
    CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&hErr), sizeof(int), cudaHostAllocDefault));
    *hErr = 0;
    CUDA_TRY(uploadConstTables());
    CUDA_TRY(arena.reserve(bytes));

    auto up = [&](const void* src, size_t n, size_t sz, cudaError_t& e) -> void* {
        void* p = nullptr;
        if (sz == 8) p = arena.take<double>(n);
        else if (sz == 4) p = arena.take<int>(n);
        else p = arena.take<uint8_t>(n);
        if (!p) { e = cudaErrorMemoryAllocation; return nullptr; }
        if (src && n) e = cudaMemcpyAsync(p, src, n * sz, cudaMemcpyHostToDevice, stream);
        return p;
    };
    cudaError_t e = cudaSuccess;
    dm.nx = static_cast<int>(nx);
    dm.ny = static_cast<int>(ny);
    dm.spherical = mesh.spherical ? 1 : 0;
    dm.N = N;
    dm.Ncg = Ncg;
    dm.Ncg1 = Ncg1;
    dm.nXe = nXe;
    dm.nYe = nYe;
    dm.vx = static_cast<const double*>(up(mesh.vx.data(), nn, 8, e));
    dm.vy = static_cast<const double*>(up(mesh.vy.data(), nn, 8, e));
    dm.ice = static_cast<const uint8_t*>(up(mesh.ice.data(), N, 1, e));
    dm.cellSeg = static_cast<const uint8_t*>(up(flags.cellSeg.data(), N, 1, e));
    dm.edgeXCount = static_cast<const uint8_t*>(up(flags.edgeXCount.data(), nXe, 1, e));
    dm.edgeYCount = static_cast<const uint8_t*>(up(flags.edgeYCount.data(), nYe, 1, e));
    dm.cg2Dir = static_cast<const uint8_t*>(up(flags.cg2Dirichlet.data(), Ncg, 1, e));
    dm.perPtr = static_cast<const int*>(up(flags.perPtr.data(), N + 1, 4, e));
    dm.perEntry = static_cast<const int*>(up(flags.perEntry.empty() ? nullptr : flags.perEntry.data(),
        std::max<size_t>(flags.perEntry.size(), 1), 4, e));
    auto upd = [&](const std::vector<double>& vsrc) {
        return static_cast<const double*>(up(vsrc.data(), vsrc.size(), 8, e));
    };
    dops.cellX = upd(ops.cellX);
    dops.cellY = upd(ops.cellY);
    dops.minv = upd(ops.minv);
    dops.jwA = upd(ops.jwA);
    dops.jw3 = upd(ops.jw3);
    dops.gx = upd(ops.gx);
    dops.gy = upd(ops.gy);
    dops.a1 = upd(ops.a1);
    dops.a2 = upd(ops.a2);
    if (bbm) {
        dops.w = upd(ops.w);
        dops.d1 = upd(ops.d1);
        dops.d2 = upd(ops.d2);
    }
    if (mesh.spherical) {
        dops.minvP = upd(ops.minvP);
        if (bbm)
            dops.minv8P = upd(ops.minv8P);
        dops.gm = upd(ops.gm);
        if (bbm)
            dops.dm = upd(ops.dm);
        else
            dops.a3 = upd(ops.a3);
    }
    dops.dxssh = upd(ops.dxssh);
    dops.dyssh = upd(ops.dyssh);
    std::vector<double> invm(Ncg);
    for (size_t i = 0; i < Ncg; ++i)
        invm[i] = 1.0 / ops.lumped2[i];
    dops.invm2 = upd(invm);
    dops.lumped1 = upd(ops.lumped1);
    if (bbm) {
        dops.cellX8 = upd(ops.cellX8);
        dops.cellY8 = upd(ops.cellY8);
        dops.minv8 = upd(ops.minv8);
        dops.wdam = upd(ops.wdam);
        dops.hsize = upd(ops.hsize);
    }
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("initialise: upload failed: ") + cudaGetErrorString(e));
    auto z = [&](size_t n) {
        double* p = arena.take<double>(n);
        if (p && e == cudaSuccess)
            e = cudaMemsetAsync(p, 0, n * sizeof(double), stream);
        if (!p)
            e = cudaErrorMemoryAllocation;
        return p;
    };
    hice = z(size_t(dg) * N);
    cice = z(size_t(dg) * N);
    ssh = z(N);
    damage = z(size_t(dg) * N);
    s11 = z(8 * N);
    s12 = z(8 * N);
    s22 = z(8 * N);
    u = z(Ncg); v = z(Ncg); uo = z(Ncg); vo = z(Ncg); ua = z(Ncg); va = z(Ncg);
    avgU = z(Ncg); avgV = z(Ncg); u0 = z(Ncg); v0 = z(Ncg); cgH = z(Ncg); cgA = z(Ncg);
    uGrad = z(Ncg); vGrad = z(Ncg); c1 = z(Ncg); c1b = z(Ncg); fau = z(Ncg); fav = z(Ncg);
    rhfc = z(Ncg); gu = z(Ncg); gv = z(Ncg);
    Pg = z(9 * N);
    contrib = z(18 * N);
    velx = z(size_t(dg) * N);
    vely = z(size_t(dg) * N);
    nvX = z(ED * nXe);
    nvY = z(ED * nYe);
    phiA = z(3 * size_t(dg) * N);
    k1 = z(3 * size_t(dg) * N);
    if (bbm) {
        velx8 = z(8 * N);
        vely8 = z(8 * N);
        nvX8 = z(3 * nXe);
        nvY8 = z(3 * nYe);
        sA = z(24 * N);
        sK1 = z(24 * N);
    }
    sshScratch = z(3 * Ncg1);
    staging = z(8 * N);
    stage2 = z(8 * N);
    dgTmp = z(8 * N);
    cgTmp = z(Ncg);
    partials = z((N + 255) / 256 + 1);
    dsum = z(1);
    if (P.precision == NSDG_PRECISION_FP64 && !bbm && !mesh.spherical) {
        // NSDG_FP64_STRESS=pairs or pairs_tma selects a float-pair stress kernel
        const char* env = std::getenv("NSDG_FP64_STRESS");
        fp64Stress = !env ? 0 : std::strcmp(env, "pairs") == 0 ? 1 : std::strcmp(env, "pairs_tma") == 0 ? 2 : 0;
        pairsLdN = pairsLd(N);
        opsPairs = arena.take<float2>(324 * pairsLdN);
        if (!opsPairs && e == cudaSuccess)
            e = cudaErrorMemoryAllocation;
        const double* src[4] = { dops.gx, dops.gy, dops.a1, dops.a2 };
        for (int b = 0; b < 4 && e == cudaSuccess; ++b)
            e = launchSplitPairs(stream, 81, N, pairsLdN, src[b], opsPairs + b * 81 * pairsLdN);
        if (e == cudaSuccess)
            e = makePairsMaps(opsPairs, pairsLdN, &pairsMaps);
    }
    auto upf = [&](const std::vector<double>& src) {
        std::vector<float> tmp(src.begin(), src.end());
        float* p = arena.take<float>(tmp.size());
        if (!p) { e = cudaErrorMemoryAllocation; return p; }
        if (e == cudaSuccess) e = cudaMemcpy(p, tmp.data(), tmp.size() * sizeof(float), cudaMemcpyHostToDevice);
        return p;
    };
    if (mixed()) {
        const char* tenv = std::getenv("NSDG_MIXED_TRANSPORT");
        transport32 = !(tenv && std::strcmp(tenv, "fp64") == 0);
        cellX32 = upf(ops.cellX);
        cellY32 = upf(ops.cellY);
        jwA32 = upf(ops.jwA);
        std::vector<float2> hl(Ncg);
        for (size_t i = 0; i < Ncg; ++i) {
            const float hi = static_cast<float>(invm[i]);
            hl[i] = make_float2(hi, static_cast<float>(invm[i] - static_cast<double>(hi)));
        }
        invmHL = arena.take<float2>(Ncg);
        if (!invmHL)
            e = cudaErrorMemoryAllocation;
        else if (e == cudaSuccess)
            e = cudaMemcpy(invmHL, hl.data(), Ncg * sizeof(float2), cudaMemcpyHostToDevice);
    }
    if (mixed() && bbm) {
        bbm32.gx = upf(ops.gx);
        bbm32.gy = upf(ops.gy);
        bbm32.w = upf(ops.w);
        bbm32.wdam = upf(ops.wdam);
        bbm32.d1 = upf(ops.d1);
        bbm32.d2 = upf(ops.d2);
        bbm32.gm = mesh.spherical ? upf(ops.gm) : nullptr;
        bbm32.dm = mesh.spherical ? upf(ops.dm) : nullptr;
        cellX8_32 = upf(ops.cellX8);
        cellY8_32 = upf(ops.cellY8);
        bbmConst.k0 = arena.take<float4>(Ncg);
        bbmConst.k1 = arena.take<float4>(Ncg);
        if (!bbmConst.k0 || !bbmConst.k1)
            e = cudaErrorMemoryAllocation;
        bbmK0 = bbmConst.k0 && bbmConst.k1;
        // parallelogram meshes: 5 coefficients per element and the unit
        // square's operators replace the per-element ones in the stress
        // kernel (NSDG_BBM_STRESS_KERNEL=general keeps those)
        const char* bk = std::getenv("NSDG_BBM_STRESS_KERNEL");
        if (!mesh.spherical && !(bk && std::strcmp(bk, "general") == 0)) {
            AffineStressOps aff;
            AffineBbmOps abb;
            const size_t ld = ops32Ld(N);
            const bool okS = buildAffineStressOps(mesh, ops, ld, 1e-9, aff);
            const bool okB = okS && buildAffineBbmOps(mesh, ops, 1e-9, abb);
            affWorst = std::max(aff.worst, abb.worst);
            if (okS && okB) {
                float* coef = arena.take<float>(aff.coef.size());
                if (!coef)
                    e = cudaErrorMemoryAllocation;
                else if (e == cudaSuccess)
                    e = cudaMemcpy(coef, aff.coef.data(), aff.coef.size() * sizeof(float), cudaMemcpyHostToDevice);
                if (e == cudaSuccess)
                    e = uploadAffineReference(aff.ref);
                if (e == cudaSuccess)
                    e = uploadAffineBbmReference(abb.w, abb.wdam, dg, abb.dxi, abb.deta);
                if (e == cudaSuccess) {
                    bbm32.coef = coef;
                    bbm32.ld = ld;
                }
            }
        }
    }
    if (mixed() && !bbm) {
        {
            // one block of 81-row operators, rows padded to ld: G_x, G_y, A_1, A_2
            // ([324][ld]); on a sphere G_x, G_y, G_m, A_1, A_2, A_3 ([486][ld])
            const size_t ld = ops32Ld(N);
            const bool sph = mesh.spherical;
            const int nb = sph ? 6 : 4;
            std::vector<float> blk(size_t(81) * nb * ld, 0.f);
            const std::vector<double>* src4[4] = { &ops.gx, &ops.gy, &ops.a1, &ops.a2 };
            const std::vector<double>* src6[6] = { &ops.gx, &ops.gy, &ops.gm, &ops.a1, &ops.a2, &ops.a3 };
            for (int b = 0; b < nb; ++b) {
                const std::vector<double>& o = sph ? *src6[b] : *src4[b];
                for (size_t r = 0; r < 81; ++r)
                    for (size_t el = 0; el < N; ++el)
                        blk[(81 * b + r) * ld + el] = static_cast<float>(o[r * N + el]);
            }
            float* p = arena.take<float>(blk.size());
            if (!p)
                e = cudaErrorMemoryAllocation;
            else if (e == cudaSuccess)
                e = cudaMemcpy(p, blk.data(), blk.size() * sizeof(float), cudaMemcpyHostToDevice);
            const size_t gRows = sph ? 243 : 162;
            dops32.ld = ld;
            dops32.rowsG = static_cast<int>(gRows);
            dops32.gx = p;
            dops32.gy = p ? p + 81 * ld : nullptr;
            dops32.gm = (p && sph) ? p + 162 * ld : nullptr;
            dops32.a1 = p ? p + gRows * ld : nullptr;
            dops32.a2 = p ? p + (gRows + 81) * ld : nullptr;
            dops32.a3 = (p && sph) ? p + (gRows + 162) * ld : nullptr;
            if (e == cudaSuccess)
                e = makeStressMaps(dops32, &maps32);
        }
        if (!mesh.spherical) {
            // parallelogram meshes: 5 coefficients per element replace the
            // operator block (the rebuilt operators must match the exact
            // ones far below FP32 rounding)
            AffineStressOps aff;
            const size_t ld = ops32Ld(N);
            if (buildAffineStressOps(mesh, ops, ld, 1e-9, aff)) {
                affCoef = arena.take<float>(aff.coef.size());
                if (!affCoef)
                    e = cudaErrorMemoryAllocation;
                else if (e == cudaSuccess)
                    e = cudaMemcpy(affCoef, aff.coef.data(), aff.coef.size() * sizeof(float), cudaMemcpyHostToDevice);
                if (e == cudaSuccess)
                    e = uploadAffineReference(aff.ref);
                affLd = ld;
            }
            affWorst = aff.worst;
            // the transport on the same coefficients: the rebuilt cell
            // operators within 1e-9 of the exact ones (far below FP32
            // rounding), M^{-1} diagonal to 1e-12 of its diagonal
            const char* tk = std::getenv("NSDG_TRANSPORT_KERNEL");
            if (affCoef && transport32 && flags.perEntry.empty()) {
                AffineTransportOps atr;
                const bool fits = buildAffineTransportOps(mesh, ops, 1e-9, 1e-12, atr);
                trAffWorst[0] = atr.worstCell;
                trAffWorst[1] = atr.worstOffDiag;
                if (fits && !(tk && std::strcmp(tk, "element") == 0)) {
                    minvDiag = arena.take<double>(atr.minvDiag.size());
                    if (!minvDiag)
                        e = cudaErrorMemoryAllocation;
                    else if (e == cudaSuccess)
                        e = cudaMemcpy(minvDiag, atr.minvDiag.data(), atr.minvDiag.size() * sizeof(double),
                            cudaMemcpyHostToDevice);
                    if (e == cudaSuccess)
                        e = uploadAffineTransportReference(dg, atr.ref);
                    trAffine = e == cudaSuccess;
                }
            }
        }
        auto zf = [&](size_t n) {
            float* p = arena.take<float>(n);
            if (!p) { e = cudaErrorMemoryAllocation; return p; }
            if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, n * sizeof(float), stream);
            return p;
        };
        tdiv32 = zf(18 * N);
        float** f32[] = { &st32.u, &st32.v, &st32.u0, &st32.v0 };
        for (float** q : f32)
            *q = zf(Ncg);
        st32.k0 = reinterpret_cast<float4*>(zf(4 * Ncg));
        st32.k1 = reinterpret_cast<float4*>(zf(4 * Ncg));
        tdivLast = zf(18 * N);
        uLast = zf(Ncg);
        vLast = zf(Ncg);
        hP32 = zf(9 * N);
    }
    derr = arena.take<int>(1);
    if (!derr)
        e = cudaErrorMemoryAllocation;
    else if (e == cudaSuccess)
        e = cudaMemsetAsync(derr, 0, sizeof(int), stream);
    (void)Qa;
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("initialise: allocation failed: ") + cudaGetErrorString(e));
    CUDA_TRY(cudaStreamSynchronize(stream));
    if (mixed() && rheology == NSDG_RHEOLOGY_MEVP) {
        const int r = chooseStress32();
        if (r)
            return r;
    }
    {
        int dev = 0, pageableAccess = 0;
        const char* hd = std::getenv("NSDG_HOST_DIRECT");
        hostDirect = cudaGetDevice(&dev) == cudaSuccess
            && cudaDeviceGetAttribute(&pageableAccess, cudaDevAttrPageableMemoryAccess, dev) == cudaSuccess
            && pageableAccess == 1 && !(hd && std::strcmp(hd, "0") == 0);
        cudaGetLastError();
    }
    ready = true;
    return ok();
}

// Picks the FP32 stress kernel.  A parallelogram mesh takes the coefficient
// kernel (5 coefficients instead of 324 operator entries per element; its
// results differ from the others' by FP32 rounding only, and ensembles of
// such members take it too, so a member's single run and its ensemble run
// agree bit for bit).  Otherwise the two operator kernels (tiles through TMA
// into shared memory, or direct global loads), which compute identical
// values, are timed on this mesh and the faster is kept: which wins depends
// on the grid size and the number of resident blocks.
int nsdg_kernel::chooseStress32()
{
    // NSDG_STRESS_KERNEL=global|tma|affine fixes the choice (for profilers,
    // whose serialised launches make the timing below meaningless)
    // NSDG_VISC_FORM=0..4 fixes the FP64 viscosity form of the
    // parallelogram kernel (0 rsqrt, 1 Newton, 2 Newton with integer
    // conversions, 3 float pairs, 4 float pairs checked against form 2 with
    // form 2 where the check fails: bitwise form 2)
    if (const char* env = std::getenv("NSDG_VISC_FORM")) {
        const int f = std::atoi(env);
        if (f >= 0 && f <= 4)
            viscMode = f;
    }
    if (const char* env = std::getenv("NSDG_STRESS_KERNEL")) {
        const char* names[3] = { "global", "tma", "affine" };
        for (int i = 0; i < 3; ++i)
            if (std::strcmp(env, names[i]) == 0 && (i < 2 || affCoef)) {
                stressKind = i;
                return NSDG_OK;
            }
    }
    if (affCoef) {
        stressKind = 2;
        return NSDG_OK;
    }
    const MevpParams mp = mevpParams(120.0);
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
        return fail(NSDG_ERR_CUDA, "initialise: event create failed");
    float best[2] = { 0, 0 };
    const int kinds = 2;
    cudaError_t e = cudaSuccess;
    for (int variant = 0; variant < kinds && e == cudaSuccess; ++variant) {
        e = launchStress32(stream, mp, derr, variant);
        if (e == cudaSuccess) e = cudaEventRecord(a, stream);
        for (int r = 0; r < 10 && e == cudaSuccess; ++r)
            e = launchStress32(stream, mp, derr, variant);
        if (e == cudaSuccess) e = cudaEventRecord(b, stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&best[variant], a, b);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    // the timing launches updated the divergence of the (zero) initial state: reset it
    if (e == cudaSuccess) e = cudaMemsetAsync(tdiv32, 0, 18 * N * sizeof(float), stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("initialise: stress kernel timing: ") + cudaGetErrorString(e));
    stressKind = 0;
    for (int variant = 1; variant < kinds; ++variant)
        if (best[variant] <= best[stressKind])
            stressKind = variant;
    return NSDG_OK;
}

int nsdg_kernel::enqueuePhases(cudaStream_t s, double dt, int phases, int& launches)
{
    launches = 0;
    cudaError_t e;
#define LCH(expr)                                                                                  \
    do {                                                                                           \
        e = (expr);                                                                                \
        if (e != cudaSuccess)                                                                      \
            return fail(NSDG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e));       \
        ++launches;                                                                                \
    } while (0)
    const size_t dN = size_t(dg) * N;
    const bool bbm = rheology == NSDG_RHEOLOGY_BBM;
    const bool prep = (phases & PHASE_PREP) != 0, loop = (phases & PHASE_LOOP) != 0;
    const bool finish = (phases & PHASE_FINISH) != 0;
    if (prep) {
    // --- advection of cice, hice (and damage for BBM), with limits
    //     (DynamicsKernel.hpp:160-172; BrittleCGDynamicsKernel.hpp:89-106) ---
    {
        const double* cgv[2] = { bbm ? avgU : u, bbm ? avgV : v };
        double* dgv[2] = { velx, vely };
        if (mixed() && jwA32 && transport32)
            LCH(launchCG2DG32(s, dm, dg, jwA32, dops.minvP ? dops.minvP : dops.minv, cgv, dgv,
                trAffine ? minvDiag : nullptr));
        else
            LCH(launchCG2DG(s, dm, dg, dops.jwA, dops.minvP ? dops.minvP : dops.minv, 2, cgv, dgv));
        LCH(launchNormalVelocity(s, dm, dg, velx, vely, nvX, nvY));
        StageFields a, b;
        const int nf = bbm ? 3 : 2;
        double* fld[3] = { cice, hice, damage };
        a.nf = b.nf = nf;
        for (int k = 0; k < nf; ++k) {
            a.src[k] = fld[k];
            a.phi[k] = fld[k];
            a.k1[k] = k1 + k * dN;
            a.dst[k] = phiA + k * dN;
            b.src[k] = phiA + k * dN;
            b.phi[k] = fld[k];
            b.k1[k] = k1 + k * dN;
            b.dst[k] = fld[k];
        }
        b.lmax[0] = 1; b.vmax[0] = 1.0; b.lmin[0] = 1; b.vmin[0] = 0.0;  // cice
        b.lmin[1] = 1; b.vmin[1] = 0.0;                                   // hice
        if (bbm) { b.lmax[2] = 1; b.vmax[2] = 1.0; b.lmin[2] = 1; b.vmin[2] = 1e-12; } // damage
        LCH(launchTransport(s, STAGE_RK2_A, dt, a));
        LCH(launchTransport(s, STAGE_RK2_B, dt, b));
    }
    if (bbm) {
        // stress transport with DGTransport<8> (BrittleCGDynamicsKernel.hpp:98-101)
        const double* cgv[2] = { avgU, avgV };
        double* dgv[2] = { velx8, vely8 };
        LCH(launchCG2DG(s, dm, 8, dops.jw3, dops.minv8P ? dops.minv8P : dops.minv8, 2, cgv, dgv));
        LCH(launchNormalVelocity(s, dm, 8, velx8, vely8, nvX8, nvY8));
        StageFields a, b;
        double* fld[3] = { s11, s12, s22 };
        a.nf = b.nf = 3;
        for (int k = 0; k < 3; ++k) {
            a.src[k] = fld[k];
            a.phi[k] = fld[k];
            a.k1[k] = sK1 + k * 8 * N;
            a.dst[k] = sA + k * 8 * N;
            b.src[k] = sA + k * 8 * N;
            b.phi[k] = fld[k];
            b.k1[k] = sK1 + k * 8 * N;
            b.dst[k] = fld[k];
        }
        const float* cx8 = mixed() ? cellX8_32 : nullptr;
        const float* cy8 = mixed() ? cellY8_32 : nullptr;
        LCH(launchTransportStage(s, dm, 8, dops.cellX8, dops.cellY8, dops.minv8, velx8, vely8, nvX8,
            nvY8, STAGE_RK2_A, dt, a, cx8, cy8));
        LCH(launchTransportStage(s, dm, 8, dops.cellX8, dops.cellY8, dops.minv8, velx8, vely8, nvX8,
            nvY8, STAGE_RK2_B, dt, b, cx8, cy8));
    }
    // --- prepareIteration (CGDynamicsKernel.cpp:260-276) ---
    {
        const double* in[2] = { hice, cice };
        double* out[2] = { cgH, cgA };
        LCH(launchDG2CG(s, dm, dg, 2, in, out));
        e = launchSSHGradient(s, dm, dops, ssh, sshScratch, uGrad, vGrad);
        if (e != cudaSuccess)
            return fail(NSDG_ERR_CUDA, std::string("ssh gradient: ") + cudaGetErrorString(e));
        launches += 3;
    }
    } // prep
    const int nS = P.n_steps;
    if (!bbm) {
        const MevpParams mp = mevpParams(dt);
        MevpNodeState st { u, v, u0, v0, cgH, cgA, uo, vo, ua, va, uGrad, vGrad, c1, c1b, fau, fav, rhfc, gu, gv };
        if (prep) {
            // the mixed path forms its FP32 node constants in one kernel
            if (!mixed())
                LCH(launchMevpPrepNodes(s, dm, st, mp));
            // a full mixed-precision update also records the sub-cycle's
            // start (the warm-start features of the next update) inside
            // the two preparation kernels
            const bool save = loop && mixed();
            LCH(launchMevpPrepElements(s, dm, dg, hice, cice, Pg, mp, mixed() ? hP32 : nullptr,
                save ? tdiv32 : nullptr, save ? tdivLast : nullptr));
            if (mixed())
                LCH(launchMevpPrepNodes32(s, dm, st, st32, dops.invm2, mp, save ? uLast : nullptr,
                    save ? vLast : nullptr));
        }
        if (loop && mixed() && !prep) {
            const int sv = saveLast(s, nullptr, nullptr, nullptr);
            if (sv != NSDG_OK)
                return sv;
            launches += 3;
        }
        if (loop) {
            for (int it = 0; it < nS; ++it) {
                if (!mixed()) {
                    if (opsPairs && fp64Stress == 2)
                        LCH(launchMevpStressPairsTma(s, dm, pairsMaps, u, v, Pg, contrib, mp, derr));
                    else if (opsPairs && fp64Stress == 1)
                        LCH(launchMevpStressPairs(s, dm, opsPairs, pairsLdN, u, v, Pg, contrib, mp));
                    else
                        LCH(launchMevpStress(s, dm, dops, u, v, Pg, contrib, mp));
                    LCH(launchMevpMomentum(s, dm, dops, st, contrib, mp, derr));
                } else {
                    LCH(launchStress32(s, mp, derr));
                    LCH(launchMevpMomentum32(s, dm, st32, tdiv32, mp, derr));
                }
            }
        }
        if (finish && mixed())
            LCH(launchWidenVelocity(s, Ncg, st32.u, st32.v, u, v));
    } else if (phases == PHASE_ALL) {
        const double rad = 0x1.1df46a2529d39p-6;
        BbmParams bp { P.rho_ice, P.F_atm, P.F_ocean, P.fc, P.gravity, dt / nS, double(nS),
            std::cos(rad * P.ocean_turning_angle), std::sin(rad * P.ocean_turning_angle),
            P.compaction_param, P.nu0, P.young, P.P0, P.undamaged_time_relaxation_sigma,
            P.exponent_relaxation_sigma, P.exponent_compression_factor, P.tan_phi, P.compr_strength, P.C_lab };
        bbmPowModes(bp);
        BbmNodeState st { u, v, avgU, avgV, cgH, cgA, uo, vo, ua, va, uGrad, vGrad };
        const BbmNodeConst32* bc = (mixed() && bbmK0) ? &bbmConst : nullptr;
        LCH(launchBbmPrepNodes(s, dm, st, &bp, bc));
        for (int it = 0; it < nS; ++it) {
            LCH(launchBbmStress(s, dm, dops, dg, u, v, hice, cice, damage, s11, s12, s22, contrib, bp, derr,
                mixed() ? &bbm32 : nullptr));
            LCH(launchBbmMomentum(s, dm, dops, st, contrib, bp, derr, mixed() ? invmHL : nullptr, bc));
        }
    }
#undef LCH
    return NSDG_OK;
}

int nsdg_kernel::mixedIterations(cudaStream_t s, double dt, int count, int* errWord, int& launches)
{
    const MevpParams mp = mevpParams(dt);
    for (int it = 0; it < count; ++it) {
        cudaError_t e = launchStress32(s, mp, errWord);
        if (e == cudaSuccess)
            e = launchMevpMomentum32(s, dm, st32, tdiv32, mp, errWord);
        if (e != cudaSuccess)
            return fail(NSDG_ERR_CUDA, std::string("mEVP iteration: ") + cudaGetErrorString(e));
        launches += 2;
    }
    return NSDG_OK;
}

WarmState nsdg_kernel::warmState() const
{
    WarmState w {};
    w.nx = dm.nx;
    w.ny = dm.ny;
    w.N = N;
    w.hice = hice; // component 0 of [dg][N] is the cell average
    w.cice = cice;
    w.ice = dm.ice;
    w.cg2Dir = dm.cg2Dir;
    w.u = st32.u;
    w.v = st32.v;
    w.ua = ua;
    w.va = va;
    w.uo = uo;
    w.vo = vo;
    w.tdiv = tdiv32;
    w.uLast = uLast;
    w.vLast = vLast;
    w.tdivLast = tdivLast;
    return w;
}

int nsdg_kernel::allocWarm()
{
    if (warmMem)
        return NSDG_OK;
    auto a = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t nPart = warmResidualPartials(Ncg);
    const size_t bytes = 4 * a(Ncg * 4) + a(18 * N * 4) + a(N * kWarmUsed * 4) + a(nPart * 8) + a(2 * 8)
        + a(4 * 8) + 2 * a(4) + 2 * a(8);
    cudaError_t e = cudaMalloc(&warmMem, bytes);
    if (e != cudaSuccess) {
        warmMem = nullptr;
        return fail(NSDG_ERR_CUDA, std::string("warm start: allocation failed: ") + cudaGetErrorString(e));
    }
    char* p = static_cast<char*>(warmMem);
    auto take = [&](size_t b) { void* r = p; p += a(b); return r; };
    bu = static_cast<float*>(take(Ncg * 4));
    bv = static_cast<float*>(take(Ncg * 4));
    uPrev = static_cast<float*>(take(Ncg * 4));
    vPrev = static_cast<float*>(take(Ncg * 4));
    btdiv = static_cast<float*>(take(18 * N * 4));
    wbase = static_cast<float*>(take(N * kWarmUsed * 4));
    wPart = static_cast<double*>(take(nPart * 8));
    wRes = static_cast<double*>(take(2 * 8));
    rec.counts = static_cast<long long*>(take(4 * 8));
    rec.warmErr = static_cast<int*>(take(4));
    rec.enabled = static_cast<int*>(take(4));
    rec.lastRatio = static_cast<double*>(take(8));
    rec.lastError = static_cast<double*>(take(8));
    e = cudaMemset(warmMem, 0, bytes);
    if (e == cudaSuccess) {
        const int one = 1;
        e = cudaMemcpy(rec.enabled, &one, sizeof(int), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("warm start: ") + cudaGetErrorString(e));
    return NSDG_OK;
}

// (uLast, vLast, tdivLast) := the current sub-cycle's start, also copied to
// the backups when given
int nsdg_kernel::saveLast(cudaStream_t s, float* bu_, float* bv_, float* btdiv_)
{
    cudaError_t e = launchWarmSave(s, Ncg, st32.u, uLast, bu_);
    if (e == cudaSuccess) e = launchWarmSave(s, Ncg, st32.v, vLast, bv_);
    if (e == cudaSuccess) e = launchWarmSave(s, 18 * N, tdiv32, tdivLast, btdiv_);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("save sub-cycle start: ") + cudaGetErrorString(e));
    return NSDG_OK;
}

// prep phase; features (network input); back up the sub-cycle's start into
// (bu, bv, btdiv) and (uLast, vLast, tdivLast); network; increments; K
// iterations with the warm error word, keeping the iterate before the last
int nsdg_kernel::enqueueWarmFront(cudaStream_t s, double dt, int& launches)
{
    int l = 0;
    int st = enqueuePhases(s, dt, PHASE_PREP, l);
    launches += l;
    if (st != NSDG_OK)
        return st;
    const WarmState ws = warmState();
    cudaError_t e = launchWarmFeaturesNet(s, ws, warmNet);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("warm start: ") + cudaGetErrorString(e));
    st = saveLast(s, bu, bv, btdiv);
    if (st != NSDG_OK)
        return st;
    e = netForward(warmNet, s, 1);
    if (e == cudaSuccess) e = launchWarmApply(s, ws, warmNet);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("warm start: ") + cudaGetErrorString(e));
    launches += 5 + netLayers(warmNet);
    st = mixedIterations(s, dt, warmK - 1, rec.warmErr, launches);
    if (st != NSDG_OK)
        return st;
    e = launchWarmSave(s, Ncg, st32.u, uPrev, nullptr);
    if (e == cudaSuccess) e = launchWarmSave(s, Ncg, st32.v, vPrev, nullptr);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("warm start: ") + cudaGetErrorString(e));
    launches += 2;
    return mixedIterations(s, dt, 1, rec.warmErr, launches);
}

// One update with the warm start, as a graph with a device-side fallback:
//   A: warm front; residual; decision (sets the conditional)
//   IF (fallback): restore u, v, tdiv; n_steps iterations
//   C: finish phase
int nsdg_kernel::captureWarmGraph(double dt, cudaGraph_t& g, int& launches)
{
    launches = 0;
    g = nullptr;
    CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("warm graph: conditional handle: ") + cudaGetErrorString(e));
    std::vector<cudaGraphNode_t> tail;
    int st = NSDG_OK;
    // ---- part A
    CUDA_TRY(cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    {
        st = enqueueWarmFront(stream, dt, launches);
        if (st == NSDG_OK) {
            cudaError_t ee = launchWarmResidual(stream, Ncg, st32.u, st32.v, uPrev, vPrev, st32.u0, st32.v0, wPart,
                wRes);
            if (ee == cudaSuccess) ee = launchWarmDecide(stream, h, wRes, warmKappa, rec);
            if (ee != cudaSuccess)
                st = fail(NSDG_ERR_CUDA, std::string("warm graph: decision: ") + cudaGetErrorString(ee));
            launches += 3;
        }
        cudaStreamCaptureStatus cs;
        const cudaGraphNode_t* deps = nullptr;
        size_t nd = 0;
        e = cudaStreamGetCaptureInfo(stream, &cs, nullptr, nullptr, &deps, nullptr, &nd);
        if (e == cudaSuccess)
            tail.assign(deps, deps + nd);
        cudaGraph_t gg = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(stream, &gg);
        if (st != NSDG_OK)
            return st;
        if (e != cudaSuccess || ec != cudaSuccess)
            return fail(NSDG_ERR_CUDA, std::string("warm graph capture: ")
                    + cudaGetErrorString(e != cudaSuccess ? e : ec));
    }
    // ---- the conditional fallback
    cudaGraphNodeParams cp {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t cn;
    e = cudaGraphAddNode(&cn, g, tail.data(), nullptr, tail.size(), &cp);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("warm graph: conditional node: ") + cudaGetErrorString(e));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    CUDA_TRY(cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    {
        int l = 3;
        cudaError_t ee = launchWarmSave(stream, Ncg, bu, st32.u, nullptr);
        if (ee == cudaSuccess) ee = launchWarmSave(stream, Ncg, bv, st32.v, nullptr);
        if (ee == cudaSuccess) ee = launchWarmSave(stream, 18 * N, btdiv, tdiv32, nullptr);
        if (ee != cudaSuccess)
            st = fail(NSDG_ERR_CUDA, std::string("warm graph: restore: ") + cudaGetErrorString(ee));
        if (st == NSDG_OK)
            st = mixedIterations(stream, dt, P.n_steps, derr, l);
        warmBodyLaunches = l;
        cudaGraph_t bb = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(stream, &bb);
        if (st != NSDG_OK)
            return st;
        if (ec != cudaSuccess)
            return fail(NSDG_ERR_CUDA, std::string("warm graph: fallback capture: ") + cudaGetErrorString(ec));
    }
    // ---- part C
    CUDA_TRY(cudaStreamBeginCaptureToGraph(stream, g, &cn, nullptr, 1, cudaStreamCaptureModeThreadLocal));
    {
        int l = 0;
        st = enqueuePhases(stream, dt, PHASE_FINISH, l);
        launches += l;
        cudaGraph_t gg = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(stream, &gg);
        if (st != NSDG_OK)
            return st;
        if (ec != cudaSuccess)
            return fail(NSDG_ERR_CUDA, std::string("warm graph: finish capture: ") + cudaGetErrorString(ec));
    }
    return NSDG_OK;
}

// A audited update: the warm attempt, then the plain sub-cycle from the same
// start (its result is kept), and the relative distance between the two
// decides whether the following updates may accept warm sub-cycles.
int nsdg_kernel::captureAuditGraph(double dt, cudaGraph_t& g, int& launches)
{
    launches = 0;
    g = nullptr;
    CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    int st = enqueueWarmFront(stream, dt, launches);
    if (st == NSDG_OK) {
        cudaError_t e = launchWarmSave(stream, Ncg, st32.u, uPrev, nullptr); // the warm result
        if (e == cudaSuccess) e = launchWarmSave(stream, Ncg, st32.v, vPrev, nullptr);
        if (e == cudaSuccess) e = launchWarmSave(stream, Ncg, bu, st32.u, nullptr);
        if (e == cudaSuccess) e = launchWarmSave(stream, Ncg, bv, st32.v, nullptr);
        if (e == cudaSuccess) e = launchWarmSave(stream, 18 * N, btdiv, tdiv32, nullptr);
        if (e != cudaSuccess)
            st = fail(NSDG_ERR_CUDA, std::string("audit graph: ") + cudaGetErrorString(e));
        launches += 5;
    }
    if (st == NSDG_OK)
        st = mixedIterations(stream, dt, P.n_steps, derr, launches);
    if (st == NSDG_OK) {
        cudaError_t e = launchWarmResidual(stream, Ncg, st32.u, st32.v, uPrev, vPrev, st32.u0, st32.v0, wPart, wRes);
        if (e == cudaSuccess) e = launchWarmAudit(stream, wRes, auditTol, rec);
        if (e != cudaSuccess)
            st = fail(NSDG_ERR_CUDA, std::string("audit graph: ") + cudaGetErrorString(e));
        launches += 3;
    }
    if (st == NSDG_OK) {
        int l = 0;
        st = enqueuePhases(stream, dt, PHASE_FINISH, l);
        launches += l;
    }
    const cudaError_t ec = cudaStreamEndCapture(stream, &g);
    if (st != NSDG_OK)
        return st;
    if (ec != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("audit graph capture: ") + cudaGetErrorString(ec));
    return NSDG_OK;
}

int nsdg_kernel::ensureGraph(double dt)
{
    if (graph && graphDt == dt)
        return NSDG_OK;
    dropGraphs();
    cudaGraph_t g = nullptr;
    int launches = 0;
    if (warmNet) {
        const int st = captureWarmGraph(dt, g, launches);
        if (st != NSDG_OK) {
            if (g)
                cudaGraphDestroy(g);
            return st;
        }
    } else {
    CUDA_TRY(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
    const int st = enqueueUpdate(dt, launches);
    const cudaError_t ec = cudaStreamEndCapture(stream, &g);
    if (st != NSDG_OK) {
        if (g)
            cudaGraphDestroy(g);
        return st;
    }
    if (ec != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
    }
    const cudaError_t ei = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        graph = nullptr;
        return fail(NSDG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
    }
    graphDt = dt;
    launchesPerUpdate = launches;
    if (warmNet && auditEvery > 0) {
        cudaGraph_t gj = nullptr;
        const int st = captureAuditGraph(dt, gj, auditLaunches);
        if (st != NSDG_OK) {
            if (gj)
                cudaGraphDestroy(gj);
            return st;
        }
        const cudaError_t ej = cudaGraphInstantiate(&auditGraph, gj, 0);
        cudaGraphDestroy(gj);
        if (ej != cudaSuccess) {
            auditGraph = nullptr;
            return fail(NSDG_ERR_CUDA, std::string("audit graph instantiate: ") + cudaGetErrorString(ej));
        }
    }
    return NSDG_OK;
}

// Launches the update graph of the next step: with a warm start attached and
// auditing on, every auditEvery-th update (the first included) is a audited one.
int nsdg_kernel::launchStep(double dt)
{
    int r = ensureGraph(dt);
    if (r)
        return r;
    cudaGraphExec_t gx = graph;
    if (warmNet && auditEvery > 0 && warmSteps % auditEvery == 0)
        gx = auditGraph;
    const cudaError_t e = cudaGraphLaunch(gx, stream);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("update: ") + cudaGetErrorString(e));
    if (warmNet)
        ++warmSteps;
    ++stepNumber;
    readCache = 0;
    return NSDG_OK;
}

// ---------------------------------------------------------------------------
// extern "C"
// ---------------------------------------------------------------------------
extern "C" {

void nsdg_default_params(nsdg_params* p)
{
    if (!p)
        return;
    std::memset(p, 0, sizeof(*p));
    // DynamicsParameters.hpp:22-40
    p->rho_ice = 900.0;
    p->rho_atm = 1.3;
    p->rho_ocean = 1026.0;
    p->C_atm = 1.2e-3;
    p->C_ocean = 5.5e-3;
    p->F_atm = p->C_atm * p->rho_atm;
    p->F_ocean = p->C_ocean * p->rho_ocean;
    p->fc = 1.45842e-4;
    p->ocean_turning_angle = 0.0;
    p->gravity = 9.81;
    // VPParameters.hpp:20-25
    p->Pstar = 27500.0;
    p->DeltaMin = 2.e-9;
    // VPCGDynamicsKernel.hpp:125-126
    p->alpha = 1500.;
    p->beta = 1500.;
    // MEBParameters.hpp:40-65
    p->compaction_param = -20.;
    p->nu0 = 1. / 3.;
    p->young = 5.96e8;
    p->P0 = 10.e3;
    p->undamaged_time_relaxation_sigma = 1e7;
    p->exponent_relaxation_sigma = 5;
    p->exponent_compression_factor = 1.5;
    p->tan_phi = 0.7;
    p->compr_strength = 1e10;
    p->C_lab = 2.0e6;
    // DynamicsKernel.hpp:187
    p->n_steps = 100;
    p->precision = NSDG_PRECISION_FP64;
}

const char* nsdg_status_string(int s)
{
    switch (s) {
    case NSDG_OK: return "ok";
    case NSDG_ERR_BAD_ARG: return "bad argument";
    case NSDG_ERR_UNKNOWN_FIELD: return "unknown field";
    case NSDG_ERR_SIZE_MISMATCH: return "size mismatch";
    case NSDG_ERR_CUDA: return "CUDA error";
    case NSDG_ERR_NUMERIC: return "non-finite values";
    case NSDG_ERR_UNSUPPORTED: return "unsupported";
    case NSDG_ERR_LOGIC: return "logic error";
    case NSDG_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

const char* nsdg_version(void) { return kVersion; }

int nsdg_kernel_create(int rheology, int dg_comp, const nsdg_params* params, nsdg_kernel** out)
{
    if (!out)
        return NSDG_ERR_BAD_ARG;
    *out = nullptr;
    if (rheology != NSDG_RHEOLOGY_MEVP && rheology != NSDG_RHEOLOGY_BBM)
        return NSDG_ERR_BAD_ARG;
    if (dg_comp != 1 && dg_comp != 3 && dg_comp != 6)
        return NSDG_ERR_BAD_ARG;
    nsdg_params p;
    if (params)
        p = *params;
    else
        nsdg_default_params(&p);
    if (p.n_steps < 1 || !(p.alpha > 0) || !(p.beta >= 0) || !(p.rho_ice > 0))
        return NSDG_ERR_BAD_ARG;
    if (p.precision != NSDG_PRECISION_FP64 && p.precision != NSDG_PRECISION_MIXED)
        return NSDG_ERR_UNSUPPORTED;
    try {
        nsdg_kernel* k = new nsdg_kernel();
        k->rheology = rheology;
        k->dg = dg_comp;
        k->P = p;
        *out = k;
    } catch (const std::exception&) {
        return NSDG_ERR_BAD_ARG;
    }
    return NSDG_OK;
}

int nsdg_kernel_destroy(nsdg_kernel* k)
{
    if (!k)
        return NSDG_ERR_BAD_ARG;
    if (k->stream)
        cudaStreamSynchronize(k->stream);
    k->releaseDevice();
    delete k;
    return NSDG_OK;
}

const char* nsdg_kernel_last_error(const nsdg_kernel* k) { return k ? k->err.c_str() : "null handle"; }

int nsdg_kernel_initialise(nsdg_kernel* k, size_t nx, size_t ny, const double* coords, int is_spherical,
    const double* mask)
{
    if (!k)
        return NSDG_ERR_BAD_ARG;
    try {
        return k->initialise(nx, ny, coords, is_spherical, mask);
    } catch (const std::exception& ex) {
        return k->fail(NSDG_ERR_BAD_ARG, std::string("initialise: ") + ex.what());
    }
}

void nsdg_benchmark_forcing_defaults(nsdg_benchmark_forcing* f, double length_x, double length_y)
{
    if (!f)
        return;
    const double fiveDays = 5.0 * 86400.0; // BenchmarkAtmosphere.cpp:41-51
    f->length_x = length_x;
    f->length_y = length_y;
    f->wind_A = 1e-5;
    f->wind_vmax = 30.0;
    f->wind_k = 1e-5;
    f->wind_angle_deg = 72.0;
    f->centre_x = 0.5 * length_x;
    f->centre_y = 0.5 * length_y;
    f->centre_vx = 0.5 * length_x / fiveDays;
    f->centre_vy = 0.5 * length_y / fiveDays;
    f->ocean_vmax = 0.01; // BenchmarkOcean.cpp:31
}

namespace {
// the one-component cell fields f0, f1 (device, [N] each) into the CG2
// targets t0, t1, as set_data of an H field does (CGDynamicsKernel.cpp:54-90)
int cellsToNodes(nsdg_kernel* k, const double* f0, const double* f1, double* t0, double* t1)
{
    const double* in[2] = { f0, f1 };
    double* out[2] = { t0, t1 };
    const cudaError_t e = launchDG2CG(k->stream, k->dm, 1, 2, in, out);
    return e == cudaSuccess ? NSDG_OK : k->fail(NSDG_ERR_CUDA, std::string("benchmark forcing: ") + cudaGetErrorString(e));
}
int forcingArgs(nsdg_kernel* k, const nsdg_benchmark_forcing* f)
{
    if (!k)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "benchmark forcing: kernel not initialised");
    if (!f || !(f->length_x > 0) || !(f->length_y > 0) || !std::isfinite(f->length_x) || !std::isfinite(f->length_y))
        return k->fail(NSDG_ERR_BAD_ARG, "benchmark forcing: positive finite box lengths needed");
    return NSDG_OK;
}
} // namespace

int nsdg_kernel_benchmark_ocean(nsdg_kernel* k, const nsdg_benchmark_forcing* f)
{
    int r = forcingArgs(k, f);
    if (r)
        return r;
    k->readCache = 0;
    const size_t nx = size_t(k->dm.nx), ny = size_t(k->dm.ny), N = k->N;
    // BenchmarkCoordinates.cpp:28-29: dx = length / n
    cudaError_t e = launchBenchmarkOcean(k->stream, nx, ny, f->length_x / double(nx), f->length_y / double(ny),
        f->ocean_vmax, k->dgTmp, k->dgTmp + N);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("benchmark ocean: ") + cudaGetErrorString(e));
    r = cellsToNodes(k, k->dgTmp, k->dgTmp + N, k->uo, k->vo);
    return r ? r : k->ok();
}

int nsdg_kernel_benchmark_atmosphere(nsdg_kernel* k, const nsdg_benchmark_forcing* f, double seconds)
{
    int r = forcingArgs(k, f);
    if (r)
        return r;
    if (!std::isfinite(seconds))
        return k->fail(NSDG_ERR_BAD_ARG, "benchmark atmosphere: finite time needed");
    k->readCache = 0;
    const size_t nx = size_t(k->dm.nx), ny = size_t(k->dm.ny), N = k->N;
    const double a = f->wind_angle_deg / 180.0 * M_PI; // BenchmarkAtmosphere.cpp:50-52
    BenchmarkWindArgs w { f->length_x / double(nx), f->length_y / double(ny), f->centre_x + f->centre_vx * seconds,
        f->centre_y + f->centre_vy * seconds, f->wind_A, f->wind_k, f->wind_vmax, std::cos(a), std::sin(a) };
    cudaError_t e = launchBenchmarkWind(k->stream, nx, ny, w, k->dgTmp, k->dgTmp + N);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("benchmark atmosphere: ") + cudaGetErrorString(e));
    r = cellsToNodes(k, k->dgTmp, k->dgTmp + N, k->ua, k->va);
    return r ? r : k->ok();
}

nsdg_kernel::SetTarget nsdg_kernel::setTarget(const std::string& s)
{
    SetTarget t;
    t.comps = dg;
    if (s == "u") t.cg = u;
    else if (s == "v") t.cg = v;
    else if (s == "uwind") t.cg = ua;
    else if (s == "vwind") t.cg = va;
    else if (s == "uocean") t.cg = uo;
    else if (s == "vocean") t.cg = vo;
    else if (s == "hice") t.dg = hice;
    else if (s == "cice") t.dg = cice;
    else if (s == "ssh") { t.dg = ssh; t.comps = 1; }
    else if (s == "damage" && rheology == NSDG_RHEOLOGY_BBM) t.dg = damage;
    return t;
}

void nsdg_kernel::storeField(const std::string& s, const double* data, size_t nComp)
{
    // DynamicsKernel.hpp:104-109: any other name is stored (ma2dg semantics)
    std::vector<double>& b = bucket[s];
    b.assign(N * dg, 0.0);
    if (nComp == size_t(dg))
        std::memcpy(b.data(), data, N * dg * sizeof(double));
    else
        for (size_t i = 0; i < N; ++i)
            b[i * dg] = data[i * nComp];
    bucketComps[s] = static_cast<int>(nComp);
}

int nsdg_kernel::enqueueConversion(const SetTarget& t, const double* staging, size_t nComp)
{
    cudaError_t e;
    if (t.cg && nComp != size_t(dg)) {
        // CGDynamicsKernel.cpp:54-90: ma2dg keeps component 0 only, so DG2CG
        // of the one-component field gives the same node values (the higher
        // components' contributions are exact zeros)
        const double* in[1] = { staging };
        double* out[1] = { t.cg };
        e = launchDG2CG(stream, dm, 1, 1, in, out);
    } else if (t.cg) {
        // CGDynamicsKernel.cpp:54-90: ma2dg into a DG vector, then DG2CG
        e = launchAosToSoa(stream, N, static_cast<int>(nComp), dg, staging, dgTmp);
        if (e == cudaSuccess) {
            const double* in[1] = { dgTmp };
            double* out[1] = { t.cg };
            e = launchDG2CG(stream, dm, dg, 1, in, out);
        }
    } else {
        e = launchAosToSoa(stream, N, static_cast<int>(nComp), t.comps, staging, t.dg);
    }
    return e == cudaSuccess ? NSDG_OK : fail(NSDG_ERR_CUDA, std::string("set_data convert: ") + cudaGetErrorString(e));
}

int nsdg_kernel_set_data(nsdg_kernel* k, const char* name, const double* data, size_t n_elements, size_t n_comp)
{
    if (!k || !name)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "set_data: kernel not initialised");
    if (!data)
        return k->fail(NSDG_ERR_BAD_ARG, "set_data: null data");
    if (n_elements != k->N || n_comp == 0 || n_comp > 8)
        return k->fail(NSDG_ERR_SIZE_MISMATCH, std::string("set_data: size mismatch for ") + name);
    k->readCache = 0;
    const std::string s(name);
    const size_t N = k->N;
    cudaStream_t st = k->stream;
    const nsdg_kernel::SetTarget target = k->setTarget(s);
    if (!target.cg && !target.dg) {
        k->storeField(s, data, n_comp);
        return k->ok();
    }
    auto cu = [&](cudaError_t e, const char* what) {
        return e == cudaSuccess ? NSDG_OK : k->fail(NSDG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    // the copy waits only for the conversion that last read its staging
    // buffer; the conversion waits for the copy (and, in stream order, for
    // everything already enqueued on the kernel's stream)
    const int slot = k->stageSlot;
    k->stageSlot ^= 1;
    double* const staging = slot ? k->stage2 : k->staging;
    int r = cu(cudaStreamWaitEvent(k->copyStream, k->converted[slot], 0), "set_data wait");
    if (r) return r;
    if (k->moveByKernel(data)) {
        HostMoves m;
        m.src[0] = data;
        m.dst[0] = staging;
        m.n[0] = N * n_comp;
        m.count = 1;
        r = cu(launchHostMove(k->copyStream, m), "set_data move");
    } else {
        r = cu(cudaMemcpyAsync(staging, data, N * n_comp * sizeof(double), cudaMemcpyHostToDevice, k->copyStream),
            "set_data copy");
    }
    if (r) return r;
    r = cu(cudaEventRecord(k->copied, k->copyStream), "set_data event");
    if (r) {
        cudaStreamSynchronize(k->copyStream); // the caller's buffer is read until the copy ends
        return r;
    }
    r = cu(cudaStreamWaitEvent(st, k->copied, 0), "set_data wait");
    if (r == NSDG_OK)
        r = k->enqueueConversion(target, staging, n_comp);
    // recorded after whatever reads this staging buffer, also on a failure
    const cudaError_t er = cudaEventRecord(k->converted[slot], st);
    if (r == NSDG_OK)
        r = cu(er, "set_data event");
    // the caller may reuse `data` once the copy has landed (on every return
    // from here); the conversion runs on behind the return
    const cudaError_t es = cudaEventSynchronize(k->copied);
    if (r)
        return r;
    r = cu(es, "set_data sync");
    return r ? r : k->ok();
}

int nsdg_kernel_update(nsdg_kernel* k, double t_start, double dt)
{
    (void)t_start;
    if (!k)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "update: kernel not initialised");
    if (!(dt > 0) || !std::isfinite(dt))
        return k->fail(NSDG_ERR_BAD_ARG, "update: dt must be positive");
    const int r = k->launchStep(dt);
    return r ? r : k->ok();
}

int nsdg_kernel_synchronize(nsdg_kernel* k)
{
    if (!k)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "synchronize: kernel not initialised");
    const int r = k->checkDeviceError();
    return r ? r : k->ok();
}

int nsdg_kernel::enqueueReadout(const std::string& s, double* out, HostMoves* batch)
{
    const bool bbm = rheology == NSDG_RHEOLOGY_BBM;
    const double* src = nullptr;
    cudaError_t e = cudaSuccess;
    const double* minvP = dops.minvP ? dops.minvP : dops.minv;
    if (s == "u" || s == "v") {
        // both components are projected on the first read after a state change
        if (!(readCache & 1)) {
            const double* in[2] = { u, v };
            double* outd[2] = { velx, vely };
            // only the cell averages are read: component 0 of the projection
            // (the mixed path's velocity is its FP32 iterate: FP32 quadrature)
            e = launchCG2DG0(stream, dm, dg, dops.jwA, mixed() ? jwA32 : nullptr, minvP, in, outd);
            if (e == cudaSuccess)
                readCache |= 1;
        }
        src = (s == "u") ? velx : vely;
    } else if (s == "uiostress" || s == "viostress") {
        if (!(readCache & 2)) {
            const double rad = 0x1.1df46a2529d39p-6;
            const double ang = bbm ? P.ocean_turning_angle : 0.0;
            double* tx = cgTmp;
            double* ty = u0; // reused as scratch outside update
            e = launchIceOceanStress(stream, Ncg, bbm ? 1 : 0, bbm ? avgU : u, bbm ? avgV : v, uo, vo, P.F_ocean,
                std::cos(rad * ang), std::sin(rad * ang), tx, ty, mixed());
            const double* in[2] = { tx, ty };
            double* outd[2] = { phiA, phiA + size_t(dg) * N };
            if (e == cudaSuccess)
                e = launchCG2DG0(stream, dm, dg, dops.jwA, mixed() ? jwA32 : nullptr, minvP, in, outd);
            if (e == cudaSuccess)
                readCache |= 2;
        }
        src = (s == "uiostress") ? phiA : phiA + size_t(dg) * N;
    } else if (s == "hice") src = hice;
    else if (s == "cice") src = cice;
    else if (s == "damage" && bbm) src = damage;
    else {
        auto it = bucket.find(s);
        if (it == bucket.end())
            return fail(NSDG_ERR_UNKNOWN_FIELD, "get_dg0: unknown field " + s);
        for (size_t i = 0; i < N; ++i)
            out[i] = it->second[i * dg];
        return NSDG_OK;
    }
    if (e == cudaSuccess) {
        if (moveByKernel(out)) {
            // into a pageable host array: a kernel writes it (batched with
            // the call's other read-outs when the caller collects them)
            if (batch && batch->count < kHostMoves) {
                batch->src[batch->count] = src;
                batch->dst[batch->count] = out;
                batch->n[batch->count] = N;
                ++batch->count;
            } else {
                HostMoves m;
                m.src[0] = src;
                m.dst[0] = out;
                m.n[0] = N;
                m.count = 1;
                e = launchHostMove(stream, m);
            }
        } else {
            e = cudaMemcpyAsync(out, src, N * sizeof(double), cudaMemcpyDeviceToHost, stream);
        }
    }
    return e == cudaSuccess ? NSDG_OK : fail(NSDG_ERR_CUDA, std::string("get_dg0: ") + cudaGetErrorString(e));
}

int nsdg_kernel_get_dg0(nsdg_kernel* k, const char* name, double* out, size_t n_elements)
{
    if (!k || !name || !out)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "get_dg0: kernel not initialised");
    if (n_elements != k->N)
        return k->fail(NSDG_ERR_SIZE_MISMATCH, "get_dg0: size mismatch");
    int r = k->enqueueReadout(std::string(name), out);
    if (r)
        return r;
    r = k->checkDeviceError();
    return r ? r : k->ok();
}

// One module step in one call (MEVPDynamics::update / BBMDynamics::update):
// every input's host copy goes out on the copy stream into one staging pool,
// the conversions follow on the kernel's stream once all have landed, then
// the update and every read-out; one wait at the end.  The same kernels as
// the separate calls, so the same results.
int nsdg_kernel_module_step(nsdg_kernel* k, const nsdg_field_in* in, size_t n_in, double t_start, double dt,
    const nsdg_field_out* out, size_t n_out)
{
    (void)t_start;
    if (!k || (n_in && !in) || (n_out && !out))
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "module_step: kernel not initialised");
    if (!(dt > 0) || !std::isfinite(dt))
        return k->fail(NSDG_ERR_BAD_ARG, "module_step: dt must be positive");
    const size_t N = k->N;
    size_t need = 0;
    std::vector<nsdg_kernel::SetTarget> targets(n_in);
    for (size_t i = 0; i < n_in; ++i) {
        if (!in[i].name || !in[i].data)
            return k->fail(NSDG_ERR_BAD_ARG, "module_step: null input name or data");
        if (in[i].n_comp == 0 || in[i].n_comp > 8)
            return k->fail(NSDG_ERR_SIZE_MISMATCH, std::string("module_step: size mismatch for ") + in[i].name);
        targets[i] = k->setTarget(in[i].name);
        if (targets[i].cg || targets[i].dg)
            need += N * in[i].n_comp;
    }
    for (size_t j = 0; j < n_out; ++j) {
        if (!out[j].name || !out[j].data)
            return k->fail(NSDG_ERR_BAD_ARG, "module_step: null output name or data");
        const std::string s(out[j].name);
        const bool known = s == "u" || s == "v" || s == "uiostress" || s == "viostress" || s == "hice"
            || s == "cice" || (s == "damage" && k->rheology == NSDG_RHEOLOGY_BBM);
        bool stored = k->bucket.count(s) > 0;
        for (size_t i = 0; i < n_in && !stored; ++i)
            stored = s == in[i].name && !targets[i].cg && !targets[i].dg;
        if (!known && !stored)
            return k->fail(NSDG_ERR_UNKNOWN_FIELD, "module_step: unknown field " + s);
    }
    auto cu = [&](cudaError_t e, const char* what) {
        return e == cudaSuccess ? NSDG_OK : k->fail(NSDG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    };
    k->readCache = 0;
    if (need > k->moduleStageDoubles) {
        // the pool is read only by this call's conversions, all finished
        // when the previous call returned
        if (k->moduleStage)
            cudaFree(k->moduleStage);
        k->moduleStage = nullptr;
        k->moduleStageDoubles = 0;
        int r = cu(cudaMalloc(&k->moduleStage, need * sizeof(double)), "module_step staging");
        if (r)
            return r;
        k->moduleStageDoubles = need;
    }
    int r = NSDG_OK;
    size_t off = 0;
    HostMoves inMoves; // pageable inputs, moved by one kernel
    for (size_t i = 0; i < n_in && r == NSDG_OK; ++i) {
        if (!targets[i].cg && !targets[i].dg) {
            k->storeField(in[i].name, in[i].data, in[i].n_comp);
            continue;
        }
        if (k->moveByKernel(in[i].data)) {
            inMoves.src[inMoves.count] = in[i].data;
            inMoves.dst[inMoves.count] = k->moduleStage + off;
            inMoves.n[inMoves.count] = N * in[i].n_comp;
            if (++inMoves.count == kHostMoves) {
                r = cu(launchHostMove(k->copyStream, inMoves), "module_step move");
                inMoves = HostMoves();
            }
        } else {
            r = cu(cudaMemcpyAsync(k->moduleStage + off, in[i].data, N * in[i].n_comp * sizeof(double),
                       cudaMemcpyHostToDevice, k->copyStream),
                "module_step copy");
        }
        off += N * in[i].n_comp;
    }
    if (r == NSDG_OK && inMoves.count)
        r = cu(launchHostMove(k->copyStream, inMoves), "module_step move");
    if (r == NSDG_OK)
        r = cu(cudaEventRecord(k->copied, k->copyStream), "module_step event");
    if (r == NSDG_OK)
        r = cu(cudaStreamWaitEvent(k->stream, k->copied, 0), "module_step wait");
    if (r) {
        cudaStreamSynchronize(k->copyStream); // the callers' buffers are read until the copies end
        return r;
    }
    off = 0;
    for (size_t i = 0; i < n_in && r == NSDG_OK; ++i) {
        if (!targets[i].cg && !targets[i].dg)
            continue;
        r = k->enqueueConversion(targets[i], k->moduleStage + off, in[i].n_comp);
        off += N * in[i].n_comp;
    }
    if (r == NSDG_OK)
        r = k->launchStep(dt);
    HostMoves outMoves; // pageable outputs, written by one kernel
    for (size_t j = 0; j < n_out && r == NSDG_OK; ++j)
        r = k->enqueueReadout(out[j].name, out[j].data, &outMoves);
    if (r == NSDG_OK && outMoves.count)
        r = cu(launchHostMove(k->stream, outMoves), "module_step move");
    const int rs = k->checkDeviceError(); // waits for the copies out as well
    if (r)
        return r;
    return rs ? rs : k->ok();
}

int nsdg_kernel_get_dg(nsdg_kernel* k, const char* name, double* out, size_t n_elements, size_t n_comp)
{
    if (!k || !name || !out)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "get_dg: kernel not initialised");
    if (n_elements != k->N)
        return k->fail(NSDG_ERR_SIZE_MISMATCH, "get_dg: size mismatch");
    const std::string s(name);
    const size_t N = k->N;
    const int dg = k->dg;
    const bool bbm = k->rheology == NSDG_RHEOLOGY_BBM;
    const double* src = nullptr;
    if (s == "hice") src = k->hice;
    else if (s == "cice") src = k->cice;
    else if (s == "damage" && bbm) src = k->damage;
    else {
        auto it = k->bucket.find(s);
        if (it == k->bucket.end())
            return k->fail(NSDG_ERR_UNKNOWN_FIELD, "get_dg: unknown field " + s);
        const size_t want = (k->bucketComps[s] == dg) ? dg : 1;
        if (n_comp != want)
            return k->fail(NSDG_ERR_SIZE_MISMATCH, "get_dg: component count mismatch");
        for (size_t i = 0; i < N; ++i)
            for (size_t j = 0; j < want; ++j)
                out[i * want + j] = it->second[i * dg + j];
        return k->ok();
    }
    if (n_comp != size_t(dg))
        return k->fail(NSDG_ERR_SIZE_MISMATCH, "get_dg: component count mismatch");
    cudaError_t e = launchSoaToAos(k->stream, N, dg, dg, src, k->staging);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, k->staging, N * dg * sizeof(double), cudaMemcpyDeviceToHost, k->stream);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("get_dg: ") + cudaGetErrorString(e));
    const int r = k->checkDeviceError();
    return r ? r : k->ok();
}

// Snapshot layout: magic, version, rheology, dg, N, Ncg, stepNumber, then the
// state arrays in a fixed order.
namespace {
struct SnapHeader {
    char magic[8];
    int version, rheology, dg, pad;
    unsigned long long N, Ncg, step;
};
// (device pointer, bytes) of every array that carries state across steps
std::vector<std::pair<void*, size_t>> snapshotArrays(nsdg_kernel* k)
{
    const size_t dN = size_t(k->dg) * k->N * sizeof(double);
    const size_t cg = k->Ncg * sizeof(double);
    std::vector<std::pair<void*, size_t>> a = { { k->hice, dN }, { k->cice, dN }, { k->ssh, k->N * sizeof(double) },
        { k->u, cg }, { k->v, cg }, { k->uo, cg }, { k->vo, cg }, { k->ua, cg }, { k->va, cg } };
    if (k->rheology == NSDG_RHEOLOGY_MEVP) {
        // the mEVP stress lives in divergence space (see kMevpStress)
        if (k->mixed()) {
            a.push_back({ k->tdiv32, 18 * k->N * sizeof(float) });
            a.push_back({ k->tdivLast, 18 * k->N * sizeof(float) });
            a.push_back({ k->uLast, k->Ncg * sizeof(float) });
            a.push_back({ k->vLast, k->Ncg * sizeof(float) });
        }
        else
            a.push_back({ k->contrib, 18 * k->N * sizeof(double) });
    } else {
        a.push_back({ k->s11, 8 * k->N * sizeof(double) });
        a.push_back({ k->s12, 8 * k->N * sizeof(double) });
        a.push_back({ k->s22, 8 * k->N * sizeof(double) });
        a.push_back({ k->damage, dN });
        a.push_back({ k->avgU, cg });
        a.push_back({ k->avgV, cg });
    }
    return a;
}
} // namespace

int nsdg_kernel_snapshot_size(nsdg_kernel* k, size_t* bytes)
{
    if (!k || !bytes)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "snapshot: kernel not initialised");
    size_t b = sizeof(SnapHeader);
    for (auto& p : snapshotArrays(k))
        b += p.second;
    *bytes = b;
    return k->ok();
}

int nsdg_kernel_snapshot_save(nsdg_kernel* k, void* buffer, size_t bytes)
{
    size_t need = 0;
    int r = nsdg_kernel_snapshot_size(k, &need);
    if (r)
        return r;
    if (!buffer || bytes < need)
        return k->fail(NSDG_ERR_SIZE_MISMATCH, "snapshot_save: buffer too small");
    SnapHeader h {};
    std::memcpy(h.magic, "NSDGSNP", 8);
    h.version = 1;
    h.rheology = k->rheology;
    h.dg = k->dg;
    h.pad = k->P.precision;
    h.N = k->N;
    h.Ncg = k->Ncg;
    h.step = k->stepNumber;
    std::memcpy(buffer, &h, sizeof(h));
    char* p = static_cast<char*>(buffer) + sizeof(h);
    for (auto& a : snapshotArrays(k)) {
        const cudaError_t e = cudaMemcpyAsync(p, a.first, a.second, cudaMemcpyDeviceToHost, k->stream);
        if (e != cudaSuccess)
            return k->fail(NSDG_ERR_CUDA, std::string("snapshot_save: ") + cudaGetErrorString(e));
        p += a.second;
    }
    r = k->checkDeviceError();
    return r ? r : k->ok();
}

int nsdg_kernel_snapshot_load(nsdg_kernel* k, const void* buffer, size_t bytes)
{
    if (k)
        k->readCache = 0;
    size_t need = 0;
    int r = nsdg_kernel_snapshot_size(k, &need);
    if (r)
        return r;
    if (!buffer || bytes < need)
        return k->fail(NSDG_ERR_SIZE_MISMATCH, "snapshot_load: buffer too small");
    SnapHeader h;
    std::memcpy(&h, buffer, sizeof(h));
    if (std::memcmp(h.magic, "NSDGSNP", 8) != 0 || h.version != 1 || h.rheology != k->rheology
        || h.dg != k->dg || h.pad != k->P.precision || h.N != k->N || h.Ncg != k->Ncg)
        return k->fail(NSDG_ERR_SIZE_MISMATCH, "snapshot_load: snapshot does not match this kernel");
    const char* p = static_cast<const char*>(buffer) + sizeof(h);
    for (auto& a : snapshotArrays(k)) {
        const cudaError_t e = cudaMemcpyAsync(a.first, p, a.second, cudaMemcpyHostToDevice, k->stream);
        if (e != cudaSuccess)
            return k->fail(NSDG_ERR_CUDA, std::string("snapshot_load: ") + cudaGetErrorString(e));
        p += a.second;
    }
    const cudaError_t e = cudaStreamSynchronize(k->stream);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("snapshot_load: ") + cudaGetErrorString(e));
    k->stepNumber = h.step;
    return k->ok();
}

int nsdg_kernel_mean_value(nsdg_kernel* k, const char* name, double* out)
{
    if (!k || !name || !out)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "mean_value: kernel not initialised");
    const std::string s(name);
    const double* src = nullptr;
    if (s == "hice") src = k->hice;
    else if (s == "cice") src = k->cice;
    else if (s == "damage" && k->rheology == NSDG_RHEOLOGY_BBM) src = k->damage;
    else return k->fail(NSDG_ERR_UNKNOWN_FIELD, "mean_value: unknown field " + s);
    cudaError_t e = launchMeanValue(k->stream, k->N, k->dg, src, k->dops.jw3, k->partials, k->dsum);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out, k->dsum, sizeof(double), cudaMemcpyDeviceToHost, k->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(k->stream);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("mean_value: ") + cudaGetErrorString(e));
    return k->ok();
}

int nsdg_kernel_time_updates(nsdg_kernel* k, double dt, int steps, float* ms)
{
    if (!k || !ms || steps < 1)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "time_updates: kernel not initialised");
    int r = k->ensureGraph(dt);
    if (r)
        return r;
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, "time_updates: event create failed");
    cudaError_t e = cudaStreamSynchronize(k->stream);
    if (e == cudaSuccess) e = cudaEventRecord(a, k->stream);
    for (int i = 0; i < steps && e == cudaSuccess && r == NSDG_OK; ++i)
        r = k->launchStep(dt);
    if (e == cudaSuccess) e = cudaEventRecord(b, k->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (r)
        return r;
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("time_updates: ") + cudaGetErrorString(e));
    r = k->checkDeviceError();
    return r ? r : k->ok();
}

int nsdg_kernel_time_kernel(nsdg_kernel* k, int kernel_id, int reps, float* mean_ms, const char** name)
{
    if (k)
        k->readCache = 0; // the timed kernels change the state
    if (!k || !mean_ms || reps < 1)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "time_kernel: kernel not initialised");
    const bool bbm = k->rheology == NSDG_RHEOLOGY_BBM;
    const double dt = k->graphDt > 0 ? k->graphDt : 120.0;
    MevpParams mp { k->P.rho_ice, k->P.F_atm, k->P.F_ocean, k->P.fc, k->P.gravity, k->P.Pstar, k->P.DeltaMin,
        k->P.alpha, k->P.beta, dt };
    MevpNodeState st { k->u, k->v, k->u0, k->v0, k->cgH, k->cgA, k->uo, k->vo, k->ua, k->va, k->uGrad,
        k->vGrad, k->c1, k->c1b, k->fau, k->fav, k->rhfc, k->gu, k->gv };
    const double rad = 0x1.1df46a2529d39p-6;
    BbmParams bp { k->P.rho_ice, k->P.F_atm, k->P.F_ocean, k->P.fc, k->P.gravity, dt / k->P.n_steps,
        double(k->P.n_steps), std::cos(rad * k->P.ocean_turning_angle), std::sin(rad * k->P.ocean_turning_angle),
        k->P.compaction_param, k->P.nu0, k->P.young, k->P.P0, k->P.undamaged_time_relaxation_sigma,
        k->P.exponent_relaxation_sigma, k->P.exponent_compression_factor, k->P.tan_phi, k->P.compr_strength,
        k->P.C_lab };
    bbmPowModes(bp);
    BbmNodeState bs { k->u, k->v, k->avgU, k->avgV, k->cgH, k->cgA, k->uo, k->vo, k->ua, k->va, k->uGrad, k->vGrad };
    const size_t dN = size_t(k->dg) * k->N;
    StageFields a;
    a.nf = bbm ? 3 : 2;
    double* fld[3] = { k->cice, k->hice, k->damage };
    for (int i = 0; i < a.nf; ++i) {
        a.src[i] = fld[i];
        a.phi[i] = fld[i];
        a.k1[i] = k->k1 + i * dN;
        a.dst[i] = k->phiA + i * dN;
    }
    auto launch = [&]() -> cudaError_t {
        switch (kernel_id) {
        case 0:
            if (!bbm && k->mixed())
                return k->launchStress32(k->stream, mp, k->derr);
            if (bbm)
                return launchBbmStress(k->stream, k->dm, k->dops, k->dg, k->u, k->v, k->hice, k->cice, k->damage,
                    k->s11, k->s12, k->s22, k->contrib, bp, k->derr, k->mixed() ? &k->bbm32 : nullptr);
            if (k->opsPairs && k->fp64Stress == 2)
                return launchMevpStressPairsTma(k->stream, k->dm, k->pairsMaps, k->u, k->v, k->Pg, k->contrib, mp,
                    k->derr);
            if (k->opsPairs && k->fp64Stress == 1)
                return launchMevpStressPairs(k->stream, k->dm, k->opsPairs, k->pairsLdN, k->u, k->v, k->Pg,
                    k->contrib, mp);
            return launchMevpStress(k->stream, k->dm, k->dops, k->u, k->v, k->Pg, k->contrib, mp);
        case 9:
            return launchMevpStress(k->stream, k->dm, k->dops, k->u, k->v, k->Pg, k->contrib, mp);
        case 10:
            return launchMevpStressPairs(k->stream, k->dm, k->opsPairs, k->pairsLdN, k->u, k->v, k->Pg, k->contrib,
                mp);
        case 11:
            return launchMevpStressPairsTma(k->stream, k->dm, k->pairsMaps, k->u, k->v, k->Pg, k->contrib, mp,
                k->derr);
        case 1:
            if (!bbm && k->mixed())
                return launchMevpMomentum32(k->stream, k->dm, k->st32, k->tdiv32, mp, k->derr);
            return bbm ? launchBbmMomentum(k->stream, k->dm, k->dops, bs, k->contrib, bp, k->derr,
                             k->mixed() ? k->invmHL : nullptr, (k->mixed() && k->bbmK0) ? &k->bbmConst : nullptr)
                       : launchMevpMomentum(k->stream, k->dm, k->dops, st, k->contrib, mp, k->derr);
        case 3:
        case 4:
            return k->launchStress32(k->stream, mp, k->derr, kernel_id == 4 ? 1 : 0);
        case 5:
        case 6:
        case 7:
        case 8:
            return k->launchStress32(k->stream, mp, k->derr, 2, kernel_id - 5);
        case 12:
            return k->launchStress32(k->stream, mp, k->derr, 2, 4);
        default: // 2: the step's transport stage; 13: the per-element transport kernel
            return k->launchTransport(k->stream, STAGE_RK2_A, dt, a, kernel_id == 13);
        }
    };
    const bool fp64Ids = kernel_id >= 9 && kernel_id <= 11;
    const bool affIds = (kernel_id >= 5 && kernel_id <= 8) || kernel_id == 12;
    if (kernel_id < 0 || kernel_id > 13 || (((kernel_id >= 3 && kernel_id <= 8) || kernel_id == 12)
            && (bbm || !k->mixed()))
        || (affIds && !k->affCoef) || (fp64Ids && (bbm || k->mixed()))
        || ((kernel_id == 10 || kernel_id == 11) && !k->opsPairs))
        return k->fail(NSDG_ERR_BAD_ARG,
            "time_kernel: kernel_id must be 0, 1, 2 (3, 4: mixed-precision mEVP; 5-8, 12: on parallelogram meshes; "
            "9-11: the FP64 mEVP stress kernels, FMA, float pairs and float pairs through TMA; 13: the "
            "per-element transport kernel)");
    static const char* kStress32Names[3] = { "kMevpStress32", "kMevpStress32Tma", "kMevpStress32Affine" };
    if (name)
        *name = kernel_id == 9 ? "kMevpStress" : kernel_id == 10 ? "kMevpStressPairs"
            : kernel_id == 11 ? "kMevpStressPairsTma"
            : kernel_id == 0 ? (bbm ? "kBbmStress"
                                    : (k->mixed() ? kStress32Names[k->stressKind]
                                                  : (k->opsPairs && k->fp64Stress == 2 ? "kMevpStressPairsTma"
                                                     : k->opsPairs && k->fp64Stress == 1 ? "kMevpStressPairs"
                                                                                         : "kMevpStress")))
            : kernel_id == 1 ? (bbm ? "kBbmMomentum" : (k->mixed() ? "kMevpMomentum32" : "kMevpMomentum"))
            : kernel_id == 2 ? (k->trAffine ? "kTransportStageAffine" : "kTransportStage")
            : kernel_id == 13 ? "kTransportStage"
            : kStress32Names[kernel_id >= 5 ? 2 : kernel_id - 3]; // 5-8, 12: the coefficient kernel
    cudaEvent_t ea, eb;
    if (cudaEventCreate(&ea) != cudaSuccess || cudaEventCreate(&eb) != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, "time_kernel: event create failed");
    cudaError_t e = launch(); // warm-up
    if (e == cudaSuccess) e = cudaStreamSynchronize(k->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ea, k->stream);
    for (int i = 0; i < reps && e == cudaSuccess; ++i)
        e = launch();
    if (e == cudaSuccess) e = cudaEventRecord(eb, k->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(eb);
    float ms = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, ea, eb);
    cudaEventDestroy(ea);
    cudaEventDestroy(eb);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("time_kernel: ") + cudaGetErrorString(e));
    *mean_ms = ms / reps;
    return k->ok();
}

int nsdg_kernel_stress_variant(nsdg_kernel* k, int* kind, double* mismatch)
{
    if (!k || !kind || !mismatch)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "stress_variant: kernel not initialised");
    if (k->mixed() && k->rheology == NSDG_RHEOLOGY_MEVP)
        *kind = k->stressKind;
    else if (k->mixed())
        *kind = k->bbm32.coef ? 2 : 0; // BBM: the parallelogram kernel or the per-element operators
    else
        *kind = -1;
    *mismatch = k->affWorst;
    return k->ok();
}

int nsdg_kernel_host_direct(nsdg_kernel* k, int* direct)
{
    if (!k || !direct)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "host_direct: kernel not initialised");
    *direct = k->hostDirect ? 1 : 0;
    return k->ok();
}

int nsdg_kernel_transport_variant(nsdg_kernel* k, int* tiled, double* cell_mismatch, double* offdiag)
{
    if (!k || !tiled || !cell_mismatch || !offdiag)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "transport_variant: kernel not initialised");
    *tiled = k->trAffine ? 1 : 0;
    *cell_mismatch = k->trAffWorst[0];
    *offdiag = k->trAffWorst[1];
    return k->ok();
}

int nsdg_kernel_viscosity_form(nsdg_kernel* k, int* form)
{
    if (!k || !form)
        return NSDG_ERR_BAD_ARG;
    *form = k->viscMode;
    return NSDG_OK;
}

int nsdg_kernel_launches_per_update(nsdg_kernel* k, int* launches)
{
    if (!k || !launches)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "launches_per_update: kernel not initialised");
    if (k->launchesPerUpdate == 0) {
        const int r = k->ensureGraph(k->graphDt > 0 ? k->graphDt : 120.0);
        if (r)
            return r;
    }
    *launches = k->launchesPerUpdate;
    return k->ok();
}

#define CUDA_TRY_K(expr)                                                                           \
    do {                                                                                           \
        cudaError_t e_ = (expr);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return k->fail(NSDG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_));    \
    } while (0)

int nsdg_kernel_warm_sample(nsdg_kernel* k, double t_start, double dt, int k_iters, nsdg_net* net, int slot,
    double* plain_ratio)
{
    if (k)
        k->readCache = 0;
    (void)t_start;
    if (!k || !net)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "warm_sample: kernel not initialised");
    if (k->rheology != NSDG_RHEOLOGY_MEVP || !k->mixed())
        return k->fail(NSDG_ERR_UNSUPPORTED, "warm_sample: mEVP in mixed precision only");
    if (!(dt > 0) || !std::isfinite(dt))
        return k->fail(NSDG_ERR_BAD_ARG, "warm_sample: dt must be positive");
    NetImpl* n = netImplOf(net);
    if (!netIsWarmShaped(n, k->dm.nx, k->dm.ny))
        return k->fail(NSDG_ERR_SIZE_MISMATCH, "warm_sample: the network does not match the grid / warm-start layout");
    if (slot >= netDatasetCapacity(n))
        return k->fail(NSDG_ERR_BAD_ARG, "warm_sample: slot outside the reserved dataset");
    if (k_iters < 1 || k_iters > k->P.n_steps)
        return k->fail(NSDG_ERR_BAD_ARG, "warm_sample: k_iters must be in [1, n_steps]");
    int r = k->allocWarm();
    if (r)
        return r;
    cudaStream_t s = k->stream;
    const bool record = slot >= 0;
    int l = 0;
    r = k->enqueuePhases(s, dt, nsdg_kernel::PHASE_PREP, l);
    if (r)
        return r;
    const WarmState ws = k->warmState();
    cudaError_t e = cudaSuccess;
    if (record) {
        e = launchWarmFeaturesRaw(s, ws, netDatasetFeatures(n, slot));
        if (e == cudaSuccess) e = launchWarmBase(s, ws, k->wbase, netDatasetMask(n, slot));
        if (e != cudaSuccess)
            return k->fail(NSDG_ERR_CUDA, std::string("warm_sample: ") + cudaGetErrorString(e));
    }
    r = k->saveLast(s, nullptr, nullptr, nullptr);
    if (r)
        return r;
    r = k->mixedIterations(s, dt, k->P.n_steps - k_iters, k->derr, l);
    if (r)
        return r;
    if (record) {
        e = launchWarmTargets(s, ws, k->wbase, netDatasetTargets(n, slot));
        if (e != cudaSuccess)
            return k->fail(NSDG_ERR_CUDA, std::string("warm_sample: ") + cudaGetErrorString(e));
    }
    r = k->mixedIterations(s, dt, k_iters - 1, k->derr, l);
    if (r)
        return r;
    e = launchWarmSave(s, k->Ncg, k->st32.u, k->uPrev, nullptr);
    if (e == cudaSuccess) e = launchWarmSave(s, k->Ncg, k->st32.v, k->vPrev, nullptr);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("warm_sample: ") + cudaGetErrorString(e));
    r = k->mixedIterations(s, dt, 1, k->derr, l);
    if (r)
        return r;
    e = launchWarmResidual(s, k->Ncg, k->st32.u, k->st32.v, k->uPrev, k->vPrev, k->st32.u0, k->st32.v0, k->wPart,
        k->wRes);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("warm_sample: ") + cudaGetErrorString(e));
    r = k->enqueuePhases(s, dt, nsdg_kernel::PHASE_FINISH, l);
    if (r)
        return r;
    double res[2] = { 0, 0 };
    e = cudaMemcpyAsync(res, k->wRes, sizeof(res), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess)
        return k->fail(NSDG_ERR_CUDA, std::string("warm_sample: ") + cudaGetErrorString(e));
    r = k->checkDeviceError();
    if (r)
        return r;
    ++k->stepNumber;
    if (plain_ratio)
        *plain_ratio = res[1] > 0 ? std::sqrt(res[0] / res[1]) : 0.0;
    return k->ok();
}

int nsdg_kernel_set_warm_start(nsdg_kernel* k, nsdg_net* net, int k_iters, double kappa, int audit_every,
    double audit_tol)
{
    if (!k)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return k->fail(NSDG_ERR_BAD_ARG, "set_warm_start: kernel not initialised");
    if (k->stream)
        cudaStreamSynchronize(k->stream);
    if (!net) {
        k->dropGraphs();
        k->warmNet = nullptr;
        k->warmK = 0;
        return k->ok();
    }
    if (k->rheology != NSDG_RHEOLOGY_MEVP || !k->mixed())
        return k->fail(NSDG_ERR_UNSUPPORTED, "set_warm_start: mEVP in mixed precision only");
    NetImpl* n = netImplOf(net);
    if (!netIsWarmShaped(n, k->dm.nx, k->dm.ny))
        return k->fail(NSDG_ERR_SIZE_MISMATCH, "set_warm_start: the network does not match the grid / warm-start layout");
    if (k_iters < 1 || k_iters > k->P.n_steps)
        return k->fail(NSDG_ERR_BAD_ARG, "set_warm_start: k_iters must be in [1, n_steps]");
    if (!(kappa >= 0) || !std::isfinite(kappa))
        return k->fail(NSDG_ERR_BAD_ARG, "set_warm_start: kappa must be finite and non-negative");
    if (audit_every < 0 || (audit_every > 0 && (!(audit_tol >= 0) || !std::isfinite(audit_tol))))
        return k->fail(NSDG_ERR_BAD_ARG, "set_warm_start: audit_every >= 0 and a finite audit_tol >= 0 needed");
    k->dropGraphs();
    const int r = k->allocWarm();
    if (r)
        return r;
    const int one = 1;
    CUDA_TRY_K(cudaMemsetAsync(k->rec.counts, 0, 4 * sizeof(long long), k->stream));
    CUDA_TRY_K(cudaMemcpyAsync(k->rec.enabled, &one, sizeof(int), cudaMemcpyHostToDevice, k->stream));
    CUDA_TRY_K(cudaStreamSynchronize(k->stream));
    k->warmNet = n;
    k->warmK = k_iters;
    k->warmKappa = kappa;
    k->auditEvery = audit_every;
    k->auditTol = audit_tol;
    k->warmSteps = 0;
    return k->ok();
}

int nsdg_kernel_warm_stats(nsdg_kernel* k, nsdg_warm_stats* out)
{
    if (!k || !out)
        return NSDG_ERR_BAD_ARG;
    if (!k->ready || !k->warmMem)
        return k->fail(NSDG_ERR_BAD_ARG, "warm_stats: no warm start attached");
    long long c[4] = { 0, 0, 0, 0 };
    double last[2] = { 0, 0 };
    int enabled = 0;
    CUDA_TRY_K(cudaMemcpyAsync(c, k->rec.counts, sizeof(c), cudaMemcpyDeviceToHost, k->stream));
    CUDA_TRY_K(cudaMemcpyAsync(&last[0], k->rec.lastRatio, sizeof(double), cudaMemcpyDeviceToHost, k->stream));
    CUDA_TRY_K(cudaMemcpyAsync(&last[1], k->rec.lastError, sizeof(double), cudaMemcpyDeviceToHost, k->stream));
    CUDA_TRY_K(cudaMemcpyAsync(&enabled, k->rec.enabled, sizeof(int), cudaMemcpyDeviceToHost, k->stream));
    CUDA_TRY_K(cudaStreamSynchronize(k->stream));
    out->accepted = c[0];
    out->fallbacks = c[1];
    out->audited = c[2];
    out->audit_rejected = c[3];
    out->last_ratio = last[0];
    out->last_audit_error = last[1];
    out->enabled = enabled;
    out->launches_warm = k->launchesPerUpdate;
    out->launches_audited = k->auditLaunches;
    out->launches_fallback = k->warmBodyLaunches;
    return k->ok();
}

} // extern "C"

// ===========================================================================
// Batched ensembles (nsdg_ensemble_*)
// ===========================================================================
struct nsdg_ensemble {
    std::vector<nsdg_kernel*> members;
    std::string err;
    cudaStream_t stream = nullptr;
    void* dmem = nullptr;
    EnsembleMember* dMembers = nullptr;
    uint16_t* dStressMap = nullptr;
    uint16_t* dNodeMap = nullptr;
    uint16_t* dTmaMap = nullptr;
    uint16_t* dNodeMapP = nullptr; // node blocks of the persistent sub-cycle
    unsigned* dBar = nullptr;      // its grid barrier (arrivals, generation)
    int* derr = nullptr;
    int stressBlocks = 0, nodeBlocks = 0, tmaBlocks = 0, nodeBlocksP = 0;
    // the sub-cycle as one persistent cooperative launch (parallelogram
    // members only) instead of two launches per iteration
    bool persistent = false;
    // element phase: 0 tiled global-load kernel, 1 TMA-staged, 2 parallelogram
    // coefficients (every member a parallelogram mesh)
    int elementKind = 0;
    int viscMode = 2;
    cudaError_t launchElements(cudaStream_t s, const EnsembleMember* table, const MevpParams& mp)
    {
        if (elementKind == 2)
            return launchMevpStress32AffineBatched(s, table, dTmaMap, tmaBlocks, mp, viscMode);
        return elementKind == 1 ? launchMevpStress32TmaBatched(s, table, dTmaMap, tmaBlocks, mp, derr)
                                : launchMevpStress32Batched(s, table, dStressMap, stressBlocks, mp);
    }
    std::vector<int> tileW;
    cudaGraphExec_t graph = nullptr;
    double graphDt = -1.0;
    int launches = 0;
    cudaEvent_t done = nullptr;

    int fail(int code, const std::string& m)
    {
        err = m;
        return code;
    }
    ~nsdg_ensemble()
    {
        if (stream)
            cudaStreamSynchronize(stream);
        if (graph)
            cudaGraphExecDestroy(graph);
        if (done)
            cudaEventDestroy(done);
        if (dmem)
            cudaFree(dmem);
        if (stream)
            cudaStreamDestroy(stream);
    }
    EnsembleMember describe(nsdg_kernel* k, int tw) const
    {
        EnsembleMember d {};
        d.nx = k->dm.nx;
        d.ny = k->dm.ny;
        d.N = k->N;
        d.Ncg = k->Ncg;
        d.ice = k->dm.ice;
        d.cg2Dir = k->dm.cg2Dir;
        d.invm2 = k->dops.invm2;
        d.o = k->dops32;
        d.st = k->st32;
        d.Pg = k->Pg;
        d.hP = k->hP32;
        d.tdiv = k->tdiv32;
        d.maps = k->maps32;
        d.affCoef = k->affCoef;
        d.affLd = k->affLd;
        d.tileW = tw;
        d.tileH = stressElementsPerBlock() / tw;
        d.tilesX = (d.nx + tw - 1) / tw;
        return d;
    }
    static int stressBlocksOf(const EnsembleMember& d) { return d.tilesX * ((d.ny + d.tileH - 1) / d.tileH); }
    static int nodeBlocksOf(const EnsembleMember& d)
    {
        return static_cast<int>((d.Ncg + nodesPerBlock() - 1) / nodesPerBlock());
    }
    static int tmaBlocksOf(const EnsembleMember& d) { return static_cast<int>((d.N + kTmaElems - 1) / kTmaElems); }
    int chooseElementKernel();
    int autotune();
    int build();
    int ensureGraph(double dt);
};

// Project-written autotuner: for every grid size in the ensemble, times the
// batched element kernel on that member alone for each tile shape
// (tileW x tileH, tileW * tileH = elements per block) and keeps the fastest.
// The divergence coefficients of the timing runs go to a scratch buffer, so
// the members' state is not touched.
int nsdg_ensemble::autotune()
{
    const int E = stressElementsPerBlock();
    std::vector<int> candidates;
    for (int w = E; w >= 8; w /= 2)
        candidates.push_back(w);
    size_t maxN = 0;
    for (auto* k : members)
        maxN = std::max(maxN, k->N);
    void* scratch = nullptr;
    EnsembleMember* dOne = nullptr;
    uint16_t* dMap = nullptr;
    size_t mapLen = 1;
    for (auto* k : members)
        for (int w : candidates)
            mapLen = std::max(mapLen, static_cast<size_t>(stressBlocksOf(describe(k, w))));
    if (cudaMalloc(&scratch, 18 * maxN * sizeof(float)) != cudaSuccess
        || cudaMalloc(&dOne, sizeof(EnsembleMember)) != cudaSuccess
        || cudaMalloc(&dMap, mapLen * sizeof(uint16_t)) != cudaSuccess) {
        cudaFree(scratch);
        cudaFree(dOne);
        return fail(NSDG_ERR_CUDA, "ensemble autotune: allocation failed");
    }
    cudaMemsetAsync(dMap, 0, mapLen * sizeof(uint16_t), stream);
    cudaMemsetAsync(scratch, 0, 18 * maxN * sizeof(float), stream);
    std::map<std::pair<int, int>, int> best;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    const nsdg_params& P = members[0]->P;
    MevpParams mp { P.rho_ice, P.F_atm, P.F_ocean, P.fc, P.gravity, P.Pstar, P.DeltaMin, P.alpha, P.beta, 120.0 };
    cudaError_t e = cudaSuccess;
    for (size_t mi = 0; mi < members.size() && e == cudaSuccess; ++mi) {
        nsdg_kernel* k = members[mi];
        const auto key = std::make_pair(k->dm.nx, k->dm.ny);
        if (best.count(key))
            continue;
        float bestMs = 1e30f;
        int bestW = E;
        for (int w : candidates) {
            EnsembleMember d = describe(k, w);
            d.tdiv = static_cast<float*>(scratch);
            d.stressBlock0 = 0;
            const int blocks = stressBlocksOf(d);
            e = cudaMemcpyAsync(dOne, &d, sizeof(d), cudaMemcpyHostToDevice, stream);
            for (int r = 0; r < 3 && e == cudaSuccess; ++r) // warm-up
                e = launchMevpStress32Batched(stream, dOne, dMap, blocks, mp);
            if (e == cudaSuccess) e = cudaEventRecord(a, stream);
            for (int r = 0; r < 10 && e == cudaSuccess; ++r)
                e = launchMevpStress32Batched(stream, dOne, dMap, blocks, mp);
            if (e == cudaSuccess) e = cudaEventRecord(b, stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(b);
            float ms = 0.f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
            if (e == cudaSuccess && ms < bestMs) {
                bestMs = ms;
                bestW = w;
            }
        }
        best[key] = bestW;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamSynchronize(stream);
    cudaFree(scratch);
    cudaFree(dOne);
    cudaFree(dMap);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("ensemble autotune: ") + cudaGetErrorString(e));
    tileW.clear();
    for (auto* k : members)
        tileW.push_back(best[std::make_pair(k->dm.nx, k->dm.ny)]);
    return NSDG_OK;
}

int nsdg_ensemble::build()
{
    std::vector<EnsembleMember> table;
    std::vector<uint16_t> smap, nmap, tmap, pmap;
    const size_t perP = static_cast<size_t>(persistentNodesPerBlock());
    for (size_t mi = 0; mi < members.size(); ++mi) {
        EnsembleMember d = describe(members[mi], tileW[mi]);
        d.stressBlock0 = static_cast<int>(smap.size());
        d.nodeBlock0 = static_cast<int>(nmap.size());
        d.tmaBlock0 = static_cast<int>(tmap.size());
        d.nodeBlockP = static_cast<int>(pmap.size());
        smap.insert(smap.end(), stressBlocksOf(d), static_cast<uint16_t>(mi));
        nmap.insert(nmap.end(), nodeBlocksOf(d), static_cast<uint16_t>(mi));
        tmap.insert(tmap.end(), tmaBlocksOf(d), static_cast<uint16_t>(mi));
        pmap.insert(pmap.end(), (d.Ncg + perP - 1) / perP, static_cast<uint16_t>(mi));
        table.push_back(d);
    }
    stressBlocks = static_cast<int>(smap.size());
    nodeBlocks = static_cast<int>(nmap.size());
    tmaBlocks = static_cast<int>(tmap.size());
    nodeBlocksP = static_cast<int>(pmap.size());
    const size_t bytes = al(table.size() * sizeof(EnsembleMember)) + al(smap.size() * 2) + al(nmap.size() * 2)
        + al(tmap.size() * 2) + al(pmap.size() * 2) + al(2 * sizeof(unsigned)) + al(4);
    if (cudaMalloc(&dmem, bytes) != cudaSuccess)
        return fail(NSDG_ERR_CUDA, "ensemble: allocation failed");
    char* p = static_cast<char*>(dmem);
    dMembers = reinterpret_cast<EnsembleMember*>(p);
    p += al(table.size() * sizeof(EnsembleMember));
    dStressMap = reinterpret_cast<uint16_t*>(p);
    p += al(smap.size() * 2);
    dNodeMap = reinterpret_cast<uint16_t*>(p);
    p += al(nmap.size() * 2);
    dTmaMap = reinterpret_cast<uint16_t*>(p);
    p += al(tmap.size() * 2);
    dNodeMapP = reinterpret_cast<uint16_t*>(p);
    p += al(pmap.size() * 2);
    dBar = reinterpret_cast<unsigned*>(p);
    p += al(2 * sizeof(unsigned));
    derr = reinterpret_cast<int*>(p);
    cudaError_t e = cudaMemcpy(dMembers, table.data(), table.size() * sizeof(EnsembleMember), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dStressMap, smap.data(), smap.size() * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dNodeMap, nmap.data(), nmap.size() * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dTmaMap, tmap.data(), tmap.size() * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dNodeMapP, pmap.data(), pmap.size() * 2, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(dBar, 0, 2 * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(derr, 0, sizeof(int));
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("ensemble: upload failed: ") + cudaGetErrorString(e));
    return chooseElementKernel();
}

// Times the element phase of the whole ensemble with the tiled global-load
// kernel (autotuned tiles) and with the TMA-staged kernel, the divergence
// redirected to scratch so that no member's state changes, and keeps the
// faster.
int nsdg_ensemble::chooseElementKernel()
{
    size_t total = 0;
    for (auto* k : members)
        total += 18 * k->N;
    std::vector<EnsembleMember> table;
    void* scratch = nullptr;
    EnsembleMember* dT = nullptr;
    if (cudaMalloc(&scratch, total * sizeof(float)) != cudaSuccess
        || cudaMalloc(&dT, members.size() * sizeof(EnsembleMember)) != cudaSuccess) {
        cudaFree(scratch);
        return fail(NSDG_ERR_CUDA, "ensemble: timing allocation failed");
    }
    std::vector<EnsembleMember> host(members.size());
    cudaError_t e = cudaMemcpy(host.data(), dMembers, host.size() * sizeof(EnsembleMember), cudaMemcpyDeviceToHost);
    size_t off = 0;
    for (size_t mi = 0; mi < host.size(); ++mi) {
        host[mi].tdiv = static_cast<float*>(scratch) + off;
        off += 18 * members[mi]->N;
    }
    if (e == cudaSuccess) e = cudaMemcpy(dT, host.data(), host.size() * sizeof(EnsembleMember), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(scratch, 0, total * sizeof(float));
    const nsdg_params& P = members[0]->P;
    MevpParams mp { P.rho_ice, P.F_atm, P.F_ocean, P.fc, P.gravity, P.Pstar, P.DeltaMin, P.alpha, P.beta, 120.0 };
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    float ms[2] = { 0, 0 };
    for (int variant = 0; variant < 2 && e == cudaSuccess; ++variant) {
        auto launch = [&]() {
            return variant == 0 ? launchMevpStress32Batched(stream, dT, dStressMap, stressBlocks, mp)
                                : launchMevpStress32TmaBatched(stream, dT, dTmaMap, tmaBlocks, mp, derr);
        };
        for (int r = 0; r < 2 && e == cudaSuccess; ++r)
            e = launch();
        if (e == cudaSuccess) e = cudaEventRecord(a, stream);
        for (int r = 0; r < 10 && e == cudaSuccess; ++r)
            e = launch();
        if (e == cudaSuccess) e = cudaEventRecord(b, stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[variant], a, b);
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaStreamSynchronize(stream);
    cudaFree(scratch);
    cudaFree(dT);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("ensemble: element kernel timing: ") + cudaGetErrorString(e));
    elementKind = ms[1] <= ms[0] ? 1 : 0;
    // parallelogram members take the coefficient kernel (as their single
    // runs do), when every member has coefficients
    bool allAffine = true;
    for (auto* k : members)
        allAffine = allAffine && k->affCoef != nullptr;
    if (allAffine) {
        elementKind = 2;
        viscMode = members[0]->viscMode;
    }
    if (const char* env = std::getenv("NSDG_STRESS_KERNEL")) {
        if (std::strcmp(env, "tma") == 0) elementKind = 1;
        if (std::strcmp(env, "global") == 0) elementKind = 0;
        if (std::strcmp(env, "affine") == 0 && allAffine) elementKind = 2;
    }
    return NSDG_OK;
}

int nsdg_ensemble::ensureGraph(double dt)
{
    if (graph && graphDt == dt)
        return NSDG_OK;
    if (graph) {
        cudaGraphExecDestroy(graph);
        graph = nullptr;
    }
    const nsdg_params& P = members[0]->P;
    MevpParams mp { P.rho_ice, P.F_atm, P.F_ocean, P.fc, P.gravity, P.Pstar, P.DeltaMin, P.alpha, P.beta, dt };
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("ensemble capture: ") + cudaGetErrorString(e));
    int total = 0, st = NSDG_OK;
    for (auto* k : members) {
        int l = 0;
        st = k->enqueuePhases(stream, dt, nsdg_kernel::PHASE_PREP, l);
        total += l;
        if (st) {
            err = k->err;
            break;
        }
    }
    if (persistent && elementKind == 2 && st == NSDG_OK) {
        e = launchEnsembleSubcyclePersistent(stream, dMembers, dTmaMap, tmaBlocks, dNodeMapP, nodeBlocksP, mp,
            viscMode, P.n_steps, dBar, derr);
        if (e != cudaSuccess)
            st = fail(NSDG_ERR_CUDA, std::string("ensemble persistent sub-cycle: ") + cudaGetErrorString(e));
        total += 1;
    }
    for (int it = 0; it < P.n_steps && st == NSDG_OK && !(persistent && elementKind == 2); ++it) {
        e = launchElements(stream, dMembers, mp);
        if (e == cudaSuccess)
            e = launchMevpMomentum32Batched(stream, dMembers, dNodeMap, nodeBlocks, mp, derr);
        if (e != cudaSuccess)
            st = fail(NSDG_ERR_CUDA, std::string("ensemble sub-cycle: ") + cudaGetErrorString(e));
        total += 2;
    }
    for (auto* k : members) {
        if (st)
            break;
        int l = 0;
        st = k->enqueuePhases(stream, dt, nsdg_kernel::PHASE_FINISH, l);
        total += l;
        if (st)
            err = k->err;
    }
    const cudaError_t ec = cudaStreamEndCapture(stream, &g);
    if (st) {
        if (g)
            cudaGraphDestroy(g);
        return st;
    }
    if (ec != cudaSuccess)
        return fail(NSDG_ERR_CUDA, std::string("ensemble capture: ") + cudaGetErrorString(ec));
    e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        graph = nullptr;
        return fail(NSDG_ERR_CUDA, std::string("ensemble instantiate: ") + cudaGetErrorString(e));
    }
    graphDt = dt;
    launches = total;
    return NSDG_OK;
}

extern "C" {

int nsdg_ensemble_create(nsdg_kernel* const* members, int n_members, nsdg_ensemble** out)
{
    if (!out || !members || n_members < 1 || n_members > 65535)
        return NSDG_ERR_BAD_ARG;
    *out = nullptr;
    const nsdg_params& P0 = members[0] ? members[0]->P : nsdg_params {};
    for (int i = 0; i < n_members; ++i) {
        const nsdg_kernel* k = members[i];
        if (!k || !k->ready || k->rheology != NSDG_RHEOLOGY_MEVP || !k->mixed() || k->mesh.spherical)
            return NSDG_ERR_UNSUPPORTED; // initialised Cartesian mEVP kernels in mixed precision only
        const nsdg_params& P = k->P;
        if (P.n_steps != P0.n_steps || P.alpha != P0.alpha || P.beta != P0.beta || P.rho_ice != P0.rho_ice
            || P.F_ocean != P0.F_ocean || P.F_atm != P0.F_atm || P.fc != P0.fc || P.gravity != P0.gravity
            || P.Pstar != P0.Pstar || P.DeltaMin != P0.DeltaMin)
            return NSDG_ERR_BAD_ARG; // the batched launches share one parameter set
        for (int j = 0; j < i; ++j)
            if (members[j] == k)
                return NSDG_ERR_BAD_ARG;
    }
    nsdg_ensemble* ens = new nsdg_ensemble();
    ens->members.assign(members, members + n_members);
    if (cudaStreamCreateWithFlags(&ens->stream, cudaStreamNonBlocking) != cudaSuccess
        || cudaEventCreateWithFlags(&ens->done, cudaEventDisableTiming) != cudaSuccess) {
        delete ens;
        return NSDG_ERR_CUDA;
    }
    for (auto* k : ens->members)
        cudaStreamSynchronize(k->stream);
    if (ens->autotune() != NSDG_OK || ens->build() != NSDG_OK) {
        delete ens;
        return NSDG_ERR_CUDA;
    }
    *out = ens;
    return NSDG_OK;
}

int nsdg_ensemble_destroy(nsdg_ensemble* ens)
{
    if (!ens)
        return NSDG_ERR_BAD_ARG;
    delete ens;
    return NSDG_OK;
}

const char* nsdg_ensemble_last_error(const nsdg_ensemble* ens) { return ens ? ens->err.c_str() : "null handle"; }

int nsdg_ensemble_update(nsdg_ensemble* ens, double t_start, double dt)
{
    if (ens)
        for (auto* m : ens->members)
            m->readCache = 0;
    (void)t_start;
    if (!ens)
        return NSDG_ERR_BAD_ARG;
    if (!(dt > 0) || !std::isfinite(dt))
        return ens->fail(NSDG_ERR_BAD_ARG, "update: dt must be positive");
    int r = ens->ensureGraph(dt);
    if (r)
        return r;
    // order the graph after the members' own streams, and their later reads after the graph
    for (auto* k : ens->members) {
        cudaEvent_t ev;
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        cudaEventRecord(ev, k->stream);
        cudaStreamWaitEvent(ens->stream, ev, 0);
        cudaEventDestroy(ev);
    }
    cudaError_t e = cudaGraphLaunch(ens->graph, ens->stream);
    if (e == cudaSuccess) e = cudaEventRecord(ens->done, ens->stream);
    for (auto* k : ens->members) {
        if (e == cudaSuccess) e = cudaStreamWaitEvent(k->stream, ens->done, 0);
        ++k->stepNumber;
    }
    if (e != cudaSuccess)
        return ens->fail(NSDG_ERR_CUDA, std::string("update: ") + cudaGetErrorString(e));
    ens->err.clear();
    return NSDG_OK;
}

int nsdg_ensemble_set_persistent(nsdg_ensemble* ens, int on)
{
    if (!ens)
        return NSDG_ERR_BAD_ARG;
    if (on && ens->elementKind != 2)
        return ens->fail(NSDG_ERR_UNSUPPORTED, "set_persistent: every member must be a parallelogram mesh");
    if (ens->stream)
        cudaStreamSynchronize(ens->stream);
    if (ens->graph) {
        cudaGraphExecDestroy(ens->graph);
        ens->graph = nullptr;
    }
    ens->persistent = on != 0;
    ens->err.clear();
    return NSDG_OK;
}

int nsdg_ensemble_synchronize(nsdg_ensemble* ens)
{
    if (!ens)
        return NSDG_ERR_BAD_ARG;
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, ens->derr, sizeof(int), cudaMemcpyDeviceToHost, ens->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ens->stream);
    if (e != cudaSuccess)
        return ens->fail(NSDG_ERR_CUDA, std::string("synchronize: ") + cudaGetErrorString(e));
    if (h) {
        cudaMemsetAsync(ens->derr, 0, sizeof(int), ens->stream);
        if (h & DEV_ERR_TIMEOUT)
            return ens->fail(NSDG_ERR_CUDA, "a bounded wait of the ensemble's sub-cycle ran out");
        return ens->fail(NSDG_ERR_NUMERIC, "non-finite velocity in an ensemble member");
    }
    return NSDG_OK;
}

int nsdg_ensemble_time_updates(nsdg_ensemble* ens, double dt, int steps, float* ms)
{
    if (ens)
        for (auto* m : ens->members)
            m->readCache = 0;
    if (!ens || !ms || steps < 1)
        return NSDG_ERR_BAD_ARG;
    int r = ens->ensureGraph(dt);
    if (r)
        return r;
    for (auto* k : ens->members)
        cudaStreamSynchronize(k->stream);
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaError_t e = cudaEventRecord(a, ens->stream);
    for (int i = 0; i < steps && e == cudaSuccess; ++i)
        e = cudaGraphLaunch(ens->graph, ens->stream);
    if (e == cudaSuccess) e = cudaEventRecord(b, ens->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (e != cudaSuccess)
        return ens->fail(NSDG_ERR_CUDA, std::string("time_updates: ") + cudaGetErrorString(e));
    for (auto* k : ens->members)
        k->stepNumber += steps;
    return nsdg_ensemble_synchronize(ens);
}

int nsdg_ensemble_tile(nsdg_ensemble* ens, int member, int* tile_w, int* tile_h)
{
    if (!ens || !tile_w || !tile_h || member < 0 || member >= static_cast<int>(ens->members.size()))
        return NSDG_ERR_BAD_ARG;
    if (ens->elementKind != 0) {
        *tile_w = kTmaElems; // consecutive elements (operators staged by TMA, or parallelogram coefficients)
        *tile_h = 1;
    } else {
        *tile_w = ens->tileW[member];
        *tile_h = stressElementsPerBlock() / ens->tileW[member];
    }
    return NSDG_OK;
}

int nsdg_ensemble_launches_per_update(nsdg_ensemble* ens, int* launches)
{
    if (!ens || !launches)
        return NSDG_ERR_BAD_ARG;
    if (!ens->graph) {
        const int r = ens->ensureGraph(120.0);
        if (r)
            return r;
    }
    *launches = ens->launches;
    return NSDG_OK;
}

int nsdg_mesh_parallelogram_mismatch(size_t nx, size_t ny, const double* coords, int dg_comp, double* mismatch)
{
    if (!coords || !mismatch || nx < 1 || ny < 1 || (dg_comp != 1 && dg_comp != 3 && dg_comp != 6))
        return NSDG_ERR_BAD_ARG;
    HostMesh m;
    m.nx = nx;
    m.ny = ny;
    const size_t nn = (nx + 1) * (ny + 1);
    m.vx.resize(nn);
    m.vy.resize(nn);
    for (size_t i = 0; i < nn; ++i) {
        m.vx[i] = coords[2 * i];
        m.vy[i] = coords[2 * i + 1];
        if (!std::isfinite(m.vx[i]) || !std::isfinite(m.vy[i]))
            return NSDG_ERR_BAD_ARG;
    }
    m.ice.assign(nx * ny, 1);
    ElementOps ops;
    buildElementOps(m, dg_comp, false, ops);
    AffineStressOps aff;
    buildAffineStressOps(m, ops, m.nelements(), 0.0, aff);
    *mismatch = aff.worst;
    return NSDG_OK;
}

int nsdg_mesh_parallelogram_checks(size_t nx, size_t ny, const double* coords, int dg_comp, double* out)
{
    if (!coords || !out || nx < 1 || ny < 1 || (dg_comp != 1 && dg_comp != 3 && dg_comp != 6))
        return NSDG_ERR_BAD_ARG;
    HostMesh m;
    m.nx = nx;
    m.ny = ny;
    const size_t nn = (nx + 1) * (ny + 1);
    m.vx.resize(nn);
    m.vy.resize(nn);
    for (size_t i = 0; i < nn; ++i) {
        m.vx[i] = coords[2 * i];
        m.vy[i] = coords[2 * i + 1];
        if (!std::isfinite(m.vx[i]) || !std::isfinite(m.vy[i]))
            return NSDG_ERR_BAD_ARG;
    }
    m.ice.assign(nx * ny, 1);
    ElementOps ops;
    buildElementOps(m, dg_comp, true, ops);
    AffineStressOps aff;
    buildAffineStressOps(m, ops, m.nelements(), 0.0, aff);
    AffineTransportOps atr;
    buildAffineTransportOps(m, ops, 0.0, 0.0, atr);
    AffineBbmOps abb;
    buildAffineBbmOps(m, ops, 0.0, abb);
    out[0] = aff.worst;
    out[1] = atr.worstCell;
    out[2] = atr.worstOffDiag;
    out[3] = abb.worst;
    return NSDG_OK;
}

int nsdg_mesh_dirichlet(size_t nx, size_t ny, const double* mask, size_t* counts, size_t* ids, size_t capacity)
{
    if (!mask || !counts || nx < 1 || ny < 1 || (capacity > 0 && !ids))
        return NSDG_ERR_BAD_ARG;
    HostMesh m;
    m.nx = nx;
    m.ny = ny;
    m.ice.resize(nx * ny);
    for (size_t i = 0; i < nx * ny; ++i)
        m.ice[i] = (mask[i] == 1.0) ? 1 : 0; // the kernel's initialise rule
    m.dirichletFromMaskAndEdges();
    size_t total = 0;
    for (int s = 0; s < 4; ++s) {
        counts[s] = m.dirichlet[s].size();
        total += counts[s];
    }
    if (total > capacity)
        return NSDG_ERR_SIZE_MISMATCH;
    for (const auto& d : m.dirichlet)
        for (size_t e : d)
            *ids++ = e;
    return NSDG_OK;
}

// the viscosity self-tests: forms = 3 (modes 0, 1, 2) or 1 (mode 3)
// kind 0: forms 0, 1, 2 (out[3 n]); 1: form 3; 2: form 4 (out[n])
static int viscositySelfTest(size_t n, const float* inv, const double* Pa, double delta_min, float* out,
    int kind)
{
    const int forms = kind == 0 ? 3 : 1;
    if (!inv || !Pa || !out || n == 0 || n > (size_t(1) << 26) || !(delta_min > 0.0))
        return NSDG_ERR_BAD_ARG;
    std::string m;
    const int st = deviceCheck(m);
    if (st != NSDG_OK)
        return st;
    float *dInv = nullptr, *dOut = nullptr;
    double* dPa = nullptr;
    cudaStream_t s = nullptr;
    const size_t nOut = size_t(forms) * n;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&dInv, n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&dPa, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dOut, nOut * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dInv, inv, n * sizeof(float), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dPa, Pa, n * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = kind == 1 ? launchViscositySelfTestFF(s, n, dInv, dPa, delta_min, dOut)
            : kind == 2   ? launchViscositySelfTestChecked(s, n, dInv, dPa, delta_min, dOut)
                          : launchViscositySelfTest(s, n, dInv, dPa, delta_min, dOut);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dOut, nOut * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (void* p : { static_cast<void*>(dInv), static_cast<void*>(dPa), static_cast<void*>(dOut) })
        if (p)
            cudaFree(p);
    if (s)
        cudaStreamDestroy(s);
    return e == cudaSuccess ? NSDG_OK : NSDG_ERR_CUDA;
}

int nsdg_selftest_viscosity(size_t n, const float* inv, const double* Pa, double delta_min, float* out)
{
    return viscositySelfTest(n, inv, Pa, delta_min, out, 0);
}

int nsdg_selftest_viscosity_ff(size_t n, const float* inv, const double* Pa, double delta_min, float* out)
{
    return viscositySelfTest(n, inv, Pa, delta_min, out, 1);
}

int nsdg_selftest_viscosity_checked(size_t n, const float* inv, const double* Pa, double delta_min, float* out)
{
    return viscositySelfTest(n, inv, Pa, delta_min, out, 2);
}

int nsdg_selftest_pairs(size_t n, const double* a, const double* x, double* out)
{
    if (!a || !x || !out || n == 0)
        return NSDG_ERR_BAD_ARG;
    std::string m;
    const int st = deviceCheck(m);
    if (st != NSDG_OK)
        return st;
    double *da = nullptr, *dx = nullptr, *dout = nullptr;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&da, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dx, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dout, 4 * n * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpyAsync(da, a, n * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, n * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launchPairsSelfTest(s, n, da, dx, dout);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, dout, 4 * n * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(da);
    cudaFree(dx);
    cudaFree(dout);
    if (s)
        cudaStreamDestroy(s);
    return e == cudaSuccess ? NSDG_OK : NSDG_ERR_CUDA;
}

int nsdg_selftest_bounded_wait(double limit_seconds, int* timed_out)
{
    if (!timed_out || !(limit_seconds > 0.0) || limit_seconds > 2.0)
        return NSDG_ERR_BAD_ARG;
    std::string m;
    const int st = deviceCheck(m);
    if (st != NSDG_OK)
        return st;
    int* d = nullptr;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&d, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0xff, sizeof(int), s);
    if (e == cudaSuccess) e = launchBoundedWaitSelfTest(s, limit_seconds, d);
    int h = -1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (d)
        cudaFree(d);
    if (s)
        cudaStreamDestroy(s);
    if (e != cudaSuccess)
        return NSDG_ERR_CUDA;
    *timed_out = h;
    return NSDG_OK;
}

int nsdg_ice_growth_exchange(nsdg_ice_growth* g, nsdg_kernel* k, int direction)
{
    if (!g || !k || (direction != 0 && direction != 1))
        return NSDG_ERR_BAD_ARG;
    if (!k->ready)
        return g->fail(NSDG_ERR_BAD_ARG, "exchange: the dynamics kernel is not initialised");
    if (k->N != g->n)
        return g->fail(NSDG_ERR_SIZE_MISMATCH, "exchange: the dynamics mesh has a different element count");
    // the damage field is device state of the BBM kernel only (an mEVP
    // handle keeps "damage" as a stored, unused field)
    double* damage = k->rheology == NSDG_RHEOLOGY_BBM ? k->damage : nullptr;
    cudaEvent_t ev = nullptr;
    cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    // the growth stream waits for the dynamics' queued work, runs the copy,
    // and the dynamics stream waits for the copy before its next work
    if (e == cudaSuccess) e = cudaEventRecord(ev, k->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(g->stream, ev, 0);
    if (e == cudaSuccess)
        e = direction == 0 ? launchIceGrowthFromDynamics(g->stream, g->n, k->hice, k->cice, damage, g->fields)
                           : launchIceGrowthToDynamics(g->stream, g->n, k->dg, g->fields, k->hice, k->cice, damage);
    if (e == cudaSuccess) e = cudaEventRecord(ev, g->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(k->stream, ev, 0);
    if (ev)
        cudaEventDestroy(ev);
    if (e != cudaSuccess)
        return g->fail(NSDG_ERR_CUDA, std::string("exchange: ") + cudaGetErrorString(e));
    if (direction == 1)
        k->readCache = 0; // the dynamics state changed
    g->err.clear();
    return NSDG_OK;
}

} // extern "C"
