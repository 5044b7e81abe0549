// nsdg_transport_capi.cpp — the stand-alone DG transport handle
// (nsdg_transport_* in include/nsdg.h), the GPU counterpart of the
// reference's DGTransport<DG> class used by its transport tests
// (dynamics/src/include/DGTransport.hpp:27-152).
#include "nsdg.h"

#include "nsdg_host.hpp"
#include "nsdg_kernels.hpp"

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

using namespace nsdg;

struct nsdg_transport {
    int dg = 1, scheme = 2;
    std::string err;
    cudaStream_t stream = nullptr;
    void* arena = nullptr;
    HostMesh mesh;
    BoundaryFlags flags;
    DevMesh dm;
    DevOps ops;
    double *phi = nullptr, *t1 = nullptr, *t2 = nullptr, *k1 = nullptr;
    double *velx = nullptr, *vely = nullptr, *nvX = nullptr, *nvY = nullptr;
    double *staging = nullptr, *partials = nullptr, *dsum = nullptr;

    int fail(int code, const std::string& m)
    {
        err = m;
        return code;
    }
    int cuda(cudaError_t e, const char* what)
    {
        if (e == cudaSuccess)
            return NSDG_OK;
        return fail(NSDG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    }
    ~nsdg_transport()
    {
        if (stream)
            cudaStreamSynchronize(stream);
        if (arena)
            cudaFree(arena);
        if (stream)
            cudaStreamDestroy(stream);
    }
};

extern "C" {

int nsdg_transport_create(int dg, size_t nx, size_t ny, const double* vertices,
    const unsigned char* landmask, const size_t* const dirichlet[4], const size_t n_dirichlet[4],
    const size_t* periodic, size_t n_periodic, int scheme, nsdg_transport** out)
{
    if (!out)
        return NSDG_ERR_BAD_ARG;
    *out = nullptr;
    if ((dg != 1 && dg != 3 && dg != 6 && dg != 8) || nx < 1 || ny < 1 || !vertices)
        return NSDG_ERR_BAD_ARG;
    if (scheme < 1 || scheme > 3)
        return NSDG_ERR_BAD_ARG;
    if (n_periodic && !periodic)
        return NSDG_ERR_BAD_ARG;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return NSDG_ERR_NO_DEVICE;
    }
    nsdg_transport* t = new nsdg_transport();
    t->dg = dg;
    t->scheme = scheme;
    HostMesh& m = t->mesh;
    m.nx = nx;
    m.ny = ny;
    const size_t nn = (nx + 1) * (ny + 1), N = nx * ny;
    m.vx.resize(nn);
    m.vy.resize(nn);
    for (size_t i = 0; i < nn; ++i) {
        m.vx[i] = vertices[2 * i];
        m.vy[i] = vertices[2 * i + 1];
    }
    m.ice.assign(N, 1);
    if (landmask)
        for (size_t i = 0; i < N; ++i)
            m.ice[i] = landmask[i] ? 1 : 0;
    for (int s = 0; s < 4; ++s) {
        const size_t n = n_dirichlet ? n_dirichlet[s] : 0;
        if (n && (!dirichlet || !dirichlet[s])) {
            delete t;
            return NSDG_ERR_BAD_ARG;
        }
        for (size_t i = 0; i < n; ++i)
            m.dirichlet[s].push_back(dirichlet[s][i]);
    }
    for (size_t i = 0; i < n_periodic; ++i)
        m.periodic.push_back({ periodic[4 * i], periodic[4 * i + 1], periodic[4 * i + 2], periodic[4 * i + 3] });
    if (!buildBoundaryFlags(m, t->flags).empty()) {
        delete t;
        return NSDG_ERR_BAD_ARG;
    }
    ElementOps eo;
    buildTransportOps(m, dg, eo);

    const size_t nXe = nx * (ny + 1), nYe = (nx + 1) * ny;
    const int ED = edgeDofs(dg);
    const size_t dN = size_t(dg) * N;
    auto al = [](size_t b) { return ((b + 255) / 256) * 256; };
    size_t bytes = 0;
    const size_t sizes8[] = { nn, nn, eo.cellX.size(), eo.cellY.size(), eo.minv.size(), eo.jwA.size(),
        eo.jw3.size(), dN, dN, dN, dN, dN, dN, ED * nXe, ED * nYe, 8 * N, (N + 255) / 256 + 1, 1 };
    for (size_t s : sizes8)
        bytes += al(s * 8);
    bytes += al(N) * 2 + al(nXe) + al(nYe) + al(size_t(2 * nx + 1) * (2 * ny + 1)) + al((N + 1) * 4)
        + al(std::max<size_t>(t->flags.perEntry.size(), 1) * 4);
    if (t->cuda(cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking), "stream") != NSDG_OK
        || t->cuda(uploadConstTables(), "tables") != NSDG_OK
        || t->cuda(cudaMalloc(&t->arena, bytes), "malloc") != NSDG_OK) {
        delete t;
        return NSDG_ERR_CUDA;
    }
    char* p = static_cast<char*>(t->arena);
    cudaError_t e = cudaSuccess;
    auto take = [&](const void* src, size_t bytesN) {
        void* q = p;
        p += al(bytesN);
        if (src && e == cudaSuccess)
            e = cudaMemcpyAsync(q, src, bytesN, cudaMemcpyHostToDevice, t->stream);
        else if (!src && e == cudaSuccess)
            e = cudaMemsetAsync(q, 0, bytesN, t->stream);
        return q;
    };
    DevMesh& d = t->dm;
    d.nx = static_cast<int>(nx);
    d.ny = static_cast<int>(ny);
    d.N = N;
    d.Ncg = size_t(2 * nx + 1) * (2 * ny + 1);
    d.Ncg1 = nn;
    d.nXe = nXe;
    d.nYe = nYe;
    d.vx = static_cast<double*>(take(m.vx.data(), nn * 8));
    d.vy = static_cast<double*>(take(m.vy.data(), nn * 8));
    d.ice = static_cast<uint8_t*>(take(m.ice.data(), N));
    d.cellSeg = static_cast<uint8_t*>(take(t->flags.cellSeg.data(), N));
    d.edgeXCount = static_cast<uint8_t*>(take(t->flags.edgeXCount.data(), nXe));
    d.edgeYCount = static_cast<uint8_t*>(take(t->flags.edgeYCount.data(), nYe));
    d.cg2Dir = static_cast<uint8_t*>(take(t->flags.cg2Dirichlet.data(), d.Ncg));
    d.perPtr = static_cast<int*>(take(t->flags.perPtr.data(), (N + 1) * 4));
    d.perEntry = static_cast<int*>(take(t->flags.perEntry.empty() ? nullptr : t->flags.perEntry.data(),
        std::max<size_t>(t->flags.perEntry.size(), 1) * 4));
    t->ops.cellX = static_cast<double*>(take(eo.cellX.data(), eo.cellX.size() * 8));
    t->ops.cellY = static_cast<double*>(take(eo.cellY.data(), eo.cellY.size() * 8));
    t->ops.minv = static_cast<double*>(take(eo.minv.data(), eo.minv.size() * 8));
    t->ops.jwA = static_cast<double*>(take(eo.jwA.data(), eo.jwA.size() * 8));
    t->ops.jw3 = static_cast<double*>(take(eo.jw3.data(), eo.jw3.size() * 8));
    t->phi = static_cast<double*>(take(nullptr, dN * 8));
    t->t1 = static_cast<double*>(take(nullptr, dN * 8));
    t->t2 = static_cast<double*>(take(nullptr, dN * 8));
    t->k1 = static_cast<double*>(take(nullptr, dN * 8));
    t->velx = static_cast<double*>(take(nullptr, dN * 8));
    t->vely = static_cast<double*>(take(nullptr, dN * 8));
    t->nvX = static_cast<double*>(take(nullptr, ED * nXe * 8));
    t->nvY = static_cast<double*>(take(nullptr, ED * nYe * 8));
    t->staging = static_cast<double*>(take(nullptr, 8 * N * 8));
    t->partials = static_cast<double*>(take(nullptr, ((N + 255) / 256 + 1) * 8));
    t->dsum = static_cast<double*>(take(nullptr, 8));
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(t->stream);
    if (e != cudaSuccess) {
        delete t;
        return NSDG_ERR_CUDA;
    }
    *out = t;
    return NSDG_OK;
}

int nsdg_transport_destroy(nsdg_transport* t)
{
    if (!t)
        return NSDG_ERR_BAD_ARG;
    delete t;
    return NSDG_OK;
}

const char* nsdg_transport_last_error(const nsdg_transport* t) { return t ? t->err.c_str() : "null handle"; }

int nsdg_transport_set_velocity(nsdg_transport* t, const double* vx, const double* vy)
{
    if (!t || !vx || !vy)
        return NSDG_ERR_BAD_ARG;
    const size_t N = t->dm.N;
    const size_t bytes = N * t->dg * sizeof(double);
    int r = t->cuda(cudaMemcpyAsync(t->staging, vx, bytes, cudaMemcpyHostToDevice, t->stream), "set_velocity");
    if (!r) r = t->cuda(launchAosToSoa(t->stream, N, t->dg, t->dg, t->staging, t->velx), "set_velocity");
    if (!r) r = t->cuda(cudaMemcpyAsync(t->staging, vy, bytes, cudaMemcpyHostToDevice, t->stream), "set_velocity");
    if (!r) r = t->cuda(launchAosToSoa(t->stream, N, t->dg, t->dg, t->staging, t->vely), "set_velocity");
    if (!r) r = t->cuda(cudaStreamSynchronize(t->stream), "set_velocity");
    return r;
}

int nsdg_transport_reinit_normal_velocity(nsdg_transport* t)
{
    if (!t)
        return NSDG_ERR_BAD_ARG;
    return t->cuda(launchNormalVelocity(t->stream, t->dm, t->dg, t->velx, t->vely, t->nvX, t->nvY),
        "reinit_normal_velocity");
}

int nsdg_transport_step(nsdg_transport* t, double dt, double* phi, int nsteps, int limit_max,
    double max_value, int limit_min, double min_value)
{
    if (!t || !phi || nsteps < 0 || !std::isfinite(dt))
        return NSDG_ERR_BAD_ARG;
    const size_t N = t->dm.N;
    const int dg = t->dg;
    const size_t bytes = N * dg * sizeof(double);
    int r = t->cuda(cudaMemcpyAsync(t->staging, phi, bytes, cudaMemcpyHostToDevice, t->stream), "step upload");
    if (!r) r = t->cuda(launchAosToSoa(t->stream, N, dg, dg, t->staging, t->phi), "step upload");
    auto stage = [&](int mode, const double* src, double* dst, bool last) {
        StageFields f;
        f.nf = 1;
        f.src[0] = src;
        f.phi[0] = t->phi;
        f.k1[0] = t->k1;
        f.dst[0] = dst;
        if (last) {
            f.lmax[0] = limit_max;
            f.vmax[0] = max_value;
            f.lmin[0] = limit_min;
            f.vmin[0] = min_value;
        }
        return t->cuda(launchTransportStage(t->stream, t->dm, dg, t->ops.cellX, t->ops.cellY, t->ops.minv,
                           t->velx, t->vely, t->nvX, t->nvY, mode, dt, f),
            "transport stage");
    };
    for (int s = 0; s < nsteps && !r; ++s) {
        if (t->scheme == 1) {
            r = stage(STAGE_RK1, t->phi, t->t1, true);
            if (!r)
                r = t->cuda(cudaMemcpyAsync(t->phi, t->t1, bytes, cudaMemcpyDeviceToDevice, t->stream), "rk1 copy");
        } else if (t->scheme == 2) {
            r = stage(STAGE_RK2_A, t->phi, t->t1, false);
            if (!r) r = stage(STAGE_RK2_B, t->t1, t->phi, true);
        } else {
            r = stage(STAGE_RK3_A, t->phi, t->t1, false);
            if (!r) r = stage(STAGE_RK3_B, t->t1, t->t2, false);
            if (!r) r = stage(STAGE_RK3_C, t->t2, t->phi, true);
        }
    }
    if (!r) r = t->cuda(launchSoaToAos(t->stream, N, dg, dg, t->phi, t->staging), "step download");
    if (!r) r = t->cuda(cudaMemcpyAsync(phi, t->staging, bytes, cudaMemcpyDeviceToHost, t->stream), "step download");
    if (!r) r = t->cuda(cudaStreamSynchronize(t->stream), "step sync");
    return r;
}

int nsdg_transport_mean_value(nsdg_transport* t, const double* phi, double* out)
{
    if (!t || !phi || !out)
        return NSDG_ERR_BAD_ARG;
    const size_t N = t->dm.N;
    const int dg = t->dg;
    int r = t->cuda(cudaMemcpyAsync(t->staging, phi, N * dg * sizeof(double), cudaMemcpyHostToDevice, t->stream),
        "mean_value upload");
    if (!r) r = t->cuda(launchAosToSoa(t->stream, N, dg, dg, t->staging, t->t2), "mean_value upload");
    if (!r) r = t->cuda(launchMeanValue(t->stream, N, dg, t->t2, t->ops.jw3, t->partials, t->dsum), "mean_value");
    if (!r) r = t->cuda(cudaMemcpyAsync(out, t->dsum, sizeof(double), cudaMemcpyDeviceToHost, t->stream), "mean_value");
    if (!r) r = t->cuda(cudaStreamSynchronize(t->stream), "mean_value sync");
    return r;
}

} // extern "C"
