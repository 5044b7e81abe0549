/*
 * nsdg_oracle.cpp — CPU FP64 oracle for the neXtSIM_DG dynamics hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: only tests/, the
 * smoke check and bench.py's CPU-baseline leg load it.  The product (the
 * CUDA library under nextsimdg_gb300/csrc) never links or calls it.
 *
 * What it is: a plain C++17 restatement (no Eigen) of the reference's
 * algorithms, function by function, each citing the reference file:line it
 * follows (paths relative to the nextsimdg project root).  The reference
 * itself cannot be compiled here: its numerics need Eigen 3.4, an external
 * library that is neither vendored nor installed.
 *
 * Parity status:
 *   - DG transport, limiters, Function2DG, L2ErrorFunctionDG, MeanValue, mesh
 *     geometry and the basis/quadrature tables are PINNED against the
 *     reference's own golden values (dynamics/test/Advection_test.cpp:274-301,
 *     dynamics/test/AdvectionPeriodicBC_test.cpp:281-290, tolerance 1e-7).
 *   - The mEVP / BBM stress updates, strain, stress divergence, momentum and
 *     the full kernel update are restated from the sources; no reference test
 *     exercises them, so that half is "parity unpinned".
 *   - Spherical meshes (pole rotation, longitude continuity, cos(lat) weights,
 *     the divM / iMM metric terms) have no reference test either; the
 *     geometry is checked against the exact area of a lon/lat rectangle on
 *     the unit sphere (tests/test_oracle_spherical.py).
 *   - The closed (Dirichlet) element sides derived from a land mask are
 *     PINNED against the lists stored in the reference's 25 km Arctic mesh
 *     fixture (dynamics/test/ParametricMesh_test.cpp:87-138, exact).
 *
 * Arithmetic: FP64 throughout, compiled with -ffp-contract=off so x86-64 and
 * aarch64 give identical results.  Sums run in the order the reference's
 * loops accumulate (row stripes, edge order), small matrix products as plain
 * sequential dot products.
 */
#include "nsdg.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

/* ------------------------------------------------------------------------ */
/* Quadrature and basis functions                                           */
/* dynamics/codegeneration/gaussquadrature.py:7-29, basisfunctions.py:33-160 */
/* ------------------------------------------------------------------------ */
struct Quadrature {
    double p[5][4];
    double w[5][4];
    Quadrature()
    {
        std::memset(p, 0, sizeof(p));
        std::memset(w, 0, sizeof(w));
        p[1][0] = 0.5;
        w[1][0] = 1.0;
        p[2][0] = 0.5 - std::sqrt(1. / 12.);
        p[2][1] = 0.5 + std::sqrt(1. / 12.);
        w[2][0] = 0.5;
        w[2][1] = 0.5;
        p[3][0] = 0.5 - std::sqrt(3. / 20.);
        p[3][1] = 0.5;
        p[3][2] = 0.5 + std::sqrt(3. / 20.);
        w[3][0] = 5. / 18.;
        w[3][1] = 8. / 18.;
        w[3][2] = 5. / 18.;
        p[4][0] = 0.5 - 0.5 * std::sqrt(3. / 7. + 2. / 7. * std::sqrt(6. / 5.));
        p[4][1] = 0.5 - 0.5 * std::sqrt(3. / 7. - 2. / 7. * std::sqrt(6. / 5.));
        p[4][2] = 0.5 + 0.5 * std::sqrt(3. / 7. - 2. / 7. * std::sqrt(6. / 5.));
        p[4][3] = 0.5 + 0.5 * std::sqrt(3. / 7. + 2. / 7. * std::sqrt(6. / 5.));
        w[4][0] = (18. - std::sqrt(30.0)) / 72.;
        w[4][1] = (18. + std::sqrt(30.0)) / 72.;
        w[4][2] = (18. + std::sqrt(30.0)) / 72.;
        w[4][3] = (18. - std::sqrt(30.0)) / 72.;
    }
};
static const Quadrature QUAD;

// basisfunctions.py:33-52 (dgbasis)
static double dgbasis(int j, double x, double y)
{
    switch (j) {
    case 0: return 1.;
    case 1: return x - 0.5;
    case 2: return y - 0.5;
    case 3: return (x - 0.5) * (x - 0.5) - 1.0 / 12.0;
    case 4: return (y - 0.5) * (y - 0.5) - 1.0 / 12.0;
    case 5: return (x - 0.5) * (y - 0.5);
    case 6: return (y - 0.5) * ((x - 0.5) * (x - 0.5) - 1.0 / 12.0);
    case 7: return (x - 0.5) * ((y - 0.5) * (y - 0.5) - 1.0 / 12.0);
    }
    return 0.0;
}
// basisfunctions.py:54-92
static double dx_dgbasis(int j, double x, double y)
{
    switch (j) {
    case 0: return 0.;
    case 1: return 1.;
    case 2: return 0.;
    case 3: return 2.0 * (x - 0.5);
    case 4: return 0.;
    case 5: return (y - 0.5);
    case 6: return (y - 0.5) * (2. * (x - 0.5));
    case 7: return ((y - 0.5) * (y - 0.5) - 1.0 / 12.0);
    }
    return 0.0;
}
static double dy_dgbasis(int j, double x, double y)
{
    switch (j) {
    case 0: return 0.;
    case 1: return 0.;
    case 2: return 1.;
    case 3: return 0.;
    case 4: return 2. * (y - 0.5);
    case 5: return (x - 0.5);
    case 6: return ((x - 0.5) * (x - 0.5) - 1.0 / 12.0);
    case 7: return (x - 0.5) * (2. * (y - 0.5));
    }
    return 0.0;
}
// basisfunctions.py:97-106
static double dgbasis_edge(int j, double x)
{
    switch (j) {
    case 0: return 1.;
    case 1: return x - 0.5;
    case 2: return (x - 0.5) * (x - 0.5) - 1.0 / 12.0;
    }
    return 0.0;
}
// basisfunctions.py:113-160 (CGbasis1d, CGbasis1d_dX)
static double cgbasis1d(int cg, int j, double x)
{
    if (cg == 1)
        return j == 0 ? 1.0 - x : x;
    if (j == 0)
        return 2.0 * (x - 0.5) * (x - 1.0);
    if (j == 1)
        return 4.0 * x * (1.0 - x);
    return 2.0 * x * (x - 0.5);
}
static double cgbasis1d_dx(int cg, int j, double x)
{
    if (cg == 1)
        return j == 0 ? -1.0 : 1.0;
    if (j == 0)
        return 4.0 * x - 3.0;
    if (j == 1)
        return 4.0 - 8.0 * x;
    return 4.0 * x - 1.0;
}

static inline int gauss1d(int dg) { return (dg == 8 || dg == 6) ? 3 : (dg == 3 ? 2 : 1); }
static inline int edgedofs(int dg) { return dg == 1 ? 1 : (dg == 3 ? 2 : 3); }

// Table accessors (codeGenerationDGinGauss.py / codeGenerationCGinGauss.py).
// Gauss point q = gy * Q + gx (x fastest).
static inline double PSI(int j, int Q, int q) { return dgbasis(j, QUAD.p[Q][q % Q], QUAD.p[Q][q / Q]); }
static inline double PSIx(int j, int Q, int q) { return dx_dgbasis(j, QUAD.p[Q][q % Q], QUAD.p[Q][q / Q]); }
static inline double PSIy(int j, int Q, int q) { return dy_dgbasis(j, QUAD.p[Q][q % Q], QUAD.p[Q][q / Q]); }
static inline double GW(int Q, int q) { return QUAD.w[Q][q % Q] * QUAD.w[Q][q / Q]; }
static inline double PSIe(int j, int G, int g) { return dgbasis_edge(j, QUAD.p[G][g]); }
// PSIe_w<DG,G,E>(g, j): codeGenerationDGinGauss.py:42-70
static inline double PSIe_w(int j, int G, int E, int g)
{
    const double t = QUAD.p[G][g];
    double x = 0, y = 0;
    if (E == 0) { x = t; y = 0.0; }
    else if (E == 1) { x = 1.0; y = t; }
    else if (E == 2) { x = t; y = 1.0; }
    else { x = 0.0; y = t; }
    return QUAD.w[G][g] * dgbasis(j, x, y);
}
// PSILagrange<DG,G>: codeGenerationDGinGauss.py:106-121; lagrange points
// gaussquadrature.py:22-24
static inline double PSILagrange(int j, int G, int q)
{
    static const double lp2[2] = { 0.0, 1.0 };
    static const double lp3[3] = { 0.0, 0.5, 1.0 };
    const double* lp = (G == 2) ? lp2 : lp3;
    return dgbasis(j, lp[q % G], lp[q / G]);
}
static inline double PHI(int cg, int j, int Q, int q)
{
    return cgbasis1d(cg, j % (cg + 1), QUAD.p[Q][q % Q]) * cgbasis1d(cg, j / (cg + 1), QUAD.p[Q][q / Q]);
}
static inline double PHIx(int cg, int j, int Q, int q)
{
    return cgbasis1d_dx(cg, j % (cg + 1), QUAD.p[Q][q % Q]) * cgbasis1d(cg, j / (cg + 1), QUAD.p[Q][q / Q]);
}
static inline double PHIy(int cg, int j, int Q, int q)
{
    return cgbasis1d(cg, j % (cg + 1), QUAD.p[Q][q % Q]) * cgbasis1d_dx(cg, j / (cg + 1), QUAD.p[Q][q / Q]);
}

/* ------------------------------------------------------------------------ */
/* Small dense helpers                                                      */
/* ------------------------------------------------------------------------ */
// Gauss-Jordan inverse with partial pivoting (stands in for Eigen's .inverse()).
static bool invert(int n, const double* A, double* inv)
{
    double m[8][16];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < 2 * n; ++j)
            m[i][j] = (j < n) ? A[i * n + j] : (j - n == i ? 1.0 : 0.0);
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(m[r][c]) > std::fabs(m[piv][c]))
                piv = r;
        if (m[piv][c] == 0.0)
            return false;
        if (piv != c)
            for (int j = 0; j < 2 * n; ++j)
                std::swap(m[c][j], m[piv][j]);
        const double d = m[c][c];
        for (int j = 0; j < 2 * n; ++j)
            m[c][j] /= d;
        for (int r = 0; r < n; ++r) {
            if (r == c)
                continue;
            const double f = m[r][c];
            if (f == 0.0)
                continue;
            for (int j = 0; j < 2 * n; ++j)
                m[r][j] -= f * m[c][j];
        }
    }
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            inv[i * n + j] = m[i][j + n];
    return true;
}

/* ------------------------------------------------------------------------ */
/* ParametricMesh (dynamics/src/include/ParametricMesh.hpp:42-442)          */
/* ------------------------------------------------------------------------ */
// NextsimDynamics.hpp:34
static constexpr double kEarthRadius = 6371000.0;

struct Mesh {
    bool spherical = false; // COORDINATES: SPHERICAL (x = lon, y = lat, radians) or CARTESIAN
    size_t nx = 0, ny = 0, nnodes = 0, nelements = 0;
    std::vector<double> vx, vy; // vertices
    std::vector<char> landmask; // 1 = ice
    std::array<std::vector<size_t>, 4> dirichlet;
    std::vector<std::vector<std::array<size_t, 4>>> periodic;

    // ParametricMesh.hpp:196-209: no longitude jump (Pi -> -Pi) inside one element
    static void correctLongitude(double c[][2], int n)
    {
        bool problem = false;
        for (int i = 1; i < n; ++i)
            if (std::fabs(c[0][0] - c[i][0]) > 2.0 / 3.0 * M_PI) {
                problem = true;
                break;
            }
        if (problem)
            for (int i = 0; i < n; ++i)
                if (c[i][0] < 0)
                    c[i][0] += 2.0 * M_PI;
    }
    // ParametricMesh.hpp:218-232
    void coordinatesOfElement(size_t eid, double c[4][2]) const
    {
        const size_t nid = (eid / nx) * (nx + 1) + (eid % nx);
        const size_t ids[4] = { nid, nid + 1, nid + nx + 1, nid + nx + 2 };
        for (int k = 0; k < 4; ++k) {
            c[k][0] = vx[ids[k]];
            c[k][1] = vy[ids[k]];
        }
        if (spherical)
            correctLongitude(c, 4);
    }
    // ParametricMesh.hpp:137-157: the poles moved to Greenland / Antarctica
    void rotatePoleToGreenland()
    {
        for (size_t i = 0; i < nnodes; ++i) {
            const double x = std::cos(vy[i]) * std::cos(vx[i]);
            const double y = std::cos(vy[i]) * std::sin(vx[i]);
            const double z = std::sin(vy[i]);
            const double aw = 40.0 * M_PI / 180.0;
            const double x1 = std::cos(aw) * x - std::sin(aw) * y;
            const double y1 = std::sin(aw) * x + std::cos(aw) * y;
            const double z1 = z;
            const double bw = 15.0 * M_PI / 180.0;
            const double x2 = std::cos(bw) * x1 - std::sin(bw) * z1;
            const double y2 = y1;
            const double z2 = std::sin(bw) * x1 + std::cos(bw) * z1;
            vy[i] = std::asin(z2);
            vx[i] = std::atan2(y2, x2);
        }
    }
    // ParametricMesh.hpp:276-299
    double area(size_t eid) const
    {
        const size_t nid = (eid / nx) * (nx + 1) + (eid % nx);
        auto sq = [&](size_t a, size_t b) {
            const double dx = vx[a] - vx[b], dy = vy[a] - vy[b];
            return dx * dx + dy * dy;
        };
        const double a = sq(nid, nid + 1);
        const double b = sq(nid + 1, nid + nx + 2);
        const double c = sq(nid + 1 + nx, nid + 2 + nx);
        const double d = sq(nid, nid + nx + 1);
        const double e = sq(nid, nid + nx + 2);
        const double f = sq(nid + 1, nid + nx + 1);
        const double t = b + d - a - c;
        return 0.25 * std::sqrt(4.0 * e * f - t * t);
    }
    double h(size_t eid) const { return std::sqrt(area(eid)); }
    // ParametricMesh.hpp:381-397
    void edgevector(size_t n1, size_t n2, double t[2]) const
    {
        t[0] = vx[n2] - vx[n1];
        t[1] = vy[n2] - vy[n1];
        if (spherical) {
            if (t[0] > 0.5 * M_PI)
                t[0] -= 2.0 * M_PI;
            if (t[0] < -0.5 * M_PI)
                t[0] += 2.0 * M_PI;
        }
    }
    void sortDirichlet(int edge) { std::sort(dirichlet[edge].begin(), dirichlet[edge].end()); }
    // ParametricMesh.cpp:228-252
    void dirichletFromMask()
    {
        const size_t startX[4] = { 0, 0, 0, 1 };
        const size_t stopX[4] = { nx, nx - 1, nx, nx };
        const size_t startY[4] = { 1, 0, 0, 0 };
        const size_t stopY[4] = { ny, ny, ny - 1, ny };
        const long deltaIdx[4] = { -static_cast<long>(nx), 1, static_cast<long>(nx), -1 };
        for (int edge = 0; edge < 4; ++edge) {
            for (size_t j = startY[edge]; j < stopY[edge]; ++j)
                for (size_t i = startX[edge]; i < stopX[edge]; ++i) {
                    const size_t idx = i + nx * j;
                    if (!landmask[idx])
                        continue;
                    if (!landmask[idx + deltaIdx[edge]])
                        dirichlet[edge].push_back(idx);
                }
            sortDirichlet(edge);
        }
    }
    // ParametricMesh.cpp:259-272
    void dirichletFromEdge(int edge)
    {
        const size_t start[4] = { 0, nx - 1, nelements - nx, 0 };
        const size_t stop[4] = { nx, nelements, nelements, nelements };
        const size_t stride[4] = { 1, nx, 1, nx };
        for (size_t idx = start[edge]; idx < stop[edge]; idx += stride[edge])
            if (landmask[idx])
                dirichlet[edge].push_back(idx);
        sortDirichlet(edge);
    }
};

/* ParametricTools (ParametricTools.hpp:73-181) */
// dxT<Q> = coords^T * PHIx<1,Q>; dyT<Q> = coords^T * PHIy<1,Q>
static void dxdyT(const Mesh& m, size_t eid, int Q, double dxT[2][16], double dyT[2][16])
{
    double c[4][2];
    m.coordinatesOfElement(eid, c);
    for (int r = 0; r < 2; ++r)
        for (int q = 0; q < Q * Q; ++q) {
            double sx = 0, sy = 0;
            for (int k = 0; k < 4; ++k) {
                sx += c[k][r] * PHIx(1, k, Q, q);
                sy += c[k][r] * PHIy(1, k, Q, q);
            }
            dxT[r][q] = sx;
            dyT[r][q] = sy;
        }
}
// ParametricTools.hpp:92-105
static void jacobian(const Mesh& m, size_t eid, int Q, double* J)
{
    double dxT[2][16], dyT[2][16];
    dxdyT(m, eid, Q, dxT, dyT);
    for (int q = 0; q < Q * Q; ++q)
        J[q] = dxT[0][q] * dyT[1][q] - dxT[1][q] * dyT[0][q];
}
// ParametricTools.hpp:159-164
static void gaussPointsInElement(const Mesh& m, size_t eid, int Q, double gp[2][16])
{
    double c[4][2];
    m.coordinatesOfElement(eid, c);
    for (int r = 0; r < 2; ++r)
        for (int q = 0; q < Q * Q; ++q) {
            double s = 0;
            for (int k = 0; k < 4; ++k)
                s += c[k][r] * PHI(1, k, Q, q);
            gp[r][q] = s;
        }
}
// cos / sin of the latitude at the Q x Q Gauss points of an element
static void latTrig(const Mesh& m, size_t eid, int Q, double* cl, double* sl)
{
    double gp[2][16];
    gaussPointsInElement(m, eid, Q, gp);
    for (int q = 0; q < Q * Q; ++q) {
        if (cl) cl[q] = std::cos(gp[1][q]);
        if (sl) sl[q] = std::sin(gp[1][q]);
    }
}
// ParametricTools.hpp:109-153: M_ij = sum_q PSI_iq (w_q J_q) PSI_jq;
// SphericalTools::massMatrix (ParametricTools.hpp:189-202) adds cos(lat_q)
static void massMatrix(const Mesh& m, size_t eid, int DG, double* M)
{
    const int Q = gauss1d(DG);
    double J[16], cl[16];
    jacobian(m, eid, Q, J);
    if (m.spherical)
        latTrig(m, eid, Q, cl, nullptr);
    for (int i = 0; i < DG; ++i)
        for (int j = 0; j < DG; ++j) {
            double s = 0;
            for (int q = 0; q < Q * Q; ++q)
                s += m.spherical ? (PSI(i, Q, q) * (GW(Q, q) * J[q] * cl[q])) * PSI(j, Q, q)
                                 : (PSI(i, Q, q) * (GW(Q, q) * J[q])) * PSI(j, Q, q);
            M[i * DG + j] = s;
        }
}
static void inverseMass(const Mesh& m, size_t eid, int DG, double* Minv)
{
    double M[64];
    massMatrix(m, eid, DG, M);
    invert(DG, M, Minv);
}

/* ------------------------------------------------------------------------ */
/* DG vectors: element-major, component fastest (dgVector.hpp:89-130)      */
/* ------------------------------------------------------------------------ */
struct DG {
    int n = 0;
    std::vector<double> a;
    DG() = default;
    DG(size_t N, int comps) : n(comps), a(N * comps, 0.0) { }
    void resize(size_t N, int comps) { n = comps; a.assign(N * comps, 0.0); }
    double* row(size_t e) { return a.data() + e * n; }
    const double* row(size_t e) const { return a.data() + e * n; }
    void zero() { std::fill(a.begin(), a.end(), 0.0); }
};

/* ------------------------------------------------------------------------ */
/* DG transport (DGTransport.cpp, ParametricMap.cpp:13-87)                  */
/* ------------------------------------------------------------------------ */
// edge traces (DGTransport.cpp:31-142)
static void leftEdge(int dg, const double* c, double* o)
{
    if (dg == 1) { o[0] = c[0]; }
    else if (dg == 3) { o[0] = c[0] - 0.5 * c[1]; o[1] = c[2]; }
    else if (dg == 6) { o[0] = c[0] - 0.5 * c[1] + 1. / 6. * c[3]; o[1] = c[2] - 0.5 * c[5]; o[2] = c[4]; }
    else { o[0] = c[0] - 0.5 * c[1] + 1. / 6. * c[3]; o[1] = c[2] - 0.5 * c[5] + 1. / 6. * c[6]; o[2] = c[4] - 0.5 * c[7]; }
}
static void rightEdge(int dg, const double* c, double* o)
{
    if (dg == 1) { o[0] = c[0]; }
    else if (dg == 3) { o[0] = c[0] + 0.5 * c[1]; o[1] = c[2]; }
    else if (dg == 6) { o[0] = c[0] + 0.5 * c[1] + 1. / 6. * c[3]; o[1] = c[2] + 0.5 * c[5]; o[2] = c[4]; }
    else { o[0] = c[0] + 0.5 * c[1] + 1. / 6. * c[3]; o[1] = c[2] + 0.5 * c[5] + 1. / 6. * c[6]; o[2] = c[4] + 0.5 * c[7]; }
}
static void bottomEdge(int dg, const double* c, double* o)
{
    if (dg == 1) { o[0] = c[0]; }
    else if (dg == 3) { o[0] = c[0] - 0.5 * c[2]; o[1] = c[1]; }
    else if (dg == 6) { o[0] = c[0] - 0.5 * c[2] + 1. / 6. * c[4]; o[1] = c[1] - 0.5 * c[5]; o[2] = c[3]; }
    else { o[0] = c[0] - 0.5 * c[2] + 1. / 6. * c[4]; o[1] = c[1] - 0.5 * c[5] + 1. / 6. * c[7]; o[2] = c[3] - 0.5 * c[6]; }
}
static void topEdge(int dg, const double* c, double* o)
{
    if (dg == 1) { o[0] = c[0]; }
    else if (dg == 3) { o[0] = c[0] + 0.5 * c[2]; o[1] = c[1]; }
    else if (dg == 6) { o[0] = c[0] + 0.5 * c[2] + 1. / 6. * c[4]; o[1] = c[1] + 0.5 * c[5]; o[2] = c[3]; }
    else { o[0] = c[0] + 0.5 * c[2] + 1. / 6. * c[4]; o[1] = c[1] + 0.5 * c[5] + 1. / 6. * c[7]; o[2] = c[3] + 0.5 * c[6]; }
}

struct Transport {
    const Mesh* mesh = nullptr;
    int dg = 0, ed = 0, Q = 0;
    std::string scheme = "rk2";
    std::vector<double> cellX, cellY; // N x (dg*QQ)   AdvectionCellTermX/Y
    std::vector<double> minv;          // N x dg*dg     InverseDGMassMatrix
    DG velx, vely;
    std::vector<double> nvX, nvY;      // edges x ed
    DG tmp1, tmp2, tmp3;

    // DGTransport.hpp:71-96 and ParametricMap.cpp:13-87
    void init(const Mesh& m, int DGc)
    {
        mesh = &m;
        dg = DGc;
        ed = edgedofs(dg);
        Q = gauss1d(dg);
        const int QQ = Q * Q;
        const size_t N = m.nelements;
        velx.resize(N, dg);
        vely.resize(N, dg);
        tmp1.resize(N, dg);
        tmp2.resize(N, dg);
        tmp3.resize(N, dg);
        nvX.assign(m.nx * (m.ny + 1) * ed, 0.0);
        nvY.assign((m.nx + 1) * m.ny * ed, 0.0);
        cellX.assign(N * dg * QQ, 0.0);
        cellY.assign(N * dg * QQ, 0.0);
        minv.assign(N * dg * dg, 0.0);
#pragma omp parallel for schedule(static)
        for (long e = 0; e < static_cast<long>(N); ++e) {
            double dxT[2][16], dyT[2][16];
            dxdyT(m, e, Q, dxT, dyT);
            for (int r = 0; r < 2; ++r)
                for (int q = 0; q < QQ; ++q) {
                    dxT[r][q] = dxT[r][q] * GW(Q, q);
                    dyT[r][q] = dyT[r][q] * GW(Q, q);
                }
            for (int i = 0; i < dg; ++i)
                for (int q = 0; q < QQ; ++q) {
                    cellX[(e * dg + i) * QQ + q] = PSIx(i, Q, q) * dyT[1][q] - PSIy(i, Q, q) * dxT[1][q];
                    cellY[(e * dg + i) * QQ + q] = PSIy(i, Q, q) * dxT[0][q] - PSIx(i, Q, q) * dyT[0][q];
                }
            inverseMass(m, e, dg, &minv[e * dg * dg]);
            if (m.spherical) // ParametricMap.cpp:74-79
                for (int k = 0; k < dg * dg; ++k)
                    minv[e * dg * dg + k] /= kEarthRadius;
        }
    }

    // DGTransport.cpp:158-252
    void reinitnormalvelocity()
    {
        const Mesh& m = *mesh;
        std::fill(nvX.begin(), nvX.end(), 0.0);
        std::fill(nvY.begin(), nvY.end(), 0.0);
        double tr[3], tv[3];
#pragma omp parallel for private(tr, tv) schedule(static)
        for (long iy = 0; iy < static_cast<long>(m.ny); ++iy) {
            size_t ey = iy * (m.nx + 1);
            size_t cy = iy * m.nx;
            for (size_t ix = 0; ix < m.nx; ++ix, ++ey, ++cy) {
                if (!m.landmask[cy])
                    continue;
                double t[2];
                m.edgevector(ey, ey + m.nx + 1, t);
                leftEdge(dg, velx.row(cy), tr);
                leftEdge(dg, vely.row(cy), tv);
                for (int k = 0; k < ed; ++k)
                    nvY[ey * ed + k] += 0.5 * (t[1] * tr[k] - t[0] * tv[k]);
                m.edgevector(ey + 1, ey + m.nx + 2, t);
                rightEdge(dg, velx.row(cy), tr);
                rightEdge(dg, vely.row(cy), tv);
                for (int k = 0; k < ed; ++k)
                    nvY[(ey + 1) * ed + k] += 0.5 * (t[1] * tr[k] - t[0] * tv[k]);
            }
        }
#pragma omp parallel for private(tr, tv) schedule(static)
        for (long ix = 0; ix < static_cast<long>(m.nx); ++ix) {
            size_t cx = ix, nxi = ix;
            for (size_t iy = 0; iy < m.ny; ++iy, cx += m.nx, nxi += m.nx + 1) {
                if (!m.landmask[cx])
                    continue;
                double t[2];
                m.edgevector(nxi, nxi + 1, t);
                bottomEdge(dg, velx.row(cx), tr);
                bottomEdge(dg, vely.row(cx), tv);
                for (int k = 0; k < ed; ++k)
                    nvX[cx * ed + k] += 0.5 * (-t[1] * tr[k] + t[0] * tv[k]);
                m.edgevector(nxi + m.nx + 1, nxi + m.nx + 2, t);
                topEdge(dg, velx.row(cx), tr);
                topEdge(dg, vely.row(cx), tv);
                for (int k = 0; k < ed; ++k)
                    nvX[(cx + m.nx) * ed + k] += 0.5 * (-t[1] * tr[k] + t[0] * tv[k]);
            }
        }
        for (int seg = 0; seg < 4; ++seg)
            for (size_t i = 0; i < m.dirichlet[seg].size(); ++i) {
                const size_t eid = m.dirichlet[seg][i];
                const size_t ix = eid % m.nx, iy = eid / m.nx;
                double* row = nullptr;
                if (seg == 0) row = &nvX[(m.nx * iy + ix) * ed];
                else if (seg == 1) row = &nvY[((m.nx + 1) * iy + ix + 1) * ed];
                else if (seg == 2) row = &nvX[(m.nx * (iy + 1) + ix) * ed];
                else row = &nvY[((m.nx + 1) * iy + ix) * ed];
                for (int k = 0; k < ed; ++k)
                    row[k] *= 2.0;
            }
    }

    // DGTransport.cpp:278-303
    void cell_term(double dt, DG& phiup, const DG& phi, size_t eid) const
    {
        if (dg == 1 || !mesh->landmask[eid])
            return;
        const int QQ = Q * Q;
        double vxg[9], vyg[9], pg[9];
        for (int q = 0; q < QQ; ++q) {
            double a = 0, b = 0, c = 0;
            for (int j = 0; j < dg; ++j) {
                a += velx.row(eid)[j] * PSI(j, Q, q);
                b += vely.row(eid)[j] * PSI(j, Q, q);
                c += phi.row(eid)[j] * PSI(j, Q, q);
            }
            vxg[q] = a;
            vyg[q] = b;
            pg[q] = c;
        }
        const double* cx = &cellX[eid * dg * QQ];
        const double* cy = &cellY[eid * dg * QQ];
        for (int i = 0; i < dg; ++i) {
            double s = 0;
            for (int q = 0; q < QQ; ++q)
                s += (cx[i * QQ + q] * vxg[q] + cy[i * QQ + q] * vyg[q]) * pg[q];
            phiup.row(eid)[i] += dt * s;
        }
    }
    // vel_gauss = nv.row(e) * PSIe<ed, ed>
    void velGauss(const double* nv, double* vg) const
    {
        for (int g = 0; g < ed; ++g) {
            double s = 0;
            for (int j = 0; j < ed; ++j)
                s += nv[j] * PSIe(j, ed, g);
            vg[g] = s;
        }
    }
    void traceGauss(const double* tr, double* tg) const { velGauss(tr, tg); }
    // phiup.row(c) += sign * dt * tmp * PSIe_w<dg, ed, E>
    void addEdge(DG& phiup, size_t c, double sdt, const double* tmp, int E) const
    {
        for (int j = 0; j < dg; ++j) {
            double s = 0;
            for (int g = 0; g < ed; ++g)
                s += tmp[g] * PSIe_w(j, ed, E, g);
            phiup.row(c)[j] += sdt * s;
        }
    }
    // DGTransport.cpp:306-351
    void boundary(int seg, double dt, DG& phiup, const DG& phi, size_t c, size_t e) const
    {
        const std::vector<double>& nv = (seg == 0 || seg == 2) ? nvX : nvY;
        double vg[3], tr[3], tg[3], tmp[3];
        velGauss(&nv[e * ed], vg);
        if (seg == 0) bottomEdge(dg, phi.row(c), tr);
        else if (seg == 1) rightEdge(dg, phi.row(c), tr);
        else if (seg == 2) topEdge(dg, phi.row(c), tr);
        else leftEdge(dg, phi.row(c), tr);
        traceGauss(tr, tg);
        for (int g = 0; g < ed; ++g) {
            const double v = (seg == 0 || seg == 3) ? std::max(-vg[g], 0.0) : std::max(vg[g], 0.0);
            tmp[g] = tg[g] * v;
        }
        const int E = (seg == 0) ? 0 : (seg == 1) ? 1 : (seg == 2) ? 2 : 3;
        addEdge(phiup, c, -dt, tmp, E);
    }
    // DGTransport.cpp:355-433
    void edge_term_X(double dt, DG& phiup, const DG& phi, size_t c1, size_t c2, size_t ie) const
    {
        if (!mesh->landmask[c1] || !mesh->landmask[c2])
            return;
        if (dg == 1) {
            const double bottom = phi.row(c1)[0], top = phi.row(c2)[0], vel = nvX[ie];
            const double f = std::max(vel, 0.) * bottom + std::min(vel, 0.) * top;
            phiup.row(c1)[0] -= dt * f;
            phiup.row(c2)[0] += dt * f;
            return;
        }
        double vg[3], t1[3], t2[3], g1[3], g2[3], tmp[3];
        velGauss(&nvX[ie * ed], vg);
        topEdge(dg, phi.row(c1), t1);
        bottomEdge(dg, phi.row(c2), t2);
        traceGauss(t1, g1);
        traceGauss(t2, g2);
        for (int g = 0; g < ed; ++g)
            tmp[g] = std::max(vg[g], 0.0) * g1[g] + std::min(vg[g], 0.0) * g2[g];
        addEdge(phiup, c1, -dt, tmp, 2);
        addEdge(phiup, c2, dt, tmp, 0);
    }
    void edge_term_Y(double dt, DG& phiup, const DG& phi, size_t c1, size_t c2, size_t ie) const
    {
        if (!mesh->landmask[c1] || !mesh->landmask[c2])
            return;
        if (dg == 1) {
            const double left = phi.row(c1)[0], right = phi.row(c2)[0], vel = nvY[ie];
            const double f = std::max(vel, 0.) * left + std::min(vel, 0.) * right;
            phiup.row(c1)[0] -= dt * f;
            phiup.row(c2)[0] += dt * f;
            return;
        }
        double vg[3], t1[3], t2[3], g1[3], g2[3], tmp[3];
        velGauss(&nvY[ie * ed], vg);
        rightEdge(dg, phi.row(c1), t1);
        leftEdge(dg, phi.row(c2), t2);
        traceGauss(t1, g1);
        traceGauss(t2, g2);
        for (int g = 0; g < ed; ++g)
            tmp[g] = std::max(vg[g], 0.0) * g1[g] + std::min(vg[g], 0.0) * g2[g];
        addEdge(phiup, c1, -dt, tmp, 1);
        addEdge(phiup, c2, dt, tmp, 3);
    }
    // DGTransport.cpp:435-512
    void operatorF(double dt, const DG& phi, DG& phiup) const
    {
        const Mesh& m = *mesh;
        phiup.zero();
#pragma omp parallel for schedule(static)
        for (long e = 0; e < static_cast<long>(m.nelements); ++e)
            cell_term(dt, phiup, phi, e);
#pragma omp parallel for schedule(static)
        for (long iy = 0; iy < static_cast<long>(m.ny); ++iy) {
            size_t ic = iy * m.nx, ie = iy * (m.nx + 1) + 1;
            for (size_t i = 0; i + 1 < m.nx; ++i, ++ic, ++ie)
                edge_term_Y(dt, phiup, phi, ic, ic + 1, ie);
        }
#pragma omp parallel for schedule(static)
        for (long ix = 0; ix < static_cast<long>(m.nx); ++ix) {
            size_t ic = ix, ie = ix + m.nx;
            for (size_t i = 0; i + 1 < m.ny; ++i, ic += m.nx, ie += m.nx)
                edge_term_X(dt, phiup, phi, ic, ic + m.nx, ie);
        }
        for (size_t pc = 0; pc < m.periodic.size(); ++pc)
            for (size_t i = 0; i < m.periodic[pc].size(); ++i) {
                const auto& p = m.periodic[pc][i];
                if (p[0] == 0)
                    edge_term_X(dt, phiup, phi, p[1], p[2], p[3]);
                else
                    edge_term_Y(dt, phiup, phi, p[1], p[2], p[3]);
            }
        for (int seg = 0; seg < 4; ++seg)
            for (size_t i = 0; i < m.dirichlet[seg].size(); ++i) {
                const size_t eid = m.dirichlet[seg][i];
                const size_t ix = eid % m.nx, iy = eid / m.nx;
                size_t e = 0;
                if (seg == 0) e = m.nx * iy + ix;
                else if (seg == 1) e = (m.nx + 1) * iy + ix + 1;
                else if (seg == 2) e = m.nx * (iy + 1) + ix;
                else e = (m.nx + 1) * iy + ix;
                boundary(seg, dt, phiup, phi, eid, e);
            }
#pragma omp parallel for schedule(static)
        for (long e = 0; e < static_cast<long>(m.nelements); ++e) {
            double r[8];
            const double* M = &minv[e * dg * dg];
            for (int i = 0; i < dg; ++i) {
                double s = 0;
                for (int j = 0; j < dg; ++j)
                    s += M[i * dg + j] * phiup.row(e)[j];
                r[i] = s;
            }
            for (int i = 0; i < dg; ++i)
                phiup.row(e)[i] = r[i];
        }
    }
    // DGTransport.cpp:514-566
    void step(double dt, DG& phi)
    {
        const size_t n = phi.a.size();
        if (scheme == "rk1") {
            operatorF(dt, phi, tmp1);
            for (size_t i = 0; i < n; ++i) phi.a[i] += tmp1.a[i];
        } else if (scheme == "rk2") {
            operatorF(dt, phi, tmp1);
            for (size_t i = 0; i < n; ++i) phi.a[i] += tmp1.a[i];
            operatorF(dt, phi, tmp2);
            for (size_t i = 0; i < n; ++i) phi.a[i] += 0.5 * (tmp2.a[i] - tmp1.a[i]);
        } else {
            operatorF(dt, phi, tmp1);
            for (size_t i = 0; i < n; ++i) tmp1.a[i] += phi.a[i];
            operatorF(dt, tmp1, tmp2);
            for (size_t i = 0; i < n; ++i) {
                tmp2.a[i] += tmp1.a[i];
                tmp2.a[i] *= 0.25;
                tmp2.a[i] += 0.75 * phi.a[i];
            }
            operatorF(dt, tmp2, tmp3);
            for (size_t i = 0; i < n; ++i) {
                tmp3.a[i] += tmp2.a[i];
                phi.a[i] *= 1.0 / 3.0;
                phi.a[i] += 2.0 / 3.0 * tmp3.a[i];
            }
        }
    }
};

/* ------------------------------------------------------------------------ */
/* Limiters (dgLimit.hpp:16-85)                                             */
/* ------------------------------------------------------------------------ */
static void LimitMax(DG& d, double max)
{
    const size_t N = d.a.size() / d.n;
    if (d.n == 1) {
        for (size_t i = 0; i < N; ++i) d.a[i] = std::min(d.a[i], max);
    } else if (d.n == 3) {
        for (size_t i = 0; i < N; ++i) {
            double* r = d.row(i);
            r[0] = std::min(max, r[0]);
            const double l0 = 2.0 * std::max(std::fabs(r[1] + r[2]), std::fabs(r[1] - r[2]));
            if (l0 == 0) continue;
            const double ex = r[0] + l0 - max;
            if (ex > 0) {
                r[1] *= (max - r[0]) / l0;
                r[2] *= (max - r[0]) / l0;
            }
        }
    } else if (d.n == 6) {
        for (size_t i = 0; i < N; ++i) {
            double* r = d.row(i);
            r[0] = std::min(max, r[0]);
            double mv = -1e300;
            for (int q = 0; q < 9; ++q) {
                double s = 0;
                for (int j = 0; j < 6; ++j) s += r[j] * PSI(j, 3, q);
                mv = std::max(mv, s);
            }
            const double l0 = mv - r[0];
            if (mv > max) {
                const double f = (max - r[0]) / l0;
                for (int j = 1; j < 6; ++j) r[j] *= f;
            }
        }
    }
}
static void LimitMin(DG& d, double min)
{
    const size_t N = d.a.size() / d.n;
    if (d.n == 1) {
        for (size_t i = 0; i < N; ++i) d.a[i] = std::max(d.a[i], min);
    } else if (d.n == 3) {
        for (size_t i = 0; i < N; ++i) {
            double* r = d.row(i);
            r[0] = std::max(min, r[0]);
            const double l0 = 2.0 * std::max(std::fabs(r[1] + r[2]), std::fabs(r[1] - r[2]));
            if (l0 == 0) continue;
            const double ex = r[0] - l0 - min;
            if (ex < 0) {
                r[1] *= (r[0] - min) / l0;
                r[2] *= (r[0] - min) / l0;
            }
        }
    } else if (d.n == 6) {
        for (size_t i = 0; i < N; ++i) {
            double* r = d.row(i);
            r[0] = std::max(min, r[0]);
            double mv = 1e300;
            for (int q = 0; q < 9; ++q) {
                double s = 0;
                for (int j = 0; j < 6; ++j) s += r[j] * PSI(j, 3, q);
                mv = std::min(mv, s);
            }
            const double l0 = mv - r[0];
            if (mv < min) {
                const double f = (r[0] - min) / l0;
                for (int j = 1; j < 6; ++j) r[j] *= f;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* Interpolations (dynamics/src/Interpolations.cpp)                         */
/* ------------------------------------------------------------------------ */
typedef double (*Function)(double, double, const double*);

// Interpolations.cpp:29-72 (Cartesian)
static void Function2DG(const Mesh& m, DG& phi, Function f, const double* fp)
{
    const int dg = phi.n, Q = gauss1d(dg), QQ = Q * Q;
    phi.zero();
    for (size_t e = 0; e < m.nelements; ++e) {
        if (!m.landmask[e]) continue;
        double gp[2][16], J[16], fg[16], Minv[64], r[8];
        gaussPointsInElement(m, e, Q, gp);
        for (int q = 0; q < QQ; ++q) fg[q] = f(gp[0][q], gp[1][q], fp);
        jacobian(m, e, Q, J);
        inverseMass(m, e, dg, Minv);
        for (int i = 0; i < dg; ++i) {
            double s = 0;
            for (int q = 0; q < QQ; ++q)
                s += m.spherical ? (PSI(i, Q, q) * (J[q] * GW(Q, q) * std::cos(gp[1][q]))) * fg[q]
                                 : (PSI(i, Q, q) * (J[q] * GW(Q, q))) * fg[q];
            r[i] = s;
        }
        for (int i = 0; i < dg; ++i) {
            double s = 0;
            for (int j = 0; j < dg; ++j) s += Minv[i * dg + j] * r[j];
            phi.row(e)[i] = s;
        }
    }
}
// Interpolations.cpp:206-247 (Cartesian)
static double L2ErrorFunctionDG(const Mesh& m, const DG& src, Function f, const double* fp)
{
    const int dg = src.n, Q = gauss1d(dg), QQ = Q * Q;
    double err = 0;
    for (size_t e = 0; e < m.nelements; ++e) {
        if (!m.landmask[e]) continue;
        double gp[2][16], J[16];
        gaussPointsInElement(m, e, Q, gp);
        jacobian(m, e, Q, J);
        double s = 0;
        for (int q = 0; q < QQ; ++q) {
            double v = 0;
            for (int j = 0; j < dg; ++j) v += src.row(e)[j] * PSI(j, Q, q);
            const double d = v - f(gp[0][q], gp[1][q], fp);
            s += m.spherical ? std::cos(gp[1][q]) * J[q] * GW(Q, q) * (d * d) : J[q] * GW(Q, q) * (d * d);
        }
        err += s;
    }
    return err;
}
// Tools.hpp:24-50 (Cartesian, NGP = 3)
static double MeanValue(const Mesh& m, const DG& phi)
{
    double mass = 0;
    for (size_t e = 0; e < m.nelements; ++e) {
        double J[16], cl[16];
        jacobian(m, e, 3, J);
        if (m.spherical)
            latTrig(m, e, 3, cl, nullptr);
        double s = 0;
        for (int q = 0; q < 9; ++q) {
            double v = 0;
            for (int j = 0; j < phi.n; ++j) v += phi.row(e)[j] * PSI(j, 3, q);
            s += m.spherical ? v * cl[q] * (J[q] * GW(3, q)) : v * (J[q] * GW(3, q));
        }
        mass += s;
    }
    return mass;
}

struct CG2DGOp {
    // per element: inverse DG mass (dg x dg) and J*w at the DG Gauss points
    int dg = 0, Q = 0;
    std::vector<double> minv, jw;
    void init(const Mesh& m, int DGc)
    {
        dg = DGc;
        Q = gauss1d(dg);
        const int QQ = Q * Q;
        minv.assign(m.nelements * dg * dg, 0.0);
        jw.assign(m.nelements * QQ, 0.0);
#pragma omp parallel for schedule(static)
        for (long e = 0; e < static_cast<long>(m.nelements); ++e) {
            double J[16], cl[16];
            jacobian(m, e, Q, J);
            if (m.spherical)
                latTrig(m, e, Q, cl, nullptr);
            for (int q = 0; q < QQ; ++q)
                jw[e * QQ + q] = m.spherical ? J[q] * GW(Q, q) * cl[q] : J[q] * GW(Q, q);
            inverseMass(m, e, dg, &minv[e * dg * dg]);
        }
    }
    // Interpolations.cpp:74-122 (CG = 2, Cartesian)
    void apply(const Mesh& m, DG& out, const std::vector<double>& cg) const
    {
        const int QQ = Q * Q;
        const size_t s = 2 * m.nx + 1;
#pragma omp parallel for schedule(static)
        for (long e = 0; e < static_cast<long>(m.nelements); ++e) {
            const size_t iy = e / m.nx, ix = e % m.nx;
            const size_t cgi = 2 * s * iy + 2 * ix;
            double loc[9];
            for (int j = 0; j < 9; ++j) loc[j] = cg[cgi + (j % 3) + (j / 3) * s];
            double t[9], r[8];
            for (int q = 0; q < QQ; ++q) {
                double v = 0;
                for (int j = 0; j < 9; ++j) v += PHI(2, j, Q, q) * loc[j];
                t[q] = jw[e * QQ + q] * v;
            }
            for (int i = 0; i < dg; ++i) {
                double a = 0;
                for (int q = 0; q < QQ; ++q) a += PSI(i, Q, q) * t[q];
                r[i] = a;
            }
            const double* M = &minv[e * dg * dg];
            for (int i = 0; i < dg; ++i) {
                double a = 0;
                for (int j = 0; j < dg; ++j) a += M[i * dg + j] * r[j];
                out.row(e)[i] = a;
            }
        }
    }
};

// Interpolations.cpp:144-204 (CG = 2): stripes with reversed parity, then
// boundary doubling
static void DG2CG2(const Mesh& m, std::vector<double>& dest, const DG& src)
{
    const size_t s = 2 * m.nx + 1;
    std::fill(dest.begin(), dest.end(), 0.0);
    static const double wts[9] = { 0.25, 0.5, 0.25, 0.5, 1.0, 0.5, 0.25, 0.5, 0.25 };
    for (size_t p = 0; p < 2; ++p) {
#pragma omp parallel for schedule(static)
        for (long cy = 0; cy < static_cast<long>(m.ny); ++cy) {
            if (static_cast<size_t>(cy) % 2 == p) continue;
            size_t c = cy * m.nx;
            for (size_t cx = 0; cx < m.nx; ++cx, ++c) {
                const size_t cgi = 2 * s * cy + 2 * cx;
                for (int q = 0; q < 9; ++q) {
                    double at = 0;
                    for (int j = 0; j < src.n; ++j) at += src.row(c)[j] * PSILagrange(j, 3, q);
                    const size_t node = cgi + (q % 3) + (q / 3) * s;
                    if (q == 4) dest[node] += at;
                    else dest[node] += wts[q] * at;
                }
            }
        }
    }
    const size_t UL = 2 * s * m.ny;
    for (size_t i = 0; i < 2 * m.nx + 1; ++i) {
        dest[i] *= 2.0;
        dest[UL + i] *= 2.0;
    }
    for (size_t i = 0; i < 2 * m.ny + 1; ++i) {
        dest[i * s] *= 2.0;
        dest[i * s + 2 * m.nx] *= 2.0;
    }
}
// Interpolations.cpp:129-143, 165-204 (CG = 1, DG0 input)
static void DG2CG1(const Mesh& m, std::vector<double>& dest, const DG& src)
{
    const size_t s = m.nx + 1;
    std::fill(dest.begin(), dest.end(), 0.0);
    for (size_t p = 0; p < 2; ++p)
        for (size_t cy = 0; cy < m.ny; ++cy) {
            if (cy % 2 == p) continue;
            size_t c = cy * m.nx;
            for (size_t cx = 0; cx < m.nx; ++cx, ++c) {
                const size_t cgi = s * cy + cx;
                double at[4];
                for (int q = 0; q < 4; ++q) {
                    double a = 0;
                    for (int j = 0; j < src.n; ++j) a += src.row(c)[j] * PSILagrange(j, 2, q);
                    at[q] = a;
                }
                dest[cgi] += 0.25 * at[0];
                dest[cgi + 1] += 0.25 * at[1];
                dest[cgi + s] += 0.25 * at[2];
                dest[cgi + s + 1] += 0.25 * at[3];
            }
        }
    const size_t UL = s * m.ny;
    for (size_t i = 0; i < m.nx + 1; ++i) {
        dest[i] *= 2.0;
        dest[UL + i] *= 2.0;
    }
    for (size_t i = 0; i < m.ny + 1; ++i) {
        dest[i * s] *= 2.0;
        dest[i * s + m.nx] *= 2.0;
    }
}

/* ------------------------------------------------------------------------ */
/* ParametricMomentumMap (ParametricMap.cpp:94-356), CG = 2, DGstress = 8   */
/* ------------------------------------------------------------------------ */
struct MomentumMap {
    std::vector<double> lumpedcgmass, lumpedcg1mass;
    std::vector<double> divS1, divS2;     // N x 9 x 8
    std::vector<double> iMgradX, iMgradY; // N x 8 x 9
    std::vector<double> iMJwPSI;          // N x 8 x 9
    std::vector<double> iMJwPSI_dam;      // N x dg x 9
    std::vector<double> dX_SSH, dY_SSH;   // N x 4 x 4
    std::vector<double> divM, iMM;        // spherical metric terms: N x 9 x 8, N x 8 x 9
    int dg = 0;

    void init(const Mesh& m, int DGadv)
    {
        dg = DGadv;
        const size_t N = m.nelements;
        // ParametricMap.cpp:94-206
        lumpedcgmass.assign((2 * m.nx + 1) * (2 * m.ny + 1), 0.0);
        for (size_t p = 0; p < 2; ++p)
            for (size_t iy = p; iy < m.ny; iy += 2)
                for (size_t ix = 0; ix < m.nx; ++ix) {
                    const size_t eid = m.nx * iy + ix;
                    double J[16], Meid[9], cl[16];
                    jacobian(m, eid, 4, J);
                    if (m.spherical) {
                        latTrig(m, eid, 4, cl, nullptr);
                        for (int q = 0; q < 16; ++q) J[q] = J[q] * GW(4, q) * cl[q];
                    } else
                        for (int q = 0; q < 16; ++q) J[q] = J[q] * GW(4, q);
                    for (int j = 0; j < 9; ++j) {
                        double s = 0;
                        for (int q = 0; q < 16; ++q) s += PHI(2, j, 4, q) * J[q];
                        Meid[j] = s;
                    }
                    const size_t sy = 2 * m.nx + 1, n0 = 2 * iy * sy + 2 * ix;
                    for (int j = 0; j < 9; ++j) lumpedcgmass[n0 + (j % 3) + (j / 3) * sy] += Meid[j];
                }
        lumpedcg1mass.assign((m.nx + 1) * (m.ny + 1), 0.0);
        for (size_t p = 0; p < 2; ++p)
            for (size_t iy = p; iy < m.ny; iy += 2)
                for (size_t ix = 0; ix < m.nx; ++ix) {
                    const size_t eid = m.nx * iy + ix;
                    double J[16], Meid[4], cl[16];
                    jacobian(m, eid, 2, J);
                    if (m.spherical) {
                        latTrig(m, eid, 2, cl, nullptr);
                        for (int q = 0; q < 4; ++q) J[q] = J[q] * GW(2, q) * cl[q];
                    } else
                        for (int q = 0; q < 4; ++q) J[q] = J[q] * GW(2, q);
                    for (int j = 0; j < 4; ++j) {
                        double s = 0;
                        for (int q = 0; q < 4; ++q) s += PHI(1, j, 2, q) * J[q];
                        Meid[j] = s;
                    }
                    const size_t sy = m.nx + 1, n0 = iy * sy + ix;
                    lumpedcg1mass[n0] += Meid[0];
                    lumpedcg1mass[n0 + 1] += Meid[1];
                    lumpedcg1mass[n0 + sy] += Meid[2];
                    lumpedcg1mass[n0 + 1 + sy] += Meid[3];
                }
        // ParametricMap.cpp:209-297 (Cartesian)
        divS1.assign(N * 72, 0.0);
        divS2.assign(N * 72, 0.0);
        iMgradX.assign(N * 72, 0.0);
        iMgradY.assign(N * 72, 0.0);
        iMJwPSI.assign(N * 72, 0.0);
        iMJwPSI_dam.assign(N * dg * 9, 0.0);
        dX_SSH.assign(N * 16, 0.0);
        dY_SSH.assign(N * 16, 0.0);
        if (m.spherical) {
            divM.assign(N * 72, 0.0);
            iMM.assign(N * 72, 0.0);
        }
#pragma omp parallel for schedule(static)
        for (long e = 0; e < static_cast<long>(N); ++e) {
            double Fx[2][16], Fy[2][16], J[16];
            dxdyT(m, e, 3, Fx, Fy);
            for (int r = 0; r < 2; ++r)
                for (int q = 0; q < 9; ++q) {
                    Fx[r][q] = Fx[r][q] * GW(3, q);
                    Fy[r][q] = Fy[r][q] * GW(3, q);
                }
            double dx2[9][9], dy2[9][9], dx1[4][9], dy1[4][9];
            for (int j = 0; j < 9; ++j)
                for (int q = 0; q < 9; ++q) {
                    dx2[j][q] = PHIx(2, j, 3, q) * Fy[1][q] - PHIy(2, j, 3, q) * Fx[1][q];
                    dy2[j][q] = PHIy(2, j, 3, q) * Fx[0][q] - PHIx(2, j, 3, q) * Fy[0][q];
                }
            for (int j = 0; j < 4; ++j)
                for (int q = 0; q < 9; ++q) {
                    dx1[j][q] = PHIx(1, j, 3, q) * Fy[1][q] - PHIy(1, j, 3, q) * Fx[1][q];
                    dy1[j][q] = PHIy(1, j, 3, q) * Fx[0][q] - PHIx(1, j, 3, q) * Fy[0][q];
                }
            jacobian(m, e, 3, J);
            double* d1 = &divS1[e * 72];
            double* d2 = &divS2[e * 72];
            // spherical (ParametricMap.cpp:298-347): (x, y) = (lon, lat); the
            // lat-derivative carries cos(lat), a divM term carries sin(lat),
            // and everything is divided by the Earth radius
            double cl[16], sl[16];
            if (m.spherical)
                latTrig(m, e, 3, cl, sl);
            for (int j = 0; j < 9; ++j)
                for (int k = 0; k < 8; ++k) {
                    double a = 0, b = 0;
                    for (int q = 0; q < 9; ++q) {
                        a += dx2[j][q] * PSI(k, 3, q);
                        b += (m.spherical ? dy2[j][q] * cl[q] : dy2[j][q]) * PSI(k, 3, q);
                    }
                    d1[j * 8 + k] = m.spherical ? a / kEarthRadius : a;
                    d2[j * 8 + k] = m.spherical ? b / kEarthRadius : b;
                }
            if (m.spherical)
                for (int j = 0; j < 9; ++j)
                    for (int k = 0; k < 8; ++k) {
                        double a = 0;
                        for (int q = 0; q < 9; ++q)
                            a += (PHI(2, j, 3, q) * (J[q] * sl[q] * GW(3, q))) * PSI(k, 3, q);
                        divM[e * 72 + j * 8 + k] = a / kEarthRadius;
                    }
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) {
                    double a = 0, b = 0;
                    for (int q = 0; q < 9; ++q) {
                        a += dx1[i][q] * PHI(1, j, 3, q);
                        b += (m.spherical ? dy1[i][q] * cl[q] : dy1[i][q]) * PHI(1, j, 3, q);
                    }
                    dX_SSH[e * 16 + i * 4 + j] = m.spherical ? a / kEarthRadius : a;
                    dY_SSH[e * 16 + i * 4 + j] = m.spherical ? b / kEarthRadius : b;
                }
            double imass[64];
            inverseMass(m, e, 8, imass);
            for (int i = 0; i < 8; ++i)
                for (int j = 0; j < 9; ++j) {
                    double a = 0, b = 0, c = 0, d = 0;
                    for (int k = 0; k < 8; ++k) {
                        a += imass[i * 8 + k] * d1[j * 8 + k];
                        b += imass[i * 8 + k] * d2[j * 8 + k];
                        c += imass[i * 8 + k] * (PSI(k, 3, j) * (GW(3, j) * J[j]));
                        if (m.spherical)
                            d += imass[i * 8 + k] * divM[e * 72 + j * 8 + k];
                    }
                    iMgradX[e * 72 + i * 9 + j] = a;
                    iMgradY[e * 72 + i * 9 + j] = b;
                    iMJwPSI[e * 72 + i * 9 + j] = c;
                    if (m.spherical)
                        iMM[e * 72 + i * 9 + j] = d;
                }
            double imd[64];
            inverseMass(m, e, dg, imd);
            for (int i = 0; i < dg; ++i)
                for (int j = 0; j < 9; ++j) {
                    double c = 0;
                    for (int k = 0; k < dg; ++k) c += imd[i * dg + k] * (PSI(k, 3, j) * (GW(3, j) * J[j]));
                    iMJwPSI_dam[(e * dg + i) * 9 + j] = c;
                }
        }
    }
};

/* ------------------------------------------------------------------------ */
/* Dynamics kernel: DynamicsKernel + CGDynamicsKernel + VPCG / Brittle       */
/* ------------------------------------------------------------------------ */
static const char* const kNames[] = { "hice", "cice", "ssh", "damage", "u", "v", "uwind", "vwind",
    "uocean", "vocean", "uiostress", "viostress" };

struct Kernel {
    int rheology = NSDG_RHEOLOGY_MEVP;
    int dg = 6;
    nsdg_params P {};
    Mesh mesh;
    Transport transport, stressTransport;
    CG2DGOp cg2dg, cg2dg8;
    MomentumMap pmap;
    DG hice, cice, ssh, damage;
    DG e11, e12, e22, s11, s12, s22;
    std::vector<double> u, v, u0, v0, cgH, cgA, uGrad, vGrad, dSx, dSy, uo, vo, ua, va, avgU, avgV;
    std::unordered_map<std::string, DG> bucket;
    std::unordered_map<std::string, int> bucketComps;
    double deltaT = 0;
    size_t stepNumber = 0;
    std::string err;
    bool ready = false;

    size_t Ncg() const { return (2 * mesh.nx + 1) * (2 * mesh.ny + 1); }

    // DynamicsKernel.hpp:44-75, CGDynamicsKernel.cpp:24-51, BrittleCGDynamicsKernel.hpp:72-86
    // DynamicsKernel.hpp:44-58
    int initialise(size_t nx, size_t ny, const double* coords, const double* mask, bool spherical = false)
    {
        Mesh& m = mesh;
        m = Mesh();
        m.spherical = spherical;
        m.nx = nx;
        m.ny = ny;
        m.nelements = nx * ny;
        m.nnodes = (nx + 1) * (ny + 1);
        m.vx.resize(m.nnodes);
        m.vy.resize(m.nnodes);
        for (size_t i = 0; i < m.nnodes; ++i) {
            m.vx[i] = coords[2 * i];
            m.vy[i] = coords[2 * i + 1];
        }
        if (spherical)
            m.rotatePoleToGreenland();
        m.landmask.resize(m.nelements);
        for (size_t i = 0; i < m.nelements; ++i) m.landmask[i] = (mask[i] == 1.) ? 1 : 0;
        m.dirichletFromMask();
        for (int e = 0; e < 4; ++e) m.dirichletFromEdge(e);
        transport.init(m, dg);
        transport.scheme = "rk2";
        cg2dg.init(m, dg);
        pmap.init(m, dg);
        const size_t N = m.nelements, Nc = Ncg();
        hice.resize(N, dg);
        cice.resize(N, dg);
        ssh.resize(N, 1);
        e11.resize(N, 8); e12.resize(N, 8); e22.resize(N, 8);
        s11.resize(N, 8); s12.resize(N, 8); s22.resize(N, 8);
        for (auto* vec : { &u, &v, &u0, &v0, &cgH, &cgA, &uGrad, &vGrad, &dSx, &dSy, &uo, &vo, &ua, &va, &avgU, &avgV })
            vec->assign(Nc, 0.0);
        if (rheology == NSDG_RHEOLOGY_BBM) {
            stressTransport.init(m, 8);
            stressTransport.scheme = "rk2";
            cg2dg8.init(m, 8);
            damage.resize(N, dg);
        }
        bucket.clear();
        bucketComps.clear();
        ready = true;
        return NSDG_OK;
    }

    // DGModelArray.hpp:20-32
    static void ma2dg(const double* data, size_t n, size_t nc, DG& d)
    {
        d.zero();
        if (static_cast<size_t>(d.n) == nc) {
            std::memcpy(d.a.data(), data, n * nc * sizeof(double));
        } else {
            for (size_t i = 0; i < n; ++i) d.a[i * d.n] = data[i * nc];
        }
    }
    // DynamicsKernel.hpp:93-110; CGDynamicsKernel.cpp:54-90; BrittleCGDynamicsKernel.hpp:138-145
    int setData(const std::string& name, const double* data, size_t n, size_t nc)
    {
        if (!ready) { err = "kernel not initialised"; return NSDG_ERR_BAD_ARG; }
        if (n != mesh.nelements || nc == 0) { err = "size mismatch for " + name; return NSDG_ERR_SIZE_MISMATCH; }
        std::vector<double>* cgTarget = nullptr;
        if (name == "u") cgTarget = &u;
        else if (name == "v") cgTarget = &v;
        else if (name == "uwind") cgTarget = &ua;
        else if (name == "vwind") cgTarget = &va;
        else if (name == "uocean") cgTarget = &uo;
        else if (name == "vocean") cgTarget = &vo;
        if (cgTarget) {
            DG tmp(mesh.nelements, dg);
            ma2dg(data, n, nc, tmp);
            DG2CG2(mesh, *cgTarget, tmp);
            return NSDG_OK;
        }
        if (rheology == NSDG_RHEOLOGY_BBM && name == "damage") { ma2dg(data, n, nc, damage); return NSDG_OK; }
        if (name == "hice") ma2dg(data, n, nc, hice);
        else if (name == "cice") ma2dg(data, n, nc, cice);
        else if (name == "ssh") { ssh.zero(); ma2dg(data, n, nc, ssh); }
        else {
            DG& d = bucket[name];
            d.resize(mesh.nelements, dg);
            ma2dg(data, n, nc, d);
            bucketComps[name] = static_cast<int>(nc);
        }
        return NSDG_OK;
    }

    // VPCGDynamicsKernel.hpp:96-120 and BrittleCGDynamicsKernel.hpp:168-192
    void iceOceanStress(std::vector<double>& tx, std::vector<double>& ty) const
    {
        const size_t Nc = Ncg();
        tx.assign(Nc, 0.0);
        ty.assign(Nc, 0.0);
        if (rheology == NSDG_RHEOLOGY_MEVP) {
            for (size_t i = 0; i < Nc; ++i) {
                const double ur = u[i] - uo[i], vr = v[i] - vo[i];
                const double a = std::sqrt(ur * ur + vr * vr);
                tx[i] = P.F_ocean * a * ur;
                ty[i] = P.F_ocean * a * vr;
            }
        } else {
            const double rad = 0x1.1df46a2529d39p-6;
            const double ca = std::cos(rad * P.ocean_turning_angle), sa = std::sin(rad * P.ocean_turning_angle);
            for (size_t i = 0; i < Nc; ++i) {
                const double ur = uo[i] - avgU[i], vr = vo[i] - avgV[i];
                const double cp = P.F_ocean * std::hypot(ur, vr);
                tx[i] = cp * (ur * ca - vr * sa);
                ty[i] = cp * (vr * ca + ur * sa);
            }
        }
    }

    // DynamicsKernel.hpp:119-130; CGDynamicsKernel.cpp:93-118
    int getDG0(const std::string& name, double* out, size_t n)
    {
        if (!ready) { err = "kernel not initialised"; return NSDG_ERR_BAD_ARG; }
        if (n != mesh.nelements) { err = "size mismatch"; return NSDG_ERR_SIZE_MISMATCH; }
        const DG* src = nullptr;
        DG tmp;
        if (name == "u" || name == "v" || name == "uiostress" || name == "viostress") {
            tmp.resize(mesh.nelements, dg);
            if (name == "u") cg2dg.apply(mesh, tmp, u);
            else if (name == "v") cg2dg.apply(mesh, tmp, v);
            else {
                std::vector<double> tx, ty;
                iceOceanStress(tx, ty);
                cg2dg.apply(mesh, tmp, name == "uiostress" ? tx : ty);
            }
            src = &tmp;
        } else if (rheology == NSDG_RHEOLOGY_BBM && name == "damage") src = &damage;
        else if (name == "hice") src = &hice;
        else if (name == "cice") src = &cice;
        else {
            auto it = bucket.find(name);
            if (it == bucket.end()) { err = "unknown field " + name; return NSDG_ERR_UNKNOWN_FIELD; }
            src = &it->second;
        }
        for (size_t i = 0; i < n; ++i) out[i] = src->a[i * src->n];
        return NSDG_OK;
    }
    // DynamicsKernel.hpp:138-156; BrittleCGDynamicsKernel.hpp:158-166
    int getDG(const std::string& name, double* out, size_t n, size_t nc)
    {
        if (!ready) { err = "kernel not initialised"; return NSDG_ERR_BAD_ARG; }
        if (n != mesh.nelements) { err = "size mismatch"; return NSDG_ERR_SIZE_MISMATCH; }
        const DG* src = nullptr;
        size_t want = dg;
        if (rheology == NSDG_RHEOLOGY_BBM && name == "damage") src = &damage;
        else if (name == "hice") src = &hice;
        else if (name == "cice") src = &cice;
        else {
            auto it = bucket.find(name);
            if (it == bucket.end()) { err = "unknown field " + name; return NSDG_ERR_UNKNOWN_FIELD; }
            src = &it->second;
            want = (bucketComps[name] == dg) ? dg : 1;
        }
        if (nc != want) { err = "component count mismatch"; return NSDG_ERR_SIZE_MISMATCH; }
        if (want == static_cast<size_t>(dg)) std::memcpy(out, src->a.data(), n * dg * sizeof(double));
        else for (size_t i = 0; i < n; ++i) out[i] = src->a[i * dg];
        return NSDG_OK;
    }

    // CGDynamicsKernel.cpp:126-258
    void computeGradientOfSSH()
    {
        const Mesh& m = mesh;
        const size_t s1 = m.nx + 1, Nc1 = (m.nx + 1) * (m.ny + 1);
        std::vector<double> cgSSH(Nc1), ug(Nc1, 0.0), vg(Nc1, 0.0);
        DG2CG1(m, cgSSH, ssh);
        for (size_t p = 0; p < 2; ++p)
            for (size_t cy = 0; cy < m.ny; ++cy) {
                if (cy % 2 != p) continue;
                size_t eid = m.nx * cy, c1 = cy * s1;
                for (size_t cx = 0; cx < m.nx; ++cx, ++eid, ++c1) {
                    const double loc[4] = { cgSSH[c1], cgSSH[c1 + 1], cgSSH[c1 + s1], cgSSH[c1 + s1 + 1] };
                    double tx[4], ty[4];
                    for (int i = 0; i < 4; ++i) {
                        double a = 0, b = 0;
                        for (int j = 0; j < 4; ++j) {
                            a += pmap.dX_SSH[eid * 16 + i * 4 + j] * loc[j];
                            b += pmap.dY_SSH[eid * 16 + i * 4 + j] * loc[j];
                        }
                        tx[i] = a;
                        ty[i] = b;
                    }
                    const size_t ids[4] = { c1, c1 + 1, c1 + s1, c1 + s1 + 1 };
                    for (int i = 0; i < 4; ++i) {
                        ug[ids[i]] -= tx[i];
                        vg[ids[i]] -= ty[i];
                    }
                }
            }
        for (size_t i = 0; i < Nc1; ++i) {
            ug[i] /= pmap.lumpedcg1mass[i];
            vg[i] /= pmap.lumpedcg1mass[i];
        }
        const size_t topleft = m.ny * s1;
        for (size_t i = 1; i < m.nx; ++i) {
            ug[i] = ug[i + s1]; vg[i] = vg[i + s1];
            ug[topleft + i] = ug[topleft + i - s1]; vg[topleft + i] = vg[topleft + i - s1];
        }
        for (size_t i = 1; i < m.ny; ++i) {
            ug[i * s1] = ug[i * s1 + 1]; vg[i * s1] = vg[i * s1 + 1];
            ug[i * s1 + s1 - 1] = ug[i * s1 + s1 - 2]; vg[i * s1 + s1 - 1] = vg[i * s1 + s1 - 2];
        }
        ug[0] = ug[s1 + 1]; vg[0] = vg[s1 + 1];
        ug[m.nx] = ug[m.nx + s1 - 1]; vg[m.nx] = vg[m.nx + s1 - 1];
        ug[m.ny * s1] = ug[(m.ny - 1) * s1 + 1]; vg[m.ny * s1] = vg[(m.ny - 1) * s1 + 1];
        ug[(m.ny + 1) * s1 - 1] = ug[m.ny * s1 - 2]; vg[(m.ny + 1) * s1 - 1] = vg[m.ny * s1 - 2];
        // CG1 -> CG2
        const size_t s2 = 2 * m.nx + 1;
        for (size_t iy = 0; iy <= m.ny; ++iy)
            for (size_t ix = 0; ix <= m.nx; ++ix) {
                uGrad[2 * iy * s2 + 2 * ix] = ug[iy * s1 + ix];
                vGrad[2 * iy * s2 + 2 * ix] = vg[iy * s1 + ix];
            }
        for (size_t iy = 0; iy <= m.ny; ++iy)
            for (size_t ix = 0; ix < m.nx; ++ix) {
                const size_t a = s1 * iy + ix, c2 = 2 * iy * s2 + 2 * ix + 1;
                uGrad[c2] = 0.5 * (ug[a] + ug[a + 1]);
                vGrad[c2] = 0.5 * (vg[a] + vg[a + 1]);
            }
        for (size_t iy = 0; iy < m.ny; ++iy)
            for (size_t ix = 0; ix <= m.nx; ++ix) {
                const size_t a = s1 * iy + ix, c2 = (2 * iy + 1) * s2 + 2 * ix;
                uGrad[c2] = 0.5 * (ug[a] + ug[a + s1]);
                vGrad[c2] = 0.5 * (vg[a] + vg[a + s1]);
            }
        for (size_t iy = 0; iy < m.ny; ++iy)
            for (size_t ix = 0; ix < m.nx; ++ix) {
                const size_t a = s1 * iy + ix, c2 = (2 * iy + 1) * s2 + 2 * ix + 1;
                uGrad[c2] = 0.25 * (ug[a] + ug[a + 1] + ug[a + s1] + ug[a + s1 + 1]);
                vGrad[c2] = 0.25 * (vg[a] + vg[a + 1] + vg[a + s1] + vg[a + s1 + 1]);
            }
    }

    // CGDynamicsKernel.cpp:260-276
    void prepareIteration()
    {
        DG2CG2(mesh, cgH, hice);
        DG2CG2(mesh, cgA, cice);
        computeGradientOfSSH();
        for (auto& a : cgA) a = std::min(a, 1.0);
        for (auto& a : cgA) a = std::max(a, 1.e-4);
        for (auto& h : cgH) h = std::max(h, 1.e-4);
    }

    // CGDynamicsKernel.cpp:300-337 (Cartesian)
    void projectVelocityToStrain()
    {
        const Mesh& m = mesh;
        const size_t s = 2 * m.nx + 1;
#pragma omp parallel for schedule(static)
        for (long row = 0; row < static_cast<long>(m.ny); ++row) {
            size_t dgi = m.nx * row, cgi = 2 * s * row;
            for (size_t col = 0; col < m.nx; ++col, ++dgi, cgi += 2) {
                if (!m.landmask[dgi]) continue;
                double ul[9], vl[9];
                for (int j = 0; j < 9; ++j) {
                    ul[j] = u[cgi + (j % 3) + (j / 3) * s];
                    vl[j] = v[cgi + (j % 3) + (j / 3) * s];
                }
                const double* GX = &pmap.iMgradX[dgi * 72];
                const double* GY = &pmap.iMgradY[dgi * 72];
                for (int i = 0; i < 8; ++i) {
                    double a = 0, b = 0, c = 0, d = 0;
                    for (int j = 0; j < 9; ++j) {
                        a += GX[i * 9 + j] * ul[j];
                        b += GY[i * 9 + j] * vl[j];
                        c += GX[i * 9 + j] * vl[j];
                        d += GY[i * 9 + j] * ul[j];
                    }
                    e11.row(dgi)[i] = a;
                    e22.row(dgi)[i] = b;
                    e12.row(dgi)[i] = 0.5 * (c + d);
                }
                if (m.spherical) { // CGDynamicsKernel.cpp:331-334
                    const double* MM = &pmap.iMM[dgi * 72];
                    for (int i = 0; i < 8; ++i) {
                        double mu = 0, mv = 0;
                        for (int j = 0; j < 9; ++j) {
                            mv += MM[i * 9 + j] * vl[j];
                            mu += MM[i * 9 + j] * ul[j];
                        }
                        e11.row(dgi)[i] -= mv;
                        e12.row(dgi)[i] += 0.5 * mu;
                    }
                }
            }
        }
    }

    // MEVPStressUpdateStep.hpp:30-118
    void mevpStress()
    {
        const double alpha = P.alpha;
        const double dmin2 = P.DeltaMin * P.DeltaMin;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < static_cast<long>(mesh.nelements); ++i) {
            double hg[9], ag[9], g11[9], g12[9], g22[9];
            for (int q = 0; q < 9; ++q) {
                double h = 0, a = 0, x = 0, y = 0, z = 0;
                for (int j = 0; j < dg; ++j) {
                    h += hice.row(i)[j] * PSI(j, 3, q);
                    a += cice.row(i)[j] * PSI(j, 3, q);
                }
                for (int j = 0; j < 8; ++j) {
                    x += e11.row(i)[j] * PSI(j, 3, q);
                    y += e12.row(i)[j] * PSI(j, 3, q);
                    z += e22.row(i)[j] * PSI(j, 3, q);
                }
                hg[q] = std::max(h, 0.0);
                ag[q] = std::min(std::max(a, 0.0), 1.0);
                g11[q] = x;
                g12[q] = y;
                g22[q] = z;
            }
            double f11[9], f12[9], f22[9];
            for (int q = 0; q < 9; ++q) {
                const double delta = std::sqrt(dmin2 + 1.25 * (g11[q] * g11[q] + g22[q] * g22[q])
                    + 1.50 * g11[q] * g22[q] + g12[q] * g12[q]);
                const double Pq = P.Pstar * hg[q] * std::exp(-20.0 * (1.0 - ag[q]));
                f11[q] = 1.0 / alpha * (Pq / 8.0 / delta * (5.0 * g11[q] + 3.0 * g22[q]) - 0.5 * Pq);
                f12[q] = 1.0 / alpha * (Pq / 4.0 / delta * g12[q]);
                f22[q] = 1.0 / alpha * (Pq / 8.0 / delta * (5.0 * g22[q] + 3.0 * g11[q]) - 0.5 * Pq);
            }
            const double* W = &pmap.iMJwPSI[i * 72];
            for (int k = 0; k < 8; ++k) {
                s11.row(i)[k] *= (1.0 - 1.0 / alpha);
                s12.row(i)[k] *= (1.0 - 1.0 / alpha);
                s22.row(i)[k] *= (1.0 - 1.0 / alpha);
            }
            for (int k = 0; k < 8; ++k) {
                double a = 0, b = 0, c = 0;
                for (int q = 0; q < 9; ++q) {
                    a += W[k * 9 + q] * f11[q];
                    b += W[k * 9 + q] * f12[q];
                    c += W[k * 9 + q] * f22[q];
                }
                s11.row(i)[k] += a;
                s12.row(i)[k] += b;
                s22.row(i)[k] += c;
            }
        }
    }

    // BBMStressUpdateStep.hpp:31-195
    void bbmStress()
    {
        const double dt = deltaT;
#pragma omp parallel for schedule(static)
        for (long i = 0; i < static_cast<long>(mesh.nelements); ++i) {
            double hG[9], aG[9], dG[9], e11G[9], e12G[9], e22G[9], s11G[9], s12G[9], s22G[9];
            for (int q = 0; q < 9; ++q) {
                double h = 0, a = 0, d = 0;
                for (int j = 0; j < dg; ++j) {
                    h += hice.row(i)[j] * PSI(j, 3, q);
                    a += cice.row(i)[j] * PSI(j, 3, q);
                    d += damage.row(i)[j] * PSI(j, 3, q);
                }
                hG[q] = std::max(h, 0.0);
                aG[q] = std::min(std::max(a, 0.0), 1.0);
                dG[q] = std::min(std::max(d, 1e-12), 1.0);
                double x = 0, y = 0, z = 0, sx = 0, sy = 0, sz = 0;
                for (int j = 0; j < 8; ++j) {
                    x += e11.row(i)[j] * PSI(j, 3, q);
                    y += e12.row(i)[j] * PSI(j, 3, q);
                    z += e22.row(i)[j] * PSI(j, 3, q);
                    sx += s11.row(i)[j] * PSI(j, 3, q);
                    sy += s12.row(i)[j] * PSI(j, 3, q);
                    sz += s22.row(i)[j] * PSI(j, 3, q);
                }
                e11G[q] = x; e12G[q] = y; e22G[q] = z;
                s11G[q] = sx; s12G[q] = sy; s22G[q] = sz;
            }
            const double hi = mesh.h(i);
            const double scale_coef = std::sqrt(0.1 / hi);
            for (int q = 0; q < 9; ++q) {
                double sigma_n = 0.5 * (s11G[q] + s22G[q]);
                const double expC = std::exp(P.compaction_param * (1.0 - aG[q]));
                const double powalphaexpC = std::pow(dG[q] * expC, P.exponent_relaxation_sigma - 1);
                const double time_viscous = P.undamaged_time_relaxation_sigma * powalphaexpC;
                const double Pmax = P.P0 * std::pow(hG[q], P.exponent_compression_factor + 1.) * expC;
                const double tildeP = (sigma_n < 0.0) ? std::min(-Pmax / sigma_n, 1.0) : 0.;
                const double multiplicator = time_viscous / (time_viscous + (1. - tildeP) * dt);
                const double elasticity = hG[q] * P.young * dG[q] * expC;
                const double Dunit_factor = dt * elasticity / (1. - (P.nu0 * P.nu0));
                s11G[q] += Dunit_factor * (e11G[q] + P.nu0 * e22G[q]);
                s22G[q] += Dunit_factor * (P.nu0 * e11G[q] + e22G[q]);
                s12G[q] += Dunit_factor * e12G[q] * (1. - P.nu0);
                s11G[q] *= multiplicator;
                s22G[q] *= multiplicator;
                s12G[q] *= multiplicator;
                sigma_n = 0.5 * (s11G[q] + s22G[q]);
                const double d = s11G[q] - s22G[q];
                const double tau = std::sqrt(0.25 * (d * d) + s12G[q] * s12G[q]);
                const double cohesion = P.C_lab * scale_coef * hG[q];
                const double compr = P.compr_strength * scale_coef * hG[q];
                double dcrit = (tau + P.tan_phi * sigma_n > 0.) ? cohesion / (tau + P.tan_phi * sigma_n) : 1.;
                dcrit = (sigma_n < -compr) ? -compr / sigma_n : dcrit;
                dcrit = std::min(dcrit, 1.0);
                const double td = hi * std::sqrt(2. * (1. + P.nu0) * P.rho_ice) / std::sqrt(elasticity);
                dG[q] -= dG[q] * (1. - dcrit) * dt / td;
                s11G[q] -= s11G[q] * (1. - dcrit) * dt / td;
                s12G[q] -= s12G[q] * (1. - dcrit) * dt / td;
                s22G[q] -= s22G[q] * (1. - dcrit) * dt / td;
            }
            const double* W = &pmap.iMJwPSI[i * 72];
            for (int k = 0; k < 8; ++k) {
                double a = 0, b = 0, c = 0;
                for (int q = 0; q < 9; ++q) {
                    a += W[k * 9 + q] * s11G[q];
                    b += W[k * 9 + q] * s12G[q];
                    c += W[k * 9 + q] * s22G[q];
                }
                s11.row(i)[k] = a;
                s12.row(i)[k] = b;
                s22.row(i)[k] = c;
            }
            const double* Wd = &pmap.iMJwPSI_dam[i * dg * 9];
            for (int k = 0; k < dg; ++k) {
                double a = 0;
                for (int q = 0; q < 9; ++q) a += Wd[k * 9 + q] * dG[q];
                damage.row(i)[k] = a;
            }
        }
    }

    // CGDynamicsKernel.cpp:401-437
    void dirichletZero(std::vector<double>& vec) const
    {
        const Mesh& m = mesh;
        const size_t s = 2 * m.nx + 1;
        for (int seg = 0; seg < 4; ++seg)
            for (size_t i = 0; i < m.dirichlet[seg].size(); ++i) {
                const size_t eid = m.dirichlet[seg][i];
                const size_t ix = eid % m.nx, iy = eid / m.nx;
                for (size_t j = 0; j < 3; ++j) {
                    size_t idx = 0;
                    if (seg == 0) idx = iy * 2 * s + 2 * ix + j;
                    else if (seg == 1) idx = iy * 2 * s + 2 * ix + 2 + s * j;
                    else if (seg == 2) idx = (iy + 1) * 2 * s + 2 * ix + j;
                    else idx = iy * 2 * s + 2 * ix + s * j;
                    vec[idx] = 0.0;
                }
            }
    }

    // CGDynamicsKernel.cpp:340-398
    void stressDivergence()
    {
        const Mesh& m = mesh;
        std::fill(dSx.begin(), dSx.end(), 0.0);
        std::fill(dSy.begin(), dSy.end(), 0.0);
        const size_t cgRow = 2 * m.nx + 1;
        for (size_t p = 0; p < 2; ++p) {
#pragma omp parallel for schedule(static)
            for (long cy = 0; cy < static_cast<long>(m.ny); ++cy) {
                if (static_cast<size_t>(cy) % 2 != p) continue;
                size_t c = m.nx * cy;
                for (size_t cx = 0; cx < m.nx; ++cx, ++c) {
                    if (!m.landmask[c]) continue;
                    const double* D1 = &pmap.divS1[c * 72];
                    const double* D2 = &pmap.divS2[c * 72];
                    const size_t cg_i = 2 * cgRow * cy + 2 * cx;
                    for (int j = 0; j < 9; ++j) {
                        double a = 0, b = 0, cc = 0, d = 0;
                        for (int k = 0; k < 8; ++k) {
                            a += D1[j * 8 + k] * s11.row(c)[k];
                            b += D2[j * 8 + k] * s12.row(c)[k];
                            cc += D1[j * 8 + k] * s12.row(c)[k];
                            d += D2[j * 8 + k] * s22.row(c)[k];
                        }
                        double tx = a + b, ty = cc + d;
                        if (m.spherical) { // CGDynamicsKernel.cpp:348-351
                            const double* DM = &pmap.divM[c * 72];
                            double e1 = 0, e2 = 0;
                            for (int k = 0; k < 8; ++k) {
                                e1 += DM[j * 8 + k] * s12.row(c)[k];
                                e2 += DM[j * 8 + k] * s11.row(c)[k];
                            }
                            tx += e1;
                            ty -= e2;
                        }
                        const size_t node = cg_i + (j % 3) + (j / 3) * cgRow;
                        dSx[node] -= tx;
                        dSy[node] -= ty;
                    }
                }
            }
        }
        dirichletZero(dSx);
        dirichletZero(dSy);
    }

    // VPCGDynamicsKernel.hpp:132-172
    void mevpMomentum()
    {
        const double beta = P.beta, dT = deltaT;
        const size_t Nc = Ncg();
#pragma omp parallel for schedule(static)
        for (long i = 0; i < static_cast<long>(Nc); ++i) {
            const double uOcnRel = uo[i] - u[i];
            const double vOcnRel = v[i] - vo[i];
            const double absatm = std::sqrt(ua[i] * ua[i] + va[i] * va[i]);
            const double absocn = std::sqrt(uOcnRel * uOcnRel + vOcnRel * vOcnRel);
            const double rhoH = P.rho_ice * cgH[i];
            const double inv = 1.0 / (rhoH / dT * (1.0 + beta) + cgA[i] * P.F_ocean * absocn);
            const double un = inv * (rhoH / dT * (beta * u[i] + u0[i])
                + cgA[i] * (P.F_atm * absatm * ua[i] + P.F_ocean * absocn * 1.0 * uo[i])
                - rhoH * P.fc * u[i] - rhoH * P.gravity * uGrad[i] + dSx[i] / pmap.lumpedcgmass[i]);
            const double vn = inv * (rhoH / dT * (beta * v[i] + v0[i])
                + cgA[i] * (P.F_atm * absatm * va[i] + P.F_ocean * absocn * 1.0 * vo[i])
                + rhoH * P.fc * v[i] - rhoH * P.gravity * vGrad[i] + dSy[i] / pmap.lumpedcgmass[i]);
            u[i] = un;
            v[i] = vn;
        }
    }

    // BrittleCGDynamicsKernel.hpp:206-254
    void bbmMomentum()
    {
        const double rad = 0x1.1df46a2529d39p-6;
        const double ca = std::cos(rad * P.ocean_turning_angle), sa = std::sin(rad * P.ocean_turning_angle);
        const size_t Nc = Ncg();
        const double dT = deltaT;
        const double nS = static_cast<double>(P.n_steps);
#pragma omp parallel for schedule(static)
        for (long i = 0; i < static_cast<long>(Nc); ++i) {
            const double dteOverMass = dT / (P.rho_ice * cgH[i]);
            const double uIce = u[i], vIce = v[i];
            const double cPrime = cgA[i] * P.F_ocean * std::hypot(uo[i] - uIce, vo[i] - vIce);
            const double tauB = 0.;
            const double alpha = 1 + dteOverMass * (cPrime * ca + tauB);
            const double beta = dT * P.fc + dteOverMass * cPrime * sa;
            const double rDenom = 1 / (alpha * alpha + beta * beta);
            const double dragAtm = cgA[i] * P.F_atm * std::hypot(ua[i], va[i]);
            const double tauX = dragAtm * ua[i] + cPrime * (uo[i] * ca - vo[i] * sa);
            const double tauY = dragAtm * va[i] + cPrime * (vo[i] * ca + uo[i] * sa);
            const double gradX = dSx[i] / pmap.lumpedcgmass[i] - P.rho_ice * cgH[i] * P.gravity * uGrad[i];
            const double gradY = dSy[i] / pmap.lumpedcgmass[i] - P.rho_ice * cgH[i] * P.gravity * vGrad[i];
            double un = alpha * uIce + beta * vIce + dteOverMass * (alpha * (gradX + tauX) + beta * (gradY + tauY));
            un *= rDenom;
            double vn = alpha * vIce - beta * uIce + dteOverMass * (alpha * (gradY + tauY) + beta * (gradX + tauX));
            vn *= rDenom;
            u[i] = un;
            v[i] = vn;
            avgU[i] += un / nS;
            avgV[i] += vn / nS;
        }
    }

    // VPCGDynamicsKernel.hpp:63-94; BrittleCGDynamicsKernel.hpp:91-136
    int update(double dt)
    {
        if (!ready) { err = "kernel not initialised"; return NSDG_ERR_BAD_ARG; }
        if (rheology == NSDG_RHEOLOGY_MEVP) {
            // DynamicsKernel::advectionAndLimits (DynamicsKernel.hpp:160-172)
            cg2dg.apply(mesh, transport.velx, u);
            cg2dg.apply(mesh, transport.vely, v);
            transport.reinitnormalvelocity();
            transport.step(dt, cice);
            transport.step(dt, hice);
            LimitMax(cice, 1.0);
            LimitMin(cice, 0.0);
            LimitMin(hice, 0.0);
            prepareIteration();
            u0 = u;
            v0 = v;
            deltaT = dt;
            for (int it = 0; it < P.n_steps; ++it) {
                projectVelocityToStrain();
                mevpStress();
                stressDivergence();
                mevpMomentum();
                dirichletZero(u);
                dirichletZero(v);
            }
        } else {
            cg2dg.apply(mesh, transport.velx, avgU);
            cg2dg.apply(mesh, transport.vely, avgV);
            transport.reinitnormalvelocity();
            transport.step(dt, cice);
            transport.step(dt, hice);
            LimitMax(cice, 1.0);
            LimitMin(cice, 0.0);
            LimitMin(hice, 0.0);
            cg2dg8.apply(mesh, stressTransport.velx, avgU);
            cg2dg8.apply(mesh, stressTransport.vely, avgV);
            stressTransport.reinitnormalvelocity();
            stressTransport.step(dt, s11);
            stressTransport.step(dt, s12);
            stressTransport.step(dt, s22);
            transport.step(dt, damage);
            LimitMax(damage, 1.0);
            LimitMin(damage, 1e-12);
            prepareIteration();
            deltaT = dt / P.n_steps;
            std::fill(avgU.begin(), avgU.end(), 0.0);
            std::fill(avgV.begin(), avgV.end(), 0.0);
            for (int it = 0; it < P.n_steps; ++it) {
                projectVelocityToStrain();
                bbmStress();
                stressDivergence();
                bbmMomentum();
                dirichletZero(u);
                dirichletZero(v);
            }
        }
        ++stepNumber;
        return NSDG_OK;
    }
};

/* ------------------------------------------------------------------------ */
/* Reference test scenarios (for the golden values)                         */
/* ------------------------------------------------------------------------ */
// dynamics/test/Advection_test.cpp:71-101 (fp: {Lx})
static double smoothBump(double x, double y, const double* fp)
{
    const double X = x / fp[0], Y = y / fp[0];
    const double r = (std::pow((X - 0.25), 2.0) + std::pow((Y - 0.5), 2.0)) / 0.025;
    return (r < 1) ? std::exp(-1.0 / (1.0 - r)) : 0.0;
}
static double rotVX(double, double y, const double* fp) { return (y - 0.5 * fp[0]) * 2.0 * M_PI / fp[0]; }
static double rotVY(double x, double, const double* fp) { return (0.5 * fp[0] - x) * 2.0 * M_PI / fp[0]; }
// dynamics/test/AdvectionPeriodicBC_test.cpp:71-113 (fp: {R1})
static double packman(double x, double y, const double*)
{
    double r = (std::pow((x + 175000.0) / 50000, 2.0) + std::pow((y) / 50000.0, 2.0));
    if (r < 1.0) return std::exp(1.0) * std::exp(-1.0 / (1.0 - r));
    r = (std::pow((x) / 50000, 2.0) + std::pow((y - 175000.0) / 50000.0, 2.0));
    if (r < 1.0) {
        if (y > 175000) return 1.0;
        if (std::fabs(x) > 15000.0) return 1.0;
        return 0.0;
    }
    r = std::sqrt(std::pow((x - 175000.0) / 50000, 2.0) + std::pow((y) / 50000.0, 2.0));
    if (r < 1.0) return 1.0 - r;
    r = std::sqrt(std::pow((x) / 50000, 2.0) + std::pow((y + 175000.) / 50000.0, 2.0));
    if (r < 1.0) return 1.0;
    return 0.0;
}
static double ringVX(double, double y, const double* fp) { return y * 2.0 * M_PI / fp[0]; }
static double ringVY(double x, double, const double* fp) { return -x * 2.0 * M_PI / fp[0]; }

// Advection_test.cpp:198-241
static void rectangleMesh(Mesh& m, double Lx, double Ly, size_t Nx, size_t Ny, double distort)
{
    m = Mesh();
    m.nx = Nx; m.ny = Ny; m.nnodes = (Nx + 1) * (Ny + 1); m.nelements = Nx * Ny;
    m.vx.resize(m.nnodes); m.vy.resize(m.nnodes);
    size_t ii = 0;
    for (size_t iy = 0; iy <= Ny; ++iy)
        for (size_t ix = 0; ix <= Nx; ++ix, ++ii) {
            m.vx[ii] = Lx * ix / Nx + Lx * distort * std::sin(M_PI * ix / Nx * 3.0) * std::sin(M_PI * iy / Ny);
            m.vy[ii] = Ly * iy / Ny + Ly * distort * std::sin(M_PI * iy / Ny * 2.0) * std::sin(M_PI * ix / Nx * 2.0);
        }
    m.landmask.assign(m.nelements, 1);
    for (size_t i = 0; i < Nx; ++i) m.dirichlet[0].push_back(i);
    for (size_t i = 0; i < Ny; ++i) m.dirichlet[1].push_back(i * Nx + Nx - 1);
    for (size_t i = 0; i < Nx; ++i) m.dirichlet[2].push_back(Nx * (Ny - 1) + i);
    for (size_t i = 0; i < Ny; ++i) m.dirichlet[3].push_back(i * Nx);
}
// AdvectionPeriodicBC_test.cpp:210-255
static void ringMesh(Mesh& m, double R0, double R1, size_t Nx, size_t Ny)
{
    m = Mesh();
    m.nx = Nx; m.ny = Ny; m.nnodes = (Nx + 1) * (Ny + 1); m.nelements = Nx * Ny;
    m.vx.resize(m.nnodes); m.vy.resize(m.nnodes);
    size_t ii = 0;
    for (size_t iy = 0; iy <= Ny; ++iy)
        for (size_t ix = 0; ix <= Nx; ++ix, ++ii) {
            const double r = R0 + (R1 - R0) * iy / Ny;
            const double p = -2.0 * M_PI * ix / Nx;
            m.vx[ii] = r * std::cos(p);
            m.vy[ii] = r * std::sin(p);
        }
    m.landmask.assign(m.nelements, 1);
    for (size_t i = 0; i < Nx; ++i) m.dirichlet[0].push_back(i);
    for (size_t i = 0; i < Nx; ++i) m.dirichlet[2].push_back(Nx * (Ny - 1) + i);
    m.periodic.resize(1);
    for (size_t i = 0; i < Ny; ++i)
        m.periodic[0].push_back({ 1, (i + 1) * Nx - 1, i * Nx, i * (Nx + 1) + i });
}

} // namespace oracle

/* ======================================================================== */
/* extern "C" API used by the tests and the CPU baseline                     */
/* ======================================================================== */
using namespace oracle;

extern "C" {

/* Reference defaults: DynamicsParameters.hpp:22-40, VPParameters.hpp:20-25,
 * MEBParameters.hpp:40-65, VPCGDynamicsKernel.hpp:125-126, DynamicsKernel.hpp:187 */
void oracle_default_params(nsdg_params* p)
{
    std::memset(p, 0, sizeof(*p));
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
    p->Pstar = 27500.0;
    p->DeltaMin = 2.e-9;
    p->alpha = 1500.;
    p->beta = 1500.;
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
    p->n_steps = 100;
    p->precision = NSDG_PRECISION_FP64;
}

void* oracle_kernel_create(int rheology, int dg, const nsdg_params* p)
{
    if (!p || (dg != 1 && dg != 3 && dg != 6)) return nullptr;
    if (rheology != NSDG_RHEOLOGY_MEVP && rheology != NSDG_RHEOLOGY_BBM) return nullptr;
    Kernel* k = new Kernel();
    k->rheology = rheology;
    k->dg = dg;
    k->P = *p;
    return k;
}
void oracle_kernel_destroy(void* k) { delete static_cast<Kernel*>(k); }
const char* oracle_kernel_last_error(void* k) { return static_cast<Kernel*>(k)->err.c_str(); }
int oracle_kernel_initialise(void* k, size_t nx, size_t ny, const double* coords, const double* mask)
{
    return static_cast<Kernel*>(k)->initialise(nx, ny, coords, mask);
}
int oracle_kernel_initialise_spherical(void* k, size_t nx, size_t ny, const double* coords, int spherical,
    const double* mask)
{
    return static_cast<Kernel*>(k)->initialise(nx, ny, coords, mask, spherical != 0);
}
int oracle_kernel_set_data(void* k, const char* name, const double* d, size_t n, size_t nc)
{
    return static_cast<Kernel*>(k)->setData(name, d, n, nc);
}
int oracle_kernel_get_dg0(void* k, const char* name, double* out, size_t n)
{
    return static_cast<Kernel*>(k)->getDG0(name, out, n);
}
int oracle_kernel_get_dg(void* k, const char* name, double* out, size_t n, size_t nc)
{
    return static_cast<Kernel*>(k)->getDG(name, out, n, nc);
}
int oracle_kernel_update(void* k, double, double dt) { return static_cast<Kernel*>(k)->update(dt); }
// CG2 node arrays (test access to internal state): "u","v","cgH","cgA"
int oracle_kernel_get_cg(void* kp, const char* name, double* out, size_t n)
{
    Kernel* k = static_cast<Kernel*>(kp);
    const std::vector<double>* src = nullptr;
    std::string s(name);
    if (s == "u") src = &k->u;
    else if (s == "v") src = &k->v;
    else if (s == "cgH") src = &k->cgH;
    else if (s == "cgA") src = &k->cgA;
    else if (s == "uwind") src = &k->ua;
    else if (s == "uocean") src = &k->uo;
    else if (s == "uGrad") src = &k->uGrad;
    else if (s == "vGrad") src = &k->vGrad;
    if (!src || n != src->size()) return NSDG_ERR_BAD_ARG;
    std::memcpy(out, src->data(), n * sizeof(double));
    return NSDG_OK;
}
// DGSTRESS state "s11","s12","s22" (N x 8)
int oracle_kernel_get_stress(void* kp, const char* name, double* out, size_t n)
{
    Kernel* k = static_cast<Kernel*>(kp);
    std::string s(name);
    const DG* src = s == "s11" ? &k->s11 : s == "s12" ? &k->s12 : s == "s22" ? &k->s22 : nullptr;
    if (!src || n != src->a.size()) return NSDG_ERR_BAD_ARG;
    std::memcpy(out, src->a.data(), n * sizeof(double));
    return NSDG_OK;
}
double oracle_kernel_mean_value(void* kp, const char* name)
{
    Kernel* k = static_cast<Kernel*>(kp);
    std::string s(name);
    if (s == "hice") return MeanValue(k->mesh, k->hice);
    if (s == "cice") return MeanValue(k->mesh, k->cice);
    if (s == "damage") return MeanValue(k->mesh, k->damage);
    return NAN;
}
/* ParametricMesh::landmaskFromModelArray + dirichletFromMask + dirichletFromEdge
 * (ParametricMesh.cpp:217-272), as the kernel's initialise runs them: counts[s]
 * ascending element ids for side s, written to ids side after side; -1 when
 * capacity is short (counts still set). */
int oracle_mesh_dirichlet(size_t nx, size_t ny, const double* mask, size_t* counts, size_t* ids, size_t capacity)
{
    Mesh m;
    m.nx = nx;
    m.ny = ny;
    m.nelements = nx * ny;
    m.nnodes = (nx + 1) * (ny + 1);
    m.landmask.resize(m.nelements);
    for (size_t i = 0; i < m.nelements; ++i) m.landmask[i] = (mask[i] == 1.) ? 1 : 0;
    m.dirichletFromMask();
    for (int e = 0; e < 4; ++e) m.dirichletFromEdge(e);
    size_t total = 0;
    for (int s = 0; s < 4; ++s) {
        counts[s] = m.dirichlet[s].size();
        total += counts[s];
    }
    if (total > capacity)
        return -1;
    for (int s = 0; s < 4; ++s)
        for (size_t e : m.dirichlet[s])
            *ids++ = e;
    return 0;
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
void oracle_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* Tables for cross-checks (row-major as in the reference). */
int oracle_table(const char* name, int a, int b, double* out)
{
    std::string s(name);
    if (s == "PSI") { for (int j = 0; j < a; ++j) for (int q = 0; q < b * b; ++q) out[j * b * b + q] = PSI(j, b, q); return 0; }
    if (s == "GAUSSWEIGHTS") { for (int q = 0; q < a * a; ++q) out[q] = GW(a, q); return 0; }
    if (s == "GAUSSPOINTS") { for (int q = 0; q < a; ++q) out[q] = QUAD.p[a][q]; return 0; }
    if (s == "PSILagrange") { for (int j = 0; j < a; ++j) for (int q = 0; q < b * b; ++q) out[j * b * b + q] = PSILagrange(j, b, q); return 0; }
    if (s == "PHI") { for (int j = 0; j < (a + 1) * (a + 1); ++j) for (int q = 0; q < b * b; ++q) out[j * b * b + q] = PHI(a, j, b, q); return 0; }
    return 1;
}

/* ---- generic stand-alone transport (mirrors nsdg_transport_*) ---------- */
struct OTransport {
    Mesh mesh;
    Transport tr;
};
void* oracle_transport_create(int dg, size_t nx, size_t ny, const double* vertices,
    const unsigned char* landmask, const size_t* const dir[4], const size_t ndir[4],
    const size_t* periodic, size_t nper, int scheme)
{
    OTransport* t = new OTransport();
    Mesh& m = t->mesh;
    m.nx = nx; m.ny = ny; m.nelements = nx * ny; m.nnodes = (nx + 1) * (ny + 1);
    m.vx.resize(m.nnodes); m.vy.resize(m.nnodes);
    for (size_t i = 0; i < m.nnodes; ++i) { m.vx[i] = vertices[2 * i]; m.vy[i] = vertices[2 * i + 1]; }
    m.landmask.assign(m.nelements, 1);
    if (landmask) for (size_t i = 0; i < m.nelements; ++i) m.landmask[i] = landmask[i] ? 1 : 0;
    for (int s = 0; s < 4; ++s) for (size_t i = 0; i < ndir[s]; ++i) m.dirichlet[s].push_back(dir[s][i]);
    if (nper) {
        m.periodic.resize(1);
        for (size_t i = 0; i < nper; ++i)
            m.periodic[0].push_back({ periodic[4 * i], periodic[4 * i + 1], periodic[4 * i + 2], periodic[4 * i + 3] });
    }
    t->tr.init(m, dg);
    t->tr.scheme = scheme == 1 ? "rk1" : scheme == 3 ? "rk3" : "rk2";
    return t;
}
void oracle_transport_destroy(void* t) { delete static_cast<OTransport*>(t); }
void oracle_transport_set_velocity(void* tp, const double* vx, const double* vy)
{
    OTransport* t = static_cast<OTransport*>(tp);
    std::memcpy(t->tr.velx.a.data(), vx, t->tr.velx.a.size() * sizeof(double));
    std::memcpy(t->tr.vely.a.data(), vy, t->tr.vely.a.size() * sizeof(double));
}
void oracle_transport_reinit(void* tp) { static_cast<OTransport*>(tp)->tr.reinitnormalvelocity(); }
void oracle_transport_step(void* tp, double dt, double* phi, int nsteps, int lmax, double maxv, int lmin, double minv)
{
    OTransport* t = static_cast<OTransport*>(tp);
    DG d(t->mesh.nelements, t->tr.dg);
    std::memcpy(d.a.data(), phi, d.a.size() * sizeof(double));
    for (int s = 0; s < nsteps; ++s) {
        t->tr.step(dt, d);
        if (lmax) LimitMax(d, maxv);
        if (lmin) LimitMin(d, minv);
    }
    std::memcpy(phi, d.a.data(), d.a.size() * sizeof(double));
}
// LimitMax / LimitMin of a host field (dgLimit.hpp:16-85)
void oracle_transport_limit(void* tp, double* phi, int lmax, double maxv, int lmin, double minv)
{
    OTransport* t = static_cast<OTransport*>(tp);
    DG d(t->mesh.nelements, t->tr.dg);
    std::memcpy(d.a.data(), phi, d.a.size() * sizeof(double));
    if (lmax) LimitMax(d, maxv);
    if (lmin) LimitMin(d, minv);
    std::memcpy(phi, d.a.data(), d.a.size() * sizeof(double));
}
double oracle_transport_mean_value(void* tp, const double* phi)
{
    OTransport* t = static_cast<OTransport*>(tp);
    DG d(t->mesh.nelements, t->tr.dg);
    std::memcpy(d.a.data(), phi, d.a.size() * sizeof(double));
    return MeanValue(t->mesh, d);
}
/* Function2DG / L2ErrorFunctionDG of the reference test functions on a
 * transport mesh.  fn: 0 smooth bump, 1 rotating vx, 2 rotating vy (param Lx);
 * 3 packman, 4 ring vx, 5 ring vy (param R1). */
static Function testFunction(int fn)
{
    switch (fn) {
    case 0: return smoothBump;
    case 1: return rotVX;
    case 2: return rotVY;
    case 3: return packman;
    case 4: return ringVX;
    default: return ringVY;
    }
}
void oracle_transport_function2dg(void* tp, int fn, double param, double* out)
{
    OTransport* t = static_cast<OTransport*>(tp);
    DG d(t->mesh.nelements, t->tr.dg);
    Function2DG(t->mesh, d, testFunction(fn), &param);
    std::memcpy(out, d.a.data(), d.a.size() * sizeof(double));
}
double oracle_transport_l2error(void* tp, int fn, double param, const double* phi)
{
    OTransport* t = static_cast<OTransport*>(tp);
    DG d(t->mesh.nelements, t->tr.dg);
    std::memcpy(d.a.data(), phi, d.a.size() * sizeof(double));
    return L2ErrorFunctionDG(t->mesh, d, testFunction(fn), &param);
}

/* The reference's golden scenarios, end to end on the CPU. */
// Advection_test.cpp:105-265: returns the L2 error, *massloss the relative mass change
double oracle_advection_golden(int dg, double distort, int it, double* massloss)
{
    const double Lx = 409600.0, Ly = 512000.0;
    const size_t Nx = 12u << it, Ny = 13u << it;
    const int deg = dg == 1 ? 0 : dg == 3 ? 1 : 2;
    const size_t NT = 100 * (deg + 1) * (deg + 1) * (1u << it);
    Mesh m;
    rectangleMesh(m, Lx, Ly, Nx, Ny, distort);
    Transport tr;
    tr.init(m, dg);
    tr.scheme = dg < 3 ? "rk2" : "rk3";
    const double dt = Lx / NT;
    DG phi(m.nelements, dg);
    Function2DG(m, phi, smoothBump, &Lx);
    const double initial = MeanValue(m, phi);
    Function2DG(m, tr.velx, rotVX, &Lx);
    Function2DG(m, tr.vely, rotVY, &Lx);
    for (size_t iter = 1; iter <= NT; ++iter) {
        tr.reinitnormalvelocity();
        tr.step(dt, phi);
    }
    if (massloss) *massloss = (initial - MeanValue(m, phi)) / initial;
    return std::sqrt(L2ErrorFunctionDG(m, phi, smoothBump, &Lx)) / Lx;
}
// AdvectionPeriodicBC_test.cpp:117-276
double oracle_periodic_golden(int dg, int it, double* massloss)
{
    const double R0 = 100000.0, R1 = 250000.0;
    const size_t Nx = 32u << it, Ny = 4u << it;
    const int deg = dg == 1 ? 0 : dg == 3 ? 1 : 2;
    const size_t NT = 50 * (deg + 1) * (deg + 1) * (1u << it);
    Mesh m;
    ringMesh(m, R0, R1, Nx, Ny);
    Transport tr;
    tr.init(m, dg);
    tr.scheme = dg < 3 ? "rk2" : "rk3";
    const double dt = R1 / NT;
    DG phi(m.nelements, dg);
    Function2DG(m, phi, packman, &R1);
    LimitMax(phi, 1.0);
    const double initial = MeanValue(m, phi);
    Function2DG(m, tr.velx, ringVX, &R1);
    Function2DG(m, tr.vely, ringVY, &R1);
    for (size_t iter = 1; iter <= NT; ++iter) {
        tr.reinitnormalvelocity();
        tr.step(dt, phi);
        LimitMax(phi, 1.0);
        LimitMin(phi, 0.0);
    }
    if (massloss) *massloss = (initial - MeanValue(m, phi)) / initial;
    return std::sqrt(L2ErrorFunctionDG(m, phi, packman, &R1)) / R0;
}

} // extern "C"
