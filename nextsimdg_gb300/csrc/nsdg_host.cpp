// nsdg_host.cpp — FP64 host precompute (see nsdg_host.hpp).
//
// Compiled with -ffp-contract=off so the operators are identical on x86-64
// and aarch64 hosts.
#include "nsdg_host.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <thread>

namespace nsdg {

// ---------------------------------------------------------------------------
// Quadrature rules and basis functions
// (dynamics/codegeneration/gaussquadrature.py:7-29; basisfunctions.py:33-160)
// ---------------------------------------------------------------------------
Basis::Basis()
{
    gp[1][0] = 0.5;
    gw[1][0] = 1.0;
    const double a2 = std::sqrt(1. / 12.);
    gp[2][0] = 0.5 - a2;
    gp[2][1] = 0.5 + a2;
    gw[2][0] = gw[2][1] = 0.5;
    const double a3 = std::sqrt(3. / 20.);
    gp[3][0] = 0.5 - a3;
    gp[3][1] = 0.5;
    gp[3][2] = 0.5 + a3;
    gw[3][0] = gw[3][2] = 5. / 18.;
    gw[3][1] = 8. / 18.;
    const double r = std::sqrt(6. / 5.);
    const double a4o = 0.5 * std::sqrt(3. / 7. + 2. / 7. * r);
    const double a4i = 0.5 * std::sqrt(3. / 7. - 2. / 7. * r);
    gp[4][0] = 0.5 - a4o;
    gp[4][1] = 0.5 - a4i;
    gp[4][2] = 0.5 + a4i;
    gp[4][3] = 0.5 + a4o;
    const double s30 = std::sqrt(30.0);
    gw[4][0] = gw[4][3] = (18. - s30) / 72.;
    gw[4][1] = gw[4][2] = (18. + s30) / 72.;
}

const Basis& basis()
{
    static const Basis b;
    return b;
}

// Legendre-type modal basis on [0,1]^2: 1, x~, y~, x~^2-1/12, y~^2-1/12, x~y~,
// y~(x~^2-1/12), x~(y~^2-1/12) with x~ = x-1/2.
double Basis::dg(int j, double x, double y)
{
    const double xs = x - 0.5, ys = y - 0.5;
    switch (j) {
    case 0: return 1.;
    case 1: return xs;
    case 2: return ys;
    case 3: return xs * xs - 1.0 / 12.0;
    case 4: return ys * ys - 1.0 / 12.0;
    case 5: return xs * ys;
    case 6: return ys * (xs * xs - 1.0 / 12.0);
    case 7: return xs * (ys * ys - 1.0 / 12.0);
    default: return 0.0;
    }
}
double Basis::dgdx(int j, double x, double y)
{
    const double xs = x - 0.5, ys = y - 0.5;
    switch (j) {
    case 1: return 1.;
    case 3: return 2.0 * xs;
    case 5: return ys;
    case 6: return ys * (2. * xs);
    case 7: return ys * ys - 1.0 / 12.0;
    default: return 0.0;
    }
}
double Basis::dgdy(int j, double x, double y)
{
    const double xs = x - 0.5, ys = y - 0.5;
    switch (j) {
    case 2: return 1.;
    case 4: return 2. * ys;
    case 5: return xs;
    case 6: return xs * xs - 1.0 / 12.0;
    case 7: return xs * (2. * ys);
    default: return 0.0;
    }
}
double Basis::edge(int j, double t)
{
    const double ts = t - 0.5;
    return j == 0 ? 1. : (j == 1 ? ts : ts * ts - 1.0 / 12.0);
}
// 1d Lagrange bases: CG1 {1-x, x}; CG2 {2(x-1/2)(x-1), 4x(1-x), 2x(x-1/2)}
double Basis::cg1d(int deg, int j, double x)
{
    if (deg == 1)
        return j == 0 ? 1.0 - x : x;
    if (j == 0)
        return 2.0 * (x - 0.5) * (x - 1.0);
    if (j == 1)
        return 4.0 * x * (1.0 - x);
    return 2.0 * x * (x - 0.5);
}
double Basis::cg1ddx(int deg, int j, double x)
{
    if (deg == 1)
        return j == 0 ? -1.0 : 1.0;
    if (j == 0)
        return 4.0 * x - 3.0;
    if (j == 1)
        return 4.0 - 8.0 * x;
    return 4.0 * x - 1.0;
}
double Basis::phi(int deg, int j, int Q, int q) const
{
    return cg1d(deg, j % (deg + 1), gp[Q][q % Q]) * cg1d(deg, j / (deg + 1), gp[Q][q / Q]);
}
double Basis::phix(int deg, int j, int Q, int q) const
{
    return cg1ddx(deg, j % (deg + 1), gp[Q][q % Q]) * cg1d(deg, j / (deg + 1), gp[Q][q / Q]);
}
double Basis::phiy(int deg, int j, int Q, int q) const
{
    return cg1d(deg, j % (deg + 1), gp[Q][q % Q]) * cg1ddx(deg, j / (deg + 1), gp[Q][q / Q]);
}
// Weighted trace of DG basis j on edge E (0 bottom, 1 right, 2 top, 3 left)
// at edge Gauss point g of a G-point rule.
double Basis::psiEdgeW(int j, int G, int E, int g) const
{
    const double t = gp[G][g];
    const double x = (E == 0 || E == 2) ? t : (E == 1 ? 1.0 : 0.0);
    const double y = (E == 1 || E == 3) ? t : (E == 2 ? 1.0 : 0.0);
    return gw[G][g] * dg(j, x, y);
}
// DG basis at the Lagrange points {0,1} (G=2) or {0,1/2,1} (G=3).
double Basis::psiLagrange(int j, int G, int q) const
{
    const double l2[2] = { 0.0, 1.0 };
    const double l3[3] = { 0.0, 0.5, 1.0 };
    const double* l = G == 2 ? l2 : l3;
    return dg(j, l[q % G], l[q / G]);
}

void fillConstTables(ConstTables& t)
{
    std::memset(&t, 0, sizeof(t));
    const Basis& b = basis();
    for (int Q = 1; Q <= 3; ++Q)
        for (int j = 0; j < 8; ++j)
            for (int q = 0; q < Q * Q; ++q) {
                t.psi[Q][j][q] = b.psi(j, Q, q);
                t.psix[Q][j][q] = b.psix(j, Q, q);
            }
    for (int j = 0; j < 8; ++j)
        for (int q = 0; q < 9; ++q)
            t.psiLag3[j][q] = b.psiLagrange(j, 3, q);
    for (int G = 1; G <= 3; ++G) {
        for (int j = 0; j < G; ++j)
            for (int g = 0; g < G; ++g)
                t.psie[G][j][g] = Basis::edge(j, b.gp[G][g]);
        for (int E = 0; E < 4; ++E)
            for (int g = 0; g < G; ++g)
                for (int j = 0; j < 8; ++j)
                    t.psiew[G][E][g][j] = b.psiEdgeW(j, G, E, g);
    }
    for (int Q = 1; Q <= 3; ++Q)
        for (int j = 0; j < 9; ++j)
            for (int q = 0; q < Q * Q; ++q)
                t.phi2[Q][j][q] = b.phi(2, j, Q, q);
    for (int Q = 1; Q <= 4; ++Q)
        for (int q = 0; q < Q * Q; ++q)
            t.gw[Q][q] = b.weight(Q, q);
}

// ---------------------------------------------------------------------------
// Mesh
// ---------------------------------------------------------------------------
void HostMesh::elementCoords(size_t e, double c[4][2]) const
{
    const size_t n0 = (e / nx) * (nx + 1) + (e % nx);
    const size_t id[4] = { n0, n0 + 1, n0 + nx + 1, n0 + nx + 2 };
    for (int k = 0; k < 4; ++k) {
        c[k][0] = vx[id[k]];
        c[k][1] = vy[id[k]];
    }
    if (spherical) {
        // no longitude jump across the element (ParametricMesh.hpp:196-209)
        bool jump = false;
        for (int k = 1; k < 4; ++k)
            jump = jump || std::fabs(c[0][0] - c[k][0]) > 2.0 / 3.0 * M_PI;
        if (jump)
            for (int k = 0; k < 4; ++k)
                if (c[k][0] < 0)
                    c[k][0] += 2.0 * M_PI;
    }
}

// The singular poles of the lon/lat grid moved to Greenland (75N 40W) and
// Antarctica: rotation by 40 degrees about z, then 15 degrees about y.
void HostMesh::rotatePoleToGreenland()
{
    const double aw = 40.0 * M_PI / 180.0, bw = 15.0 * M_PI / 180.0;
    for (size_t i = 0; i < vx.size(); ++i) {
        const double x = std::cos(vy[i]) * std::cos(vx[i]);
        const double y = std::cos(vy[i]) * std::sin(vx[i]);
        const double z = std::sin(vy[i]);
        const double x1 = std::cos(aw) * x - std::sin(aw) * y;
        const double y1 = std::sin(aw) * x + std::cos(aw) * y;
        const double z1 = z;
        const double x2 = std::cos(bw) * x1 - std::sin(bw) * z1;
        const double y2 = y1;
        const double z2 = std::sin(bw) * x1 + std::cos(bw) * z1;
        vy[i] = std::asin(z2);
        vx[i] = std::atan2(y2, x2);
    }
}

// Bretschneider's formula for the quadrilateral area (ParametricMesh.hpp:276-295).
double HostMesh::area(size_t e) const
{
    const size_t n0 = (e / nx) * (nx + 1) + (e % nx);
    auto d2 = [&](size_t a, size_t b) {
        const double dx = vx[a] - vx[b], dy = vy[a] - vy[b];
        return dx * dx + dy * dy;
    };
    const double lower = d2(n0, n0 + 1), right = d2(n0 + 1, n0 + nx + 2);
    const double top = d2(n0 + nx + 1, n0 + nx + 2), left = d2(n0, n0 + nx + 1);
    const double diag1 = d2(n0, n0 + nx + 2), diag2 = d2(n0 + 1, n0 + nx + 1);
    const double k = right + left - lower - top;
    return 0.25 * std::sqrt(4.0 * diag1 * diag2 - k * k);
}

// A cell gets a Dirichlet edge where its neighbour across that edge is land
// or outside the domain; each list is sorted (ParametricMesh.cpp:228-292).
void HostMesh::dirichletFromMaskAndEdges()
{
    for (auto& d : dirichlet)
        d.clear();
    for (size_t j = 0; j < ny; ++j)
        for (size_t i = 0; i < nx; ++i) {
            const size_t c = i + nx * j;
            if (!ice[c])
                continue;
            if (j == 0 || !ice[c - nx])
                dirichlet[0].push_back(c);
            if (i == nx - 1 || !ice[c + 1])
                dirichlet[1].push_back(c);
            if (j == ny - 1 || !ice[c + nx])
                dirichlet[2].push_back(c);
            if (i == 0 || !ice[c - 1])
                dirichlet[3].push_back(c);
        }
    // row-major generation order is already ascending
}

// ---------------------------------------------------------------------------
// Small dense algebra
// ---------------------------------------------------------------------------
namespace {

// Inverse by LU factorisation with partial pivoting; false if singular.
bool luInverse(int n, const double* A, double* out)
{
    double lu[64];
    int piv[8];
    std::memcpy(lu, A, sizeof(double) * n * n);
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = std::fabs(lu[k * n + k]);
        for (int r = k + 1; r < n; ++r)
            if (std::fabs(lu[r * n + k]) > best) {
                best = std::fabs(lu[r * n + k]);
                p = r;
            }
        if (best == 0.0)
            return false;
        piv[k] = p;
        if (p != k)
            for (int c = 0; c < n; ++c)
                std::swap(lu[k * n + c], lu[p * n + c]);
        for (int r = k + 1; r < n; ++r) {
            lu[r * n + k] /= lu[k * n + k];
            for (int c = k + 1; c < n; ++c)
                lu[r * n + c] -= lu[r * n + k] * lu[k * n + c];
        }
    }
    for (int col = 0; col < n; ++col) {
        double x[8];
        for (int i = 0; i < n; ++i)
            x[i] = (i == col) ? 1.0 : 0.0;
        for (int k = 0; k < n; ++k)
            if (piv[k] != k)
                std::swap(x[k], x[piv[k]]);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < i; ++k)
                x[i] -= lu[i * n + k] * x[k];
        for (int i = n - 1; i >= 0; --i) {
            for (int k = i + 1; k < n; ++k)
                x[i] -= lu[i * n + k] * x[k];
            x[i] /= lu[i * n + i];
        }
        for (int i = 0; i < n; ++i)
            out[i * n + col] = x[i];
    }
    return true;
}

// Geometry of one element at a Q x Q rule: the derivatives of the bilinear
// map T (dT/dxi in rows 0..1 of dxi, dT/deta in dxe) and J = det(dT).
struct Geom {
    double dxi[2][16], deta[2][16], J[16];
    double cl[16], sl[16]; // cos / sin of the latitude at the Gauss points (spherical)
    bool spherical;
};
void geometry(const HostMesh& m, size_t e, int Q, Geom& g)
{
    const Basis& b = basis();
    double c[4][2];
    m.elementCoords(e, c);
    g.spherical = m.spherical;
    for (int q = 0; q < Q * Q; ++q) {
        double lat = 0;
        for (int k = 0; k < 4; ++k)
            lat += c[k][1] * b.phi(1, k, Q, q);
        g.cl[q] = std::cos(lat);
        g.sl[q] = std::sin(lat);
        for (int r = 0; r < 2; ++r) {
            double sx = 0, sy = 0;
            for (int k = 0; k < 4; ++k) {
                sx += c[k][r] * b.phix(1, k, Q, q);
                sy += c[k][r] * b.phiy(1, k, Q, q);
            }
            g.dxi[r][q] = sx;
            g.deta[r][q] = sy;
        }
        g.J[q] = g.dxi[0][q] * g.deta[1][q] - g.dxi[1][q] * g.deta[0][q];
    }
}

// Inverse of the DG mass matrix M_ij = sum_q psi_i psi_j w_q J_q (times
// cos(lat_q) on a spherical mesh: ParametricTools.hpp:109-153, 189-202).
void inverseMass(const Geom& g, int dg, double* inv)
{
    const Basis& b = basis();
    const int Q = gaussPoints1d(dg);
    double M[64];
    for (int i = 0; i < dg; ++i)
        for (int j = 0; j < dg; ++j) {
            double s = 0;
            for (int q = 0; q < Q * Q; ++q)
                s += g.spherical ? (b.psi(i, Q, q) * (b.weight(Q, q) * g.J[q] * g.cl[q])) * b.psi(j, Q, q)
                                 : (b.psi(i, Q, q) * (b.weight(Q, q) * g.J[q])) * b.psi(j, Q, q);
            M[i * dg + j] = s;
        }
    if (!luInverse(dg, M, inv))
        for (int i = 0; i < dg * dg; ++i)
            inv[i] = NAN;
}

// Advection cell term J dT^{-T} grad(psi_i) w_q (ParametricMap.cpp:13-66).
void cellTerms(const Geom& g, int dg, size_t N, size_t e, std::vector<double>& cx,
    std::vector<double>& cy)
{
    const Basis& b = basis();
    const int Q = gaussPoints1d(dg), QQ = Q * Q;
    for (int i = 0; i < dg; ++i)
        for (int q = 0; q < QQ; ++q) {
            const double w = b.weight(Q, q);
            const double xi0 = g.dxi[0][q] * w, xi1 = g.dxi[1][q] * w;
            const double et0 = g.deta[0][q] * w, et1 = g.deta[1][q] * w;
            cx[(i * QQ + q) * N + e] = b.psix(i, Q, q) * et1 - b.psiy(i, Q, q) * xi1;
            cy[(i * QQ + q) * N + e] = b.psiy(i, Q, q) * xi0 - b.psix(i, Q, q) * et0;
        }
}

template <class F> void parallelFor(size_t n, unsigned threads, F&& f)
{
    if (threads == 0)
        threads = std::max(1u, std::thread::hardware_concurrency());
    threads = static_cast<unsigned>(std::min<size_t>(threads, std::max<size_t>(1, n / 256)));
    if (threads <= 1) {
        f(size_t(0), n);
        return;
    }
    std::vector<std::thread> pool;
    const size_t chunk = (n + threads - 1) / threads;
    for (unsigned t = 0; t < threads; ++t) {
        const size_t lo = t * chunk, hi = std::min(n, lo + chunk);
        if (lo >= hi)
            break;
        pool.emplace_back([&f, lo, hi] { f(lo, hi); });
    }
    for (auto& th : pool)
        th.join();
}

void transportOps(const HostMesh& m, int dg, ElementOps& ops, unsigned threads)
{
    const size_t N = m.nelements();
    const int Q = gaussPoints1d(dg), QQ = Q * Q;
    ops.cellX.assign(size_t(dg) * QQ * N, 0.0);
    ops.cellY.assign(size_t(dg) * QQ * N, 0.0);
    ops.minv.assign(size_t(dg) * dg * N, 0.0);
    if (m.spherical)
        ops.minvP.assign(size_t(dg) * dg * N, 0.0);
    else
        ops.minvP.clear();
    ops.jwA.assign(size_t(QQ) * N, 0.0);
    ops.jw3.assign(9 * N, 0.0);
    const Basis& b = basis();
    parallelFor(N, threads, [&](size_t lo, size_t hi) {
        Geom g, g3;
        double inv[64];
        for (size_t e = lo; e < hi; ++e) {
            geometry(m, e, Q, g);
            cellTerms(g, dg, N, e, ops.cellX, ops.cellY);
            inverseMass(g, dg, inv);
            for (int k = 0; k < dg * dg; ++k) { // transport: M^{-1} / R on a sphere (ParametricMap.cpp:74-79)
                ops.minv[k * N + e] = m.spherical ? inv[k] / kEarthRadius : inv[k];
                if (m.spherical)
                    ops.minvP[k * N + e] = inv[k];
            }
            for (int q = 0; q < QQ; ++q) // CG2DG weights (Interpolations.cpp:100-110)
                ops.jwA[q * N + e] = m.spherical ? g.J[q] * b.weight(Q, q) * g.cl[q] : g.J[q] * b.weight(Q, q);
            geometry(m, e, 3, g3);
            for (int q = 0; q < 9; ++q) // MeanValue / DG8 CG2DG weights (Tools.hpp:28-36)
                ops.jw3[q * N + e] = m.spherical ? g3.J[q] * b.weight(3, q) * g3.cl[q] : g3.J[q] * b.weight(3, q);
        }
    });
}

} // namespace

bool buildAffineStressOps(const HostMesh& m, const ElementOps& ops, size_t ld, double tol,
    AffineStressOps& out, unsigned threads)
{
    const size_t N = m.nelements();
    if (m.spherical || N == 0 || ops.gx.size() != 81 * N || ld < N)
        return false;
    // the unit-square operators: one element with vertices (0,0) (1,0) (0,1) (1,1)
    HostMesh u;
    u.nx = u.ny = 1;
    u.vx = { 0.0, 1.0, 0.0, 1.0 };
    u.vy = { 0.0, 0.0, 1.0, 1.0 };
    u.ice = { 1 };
    ElementOps uo;
    buildElementOps(u, ops.dg, false, uo, 1);
    for (int r = 0; r < 81; ++r) {
        out.ref[0][r] = uo.gx[r];
        out.ref[1][r] = uo.gy[r];
        out.ref[2][r] = uo.a1[r];
        out.ref[3][r] = uo.a2[r];
    }
    out.ld = ld;
    out.coef.assign(5 * ld, 0.f);
    std::mutex mu;
    out.worst = 0;
    parallelFor(N, threads, [&](size_t lo, size_t hi) {
        double worst = 0;
        Geom g;
        for (size_t e = lo; e < hi; ++e) {
            geometry(m, e, 3, g);
            const int qc = 4; // the element centre
            const double J = g.J[qc];
            const double c[5] = { g.deta[1][qc], -g.dxi[1][qc], -g.deta[0][qc], g.dxi[0][qc], 1.0 / J };
            const std::vector<double>* exact[4] = { &ops.gx, &ops.gy, &ops.a1, &ops.a2 };
            for (int b = 0; b < 4; ++b) {
                const double s = b < 2 ? c[4] : 1.0;
                const double k0 = (b % 2 == 0) ? c[0] : c[2], k1 = (b % 2 == 0) ? c[1] : c[3];
                const int r0 = b < 2 ? 0 : 2;
                double mx = 0, diff = 0;
                for (int r = 0; r < 81; ++r) {
                    const double x = (*exact[b])[size_t(r) * N + e];
                    const double y = s * (k0 * out.ref[r0][r] + k1 * out.ref[r0 + 1][r]);
                    mx = std::max(mx, std::fabs(x));
                    diff = std::max(diff, std::fabs(x - y));
                }
                if (mx > 0)
                    worst = std::max(worst, diff / mx);
            }
            for (int k = 0; k < 5; ++k)
                out.coef[k * ld + e] = static_cast<float>(c[k]);
        }
        std::lock_guard<std::mutex> lk(mu);
        out.worst = std::max(out.worst, worst);
    });
    return out.worst <= tol;
}

bool buildAffineBbmOps(const HostMesh& m, const ElementOps& ops, double tol, AffineBbmOps& out, unsigned threads)
{
    const size_t N = m.nelements();
    const int dg = ops.dg;
    if (m.spherical || N == 0 || ops.w.size() != 72 * N || ops.wdam.size() != size_t(dg) * 9 * N
        || ops.d1.size() != 72 * N || ops.d2.size() != 72 * N || dg * 9 > 72)
        return false;
    HostMesh u;
    u.nx = u.ny = 1;
    u.vx = { 0.0, 1.0, 0.0, 1.0 };
    u.vy = { 0.0, 0.0, 1.0, 1.0 };
    u.ice = { 1 };
    ElementOps uo;
    buildElementOps(u, dg, true, uo, 1);
    for (int r = 0; r < 72; ++r) {
        out.w[r] = uo.w[r];
        out.dxi[r] = uo.d1[r];  // on the unit square c0 = 1, c1 = 0
        out.deta[r] = uo.d2[r]; // and c2 = 0, c3 = 1
    }
    for (int r = 0; r < dg * 9; ++r)
        out.wdam[r] = uo.wdam[r];
    std::mutex mu;
    out.worst = 0;
    parallelFor(N, threads, [&](size_t lo, size_t hi) {
        double worst = 0;
        Geom g;
        auto rel = [&](const std::vector<double>& exact, size_t rows, auto rebuilt, size_t e) {
            double mx = 0, diff = 0;
            for (size_t r = 0; r < rows; ++r) {
                const double x = exact[r * N + e];
                mx = std::max(mx, std::fabs(x));
                diff = std::max(diff, std::fabs(x - rebuilt(r)));
            }
            return mx > 0 ? diff / mx : 0.0;
        };
        for (size_t e = lo; e < hi; ++e) {
            geometry(m, e, 3, g);
            const int qc = 4;
            const double c[4] = { g.deta[1][qc], -g.dxi[1][qc], -g.deta[0][qc], g.dxi[0][qc] };
            worst = std::max(worst, rel(ops.w, 72, [&](size_t r) { return out.w[r]; }, e));
            worst = std::max(worst, rel(ops.wdam, size_t(dg) * 9, [&](size_t r) { return out.wdam[r]; }, e));
            worst = std::max(worst, rel(ops.d1, 72, [&](size_t r) { return c[0] * out.dxi[r] + c[1] * out.deta[r]; }, e));
            worst = std::max(worst, rel(ops.d2, 72, [&](size_t r) { return c[2] * out.dxi[r] + c[3] * out.deta[r]; }, e));
        }
        std::lock_guard<std::mutex> lk(mu);
        out.worst = std::max(out.worst, worst);
    });
    return out.worst <= tol;
}

bool buildAffineTransportOps(const HostMesh& m, const ElementOps& ops, double tol, double offDiagTol,
    AffineTransportOps& out, unsigned threads)
{
    const size_t N = m.nelements();
    const int dg = ops.dg;
    const int Q = gaussPoints1d(dg), QQ = Q * Q;
    out.dg = dg;
    if (m.spherical || N == 0 || (dg != 1 && dg != 3 && dg != 6) || ops.minv.size() != size_t(dg) * dg * N
        || ops.cellX.size() != size_t(dg) * QQ * N)
        return false;
    // the unit square's cell operators: U_xi and U_eta
    HostMesh u;
    u.nx = u.ny = 1;
    u.vx = { 0.0, 1.0, 0.0, 1.0 };
    u.vy = { 0.0, 0.0, 1.0, 1.0 };
    u.ice = { 1 };
    ElementOps uo;
    buildTransportOps(u, dg, uo, 1);
    for (int r = 0; r < dg * QQ; ++r) {
        out.ref[0][r] = uo.cellX[r];
        out.ref[1][r] = uo.cellY[r];
    }
    out.minvDiag.assign(size_t(dg) * N, 0.0);
    std::mutex mu;
    out.worstCell = 0;
    out.worstOffDiag = 0;
    parallelFor(N, threads, [&](size_t lo, size_t hi) {
        double wc = 0, wo = 0;
        Geom g;
        for (size_t e = lo; e < hi; ++e) {
            geometry(m, e, 3, g);
            const int qc = 4; // the element centre, as for the stress coefficients
            const double c[4] = { g.deta[1][qc], -g.dxi[1][qc], -g.deta[0][qc], g.dxi[0][qc] };
            for (int b = 0; b < 2; ++b) {
                const std::vector<double>& exact = b == 0 ? ops.cellX : ops.cellY;
                const double k0 = b == 0 ? c[0] : c[2], k1 = b == 0 ? c[1] : c[3];
                double mx = 0, diff = 0;
                for (int r = 0; r < dg * QQ; ++r) {
                    const double x = exact[size_t(r) * N + e];
                    mx = std::max(mx, std::fabs(x));
                    diff = std::max(diff, std::fabs(x - (k0 * out.ref[0][r] + k1 * out.ref[1][r])));
                }
                if (mx > 0)
                    wc = std::max(wc, diff / mx);
            }
            double dmax = 0, omax = 0;
            for (int i = 0; i < dg; ++i)
                for (int j = 0; j < dg; ++j) {
                    const double x = std::fabs(ops.minv[size_t(i * dg + j) * N + e]);
                    if (i == j)
                        dmax = std::max(dmax, x);
                    else
                        omax = std::max(omax, x);
                }
            wo = std::max(wo, dmax > 0 ? omax / dmax : (omax > 0 ? INFINITY : 0.0));
            for (int i = 0; i < dg; ++i)
                out.minvDiag[size_t(i) * N + e] = ops.minv[size_t(i * dg + i) * N + e];
        }
        std::lock_guard<std::mutex> lk(mu);
        out.worstCell = std::max(out.worstCell, wc);
        out.worstOffDiag = std::max(out.worstOffDiag, wo);
    });
    return out.worstCell <= tol && out.worstOffDiag <= offDiagTol;
}

void buildTransportOps(const HostMesh& m, int dg, ElementOps& ops, unsigned threads)
{
    ops.dg = dg;
    ops.N = m.nelements();
    transportOps(m, dg, ops, threads);
}

void buildElementOps(const HostMesh& m, int dg, bool stressTransport, ElementOps& ops,
    unsigned threads)
{
    const Basis& b = basis();
    const size_t N = m.nelements();
    ops.dg = dg;
    ops.N = N;
    transportOps(m, dg, ops, threads);

    ops.gx.assign(81 * N, 0.0);
    ops.gy.assign(81 * N, 0.0);
    ops.w.assign(72 * N, 0.0);
    ops.a1.assign(81 * N, 0.0);
    ops.a2.assign(81 * N, 0.0);
    ops.d1.assign(72 * N, 0.0);
    ops.d2.assign(72 * N, 0.0);
    ops.dxssh.assign(16 * N, 0.0);
    ops.dyssh.assign(16 * N, 0.0);
    const bool sph = m.spherical;
    if (sph) {
        ops.gm.assign(81 * N, 0.0);
        ops.a3.assign(81 * N, 0.0);
        ops.dm.assign(72 * N, 0.0);
    } else {
        ops.gm.clear();
        ops.a3.clear();
        ops.dm.clear();
    }
    if (stressTransport) {
        ops.cellX8.assign(72 * N, 0.0);
        ops.cellY8.assign(72 * N, 0.0);
        ops.minv8.assign(64 * N, 0.0);
        if (sph)
            ops.minv8P.assign(64 * N, 0.0);
        ops.wdam.assign(size_t(dg) * 9 * N, 0.0);
        ops.hsize.assign(N, 0.0);
    }
    parallelFor(N, threads, [&](size_t lo, size_t hi) {
        Geom g;
        double im8[64], imd[64];
        for (size_t e = lo; e < hi; ++e) {
            geometry(m, e, 3, g);
            // Transformed gradients of the CG2 / CG1 basis, weighted
            // (ParametricMap.cpp:232-263): gx_j(q) = [J dT^{-T} grad phi_j]_x w_q
            double dx2[9][9], dy2[9][9], dx1[4][9], dy1[4][9];
            for (int q = 0; q < 9; ++q) {
                const double w = b.weight(3, q);
                const double xi0 = g.dxi[0][q] * w, xi1 = g.dxi[1][q] * w;
                const double et0 = g.deta[0][q] * w, et1 = g.deta[1][q] * w;
                for (int j = 0; j < 9; ++j) {
                    dx2[j][q] = b.phix(2, j, 3, q) * et1 - b.phiy(2, j, 3, q) * xi1;
                    dy2[j][q] = b.phiy(2, j, 3, q) * xi0 - b.phix(2, j, 3, q) * et0;
                }
                for (int j = 0; j < 4; ++j) {
                    dx1[j][q] = b.phix(1, j, 3, q) * et1 - b.phiy(1, j, 3, q) * xi1;
                    dy1[j][q] = b.phiy(1, j, 3, q) * xi0 - b.phix(1, j, 3, q) * et0;
                }
            }
            // divS1/divS2 (9 x 8): (grad phi_j, psi_k).  On a sphere
            // (ParametricMap.cpp:298-347) the lat-derivative carries cos(lat),
            // divM = (phi_j, J sin(lat) w psi_k) is added and all is / R.
            double D1[9][8], D2[9][8], DM[9][8];
            for (int j = 0; j < 9; ++j)
                for (int k = 0; k < 8; ++k) {
                    double s1 = 0, s2 = 0;
                    for (int q = 0; q < 9; ++q) {
                        s1 += dx2[j][q] * b.psi(k, 3, q);
                        s2 += (sph ? dy2[j][q] * g.cl[q] : dy2[j][q]) * b.psi(k, 3, q);
                    }
                    if (sph) {
                        s1 /= kEarthRadius;
                        s2 /= kEarthRadius;
                        double s3 = 0;
                        for (int q = 0; q < 9; ++q)
                            s3 += (b.phi(2, j, 3, q) * (g.J[q] * g.sl[q] * b.weight(3, q))) * b.psi(k, 3, q);
                        DM[j][k] = s3 / kEarthRadius;
                        ops.dm[(j * 8 + k) * N + e] = DM[j][k];
                    }
                    D1[j][k] = s1;
                    D2[j][k] = s2;
                    ops.d1[(j * 8 + k) * N + e] = s1;
                    ops.d2[(j * 8 + k) * N + e] = s2;
                }
            // dX_SSH / dY_SSH (4 x 4)
            for (int i = 0; i < 4; ++i)
                for (int j = 0; j < 4; ++j) {
                    double s1 = 0, s2 = 0;
                    for (int q = 0; q < 9; ++q) {
                        s1 += dx1[i][q] * b.phi(1, j, 3, q);
                        s2 += (sph ? dy1[i][q] * g.cl[q] : dy1[i][q]) * b.phi(1, j, 3, q);
                    }
                    ops.dxssh[(i * 4 + j) * N + e] = sph ? s1 / kEarthRadius : s1;
                    ops.dyssh[(i * 4 + j) * N + e] = sph ? s2 / kEarthRadius : s2;
                }
            inverseMass(g, 8, im8);
            // iMgrad = M8^{-1} divS^T (8 x 9); the strain at the Gauss points
            // is psi(q)^T iMgrad u, so the device stores the composite
            // G(q, j) = sum_k psi_k(q) iMgrad(k, j) (9 x 9).
            double iGx[8][9], iGy[8][9], iGm[8][9];
            for (int k = 0; k < 8; ++k)
                for (int j = 0; j < 9; ++j) {
                    double s1 = 0, s2 = 0, s3 = 0;
                    for (int mm = 0; mm < 8; ++mm) {
                        s1 += im8[k * 8 + mm] * D1[j][mm];
                        s2 += im8[k * 8 + mm] * D2[j][mm];
                        if (sph)
                            s3 += im8[k * 8 + mm] * DM[j][mm];
                    }
                    iGx[k][j] = s1;
                    iGy[k][j] = s2;
                    iGm[k][j] = s3; // iMM = M8^{-1} divM^T (spherical strain term)
                }
            for (int q = 0; q < 9; ++q)
                for (int j = 0; j < 9; ++j) {
                    double s1 = 0, s2 = 0, s3 = 0;
                    for (int k = 0; k < 8; ++k) {
                        s1 += b.psi(k, 3, q) * iGx[k][j];
                        s2 += b.psi(k, 3, q) * iGy[k][j];
                        if (sph)
                            s3 += b.psi(k, 3, q) * iGm[k][j];
                    }
                    ops.gx[(q * 9 + j) * N + e] = s1;
                    ops.gy[(q * 9 + j) * N + e] = s2;
                    if (sph)
                        ops.gm[(q * 9 + j) * N + e] = s3;
                }
            // iMJwPSI = M8^{-1} (psi_k(q) w_q J_q)   (8 x 9)
            double W[8][9];
            for (int k = 0; k < 8; ++k)
                for (int q = 0; q < 9; ++q) {
                    double s = 0;
                    for (int mm = 0; mm < 8; ++mm)
                        s += im8[k * 8 + mm] * (b.psi(mm, 3, q) * (b.weight(3, q) * g.J[q]));
                    W[k][q] = s;
                    ops.w[(k * 9 + q) * N + e] = s;
                }
            // divergence of a Gauss-point stress increment: A = divS iMJwPSI (9 x 9)
            for (int j = 0; j < 9; ++j)
                for (int q = 0; q < 9; ++q) {
                    double s1 = 0, s2 = 0, s3 = 0;
                    for (int k = 0; k < 8; ++k) {
                        s1 += D1[j][k] * W[k][q];
                        s2 += D2[j][k] * W[k][q];
                        if (sph)
                            s3 += DM[j][k] * W[k][q];
                    }
                    ops.a1[(j * 9 + q) * N + e] = s1;
                    ops.a2[(j * 9 + q) * N + e] = s2;
                    if (sph)
                        ops.a3[(j * 9 + q) * N + e] = s3;
                }
            if (stressTransport) {
                cellTerms(g, 8, N, e, ops.cellX8, ops.cellY8);
                for (int k = 0; k < 64; ++k) { // the DG8 stress transport's M^{-1} (/ R on a sphere)
                    ops.minv8[k * N + e] = sph ? im8[k] / kEarthRadius : im8[k];
                    if (sph)
                        ops.minv8P[k * N + e] = im8[k];
                }
                // iMJwPSI_dam = M_dg^{-1} (psi_k(q) w_q J_q) at the 3x3 rule
                Geom ga;
                geometry(m, e, gaussPoints1d(dg), ga);
                inverseMass(ga, dg, imd);
                for (int k = 0; k < dg; ++k)
                    for (int q = 0; q < 9; ++q) {
                        double s = 0;
                        for (int mm = 0; mm < dg; ++mm)
                            s += imd[k * dg + mm] * (b.psi(mm, 3, q) * (b.weight(3, q) * g.J[q]));
                        ops.wdam[(k * 9 + q) * N + e] = s;
                    }
                ops.hsize[e] = std::sqrt(m.area(e));
            }
        }
    });

    // Lumped masses: CG2 from a 4x4 rule, CG1 from a 2x2 rule, assembled in
    // even-rows-then-odd-rows order (ParametricMap.cpp:94-206).
    const size_t s2 = 2 * m.nx + 1, s1 = m.nx + 1;
    ops.lumped2.assign(s2 * (2 * m.ny + 1), 0.0);
    ops.lumped1.assign(s1 * (m.ny + 1), 0.0);
    Geom g4, g2;
    for (size_t p = 0; p < 2; ++p)
        for (size_t iy = p; iy < m.ny; iy += 2)
            for (size_t ix = 0; ix < m.nx; ++ix) {
                const size_t e = m.nx * iy + ix;
                geometry(m, e, 4, g4);
                const size_t n0 = 2 * iy * s2 + 2 * ix;
                for (int j = 0; j < 9; ++j) {
                    double s = 0;
                    for (int q = 0; q < 16; ++q)
                        s += b.phi(2, j, 4, q) * (sph ? g4.J[q] * b.weight(4, q) * g4.cl[q] : g4.J[q] * b.weight(4, q));
                    ops.lumped2[n0 + (j % 3) + (j / 3) * s2] += s;
                }
            }
    for (size_t p = 0; p < 2; ++p)
        for (size_t iy = p; iy < m.ny; iy += 2)
            for (size_t ix = 0; ix < m.nx; ++ix) {
                const size_t e = m.nx * iy + ix;
                geometry(m, e, 2, g2);
                const size_t n0 = iy * s1 + ix;
                for (int j = 0; j < 4; ++j) {
                    double s = 0;
                    for (int q = 0; q < 4; ++q)
                        s += b.phi(1, j, 2, q) * (sph ? g2.J[q] * b.weight(2, q) * g2.cl[q] : g2.J[q] * b.weight(2, q));
                    ops.lumped1[n0 + (j % 2) + (j / 2) * s1] += s;
                }
            }
}

std::string buildBoundaryFlags(const HostMesh& m, BoundaryFlags& f)
{
    const size_t N = m.nelements(), nx = m.nx, ny = m.ny;
    f.cellSeg.assign(N, 0);
    f.edgeXCount.assign(nx * (ny + 1), 0);
    f.edgeYCount.assign((nx + 1) * ny, 0);
    const size_t s2 = 2 * nx + 1;
    f.cg2Dirichlet.assign(s2 * (2 * ny + 1), 0);
    for (int seg = 0; seg < 4; ++seg)
        for (size_t c : m.dirichlet[seg]) {
            if (c >= N)
                return "dirichlet element id out of range";
            if (f.cellSeg[c] & (1u << seg))
                return "duplicate dirichlet entry";
            f.cellSeg[c] |= static_cast<uint8_t>(1u << seg);
            const size_t ix = c % nx, iy = c / nx;
            // edge doubled by reinitnormalvelocity (DGTransport.cpp:234-251)
            if (seg == 0)
                f.edgeXCount[nx * iy + ix]++;
            else if (seg == 1)
                f.edgeYCount[(nx + 1) * iy + ix + 1]++;
            else if (seg == 2)
                f.edgeXCount[nx * (iy + 1) + ix]++;
            else
                f.edgeYCount[(nx + 1) * iy + ix]++;
            // CG2 nodes zeroed by dirichletZero (CGDynamicsKernel.cpp:401-437)
            const size_t base = 2 * iy * s2 + 2 * ix;
            for (size_t j = 0; j < 3; ++j) {
                size_t idx;
                if (seg == 0)
                    idx = base + j;
                else if (seg == 1)
                    idx = base + 2 + s2 * j;
                else if (seg == 2)
                    idx = base + 2 * s2 + j;
                else
                    idx = base + s2 * j;
                f.cg2Dirichlet[idx] = 1;
            }
        }
    // periodic entries in CSR by cell, each cell listing the entries that
    // touch it in the reference's order
    std::vector<std::vector<int>> byCell(N);
    for (size_t i = 0; i < m.periodic.size(); ++i) {
        const auto& p = m.periodic[i];
        if (p[0] > 1 || p[1] >= N || p[2] >= N)
            return "bad periodic entry";
        if (p[0] == 0 && p[3] >= nx * (ny + 1))
            return "bad periodic X-edge id";
        if (p[0] == 1 && p[3] >= (nx + 1) * ny)
            return "bad periodic Y-edge id";
        byCell[p[1]].push_back(static_cast<int>(i));
        if (p[2] != p[1])
            byCell[p[2]].push_back(static_cast<int>(i));
    }
    f.perPtr.assign(N + 1, 0);
    f.perEntry.clear();
    for (size_t c = 0; c < N; ++c) {
        f.perPtr[c] = static_cast<int>(f.perEntry.size() / 4);
        for (int i : byCell[c])
            for (int k = 0; k < 4; ++k)
                f.perEntry.push_back(static_cast<int>(m.periodic[i][k]));
    }
    f.perPtr[N] = static_cast<int>(f.perEntry.size() / 4);
    return "";
}

} // namespace nsdg
