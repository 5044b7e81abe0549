// nsdg_host.hpp — host-side FP64 precompute for the GB300 dynamics kernel.
//
// The reference builds its geometry once per initialise on the CPU
// (ParametricMesh, ParametricTransportMap, ParametricMomentumMap:
// dynamics/src/ParametricMap.cpp:13-356, dynamics/src/include/ParametricTools.hpp:73-181).
// This file does the same work, in FP64, but emits the per-element operators
// directly in the device layout: structure-of-arrays, one contiguous
// N-element array per matrix entry ("entry-major"), so that thread e of a
// warp reads entry k of element e at base + k*N + e (coalesced).
#pragma once

#include <array>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace nsdg {

// Quadrature (Gauss-Legendre on [0,1]) and the DG / CG2 basis functions the
// reference generates in dynamics/codegeneration/{gaussquadrature,basisfunctions}.py.
struct Basis {
    double gp[5][4] = {};
    double gw[5][4] = {};
    Basis();
    static double dg(int j, double x, double y);
    static double dgdx(int j, double x, double y);
    static double dgdy(int j, double x, double y);
    static double edge(int j, double t);
    static double cg1d(int deg, int j, double x);
    static double cg1ddx(int deg, int j, double x);
    // tables with Gauss point q = gy*Q + gx
    double psi(int j, int Q, int q) const { return dg(j, gp[Q][q % Q], gp[Q][q / Q]); }
    double psix(int j, int Q, int q) const { return dgdx(j, gp[Q][q % Q], gp[Q][q / Q]); }
    double psiy(int j, int Q, int q) const { return dgdy(j, gp[Q][q % Q], gp[Q][q / Q]); }
    double weight(int Q, int q) const { return gw[Q][q % Q] * gw[Q][q / Q]; }
    double phi(int deg, int j, int Q, int q) const;
    double phix(int deg, int j, int Q, int q) const;
    double phiy(int deg, int j, int Q, int q) const;
    double psiEdgeW(int j, int G, int E, int g) const; // PSIe_w
    double psiLagrange(int j, int G, int q) const;     // PSILagrange
};
const Basis& basis();

inline int gaussPoints1d(int dg) { return (dg == 8 || dg == 6) ? 3 : (dg == 3 ? 2 : 1); }
inline int edgeDofs(int dg) { return dg == 1 ? 1 : (dg == 3 ? 2 : 3); }

// Constant tables uploaded to __constant__ memory (layout shared with the
// device code in nsdg_common.cuh).
struct ConstTables {
    double psi[4][8][16];     // [Q][j][q]    DG basis at the Q x Q Gauss points
    double psix[4][8][16];    // unused on device, kept for completeness of the table set
    double psiLag3[8][9];     // PSILagrange<DG,3>[j][q]
    double psie[4][3][3];     // [G][j][g]    edge basis at G Gauss points
    double psiew[4][4][3][8]; // [G][E][g][j] weighted edge traces (PSIe_w)
    double phi2[4][9][16];    // [Q][j][q]    CG2 basis at Q x Q Gauss points
    double gw[5][16];         // [Q][q]       tensor Gauss weights
};
void fillConstTables(ConstTables& t);
// FP32 copies of the tables the FP32 transport reads (same layout)
struct ConstTables32 {
    float psi[4][8][16];
    float psie[4][3][3];
    float psiew[4][4][3][8];
    float phi2[4][9][16];
};

// The structured quad mesh with arbitrary vertex positions (ParametricMesh).
constexpr double kEarthRadius = 6371000.0; // NextsimDynamics.hpp:34

struct HostMesh {
    bool spherical = false;                   // x = lon, y = lat (radians); else Cartesian
    size_t nx = 0, ny = 0;
    std::vector<double> vx, vy;               // (nx+1)*(ny+1) vertices
    std::vector<uint8_t> ice;                 // nx*ny, 1 = ice
    std::array<std::vector<size_t>, 4> dirichlet;  // bottom, right, top, left
    std::vector<std::array<size_t, 4>> periodic;   // {type, c1, c2, edge}
    size_t nelements() const { return nx * ny; }
    // ParametricMesh::dirichletFromMask / dirichletFromEdge (ParametricMesh.cpp:228-272)
    void dirichletFromMaskAndEdges();
    void elementCoords(size_t e, double c[4][2]) const; // longitudes made continuous (spherical)
    double area(size_t e) const; // ParametricMesh.hpp:276-295
    void rotatePoleToGreenland(); // ParametricMesh.hpp:137-157
};

// Element operators in SoA layout (entry-major: [entry][N]).
struct ElementOps {
    int dg = 0;
    size_t N = 0;
    // DG transport of the advected fields (DG comps) and of the stress (8 comps)
    std::vector<double> cellX, cellY, minv;      // dg*Qa^2, dg*Qa^2, dg*dg
    std::vector<double> jwA;                     // Qa^2   J*w at the advection Gauss points
    std::vector<double> cellX8, cellY8, minv8;   // 8*9, 8*9, 64 (BBM stress transport)
    std::vector<double> jw3;                     // 9      J*w at the 3x3 Gauss points
    // spherical meshes: the transport's M^{-1} carries 1 / R, the CG2DG
    // projection's does not (Interpolations.cpp:100-110)
    std::vector<double> minvP, minv8P;           // dg*dg, 64 (empty on Cartesian meshes)
    // momentum (CG2 / DG-stress 8)
    std::vector<double> gx, gy;                  // 81: strain at Gauss points from CG2 nodes
    std::vector<double> w;                       // 72: iMJwPSI[k][q]
    std::vector<double> a1, a2;                  // 81: divS1 iMJwPSI, divS2 iMJwPSI [j][q]
    std::vector<double> d1, d2;                  // 72: divS1[j][k], divS2[j][k]
    std::vector<double> wdam;                    // dg*9: iMJwPSI_dam (BBM)
    std::vector<double> dxssh, dyssh;            // 16: dX_SSH[i][j], dY_SSH[i][j]
    std::vector<double> hsize;                   // 1: sqrt(area)  (BBM)
    // spherical metric terms (empty on Cartesian meshes)
    std::vector<double> gm;                      // 81: the iMM strain term at Gauss points [q][j]
    std::vector<double> a3;                      // 81: divM iMJwPSI [j][q]
    std::vector<double> dm;                      // 72: divM[j][k] (BBM)
    // node arrays
    std::vector<double> lumped2;                 // (2nx+1)(2ny+1)
    std::vector<double> lumped1;                 // (nx+1)(ny+1)
};

// Builds every operator the device needs.  `stressTransport` adds the DG8
// transport operators and damage projection used by the BBM rheology.
// Work is split across `threads` host threads (0 = hardware concurrency).
void buildElementOps(const HostMesh& m, int dg, bool stressTransport, ElementOps& ops,
    unsigned threads = 0);

// Parallelogram (affine) elements.  When every element is a parallelogram,
// its Jacobian is constant and the mEVP stress operators are fixed linear
// combinations of the unit-square ones: with (x_xi, y_xi, x_eta, y_eta) the
// Jacobian entries, J its determinant and
//   c = (y_eta, -y_xi, -x_eta, x_xi, 1/J),
//   G_x = c4 (c0 G_xi + c1 G_eta),   G_y = c4 (c2 G_xi + c3 G_eta),
//   A_1 = c0 A_xi + c1 A_eta,        A_2 = c2 A_xi + c3 A_eta,
// because the transformed gradients are c0 d_xi + c1 d_eta (times 1/J), the
// mass matrix is J M_ref and iMJwPSI does not depend on J
// (ParametricMap.cpp:232-263, ParametricTools.hpp:109-153).  The mixed
// precision path then streams 5 coefficients per element instead of 324
// operator entries.
struct AffineStressOps {
    double ref[4][81] {};          // G_xi [q][j], G_eta [q][j], A_xi [j][q], A_eta [j][q]
    std::vector<float> coef;       // [5][ld]: c0 .. c4 per element (ld >= N, zero padded)
    size_t ld = 0;
    double worst = 0;              // max over elements of |rebuilt - exact| / max |exact| (FP64)
};
// Fills `out` and returns true if the mesh is Cartesian and every element's
// operators, rebuilt from its coefficients in FP64, match `ops` (from
// buildElementOps) within `tol` relative to each operator's largest entry.
bool buildAffineStressOps(const HostMesh& m, const ElementOps& ops, size_t ld, double tol,
    AffineStressOps& out, unsigned threads = 0);

// Parallelogram meshes, BBM: the stress projection iMJwPSI (8 x 9) and the
// damage projection (DG x 9) do not depend on J (M = J M_ref), and the
// divergence operators are divS1 = c0 D_xi + c1 D_eta, divS2 = c2 D_xi +
// c3 D_eta with D_xi[j][k] = sum_q w_q dphi_j/dxi(q) psi_k(q) (and D_eta) on
// the unit square and c the coefficients above.
struct AffineBbmOps {
    double w[72] {};    // iMJwPSI [k][q]
    double wdam[72] {}; // damage projection [k][q], k < dg
    double dxi[72] {};  // D_xi [j][k]
    double deta[72] {}; // D_eta [j][k]
    double worst = 0;   // max relative mismatch of the rebuilt operators (FP64)
};
// Fills `out` and returns true if the mesh is Cartesian, `ops` has the BBM
// operators, and every element's w, wdam, divS1 and divS2 rebuilt from the
// unit square's and its coefficients match `ops` within `tol`.
bool buildAffineBbmOps(const HostMesh& m, const ElementOps& ops, double tol, AffineBbmOps& out,
    unsigned threads = 0);

// Parallelogram meshes, transport: the cell operators of DGTransport
// (J dT^{-T} grad psi_i w_q, ParametricMap.cpp:13-66) are
//   cellX = c0 U_xi + c1 U_eta,   cellY = c2 U_xi + c3 U_eta
// with U_xi[i][q] = w_q dpsi_i/dxi(q), U_eta[i][q] = w_q dpsi_i/deta(q) on
// the unit square and c the coefficients above, and the mass matrix is J
// times the unit square's, which the Legendre basis makes diagonal.
struct AffineTransportOps {
    int dg = 0;
    double ref[2][8 * 16] {};     // U_xi [i * Q^2 + q], U_eta
    std::vector<double> minvDiag; // [dg][N]: the diagonal of each element's M^{-1}
    double worstCell = 0;         // max relative mismatch of the rebuilt cell operators (FP64)
    double worstOffDiag = 0;      // max |off-diagonal| / max |diagonal| of M^{-1} over the elements
};
// Fills `out` and returns true if the mesh is Cartesian, has the transport
// operators of `ops.dg` in {1, 3, 6}, every element's cell operators rebuilt
// from its coefficients match `ops` within `tol` and every M^{-1} is diagonal
// within `offDiagTol` (relative to its largest diagonal entry).
bool buildAffineTransportOps(const HostMesh& m, const ElementOps& ops, double tol, double offDiagTol,
    AffineTransportOps& out, unsigned threads = 0);

// Builds only the transport operators (cellX/Y, minv, jwA, jw3) for a DG
// degree (used by the stand-alone transport handle).
void buildTransportOps(const HostMesh& m, int dg, ElementOps& ops, unsigned threads = 0);

// Node / edge / element flags derived from the Dirichlet and periodic lists.
struct BoundaryFlags {
    std::vector<uint8_t> cellSeg;      // nx*ny: bit s set if the cell is in dirichlet[s]
    std::vector<uint8_t> edgeXCount;   // nx*(ny+1): times the X-edge is doubled
    std::vector<uint8_t> edgeYCount;   // (nx+1)*ny: times the Y-edge is doubled
    std::vector<uint8_t> cg2Dirichlet; // (2nx+1)(2ny+1): node zeroed by dirichletZero
    // periodic entries, CSR by cell: for cell c, entries [ptr[c], ptr[c+1]) of
    // {type, c1, c2, edge} in the reference's processing order
    std::vector<int> perPtr;
    std::vector<int> perEntry;         // 4 ints per entry
};
// Returns "" on success, else a message (e.g. duplicate Dirichlet entry).
std::string buildBoundaryFlags(const HostMesh& m, BoundaryFlags& f);

} // namespace nsdg
