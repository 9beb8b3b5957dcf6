// Reference-element tables for the nodal DG Maxwell operator (FP64, host).
//
// Node set and ordering follow the reference's finite-element space:
// L2_FECollection(p, dim, BasisType::GaussLobatto) (src/solver/Solver.cpp:86,
// src/evolution/HesthavenEvolution.cpp:48). On the tetrahedron the nodes are
// the barycentric blend of 1D Gauss-Lobatto points, enumerated with the first
// barycentric index fastest:
//     for k, for j, for i (i+j+k <= p):  w = g[i]+g[j]+g[k]+g[p-i-j-k],
//     node = (g[i]/w, g[j]/w, g[k]/w)   on the (0,0,0),(1,0,0),(0,1,0),(0,0,1) tet.
// Faces are numbered as in that element family: face f lies opposite vertex f,
// and the nodes of a face are listed in ascending volume-node order, which is
// the order HesthavenEvolutionMethods.cpp:340-349 (assembleEmat, after
// removeZeroColumns) produces.
//
// The matrices themselves are built with the published nodal-DG construction
// of Hesthaven & Warburton, "Nodal Discontinuous Galerkin Methods" (2008):
// orthonormal PKDO Vandermonde V, Dr = Vr V^-1, M^-1 = V V^T, LIFT = V V^T Emat,
// with Emat the reference-triangle face mass (HesthavenEvolution.cpp:53-81,
// 364-366 build the same LIFT from MFEM forms).
#pragma once
#include <cstdint>
#include <vector>

namespace dgtd {

// 1D Gauss-Lobatto points of degree p on [-1, 1], ascending.
std::vector<double> gauss_lobatto(int p);

// Orthonormal Jacobi polynomial P_n^{(a,b)}(x) and its derivative.
double jacobi_p(double x, double alpha, double beta, int n);
double grad_jacobi_p(double x, double alpha, double beta, int n);

struct RefTet {
    int p = 0, Np = 0, Nfp = 0;
    std::vector<double> r, s, t;          // Hesthaven coordinates in [-1,1]^3
    std::vector<double> bary;             // [Np][4] barycentric (l0, l1, l2, l3)
    std::vector<double> Dr, Ds, Dt;       // [Np][Np] row-major
    std::vector<double> Minv;             // [Np][Np] inverse mass on the (-1,1) tet
    std::vector<double> LIFT;             // [Np][4*Nfp]
    std::vector<int> Fmask;               // [4][Nfp] volume node of each face node
    std::vector<double> Vinv;             // [Np][Np] inverse Vandermonde (modal <- nodal)
    std::vector<double> face_w;           // [4][Nfp] face-node quadrature weights on a reference face of area 2
};

struct RefSeg {
    int p = 0, Np = 0;
    std::vector<double> r;                // GLL points on [-1,1]
    std::vector<double> Dr;               // [Np][Np]
    std::vector<double> LIFT;             // [Np][2]
};

RefTet build_ref_tet(int p);

// Values of the Np nodal basis functions at reference point (r, s, t) (Hesthaven
// coordinates): phi_n = sum_m Vinv[m][n] psi_m(r, s, t).
void nodal_basis_at(const RefTet& T, double r, double s, double t, double* phi);
// Their derivatives: dphi[n][0..2] = d phi_n / d (r, s, t).
void nodal_basis_grad_at(const RefTet& T, double r, double s, double t, double* dphi);
// Gauss-Legendre points and weights on [0, 1] (n points, exact to degree 2n - 1).
void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w);
RefSeg build_ref_seg(int p);

// MFEM basis types of the tetrahedron's L2 node sets (the reference's solver_options.basis_type):
// the operator runs on the Gauss-Lobatto set; the Gauss-Legendre set (L2_FECollection(p, 3,
// BasisType::GaussLegendre)) is the same barycentric blend of the p + 1 Gauss-Legendre points of
// (0, 1), enumerated in the same order, with no node on a face.
constexpr int kBasisGaussLegendre = 0;
constexpr int kBasisGaussLobatto = 1;
// Barycentric coordinates [Np][4] (l0, l1, l2, l3) of the order-p nodes of that set.
std::vector<double> tet_node_bary(int p, int basis_type);
// Change of nodal basis on the order-p tetrahedron, [Np][Np] row-major: v_to = M v_from for the
// nodal values of any polynomial of degree p (M[i][j] = phi^from_j at node i of `to`).
std::vector<double> tet_basis_change(int p, int from_basis, int to_basis);

inline int tet_np(int p) { return (p + 1) * (p + 2) * (p + 3) / 6; }
inline int tri_np(int p) { return (p + 1) * (p + 2) / 2; }

// Small dense helpers (row-major).
bool invert_matrix(std::vector<double>& a, int n);   // in place, partial pivoting
void matmul(const double* a, const double* b, double* c, int m, int k, int n);

}  // namespace dgtd
