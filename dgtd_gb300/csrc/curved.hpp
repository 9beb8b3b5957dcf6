// Second-order (curved) tetrahedra: their rows of the assembled operator, built on the host.
//
// The reference applies its assembled, quadrature-based global operator to curved elements
// (GlobalEvolution; HesthavenEvolution copies those rows for its curved elements,
// src/evolution/HesthavenEvolution.cpp:207-241, 411-435, 538-540). Here each curved element e
// gets dense blocks of dU_e/dt over its own state and each face neighbour's:
//   dU_e/dt = B_0 U_e + sum_f B_(1+f) U_nbr(f),
// from the weak form on the isoparametric map: M_e = int phi phi |J|, the strong-form derivatives
// M_e^-1 int phi d(phi)/dx |J|, and M_e^-1 int_face phi F(u-, u+) dS with the upwind flux F at each
// face point (its own normal and surface measure). Boundary codes and interior sheets fold into
// B_0. The FP64 stage kernel skips these elements and curved_dev.cu applies the blocks.
#pragma once
#include <cstdint>
#include <vector>

#include "mesh.hpp"
#include "refelem.hpp"

namespace dgtd {

struct CurvedRows {
    int Np = 0;
    std::vector<int32_t> elems;    // curved elements (the mesh's order)
    std::vector<int32_t> nbr;      // [n][4] face neighbour or -1
    std::vector<double> blocks;    // [n][5][6 Np][6 Np], row-major: row (component, node), column
                                   // (component, node) of the own state (block 0) or of the
                                   // neighbour across face f (block 1 + f)
};

// Quadrature: collapsed Gauss-Legendre rules with p + 4 points per direction on the element and on
// its faces (faces parametrised from their first element, the lower index).
// Materials come from T.mat, faces from T.nbr / T.fcode (TF/SF faces are refused; SGBC faces get
// no terms here: their flux is the SGBC injection, build_curved_sgbc_face).
CurvedRows build_curved_rows(const MeshTables& T, const RefTet& ref, double alpha);

// Unit normal, out of element e, of its face f at the point with barycentric coordinates l (e's
// vertex order; l[f] = 0), from e's geometry map (second-order or affine).
void element_face_normal(const MeshTables& T, int64_t e, int f, const double* l, double* n);

// The SGBC injection on face f of curved element e: dU_e/dt += Bm U_e + Bp t, t the slab traces
// at e's face nodes (component-major: [6][Nfp], face nodes in e's face order), for the interior
// upwind flux with upwind coefficient alpha. Bm [6 Np][6 Np] and Bp [6 Np][6 Nfp], row-major.
void build_curved_sgbc_face(const MeshTables& T, const RefTet& ref, double alpha, int64_t e, int f,
                            std::vector<double>& Bm, std::vector<double>& Bp);

}  // namespace dgtd
