// Mesh, connectivity and per-element geometry for the DG Maxwell operator.
//
// The reference reads these from an MFEM ParMesh: element attributes carry
// the material (src/components/Model.cpp:145-161), boundary attributes carry
// PEC/PMC/SMA (src/components/Types.h:47-55, src/driver/driver.cpp:870-887),
// and interior boundary attributes mark total-field/scattered-field faces
// (src/components/SubMesher.cpp:359-775) and interior PEC/PMC/SMA sheets
// (src/components/DGOperatorFactory.h:577-675). Here the same information is a
// set of flat tables; connectivity is derived from shared vertex triples.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "refelem.hpp"

namespace dgtd {

// Face codes stored per (element, local face).
enum FaceCode : int32_t {
    FACE_INTERIOR = 0,
    FACE_PEC = 1,
    FACE_PMC = 2,
    FACE_SMA = 3,
    FACE_TFSF_TF = 4,     // interior face, this side is in the total-field region
    FACE_TFSF_SF = 5,     // interior face, this side is in the scattered-field region
    FACE_INT_PEC = 6,     // interior PEC sheet
    FACE_INT_PMC = 7,
    FACE_INT_SMA = 8,
    FACE_OPEN = 9,        // boundary face with no condition: zero jump
    FACE_SGBC = 10,       // interior thin-layer (SGBC) face: no flux in the stage kernels; the SGBC
                          // kernels add the flux with the sub-solver's interface values
};

struct MeshInput {
    int dim = 3;
    std::vector<double> vertices;      // [nv][3]
    std::vector<int32_t> elements;     // [ne][4] (dim 3) or [ne][2] (dim 1)
    std::vector<double> eps, mu, sigma;  // per element; empty means 1, 1, 0
    std::vector<int32_t> bdr_faces;    // [nb][3] (dim 3) or [nb][1] (dim 1) vertex ids
    std::vector<int32_t> bdr_codes;    // [nb] 1 PEC, 2 PMC, 3 SMA, 0 open
    std::vector<int32_t> tfsf_faces;   // [nt][3]: oriented so the winding normal points into the TF side
    std::vector<int32_t> int_faces;    // [ni][3]: interior PEC/PMC/SMA sheets and thin layers
    std::vector<int32_t> int_codes;    // [ni] 1 PEC, 2 PMC, 3 SMA, 4 SGBC
    // second-order (curved) elements: ids and [n][10][3] geometry nodes = the element's corners (its
    // vertex order) then the edge nodes of (0,1) (0,2) (0,3) (1,2) (1,3) (2,3)
    std::vector<int32_t> curved_elems;
    std::vector<double> curved_nodes;
};

// Device-ready tables (host copies).
struct MeshTables {
    int dim = 3, p = 0, Np = 0, Nfp = 0, Nfaces = 4;
    int64_t K = 0;
    std::vector<double> x, y, z;        // [K*Np] node coordinates
    std::vector<double> geo;            // [K][9]  rx ry rz sx sy sz tx ty tz
    std::vector<double> fgeo;           // [K][4][4]  nx ny nz Fscale
    std::vector<double> mat;            // [K][3]  1/eps, 1/mu, sigma/eps
    std::vector<int32_t> vmapP;         // [K][Nfaces][Nfp] global neighbour node (own node on boundaries)
    std::vector<int32_t> fcode;         // [K][Nfaces]
    std::vector<int32_t> nbr;           // [K][Nfaces] neighbour element or -1
    std::vector<int32_t> tfsf_elems;    // elements adjacent to a TF/SF face (unique, ascending)
    std::vector<int32_t> curved_elems;  // curved elements (input order) and their geometry nodes
    std::vector<double> curved_nodes;   // [n][10][3] (MeshInput layout); their DOF nodes lie on the curved map
    std::vector<int32_t> sgbc_faces;    // [n][4] e1 f1 e2 f2 of the SGBC faces, in input order
                                        // (e1 < e2: the face's first element)
    std::vector<int32_t> elem_vertices; // [K][4] vertex ids (input order)
    std::vector<double> vertices;       // [nv][3]
    double min_edge = 0.0;              // smallest edge length
    double dt_scale_min = 0.0;          // min over elements of vol / (sum of face areas / 2)
};

MeshTables build_tables(const MeshInput& in, const RefTet& ref);

// The reference's automatic time step (Solver::estimateTimeStep, src/solver/Solver.cpp:289-345)
// for the 3D evolution operators: base = dtscale_min * rmin * 2/3 * 0.75 * cfl (rmin the smallest
// Gauss-Lobatto spacing on [-1, 1]); global: base / 0.8; maxwell: base; hesthaven:
// cfl / (max Fscale * p^2), Fscale = 2 sJ / J per face. evolution: 0 maxwell, 1 global,
// 2 hesthaven (the reference's EvolutionOperatorType).
double estimate_dt(const MeshTables& T, int p, double cfl, int evolution);

// Structured box [x0,x1]x[y0,y1]x[z0,z1] of n cells per axis, each hex split
// into 6 tetrahedra around its (0,0,0)-(1,1,1) diagonal. Optional hole (cells
// [hole_lo, hole_hi) removed) and TF/SF box (cells [tf_lo, tf_hi) are the
// total-field region).
struct BoxSpec {
    int n[3] = {1, 1, 1};
    double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
    int hole_lo[3] = {0, 0, 0}, hole_hi[3] = {0, 0, 0};
    int tf_lo[3] = {0, 0, 0}, tf_hi[3] = {0, 0, 0};
    int outer_bc = FACE_PEC;
    int hole_bc = FACE_PEC;
};
MeshInput make_box(const BoxSpec& spec);

}  // namespace dgtd
