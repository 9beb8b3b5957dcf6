// Thin-layer boundaries (SGBC): host-side tables.
//
// The reference couples a thin layer stack to the 3D mesh through one 1D DG sub-solver per
// face node pair (SGBCWrapper, src/solver/SolverExtension.cpp:49-559; coupling in
// GlobalEvolution, src/evolution/GlobalEvolution.cpp:48-300, 395-545, 639-1001):
//  - the sub-solver mesh is the stack's layers with max(3, p+1) vacuum ghost segments on each
//    side, SMA at both ends and the stack's optional PEC/PMC/SMA sheets at the ghost/layer
//    interfaces; ghost nodes hold the face-local fields of the pair's two 3D nodes;
//  - it steps with SDIRK33, each implicit solve a dense (I - h A) solve;
//  - every RK stage restarts it from the step's checkpoint and advances it to the stage time,
//    and the face flux of the two 3D elements takes the slab's interface values as the
//    neighbour trace; after the step it advances over the whole step with ghosts interpolated.
//
// Here the sub-solver of a stack is linear with constant coefficients, so a sub-step
// (ghosts set, one SDIRK33 step) is an affine map x <- S(P x + Q g). The maps of a whole stage
// advance are composed once per step size on the host:
//  - stage (ghosts held): the 12 interface values = R x_cp + G g, R 12 x n, G 12 x 12;
//  - finalisation (ghosts interpolated): x = F x_cp + Vo g_old + Vn g_new.
// The device then applies them to all pairs of the stack at once (sgbc.cu).
#pragma once
#include <cstdint>
#include <vector>

#include "mesh.hpp"
#include "refelem.hpp"

namespace dgtd {

struct SgbcLayer {
    double eps = 1.0, mu = 1.0, sigma = 0.0;   // sigma in solver units (S/m x free-space impedance)
    double width = 0.0;                        // mesh units
    int segments = 0, order = 1;
};

struct SgbcStackSpec {
    std::vector<SgbcLayer> layers;
    int left_bc = 0, right_bc = 0;   // 0 transparent, else 1 PEC, 2 PMC, 3 SMA sheet
    double sub_dt = 0.0;             // recommended sub-step (normalised time); <= 0: one sub-step
};

// The largest sub-solver this build factorises densely (the reference's dense-solve limit,
// GlobalEvolution.h:102-107; above it the reference iterates with GMRES).
constexpr int64_t kSgbcMaxDofs = 600;

struct SgbcStack1D {
    SgbcStackSpec spec;
    int p = 1, Np1 = 2, nghost = 3;
    int64_t K1 = 0, local = 0, n = 0;   // segments, nodes per component, 6 * local
    int64_t idx_left = 0, idx_right = 0;
    std::vector<double> A;              // [n][n] sub-solver operator
};

// Builds the sub-solver mesh and its operator (nodal DG, upwind alpha 1). Throws
// std::invalid_argument on invalid layers or a sub-solver above kSgbcMaxDofs.
SgbcStack1D build_sgbc_stack(const SgbcStackSpec& spec);

// Number of sub-steps over span: ceil(span / sub_dt) when 0 < sub_dt < span, else 1.
int sgbc_nsteps(double sub_dt, double span);

struct SgbcStageMap {
    std::vector<double> R;   // [12][n]: rows = left interface E,H then right interface E,H
    std::vector<double> G;   // [12][12]
};
struct SgbcFinalMap {
    std::vector<double> FT;  // [n][n] transposed: FT[j * n + i] = F[i][j]
    std::vector<double> Vo;  // [n][12]
    std::vector<double> Vn;  // [n][12]
};

// nsteps sub-steps of span / nsteps each with the ghosts held at g.
SgbcStageMap sgbc_stage_map(const SgbcStack1D& S, double span, int nsteps);
// nsteps sub-steps with ghosts (1 - a_k) g_old + a_k g_new, a_k = (k + 1) / nsteps.
SgbcFinalMap sgbc_final_map(const SgbcStack1D& S, double span, int nsteps);

// Face node pairs of the SGBC faces and the flux entries of their elements.
struct SgbcLayout {
    std::vector<int32_t> gl, gr, stack;   // per pair: node on the face's first element, its partner
    std::vector<double> rot;              // [pairs][9] global -> face-local (row 0: first element's normal)
    std::vector<int32_t> el_elem;         // elements with SGBC faces (ascending)
    std::vector<int32_t> el_start;        // [n_elems + 1] entry ranges
    std::vector<int32_t> ent_face, ent_role;   // per entry: local face, 0 first side / 1 second side
    std::vector<int32_t> ent_pairs;       // [entries][Nfp] pair of each face node (element's face order)
};

// face_stack: stack of each SGBC face, in the order of MeshTables::sgbc_faces.
SgbcLayout build_sgbc_layout(const MeshTables& T, const RefTet& ref, const std::vector<int32_t>& face_stack,
                             int n_stacks);

// The reference's face rotation (buildFaceRotationMatrix, SolverExtension.h:68-107, 3D).
void sgbc_rotation(const double* normal, double* R);

}  // namespace dgtd
