// JSON-case front end: the reference's case files (src/driver/driver.cpp,
// buildSolverJson :1545 and the parsers it calls, :531-705, :707-868, :946-1060)
// read into the flat mesh / options / sources / probes tables of this library.
//
// Supported: gmsh 2.2 ASCII meshes with first-order tetrahedra (physical tags
// as attributes), uniform refinement, materials by volume tag (relative
// permittivity / permeability / bulk conductivity in S/m), PEC / PMC / SMA
// boundaries by surface tag (interior when the tagged faces lie between two
// elements), Gaussian and resonant-mode initial fields, Gaussian and modulated
// Gaussian plane waves on a tagged TF/SF surface (explicit or automatic delay),
// point probes and near-to-far ("rcssurface" / "farfield") surfaces by tag.
// Rejected with a clear error: SGBC boundaries, dipole and Bessel sources,
// curved (second-order) elements, 1D/2D meshes.
#pragma once
#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/dgtd_gb300.h"
#include "sgbc.hpp"

namespace dgtd {

// Minimal JSON value (objects keep insertion order).
struct Json {
    enum Type { Null, Bool, Number, String, Array, Object } type = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json* find(const std::string& key) const;
    bool has(const std::string& key) const { return find(key) != nullptr; }
    const Json& at(const std::string& key) const;   // throws if missing
    double number() const;
    int integer() const;
    const std::string& string() const;
    std::vector<double> numbers() const;             // array of numbers
};

Json parse_json(const std::string& text);

struct GmshMesh {
    std::vector<double> xyz;           // [nv][3]
    std::vector<int32_t> tets;         // [ne][4] vertex indices
    std::vector<int32_t> tet_tag;      // physical tag per tet
    std::vector<int32_t> tris;         // [nt][3]
    std::vector<int32_t> tri_tag;
    // curved second-order tetrahedra: tet index and [6][3] edge-node positions on the edges
    // (0,1) (0,2) (0,3) (1,2) (1,3) (2,3) of the tet's corner order
    std::vector<int32_t> curved_tets;
    std::vector<double> curved_edges;
};

GmshMesh read_gmsh22(const std::string& path);
// One level of uniform refinement: every tetrahedron into 8 (edge midpoints), every
// tagged triangle into 4, tags inherited.
void refine_uniform(GmshMesh& m);

struct CaseInitialField {
    int field = 0;                  // 0 electric, 1 magnetic
    int kind = 0;                   // 0 gaussian, 1 resonant mode, 2 besselj6_2D, 3 besselj6_3D
    double spread = 0.1;
    double center[3] = {0, 0, 0};
    double pol[3] = {0, 0, 1};
    int dimension = 1;
    std::vector<int> modes;
};

struct CaseSurface {
    std::string name;
    std::vector<int> tags;
    int interval = 1;
    std::vector<int32_t> faces;     // [n][3], winding normal pointing away from the region the surface encloses
};

struct Case {
    std::string dir, name;
    // defaults of the reference's SolverOptions / EvolutionOptions (SolverOptions.h:19-24,
    // EvolutionOptions.h:13-16)
    int order = 2;
    double alpha = 1.0;
    double dt = 0.0;                // 0: estimate from cfl
    double final_time = 2.0;
    double cfl = 1.0;
    int integrator = DGTD_RK4;
    std::string evolution_operator = "global";
    // MFEM BasisType of the case's nodal basis: 1 Gauss-Lobatto (the operator's own node set),
    // 0 Gauss-Legendre (the same polynomial space; the runner changes basis at the run's ends)
    int basis_type = 1;
    // mesh
    std::vector<double> vertices;
    std::vector<int32_t> elements;
    std::vector<double> eps, mu, sigma;
    std::vector<int32_t> bdr_faces, bdr_codes, tfsf_faces, int_faces, int_codes;
    // thin-layer (SGBC) boundaries: one stack per "SGBC" boundary entry, and the stack of each
    // interior face given with code DGTD_BC_SGBC (in int_faces order)
    std::vector<SgbcStackSpec> sgbc_stacks;
    std::vector<int32_t> sgbc_face_stack;
    // curved (second-order) elements: ids and [n][10][3] geometry nodes (dgtd_mesh_desc layout)
    std::vector<int32_t> curved_elems;
    std::vector<double> curved_nodes;
    // sources
    std::vector<dgtd_planewave> waves;
    std::vector<CaseInitialField> initial;
    // probes
    std::vector<double> point_pos;  // [n][3]
    std::vector<int> point_interval;   // sampling interval in steps ("steps", or from "saves")
    std::vector<int> point_saves;      // requested number of saves (0: none); the runner turns it
                                       // into an interval once dt is known (probe_interval)
    std::vector<CaseSurface> surfaces;
};

Case load_case(const std::string& json_path);

// Sampling interval of a probe that asked for `saves` samples over a run of final_time with step
// dt (reference ProbesManager::recalculateExportSteps, src/solver/ProbesManager.cpp:578-607, run
// with the solver's dt, Solver.cpp:122): max(1, ceil(final_time / dt) / saves); saves <= 0
// keeps `steps_interval`.
int probe_interval(int saves, int steps_interval, double final_time, double dt);

// Initial field at the nodes (reference SourcesManager::setInitialFields,
// src/solver/SourcesManager.cpp:16-36: nodal projection of InitialField::eval,
// src/components/Sources.cpp:37-57). xyz is [3][n]; returns [6][n].
std::vector<double> case_initial_state(const Case& c, const double* xyz, int64_t n);

}  // namespace dgtd
