// C ABI of the JSON-case front end: load a reference case file and run it on the GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <limits>
#include <chrono>
#include <cstdio>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/dgtd_gb300.h"
#include "jsoncase.hpp"
#include "mesh.hpp"
#include "refelem.hpp"

namespace dgtd {
int set_last_error(int code, const std::string& msg);   // capi.cu
}

struct dgtd_case {
    dgtd::Case c;
};

namespace {

int cfail(int code, const std::string& msg) { return dgtd::set_last_error(code, msg); }

bool unsupported(const std::string& m)
{
    return m.find("not supported") != std::string::npos;
}

// Raises with the library's last error message on a non-OK status.
void ok(int rc, const char* what)
{
    if (rc != DGTD_OK) throw std::runtime_error(std::string(what) + ": " + dgtd_last_error());
}

}  // namespace

extern "C" {

int dgtd_case_load(const char* json_path, dgtd_case** out)
{
    if (!json_path || !out) return cfail(DGTD_ERR_INVALID, "NULL argument");
    *out = nullptr;
    try {
        auto c = std::make_unique<dgtd_case>();
        c->c = dgtd::load_case(json_path);
        *out = c.release();
    } catch (const std::exception& e) {
        return cfail(unsupported(e.what()) ? DGTD_ERR_UNSUPPORTED : DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

void dgtd_case_destroy(dgtd_case* c) { delete c; }

int dgtd_case_get_info(const dgtd_case* cs, dgtd_case_info* info)
{
    if (!cs || !info) return cfail(DGTD_ERR_INVALID, "NULL argument");
    const dgtd::Case& c = cs->c;
    info->order = c.order;
    info->integrator = c.integrator;
    info->alpha = c.alpha;
    info->time_step = c.dt;
    info->final_time = c.final_time;
    info->cfl = c.cfl;
    info->n_waves = static_cast<int32_t>(c.waves.size());
    info->n_initial_fields = static_cast<int32_t>(c.initial.size());
    info->n_point_probes = static_cast<int32_t>(c.point_pos.size() / 3);
    info->n_surfaces = static_cast<int32_t>(c.surfaces.size());
    info->n_elements = static_cast<int64_t>(c.elements.size() / 4);
    info->n_vertices = static_cast<int64_t>(c.vertices.size() / 3);
    info->n_sgbc_stacks = static_cast<int32_t>(c.sgbc_stacks.size());
    int32_t nl = 0;
    for (const auto& st : c.sgbc_stacks) nl += static_cast<int32_t>(st.layers.size());
    info->n_sgbc_layers = nl;
    info->n_sgbc_faces = static_cast<int64_t>(c.sgbc_face_stack.size());
    info->basis_type = c.basis_type;
    return DGTD_OK;
}

int dgtd_case_sgbc(const dgtd_case* cs, dgtd_sgbc_stack* stacks, dgtd_sgbc_layer* layers, int32_t* face_stack)
{
    if (!cs) return cfail(DGTD_ERR_INVALID, "NULL argument");
    const dgtd::Case& c = cs->c;
    if (!c.sgbc_stacks.empty() && (!stacks || !layers)) return cfail(DGTD_ERR_INVALID, "NULL stack or layer array");
    if (!c.sgbc_face_stack.empty() && !face_stack) return cfail(DGTD_ERR_INVALID, "NULL face_stack");
    int32_t li = 0;
    for (size_t i = 0; i < c.sgbc_stacks.size(); ++i) {
        const dgtd::SgbcStackSpec& sp = c.sgbc_stacks[i];
        stacks[i].n_layers = static_cast<int32_t>(sp.layers.size());
        stacks[i].layers = layers + li;
        stacks[i].left_bc = sp.left_bc;
        stacks[i].right_bc = sp.right_bc;
        stacks[i].sub_dt = sp.sub_dt;
        for (const auto& L : sp.layers) layers[li++] = dgtd_sgbc_layer{L.eps, L.mu, L.sigma, L.width, L.segments, L.order};
    }
    std::copy(c.sgbc_face_stack.begin(), c.sgbc_face_stack.end(), face_stack);
    return DGTD_OK;
}

int dgtd_case_mesh(const dgtd_case* cs, dgtd_mesh_desc* m)
{
    if (!cs || !m) return cfail(DGTD_ERR_INVALID, "NULL argument");
    const dgtd::Case& c = cs->c;
    *m = dgtd_mesh_desc{};
    m->dim = 3;
    m->n_vertices = static_cast<int64_t>(c.vertices.size() / 3);
    m->vertices = c.vertices.data();
    m->n_elements = static_cast<int64_t>(c.elements.size() / 4);
    m->elements = c.elements.data();
    m->eps_r = c.eps.data();
    m->mu_r = c.mu.data();
    m->sigma = c.sigma.data();
    m->n_bdr_faces = static_cast<int64_t>(c.bdr_codes.size());
    m->bdr_faces = c.bdr_faces.data();
    m->bdr_codes = c.bdr_codes.data();
    m->n_tfsf_faces = static_cast<int64_t>(c.tfsf_faces.size() / 3);
    m->tfsf_faces = c.tfsf_faces.data();
    m->n_int_faces = static_cast<int64_t>(c.int_codes.size());
    m->int_faces = c.int_faces.data();
    m->int_codes = c.int_codes.data();
    m->n_curved = static_cast<int64_t>(c.curved_elems.size());
    m->curved_elems = c.curved_elems.data();
    m->curved_nodes = c.curved_nodes.data();
    return DGTD_OK;
}

int dgtd_case_auto_dt(const dgtd_case* cs, double* dt)
{
    if (!cs || !dt) return cfail(DGTD_ERR_INVALID, "NULL argument");
    const dgtd::Case& c = cs->c;
    try {
        dgtd::MeshInput in;
        in.dim = 3;
        in.vertices = c.vertices;
        in.elements = c.elements;
        in.eps = c.eps;
        in.mu = c.mu;
        in.sigma = c.sigma;
        in.bdr_faces = c.bdr_faces;
        in.bdr_codes = c.bdr_codes;
        in.tfsf_faces = c.tfsf_faces;
        in.int_faces = c.int_faces;
        in.int_codes = c.int_codes;
        in.curved_elems = c.curved_elems;
        in.curved_nodes = c.curved_nodes;
        const dgtd::MeshTables T = dgtd::build_tables(in, dgtd::build_ref_tet(c.order));
        const int evolution = c.evolution_operator == "maxwell" ? 0 : (c.evolution_operator == "hesthaven" ? 2 : 1);
        *dt = dgtd::estimate_dt(T, c.order, c.cfl, evolution);
    } catch (const std::exception& e) {
        return cfail(DGTD_ERR_INVALID, e.what());
    }
    return DGTD_OK;
}

int dgtd_case_planewaves(const dgtd_case* cs, dgtd_planewave* out, int32_t capacity)
{
    if (!cs || (!out && capacity > 0)) return cfail(DGTD_ERR_INVALID, "NULL argument");
    const auto& w = cs->c.waves;
    if (capacity < static_cast<int32_t>(w.size())) return cfail(DGTD_ERR_INVALID, "capacity below the number of plane waves");
    std::copy(w.begin(), w.end(), out);
    return DGTD_OK;
}

int dgtd_case_point_probes(const dgtd_case* cs, double* h_points)
{
    if (!cs || !h_points) return cfail(DGTD_ERR_INVALID, "NULL argument");
    std::copy(cs->c.point_pos.begin(), cs->c.point_pos.end(), h_points);
    return DGTD_OK;
}

int dgtd_case_surface(const dgtd_case* cs, int32_t s, int32_t* faces, int64_t* n_faces)
{
    if (!cs) return cfail(DGTD_ERR_INVALID, "NULL argument");
    if (s < 0 || s >= static_cast<int32_t>(cs->c.surfaces.size())) return cfail(DGTD_ERR_INVALID, "no such surface");
    const auto& f = cs->c.surfaces[s].faces;
    if (n_faces) *n_faces = static_cast<int64_t>(f.size() / 3);
    if (faces) std::copy(f.begin(), f.end(), faces);
    return DGTD_OK;
}

int dgtd_case_initial_state(const dgtd_case* cs, const double* h_xyz, int64_t n, double* h_state)
{
    if (!cs || !h_xyz || !h_state || n < 0) return cfail(DGTD_ERR_INVALID, "bad argument");
    auto u = dgtd::case_initial_state(cs->c, h_xyz, n);
    std::copy(u.begin(), u.end(), h_state);
    return DGTD_OK;
}

int dgtd_case_run(const dgtd_case* cs, const dgtd_case_run_opts* ro, double* h_state, dgtd_case_result* res)
{
    if (!cs) return cfail(DGTD_ERR_INVALID, "NULL case");
    const dgtd::Case& c = cs->c;
    if (ro && ro->precision != DGTD_FP64) return cfail(DGTD_ERR_UNSUPPORTED, "cases run on the plain FP64 form");
    if (ro && ro->n_freqs > 0 && !ro->freqs) return cfail(DGTD_ERR_INVALID, "frequency array missing");
    if (!(c.final_time >= 0.0)) return cfail(DGTD_ERR_INVALID, "final_time must be >= 0");
    dgtd_op* op = nullptr;
    double* d = nullptr;
    int rc = DGTD_OK;
    try {
        dgtd_mesh_desc m;
        ok(dgtd_case_mesh(cs, &m), "case mesh");
        dgtd_op_opts o{};
        o.order = c.order;
        o.alpha = c.alpha;
        o.precision = DGTD_FP64;
        o.batch = 1;
        ok(dgtd_op_create(&m, &o, &op), "dgtd_op_create");
        if (!c.waves.empty())
            ok(dgtd_op_set_planewaves(op, c.waves.data(), static_cast<int32_t>(c.waves.size())), "set_planewaves");
        if (!c.sgbc_face_stack.empty()) {
            dgtd_case_info ci;
            ok(dgtd_case_get_info(cs, &ci), "case info");
            std::vector<dgtd_sgbc_stack> st(ci.n_sgbc_stacks);
            std::vector<dgtd_sgbc_layer> ly(ci.n_sgbc_layers);
            std::vector<int32_t> fs(ci.n_sgbc_faces);
            ok(dgtd_case_sgbc(cs, st.data(), ly.data(), fs.data()), "case SGBC stacks");
            ok(dgtd_op_set_sgbc(op, st.data(), ci.n_sgbc_stacks, fs.data()), "set_sgbc");
        }
        double dt = c.dt;
        if (!(dt > 0.0)) ok(dgtd_case_auto_dt(cs, &dt), "automatic time step");
        dgtd_op_info info;
        ok(dgtd_op_get_info(op, &info), "get_info");
        const int64_t N = info.ndofs;
        std::vector<double> xyz(3 * N);
        ok(dgtd_op_node_coords(op, xyz.data()), "node_coords");
        // a Gauss-Legendre case: its initial fields are interpolated at its own nodes (straight
        // elements: the affine image of the node set), then moved to the operator's node set
        const bool legendre = c.basis_type == dgtd::kBasisGaussLegendre;
        const int64_t K = info.n_elements;
        const int Np = info.np;
        std::vector<double> to_lobatto, to_legendre;
        if (legendre) {
            // the element's corners as the operator holds them: its Gauss-Lobatto nodes at the
            // vertices (barycentric unit vectors), so both node sets share its vertex order
            const std::vector<double> bl = dgtd::tet_node_bary(c.order, dgtd::kBasisGaussLobatto);
            int corner[4] = {-1, -1, -1, -1};
            for (int n = 0; n < Np; ++n)
                for (int v = 0; v < 4; ++v)
                    if (bl[4 * n + v] == 1.0) corner[v] = n;
            for (int v = 0; v < 4; ++v)
                if (corner[v] < 0) throw std::runtime_error("Gauss-Lobatto node set without a vertex node");
            const std::vector<double> b = dgtd::tet_node_bary(c.order, dgtd::kBasisGaussLegendre);
            std::vector<double> gl(3 * static_cast<size_t>(N));
            for (int64_t e = 0; e < K; ++e)
                for (int n = 0; n < Np; ++n)
                    for (int r = 0; r < 3; ++r) {
                        double x = 0.0;
                        for (int v = 0; v < 4; ++v) x += b[4 * n + v] * xyz[r * N + e * Np + corner[v]];
                        gl[r * N + e * Np + n] = x;
                    }
            xyz.swap(gl);
            to_lobatto = dgtd::tet_basis_change(c.order, dgtd::kBasisGaussLegendre, dgtd::kBasisGaussLobatto);
            to_legendre = dgtd::tet_basis_change(c.order, dgtd::kBasisGaussLobatto, dgtd::kBasisGaussLegendre);
        }
        // element-block change of nodal basis of all six components, in place
        auto change_basis = [&](std::vector<double>& v, const std::vector<double>& M) {
            std::vector<double> tmp(Np);
            for (int64_t blk = 0; blk < 6 * K; ++blk) {
                double* x = &v[static_cast<size_t>(blk) * Np];
                for (int i = 0; i < Np; ++i) {
                    double a = 0.0;
                    for (int j = 0; j < Np; ++j) a += M[static_cast<size_t>(i) * Np + j] * x[j];
                    tmp[i] = a;
                }
                std::copy(tmp.begin(), tmp.end(), x);
            }
        };
        std::vector<double> u = dgtd::case_initial_state(c, xyz.data(), N);
        if (legendre) change_basis(u, to_lobatto);

        // probes: points at the smallest requested interval, all surfaces in one set
        const int32_t npts = static_cast<int32_t>(c.point_pos.size() / 3);
        std::vector<int32_t> faces;
        for (const auto& s : c.surfaces) faces.insert(faces.end(), s.faces.begin(), s.faces.end());
        int every = 1;
        if (npts > 0) {
            every = std::numeric_limits<int>::max();
            for (int32_t k = 0; k < npts; ++k)
                every = std::min(every, dgtd::probe_interval(c.point_saves[k], c.point_interval[k], c.final_time, dt));
            every = std::max(1, every);
        }
        const int64_t est_steps = dt > 0.0 ? static_cast<int64_t>(c.final_time / dt) + 2 : 2;
        const bool probes = npts > 0 || !faces.empty();
        if (probes) {
            dgtd_probe_spec ps{};
            ps.n_points = npts;
            ps.points = c.point_pos.data();
            ps.n_surface_faces = static_cast<int64_t>(faces.size() / 3);
            ps.surface_faces = faces.data();
            ps.n_freqs = ro ? ro->n_freqs : 0;
            ps.freqs = ro ? ro->freqs : nullptr;
            ps.every = every;
            ps.max_records = npts > 0 ? static_cast<int32_t>(std::min<int64_t>(est_steps / every + 3, 1 << 24)) : 0;
            ok(dgtd_op_set_probes(op, &ps), "set_probes");
        }
        const size_t bytes = u.size() * sizeof(double);
        if (cudaMalloc(&d, bytes) != cudaSuccess) throw std::runtime_error("cudaMalloc of the case state failed");
        if (cudaMemcpy(d, u.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess) throw std::runtime_error("H2D failed");
        const auto t0 = std::chrono::steady_clock::now();
        double t = 0.0;
        int64_t steps = 0;
        // instability detector of Solver::run (reference Solver.cpp:500-516): a device check every
        // kStabEvery steps and of the final state, read back at the end
        constexpr int64_t kStabEvery = 10;
        ok(dgtd_op_stability_reset(op), "stability reset");
        // probes: the initial state (the reference's Solver constructor samples at cycle 0,
        // Solver.cpp:129), then every `every` steps inside dgtd_op_step, and the final state
        if (probes) ok(dgtd_op_probe_sample(op, d, 0.0, nullptr), "initial probe sample");
        while (t <= c.final_time - 1e-8 * dt) {
            const double h = std::min(dt, c.final_time - t);
            ok(dgtd_op_step(op, d, t, h, 1, c.integrator, nullptr), "dgtd_op_step");
            t += h;
            ++steps;
            if (steps % kStabEvery == 0) ok(dgtd_op_stability_check(op, d, steps, t, nullptr), "stability check");
        }
        if (steps % kStabEvery != 0) ok(dgtd_op_stability_check(op, d, steps, t, nullptr), "stability check");
        if (probes && npts > 0 && steps % every != 0) ok(dgtd_op_probe_sample(op, d, t, nullptr), "final probe sample");
        if (cudaDeviceSynchronize() != cudaSuccess) throw std::runtime_error("device synchronisation failed");
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (h_state && cudaMemcpy(h_state, d, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
            throw std::runtime_error("D2H failed");
        if (h_state && legendre) {
            std::vector<double> v(h_state, h_state + u.size());
            change_basis(v, to_legendre);
            std::copy(v.begin(), v.end(), h_state);
        }
        int64_t nrec = 0;
        if (probes) {
            ok(dgtd_op_probe_info(op, nullptr, nullptr, &nrec), "probe_info");
            if (ro && ro->out_dir && npts > 0) {
                std::vector<double> series(static_cast<size_t>(nrec) * npts * 6), times(nrec);
                ok(dgtd_op_probe_read(op, nullptr, nullptr, series.data(), times.data(), nullptr), "probe_read");
                // the reference's point-probe file (ProbesManager.cpp:203-215, 400-407): four header
                // lines (ID, "Spatial Position (X, Y, Z)", the position, the column names), then per
                // sample the time in seconds (normalised time / c) and the six field values
                constexpr double kSpeedOfLightSI = 299792458.0;
                for (int32_t k = 0; k < npts; ++k) {
                    const std::string path = std::string(ro->out_dir) + "/PointProbe" + std::to_string(k) + ".dat";
                    FILE* f = std::fopen(path.c_str(), "w");
                    if (!f) throw std::runtime_error("cannot write " + path);
                    const double* x = &c.point_pos[3 * static_cast<size_t>(k)];
                    std::fprintf(f, "PointProbe ID %d\nSpatial Position (X, Y, Z) \n%s %s %s\n", k,
                                 std::to_string(x[0]).c_str(), std::to_string(x[1]).c_str(), std::to_string(x[2]).c_str());
                    std::fprintf(f, "Time (s) // Ex // Ey // Ez // Hx // Hy // Hz \n");
                    for (int64_t r = 0; r < nrec; ++r) {
                        const double* v = &series[(static_cast<size_t>(r) * npts + k) * 6];
                        std::fprintf(f, "%.10e %.10e %.10e %.10e %.10e %.10e %.10e\n", times[r] / kSpeedOfLightSI, v[0],
                                     v[1], v[2], v[3], v[4], v[5]);
                    }
                    std::fclose(f);
                }
            }
        }
        int64_t unstable_step = -1;
        double unstable_t = 0.0, unstable_norm = 0.0;
        ok(dgtd_op_stability(op, &unstable_step, &unstable_t, &unstable_norm, nullptr), "stability record");
        if (unstable_step >= 0)
            std::fprintf(stderr,
                         "dgtd_gb300: WARNING: simulation is potentially unstable (field norm = %g at step %lld, "
                         "time %g / %g, dt %g); verify the setup and consider a smaller time step\n",
                         unstable_norm, static_cast<long long>(unstable_step), unstable_t, c.final_time, dt);
        if (res) {
            res->steps = steps;
            res->dt = dt;
            res->final_time = t;
            res->n_records = nrec;
            res->seconds = secs;
            res->unstable_step = unstable_step;
        }
    } catch (const std::exception& e) {
        rc = cfail(DGTD_ERR_CUDA, e.what());
    }
    if (d) cudaFree(d);
    if (op) dgtd_op_destroy(op);
    return rc;
}

}  // extern "C"
