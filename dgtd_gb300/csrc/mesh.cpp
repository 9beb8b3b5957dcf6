// Mesh tables: connectivity, node maps, geometric factors (FP64, host).
#include "mesh.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <stdexcept>

namespace dgtd {

namespace {

struct FaceKey {
    int32_t a, b, c;
    bool operator<(const FaceKey& o) const {
        if (a != o.a) return a < o.a;
        if (b != o.b) return b < o.b;
        return c < o.c;
    }
    bool operator==(const FaceKey& o) const { return a == o.a && b == o.b && c == o.c; }
};

FaceKey make_key(int32_t u, int32_t v, int32_t w)
{
    int32_t t[3] = {u, v, w};
    std::sort(t, t + 3);
    return {t[0], t[1], t[2]};
}

struct FaceRec {
    FaceKey key;
    int64_t e;
    int f;
    bool operator<(const FaceRec& o) const {
        if (!(key == o.key)) return key < o.key;
        if (e != o.e) return e < o.e;
        return f < o.f;
    }
};

inline void sub3(const double* a, const double* b, double* c) { c[0] = a[0] - b[0]; c[1] = a[1] - b[1]; c[2] = a[2] - b[2]; }
inline void cross3(const double* a, const double* b, double* c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

}  // namespace

double estimate_dt(const MeshTables& T, int p, double cfl, int evolution)
{
    if (evolution == 2) {
        double maxf = 0.0;
        for (size_t q = 3; q < T.fgeo.size(); q += 4) maxf = std::max(maxf, T.fgeo[q]);
        return 1.0 * cfl / (maxf * p * p);
    }
    const auto g = gauss_lobatto(p);
    const double rmin = std::fabs(g[1] - g[0]);   // GLL spacing on a segment of length 2
    const double base = T.dt_scale_min * rmin * 2.0 / 3.0 * 0.75 * cfl;
    return evolution == 1 ? base / 0.8 : base;
}

MeshTables build_tables(const MeshInput& in, const RefTet& ref)
{
    if (in.dim != 3) throw std::runtime_error("build_tables: only 3D tetrahedral meshes");
    MeshTables T;
    T.dim = 3; T.p = ref.p; T.Np = ref.Np; T.Nfp = ref.Nfp; T.Nfaces = 4;
    const int Np = ref.Np, Nfp = ref.Nfp;
    const int64_t nv = static_cast<int64_t>(in.vertices.size() / 3);
    const int64_t K = static_cast<int64_t>(in.elements.size() / 4);
    if (K <= 0) throw std::runtime_error("mesh has no elements");
    if (K * Np > INT32_MAX) throw std::runtime_error("mesh too large for 32-bit node indices");
    T.K = K;
    for (int64_t i = 0; i < 4 * K; ++i)
        if (in.elements[i] < 0 || in.elements[i] >= nv) throw std::runtime_error("element references a missing vertex");
    const double* X = in.vertices.data();

    // ---- geometry ------------------------------------------------------------
    T.x.resize(K * Np); T.y.resize(K * Np); T.z.resize(K * Np);
    T.geo.resize(K * 9); T.fgeo.resize(K * 16); T.mat.resize(K * 3);
    double min_edge = 1e300, dts = 1e300;
    for (int64_t e = 0; e < K; ++e) {
        const double* v[4];
        for (int q = 0; q < 4; ++q) v[q] = X + 3 * in.elements[4 * e + q];
        for (int n = 0; n < Np; ++n) {
            double px = 0, py = 0, pz = 0;
            for (int q = 0; q < 4; ++q) {
                double l = ref.bary[4 * n + q];
                px += l * v[q][0]; py += l * v[q][1]; pz += l * v[q][2];
            }
            T.x[e * Np + n] = px; T.y[e * Np + n] = py; T.z[e * Np + n] = pz;
        }
        double xr[3], xs[3], xt[3];
        sub3(v[1], v[0], xr); sub3(v[2], v[0], xs); sub3(v[3], v[0], xt);
        for (int d = 0; d < 3; ++d) { xr[d] *= 0.5; xs[d] *= 0.5; xt[d] *= 0.5; }
        // J = det [xr xs xt] (columns)
        double c[3];
        cross3(xs, xt, c);
        double J = dot3(xr, c);
        if (!(J > 0.0)) throw std::runtime_error("tetrahedron with non-positive Jacobian (vertex order must be positively oriented)");
        // rows of inverse: grad r = (xs x xt)/J, grad s = (xt x xr)/J, grad t = (xr x xs)/J
        double gr[3], gs[3], gt[3];
        cross3(xs, xt, gr); cross3(xt, xr, gs); cross3(xr, xs, gt);
        for (int d = 0; d < 3; ++d) { gr[d] /= J; gs[d] /= J; gt[d] /= J; }
        double* G = &T.geo[e * 9];
        G[0] = gr[0]; G[1] = gr[1]; G[2] = gr[2];
        G[3] = gs[0]; G[4] = gs[1]; G[5] = gs[2];
        G[6] = gt[0]; G[7] = gt[1]; G[8] = gt[2];
        // grad of barycentrics: l1 = (1+r)/2, l2 = (1+s)/2, l3 = (1+t)/2, l0 = 1-l1-l2-l3
        double gl[4][3];
        for (int d = 0; d < 3; ++d) {
            gl[1][d] = 0.5 * gr[d]; gl[2][d] = 0.5 * gs[d]; gl[3][d] = 0.5 * gt[d];
            gl[0][d] = -(gl[1][d] + gl[2][d] + gl[3][d]);
        }
        double area_sum = 0.0;
        for (int f = 0; f < 4; ++f) {
            double nrm = std::sqrt(dot3(gl[f], gl[f]));
            double* F = &T.fgeo[e * 16 + f * 4];
            F[0] = -gl[f][0] / nrm; F[1] = -gl[f][1] / nrm; F[2] = -gl[f][2] / nrm;
            F[3] = 2.0 * nrm;     // Fscale = sJ / J
            area_sum += 3.0 * (J * 4.0 / 3.0) * nrm;   // area_f = 3 vol |grad l_f|
        }
        double vol = J * 4.0 / 3.0;
        dts = std::min(dts, vol / (0.5 * area_sum));
        for (int a = 0; a < 4; ++a)
            for (int b = a + 1; b < 4; ++b) {
                double d[3]; sub3(v[a], v[b], d);
                min_edge = std::min(min_edge, std::sqrt(dot3(d, d)));
            }
        double eps = in.eps.empty() ? 1.0 : in.eps[e];
        double mu = in.mu.empty() ? 1.0 : in.mu[e];
        double sg = in.sigma.empty() ? 0.0 : in.sigma[e];
        if (!(eps > 0.0) || !(mu > 0.0)) throw std::runtime_error("permittivity and permeability must be positive");
        T.mat[e * 3 + 0] = 1.0 / eps;
        T.mat[e * 3 + 1] = 1.0 / mu;
        T.mat[e * 3 + 2] = sg / eps;
    }
    T.min_edge = min_edge;
    T.dt_scale_min = dts;

    // ---- connectivity ---------------------------------------------------------
    std::vector<FaceRec> recs;
    recs.reserve(4 * K);
    for (int64_t e = 0; e < K; ++e) {
        const int32_t* ev = &in.elements[4 * e];
        for (int f = 0; f < 4; ++f) {
            int32_t w[3]; int c = 0;
            for (int q = 0; q < 4; ++q) if (q != f) w[c++] = ev[q];
            recs.push_back({make_key(w[0], w[1], w[2]), e, f});
        }
    }
    std::sort(recs.begin(), recs.end());
    T.nbr.assign(4 * K, -1);
    std::vector<int32_t> nbr_face(4 * K, -1);
    for (size_t i = 0; i < recs.size();) {
        size_t j = i + 1;
        while (j < recs.size() && recs[j].key == recs[i].key) ++j;
        if (j - i > 2) throw std::runtime_error("non-manifold mesh: a face is shared by more than two elements");
        if (j - i == 2) {
            const auto& A = recs[i]; const auto& B = recs[i + 1];
            T.nbr[A.e * 4 + A.f] = static_cast<int32_t>(B.e); nbr_face[A.e * 4 + A.f] = B.f;
            T.nbr[B.e * 4 + B.f] = static_cast<int32_t>(A.e); nbr_face[B.e * 4 + B.f] = A.f;
        }
        i = j;
    }
    auto find_face = [&](int32_t u, int32_t v, int32_t w, int64_t& e1, int& f1, int64_t& e2, int& f2) {
        FaceKey k = make_key(u, v, w);
        FaceRec probe{k, -1, -1};
        auto it = std::lower_bound(recs.begin(), recs.end(), probe);
        if (it == recs.end() || !(it->key == k)) return false;
        e1 = it->e; f1 = it->f; e2 = -1; f2 = -1;
        auto it2 = it + 1;
        if (it2 != recs.end() && it2->key == k) { e2 = it2->e; f2 = it2->f; }
        return true;
    };

    T.fcode.assign(4 * K, FACE_INTERIOR);
    for (int64_t e = 0; e < K; ++e)
        for (int f = 0; f < 4; ++f)
            if (T.nbr[e * 4 + f] < 0) T.fcode[e * 4 + f] = FACE_OPEN;

    const int64_t nb = static_cast<int64_t>(in.bdr_codes.size());
    if (static_cast<int64_t>(in.bdr_faces.size()) != 3 * nb) throw std::runtime_error("boundary face/code size mismatch");
    for (int64_t b = 0; b < nb; ++b) {
        int64_t e1, e2; int f1, f2;
        if (!find_face(in.bdr_faces[3 * b], in.bdr_faces[3 * b + 1], in.bdr_faces[3 * b + 2], e1, f1, e2, f2))
            throw std::runtime_error("boundary face does not match any element face");
        if (e2 >= 0) throw std::runtime_error("boundary condition given on an interior face (use interior faces for sheets)");
        int code = in.bdr_codes[b];
        if (code < 0 || code > 3) throw std::runtime_error("unknown boundary code");
        T.fcode[e1 * 4 + f1] = (code == 0) ? FACE_OPEN : code;
    }

    const int64_t ni = static_cast<int64_t>(in.int_codes.size());
    if (static_cast<int64_t>(in.int_faces.size()) != 3 * ni) throw std::runtime_error("interior face/code size mismatch");
    for (int64_t b = 0; b < ni; ++b) {
        int64_t e1, e2; int f1, f2;
        if (!find_face(in.int_faces[3 * b], in.int_faces[3 * b + 1], in.int_faces[3 * b + 2], e1, f1, e2, f2) || e2 < 0)
            throw std::runtime_error("interior boundary face is not shared by two elements");
        int code = in.int_codes[b];
        if (code < 1 || code > 4) throw std::runtime_error("unknown interior boundary code");
        if (code == 4) {   // thin layer: the first element is the lower index (the face's owner)
            T.fcode[e1 * 4 + f1] = FACE_SGBC;
            T.fcode[e2 * 4 + f2] = FACE_SGBC;
            T.sgbc_faces.insert(T.sgbc_faces.end(), {static_cast<int32_t>(e1), f1, static_cast<int32_t>(e2), f2});
            continue;
        }
        T.fcode[e1 * 4 + f1] = FACE_INT_PEC + (code - 1);
        T.fcode[e2 * 4 + f2] = FACE_INT_PEC + (code - 1);
    }

    // TF/SF faces: the winding normal points into the total-field side
    // (the reference's buildFaceOrientation, SubMesher.cpp:582-597).
    const int64_t nt = static_cast<int64_t>(in.tfsf_faces.size() / 3);
    std::vector<char> tfsf_elem(K, 0);
    for (int64_t b = 0; b < nt; ++b) {
        const int32_t* fv = &in.tfsf_faces[3 * b];
        int64_t e1, e2; int f1, f2;
        if (!find_face(fv[0], fv[1], fv[2], e1, f1, e2, f2) || e2 < 0)
            throw std::runtime_error("TF/SF face is not shared by two elements");
        double a[3], bb[3], nrm[3];
        sub3(X + 3 * fv[1], X + 3 * fv[0], a); sub3(X + 3 * fv[2], X + 3 * fv[0], bb);
        cross3(a, bb, nrm);
        auto bary = [&](int64_t e, double* c) {
            c[0] = c[1] = c[2] = 0.0;
            for (int q = 0; q < 4; ++q)
                for (int d = 0; d < 3; ++d) c[d] += 0.25 * X[3 * in.elements[4 * e + q] + d];
        };
        double c1[3], c2[3], d12[3];
        bary(e1, c1); bary(e2, c2); sub3(c2, c1, d12);
        bool e2_is_tf = dot3(d12, nrm) >= 0.0;
        T.fcode[e1 * 4 + f1] = e2_is_tf ? FACE_TFSF_SF : FACE_TFSF_TF;
        T.fcode[e2 * 4 + f2] = e2_is_tf ? FACE_TFSF_TF : FACE_TFSF_SF;
        tfsf_elem[e1] = 1; tfsf_elem[e2] = 1;
    }
    for (int64_t e = 0; e < K; ++e) if (tfsf_elem[e]) T.tfsf_elems.push_back(static_cast<int32_t>(e));

    // ---- curved (second-order) elements: DOF nodes on the isoparametric map
    //   x = sum_k l_k (2 l_k - 1) X_k + sum_(a<b) 4 l_a l_b X_ab
    const int64_t ncv = static_cast<int64_t>(in.curved_elems.size());
    if (static_cast<int64_t>(in.curved_nodes.size()) != 30 * ncv) throw std::runtime_error("curved element geometry size mismatch");
    {
        static const int ea[6] = {0, 0, 0, 1, 1, 2}, eb[6] = {1, 2, 3, 2, 3, 3};
        std::vector<char> seen(K, 0);
        for (int64_t c = 0; c < ncv; ++c) {
            const int64_t e = in.curved_elems[c];
            if (e < 0 || e >= K || seen[e]) throw std::runtime_error("curved element ids must be distinct elements");
            seen[e] = 1;
            const double* G = &in.curved_nodes[30 * c];
            for (int q = 0; q < 4; ++q)
                for (int d = 0; d < 3; ++d)
                    if (G[3 * q + d] != X[3 * in.elements[4 * e + q] + d])
                        throw std::runtime_error("curved element geometry: corners must be the element's vertices");
            for (int n = 0; n < Np; ++n) {
                const double* l = &ref.bary[4 * n];
                double P[3] = {0.0, 0.0, 0.0};
                for (int k = 0; k < 4; ++k)
                    for (int d = 0; d < 3; ++d) P[d] += l[k] * (2.0 * l[k] - 1.0) * G[3 * k + d];
                for (int m = 0; m < 6; ++m)
                    for (int d = 0; d < 3; ++d) P[d] += 4.0 * l[ea[m]] * l[eb[m]] * G[3 * (4 + m) + d];
                T.x[e * Np + n] = P[0]; T.y[e * Np + n] = P[1]; T.z[e * Np + n] = P[2];
            }
        }
        for (int32_t e : T.tfsf_elems)
            if (seen[e]) throw std::runtime_error("TF/SF faces on curved elements are not supported");
        T.curved_elems = in.curved_elems;
        T.curved_nodes = in.curved_nodes;
    }

    // ---- node maps ----------------------------------------------------------------
    // A face node's partner is the neighbour's face node with the same barycentric coordinates on
    // the same three (global) vertices; positions only confirm it. A curved element and a straight
    // neighbour (edge nodes within 1e-5 of the midpoints, taken as affine) may place a shared
    // face's nodes up to a few 1e-5 apart, so faces touching a curved element get that slack.
    T.vmapP.resize(K * 4 * Nfp);
    const double tol = 1e-7 * min_edge;
    std::vector<char> curved_el(K, 0);
    for (int32_t e : in.curved_elems) curved_el[e] = 1;
    for (int64_t e = 0; e < K; ++e)
        for (int f = 0; f < 4; ++f) {
            int32_t* out = &T.vmapP[(e * 4 + f) * Nfp];
            int64_t en = T.nbr[e * 4 + f];
            if (en < 0) {
                for (int a = 0; a < Nfp; ++a) out[a] = static_cast<int32_t>(e * Np + ref.Fmask[f * Nfp + a]);
                continue;
            }
            int fn = nbr_face[e * 4 + f];
            // local vertex of the neighbour for each local vertex of e on this face
            int loc[4] = {-1, -1, -1, -1};
            for (int q = 0; q < 4; ++q) {
                if (q == f) continue;
                for (int r = 0; r < 4; ++r)
                    if (in.elements[4 * en + r] == in.elements[4 * e + q]) loc[q] = r;
                if (loc[q] < 0) throw std::runtime_error("neighbouring elements do not share a face's vertices");
            }
            const double slack = (curved_el[e] || curved_el[en]) ? 5e-5 : 0.0;
            for (int a = 0; a < Nfp; ++a) {
                const int vm = ref.Fmask[f * Nfp + a];
                const int64_t gm = e * Np + vm;
                int best = -1;
                double bw = 1e300;
                for (int b = 0; b < Nfp; ++b) {
                    const int vp = ref.Fmask[fn * Nfp + b];
                    double w = 0.0;
                    for (int q = 0; q < 4; ++q)
                        if (q != f) w += std::fabs(ref.bary[4 * vm + q] - ref.bary[4 * vp + loc[q]]);
                    if (w < bw) { bw = w; best = b; }
                }
                const int64_t gp = en * Np + ref.Fmask[fn * Nfp + best];
                const double dx = T.x[gm] - T.x[gp], dy = T.y[gm] - T.y[gp], dz = T.z[gm] - T.z[gp];
                if (bw > 1e-9 || std::sqrt(dx * dx + dy * dy + dz * dz) > tol + slack)
                    throw std::runtime_error("face nodes of neighbouring elements do not coincide");
                out[a] = static_cast<int32_t>(gp);
            }
        }
    T.elem_vertices = in.elements;
    T.vertices = in.vertices;
    return T;
}

MeshInput make_box(const BoxSpec& s)
{
    MeshInput m;
    m.dim = 3;
    const int nx = s.n[0], ny = s.n[1], nz = s.n[2];
    if (nx < 1 || ny < 1 || nz < 1) throw std::runtime_error("box needs at least one cell per axis");
    auto vid = [&](int i, int j, int k) { return static_cast<int32_t>(i + (nx + 1) * (j + (ny + 1) * k)); };
    m.vertices.resize(3 * static_cast<size_t>(nx + 1) * (ny + 1) * (nz + 1));
    for (int k = 0; k <= nz; ++k)
        for (int j = 0; j <= ny; ++j)
            for (int i = 0; i <= nx; ++i) {
                int32_t v = vid(i, j, k);
                m.vertices[3 * v + 0] = s.lo[0] + (s.hi[0] - s.lo[0]) * i / nx;
                m.vertices[3 * v + 1] = s.lo[1] + (s.hi[1] - s.lo[1]) * j / ny;
                m.vertices[3 * v + 2] = s.lo[2] + (s.hi[2] - s.lo[2]) * k / nz;
            }
    auto in_range = [](int i, int j, int k, const int* lo, const int* hi) {
        return i >= lo[0] && i < hi[0] && j >= lo[1] && j < hi[1] && k >= lo[2] && k < hi[2];
    };
    auto in_hole = [&](int i, int j, int k) { return in_range(i, j, k, s.hole_lo, s.hole_hi); };
    auto in_tf = [&](int i, int j, int k) { return in_range(i, j, k, s.tf_lo, s.tf_hi); };
    auto cell_exists = [&](int i, int j, int k) {
        return i >= 0 && i < nx && j >= 0 && j < ny && k >= 0 && k < nz && !in_hole(i, j, k);
    };
    // 6 tetrahedra sharing the c0-c6 diagonal, all positively oriented
    static const int kuhn[6][4] = {{0, 1, 2, 6}, {0, 5, 1, 6}, {0, 4, 5, 6},
                                   {0, 2, 3, 6}, {0, 3, 7, 6}, {0, 7, 4, 6}};
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                if (in_hole(i, j, k)) continue;
                int32_t c[8] = {vid(i, j, k), vid(i + 1, j, k), vid(i + 1, j + 1, k), vid(i, j + 1, k),
                                vid(i, j, k + 1), vid(i + 1, j, k + 1), vid(i + 1, j + 1, k + 1), vid(i, j + 1, k + 1)};
                for (auto& t : kuhn)
                    for (int q = 0; q < 4; ++q) m.elements.push_back(c[t[q]]);
            }
    // Boundary and TF/SF faces: each hex face is two triangles split along the
    // diagonal through its lowest and highest corner (consistent with the Kuhn split).
    auto add_quad = [&](std::vector<int32_t>& dst, int32_t a, int32_t b, int32_t c, int32_t d, bool flip) {
        // quad a-b-c-d (cyclic), diagonal a-c
        if (!flip) { dst.insert(dst.end(), {a, b, c}); dst.insert(dst.end(), {a, c, d}); }
        else       { dst.insert(dst.end(), {a, c, b}); dst.insert(dst.end(), {a, d, c}); }
    };
    bool have_tf = s.tf_hi[0] > s.tf_lo[0] && s.tf_hi[1] > s.tf_lo[1] && s.tf_hi[2] > s.tf_lo[2];
    // visit every cell face between cell (i,j,k) and its +axis neighbour
    for (int axis = 0; axis < 3; ++axis) {
        int lim[3] = {nx, ny, nz};
        lim[axis] += 1;
        for (int k = 0; k < lim[2]; ++k)
            for (int j = 0; j < lim[1]; ++j)
                for (int i = 0; i < lim[0]; ++i) {
                    int im[3] = {i, j, k};
                    im[axis] -= 1;                    // cell on the minus side
                    bool a_ex = cell_exists(im[0], im[1], im[2]);
                    bool b_ex = cell_exists(i, j, k);
                    if (!a_ex && !b_ex) continue;
                    // quad corners in the plane at index i/j/k along axis, with the
                    // lowest corner first and the highest third (diagonal of the split).
                    int32_t q0, q1, q2, q3;
                    if (axis == 0) { q0 = vid(i, j, k); q1 = vid(i, j + 1, k); q2 = vid(i, j + 1, k + 1); q3 = vid(i, j, k + 1); }
                    else if (axis == 1) { q0 = vid(i, j, k); q1 = vid(i + 1, j, k); q2 = vid(i + 1, j, k + 1); q3 = vid(i, j, k + 1); }
                    else { q0 = vid(i, j, k); q1 = vid(i + 1, j, k); q2 = vid(i + 1, j + 1, k); q3 = vid(i, j + 1, k); }
                    if (a_ex != b_ex) {
                        bool on_outer = (axis == 0 && (i == 0 || i == nx)) || (axis == 1 && (j == 0 || j == ny)) ||
                                        (axis == 2 && (k == 0 || k == nz));
                        int code = on_outer ? s.outer_bc : s.hole_bc;
                        size_t before = m.bdr_faces.size();
                        add_quad(m.bdr_faces, q0, q1, q2, q3, false);
                        for (size_t t = before; t < m.bdr_faces.size(); t += 3) m.bdr_codes.push_back(code);
                    } else if (have_tf) {
                        bool a_tf = in_tf(im[0], im[1], im[2]);
                        bool b_tf = in_tf(i, j, k);
                        if (a_tf != b_tf) {
                            // winding normal of (q0,q1,q2) points to +axis for axis 2, check others numerically
                            const double* P0 = &m.vertices[3 * q0];
                            const double* P1 = &m.vertices[3 * q1];
                            const double* P2 = &m.vertices[3 * q2];
                            double u[3], w[3], nrm[3];
                            sub3(P1, P0, u); sub3(P2, P0, w); cross3(u, w, nrm);
                            bool plus = nrm[axis] > 0.0;      // winding normal towards +axis
                            bool want_plus = b_tf;            // TF cell on the + side
                            add_quad(m.tfsf_faces, q0, q1, q2, q3, plus != want_plus);
                        }
                    }
                }
    }
    return m;
}

}  // namespace dgtd
