// Second-order (curved) tetrahedra: block rows of the assembled operator (host).
#include "curved.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <exception>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>

namespace dgtd {

namespace {

const int kEa[6] = {0, 0, 0, 1, 1, 2}, kEb[6] = {1, 2, 3, 2, 3, 3};
const double kRefV[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};   // unit-simplex vertices

// Geometry of element e at unit-simplex point xi: position and J[r][d] = dx_r / dxi_d (curved: the
// second-order map of its ten nodes G; affine: its four vertices).
void geom(const MeshTables& T, int64_t e, const double* G, const double* xi, double* x, double* J)
{
    const double l[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
    static const double dl[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int r = 0; r < 3; ++r) { x[r] = 0.0; for (int d = 0; d < 3; ++d) J[r * 3 + d] = 0.0; }
    if (!G) {
        for (int k = 0; k < 4; ++k) {
            const double* v = &T.vertices[3 * static_cast<size_t>(T.elem_vertices[4 * e + k])];
            for (int r = 0; r < 3; ++r) {
                x[r] += l[k] * v[r];
                for (int d = 0; d < 3; ++d) J[r * 3 + d] += dl[k][d] * v[r];
            }
        }
        return;
    }
    for (int k = 0; k < 4; ++k)
        for (int r = 0; r < 3; ++r) {
            x[r] += l[k] * (2.0 * l[k] - 1.0) * G[3 * k + r];
            for (int d = 0; d < 3; ++d) J[r * 3 + d] += (4.0 * l[k] - 1.0) * dl[k][d] * G[3 * k + r];
        }
    for (int m = 0; m < 6; ++m) {
        const int a = kEa[m], b = kEb[m];
        for (int r = 0; r < 3; ++r) {
            x[r] += 4.0 * l[a] * l[b] * G[3 * (4 + m) + r];
            for (int d = 0; d < 3; ++d) J[r * 3 + d] += 4.0 * (l[b] * dl[a][d] + l[a] * dl[b][d]) * G[3 * (4 + m) + r];
        }
    }
}

double inv3(const double* J, double* Ji)   // Ji[d][r] = dxi_d / dx_r; returns det J
{
    const double c0 = J[4] * J[8] - J[5] * J[7], c1 = J[5] * J[6] - J[3] * J[8], c2 = J[3] * J[7] - J[4] * J[6];
    const double det = J[0] * c0 + J[1] * c1 + J[2] * c2;
    Ji[0] = c0 / det; Ji[3] = c1 / det; Ji[6] = c2 / det;
    Ji[1] = (J[2] * J[7] - J[1] * J[8]) / det; Ji[4] = (J[0] * J[8] - J[2] * J[6]) / det; Ji[7] = (J[1] * J[6] - J[0] * J[7]) / det;
    Ji[2] = (J[1] * J[5] - J[2] * J[4]) / det; Ji[5] = (J[2] * J[3] - J[0] * J[5]) / det; Ji[8] = (J[0] * J[4] - J[1] * J[3]) / det;
    return det;
}

// Nodal basis at a unit-simplex point (the reference element's (r, s, t) = 2 xi - 1).
void basis(const RefTet& ref, const double* xi, double* phi) { nodal_basis_at(ref, 2 * xi[0] - 1, 2 * xi[1] - 1, 2 * xi[2] - 1, phi); }

// Flux coefficients of one face point: F = Cm u- + Cp u+ (6 x 6 each, rows E,H of the flux,
// columns E,H of the trace), for the face code and the unit outward normal n. The same flux as
// the stage kernel's: F_E = 1/2 (n x dH + aE (dE - (n.dE) n)), F_H = 1/2 (-n x dE + aH (dH - (n.dH) n)).
void flux_coeffs(int code, const double* n, double alpha, double* Cm, double* Cp)
{
    double X[9] = {0, -n[2], n[1], n[2], 0, -n[0], -n[1], n[0], 0};   // X v = n x v
    double P[9];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) P[a * 3 + b] = (a == b ? 1.0 : 0.0) - n[a] * n[b];
    for (int i = 0; i < 36; ++i) { Cm[i] = 0.0; Cp[i] = 0.0; }
    auto put = [](double* C, int ro, int co, const double* B, double s) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) C[(ro + a) * 6 + co + b] += s * B[a * 3 + b];
    };
    switch (code) {
    case FACE_INTERIOR:
        put(Cp, 0, 0, P, 0.5 * alpha); put(Cp, 0, 3, X, 0.5); put(Cp, 3, 0, X, -0.5); put(Cp, 3, 3, P, 0.5 * alpha);
        for (int i = 0; i < 36; ++i) Cm[i] = -Cp[i];
        break;
    case FACE_PEC: case FACE_INT_PEC:   // dE = -2 E-, dH = 0
        put(Cm, 0, 0, P, -alpha); put(Cm, 3, 0, X, 1.0);
        break;
    case FACE_PMC: case FACE_INT_PMC:   // dE = 0, dH = -2 H-
        put(Cm, 0, 3, X, -1.0); put(Cm, 3, 3, P, -alpha);
        break;
    case FACE_SMA: case FACE_INT_SMA:   // dE = -E-, dH = -H-, penalty 1
        put(Cm, 0, 0, P, -0.5); put(Cm, 0, 3, X, -0.5); put(Cm, 3, 0, X, 0.5); put(Cm, 3, 3, P, -0.5);
        break;
    default:   // open: zero jump
        break;
    }
}

}  // namespace

CurvedRows build_curved_rows(const MeshTables& T, const RefTet& ref, double alpha)
{
    CurvedRows C;
    const int Np = ref.Np, R = 6 * Np;
    C.Np = Np;
    const int64_t nc = static_cast<int64_t>(T.curved_elems.size());
    std::vector<int64_t> cidx(T.K, -1);
    for (int64_t c = 0; c < nc; ++c) cidx[T.curved_elems[c]] = c;
    auto geo_of = [&](int64_t e) -> const double* { return cidx[e] >= 0 ? &T.curved_nodes[30 * cidx[e]] : nullptr; };

    // collapsed Gauss-Legendre rules on the unit tetrahedron and triangle, p + 4 points per direction,
    // with the basis tabulated once at the volume points and, per ordered triple of local vertices,
    // at the face points
    std::vector<double> g, gw;
    gauss_legendre01(ref.p + 4, g, gw);
    const int ng = static_cast<int>(g.size());
    std::vector<double> vx, vw, vphi, vdphi;
    for (int a = 0; a < ng; ++a)
        for (int b = 0; b < ng; ++b)
            for (int q = 0; q < ng; ++q) {
                const double u = g[a], v = g[b], w = g[q];
                const double xi[3] = {u * (1 - v) * (1 - w), v * (1 - w), w};
                vx.insert(vx.end(), xi, xi + 3);
                vw.push_back(gw[a] * gw[b] * gw[q] * (1 - v) * (1 - w) * (1 - w));
                std::vector<double> ph(Np), dp(3 * Np);
                basis(ref, xi, ph.data());
                nodal_basis_grad_at(ref, 2 * xi[0] - 1, 2 * xi[1] - 1, 2 * xi[2] - 1, dp.data());
                vphi.insert(vphi.end(), ph.begin(), ph.end());
                vdphi.insert(vdphi.end(), dp.begin(), dp.end());
            }
    const int nvq = static_cast<int>(vw.size());
    std::vector<double> fu, fv, fwt;
    for (int a = 0; a < ng; ++a)
        for (int b = 0; b < ng; ++b) {
            fu.push_back(g[a] * (1 - g[b])); fv.push_back(g[b]); fwt.push_back(gw[a] * gw[b] * (1 - g[b]));
        }
    const int nfq = static_cast<int>(fwt.size());
    std::map<int, std::vector<double>> ftab;   // key l0*16 + l1*4 + l2 -> [nfq][Np]
    std::mutex ftab_mu;
    auto face_table = [&](const int* l) -> const std::vector<double>& {
        const int key = l[0] * 16 + l[1] * 4 + l[2];
        std::lock_guard<std::mutex> lk(ftab_mu);
        auto it = ftab.find(key);
        if (it != ftab.end()) return it->second;
        std::vector<double> t(static_cast<size_t>(nfq) * Np);
        for (int k = 0; k < nfq; ++k) {
            const double bc[3] = {1.0 - fu[k] - fv[k], fu[k], fv[k]};
            double xi[3] = {0, 0, 0};
            for (int r = 0; r < 3; ++r)
                for (int m = 0; m < 3; ++m) xi[r] += bc[m] * kRefV[l[m]][r];
            basis(ref, xi, &t[static_cast<size_t>(k) * Np]);
        }
        return ftab.emplace(key, std::move(t)).first->second;
    };

    C.elems = T.curved_elems;
    C.nbr.assign(4 * nc, -1);
    C.blocks.assign(static_cast<size_t>(nc) * 5 * R * R, 0.0);

    auto assemble = [&](int64_t c) {
        const int64_t e = T.curved_elems[c];
        const double* G = geo_of(e);
        std::vector<double> M(Np * Np, 0.0), S[3], D[3], Minv;
        for (int d = 0; d < 3; ++d) S[d].assign(Np * Np, 0.0);
        std::vector<double> gx(3 * Np);
        for (int k = 0; k < nvq; ++k) {
            double x[3], J[9], Ji[9];
            geom(T, e, G, &vx[3 * k], x, J);
            const double det = inv3(J, Ji);
            if (!(det > 0.0)) throw std::runtime_error("curved element " + std::to_string(e) + " with a non-positive Jacobian");
            const double* phi = &vphi[static_cast<size_t>(k) * Np];
            const double* dphi = &vdphi[static_cast<size_t>(k) * 3 * Np];
            const double ww = vw[k] * det;
            for (int j = 0; j < Np; ++j)
                for (int d = 0; d < 3; ++d) {
                    // d phi_j / dx_d = sum_r (2 d phi_j / d rst_r) dxi_r / dx_d
                    double a = 0.0;
                    for (int r = 0; r < 3; ++r) a += 2.0 * dphi[3 * j + r] * Ji[r * 3 + d];
                    gx[3 * j + d] = a;
                }
            for (int i = 0; i < Np; ++i) {
                const double wi = ww * phi[i];
                for (int j = 0; j < Np; ++j) {
                    M[i * Np + j] += wi * phi[j];
                    S[0][i * Np + j] += wi * gx[3 * j];
                    S[1][i * Np + j] += wi * gx[3 * j + 1];
                    S[2][i * Np + j] += wi * gx[3 * j + 2];
                }
            }
        }
        Minv = M;
        if (!invert_matrix(Minv, Np)) throw std::runtime_error("singular curved-element mass matrix");
        for (int d = 0; d < 3; ++d) {
            D[d].assign(Np * Np, 0.0);
            matmul(Minv.data(), S[d].data(), D[d].data(), Np, Np, Np);
        }
        double* B0 = &C.blocks[(static_cast<size_t>(c) * 5) * R * R];
        const double ie = T.mat[3 * e], im = T.mat[3 * e + 1], se = T.mat[3 * e + 2];
        // curl H into E rows, -curl E into H rows (component blocks of D), conductivity on E
        auto vol = [&](int row, int col, int d, double sg) {
            for (int i = 0; i < Np; ++i)
                for (int j = 0; j < Np; ++j) B0[(row * Np + i) * R + col * Np + j] += sg * D[d][i * Np + j];
        };
        vol(0, 5, 1, ie); vol(0, 4, 2, -ie);    // Ex: dy Hz - dz Hy
        vol(1, 3, 2, ie); vol(1, 5, 0, -ie);    // Ey: dz Hx - dx Hz
        vol(2, 4, 0, ie); vol(2, 3, 1, -ie);    // Ez: dx Hy - dy Hx
        vol(3, 2, 1, -im); vol(3, 1, 2, im);    // Hx: -(dy Ez - dz Ey)
        vol(4, 0, 2, -im); vol(4, 2, 0, im);    // Hy: -(dz Ex - dx Ez)
        vol(5, 1, 0, -im); vol(5, 0, 1, im);    // Hz: -(dx Ey - dy Ex)
        for (int cmp = 0; cmp < 3; ++cmp)
            for (int i = 0; i < Np; ++i) B0[(cmp * Np + i) * R + cmp * Np + i] -= se;

        // ---- faces: Minv int phi F dS, F from the traces at each face point
        std::vector<double> W(36 * Np * Np), Wn(36 * Np * Np), tmp(Np * Np);
        for (int f = 0; f < 4; ++f) {
            const int64_t nb = T.nbr[4 * e + f];
            const int code = T.fcode[4 * e + f];
            if (code == FACE_TFSF_TF || code == FACE_TFSF_SF)
                throw std::runtime_error("TF/SF faces on curved elements are not supported");
            if (code == FACE_OPEN || code == FACE_SGBC) continue;   // SGBC: the injection's terms
            C.nbr[4 * c + f] = (code == FACE_INTERIOR) ? static_cast<int32_t>(nb) : -1;
            // the face's first element (lower index) parametrises it
            int64_t fe = e;
            int ff = f;
            if (nb >= 0 && nb < e) {
                fe = nb;
                ff = -1;
                for (int q = 0; q < 4; ++q) {
                    bool on_face = false;
                    for (int m = 0; m < 4; ++m)
                        if (m != f && T.elem_vertices[4 * e + m] == T.elem_vertices[4 * nb + q]) on_face = true;
                    if (!on_face) ff = q;   // the neighbour's vertex off the shared face
                }
                if (ff < 0) throw std::runtime_error("curved element: face not found on its neighbour");
            }
            int l1[3], le[3], ln[3] = {0, 0, 0}, k1 = 0;
            for (int q = 0; q < 4; ++q) if (q != ff) l1[k1++] = q;
            for (int k = 0; k < 3; ++k) {
                const int32_t gv = T.elem_vertices[4 * fe + l1[k]];
                le[k] = ln[k] = -1;
                for (int q = 0; q < 4; ++q) {
                    if (T.elem_vertices[4 * e + q] == gv) le[k] = q;
                    if (nb >= 0 && T.elem_vertices[4 * nb + q] == gv) ln[k] = q;
                }
                if (le[k] < 0 || (nb >= 0 && ln[k] < 0)) throw std::runtime_error("curved element: face vertices do not match");
            }
            const bool coupled = (code == FACE_INTERIOR);
            const std::vector<double>& te = face_table(le);
            const std::vector<double>* tn = coupled ? &face_table(ln) : nullptr;
            const double* nA = &T.fgeo[(4 * e + f) * 4];   // e's outward (affine) normal: orientation only
            const double* Gf = geo_of(fe);
            std::fill(W.begin(), W.end(), 0.0);
            std::fill(Wn.begin(), Wn.end(), 0.0);
            double du[3], dv[3];
            for (int r = 0; r < 3; ++r) {
                du[r] = kRefV[l1[1]][r] - kRefV[l1[0]][r];
                dv[r] = kRefV[l1[2]][r] - kRefV[l1[0]][r];
            }
            for (int k = 0; k < nfq; ++k) {
                const double bc[3] = {1.0 - fu[k] - fv[k], fu[k], fv[k]};
                double xf[3] = {0, 0, 0};
                for (int r = 0; r < 3; ++r)
                    for (int m = 0; m < 3; ++m) xf[r] += bc[m] * kRefV[l1[m]][r];
                double x[3], J[9], tu[3], tv[3];
                geom(T, fe, Gf, xf, x, J);
                for (int r = 0; r < 3; ++r) {
                    tu[r] = J[r * 3] * du[0] + J[r * 3 + 1] * du[1] + J[r * 3 + 2] * du[2];
                    tv[r] = J[r * 3] * dv[0] + J[r * 3 + 1] * dv[1] + J[r * 3 + 2] * dv[2];
                }
                double cr[3] = {tu[1] * tv[2] - tu[2] * tv[1], tu[2] * tv[0] - tu[0] * tv[2], tu[0] * tv[1] - tu[1] * tv[0]};
                if (cr[0] * nA[0] + cr[1] * nA[1] + cr[2] * nA[2] < 0.0) for (int r = 0; r < 3; ++r) cr[r] = -cr[r];
                const double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
                const double n[3] = {cr[0] / len, cr[1] / len, cr[2] / len};
                double Cm[36], Cp[36];
                flux_coeffs(code, n, alpha, Cm, Cp);
                const double* phi = &te[static_cast<size_t>(k) * Np];
                const double* pn = coupled ? &(*tn)[static_cast<size_t>(k) * Np] : nullptr;
                const double ds = fwt[k] * len;
                for (int rc = 0; rc < 36; ++rc) {
                    const double cm = ds * Cm[rc], cp = ds * Cp[rc];
                    if (cm != 0.0) {
                        double* w0 = &W[static_cast<size_t>(rc) * Np * Np];
                        for (int i = 0; i < Np; ++i) {
                            const double a = cm * phi[i];
                            for (int j = 0; j < Np; ++j) w0[i * Np + j] += a * phi[j];
                        }
                    }
                    if (coupled && cp != 0.0) {
                        double* w1 = &Wn[static_cast<size_t>(rc) * Np * Np];
                        for (int i = 0; i < Np; ++i) {
                            const double a = cp * phi[i];
                            for (int j = 0; j < Np; ++j) w1[i * Np + j] += a * pn[j];
                        }
                    }
                }
            }
            // B += scale(row) Minv W  (per component pair)
            double* Bf = &C.blocks[(static_cast<size_t>(c) * 5 + 1 + f) * R * R];
            for (int rc = 0; rc < 36; ++rc) {
                const int row = rc / 6, col = rc % 6;
                const double sc = row < 3 ? ie : im;
                for (int pass = 0; pass < (coupled ? 2 : 1); ++pass) {
                    const double* w = &(pass == 0 ? W : Wn)[static_cast<size_t>(rc) * Np * Np];
                    bool any = false;
                    for (int q = 0; q < Np * Np && !any; ++q) any = (w[q] != 0.0);
                    if (!any) continue;
                    matmul(Minv.data(), w, tmp.data(), Np, Np, Np);
                    double* B = pass == 0 ? B0 : Bf;
                    for (int i = 0; i < Np; ++i)
                        for (int j = 0; j < Np; ++j) B[(row * Np + i) * R + col * Np + j] += sc * tmp[i * Np + j];
                }
            }
        }
    };

    // elements in parallel (each writes its own blocks)
    const int nth = static_cast<int>(std::max<int64_t>(1, std::min<int64_t>(nc, std::max(1u, std::thread::hardware_concurrency()))));
    std::atomic<int64_t> next(0);
    std::exception_ptr err;
    std::mutex err_mu;
    auto worker = [&]() {
        for (;;) {
            const int64_t c = next.fetch_add(1);
            if (c >= nc) return;
            try {
                assemble(c);
            } catch (...) {
                std::lock_guard<std::mutex> lk(err_mu);
                if (!err) err = std::current_exception();
                next.store(nc);
                return;
            }
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nth; ++t) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
    if (err) std::rethrow_exception(err);
    return C;
}

namespace {

// the geometry of element e (second-order nodes when it is curved)
const double* curved_geometry(const MeshTables& T, int64_t e)
{
    for (size_t c = 0; c < T.curved_elems.size(); ++c)
        if (T.curved_elems[c] == e) return &T.curved_nodes[30 * c];
    return nullptr;
}

}  // namespace

void element_face_normal(const MeshTables& T, int64_t e, int f, const double* l, double* n)
{
    int l1[3], k1 = 0;
    for (int q = 0; q < 4; ++q) if (q != f) l1[k1++] = q;
    const double xi[3] = {l[1], l[2], l[3]};
    double x[3], J[9], tu[3], tv[3];
    geom(T, e, curved_geometry(T, e), xi, x, J);
    for (int r = 0; r < 3; ++r) {
        tu[r] = tv[r] = 0.0;
        for (int d = 0; d < 3; ++d) {
            tu[r] += J[r * 3 + d] * (kRefV[l1[1]][d] - kRefV[l1[0]][d]);
            tv[r] += J[r * 3 + d] * (kRefV[l1[2]][d] - kRefV[l1[0]][d]);
        }
    }
    double cr[3] = {tu[1] * tv[2] - tu[2] * tv[1], tu[2] * tv[0] - tu[0] * tv[2], tu[0] * tv[1] - tu[1] * tv[0]};
    const double* nA = &T.fgeo[(4 * e + f) * 4];
    if (cr[0] * nA[0] + cr[1] * nA[1] + cr[2] * nA[2] < 0.0) for (int r = 0; r < 3; ++r) cr[r] = -cr[r];
    const double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    for (int r = 0; r < 3; ++r) n[r] = cr[r] / len;
}

void build_curved_sgbc_face(const MeshTables& T, const RefTet& ref, double alpha, int64_t e, int f,
                            std::vector<double>& Bm, std::vector<double>& Bp)
{
    const int Np = ref.Np, Nfp = ref.Nfp, R = 6 * Np;
    const double* G = curved_geometry(T, e);
    std::vector<double> g, gw;
    gauss_legendre01(ref.p + 4, g, gw);
    const int ng = static_cast<int>(g.size());
    // mass matrix on e's map
    std::vector<double> M(Np * Np, 0.0), phi(Np), pf(Nfp);
    for (int a = 0; a < ng; ++a)
        for (int b = 0; b < ng; ++b)
            for (int q = 0; q < ng; ++q) {
                const double u = g[a], v = g[b], w = g[q];
                const double xi[3] = {u * (1 - v) * (1 - w), v * (1 - w), w};
                double x[3], J[9], Ji[9];
                geom(T, e, G, xi, x, J);
                const double ww = gw[a] * gw[b] * gw[q] * (1 - v) * (1 - w) * (1 - w) * inv3(J, Ji);
                basis(ref, xi, phi.data());
                for (int i = 0; i < Np; ++i)
                    for (int j = 0; j < Np; ++j) M[i * Np + j] += ww * phi[i] * phi[j];
            }
    std::vector<double> Minv = M;
    if (!invert_matrix(Minv, Np)) throw std::runtime_error("singular curved-element mass matrix");
    // the face parametrised from its first element (lower index), as the rows
    const int64_t nb = T.nbr[4 * e + f];
    int64_t fe = e;
    int ff = f;
    if (nb >= 0 && nb < e) {
        fe = nb;
        ff = -1;
        for (int q = 0; q < 4; ++q) {
            bool on_face = false;
            for (int m = 0; m < 4; ++m)
                if (m != f && T.elem_vertices[4 * e + m] == T.elem_vertices[4 * nb + q]) on_face = true;
            if (!on_face) ff = q;
        }
    }
    int l1[3], le[3], k1 = 0;
    for (int q = 0; q < 4; ++q) if (q != ff) l1[k1++] = q;
    for (int k = 0; k < 3; ++k) {
        const int32_t gv = T.elem_vertices[4 * fe + l1[k]];
        le[k] = -1;
        for (int q = 0; q < 4; ++q) if (T.elem_vertices[4 * e + q] == gv) le[k] = q;
        if (le[k] < 0) throw std::runtime_error("curved SGBC face: vertices do not match");
    }
    const double* Gf = (fe == e) ? G : curved_geometry(T, fe);
    const double* nA = &T.fgeo[(4 * e + f) * 4];
    std::vector<double> Wm(36 * Np * Np, 0.0), Wp(36 * Np * Nfp, 0.0);
    double du[3], dv[3];
    for (int r = 0; r < 3; ++r) {
        du[r] = kRefV[l1[1]][r] - kRefV[l1[0]][r];
        dv[r] = kRefV[l1[2]][r] - kRefV[l1[0]][r];
    }
    for (int a = 0; a < ng; ++a)
        for (int b = 0; b < ng; ++b) {
            const double u = g[a] * (1 - g[b]), v = g[b], wt = gw[a] * gw[b] * (1 - g[b]);
            const double bc[3] = {1.0 - u - v, u, v};
            double xf[3] = {0, 0, 0}, xe[3] = {0, 0, 0};
            for (int r = 0; r < 3; ++r)
                for (int m = 0; m < 3; ++m) { xf[r] += bc[m] * kRefV[l1[m]][r]; xe[r] += bc[m] * kRefV[le[m]][r]; }
            double x[3], J[9], tu[3], tv[3];
            geom(T, fe, Gf, xf, x, J);
            for (int r = 0; r < 3; ++r) {
                tu[r] = J[r * 3] * du[0] + J[r * 3 + 1] * du[1] + J[r * 3 + 2] * du[2];
                tv[r] = J[r * 3] * dv[0] + J[r * 3 + 1] * dv[1] + J[r * 3 + 2] * dv[2];
            }
            double cr[3] = {tu[1] * tv[2] - tu[2] * tv[1], tu[2] * tv[0] - tu[0] * tv[2], tu[0] * tv[1] - tu[1] * tv[0]};
            if (cr[0] * nA[0] + cr[1] * nA[1] + cr[2] * nA[2] < 0.0) for (int r = 0; r < 3; ++r) cr[r] = -cr[r];
            const double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
            const double n[3] = {cr[0] / len, cr[1] / len, cr[2] / len};
            double Cm[36], Cp[36];
            flux_coeffs(FACE_INTERIOR, n, alpha, Cm, Cp);
            basis(ref, xe, phi.data());
            for (int q = 0; q < Nfp; ++q) pf[q] = phi[ref.Fmask[f * Nfp + q]];   // e's face-node basis
            const double ds = wt * len;
            for (int rc = 0; rc < 36; ++rc) {
                const double cm = ds * Cm[rc], cp = ds * Cp[rc];
                if (cm != 0.0)
                    for (int i = 0; i < Np; ++i)
                        for (int j = 0; j < Np; ++j) Wm[(static_cast<size_t>(rc) * Np + i) * Np + j] += cm * phi[i] * phi[j];
                if (cp != 0.0)
                    for (int i = 0; i < Np; ++i)
                        for (int q = 0; q < Nfp; ++q) Wp[(static_cast<size_t>(rc) * Np + i) * Nfp + q] += cp * phi[i] * pf[q];
            }
        }
    const double ie = T.mat[3 * e], im = T.mat[3 * e + 1];
    Bm.assign(static_cast<size_t>(R) * R, 0.0);
    Bp.assign(static_cast<size_t>(R) * 6 * Nfp, 0.0);
    std::vector<double> tmp(static_cast<size_t>(Np) * std::max(Np, Nfp));
    for (int rc = 0; rc < 36; ++rc) {
        const int row = rc / 6, col = rc % 6;
        const double sc = row < 3 ? ie : im;
        matmul(Minv.data(), &Wm[static_cast<size_t>(rc) * Np * Np], tmp.data(), Np, Np, Np);
        for (int i = 0; i < Np; ++i)
            for (int j = 0; j < Np; ++j) Bm[(row * Np + i) * static_cast<size_t>(R) + col * Np + j] += sc * tmp[i * Np + j];
        matmul(Minv.data(), &Wp[static_cast<size_t>(rc) * Np * Nfp], tmp.data(), Np, Np, Nfp);
        for (int i = 0; i < Np; ++i)
            for (int q = 0; q < Nfp; ++q)
                Bp[(row * Np + i) * static_cast<size_t>(6 * Nfp) + col * Nfp + q] += sc * tmp[i * Nfp + q];
    }
}

}  // namespace dgtd
