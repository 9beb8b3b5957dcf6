// Thin-layer boundaries (SGBC): sub-solver operators, sub-step maps and face node pairs.
#include "sgbc.hpp"

#include "curved.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>
#include <unordered_map>

namespace dgtd {

namespace {

// Sub-solver vertex kinds: 0 interior, 1/2/3 PEC/PMC/SMA sheet, 4 SMA end.
constexpr int kVertexEnd = 4;

struct Seg1D {
    const SgbcStack1D* S;
    RefSeg ref;
    std::vector<double> h, ie, im, se;   // per segment: width, 1/eps, 1/mu, sigma/eps
    std::vector<int> vkind;              // per vertex
};

// dU/dt of the sub-solver's nodal DG form (upwind alpha 1), the 1D restriction of the 3D
// stage kernel: only x-derivatives, face normals -1 (left end) and +1 (right end),
// Fscale = 2 / width.
void apply_1d(const Seg1D& D, const double* u, double* out)
{
    const SgbcStack1D& S = *D.S;
    const int Np = S.Np1;
    const int64_t L = S.local;
    const RefSeg& R = D.ref;
    for (int64_t e = 0; e < S.K1; ++e) {
        const double rx = 2.0 / D.h[e];
        double fl[2][6];
        for (int f = 0; f < 2; ++f) {
            const int vm = (f == 0) ? 0 : Np - 1;
            const int64_t vert = e + f;
            const double nx = (f == 0) ? -1.0 : 1.0;
            double uM[6], dE[3], dH[3];
            for (int c = 0; c < 6; ++c) uM[c] = u[c * L + e * Np + vm];
            double aE = 1.0, aH = 1.0;
            const int kind = D.vkind[vert];
            if (kind == 0) {
                const int64_t nb = (f == 0) ? (e - 1) * Np + (Np - 1) : (e + 1) * Np;
                for (int c = 0; c < 3; ++c) { dE[c] = u[c * L + nb] - uM[c]; dH[c] = u[(c + 3) * L + nb] - uM[c + 3]; }
            } else if (kind == 1) {
                for (int c = 0; c < 3; ++c) { dE[c] = -2.0 * uM[c]; dH[c] = 0.0; }
            } else if (kind == 2) {
                for (int c = 0; c < 3; ++c) { dE[c] = 0.0; dH[c] = -2.0 * uM[c + 3]; }
            } else {   // SMA sheet or SMA end: penalty 1
                for (int c = 0; c < 3; ++c) { dE[c] = -uM[c]; dH[c] = -uM[c + 3]; }
            }
            const double ny = 0.0, nz = 0.0;
            const double ndE = nx * dE[0], ndH = nx * dH[0];
            const double hf = 0.5 * rx;   // 0.5 * Fscale
            fl[f][0] = hf * ((ny * dH[2] - nz * dH[1]) + aE * (dE[0] - ndE * nx));
            fl[f][1] = hf * ((nz * dH[0] - nx * dH[2]) + aE * (dE[1] - ndE * ny));
            fl[f][2] = hf * ((nx * dH[1] - ny * dH[0]) + aE * (dE[2] - ndE * nz));
            fl[f][3] = hf * (-(ny * dE[2] - nz * dE[1]) + aH * (dH[0] - ndH * nx));
            fl[f][4] = hf * (-(nz * dE[0] - nx * dE[2]) + aH * (dH[1] - ndH * ny));
            fl[f][5] = hf * (-(nx * dE[1] - ny * dE[0]) + aH * (dH[2] - ndH * nz));
        }
        for (int i = 0; i < Np; ++i) {
            double d[6], lf[6];
            for (int c = 0; c < 6; ++c) {
                double a = 0.0;
                for (int j = 0; j < Np; ++j) a += R.Dr[i * Np + j] * u[c * L + e * Np + j];
                d[c] = rx * a;
                lf[c] = R.LIFT[i * 2 + 0] * fl[0][c] + R.LIFT[i * 2 + 1] * fl[1][c];
            }
            const int64_t o = e * Np + i;
            // curl H = (0, -dHz/dx, dHy/dx), curl E = (0, -dEz/dx, dEy/dx)
            out[0 * L + o] = D.ie[e] * lf[0] - D.se[e] * u[0 * L + o];
            out[1 * L + o] = D.ie[e] * (-d[5] + lf[1]) - D.se[e] * u[1 * L + o];
            out[2 * L + o] = D.ie[e] * (d[4] + lf[2]) - D.se[e] * u[2 * L + o];
            out[3 * L + o] = D.im[e] * lf[3];
            out[4 * L + o] = D.im[e] * (d[2] + lf[4]);
            out[5 * L + o] = D.im[e] * (-d[1] + lf[5]);
        }
    }
}

// c = a * b, all n x n row-major
void mm(const std::vector<double>& a, const std::vector<double>& b, std::vector<double>& c, int64_t n, int64_t m = -1)
{
    // a: n x k (k = n), b: k x m
    if (m < 0) m = n;
    c.assign(n * m, 0.0);
    for (int64_t i = 0; i < n; ++i)
        for (int64_t k = 0; k < n; ++k) {
            const double aik = a[i * n + k];
            if (aik == 0.0) continue;
            const double* br = &b[k * m];
            double* cr = &c[i * m];
            for (int64_t j = 0; j < m; ++j) cr[j] += aik * br[j];
        }
}

// B <- M^-1 B for n x n M (destroyed) and n x m B, Gaussian elimination with partial pivoting.
void solve_rows(std::vector<double>& M, std::vector<double>& B, int64_t n, int64_t m)
{
    for (int64_t c = 0; c < n; ++c) {
        int64_t pr = c;
        double best = std::fabs(M[c * n + c]);
        for (int64_t r = c + 1; r < n; ++r)
            if (std::fabs(M[r * n + c]) > best) { best = std::fabs(M[r * n + c]); pr = r; }
        if (!(best > 0.0)) throw std::runtime_error("singular SGBC sub-step matrix");
        if (pr != c) {
            for (int64_t q = 0; q < n; ++q) std::swap(M[c * n + q], M[pr * n + q]);
            for (int64_t q = 0; q < m; ++q) std::swap(B[c * m + q], B[pr * m + q]);
        }
        const double d = M[c * n + c];
        for (int64_t r = c + 1; r < n; ++r) {
            const double f = M[r * n + c] / d;
            if (f == 0.0) continue;
            for (int64_t q = c; q < n; ++q) M[r * n + q] -= f * M[c * n + q];
            for (int64_t q = 0; q < m; ++q) B[r * m + q] -= f * B[c * m + q];
        }
    }
    for (int64_t r = n - 1; r >= 0; --r) {
        for (int64_t q = r + 1; q < n; ++q) {
            const double f = M[r * n + q];
            if (f == 0.0) continue;
            for (int64_t j = 0; j < m; ++j) B[r * m + j] -= f * B[q * m + j];
        }
        const double d = M[r * n + r];
        for (int64_t j = 0; j < m; ++j) B[r * m + j] /= d;
    }
}

// One SDIRK33 step of the linear sub-solver as a matrix: x <- S x (Alexander's L-stable
// three-stage tableau, the method of the reference's sub-solver, SolverExtension.cpp:163-170).
std::vector<double> sdirk_matrix(const SgbcStack1D& S, double h)
{
    const int64_t n = S.n;
    std::vector<double> I(n * n, 0.0);
    for (int64_t i = 0; i < n; ++i) I[i * n + i] = 1.0;
    if (std::fabs(h) < 1e-9) return I;   // the sub-solver takes no step below 1e-9
    const double g = 0.43586652150845899941601945;   // root of 6x^3 - 18x^2 + 9x - 1 in (1/6, 1/2)
    const double a21 = 0.5 * (1.0 - g);
    const double b1 = -(6.0 * g * g - 16.0 * g + 1.0) / 4.0;
    const double b2 = (6.0 * g * g - 20.0 * g + 5.0) / 4.0;
    // K = (I - g h A)^-1 A
    std::vector<double> M(n * n), K = S.A;
    for (int64_t i = 0; i < n * n; ++i) M[i] = -g * h * S.A[i];
    for (int64_t i = 0; i < n; ++i) M[i * n + i] += 1.0;
    solve_rows(M, K, n, n);
    // stage 1: k1 = K x; y = x + a21 h k1; x1 = x + b1 h k1
    // stage 2: k2 = K y; x2 = x1 + b2 h k2
    // stage 3: k3 = K x2; x3 = x2 + g h k3
    std::vector<double> Y(n * n), K2, X2(n * n), K3, Sx(n * n);
    for (int64_t i = 0; i < n * n; ++i) Y[i] = I[i] + a21 * h * K[i];
    mm(K, Y, K2, n);
    for (int64_t i = 0; i < n * n; ++i) X2[i] = I[i] + b1 * h * K[i] + b2 * h * K2[i];
    mm(K, X2, K3, n);
    for (int64_t i = 0; i < n * n; ++i) Sx[i] = X2[i] + g * h * K3[i];
    return Sx;
}

// Ghost DOF groups: 12 groups (left E,H components, then right), each the component's first
// (left) or last (right) nghost * (p+1) nodes.
template <typename Fn>
void for_ghosts(const SgbcStack1D& S, Fn&& fn)
{
    const int64_t tg = static_cast<int64_t>(S.nghost) * S.Np1, L = S.local;
    for (int c = 0; c < 6; ++c)
        for (int64_t q = 0; q < tg; ++q) {
            fn(c, c * L + q);
            fn(6 + c, c * L + (L - 1 - q));
        }
}

// SP = S with the ghost columns cleared, SQ[:, grp] = sum of S's columns of group grp.
void split_ghosts(const SgbcStack1D& S, const std::vector<double>& Sx, std::vector<double>& SP, std::vector<double>& SQ)
{
    const int64_t n = S.n;
    SP = Sx;
    SQ.assign(n * 12, 0.0);
    for_ghosts(S, [&](int grp, int64_t col) {
        for (int64_t i = 0; i < n; ++i) {
            SQ[i * 12 + grp] += Sx[i * n + col];
            SP[i * n + col] = 0.0;
        }
    });
}

}  // namespace

int sgbc_nsteps(double sub_dt, double span)
{
    return (sub_dt > 0.0 && sub_dt < span) ? static_cast<int>(std::ceil(span / sub_dt)) : 1;
}

void sgbc_rotation(const double* normal, double* R)
{
    double nx = normal[0], ny = normal[1], nz = normal[2];
    const double len = std::sqrt(nx * nx + ny * ny + nz * nz);
    nx /= len; ny /= len; nz /= len;
    R[0] = nx; R[1] = ny; R[2] = nz;
    // first tangent: n x ref with ref = x unless n is close to x
    double rx = 0.0, ry = 0.0, rz = 0.0;
    if (std::fabs(nx) < 0.9) rx = 1.0; else ry = 1.0;
    double t1x = ny * rz - nz * ry, t1y = nz * rx - nx * rz, t1z = nx * ry - ny * rx;
    const double tl = std::sqrt(t1x * t1x + t1y * t1y + t1z * t1z);
    t1x /= tl; t1y /= tl; t1z /= tl;
    R[3] = t1x; R[4] = t1y; R[5] = t1z;
    R[6] = ny * t1z - nz * t1y; R[7] = nz * t1x - nx * t1z; R[8] = nx * t1y - ny * t1x;
}

SgbcStack1D build_sgbc_stack(const SgbcStackSpec& spec)
{
    if (spec.layers.empty()) throw std::invalid_argument("an SGBC stack needs at least one layer");
    for (int bc : {spec.left_bc, spec.right_bc})
        if (bc < 0 || bc > 3) throw std::invalid_argument("SGBC stack boundary must be 0 (none), 1 PEC, 2 PMC or 3 SMA");
    SgbcStack1D S;
    S.spec = spec;
    int64_t nseg = 0;
    double width = 0.0;
    int p = 1;
    for (const auto& L : spec.layers) {
        if (L.segments < 1 || !(L.width > 0.0) || L.order < 1 || L.order > 16 || !(L.eps > 0.0) || !(L.mu > 0.0) ||
            !(L.sigma >= 0.0))
            throw std::invalid_argument("SGBC layer needs segments >= 1, width > 0, order 1..16, eps, mu > 0, sigma >= 0");
        nseg += L.segments;
        width += L.width;
        p = std::max(p, L.order);
    }
    S.p = p; S.Np1 = p + 1; S.nghost = std::max(3, p + 1);
    S.K1 = nseg + 2 * S.nghost;
    S.local = S.K1 * S.Np1;
    S.n = 6 * S.local;
    if (S.n > kSgbcMaxDofs)
        throw std::invalid_argument("SGBC sub-solver of " + std::to_string(S.n) + " unknowns is above the dense limit of " +
                                    std::to_string(kSgbcMaxDofs) + " (the reference iterates with GMRES there)");
    S.idx_left = static_cast<int64_t>(S.nghost) * S.Np1;
    S.idx_right = S.local - 1 - S.idx_left;

    Seg1D D;
    D.S = &S;
    D.ref = build_ref_seg(p);
    const double gdx = width / static_cast<double>(nseg);
    // vertex coordinates as the reference builds them (ghosts, layers, ghosts), widths from them
    std::vector<double> xs;
    for (int i = 0; i <= S.nghost; ++i) xs.push_back(i * gdx);
    double x = S.nghost * gdx;
    for (const auto& L : spec.layers) {
        const double dx = L.width / L.segments;
        for (int i = 0; i < L.segments; ++i) { x += dx; xs.push_back(x); }
    }
    for (int i = 1; i <= S.nghost; ++i) xs.push_back(x + i * gdx);
    D.h.resize(S.K1); D.ie.assign(S.K1, 1.0); D.im.assign(S.K1, 1.0); D.se.assign(S.K1, 0.0);
    for (int64_t e = 0; e < S.K1; ++e) {
        D.h[e] = xs[e + 1] - xs[e];
        if (!(D.h[e] > 0.0)) throw std::invalid_argument("SGBC sub-solver segment of non-positive width");
    }
    int64_t e = S.nghost;
    for (const auto& L : spec.layers)
        for (int i = 0; i < L.segments; ++i, ++e) { D.ie[e] = 1.0 / L.eps; D.im[e] = 1.0 / L.mu; D.se[e] = L.sigma / L.eps; }
    D.vkind.assign(S.K1 + 1, 0);
    D.vkind[0] = kVertexEnd;
    D.vkind[S.K1] = kVertexEnd;
    if (spec.left_bc) D.vkind[S.nghost] = spec.left_bc;
    if (spec.right_bc) D.vkind[S.nghost + nseg] = spec.right_bc;

    const int64_t n = S.n;
    S.A.assign(n * n, 0.0);
    std::vector<double> u(n, 0.0), out(n);
    for (int64_t j = 0; j < n; ++j) {
        u[j] = 1.0;
        apply_1d(D, u.data(), out.data());
        for (int64_t i = 0; i < n; ++i) S.A[i * n + j] = out[i];
        u[j] = 0.0;
    }
    return S;
}

SgbcStageMap sgbc_stage_map(const SgbcStack1D& S, double span, int nsteps)
{
    const int64_t n = S.n;
    std::vector<double> SP, SQ;
    split_ghosts(S, sdirk_matrix(S, span / nsteps), SP, SQ);
    // W = E (SP)^j, starting from the interface rows
    std::vector<double> W(12 * n, 0.0), W2;
    for (int c = 0; c < 6; ++c) {
        W[c * n + c * S.local + S.idx_left] = 1.0;
        W[(6 + c) * n + c * S.local + S.idx_right] = 1.0;
    }
    SgbcStageMap M;
    M.G.assign(144, 0.0);
    for (int j = 0; j < nsteps; ++j) {
        for (int r = 0; r < 12; ++r)
            for (int64_t k = 0; k < n; ++k) {
                const double w = W[r * n + k];
                if (w == 0.0) continue;
                for (int c = 0; c < 12; ++c) M.G[r * 12 + c] += w * SQ[k * 12 + c];
            }
        W2.assign(12 * n, 0.0);
        for (int r = 0; r < 12; ++r)
            for (int64_t k = 0; k < n; ++k) {
                const double w = W[r * n + k];
                if (w == 0.0) continue;
                for (int64_t c = 0; c < n; ++c) W2[r * n + c] += w * SP[k * n + c];
            }
        W.swap(W2);
    }
    M.R = W;
    return M;
}

SgbcFinalMap sgbc_final_map(const SgbcStack1D& S, double span, int nsteps)
{
    const int64_t n = S.n;
    std::vector<double> SP, SQ;
    split_ghosts(S, sdirk_matrix(S, span / nsteps), SP, SQ);
    std::vector<double> F(n * n, 0.0), Vo(n * 12, 0.0), Vn(n * 12, 0.0), T;
    for (int64_t i = 0; i < n; ++i) F[i * n + i] = 1.0;
    for (int k = 0; k < nsteps; ++k) {
        const double a = static_cast<double>(k + 1) / nsteps, b = 1.0 - a;
        mm(SP, F, T, n); F.swap(T);
        mm(SP, Vo, T, n, 12); Vo.swap(T);
        mm(SP, Vn, T, n, 12); Vn.swap(T);
        for (int64_t i = 0; i < n * 12; ++i) { Vo[i] += b * SQ[i]; Vn[i] += a * SQ[i]; }
    }
    SgbcFinalMap M;
    M.FT.resize(n * n);
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = 0; j < n; ++j) M.FT[j * n + i] = F[i * n + j];
    M.Vo = std::move(Vo);
    M.Vn = std::move(Vn);
    return M;
}

SgbcLayout build_sgbc_layout(const MeshTables& T, const RefTet& ref, const std::vector<int32_t>& face_stack,
                             int n_stacks)
{
    const int64_t nf = static_cast<int64_t>(T.sgbc_faces.size() / 4);
    if (static_cast<int64_t>(face_stack.size()) != nf)
        throw std::invalid_argument("SGBC: one stack index per SGBC face is needed (" + std::to_string(nf) + " faces)");
    const int Np = T.Np, Nfp = T.Nfp;
    SgbcLayout Lo;
    struct Ent { int32_t e, f, role, q; };
    std::vector<Ent> ents;
    std::unordered_map<int64_t, int32_t> pair_of_gr;
    std::vector<char> curved(T.K, 0);
    for (int32_t e : T.curved_elems) curved[e] = 1;
    for (int64_t q = 0; q < nf; ++q) {
        const int32_t e1 = T.sgbc_faces[4 * q], f1 = T.sgbc_faces[4 * q + 1];
        const int32_t e2 = T.sgbc_faces[4 * q + 2], f2 = T.sgbc_faces[4 * q + 3];
        const int32_t st = face_stack[q];
        if (st < 0 || st >= n_stacks) throw std::invalid_argument("SGBC: face stack index out of range");
        double R[9];
        sgbc_rotation(&T.fgeo[(static_cast<int64_t>(e1) * 4 + f1) * 4], R);
        const bool curved_face = curved[e1] || curved[e2];
        for (int a = 0; a < Nfp; ++a) {
            const int64_t gl = static_cast<int64_t>(e1) * Np + ref.Fmask[f1 * Nfp + a];
            if (curved_face) {   // per-node normal on a curved face (the reference's per-DOF normals)
                double n[3];
                element_face_normal(T, e1, f1, &ref.bary[4 * ref.Fmask[f1 * Nfp + a]], n);
                sgbc_rotation(n, R);
            }
            const int64_t gr = T.vmapP[(static_cast<int64_t>(e1) * 4 + f1) * Nfp + a];
            if (gr / Np != e2) throw std::runtime_error("SGBC: face node partner outside the face's second element");
            const int32_t pid = static_cast<int32_t>(Lo.gl.size());
            Lo.gl.push_back(static_cast<int32_t>(gl));
            Lo.gr.push_back(static_cast<int32_t>(gr));
            Lo.stack.push_back(st);
            Lo.rot.insert(Lo.rot.end(), R, R + 9);
            if (!pair_of_gr.emplace(gr, pid).second) throw std::runtime_error("SGBC: two pairs share a node");
        }
        ents.push_back({e1, f1, 0, static_cast<int32_t>(q)});
        ents.push_back({e2, f2, 1, static_cast<int32_t>(q)});
    }
    std::stable_sort(ents.begin(), ents.end(), [](const Ent& a, const Ent& b) { return a.e < b.e; });
    for (size_t i = 0; i < ents.size(); ++i) {
        const Ent& E = ents[i];
        if (Lo.el_elem.empty() || Lo.el_elem.back() != E.e) {
            Lo.el_elem.push_back(E.e);
            Lo.el_start.push_back(static_cast<int32_t>(i));
        }
        Lo.ent_face.push_back(E.f);
        Lo.ent_role.push_back(E.role);
        for (int a = 0; a < Nfp; ++a) {
            if (E.role == 0) {
                Lo.ent_pairs.push_back(static_cast<int32_t>(E.q * Nfp + a));
            } else {
                const int64_t g2 = static_cast<int64_t>(E.e) * Np + ref.Fmask[E.f * Nfp + a];
                auto it = pair_of_gr.find(g2);
                if (it == pair_of_gr.end()) throw std::runtime_error("SGBC: second-side face node without a pair");
                Lo.ent_pairs.push_back(it->second);
            }
        }
    }
    Lo.el_start.push_back(static_cast<int32_t>(ents.size()));
    for (size_t i = 0; i + 1 < Lo.el_start.size(); ++i)
        if (Lo.el_start[i + 1] - Lo.el_start[i] > 4) throw std::runtime_error("SGBC: more than four SGBC faces on an element");
    return Lo;
}

}  // namespace dgtd
