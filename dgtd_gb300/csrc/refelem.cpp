// Reference-element construction (FP64). See refelem.hpp for the conventions.
#include "refelem.hpp"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace dgtd {

// Legendre P_n and P_n' by the three-term recurrence.
static void legendre(int n, double x, double& pn, double& dpn)
{
    double p0 = 1.0, p1 = x;
    if (n == 0) { pn = 1.0; dpn = 0.0; return; }
    for (int k = 2; k <= n; ++k) {
        double pk = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = pk;
    }
    pn = p1;
    // P_n'(x) = n (x P_n - P_{n-1}) / (x^2 - 1), valid away from +-1
    dpn = n * (x * p1 - p0) / (x * x - 1.0);
}

std::vector<double> gauss_lobatto(int p)
{
    std::vector<double> x(p + 1);
    if (p == 0) { x[0] = 0.0; return x; }
    x[0] = -1.0; x[p] = 1.0;
    // Interior points: roots of P_p'. Newton from Chebyshev-Lobatto guesses,
    // using (1-x^2) P_p' = p (P_{p-1} - x P_p) and its derivative
    // d/dx[(1-x^2)P_p'] = -p(p+1) P_p.
    for (int i = 1; i < p; ++i) {
        double xi = -std::cos(M_PI * i / p);
        for (int it = 0; it < 100; ++it) {
            double pn, dpn;
            legendre(p, xi, pn, dpn);
            double p0 = 1.0, p1 = xi;           // P_{p-1}
            for (int k = 2; k <= p - 1; ++k) {
                double pk = ((2.0 * k - 1.0) * xi * p1 - (k - 1.0) * p0) / k;
                p0 = p1; p1 = pk;
            }
            double pm1 = (p == 1) ? 1.0 : p1;
            double f = p * (pm1 - xi * pn);       // (1-x^2) P_p'
            double df = -p * (p + 1.0) * pn;
            double dx = f / df;
            xi -= dx;
            if (std::fabs(dx) < 1e-16) break;
        }
        x[i] = xi;
    }
    // enforce exact symmetry
    for (int i = 0; i <= p / 2; ++i) {
        double v = 0.5 * (x[p - i] - x[i]);
        x[i] = -v; x[p - i] = v;
    }
    if (p % 2 == 0) x[p / 2] = 0.0;
    return x;
}

double jacobi_p(double x, double alpha, double beta, int n)
{
    double g0 = std::pow(2.0, alpha + beta + 1.0) / (alpha + beta + 1.0) *
                std::tgamma(alpha + 1.0) * std::tgamma(beta + 1.0) / std::tgamma(alpha + beta + 1.0);
    double p0 = 1.0 / std::sqrt(g0);
    if (n == 0) return p0;
    double g1 = (alpha + 1.0) * (beta + 1.0) / (alpha + beta + 3.0) * g0;
    double p1 = ((alpha + beta + 2.0) * x / 2.0 + (alpha - beta) / 2.0) / std::sqrt(g1);
    if (n == 1) return p1;
    double aold = 2.0 / (2.0 + alpha + beta) *
                  std::sqrt((alpha + 1.0) * (beta + 1.0) / (alpha + beta + 3.0));
    for (int i = 1; i < n; ++i) {
        double h1 = 2.0 * i + alpha + beta;
        double anew = 2.0 / (h1 + 2.0) *
                      std::sqrt((i + 1.0) * (i + 1.0 + alpha + beta) * (i + 1.0 + alpha) *
                                (i + 1.0 + beta) / (h1 + 1.0) / (h1 + 3.0));
        double bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2.0);
        double p2 = 1.0 / anew * (-aold * p0 + (x - bnew) * p1);
        aold = anew; p0 = p1; p1 = p2;
    }
    return p1;
}

double grad_jacobi_p(double x, double alpha, double beta, int n)
{
    if (n == 0) return 0.0;
    return std::sqrt(n * (n + alpha + beta + 1.0)) * jacobi_p(x, alpha + 1.0, beta + 1.0, n - 1);
}

bool invert_matrix(std::vector<double>& a, int n)
{
    std::vector<int> piv(n);
    std::vector<double> inv(static_cast<size_t>(n) * n, 0.0);
    for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
    for (int c = 0; c < n; ++c) {
        int best = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(a[r * n + c]) > std::fabs(a[best * n + c])) best = r;
        if (std::fabs(a[best * n + c]) < 1e-300) return false;
        if (best != c) {
            for (int k = 0; k < n; ++k) {
                std::swap(a[c * n + k], a[best * n + k]);
                std::swap(inv[c * n + k], inv[best * n + k]);
            }
        }
        double d = 1.0 / a[c * n + c];
        for (int k = 0; k < n; ++k) { a[c * n + k] *= d; inv[c * n + k] *= d; }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = a[r * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) {
                a[r * n + k] -= f * a[c * n + k];
                inv[r * n + k] -= f * inv[c * n + k];
            }
        }
    }
    a.swap(inv);
    return true;
}

void matmul(const double* a, const double* b, double* c, int m, int k, int n)
{
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < n; ++j) {
            double acc = 0.0;
            for (int l = 0; l < k; ++l) acc += a[i * k + l] * b[l * n + j];
            c[i * n + j] = acc;
        }
}

// ---- PKDO basis on the reference triangle / tetrahedron ---------------------

static double simplex2d(double r, double s, int i, int j)
{
    double a = (std::fabs(1.0 - s) > 1e-12) ? 2.0 * (1.0 + r) / (1.0 - s) - 1.0 : -1.0;
    double b = s;
    double h1 = jacobi_p(a, 0.0, 0.0, i);
    double h2 = jacobi_p(b, 2.0 * i + 1.0, 0.0, j);
    return std::sqrt(2.0) * h1 * h2 * std::pow(1.0 - b, i);
}

static void rst_to_abc(double r, double s, double t, double& a, double& b, double& c)
{
    a = (std::fabs(s + t) > 1e-12) ? 2.0 * (1.0 + r) / (-s - t) - 1.0 : -1.0;
    b = (std::fabs(t - 1.0) > 1e-12) ? 2.0 * (1.0 + s) / (1.0 - t) - 1.0 : -1.0;
    c = t;
}

static double simplex3d(double r, double s, double t, int i, int j, int k)
{
    double a, b, c;
    rst_to_abc(r, s, t, a, b, c);
    double h1 = jacobi_p(a, 0.0, 0.0, i);
    double h2 = jacobi_p(b, 2.0 * i + 1.0, 0.0, j);
    double h3 = jacobi_p(c, 2.0 * (i + j) + 2.0, 0.0, k);
    return 2.0 * std::sqrt(2.0) * h1 * h2 * std::pow(1.0 - b, i) * h3 * std::pow(1.0 - c, i + j);
}

static void grad_simplex3d(double r, double s, double t, int i, int j, int k,
                           double& dr, double& ds, double& dt)
{
    double a, b, c;
    rst_to_abc(r, s, t, a, b, c);
    double fa = jacobi_p(a, 0.0, 0.0, i), dfa = grad_jacobi_p(a, 0.0, 0.0, i);
    double gb = jacobi_p(b, 2.0 * i + 1.0, 0.0, j), dgb = grad_jacobi_p(b, 2.0 * i + 1.0, 0.0, j);
    double hc = jacobi_p(c, 2.0 * (i + j) + 2.0, 0.0, k);
    double dhc = grad_jacobi_p(c, 2.0 * (i + j) + 2.0, 0.0, k);
    double hb = 0.5 * (1.0 - b), hcc = 0.5 * (1.0 - c);

    dr = dfa * gb * hc;
    if (i > 0) dr *= std::pow(hb, i - 1);
    if (i + j > 0) dr *= std::pow(hcc, i + j - 1);

    ds = 0.5 * (1.0 + a) * dr;
    double tmp = dgb * std::pow(hb, i);
    if (i > 0) tmp += -0.5 * i * gb * std::pow(hb, i - 1);
    if (i + j > 0) tmp *= std::pow(hcc, i + j - 1);
    tmp = fa * tmp * hc;
    ds += tmp;

    dt = 0.5 * (1.0 + a) * dr + 0.5 * (1.0 + b) * tmp;
    tmp = dhc * std::pow(hcc, i + j);
    if (i + j > 0) tmp -= 0.5 * (i + j) * hc * std::pow(hcc, i + j - 1);
    tmp = fa * gb * tmp * std::pow(hb, i);
    dt += tmp;

    double sc = std::pow(2.0, 2 * i + j + 1.5);
    dr *= sc; ds *= sc; dt *= sc;
}

RefTet build_ref_tet(int p)
{
    if (p < 1 || p > 10) throw std::runtime_error("tetrahedron order must be in [1, 10]");
    RefTet T;
    T.p = p; T.Np = tet_np(p); T.Nfp = tri_np(p);
    const int Np = T.Np, Nfp = T.Nfp;
    auto g = gauss_lobatto(p);
    for (auto& v : g) v = 0.5 * (v + 1.0);   // to [0,1]

    T.r.resize(Np); T.s.resize(Np); T.t.resize(Np); T.bary.resize(4 * Np);
    int o = 0;
    for (int k = 0; k <= p; ++k)
        for (int j = 0; j + k <= p; ++j)
            for (int i = 0; i + j + k <= p; ++i) {
                int l = p - i - j - k;
                double w = g[i] + g[j] + g[k] + g[l];
                double l1 = g[i] / w, l2 = g[j] / w, l3 = g[k] / w, l0 = g[l] / w;
                T.bary[4 * o + 0] = l0; T.bary[4 * o + 1] = l1;
                T.bary[4 * o + 2] = l2; T.bary[4 * o + 3] = l3;
                T.r[o] = 2.0 * l1 - 1.0; T.s[o] = 2.0 * l2 - 1.0; T.t[o] = 2.0 * l3 - 1.0;
                ++o;
            }

    // Vandermonde and gradients
    std::vector<double> V(Np * Np), Vr(Np * Np), Vs(Np * Np), Vt(Np * Np);
    int m = 0;
    for (int i = 0; i <= p; ++i)
        for (int j = 0; i + j <= p; ++j)
            for (int k = 0; i + j + k <= p; ++k) {
                for (int n = 0; n < Np; ++n) {
                    V[n * Np + m] = simplex3d(T.r[n], T.s[n], T.t[n], i, j, k);
                    grad_simplex3d(T.r[n], T.s[n], T.t[n], i, j, k,
                                   Vr[n * Np + m], Vs[n * Np + m], Vt[n * Np + m]);
                }
                ++m;
            }
    std::vector<double> Vinv = V;
    if (!invert_matrix(Vinv, Np)) throw std::runtime_error("singular tet Vandermonde");
    T.Vinv = Vinv;
    T.Dr.resize(Np * Np); T.Ds.resize(Np * Np); T.Dt.resize(Np * Np);
    matmul(Vr.data(), Vinv.data(), T.Dr.data(), Np, Np, Np);
    matmul(Vs.data(), Vinv.data(), T.Ds.data(), Np, Np, Np);
    matmul(Vt.data(), Vinv.data(), T.Dt.data(), Np, Np, Np);

    // M^-1 = V V^T
    T.Minv.assign(Np * Np, 0.0);
    for (int a = 0; a < Np; ++a)
        for (int b = 0; b < Np; ++b) {
            double acc = 0.0;
            for (int q = 0; q < Np; ++q) acc += V[a * Np + q] * V[b * Np + q];
            T.Minv[a * Np + b] = acc;
        }

    // Face masks: face f is opposite vertex f, i.e. barycentric l_f == 0.
    T.Fmask.assign(4 * Nfp, -1);
    for (int f = 0; f < 4; ++f) {
        int c = 0;
        for (int n = 0; n < Np; ++n)
            if (T.bary[4 * n + f] < 1e-12) {
                if (c >= Nfp) throw std::runtime_error("face node count mismatch");
                T.Fmask[f * Nfp + c++] = n;
            }
        if (c != Nfp) throw std::runtime_error("face node count mismatch");
    }

    // Emat: reference-triangle (area 2) mass of each face's nodal basis.
    std::vector<double> Emat(static_cast<size_t>(Np) * 4 * Nfp, 0.0);
    T.face_w.assign(4 * Nfp, 0.0);
    for (int f = 0; f < 4; ++f) {
        int verts[3], c = 0;
        for (int v = 0; v < 4; ++v) if (v != f) verts[c++] = v;
        std::vector<double> V2(Nfp * Nfp);
        for (int a = 0; a < Nfp; ++a) {
            int n = T.Fmask[f * Nfp + a];
            double rr = 2.0 * T.bary[4 * n + verts[1]] - 1.0;
            double ss = 2.0 * T.bary[4 * n + verts[2]] - 1.0;
            int mm = 0;
            for (int i = 0; i <= p; ++i)
                for (int j = 0; i + j <= p; ++j) V2[a * Nfp + mm++] = simplex2d(rr, ss, i, j);
        }
        std::vector<double> VVt(Nfp * Nfp, 0.0);
        for (int a = 0; a < Nfp; ++a)
            for (int b = 0; b < Nfp; ++b) {
                double acc = 0.0;
                for (int q = 0; q < Nfp; ++q) acc += V2[a * Nfp + q] * V2[b * Nfp + q];
                VVt[a * Nfp + b] = acc;
            }
        if (!invert_matrix(VVt, Nfp)) throw std::runtime_error("singular face Vandermonde");
        for (int a = 0; a < Nfp; ++a)
            for (int b = 0; b < Nfp; ++b) {
                Emat[static_cast<size_t>(T.Fmask[f * Nfp + a]) * 4 * Nfp + f * Nfp + b] = VVt[a * Nfp + b];
                T.face_w[f * Nfp + a] += VVt[a * Nfp + b];   // row sum of the face mass = quadrature weight
            }
    }
    T.LIFT.resize(static_cast<size_t>(Np) * 4 * Nfp);
    matmul(T.Minv.data(), Emat.data(), T.LIFT.data(), Np, Np, 4 * Nfp);
    return T;
}

void nodal_basis_at(const RefTet& T, double r, double s, double t, double* phi)
{
    const int p = T.p, Np = T.Np;
    std::vector<double> psi(Np);
    int m = 0;
    for (int i = 0; i <= p; ++i)
        for (int j = 0; i + j <= p; ++j)
            for (int k = 0; i + j + k <= p; ++k) psi[m++] = simplex3d(r, s, t, i, j, k);
    for (int n = 0; n < Np; ++n) {
        double acc = 0.0;
        for (int q = 0; q < Np; ++q) acc += T.Vinv[static_cast<size_t>(q) * Np + n] * psi[q];
        phi[n] = acc;
    }
}

void nodal_basis_grad_at(const RefTet& T, double r, double s, double t, double* dphi)
{
    const int p = T.p, Np = T.Np;
    std::vector<double> gr(Np), gs(Np), gt(Np);
    int m = 0;
    for (int i = 0; i <= p; ++i)
        for (int j = 0; i + j <= p; ++j)
            for (int k = 0; i + j + k <= p; ++k, ++m) grad_simplex3d(r, s, t, i, j, k, gr[m], gs[m], gt[m]);
    for (int n = 0; n < Np; ++n) {
        double a = 0.0, b = 0.0, c = 0.0;
        for (int q = 0; q < Np; ++q) {
            const double v = T.Vinv[static_cast<size_t>(q) * Np + n];
            a += v * gr[q]; b += v * gs[q]; c += v * gt[q];
        }
        dphi[3 * n] = a; dphi[3 * n + 1] = b; dphi[3 * n + 2] = c;
    }
}

void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w)
{
    // Newton on P_n from the Chebyshev-like first guesses; P_n and P_n' by the three-term recurrence
    x.resize(n); w.resize(n);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                const double pk = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
                p0 = p1; p1 = pk;
            }
            const double pn = (n == 1) ? z : p1, pm = (n == 1) ? 1.0 : p0;
            dp = n * (z * pn - pm) / (z * z - 1.0);
            const double dz = pn / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[i] = 0.5 * (1.0 - z);
        w[i] = 1.0 / ((1.0 - z * z) * dp * dp);
    }
}

std::vector<double> tet_node_bary(int p, int basis_type)
{
    if (p < 1 || p > 10) throw std::runtime_error("tetrahedron order must be in [1, 10]");
    std::vector<double> g;
    if (basis_type == kBasisGaussLobatto) {
        g = gauss_lobatto(p);
        for (auto& v : g) v = 0.5 * (v + 1.0);
    } else if (basis_type == kBasisGaussLegendre) {
        std::vector<double> w;
        gauss_legendre01(p + 1, g, w);
        std::sort(g.begin(), g.end());
    } else {
        throw std::runtime_error("basis_type must be 0 (Gauss-Legendre) or 1 (Gauss-Lobatto)");
    }
    std::vector<double> b;
    b.reserve(4 * tet_np(p));
    for (int k = 0; k <= p; ++k)
        for (int j = 0; j + k <= p; ++j)
            for (int i = 0; i + j + k <= p; ++i) {
                const int l = p - i - j - k;
                const double w = g[i] + g[j] + g[k] + g[l];
                b.insert(b.end(), {g[l] / w, g[i] / w, g[j] / w, g[k] / w});
            }
    return b;
}

std::vector<double> tet_basis_change(int p, int from_basis, int to_basis)
{
    // M = V_to V_from^-1 with V[n][m] the orthonormal modes at the nodes
    const int Np = tet_np(p);
    auto vander = [&](int basis) {
        const std::vector<double> b = tet_node_bary(p, basis);
        std::vector<double> V(static_cast<size_t>(Np) * Np);
        int m = 0;
        for (int i = 0; i <= p; ++i)
            for (int j = 0; i + j <= p; ++j)
                for (int k = 0; i + j + k <= p; ++k) {
                    for (int n = 0; n < Np; ++n)
                        V[n * Np + m] = simplex3d(2.0 * b[4 * n + 1] - 1.0, 2.0 * b[4 * n + 2] - 1.0,
                                                  2.0 * b[4 * n + 3] - 1.0, i, j, k);
                    ++m;
                }
        return V;
    };
    std::vector<double> Vf = vander(from_basis), Vt = vander(to_basis), M(static_cast<size_t>(Np) * Np);
    if (!invert_matrix(Vf, Np)) throw std::runtime_error("singular tet Vandermonde");
    matmul(Vt.data(), Vf.data(), M.data(), Np, Np, Np);
    return M;
}

RefSeg build_ref_seg(int p)
{
    if (p < 1 || p > 16) throw std::runtime_error("segment order must be in [1, 16]");
    RefSeg S;
    S.p = p; S.Np = p + 1;
    const int Np = S.Np;
    S.r = gauss_lobatto(p);
    std::vector<double> V(Np * Np), Vr(Np * Np);
    for (int n = 0; n < Np; ++n)
        for (int j = 0; j < Np; ++j) {
            V[n * Np + j] = jacobi_p(S.r[n], 0.0, 0.0, j);
            Vr[n * Np + j] = grad_jacobi_p(S.r[n], 0.0, 0.0, j);
        }
    std::vector<double> Vinv = V;
    if (!invert_matrix(Vinv, Np)) throw std::runtime_error("singular segment Vandermonde");
    S.Dr.resize(Np * Np);
    matmul(Vr.data(), Vinv.data(), S.Dr.data(), Np, Np, Np);
    // LIFT = V V^T E with E picking the two end nodes
    S.LIFT.assign(Np * 2, 0.0);
    for (int a = 0; a < Np; ++a) {
        double m0 = 0.0, m1 = 0.0;
        for (int q = 0; q < Np; ++q) {
            m0 += V[a * Np + q] * V[0 * Np + q];
            m1 += V[a * Np + q] * V[(Np - 1) * Np + q];
        }
        S.LIFT[a * 2 + 0] = m0;
        S.LIFT[a * 2 + 1] = m1;
    }
    return S;
}

}  // namespace dgtd
