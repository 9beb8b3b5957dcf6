// CPU oracle for the DG Maxwell step — TEST INFRASTRUCTURE ONLY.
//
// This file restates, on the CPU in FP64, the algorithm of the reference's
// evolution operator so that the GPU path can be checked against it. It is
// never part of the product: only tests/, __graft_entry__.smoke() and the
// cpu_baseline leg of bench.py load it.
//
// Two independent restatements are provided:
//  (A) "global": the assembled sparse operator of GlobalEvolution
//      (src/evolution/GlobalEvolution.cpp:628-826) built like
//      DGOperatorFactory::buildGlobalOperator (src/components/DGOperatorFactory.h:1428-1602):
//      weak-form element matrices by exact quadrature (mass, strong-form
//      derivative ∫ v du/dx, the zero/one/two-normal face "jump" integrators of
//      src/mfemExtension/BilinearIntegrators.cpp:9-149 and the interior-boundary
//      integrator :356-412), multiplied by the piecewise-eps/mu inverse mass
//      (DGOperatorFactory.h:413-424) and placed with the signs of
//      DGOperatorFactory.h:1061-1208; TF/SF through a second face operator
//      applied to the +-0.5 masked plane wave (GlobalEvolution.cpp:551-626,
//      SourcesManager.cpp:129-231) with the ||pw|| < 1e-8 skip.
//  (B) "nodal": the matrix-free nodal form of HesthavenEvolution::Mult
//      (src/evolution/HesthavenEvolution.cpp:450-541): node jumps, boundary
//      rules, TF/SF, upwind flux, per-element derivative and lift matrices,
//      with the boundary coefficients of (A).
// Time integration: classical RK4 with mfem::RK4Solver's register sequence
// (used by src/solver/Solver.cpp:45-47, 535-551) and the run loop of
// Solver::run (Solver.cpp:483-533); optionally the 5-stage low-storage RK4.
//
// Element basis: Lagrange polynomials on the node set of
// L2_FECollection(p, dim, GaussLobatto) (barycentric blend of Gauss-Lobatto
// points), represented through the Bernstein basis; quadrature: collapsed
// (Duffy) Gauss-Legendre products, exact for the polynomial integrands of
// affine elements. Nothing here is shared with the product's code.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

using std::vector;

// ---------------------------------------------------------------- 1D rules
static void gauss_legendre01(int n, vector<double>& x, vector<double>& w)
{
    x.resize(n); w.resize(n);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 200; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) { double pk = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k; p0 = p1; p1 = pk; }
            double pn = (n == 1) ? z : p1, pm = (n == 1) ? 1.0 : p0;
            dp = n * (z * pn - pm) / (z * z - 1.0);
            double dz = pn / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[i] = 0.5 * (1.0 - z);
        w[i] = 1.0 / ((1.0 - z * z) * dp * dp);   // 2/((1-z^2)P'^2) scaled by 1/2 for [0,1]
    }
}

// Gauss-Lobatto points on [0,1]: ends plus the extrema of P_p, found by
// bisection-refined Newton on the derivative of the Legendre recurrence.
static vector<double> lobatto01(int p)
{
    vector<double> g(p + 1);
    if (p == 0) { g[0] = 0.5; return g; }
    g[0] = 0.0; g[p] = 1.0;
    auto dleg = [p](double z, double& d1, double& d2) {
        // P_p'(z) and P_p''(z) by the recurrence for (P, P', P'')
        double P0 = 1, P1 = z, D0 = 0, D1 = 1, S0 = 0, S1 = 0;
        for (int k = 2; k <= p; ++k) {
            double Pk = ((2 * k - 1) * z * P1 - (k - 1) * P0) / k;
            double Dk = ((2 * k - 1) * (P1 + z * D1) - (k - 1) * D0) / k;
            double Sk = ((2 * k - 1) * (2 * D1 + z * S1) - (k - 1) * S0) / k;
            P0 = P1; P1 = Pk; D0 = D1; D1 = Dk; S0 = S1; S1 = Sk;
        }
        if (p == 1) { d1 = 1.0; d2 = 0.0; } else { d1 = D1; d2 = S1; }
    };
    for (int i = 1; i < p; ++i) {
        double z = -std::cos(M_PI * i / p);
        for (int it = 0; it < 200; ++it) {
            double d1, d2; dleg(z, d1, d2);
            double dz = d1 / d2;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        g[i] = 0.5 * (1.0 + z);
    }
    for (int i = 0; i <= p / 2; ++i) { double v = 0.5 * (g[i] + 1.0 - g[p - i]); g[i] = v; g[p - i] = 1.0 - v; }
    return g;
}

// ---------------------------------------------------------------- dense LU
struct LU {
    int n = 0; vector<double> a; vector<int> piv;
    explicit LU(const vector<double>& m, int n_) : n(n_), a(m), piv(n_)
    {
        for (int k = 0; k < n; ++k) {
            int p = k;
            for (int i = k + 1; i < n; ++i) if (std::fabs(a[i * n + k]) > std::fabs(a[p * n + k])) p = i;
            piv[k] = p;
            if (p != k) for (int j = 0; j < n; ++j) std::swap(a[k * n + j], a[p * n + j]);
            if (a[k * n + k] == 0.0) throw std::runtime_error("oracle: singular matrix");
            for (int i = k + 1; i < n; ++i) {
                double f = a[i * n + k] /= a[k * n + k];
                for (int j = k + 1; j < n; ++j) a[i * n + j] -= f * a[k * n + j];
            }
        }
    }
    void solve(double* b) const
    {
        // rows were swapped as whole rows during factorisation (PA = LU): permute b first
        for (int k = 0; k < n; ++k) std::swap(b[k], b[piv[k]]);
        for (int k = 0; k < n; ++k) for (int i = k + 1; i < n; ++i) b[i] -= a[i * n + k] * b[k];
        for (int k = n - 1; k >= 0; --k) { for (int j = k + 1; j < n; ++j) b[k] -= a[k * n + j] * b[j]; b[k] /= a[k * n + k]; }
    }
    vector<double> inverse() const
    {
        vector<double> inv(n * n), col(n);
        for (int j = 0; j < n; ++j) {
            std::fill(col.begin(), col.end(), 0.0); col[j] = 1.0; solve(col.data());
            for (int i = 0; i < n; ++i) inv[i * n + j] = col[i];
        }
        return inv;
    }
};

// ---------------------------------------------------------------- element basis
// Lagrange basis on the GaussLobatto node set of the reference simplex
// (dim 1: [0,1]; dim 3: tet (0,0,0),(1,0,0),(0,1,0),(0,0,1)), through Bernstein polynomials.
// With `legendre` the node set is MFEM's GaussLegendre one instead (L2_FECollection(p, 3,
// BasisType::GaussLegendre), the reference's basis_type 0): the same barycentric blend of the
// p + 1 Gauss-Legendre points, which puts no node on a face.
struct Basis {
    // Evaluated in extended precision: the Bernstein-to-Lagrange change of
    // basis is moderately ill-conditioned at p = 6.
    typedef long double R;
    int dim = 3, p = 1, Np = 0;
    vector<double> nodes;                 // [Np][dim] reference coordinates
    vector<std::array<int, 4>> bidx;      // Bernstein multi-indices (l0, l1, l2, l3)
    vector<R> C;                          // [Np][Np]: phi_i = sum_m B_m C[m][i]
    vector<R> fact;

    R bern(const std::array<int, 4>& a, const R* lam, int deg) const
    {
        R v = fact[deg];
        for (int q = 0; q <= dim; ++q) {
            R pw = 1; for (int e = 0; e < a[q]; ++e) pw *= lam[q];
            v *= pw / fact[a[q]];
        }
        return v;
    }
    void lam_of(const double* xi, double* lam) const
    {
        double s = 0;
        for (int d = 0; d < dim; ++d) { lam[d + 1] = xi[d]; s += xi[d]; }
        lam[0] = 1.0 - s;
    }
    void lamR(const double* xi, R* lam) const
    {
        R s = 0;
        for (int d = 0; d < dim; ++d) { lam[d + 1] = xi[d]; s += xi[d]; }
        lam[0] = 1 - s;
    }
    void init(int dim_, int p_, bool legendre = false)
    {
        dim = dim_; p = p_;
        fact.resize(p + 2); fact[0] = 1; for (int i = 1; i < p + 2; ++i) fact[i] = fact[i - 1] * i;
        vector<double> g, gw;
        if (legendre) { gauss_legendre01(p + 1, g, gw); std::sort(g.begin(), g.end()); }
        else g = lobatto01(p);
        nodes.clear(); bidx.clear();
        if (dim == 1) {
            Np = p + 1;
            for (int i = 0; i <= p; ++i) nodes.push_back(g[i]);
            for (int i = 0; i <= p; ++i) bidx.push_back({p - i, i, 0, 0});
        } else {
            for (int k = 0; k <= p; ++k)
                for (int j = 0; j + k <= p; ++j)
                    for (int i = 0; i + j + k <= p; ++i) {
                        int l = p - i - j - k;
                        double w = g[i] + g[j] + g[k] + g[l];
                        nodes.push_back(g[i] / w); nodes.push_back(g[j] / w); nodes.push_back(g[k] / w);
                        bidx.push_back({l, i, j, k});
                    }
            Np = static_cast<int>(bidx.size());
        }
        // Gauss-Jordan inverse of the Bernstein Vandermonde in extended precision
        vector<R> V(Np * Np), I(Np * Np, 0);
        for (int n = 0; n < Np; ++n) {
            R lam[4] = {0, 0, 0, 0};
            lamR(&nodes[n * dim], lam);
            for (int m = 0; m < Np; ++m) V[n * Np + m] = bern(bidx[m], lam, p);
            I[n * Np + n] = 1;
        }
        for (int c = 0; c < Np; ++c) {
            int best = c;
            for (int r = c + 1; r < Np; ++r) if (fabsl(V[r * Np + c]) > fabsl(V[best * Np + c])) best = r;
            if (V[best * Np + c] == 0) throw std::runtime_error("oracle: singular Bernstein Vandermonde");
            for (int k = 0; k < Np; ++k) { std::swap(V[c * Np + k], V[best * Np + k]); std::swap(I[c * Np + k], I[best * Np + k]); }
            R d = 1 / V[c * Np + c];
            for (int k = 0; k < Np; ++k) { V[c * Np + k] *= d; I[c * Np + k] *= d; }
            for (int r = 0; r < Np; ++r) {
                if (r == c) continue;
                R f = V[r * Np + c];
                if (f == 0) continue;
                for (int k = 0; k < Np; ++k) { V[r * Np + k] -= f * V[c * Np + k]; I[r * Np + k] -= f * I[c * Np + k]; }
            }
        }
        C = I;
    }
    void shapeR(const double* xi, R* phi) const
    {
        R lam[4] = {0, 0, 0, 0}; lamR(xi, lam);
        vector<R> b(Np);
        for (int m = 0; m < Np; ++m) b[m] = bern(bidx[m], lam, p);
        for (int i = 0; i < Np; ++i) { R s = 0; for (int m = 0; m < Np; ++m) s += b[m] * C[m * Np + i]; phi[i] = s; }
    }
    void dshapeR(const double* xi, R* dphi) const
    {
        R lam[4] = {0, 0, 0, 0}; lamR(xi, lam);
        vector<R> db(Np * dim, 0);
        for (int m = 0; m < Np; ++m) {
            R dl[4] = {0, 0, 0, 0};
            for (int q = 0; q <= dim; ++q) {
                if (bidx[m][q] == 0) continue;
                auto a = bidx[m]; a[q] -= 1;
                dl[q] = static_cast<R>(p) * bern(a, lam, p - 1);
            }
            for (int d = 0; d < dim; ++d) db[m * dim + d] = dl[d + 1] - dl[0];
        }
        for (int i = 0; i < Np; ++i)
            for (int d = 0; d < dim; ++d) {
                R s = 0; for (int m = 0; m < Np; ++m) s += db[m * dim + d] * C[m * Np + i];
                dphi[i * dim + d] = s;
            }
    }
    void shape(const double* xi, double* phi) const
    {
        R lam[4] = {0, 0, 0, 0}; lamR(xi, lam);
        vector<R> b(Np);
        for (int m = 0; m < Np; ++m) b[m] = bern(bidx[m], lam, p);
        for (int i = 0; i < Np; ++i) { R s = 0; for (int m = 0; m < Np; ++m) s += b[m] * C[m * Np + i]; phi[i] = static_cast<double>(s); }
    }
    // dphi[i*dim + d] = d phi_i / d xi_d
    void dshape(const double* xi, double* dphi) const
    {
        R lam[4] = {0, 0, 0, 0}; lamR(xi, lam);
        vector<R> db(Np * dim, 0);
        for (int m = 0; m < Np; ++m) {
            R dl[4] = {0, 0, 0, 0};
            for (int q = 0; q <= dim; ++q) {
                if (bidx[m][q] == 0) continue;
                auto a = bidx[m]; a[q] -= 1;
                // d/d lam_q of p!/a! prod lam^a  =  p * B^{p-1}_{a - e_q}
                dl[q] = static_cast<R>(p) * bern(a, lam, p - 1);
            }
            for (int d = 0; d < dim; ++d) db[m * dim + d] = dl[d + 1] - dl[0];
        }
        for (int i = 0; i < Np; ++i)
            for (int d = 0; d < dim; ++d) {
                R s = 0; for (int m = 0; m < Np; ++m) s += db[m * dim + d] * C[m * Np + i];
                dphi[i * dim + d] = static_cast<double>(s);
            }
    }
};

// Quadrature on the reference simplex (weights sum to its measure).
struct Quad { vector<double> x; vector<double> w; };

static Quad tet_quad(int n)
{
    vector<double> g, gw; gauss_legendre01(n, g, gw);
    Quad q;
    for (int a = 0; a < n; ++a) for (int b = 0; b < n; ++b) for (int c = 0; c < n; ++c) {
        double u = g[a], v = g[b], w = g[c];
        q.x.push_back(u * (1 - v) * (1 - w)); q.x.push_back(v * (1 - w)); q.x.push_back(w);
        q.w.push_back(gw[a] * gw[b] * gw[c] * (1 - v) * (1 - w) * (1 - w));
    }
    return q;
}
static Quad tri_quad(int n)
{
    vector<double> g, gw; gauss_legendre01(n, g, gw);
    Quad q;
    for (int a = 0; a < n; ++a) for (int b = 0; b < n; ++b) {
        double u = g[a], v = g[b];
        q.x.push_back(u * (1 - v)); q.x.push_back(v);
        q.w.push_back(gw[a] * gw[b] * (1 - v));
    }
    return q;
}

// ---------------------------------------------------------------- CSR builder
struct CSR {
    int64_t rows = 0, cols = 0;
    vector<int64_t> rp; vector<int32_t> ci; vector<double> v;
    void spmv(const double* x, double* y, double scale, bool accumulate) const
    {
#pragma omp parallel for schedule(static)
        for (int64_t r = 0; r < rows; ++r) {
            double s = 0;
            for (int64_t k = rp[r]; k < rp[r + 1]; ++k) s += v[k] * x[ci[k]];
            y[r] = accumulate ? y[r] + scale * s : scale * s;
        }
    }
};

// Row-wise triplet accumulation (rows are owned by one element block, so each
// element's rows are built independently and merged).

enum { BC_OPEN = 0, BC_PEC = 1, BC_PMC = 2, BC_SMA = 3, BC_SGBC = 4 };

struct Face {
    int64_t e1, e2;      // e2 = -1 on the boundary
    int f1, f2;
    int kind;            // 0 interior, 1 boundary, 2 TF/SF (interior), 3 interior PEC/PMC/SMA sheet,
                         // 4 thin-layer (SGBC) sheet (interior)
    int bc;              // BC code for kinds 1 and 3
    double n[3];         // unit normal, outward from e1
    double jac;          // face Jacobian |J_f| w.r.t. the reference face (MFEM measure: tri 1/2, point 1)
    int tf_side;         // kind 2: +1 if e1 is in the total field, -1 otherwise
};

struct PW { double k[3], pol[3], kxp[3], spread, mean, freq; };

struct Oracle {
    int dim = 3, p = 1, Np = 0, Nfp = 0, nfaces = 4;
    double alpha = 1.0;
    int64_t K = 0, N = 0;
    Basis B;
    bool legendre = false;   // Gauss-Legendre node set (orc_set_basis): no face nodes
    vector<double> verts; vector<int32_t> elems;
    vector<double> eps, mu, sig;
    vector<double> A;      // per element affine map: x = v0 + A xi, A [3][dim]
    vector<double> Ainv;   // [dim][3]
    vector<double> detJ;
    vector<double> X;      // [3][N] node coordinates
    vector<Face> faces;
    vector<int64_t> elem_face;   // [K][nfaces] -> face index
    vector<int> fnodes;          // [nfaces][Nfp] reference nodes on each local face
    vector<int32_t> tfsf_elems;
    vector<PW> pws;
    // (A) global
    bool have_csr = false; CSR Aglob, Ttfsf, Tsgbc;
    vector<int64_t> sgbc_faces;   // kind-4 faces in the order their interior-face records were given
    // (B) nodal
    bool have_nodal = false;
    vector<double> Dx;            // per shape class: [3][Np][Np] physical derivative M^-1 S_d
    vector<double> Lf;            // per shape class: [nfaces][Np][Nfp] M^-1 * face mass (face nodes)
    vector<int> shape_of;         // element -> shape class
    vector<int64_t> vmapP;        // [K][nfaces][Nfp]
    // thin-layer (SGBC) sub-solvers, set by orc_set_sgbc
    std::shared_ptr<struct Sgbc> sgbc;
    // second-order (curved) elements, set by orc_set_curved: per element its index into cnodes
    // (-1: affine), cnodes [n][10][3] = corners, then edge nodes of (0,1) (0,2) (0,3) (1,2) (1,3) (2,3)
    vector<int64_t> cidx;
    vector<double> cnodes;
    bool is_curved(int64_t e) const { return !cidx.empty() && cidx[e] >= 0; }

    // ---- geometry
    void ref_to_phys(int64_t e, const double* xi, double* x) const
    {
        const double* v0 = &verts[3 * elems[e * (dim + 1)]];
        for (int r = 0; r < 3; ++r) { x[r] = v0[r]; for (int d = 0; d < dim; ++d) x[r] += A[e * 3 * dim + r * dim + d] * xi[d]; }
    }
    void phys_to_ref(int64_t e, const double* x, double* xi) const
    {
        const double* v0 = &verts[3 * elems[e * (dim + 1)]];
        for (int d = 0; d < dim; ++d) { xi[d] = 0; for (int r = 0; r < 3; ++r) xi[d] += Ainv[e * 3 * dim + d * 3 + r] * (x[r] - v0[r]); }
    }
};

static void cross(const double* a, const double* b, double* c)
{
    c[0] = a[1] * b[2] - a[2] * b[1]; c[1] = a[2] * b[0] - a[0] * b[2]; c[2] = a[0] * b[1] - a[1] * b[0];
}

// Reference boundary coefficient table (DGOperatorFactory.h:21-35): c[bc][field]
static double bc_coeff(int bc, int field)
{
    switch (bc) {
    case BC_PEC: return field == 0 ? 2.0 : 0.0;
    case BC_PMC: return field == 0 ? 0.0 : 2.0;
    case BC_SMA: return 1.0;
    default: return 0.0;
    }
}

static void build_geometry(Oracle& O)
{
    const int dim = O.dim, nv = dim + 1;
    O.A.assign(O.K * 3 * dim, 0.0); O.Ainv.assign(O.K * 3 * dim, 0.0); O.detJ.resize(O.K);
    for (int64_t e = 0; e < O.K; ++e) {
        const double* v0 = &O.verts[3 * O.elems[e * nv]];
        double* Ae = &O.A[e * 3 * dim];
        for (int d = 0; d < dim; ++d) {
            const double* vd = &O.verts[3 * O.elems[e * nv + d + 1]];
            for (int r = 0; r < 3; ++r) Ae[r * dim + d] = vd[r] - v0[r];
        }
        if (dim == 1) {
            double h = Ae[0];
            if (!(h > 0)) throw std::runtime_error("oracle: 1D segment with non-positive length");
            O.detJ[e] = h; O.Ainv[e * 3 + 0] = 1.0 / h;
        } else {
            double c0[3] = {Ae[0], Ae[3], Ae[6]}, c1[3] = {Ae[1], Ae[4], Ae[7]}, c2[3] = {Ae[2], Ae[5], Ae[8]};
            double x12[3]; cross(c1, c2, x12);
            double det = c0[0] * x12[0] + c0[1] * x12[1] + c0[2] * x12[2];
            if (!(det > 0)) throw std::runtime_error("oracle: tetrahedron with non-positive Jacobian");
            O.detJ[e] = det;
            double x20[3], x01[3]; cross(c2, c0, x20); cross(c0, c1, x01);
            double* Ai = &O.Ainv[e * 9];
            for (int r = 0; r < 3; ++r) { Ai[0 * 3 + r] = x12[r] / det; Ai[1 * 3 + r] = x20[r] / det; Ai[2 * 3 + r] = x01[r] / det; }
        }
    }
    O.N = O.K * O.Np;
    O.X.assign(3 * O.N, 0.0);
    for (int64_t e = 0; e < O.K; ++e)
        for (int n = 0; n < O.Np; ++n) {
            double x[3]; O.ref_to_phys(e, &O.B.nodes[n * dim], x);
            for (int r = 0; r < 3; ++r) O.X[r * O.N + e * O.Np + n] = x[r];
        }
}

// local face f of the reference simplex: the face opposite vertex f
static void local_face_nodes(Oracle& O)
{
    const int dim = O.dim;
    O.nfaces = dim + 1;
    O.Nfp = (dim == 1) ? 1 : (O.p + 1) * (O.p + 2) / 2;
    O.fnodes.assign(O.nfaces * O.Nfp, -1);
    for (int f = 0; f < O.nfaces; ++f) {
        int c = 0;
        for (int n = 0; n < O.Np; ++n) {
            double lam[4] = {0, 0, 0, 0}; O.B.lam_of(&O.B.nodes[n * dim], lam);
            if (std::fabs(lam[f]) < 1e-12) O.fnodes[f * O.Nfp + c++] = n;
        }
        if (c != O.Nfp) throw std::runtime_error("oracle: face node count");
    }
}

static std::array<int32_t, 3> face_key(const Oracle& O, int64_t e, int f)
{
    const int nv = O.dim + 1;
    std::array<int32_t, 3> k = {-1, -1, -1};
    int c = 0;
    for (int q = 0; q < nv; ++q) if (q != f) k[c++] = O.elems[e * nv + q];
    std::sort(k.begin(), k.begin() + c);
    return k;
}

static void face_normal(const Oracle& O, int64_t e, int f, double* n, double& jac)
{
    if (O.dim == 1) {
        // MFEM 1D face "normal" 2x-1 at the element-local face point (IntegratorFunctions.cpp:56-63)
        n[0] = (f == 1) ? -1.0 : 1.0;   // face 0 is opposite vertex 0 -> the x = 1 end
        n[1] = n[2] = 0.0; jac = 1.0;
        return;
    }
    const int nv = 4;
    const double* P[3]; int c = 0;
    for (int q = 0; q < nv; ++q) if (q != f) P[c++] = &O.verts[3 * O.elems[e * nv + q]];
    double a[3], b[3], cr[3];
    for (int r = 0; r < 3; ++r) { a[r] = P[1][r] - P[0][r]; b[r] = P[2][r] - P[0][r]; }
    cross(a, b, cr);
    double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
    // orient outward: away from the opposite vertex
    const double* vf = &O.verts[3 * O.elems[e * nv + f]];
    double d = 0; for (int r = 0; r < 3; ++r) d += cr[r] * (P[0][r] - vf[r]);
    double s = d > 0 ? 1.0 : -1.0;
    for (int r = 0; r < 3; ++r) n[r] = s * cr[r] / len;
    jac = len;   // |J_f| = 2 area = |cross|, reference triangle measure 1/2
}

static void build_faces(Oracle& O, int64_t nb, const int32_t* bf, const int32_t* bc, int64_t nt, const int32_t* tf,
                        int64_t ni, const int32_t* ifc, const int32_t* icodes)
{
    const int dim = O.dim, nf = O.nfaces;
    std::map<std::array<int32_t, 3>, std::pair<int64_t, int>> open;
    O.elem_face.assign(O.K * nf, -1);
    for (int64_t e = 0; e < O.K; ++e)
        for (int f = 0; f < nf; ++f) {
            auto k = face_key(O, e, f);
            auto it = open.find(k);
            if (it == open.end()) { open[k] = {e, f}; continue; }
            Face F{};
            F.e1 = it->second.first; F.f1 = it->second.second; F.e2 = e; F.f2 = f; F.kind = 0; F.bc = 0;
            face_normal(O, F.e1, F.f1, F.n, F.jac);
            O.elem_face[F.e1 * nf + F.f1] = static_cast<int64_t>(O.faces.size());
            O.elem_face[F.e2 * nf + F.f2] = static_cast<int64_t>(O.faces.size());
            O.faces.push_back(F);
            open.erase(it);
        }
    std::map<std::array<int32_t, 3>, int64_t> key_to_face;
    for (auto& kv : open) {
        Face F{};
        F.e1 = kv.second.first; F.f1 = kv.second.second; F.e2 = -1; F.f2 = -1; F.kind = 1; F.bc = BC_OPEN;
        face_normal(O, F.e1, F.f1, F.n, F.jac);
        O.elem_face[F.e1 * nf + F.f1] = static_cast<int64_t>(O.faces.size());
        O.faces.push_back(F);
    }
    for (size_t i = 0; i < O.faces.size(); ++i) key_to_face[face_key(O, O.faces[i].e1, O.faces[i].f1)] = i;
    const int fv = (dim == 1) ? 1 : 3;
    auto lookup = [&](const int32_t* v) {
        std::array<int32_t, 3> k = {-1, -1, -1};
        for (int q = 0; q < fv; ++q) k[q] = v[q];
        std::sort(k.begin(), k.begin() + fv);
        auto it = key_to_face.find(k);
        if (it == key_to_face.end()) throw std::runtime_error("oracle: face not found");
        return it->second;
    };
    for (int64_t b = 0; b < nb; ++b) {
        int64_t fi = lookup(&bf[b * fv]);
        if (O.faces[fi].kind != 1) throw std::runtime_error("oracle: boundary code on interior face");
        O.faces[fi].bc = bc[b];
    }
    for (int64_t b = 0; b < ni; ++b) {
        int64_t fi = lookup(&ifc[b * fv]);
        if (O.faces[fi].kind != 0) throw std::runtime_error("oracle: interior sheet on boundary face");
        if (icodes[b] == BC_SGBC) { O.faces[fi].kind = 4; O.faces[fi].bc = 0; O.sgbc_faces.push_back(fi); }
        else { O.faces[fi].kind = 3; O.faces[fi].bc = icodes[b]; }
    }
    vector<char> mark(O.K, 0);
    for (int64_t b = 0; b < nt; ++b) {
        const int32_t* v = &tf[b * (dim == 1 ? 2 : 3)];
        int64_t fi = lookup(v);
        Face& F = O.faces[fi];
        if (F.kind != 0) throw std::runtime_error("oracle: TF/SF face must be interior");
        F.kind = 2;
        // orientation of the given face: 3D winding normal / 1D given direction
        double gn[3] = {0, 0, 0};
        if (dim == 1) gn[0] = (v[1] >= 0) ? 1.0 : -1.0;
        else {
            const double* P0 = &O.verts[3 * v[0]]; const double* P1 = &O.verts[3 * v[1]]; const double* P2 = &O.verts[3 * v[2]];
            double a[3], bb[3]; for (int r = 0; r < 3; ++r) { a[r] = P1[r] - P0[r]; bb[r] = P2[r] - P0[r]; }
            cross(a, bb, gn);
        }
        // the given normal points into the TF side; F.n points from e1 to e2
        double d = F.n[0] * gn[0] + F.n[1] * gn[1] + F.n[2] * gn[2];
        F.tf_side = (d > 0) ? -1 : +1;   // e2 is TF when the normals agree -> e1 is SF
        mark[F.e1] = 1; mark[F.e2] = 1;
    }
    for (int64_t e = 0; e < O.K; ++e) if (mark[e]) O.tfsf_elems.push_back(static_cast<int32_t>(e));
}

// ---------------------------------------------------------------- (A) global
// Element matrices: mass M, its inverse, strong-form derivative S_d = int phi_i dphi_j/dx_d
// and the physical derivative D_d = M^-1 S_d, accumulated and inverted in extended
// precision (the mass matrix of the p = 6 node set has condition number ~2e3).
struct ElemMats { vector<double> M, Minv, S[3], D[3]; };

// Geometry map of element e at reference point xi: position x and Jacobian J[r][d] = dx_r/dxi_d
// (affine, or the second-order isoparametric map x = sum_k l_k (2 l_k - 1) X_k + sum 4 l_a l_b X_ab).
static const int kEdgeA[6] = {0, 0, 0, 1, 1, 2}, kEdgeB[6] = {1, 2, 3, 2, 3, 3};
static void geom(const Oracle& O, int64_t e, const double* xi, double* x, double* J)
{
    if (!O.is_curved(e)) {
        O.ref_to_phys(e, xi, x);
        for (int r = 0; r < 3; ++r) for (int d = 0; d < 3; ++d) J[r * 3 + d] = (d < O.dim) ? O.A[e * 3 * O.dim + r * O.dim + d] : 0.0;
        return;
    }
    const double* G = &O.cnodes[O.cidx[e] * 30];
    const double l[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
    static const double dl[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int r = 0; r < 3; ++r) { x[r] = 0.0; for (int d = 0; d < 3; ++d) J[r * 3 + d] = 0.0; }
    for (int k = 0; k < 4; ++k) {
        const double N = l[k] * (2.0 * l[k] - 1.0);
        for (int r = 0; r < 3; ++r) {
            x[r] += N * G[3 * k + r];
            for (int d = 0; d < 3; ++d) J[r * 3 + d] += (4.0 * l[k] - 1.0) * dl[k][d] * G[3 * k + r];
        }
    }
    for (int m = 0; m < 6; ++m) {
        const int a = kEdgeA[m], b = kEdgeB[m];
        const double N = 4.0 * l[a] * l[b];
        for (int r = 0; r < 3; ++r) {
            x[r] += N * G[3 * (4 + m) + r];
            for (int d = 0; d < 3; ++d) J[r * 3 + d] += 4.0 * (l[b] * dl[a][d] + l[a] * dl[b][d]) * G[3 * (4 + m) + r];
        }
    }
}

static double det3(const double* J, double* Jinv)
{
    const double c0 = J[4] * J[8] - J[5] * J[7], c1 = J[5] * J[6] - J[3] * J[8], c2 = J[3] * J[7] - J[4] * J[6];
    const double det = J[0] * c0 + J[1] * c1 + J[2] * c2;
    // Jinv[d][r] = d xi_d / d x_r
    Jinv[0] = c0 / det; Jinv[3] = c1 / det; Jinv[6] = c2 / det;
    Jinv[1] = (J[2] * J[7] - J[1] * J[8]) / det; Jinv[4] = (J[0] * J[8] - J[2] * J[6]) / det; Jinv[7] = (J[1] * J[6] - J[0] * J[7]) / det;
    Jinv[2] = (J[1] * J[5] - J[2] * J[4]) / det; Jinv[5] = (J[2] * J[3] - J[0] * J[5]) / det; Jinv[8] = (J[0] * J[4] - J[1] * J[3]) / det;
    return det;
}

static ElemMats elem_mats(const Oracle& O, int64_t e, const Quad& q)
{
    typedef long double R;
    const int Np = O.Np, dim = O.dim;
    const bool curved = O.is_curved(e);
    vector<R> M(Np * Np, 0), S[3];
    for (int d = 0; d < 3; ++d) S[d].assign(Np * Np, 0);
    vector<R> phi(Np), dphi(Np * dim), g(Np);
    const size_t nq = q.w.size();
    for (size_t k = 0; k < nq; ++k) {
        const double* xi = &q.x[k * dim];
        O.B.shapeR(xi, phi.data()); O.B.dshapeR(xi, dphi.data());
        double Jinv[9], detJ = O.detJ[e];
        if (curved) {
            double x[3], J[9];
            geom(O, e, xi, x, J);
            detJ = det3(J, Jinv);
            if (!(detJ > 0)) throw std::runtime_error("oracle: curved element with a non-positive Jacobian");
        }
        R w = static_cast<R>(q.w[k]) * detJ;
        for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) M[i * Np + j] += w * phi[i] * phi[j];
        for (int d = 0; d < dim; ++d) {
            // d phi_j / d x_d = sum_r dphi_j/dxi_r * Ainv[r][d]
            for (int j = 0; j < Np; ++j) {
                R gg = 0;
                for (int r = 0; r < dim; ++r) gg += dphi[j * dim + r] * (curved ? Jinv[r * 3 + d] : O.Ainv[e * 3 * dim + r * 3 + d]);
                g[j] = gg;
            }
            for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) S[d][i * Np + j] += w * phi[i] * g[j];
        }
    }
    // Gauss-Jordan inverse of M in extended precision
    vector<R> A = M, I(Np * Np, 0);
    for (int i = 0; i < Np; ++i) I[i * Np + i] = 1;
    for (int c = 0; c < Np; ++c) {
        int best = c;
        for (int r = c + 1; r < Np; ++r) if (fabsl(A[r * Np + c]) > fabsl(A[best * Np + c])) best = r;
        for (int k = 0; k < Np; ++k) { std::swap(A[c * Np + k], A[best * Np + k]); std::swap(I[c * Np + k], I[best * Np + k]); }
        R dv = 1 / A[c * Np + c];
        for (int k = 0; k < Np; ++k) { A[c * Np + k] *= dv; I[c * Np + k] *= dv; }
        for (int r = 0; r < Np; ++r) {
            if (r == c) continue;
            R f = A[r * Np + c];
            if (f == 0) continue;
            for (int k = 0; k < Np; ++k) { A[r * Np + k] -= f * A[c * Np + k]; I[r * Np + k] -= f * I[c * Np + k]; }
        }
    }
    ElemMats m;
    m.M.resize(Np * Np); m.Minv.resize(Np * Np);
    for (int q2 = 0; q2 < Np * Np; ++q2) { m.M[q2] = static_cast<double>(M[q2]); m.Minv[q2] = static_cast<double>(I[q2]); }
    for (int d = 0; d < 3; ++d) {
        m.S[d].resize(Np * Np); m.D[d].assign(Np * Np, 0.0);
        for (int q2 = 0; q2 < Np * Np; ++q2) m.S[d][q2] = static_cast<double>(S[d][q2]);
        if (d >= dim) continue;
        for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) {
            R acc = 0; for (int l = 0; l < Np; ++l) acc += I[i * Np + l] * S[d][l * Np + j];
            m.D[d][i * Np + j] = static_cast<double>(acc);
        }
    }
    return m;
}

// Elements sharing one affine map matrix share element matrices.
static void shape_classes(Oracle& O, vector<int64_t>& rep)
{
    const int dim = O.dim;
    std::map<vector<double>, int> cls;
    O.shape_of.resize(O.K);
    rep.clear();
    for (int64_t e = 0; e < O.K; ++e) {
        if (O.is_curved(e)) { O.shape_of[e] = static_cast<int>(rep.size()); rep.push_back(e); continue; }
        vector<double> key(O.A.begin() + e * 3 * dim, O.A.begin() + (e + 1) * 3 * dim);
        for (auto& v : key) v = std::round(v * 1e12) / 1e12;
        auto it = cls.find(key);
        if (it == cls.end()) { int id = static_cast<int>(rep.size()); cls[key] = id; rep.push_back(e); O.shape_of[e] = id; }
        else O.shape_of[e] = it->second;
    }
}

// Face quadrature: physical points and weights (MFEM measure: ip.weight * |J_f|).
static void face_points(const Oracle& O, const Face& F, vector<double>& xq, vector<double>& wq)
{
    xq.clear(); wq.clear();
    if (O.dim == 1) {
        double xi = (F.f1 == 0) ? 1.0 : 0.0, x[3];
        O.ref_to_phys(F.e1, &xi, x);
        xq.insert(xq.end(), x, x + 3); wq.push_back(1.0);
        return;
    }
    Quad tq = tri_quad(O.p + 2);
    const int nv = 4; const double* P[3]; int c = 0;
    for (int q = 0; q < nv; ++q) if (q != F.f1) P[c++] = &O.verts[3 * O.elems[F.e1 * nv + q]];
    for (size_t k = 0; k < tq.w.size(); ++k) {
        double u = tq.x[2 * k], v = tq.x[2 * k + 1];
        for (int r = 0; r < 3; ++r) xq.push_back(P[0][r] + u * (P[1][r] - P[0][r]) + v * (P[2][r] - P[0][r]));
        wq.push_back(tq.w[k]);   // reference weight; |J_f| applied by the caller
    }
}

// Rows of element `side` (1 = F.e1, 2 = F.e2) of one face integrator:
// own block (rows and columns of that element) and coupling block (columns of
// the other element). mode 0: zero-normal (w = beta/2 wq |J|), 1: one-normal
// dir d (w = beta/2 wq n_d |J|, un-normalised normal), 2: two-normal (d, d2)
// (w = beta/2 wq n_d n_d2 / |J| with the un-normalised normal).
static void face_rows_curved(const Oracle& O, const Face& F, int side, int mode, int d, int d2, double beta,
                             bool decoupled, double* own, double* coup);

static void face_rows(const Oracle& O, const Face& F, int side, int mode, int d, int d2, double beta, bool decoupled,
                      double* own, double* coup)
{
    if (O.is_curved(F.e1) || (F.e2 >= 0 && O.is_curved(F.e2))) {
        face_rows_curved(O, F, side, mode, d, d2, beta, decoupled, own, coup);
        return;
    }
    const int Np = O.Np;
    vector<double> xq, wq; face_points(O, F, xq, wq);
    double nn = 1.0;
    if (mode == 0) nn = F.jac;
    if (mode == 1) nn = F.n[d] * F.jac;
    if (mode == 2) nn = F.n[d] * F.n[d2] * F.jac;
    const bool has2 = F.e2 >= 0;
    std::fill(own, own + Np * Np, 0.0);
    std::fill(coup, coup + Np * Np, 0.0);
    vector<double> p1(Np), p2(Np);
    for (size_t k = 0; k < wq.size(); ++k) {
        double xi1[3], xi2[3];
        O.phys_to_ref(F.e1, &xq[3 * k], xi1); O.B.shape(xi1, p1.data());
        if (has2) { O.phys_to_ref(F.e2, &xq[3 * k], xi2); O.B.shape(xi2, p2.data()); }
        const double w = 0.5 * beta * wq[k] * nn;
        if (side == 1) {
            // TL: +w p1 p1 ; TR: -w p1 p2 (buildFaceMatrix off-diagonal sign, IntegratorFunctions.cpp:85-98)
            for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) {
                own[i * Np + j] += w * p1[i] * p1[j];
                if (has2 && !decoupled) coup[i * Np + j] -= w * p1[i] * p2[j];
            }
        } else {
            // element-2 rows: the one-normal integrator passes -w (BilinearIntegrators.cpp:83-90),
            // the zero/two-normal ones +w; the interior-boundary integrator keeps only BR (:356-412).
            const double s2 = (mode == 1) ? -1.0 : 1.0;
            for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) {
                own[i * Np + j] += s2 * w * p2[i] * p2[j];
                if (!decoupled) coup[i * Np + j] -= s2 * w * p2[i] * p1[j];
            }
        }
    }
}

// The same rows on a face with a curved side: points from the reference face of e1, mapped to
// each element's reference coordinates through the shared vertices (the face's barycentric
// coordinates), and the face's un-normalised normal t_u x t_v from e1's geometry map at each
// point (oriented out of e1): mode 0 weighs by |t_u x t_v|, mode 1 by its component d, mode 2 by
// c_d c_d2 / |c|.
static void face_rows_curved(const Oracle& O, const Face& F, int side, int mode, int d, int d2, double beta,
                             bool decoupled, double* own, double* coup)
{
    const int Np = O.Np;
    static const double rv[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    int l1[3], l2[3] = {0, 0, 0}, c = 0;
    for (int q = 0; q < 4; ++q) if (q != F.f1) l1[c++] = q;
    const bool has2 = F.e2 >= 0;
    if (has2)
        for (int k = 0; k < 3; ++k) {
            const int32_t g = O.elems[F.e1 * 4 + l1[k]];
            int found = -1;
            for (int q = 0; q < 4; ++q) if (O.elems[F.e2 * 4 + q] == g) found = q;
            if (found < 0) throw std::runtime_error("oracle: face vertices do not match");
            l2[k] = found;
        }
    std::fill(own, own + Np * Np, 0.0);
    std::fill(coup, coup + Np * Np, 0.0);
    const Quad tq = tri_quad(O.p + 4);
    vector<double> p1(Np), p2(Np);
    for (size_t k = 0; k < tq.w.size(); ++k) {
        const double u = tq.x[2 * k], v = tq.x[2 * k + 1];
        const double b[3] = {1.0 - u - v, u, v};
        double xi1[3] = {0, 0, 0}, xi2[3] = {0, 0, 0}, du[3], dv[3];
        for (int r = 0; r < 3; ++r) {
            for (int q = 0; q < 3; ++q) { xi1[r] += b[q] * rv[l1[q]][r]; xi2[r] += b[q] * rv[l2[q]][r]; }
            du[r] = rv[l1[1]][r] - rv[l1[0]][r];
            dv[r] = rv[l1[2]][r] - rv[l1[0]][r];
        }
        double x[3], J[9], tu[3], tv[3], cr[3];
        geom(O, F.e1, xi1, x, J);
        for (int r = 0; r < 3; ++r) {
            tu[r] = J[r * 3] * du[0] + J[r * 3 + 1] * du[1] + J[r * 3 + 2] * du[2];
            tv[r] = J[r * 3] * dv[0] + J[r * 3 + 1] * dv[1] + J[r * 3 + 2] * dv[2];
        }
        cross(tu, tv, cr);
        if (cr[0] * F.n[0] + cr[1] * F.n[1] + cr[2] * F.n[2] < 0) for (int r = 0; r < 3; ++r) cr[r] = -cr[r];
        const double len = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        const double nn = (mode == 0) ? len : (mode == 1 ? cr[d] : cr[d] * cr[d2] / len);
        O.B.shape(xi1, p1.data());
        if (has2) O.B.shape(xi2, p2.data());
        const double w = 0.5 * beta * tq.w[k] * nn;
        if (side == 1) {
            for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) {
                own[i * Np + j] += w * p1[i] * p1[j];
                if (has2 && !decoupled) coup[i * Np + j] -= w * p1[i] * p2[j];
            }
        } else {
            const double s2 = (mode == 1) ? -1.0 : 1.0;
            for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) {
                own[i * Np + j] += s2 * w * p2[i] * p2[j];
                if (!decoupled) coup[i * Np + j] -= s2 * w * p2[i] * p1[j];
            }
        }
    }
}

static void build_global(Oracle& O)
{
    const int Np = O.Np, dim = O.dim, nf = O.nfaces, R = 6 * Np, S = (1 + nf);
    const int64_t N = O.N;
    Quad vq;
    if (dim == 3) vq = tet_quad(O.p + 3);
    else { vector<double> g, gw; gauss_legendre01(O.p + 2, g, gw); vq.x = g; vq.w = gw; }

    vector<int64_t> rep;
    shape_classes(O, rep);
    vector<ElemMats> cls_mats(rep.size());
    const Quad vqc = (dim == 3) ? tet_quad(O.p + 4) : vq;   // curved elements: one point more per direction
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t c = 0; c < static_cast<int64_t>(rep.size()); ++c)
        cls_mats[c] = elem_mats(O, rep[c], O.is_curved(rep[c]) ? vqc : vq);

    // per element: dense local rows [R][S slots][6][Np] -> compressed rows
    vector<vector<int32_t>> colsA(O.K), colsT(O.K), colsS(O.K);
    vector<vector<double>> valsA(O.K), valsT(O.K), valsS(O.K);
    vector<vector<int32_t>> cntA(O.K), cntT(O.K), cntS(O.K);
#pragma omp parallel
    {
        vector<double> LA(static_cast<size_t>(R) * S * R), LT(static_cast<size_t>(R) * S * R),
            LS(static_cast<size_t>(R) * S * R);
        vector<double> own(Np * Np), coup(Np * Np), tmp(Np * Np);
#pragma omp for schedule(dynamic, 8)
        for (int64_t e = 0; e < O.K; ++e) {
            std::fill(LA.begin(), LA.end(), 0.0);
            std::fill(LT.begin(), LT.end(), 0.0);
            std::fill(LS.begin(), LS.end(), 0.0);
            const ElemMats& m = cls_mats[O.shape_of[e]];
            int64_t slot_elem[5] = {e, -1, -1, -1, -1};
            // add sign * scale * (Minv * blk | blk) at rows (field, rc), slot s cols (gfield, cc)
            auto place_m = [&](vector<double>& L, int field, int rc, int gfield, int cc, int s, const double* bm, double sign,
                               bool premultiplied) {
                const double sc = sign * (field == 0 ? 1.0 / O.eps[e] : 1.0 / O.mu[e]);
                for (int i = 0; i < Np; ++i)
                    for (int j = 0; j < Np; ++j) {
                        double acc;
                        if (premultiplied) acc = bm[i * Np + j];
                        else { acc = 0; for (int l = 0; l < Np; ++l) acc += m.Minv[i * Np + l] * bm[l * Np + j]; }
                        L[(static_cast<size_t>((3 * field + rc) * Np + i) * S + s) * R + (3 * gfield + cc) * Np + j] += sc * acc;
                    }
            };
            auto place = [&](vector<double>& L, int field, int rc, int gfield, int cc, int s, const double* bm, double sign) {
                place_m(L, field, rc, gfield, cc, s, bm, sign, false);
            };
            // volume: directional operators MInv_f D_x (DGOperatorFactory.h:1061-1086)
            for (int f = 0; f < 2; ++f)
                for (int x = 0; x < dim; ++x) {
                    int y = (x + 1) % 3, z = (x + 2) % 3;
                    double sg = 1.0 - 2.0 * f;
                    place_m(LA, f, z, 1 - f, y, 0, m.D[x].data(), sg, true);
                    place_m(LA, f, y, 1 - f, z, 0, m.D[x].data(), -sg, true);
                }
            // conductivity (DGOperatorFactory.h:1194-1208): -MInv_E (sigma M) = -(sigma/eps) I
            if (O.sig[e] != 0.0) {
                std::fill(tmp.begin(), tmp.end(), 0.0);
                for (int q = 0; q < Np; ++q) tmp[q * Np + q] = O.sig[e];
                for (int d = 0; d < 3; ++d) place_m(LA, 0, d, 0, d, 0, tmp.data(), -1.0, true);
            }
            for (int lf = 0; lf < nf; ++lf) {
                const Face& F = O.faces[O.elem_face[e * nf + lf]];
                const int side = (F.e1 == e && F.f1 == lf) ? 1 : 2;
                const int s = 1 + lf;
                slot_elem[s] = (side == 1) ? F.e2 : F.e1;
                if (F.kind == 1 && F.bc == BC_OPEN) continue;
                // thin-layer (SGBC) faces are left out of the interior flux (the interior ignore marker,
                // DGOperatorFactory.h:373-389, 473-481) and get the interior-face integrators in their own
                // source-face operator instead (buildSGBCGlobalOperator, DGOperatorFactory.h:1364-1425)
                const bool interior = (F.kind == 0 || F.kind == 2 || F.kind == 4);
                const bool sheet = (F.kind == 3);
                for (int f = 0; f < 2; ++f) {
                    const int g = 1 - f;
                    // coefficients (DGOperatorFactory.h:469-573, 577-675): zero/two-normal
                    // c[bc][f]*alpha (SMA: 1), one-normal c[bc][alt f] (SMA: 1); interior alpha / 1.
                    double beta0, beta1;
                    if (interior) { beta0 = O.alpha; beta1 = 1.0; }
                    else if (F.bc == BC_SMA) { beta0 = 1.0; beta1 = 1.0; }
                    else { beta0 = bc_coeff(F.bc, f) * O.alpha; beta1 = bc_coeff(F.bc, g); }
                    auto both = [&](auto&& fn) {
                        if (F.kind == 4) { fn(LS); return; }
                        fn(LA);
                        if (F.kind == 2) fn(LT);
                    };
                    if (beta0 != 0.0) {
                        face_rows(O, F, side, 0, 0, 0, beta0, sheet, own.data(), coup.data());
                        both([&](vector<double>& L) {
                            for (int d = 0; d < 3; ++d) {
                                place(L, f, d, f, d, 0, own.data(), -1.0);
                                if (slot_elem[s] >= 0 && !sheet) place(L, f, d, f, d, s, coup.data(), -1.0);
                            }
                        });
                        for (int d = 0; d < dim; ++d)
                            for (int d2 = 0; d2 < dim; ++d2) {
                                face_rows(O, F, side, 2, d, d2, beta0, sheet, own.data(), coup.data());
                                both([&](vector<double>& L) {
                                    place(L, f, d, f, d2, 0, own.data(), 1.0);
                                    if (slot_elem[s] >= 0 && !sheet) place(L, f, d, f, d2, s, coup.data(), 1.0);
                                });
                            }
                    }
                    if (beta1 != 0.0)
                        for (int x = 0; x < dim; ++x) {
                            int y = (x + 1) % 3, z = (x + 2) % 3;
                            double sg = 1.0 - 2.0 * f;
                            face_rows(O, F, side, 1, x, 0, beta1, sheet, own.data(), coup.data());
                            both([&](vector<double>& L) {
                                place(L, f, y, g, z, 0, own.data(), sg);
                                place(L, f, z, g, y, 0, own.data(), -sg);
                                if (slot_elem[s] >= 0 && !sheet) {
                                    place(L, f, y, g, z, s, coup.data(), sg);
                                    place(L, f, z, g, y, s, coup.data(), -sg);
                                }
                            });
                        }
                }
            }
            // compress (Threshold(1e-20), DGOperatorFactory.h:1569-1570)
            auto compress = [&](const vector<double>& L, vector<int32_t>& cols, vector<double>& vals, vector<int32_t>& cnt) {
                cnt.assign(R, 0);
                for (int r = 0; r < R; ++r)
                    for (int s = 0; s < S; ++s) {
                        if (slot_elem[s] < 0) continue;
                        for (int c = 0; c < R; ++c) {
                            double v = L[(static_cast<size_t>(r) * S + s) * R + c];
                            if (std::fabs(v) <= 1e-20) continue;
                            cols.push_back(static_cast<int32_t>((c / Np) * N + slot_elem[s] * Np + (c % Np)));
                            vals.push_back(v);
                            ++cnt[r];
                        }
                    }
            };
            compress(LA, colsA[e], valsA[e], cntA[e]);
            compress(LT, colsT[e], valsT[e], cntT[e]);
            compress(LS, colsS[e], valsS[e], cntS[e]);
        }
    }
    auto finalize = [&](vector<vector<int32_t>>& cols, vector<vector<double>>& vals, vector<vector<int32_t>>& cnt, CSR& M) {
        M.rows = 6 * N; M.cols = 6 * N;
        M.rp.assign(6 * N + 1, 0);
        for (int64_t e = 0; e < O.K; ++e)
            for (int r = 0; r < R; ++r) M.rp[(r / Np) * N + e * Np + (r % Np) + 1] = cnt[e][r];
        for (int64_t r = 0; r < 6 * N; ++r) M.rp[r + 1] += M.rp[r];
        M.ci.resize(M.rp[6 * N]); M.v.resize(M.rp[6 * N]);
#pragma omp parallel for schedule(dynamic, 64)
        for (int64_t e = 0; e < O.K; ++e) {
            size_t off = 0;
            for (int r = 0; r < R; ++r) {
                int64_t k = M.rp[(r / Np) * N + e * Np + (r % Np)];
                for (int q = 0; q < cnt[e][r]; ++q) { M.ci[k + q] = cols[e][off + q]; M.v[k + q] = vals[e][off + q]; }
                off += cnt[e][r];
            }
            vector<int32_t>().swap(cols[e]); vector<double>().swap(vals[e]);
        }
    };
    finalize(colsA, valsA, cntA, O.Aglob);
    finalize(colsT, valsT, cntT, O.Ttfsf);
    finalize(colsS, valsS, cntS, O.Tsgbc);
    O.have_csr = true;
}

// ---------------------------------------------------------------- sources
static double profile(const PW& w, double s)
{
    double a = s - w.mean;
    double g = std::exp(-a * a / (2.0 * w.spread * w.spread));
    if (w.freq != 0.0) g *= std::cos(2.0 * M_PI * w.freq * a);
    return g;
}
static void pw_at(const Oracle& O, const double* x, double t, double* e, double* h)
{
    for (int c = 0; c < 3; ++c) e[c] = h[c] = 0.0;
    for (const PW& w : O.pws) {
        double s = x[0] * w.k[0] + x[1] * w.k[1] + x[2] * w.k[2] - t;
        double g = profile(w, s);
        for (int c = 0; c < 3; ++c) { e[c] += g * w.pol[c]; h[c] += g * w.kxp[c]; }
    }
}

// ||0.5 pw||^2 over all nodes of the TF/SF-adjacent elements (GlobalEvolution.cpp:587-598)
static bool tfsf_skip(const Oracle& O, double t)
{
    if (O.pws.empty() || O.tfsf_elems.empty()) return true;
    double acc = 0.0;
    for (int32_t e : O.tfsf_elems)
        for (int n = 0; n < O.Np; ++n) {
            int64_t gi = static_cast<int64_t>(e) * O.Np + n;
            double x[3] = {O.X[gi], O.X[O.N + gi], O.X[2 * O.N + gi]}, pe[3], ph[3];
            pw_at(O, x, t, pe, ph);
            for (int c = 0; c < 3; ++c) acc += 0.25 * (pe[c] * pe[c] + ph[c] * ph[c]);
        }
    return acc < 1e-16;
}

static void sgbc_stage(Oracle& O, const double* x, double t, bool& quiescent);
static void sgbc_inject(Oracle& O, const double* x, double* y);
static void tfsf_apply(Oracle& O, double* y, double t);

static void mult_global(Oracle& O, const double* x, double* y, double t)
{
    if (!O.have_csr) build_global(O);
    // GlobalEvolution::Mult order (GlobalEvolution.cpp:639-1001): sub-solves, A x, TF/SF, injection
    bool quiescent = true;
    if (O.sgbc) sgbc_stage(O, x, t, quiescent);
    O.Aglob.spmv(x, y, 1.0, false);
    tfsf_apply(O, y, t);
    if (O.sgbc && !quiescent) sgbc_inject(O, x, y);
}

static void tfsf_apply(Oracle& O, double* y, double t)
{
    if (O.tfsf_elems.empty() || tfsf_skip(O, t)) return;
    // w = +-0.5 pw on every DOF of the TF/SF-adjacent elements; out -= T w
    vector<double> w(6 * O.N, 0.0);
    vector<int> side(O.K, 0);
    for (const Face& F : O.faces)
        if (F.kind == 2) { side[F.e1] = F.tf_side; side[F.e2] = -F.tf_side; }
    for (int32_t e : O.tfsf_elems) {
        double sg = 0.5 * side[e];
        for (int n = 0; n < O.Np; ++n) {
            int64_t gi = static_cast<int64_t>(e) * O.Np + n;
            double xx[3] = {O.X[gi], O.X[O.N + gi], O.X[2 * O.N + gi]}, pe[3], ph[3];
            pw_at(O, xx, t, pe, ph);
            for (int c = 0; c < 3; ++c) { w[c * O.N + gi] = sg * pe[c]; w[(3 + c) * O.N + gi] = sg * ph[c]; }
        }
    }
    O.Ttfsf.spmv(w.data(), y, -1.0, true);
}

// ---------------------------------------------------------------- (B) nodal
static void build_nodal(Oracle& O)
{
    if (O.legendre) throw std::runtime_error("oracle: the nodal form needs face nodes (Gauss-Lobatto basis)");
    const int Np = O.Np, Nfp = O.Nfp, dim = O.dim, nf = O.nfaces;
    if (!O.sgbc_faces.empty())
        throw std::runtime_error("oracle: thin-layer (SGBC) faces exist in the global form only (GlobalEvolution)");
    if (!O.cidx.empty())
        throw std::runtime_error("oracle: curved elements are assembled in the global form only");
    Quad vq;
    if (dim == 3) vq = tet_quad(O.p + 3);
    else { vector<double> g, gw; gauss_legendre01(O.p + 2, g, gw); vq.x = g; vq.w = gw; }
    vector<int64_t> rep;
    shape_classes(O, rep);
    const int nc = static_cast<int>(rep.size());
    O.Dx.assign(static_cast<size_t>(nc) * 3 * Np * Np, 0.0);
    O.Lf.assign(static_cast<size_t>(nc) * nf * Np * Nfp, 0.0);
    for (int c = 0; c < nc; ++c) {
        int64_t e = rep[c];
        ElemMats m = elem_mats(O, e, vq);
        for (int d = 0; d < dim; ++d)
            for (int q = 0; q < Np * Np; ++q) O.Dx[(static_cast<size_t>(c) * 3 + d) * Np * Np + q] = m.D[d][q];
        // face mass of each local face, restricted to its nodes, premultiplied by M^-1
        for (int f = 0; f < nf; ++f) {
            Face tmp{}; tmp.e1 = e; tmp.f1 = f; tmp.e2 = -1;
            double nrm[3]; double jac; face_normal(O, e, f, nrm, jac);
            vector<double> xq, wq; face_points(O, tmp, xq, wq);
            vector<double> Mf(Np * Nfp, 0.0), phi(Np);
            for (size_t k = 0; k < wq.size(); ++k) {
                double xi[3]; O.phys_to_ref(e, &xq[3 * k], xi); O.B.shape(xi, phi.data());
                double w = wq[k] * jac;
                for (int i = 0; i < Np; ++i)
                    for (int a = 0; a < Nfp; ++a) Mf[i * Nfp + a] += w * phi[i] * phi[O.fnodes[f * Nfp + a]];
            }
            for (int i = 0; i < Np; ++i) for (int a = 0; a < Nfp; ++a) {
                double s = 0; for (int l = 0; l < Np; ++l) s += m.Minv[i * Np + l] * Mf[l * Nfp + a];
                O.Lf[((static_cast<size_t>(c) * nf + f) * Np + i) * Nfp + a] = s;
            }
        }
    }
    // node maps by coordinate matching
    O.vmapP.assign(O.K * nf * Nfp, -1);
    for (int64_t e = 0; e < O.K; ++e)
        for (int f = 0; f < nf; ++f) {
            const Face& F = O.faces[O.elem_face[e * nf + f]];
            int64_t en = (F.e1 == e) ? F.e2 : F.e1;
            int fn = (F.e1 == e) ? F.f2 : F.f1;
            for (int a = 0; a < Nfp; ++a) {
                int64_t gm = e * Np + O.fnodes[f * Nfp + a];
                if (en < 0) { O.vmapP[(e * nf + f) * Nfp + a] = gm; continue; }
                double best = 1e300; int64_t bi = -1;
                for (int b = 0; b < Nfp; ++b) {
                    int64_t gp = en * Np + O.fnodes[fn * Nfp + b];
                    double d = 0; for (int r = 0; r < 3; ++r) { double q = O.X[r * O.N + gm] - O.X[r * O.N + gp]; d += q * q; }
                    if (d < best) { best = d; bi = gp; }
                }
                O.vmapP[(e * nf + f) * Nfp + a] = bi;
            }
        }
    O.have_nodal = true;
}

static void mult_nodal(Oracle& O, const double* u, double* out, double t)
{
    if (!O.have_nodal) build_nodal(O);
    const int Np = O.Np, Nfp = O.Nfp, nf = O.nfaces, dim = O.dim;
    const int64_t N = O.N;
    const bool skip = O.tfsf_elems.empty() || tfsf_skip(O, t);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < O.K; ++e) {
        const int c = O.shape_of[e];
        vector<double> flux(6 * nf * Nfp);
        for (int f = 0; f < nf; ++f) {
            const Face& F = O.faces[O.elem_face[e * nf + f]];
            double n[3] = {F.n[0], F.n[1], F.n[2]};
            if (F.e1 != e) for (int r = 0; r < 3; ++r) n[r] = -n[r];
            for (int a = 0; a < Nfp; ++a) {
                int64_t gm = e * Np + O.fnodes[f * Nfp + a];
                int64_t gp = O.vmapP[(e * nf + f) * Nfp + a];
                double dE[3], dH[3], aE = O.alpha, aH = O.alpha;
                for (int q = 0; q < 3; ++q) { dE[q] = u[q * N + gp] - u[q * N + gm]; dH[q] = u[(3 + q) * N + gp] - u[(3 + q) * N + gm]; }
                int bc = -1;
                if (F.kind == 1 || F.kind == 3) bc = F.bc;
                if (bc >= 0) {
                    // image rules equivalent to the assembled boundary coefficients
                    double cE = bc_coeff(bc, 0), cH = bc_coeff(bc, 1);
                    if (bc == BC_OPEN) { cE = 0; cH = 0; }
                    for (int q = 0; q < 3; ++q) { dE[q] = -cE * u[q * N + gm]; dH[q] = -cH * u[(3 + q) * N + gm]; }
                    if (bc == BC_SMA) { aE = 1.0; aH = 1.0; }
                }
                if (F.kind == 2 && !skip) {
                    int side = (F.e1 == e) ? F.tf_side : -F.tf_side;
                    double xx[3] = {O.X[gm], O.X[N + gm], O.X[2 * N + gm]}, pe[3], ph[3];
                    pw_at(O, xx, t, pe, ph);
                    for (int q = 0; q < 3; ++q) { dE[q] += side * pe[q]; dH[q] += side * ph[q]; }
                }
                double ndE = n[0] * dE[0] + n[1] * dE[1] + n[2] * dE[2];
                double ndH = n[0] * dH[0] + n[1] * dH[1] + n[2] * dH[2];
                double fe[3], fh[3];
                fe[0] = (n[1] * dH[2] - n[2] * dH[1]) + aE * (dE[0] - ndE * n[0]);
                fe[1] = (n[2] * dH[0] - n[0] * dH[2]) + aE * (dE[1] - ndE * n[1]);
                fe[2] = (n[0] * dH[1] - n[1] * dH[0]) + aE * (dE[2] - ndE * n[2]);
                fh[0] = -(n[1] * dE[2] - n[2] * dE[1]) + aH * (dH[0] - ndH * n[0]);
                fh[1] = -(n[2] * dE[0] - n[0] * dE[2]) + aH * (dH[1] - ndH * n[1]);
                fh[2] = -(n[0] * dE[1] - n[1] * dE[0]) + aH * (dH[2] - ndH * n[2]);
                for (int q = 0; q < 3; ++q) {
                    flux[(q * nf + f) * Nfp + a] = 0.5 * fe[q];
                    flux[((3 + q) * nf + f) * Nfp + a] = 0.5 * fh[q];
                }
            }
        }
        const double ie = 1.0 / O.eps[e], im = 1.0 / O.mu[e], se = O.sig[e] / O.eps[e];
        for (int i = 0; i < Np; ++i) {
            double d[6][3] = {};
            for (int dd = 0; dd < dim; ++dd) {
                const double* Drow = &O.Dx[((static_cast<size_t>(c) * 3 + dd) * Np + i) * Np];
                for (int q = 0; q < 6; ++q) {
                    double s = 0; for (int j = 0; j < Np; ++j) s += Drow[j] * u[q * N + e * Np + j];
                    d[q][dd] = s;
                }
            }
            double lf[6] = {};
            for (int f = 0; f < nf; ++f) {
                const double* L = &O.Lf[((static_cast<size_t>(c) * nf + f) * Np + i) * Nfp];
                for (int q = 0; q < 6; ++q) {
                    double s = 0; for (int a = 0; a < Nfp; ++a) s += L[a] * flux[(q * nf + f) * Nfp + a];
                    lf[q] += s;
                }
            }
            // curl: (curl F)_x = dF_z/dy - dF_y/dz ...
            double cH[3] = {d[5][1] - d[4][2], d[3][2] - d[5][0], d[4][0] - d[3][1]};
            double cE[3] = {d[2][1] - d[1][2], d[0][2] - d[2][0], d[1][0] - d[0][1]};
            int64_t gi = e * Np + i;
            for (int q = 0; q < 3; ++q) {
                out[q * N + gi] = ie * (cH[q] + lf[q]) - se * u[q * N + gi];
                out[(3 + q) * N + gi] = im * (-cE[q] + lf[3 + q]);
            }
        }
    }
}

static void mult(Oracle& O, int form, const double* x, double* y, double t)
{
    if (form == 0) mult_global(O, x, y, t);
    else mult_nodal(O, x, y, t);
}

// mfem::RK4Solver::Step register sequence.
static void rk4_step(Oracle& O, int form, double* x, double t, double dt, vector<double>& k, vector<double>& y,
                     vector<double>& z)
{
    const int64_t L = 6 * O.N;
    mult(O, form, x, k.data(), t);
    for (int64_t i = 0; i < L; ++i) { y[i] = x[i] + dt / 2 * k[i]; z[i] = x[i] + dt / 6 * k[i]; }
    mult(O, form, y.data(), k.data(), t + dt / 2);
    for (int64_t i = 0; i < L; ++i) { y[i] = x[i] + dt / 2 * k[i]; z[i] += dt / 3 * k[i]; }
    mult(O, form, y.data(), k.data(), t + dt / 2);
    for (int64_t i = 0; i < L; ++i) { y[i] = x[i] + dt * k[i]; z[i] += dt / 3 * k[i]; }
    mult(O, form, y.data(), k.data(), t + dt);
    for (int64_t i = 0; i < L; ++i) x[i] = z[i] + dt / 6 * k[i];
}

static const double LSA[5] = {0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
                              -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0};
static const double LSB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                              1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                              2277821191437.0 / 14882151754819.0};
static const double LSC[5] = {0.0, 1432997174477.0 / 9575080441755.0, 2526269341429.0 / 6820363962896.0,
                              2006345519317.0 / 3224310063776.0, 2802321613138.0 / 2924317926251.0};

static void lserk_step(Oracle& O, int form, double* x, double t, double dt, vector<double>& k, vector<double>& res)
{
    const int64_t L = 6 * O.N;
    for (int s = 0; s < 5; ++s) {
        mult(O, form, x, k.data(), t + LSC[s] * dt);
        for (int64_t i = 0; i < L; ++i) { res[i] = LSA[s] * res[i] + dt * k[i]; x[i] += LSB[s] * res[i]; }
    }
}


// ---------------------------------------------------------------- thin layers (SGBC)
// Restates the reference's SGBC coupling:
//  - one 1D DG sub-solver per face node pair (SGBCWrapper, src/solver/SolverExtension.cpp:49-173,
//    509-559): n_ghost = max(3, p+1) vacuum ghost segments of width (total width / total segments)
//    on each side of the layers, SMA at both ends, the stack's optional PEC/PMC/SMA sheets at the
//    ghost/layer interfaces, order max over layers, upwind alpha 1;
//  - SDIRK33 steps (Solver options of the sub-solver, SolverExtension.cpp:163-170) whose implicit
//    solves use the dense (I - h A) factorisation (GlobalEvolution::ImplicitSolve,
//    GlobalEvolution.cpp:1118-1168), Alexander's three-stage L-stable tableau;
//  - pairs: per face node, (node of the face's first element, matching node of the second),
//    rotation from the first element's outward normal (GlobalEvolution.cpp:48-127,
//    SolverExtension.h:68-107);
//  - per step: checkpoint, per stage a sub-solve from the checkpoint to the stage time with the
//    stage vector as ghost data and the 1e-8 quiescence skips, two-pass injection through the
//    source-face operator, and a final advance over the whole step with ghosts interpolated
//    linearly between the step's end points (GlobalEvolution.cpp:395-545, 639-1001;
//    Solver::step, Solver.cpp:535-551).
struct SgbcLayerP { double eps, mu, sigma, width; int segments, order; };

struct SgbcStack {
    vector<SgbcLayerP> layers;
    int left_bc = 0, right_bc = 0;   // 0: transparent, else BC_PEC / BC_PMC / BC_SMA
    double sub_dt = 0.0;
    int p = 1, nghost = 3, Np1 = 2;
    int64_t K1 = 0, local = 0, n = 0;   // local = K1 * Np1 nodes per component; n = 6 * local
    vector<double> A;                    // dense n x n sub-solver operator
    double lu_h = -1.0; vector<double> LU; vector<int> piv;
    int64_t idx_left() const { return static_cast<int64_t>(nghost) * Np1; }
    int64_t idx_right() const { return local - 1 - static_cast<int64_t>(nghost) * Np1; }
};

struct SgbcPair {
    int64_t gl, gr;
    double rot[9];
    int stack;
    vector<double> state, cp;
    double ghost_old[12], ghost_new[12];
};

struct Sgbc {
    vector<SgbcStack> stacks;
    vector<SgbcPair> pairs;
    vector<int64_t> elem1, elem2;   // elements of the pairs' first / second nodes (unique, ascending)
    double base = 0.0, dt = 0.0;
};

static void sgbc_rotation(const double* nrm, double* R)
{
    // buildFaceRotationMatrix, 3D branch (SolverExtension.h:68-107)
    double nx = nrm[0], ny = nrm[1], nz = nrm[2];
    const double len = std::sqrt(nx * nx + ny * ny + nz * nz);
    nx /= len; ny /= len; nz /= len;
    R[0] = nx; R[1] = ny; R[2] = nz;
    double rx = 0, ry = 0, rz = 0;
    if (std::fabs(nx) < 0.9) rx = 1.0; else ry = 1.0;
    double t1x = ny * rz - nz * ry, t1y = nz * rx - nx * rz, t1z = nx * ry - ny * rx;
    const double tl = std::sqrt(t1x * t1x + t1y * t1y + t1z * t1z);
    t1x /= tl; t1y /= tl; t1z /= tl;
    R[3] = t1x; R[4] = t1y; R[5] = t1z;
    R[6] = ny * t1z - nz * t1y; R[7] = nz * t1x - nx * t1z; R[8] = nx * t1y - ny * t1x;
}

// The sub-solver mesh (buildSGBCMesh, SolverExtension.cpp:49-118) and its assembled operator.
static void sgbc_build_stack(SgbcStack& S)
{
    if (S.layers.empty()) throw std::runtime_error("oracle: SGBC stack without layers");
    int64_t nseg = 0; double width = 0.0; int p = 1;
    for (auto& L : S.layers) {
        if (L.segments < 1 || !(L.width > 0)) throw std::runtime_error("oracle: SGBC layer needs segments >= 1, width > 0");
        nseg += L.segments; width += L.width; p = std::max(p, L.order);
    }
    S.p = p; S.Np1 = p + 1; S.nghost = std::max(3, p + 1);
    const double gdx = width / static_cast<double>(nseg);
    vector<double> xs;
    for (int i = 0; i <= S.nghost; ++i) xs.push_back(i * gdx);
    double x = S.nghost * gdx;
    for (auto& L : S.layers) {
        const double dx = L.width / L.segments;
        for (int i = 0; i < L.segments; ++i) { x += dx; xs.push_back(x); }
    }
    for (int i = 1; i <= S.nghost; ++i) xs.push_back(x + i * gdx);
    const int64_t nv = static_cast<int64_t>(xs.size()), ne = nv - 1;
    vector<double> verts(3 * nv, 0.0);
    for (int64_t i = 0; i < nv; ++i) verts[3 * i] = xs[i];
    vector<int32_t> el(2 * ne);
    vector<double> eps(ne, 1.0), mu(ne, 1.0), sig(ne, 0.0);
    for (int64_t i = 0; i < ne; ++i) { el[2 * i] = static_cast<int32_t>(i); el[2 * i + 1] = static_cast<int32_t>(i + 1); }
    int64_t e = S.nghost;
    for (auto& L : S.layers)
        for (int i = 0; i < L.segments; ++i, ++e) { eps[e] = L.eps; mu[e] = L.mu; sig[e] = L.sigma; }
    Oracle O;
    O.dim = 1; O.p = p; O.alpha = 1.0; O.K = ne;
    O.B.init(1, p);
    O.Np = O.B.Np;
    O.verts = verts; O.elems = el; O.eps = eps; O.mu = mu; O.sig = sig;
    build_geometry(O);
    local_face_nodes(O);
    int32_t bf[2] = {0, static_cast<int32_t>(nv - 1)}, bc[2] = {BC_SMA, BC_SMA};
    vector<int32_t> ifc, ic;
    if (S.left_bc) { ifc.push_back(S.nghost); ic.push_back(S.left_bc); }
    if (S.right_bc) { ifc.push_back(static_cast<int32_t>(S.nghost + nseg)); ic.push_back(S.right_bc); }
    build_faces(O, 2, bf, bc, 0, nullptr, static_cast<int64_t>(ic.size()), ifc.data(), ic.data());
    build_global(O);
    S.K1 = ne; S.local = O.N; S.n = 6 * O.N;
    if (O.Np != S.Np1) throw std::runtime_error("oracle: 1D node count");
    S.A.assign(S.n * S.n, 0.0);
    for (int64_t r = 0; r < S.n; ++r)
        for (int64_t k = O.Aglob.rp[r]; k < O.Aglob.rp[r + 1]; ++k) S.A[r * S.n + O.Aglob.ci[k]] += O.Aglob.v[k];
}

// LU factorisation (partial pivoting) of I - h A, kept until h changes
static void sgbc_factor(SgbcStack& S, double h)
{
    const int64_t n = S.n;
    if (h != S.lu_h) {
        S.LU.assign(n * n, 0.0); S.piv.resize(n);
        for (int64_t i = 0; i < n * n; ++i) S.LU[i] = -h * S.A[i];
        for (int64_t i = 0; i < n; ++i) S.LU[i * n + i] += 1.0;
        for (int64_t c = 0; c < n; ++c) {
            int64_t pr = c; double best = std::fabs(S.LU[c * n + c]);
            for (int64_t r = c + 1; r < n; ++r) if (std::fabs(S.LU[r * n + c]) > best) { best = std::fabs(S.LU[r * n + c]); pr = r; }
            S.piv[c] = static_cast<int>(pr);
            if (pr != c) for (int64_t q = 0; q < n; ++q) std::swap(S.LU[c * n + q], S.LU[pr * n + q]);
            const double d = S.LU[c * n + c];
            for (int64_t r = c + 1; r < n; ++r) {
                const double f = S.LU[r * n + c] / d;
                S.LU[r * n + c] = f;
                if (f != 0.0) for (int64_t q = c + 1; q < n; ++q) S.LU[r * n + q] -= f * S.LU[c * n + q];
            }
        }
        S.lu_h = h;
    }
}

// k = (I - h A)^-1 A x with the factorisation of sgbc_factor (read only: safe across threads)
static void sgbc_implicit(const SgbcStack& S, const double* x, double* k)
{
    const int64_t n = S.n;
    for (int64_t r = 0; r < n; ++r) {
        double a = 0; for (int64_t q = 0; q < n; ++q) a += S.A[r * n + q] * x[q];
        k[r] = a;
    }
    for (int64_t c = 0; c < n; ++c) if (S.piv[c] != c) std::swap(k[c], k[S.piv[c]]);
    for (int64_t r = 0; r < n; ++r) { double a = k[r]; for (int64_t q = 0; q < r; ++q) a -= S.LU[r * n + q] * k[q]; k[r] = a; }
    for (int64_t r = n - 1; r >= 0; --r) {
        double a = k[r]; for (int64_t q = r + 1; q < n; ++q) a -= S.LU[r * n + q] * k[q];
        k[r] = a / S.LU[r * n + r];
    }
}

static const double kSdirkGamma = 0.43586652150845899941601945;   // root of 6x^3 - 18x^2 + 9x - 1 in (1/6, 1/2)

// The step SGBCWrapper::solve takes (SolverExtension.cpp:412-445): the sub-solver's Solver::step
// of dt from t is one SDIRK33 step of min(dt, (t + dt) - t); none below 1e-9 (returns 0).
static double sgbc_step_size(double t, double dt)
{
    if (std::fabs(dt) < 1e-9) return 0.0;
    return std::min(dt, (t + dt) - t);
}

// One SDIRK33 step of size h (> 0) with the factorisation of I - gamma h A in place.
static void sgbc_sdirk(const SgbcStack& S, double* x, double h)
{
    const double g = kSdirkGamma;
    const double a21 = 0.5 * (1.0 - g);
    const double b1 = -(6.0 * g * g - 16.0 * g + 1.0) / 4.0;
    const double b2 = (6.0 * g * g - 20.0 * g + 5.0) / 4.0;
    const int64_t n = S.n;
    vector<double> k(n), y(n);
    sgbc_implicit(S, x, k.data());
    for (int64_t i = 0; i < n; ++i) { y[i] = x[i] + a21 * h * k[i]; x[i] += b1 * h * k[i]; }
    sgbc_implicit(S, y.data(), k.data());
    for (int64_t i = 0; i < n; ++i) x[i] += b2 * h * k[i];
    sgbc_implicit(S, x, k.data());
    for (int64_t i = 0; i < n; ++i) x[i] += g * h * k[i];
}

static void sgbc_set_ghosts(const SgbcStack& S, double* x, const double* g);

// Sub-step q of every listed pair of stack S: ghosts (per pair, from ghost(P, g)), then the
// SDIRK33 step from t; the factorisation is made once, the pairs run in parallel.
template <typename GhostFn>
static void sgbc_substep(SgbcStack& S, vector<SgbcPair*>& pairs, double t, double dt, GhostFn&& ghost)
{
    const double h = sgbc_step_size(t, dt);
    if (h > 0.0) sgbc_factor(S, kSdirkGamma * h);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t i = 0; i < static_cast<int64_t>(pairs.size()); ++i) {
        SgbcPair& P = *pairs[i];
        double g[12];
        ghost(P, g);
        sgbc_set_ghosts(S, P.state.data(), g);
        if (h > 0.0) sgbc_sdirk(S, P.state.data(), h);
    }
}

// Ghost elements take the face-local values (updateFieldsWithGlobalVector /
// updateFieldsWithInterpolatedGhost, SolverExtension.cpp:250-371): g[0..5] left, g[6..11] right.
static void sgbc_set_ghosts(const SgbcStack& S, double* x, const double* g)
{
    const int64_t tg = static_cast<int64_t>(S.nghost) * S.Np1, L = S.local;
    for (int c = 0; c < 6; ++c)
        for (int64_t q = 0; q < tg; ++q) { x[c * L + q] = g[c]; x[c * L + (L - 1 - q)] = g[6 + c]; }
}

static void sgbc_local(const SgbcPair& P, const double* x, int64_t N, int64_t node, double* out6)
{
    double eg[3], hg[3];
    for (int d = 0; d < 3; ++d) { eg[d] = x[d * N + node]; hg[d] = x[(3 + d) * N + node]; }
    for (int i = 0; i < 3; ++i) {
        out6[i] = P.rot[3 * i] * eg[0] + P.rot[3 * i + 1] * eg[1] + P.rot[3 * i + 2] * eg[2];
        out6[3 + i] = P.rot[3 * i] * hg[0] + P.rot[3 * i + 1] * hg[1] + P.rot[3 * i + 2] * hg[2];
    }
}

static double sgbc_norm(const vector<double>& v)
{
    double a = 0; for (double q : v) a += q * q;
    return std::sqrt(a);
}

static double sgbc_iface2(const SgbcPair& P, const double* x, int64_t N)
{
    double a = 0;
    for (int c = 0; c < 6; ++c) { const double u = x[c * N + P.gl], w = x[c * N + P.gr]; a += u * u + w * w; }
    return a;
}

static int sgbc_nsteps(double sub_dt, double span)
{
    return (sub_dt > 0.0 && sub_dt < span) ? static_cast<int>(std::ceil(span / sub_dt)) : 1;
}

static const double kSgbcThr = 1e-8;

static void sgbc_stage(Oracle& O, const double* x, double t, bool& quiescent)
{
    Sgbc& G = *O.sgbc;
    const double thr2 = kSgbcThr * kSgbcThr;
    for (auto& P : G.pairs) P.state = P.cp;
    quiescent = true;
    for (auto& P : G.pairs)
        if (sgbc_norm(P.state) >= kSgbcThr || sgbc_iface2(P, x, O.N) >= thr2) { quiescent = false; break; }
    const double span = t - G.base;
    if (quiescent || !(span > 1e-12)) return;
    for (size_t s = 0; s < G.stacks.size(); ++s) {
        SgbcStack& S = G.stacks[s];
        const int ns = sgbc_nsteps(S.sub_dt, span);
        const double h = span / ns;
        vector<SgbcPair*> list;
        for (auto& P : G.pairs) {
            if (P.stack != static_cast<int>(s)) continue;
            if (sgbc_norm(P.state) < kSgbcThr && sgbc_iface2(P, x, O.N) < thr2) continue;
            list.push_back(&P);
        }
        const int64_t N = O.N;
        for (int q = 0; q < ns; ++q)
            sgbc_substep(S, list, G.base + q * h, h, [&](const SgbcPair& P, double* g) {
                sgbc_local(P, x, N, P.gl, g);
                sgbc_local(P, x, N, P.gr, g + 6);
            });
    }
}

// Slot values of the injection (fillBCSlot, GlobalEvolution.cpp:839-871)
static void sgbc_slot(const SgbcPair& P, const SgbcStack& S, int bc, const double* x, int64_t N, int64_t src,
                      int64_t idx, double* out6)
{
    if (bc == BC_PEC || bc == BC_PMC || bc == BC_SMA) {
        const double se = (bc == BC_PEC) ? -1.0 : 1.0, sh = (bc == BC_PMC) ? -1.0 : 1.0;
        for (int d = 0; d < 3; ++d) { out6[d] = se * x[d * N + src]; out6[3 + d] = sh * x[(3 + d) * N + src]; }
        return;
    }
    double el[3], hl[3];
    for (int d = 0; d < 3; ++d) { el[d] = P.state[d * S.local + idx]; hl[d] = P.state[(3 + d) * S.local + idx]; }
    for (int d = 0; d < 3; ++d) {
        out6[d] = P.rot[d] * el[0] + P.rot[3 + d] * el[1] + P.rot[6 + d] * el[2];
        out6[3 + d] = P.rot[d] * hl[0] + P.rot[3 + d] * hl[1] + P.rot[6 + d] * hl[2];
    }
}

static void sgbc_rows(const Oracle& O, const vector<int64_t>& elems, const vector<double>& sv, double* y)
{
    for (int c = 0; c < 6; ++c)
        for (int64_t e : elems)
            for (int i = 0; i < O.Np; ++i) {
                const int64_t r = c * O.N + e * O.Np + i;
                double a = 0;
                for (int64_t k = O.Tsgbc.rp[r]; k < O.Tsgbc.rp[r + 1]; ++k) a += O.Tsgbc.v[k] * sv[O.Tsgbc.ci[k]];
                y[r] += a;
            }
}

// Two-pass injection (GlobalEvolution.cpp:822-986): rows of the first elements with
// (u at the first node, slab left value) and rows of the second elements with
// (slab right value, u at the second node).
static void sgbc_inject(Oracle& O, const double* x, double* y)
{
    Sgbc& G = *O.sgbc;
    const int64_t N = O.N;
    vector<double> sv(6 * N, 0.0);
    double v[6];
    for (auto& P : G.pairs) {
        const SgbcStack& S = G.stacks[P.stack];
        for (int c = 0; c < 6; ++c) sv[c * N + P.gl] = x[c * N + P.gl];
        sgbc_slot(P, S, S.left_bc, x, N, P.gl, S.idx_left(), v);
        for (int c = 0; c < 6; ++c) sv[c * N + P.gr] = v[c];
    }
    sgbc_rows(O, G.elem1, sv, y);
    std::fill(sv.begin(), sv.end(), 0.0);
    for (auto& P : G.pairs) {
        const SgbcStack& S = G.stacks[P.stack];
        sgbc_slot(P, S, S.right_bc, x, N, P.gr, S.idx_right(), v);
        for (int c = 0; c < 6; ++c) sv[c * N + P.gl] = v[c];
        for (int c = 0; c < 6; ++c) sv[c * N + P.gr] = x[c * N + P.gr];
    }
    sgbc_rows(O, G.elem2, sv, y);
}

static void sgbc_commit(Oracle& O, double t, double dt, const double* x)
{
    Sgbc& G = *O.sgbc;
    G.base = t; G.dt = dt;
    for (auto& P : G.pairs) {
        P.cp = P.state;
        sgbc_local(P, x, O.N, P.gl, P.ghost_old);
        sgbc_local(P, x, O.N, P.gr, P.ghost_old + 6);
    }
}

static void sgbc_finalize(Oracle& O, const double* x)
{
    Sgbc& G = *O.sgbc;
    const double thr2 = kSgbcThr * kSgbcThr;
    bool quiescent = true;
    for (auto& P : G.pairs) {
        P.state = P.cp;
        sgbc_local(P, x, O.N, P.gl, P.ghost_new);
        sgbc_local(P, x, O.N, P.gr, P.ghost_new + 6);
    }
    for (auto& P : G.pairs)
        if (sgbc_norm(P.state) >= kSgbcThr || sgbc_iface2(P, x, O.N) >= thr2) { quiescent = false; break; }
    if (quiescent) return;
    for (size_t s = 0; s < G.stacks.size(); ++s) {
        SgbcStack& S = G.stacks[s];
        const int ns = sgbc_nsteps(S.sub_dt, G.dt);
        const double h = G.dt / ns;
        vector<SgbcPair*> list;
        for (auto& P : G.pairs)
            if (P.stack == static_cast<int>(s)) list.push_back(&P);
        for (int q = 0; q < ns; ++q) {
            const double a = static_cast<double>(q + 1) / ns, b = 1.0 - a;
            sgbc_substep(S, list, G.base + q * h, h, [&](const SgbcPair& P, double* g) {
                for (int c = 0; c < 12; ++c) g[c] = b * P.ghost_old[c] + a * P.ghost_new[c];
            });
        }
    }
}

// Pairs of the kind-4 faces: (node of e1, node of e2 at the same position), stack per face.
static void sgbc_setup(Oracle& O, vector<SgbcStack> stacks, const int32_t* face_stack)
{
    if (O.dim != 3) throw std::runtime_error("oracle: SGBC coupling is 3D");
    auto G = std::make_shared<Sgbc>();
    G->stacks = std::move(stacks);
    for (auto& S : G->stacks) sgbc_build_stack(S);
    vector<char> m1(O.K, 0), m2(O.K, 0);
    for (size_t q = 0; q < O.sgbc_faces.size(); ++q) {
        const Face& F = O.faces[O.sgbc_faces[q]];
        const int st = face_stack[q];
        if (st < 0 || st >= static_cast<int>(G->stacks.size())) throw std::runtime_error("oracle: SGBC stack index");
        double R[9]; sgbc_rotation(F.n, R);
        const bool curved_face = O.is_curved(F.e1) || O.is_curved(F.e2);
        for (int a = 0; a < O.Nfp; ++a) {
            const int n1 = O.fnodes[F.f1 * O.Nfp + a];
            const int64_t g1 = F.e1 * O.Np + n1;
            if (curved_face) {
                // per-node normal on a curved face (computePerDofFaceNormals, SubMesher.cpp:138-194;
                // here exactly at the node): the face tangents of e1's map there, out of e1
                static const double rv[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
                int l1[3], c = 0;
                for (int q = 0; q < 4; ++q) if (q != F.f1) l1[c++] = q;
                double x[3], J[9], tu[3], tv[3], cr[3];
                geom(O, F.e1, &O.B.nodes[n1 * 3], x, J);
                for (int r = 0; r < 3; ++r) {
                    tu[r] = tv[r] = 0.0;
                    for (int d = 0; d < 3; ++d) {
                        tu[r] += J[r * 3 + d] * (rv[l1[1]][d] - rv[l1[0]][d]);
                        tv[r] += J[r * 3 + d] * (rv[l1[2]][d] - rv[l1[0]][d]);
                    }
                }
                cross(tu, tv, cr);
                if (cr[0] * F.n[0] + cr[1] * F.n[1] + cr[2] * F.n[2] < 0) for (int r = 0; r < 3; ++r) cr[r] = -cr[r];
                sgbc_rotation(cr, R);
            }
            int64_t g2 = -1; double best = 1e300;
            for (int b = 0; b < O.Nfp; ++b) {
                const int64_t c2 = F.e2 * O.Np + O.fnodes[F.f2 * O.Nfp + b];
                double d = 0; for (int r = 0; r < 3; ++r) { const double u = O.X[r * O.N + g1] - O.X[r * O.N + c2]; d += u * u; }
                if (d < best) { best = d; g2 = c2; }
            }
            SgbcPair P;
            P.gl = g1; P.gr = g2; std::memcpy(P.rot, R, sizeof R); P.stack = st;
            P.state.assign(G->stacks[st].n, 0.0); P.cp = P.state;
            std::fill(P.ghost_old, P.ghost_old + 12, 0.0); std::fill(P.ghost_new, P.ghost_new + 12, 0.0);
            G->pairs.push_back(std::move(P));
        }
        m1[F.e1] = 1; m2[F.e2] = 1;
    }
    for (int64_t e = 0; e < O.K; ++e) { if (m1[e]) G->elem1.push_back(e); if (m2[e]) G->elem2.push_back(e); }
    O.sgbc = G;
}

static vector<SgbcStack> sgbc_stacks_from(int n_stacks, const int32_t* layer_counts, const double* layer_prm,
                                          const int32_t* bcs, const double* sub_dts)
{
    vector<SgbcStack> out(n_stacks);
    int64_t li = 0;
    for (int s = 0; s < n_stacks; ++s) {
        for (int q = 0; q < layer_counts[s]; ++q, ++li) {
            const double* L = layer_prm + 6 * li;
            out[s].layers.push_back({L[0], L[1], L[2], L[3], static_cast<int>(L[4]), static_cast<int>(L[5])});
        }
        out[s].left_bc = bcs[2 * s]; out[s].right_bc = bcs[2 * s + 1];
        out[s].sub_dt = sub_dts[s];
    }
    return out;
}

// One RK step with the SGBC checkpoint and finalisation around it (Solver::step)
static void step_any(Oracle& O, int form, double* x, double t, double dt, int integrator, vector<double>& k,
                     vector<double>& y, vector<double>& z)
{
    if (O.sgbc) {
        if (form != 0) throw std::runtime_error("oracle: thin-layer (SGBC) faces exist in the global form only");
        sgbc_commit(O, t, dt, x);
    }
    if (integrator == 0) rk4_step(O, form, x, t, dt, k, y, z);
    else lserk_step(O, form, x, t, dt, k, z);
    if (O.sgbc) sgbc_finalize(O, x);
}

}  // namespace orc

// ================================================================ C API
extern "C" {

static thread_local std::string g_orc_err;
const char* orc_last_error(void) { return g_orc_err.c_str(); }

void* orc_create(int dim, int order, double alpha, int64_t nv, const double* verts, int64_t ne, const int32_t* elems,
                 const double* eps, const double* mu, const double* sigma, int64_t nb, const int32_t* bfaces,
                 const int32_t* bcodes, int64_t nt, const int32_t* tfaces, int64_t ni, const int32_t* ifaces,
                 const int32_t* icodes)
{
    try {
        if (dim != 1 && dim != 3) throw std::runtime_error("oracle: dim must be 1 or 3");
        auto O = std::make_unique<orc::Oracle>();
        O->dim = dim; O->p = order; O->alpha = alpha; O->K = ne;
        O->B.init(dim, order);
        O->Np = O->B.Np;
        O->verts.assign(verts, verts + 3 * nv);
        O->elems.assign(elems, elems + (dim + 1) * ne);
        O->eps.assign(ne, 1.0); O->mu.assign(ne, 1.0); O->sig.assign(ne, 0.0);
        if (eps) O->eps.assign(eps, eps + ne);
        if (mu) O->mu.assign(mu, mu + ne);
        if (sigma) O->sig.assign(sigma, sigma + ne);
        orc::build_geometry(*O);
        orc::local_face_nodes(*O);
        orc::build_faces(*O, nb, bfaces, bcodes, nt, tfaces, ni, ifaces, icodes);
        return O.release();
    } catch (const std::exception& e) {
        g_orc_err = e.what();
        return nullptr;
    }
}

// Switch a fresh 3D oracle to the Gauss-Legendre node set (basis_type 0; 1 keeps Gauss-Lobatto):
// the global form is assembled by quadrature and holds for either; the nodal form, SGBC and
// curved elements need the Gauss-Lobatto set's face nodes and are refused afterwards.
int orc_set_basis(void* h, int basis_type)
{
    try {
        auto* O = static_cast<orc::Oracle*>(h);
        if (basis_type == 1 && !O->legendre) return 0;
        if (basis_type != 0) throw std::runtime_error("oracle: basis_type must be 0 or 1 (and set once)");
        if (O->dim != 3) throw std::runtime_error("oracle: Gauss-Legendre basis in 3D only");
        if (O->have_csr || O->have_nodal || O->sgbc || !O->cidx.empty())
            throw std::runtime_error("oracle: set the basis before assembling, SGBC or curved elements");
        O->B.init(3, O->p, true);
        O->legendre = true;
        orc::build_geometry(*O);
        O->Nfp = 0;
        O->fnodes.clear();
        return 0;
    } catch (const std::exception& e) {
        g_orc_err = e.what();
        return -1;
    }
}

void orc_destroy(void* h) { delete static_cast<orc::Oracle*>(h); }
int64_t orc_ndofs(void* h) { return static_cast<orc::Oracle*>(h)->N; }
int orc_np(void* h) { return static_cast<orc::Oracle*>(h)->Np; }
void orc_nodes(void* h, double* xyz)
{
    auto* O = static_cast<orc::Oracle*>(h);
    std::memcpy(xyz, O->X.data(), O->X.size() * sizeof(double));
}

// params: [n][11] = k(3), pol(3), spread, mean, freq, unused, unused
void orc_set_planewaves(void* h, int n, const double* prm)
{
    auto* O = static_cast<orc::Oracle*>(h);
    O->pws.clear();
    for (int i = 0; i < n; ++i) {
        const double* q = prm + 11 * i;
        orc::PW w{};
        double kn = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
        double pn = std::sqrt(q[3] * q[3] + q[4] * q[4] + q[5] * q[5]);
        for (int c = 0; c < 3; ++c) { w.k[c] = q[c] / kn; w.pol[c] = q[3 + c] / pn; }
        orc::cross(w.k, w.pol, w.kxp);
        w.spread = q[6]; w.mean = q[7]; w.freq = q[8];
        O->pws.push_back(w);
    }
}

int orc_mult(void* h, int form, const double* x, double* y, double t)
{
    try { orc::mult(*static_cast<orc::Oracle*>(h), form, x, y, t); }
    catch (const std::exception& e) { g_orc_err = e.what(); return -1; }
    return 0;
}

int orc_step(void* h, int form, double* x, double t0, double dt, int nsteps, int integrator)
{
    try {
        auto& O = *static_cast<orc::Oracle*>(h);
        const int64_t L = 6 * O.N;
        std::vector<double> k(L), y(L), z(L, 0.0);
        double t = t0;
        for (int s = 0; s < nsteps; ++s) {
            orc::step_any(O, form, x, t, dt, integrator, k, y, z);
            t += dt;
        }
    } catch (const std::exception& e) { g_orc_err = e.what(); return -1; }
    return 0;
}

// Reference run loop (Solver::run, Solver.cpp:483-551)
int orc_run(void* h, int form, double* x, double t0, double dt, double T, int integrator, int64_t* steps)
{
    try {
        auto& O = *static_cast<orc::Oracle*>(h);
        const int64_t L = 6 * O.N;
        std::vector<double> k(L), y(L), z(L, 0.0);
        double t = t0; int64_t n = 0;
        while (t <= T - 1e-8 * dt) {
            double h2 = std::min(dt, T - t);
            orc::step_any(O, form, x, t, h2, integrator, k, y, z);
            t += h2; ++n;
        }
        if (steps) *steps = n;
    } catch (const std::exception& e) { g_orc_err = e.what(); return -1; }
    return 0;
}

int64_t orc_nnz(void* h)
{
    auto& O = *static_cast<orc::Oracle*>(h);
    if (!O.have_csr) orc::build_global(O);
    return static_cast<int64_t>(O.Aglob.v.size());
}

// Element matrices on one element with the given vertices (for known-answer tests):
// M, Minv, D_x, D_y, D_z (each Np x Np); D_d = M^-1 S_d, S_d = int phi_i dphi_j/dx_d.
int orc_element_matrices(int dim, int order, const double* verts, double* M, double* Minv, double* Sx, double* Sy,
                         double* Sz)
{
    try {
        int32_t el[4] = {0, 1, 2, 3};
        void* h = orc_create(dim, order, 1.0, dim + 1, verts, 1, el, nullptr, nullptr, nullptr, 0, nullptr, nullptr, 0,
                             nullptr, 0, nullptr, nullptr);
        if (!h) return -1;
        auto& O = *static_cast<orc::Oracle*>(h);
        orc::Quad vq;
        if (dim == 3) vq = orc::tet_quad(order + 3);
        else { std::vector<double> g, gw; orc::gauss_legendre01(order + 2, g, gw); vq.x = g; vq.w = gw; }
        auto m = orc::elem_mats(O, 0, vq);
        const size_t n2 = static_cast<size_t>(O.Np) * O.Np;
        if (M) std::memcpy(M, m.M.data(), n2 * sizeof(double));
        if (Minv) std::memcpy(Minv, m.Minv.data(), n2 * sizeof(double));
        if (Sx) std::memcpy(Sx, m.D[0].data(), n2 * sizeof(double));
        if (Sy) std::memcpy(Sy, m.D[1].data(), n2 * sizeof(double));
        if (Sz) std::memcpy(Sz, m.D[2].data(), n2 * sizeof(double));
        orc_destroy(h);
    } catch (const std::exception& e) { g_orc_err = e.what(); return -1; }
    return 0;
}

// One scalar sub-operator as a dense [N x N] matrix (N = K Np), for known-answer
// tests of the integrators (reference test/hesthavenComparison/Hesthaven1DTest.cpp):
// out = (M^-1 / minv_coef) * F with F one of
//   kind 0: zero-normal jump form, 1: one-normal (dir d), 2: two-normal (d, d2),
//   3: strong derivative S_d = int phi_i dphi_j/dx_d (no faces),
// assembled with beta_int on interior faces and beta_bdr on every boundary face.
int orc_subop(void* h, int kind, int d, int d2, double beta_int, double beta_bdr, double minv_coef, double* out)
{
    try {
        auto& O = *static_cast<orc::Oracle*>(h);
        const int Np = O.Np, nf = O.nfaces;
        const int64_t N = O.N;
        std::memset(out, 0, sizeof(double) * N * N);
        orc::Quad vq;
        if (O.dim == 3) vq = orc::tet_quad(O.p + 3);
        else { std::vector<double> g, gw; orc::gauss_legendre01(O.p + 2, g, gw); vq.x = g; vq.w = gw; }
        std::vector<double> own(Np * Np), coup(Np * Np);
        for (int64_t e = 0; e < O.K; ++e) {
            orc::ElemMats m = orc::elem_mats(O, e, vq);
            std::vector<double> rows(static_cast<size_t>(Np) * N, 0.0);
            if (kind == 3) {
                // D = M^-1 S  -> S = M D
                for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) {
                    double acc = 0; for (int l = 0; l < Np; ++l) acc += m.M[i * Np + l] * m.D[d][l * Np + j];
                    rows[static_cast<size_t>(i) * N + e * Np + j] = acc;
                }
            } else {
                for (int lf = 0; lf < nf; ++lf) {
                    const orc::Face& F = O.faces[O.elem_face[e * nf + lf]];
                    const int side = (F.e1 == e && F.f1 == lf) ? 1 : 2;
                    const double beta = (F.e2 >= 0) ? beta_int : beta_bdr;
                    orc::face_rows(O, F, side, kind, d, d2, beta, false, own.data(), coup.data());
                    int64_t other = (side == 1) ? F.e2 : F.e1;
                    for (int i = 0; i < Np; ++i) for (int j = 0; j < Np; ++j) {
                        rows[static_cast<size_t>(i) * N + e * Np + j] += own[i * Np + j];
                        if (other >= 0) rows[static_cast<size_t>(i) * N + other * Np + j] += coup[i * Np + j];
                    }
                }
            }
            for (int i = 0; i < Np; ++i)
                for (int64_t c = 0; c < N; ++c) {
                    double acc = 0; for (int l = 0; l < Np; ++l) acc += m.Minv[i * Np + l] * rows[static_cast<size_t>(l) * N + c];
                    out[(e * Np + i) * N + c] = acc / minv_coef;
                }
        }
    } catch (const std::exception& ex) { g_orc_err = ex.what(); return -1; }
    return 0;
}

// Emat of the reference's Hesthaven reference tetrahedron ((0,0,0),(2,0,0),(0,2,0),(0,0,2)),
// as assembled by assembleHesthavenRefElemEmat (HesthavenEvolution.cpp:53-81): for each
// face f, the face mass of the element basis (weight 2 * ip.weight, no face Jacobian),
// columns restricted to the face's nodes in ascending order, times 2 for tetrahedra.
int orc_ref_emat(int order, double* emat)
{
    try {
        orc::Basis B; B.init(3, order);
        const int Np = B.Np, Nfp = (order + 1) * (order + 2) / 2;
        orc::Quad tq = orc::tri_quad(order + 2);
        std::memset(emat, 0, sizeof(double) * Np * 4 * Nfp);
        // MFEM reference-tet face vertex sets, face f opposite vertex f
        const double V[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        std::vector<double> phi(Np);
        for (int f = 0; f < 4; ++f) {
            int vv[3], c = 0; for (int q = 0; q < 4; ++q) if (q != f) vv[c++] = q;
            std::vector<int> fn;
            for (int n = 0; n < Np; ++n) { double lam[4]; B.lam_of(&B.nodes[3 * n], lam); if (std::fabs(lam[f]) < 1e-12) fn.push_back(n); }
            for (size_t k = 0; k < tq.w.size(); ++k) {
                double u = tq.x[2 * k], v = tq.x[2 * k + 1], xi[3];
                for (int r = 0; r < 3; ++r) xi[r] = V[vv[0]][r] + u * (V[vv[1]][r] - V[vv[0]][r]) + v * (V[vv[2]][r] - V[vv[0]][r]);
                B.shape(xi, phi.data());
                double w = 2.0 * tq.w[k] * 2.0;
                for (int i = 0; i < Np; ++i)
                    for (int a = 0; a < Nfp; ++a) emat[i * 4 * Nfp + f * Nfp + a] += w * phi[i] * phi[fn[a]];
            }
        }
    } catch (const std::exception& e) { g_orc_err = e.what(); return -1; }
    return 0;
}

// Incident field of the operator's plane waves at point x and time t (E and H, 3 each), for
// tests of the source definition (reference Planewave / Gaussian / ModulatedGaussian,
// src/math/Function.h:45-143, 329-416).
void orc_pw_eval(void* h, const double* x, double t, double* e, double* hf)
{
    orc::pw_at(*static_cast<orc::Oracle*>(h), x, t, e, hf);
}

// Gauss-Lobatto points on [0,1] (the 1D node set), for tests.
int orc_lobatto(int p, double* out)
{
    auto g = orc::lobatto01(p);
    std::memcpy(out, g.data(), g.size() * sizeof(double));
    return 0;
}

int orc_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// Second-order (curved) geometry of n elements: elems[n] element ids, nodes [n][10][3] = the
// element's four corners (its vertex order) then its edge nodes of (0,1) (0,2) (0,3) (1,2) (1,3)
// (2,3). Their DOF node positions move onto the curved map; the global form assembles them with
// per-point Jacobians. Affine meshes need no call.
int orc_set_curved(void* h, int64_t n, const int32_t* elems, const double* nodes)
{
    try {
        auto& O = *static_cast<orc::Oracle*>(h);
        if (O.dim != 3) throw std::runtime_error("oracle: curved elements are 3D");
        if (O.legendre) throw std::runtime_error("oracle: curved elements with the Gauss-Legendre basis");
        O.cidx.assign(O.K, -1);
        O.cnodes.assign(nodes, nodes + 30 * n);
        for (int64_t i = 0; i < n; ++i) {
            if (elems[i] < 0 || elems[i] >= O.K) throw std::runtime_error("oracle: curved element id out of range");
            O.cidx[elems[i]] = i;
        }
        for (int32_t e : O.tfsf_elems)
            if (O.cidx[e] >= 0) throw std::runtime_error("oracle: TF/SF faces on curved elements are not supported");
        for (int64_t i = 0; i < n; ++i) {
            const int64_t e = elems[i];
            for (int k = 0; k < O.Np; ++k) {
                double x[3], J[9], Ji[9];
                orc::geom(O, e, &O.B.nodes[k * 3], x, J);
                if (!(orc::det3(J, Ji) > 0)) throw std::runtime_error("oracle: curved element with a non-positive Jacobian");
                for (int r = 0; r < 3; ++r) O.X[r * O.N + e * O.Np + k] = x[r];
            }
        }
        O.have_csr = false;
    } catch (const std::exception& e) { g_orc_err = e.what(); return -1; }
    return 0;
}

// Thin-layer (SGBC) stacks: layer_prm [total layers][6] = eps_r, mu_r, sigma (solver units), width,
// segments, order; layer_counts [n_stacks]; bcs [n_stacks][2] left/right (0 none, 1 PEC, 2 PMC,
// 3 SMA); sub_dts [n_stacks]; face_stack [SGBC interior faces, in the order given] stack index.
int orc_set_sgbc(void* h, int n_stacks, const int32_t* layer_counts, const double* layer_prm, const int32_t* bcs,
                 const double* sub_dts, const int32_t* face_stack)
{
    try {
        auto& O = *static_cast<orc::Oracle*>(h);
        if (O.legendre) throw std::runtime_error("oracle: SGBC needs face nodes (Gauss-Lobatto basis)");
        orc::sgbc_setup(O, orc::sgbc_stacks_from(n_stacks, layer_counts, layer_prm, bcs, sub_dts), face_stack);
    } catch (const std::exception& e) { g_orc_err = e.what(); return -1; }
    return 0;
}

int64_t orc_sgbc_pairs(void* h)
{
    auto& O = *static_cast<orc::Oracle*>(h);
    return O.sgbc ? static_cast<int64_t>(O.sgbc->pairs.size()) : 0;
}

// One stack on its own, for tests of the sub-solver: its size n, its dense operator, and the
// advance of a state x by span from t0 (ghosts g_old[12] held, or interpolated to g_new[12]).
void* orc_sgbc_stack_create(int n_layers, const double* layer_prm, int left_bc, int right_bc, double sub_dt)
{
    try {
        int32_t cnt = n_layers, bc[2] = {left_bc, right_bc};
        auto v = orc::sgbc_stacks_from(1, &cnt, layer_prm, bc, &sub_dt);
        auto S = std::make_unique<orc::SgbcStack>(std::move(v[0]));
        orc::sgbc_build_stack(*S);
        return S.release();
    } catch (const std::exception& e) { g_orc_err = e.what(); return nullptr; }
}
void orc_sgbc_stack_destroy(void* s) { delete static_cast<orc::SgbcStack*>(s); }
int64_t orc_sgbc_stack_size(void* s) { return static_cast<orc::SgbcStack*>(s)->n; }
void orc_sgbc_stack_matrix(void* s, double* A)
{
    auto& S = *static_cast<orc::SgbcStack*>(s);
    std::memcpy(A, S.A.data(), S.A.size() * sizeof(double));
}
void orc_sgbc_stack_advance(void* s, double* x, const double* g_old, const double* g_new, double t0, double span,
                            int interpolate)
{
    auto& S = *static_cast<orc::SgbcStack*>(s);
    if (!(span > 1e-12)) return;
    const int ns = orc::sgbc_nsteps(S.sub_dt, span);
    const double hh = span / ns;
    for (int q = 0; q < ns; ++q) {
        double g[12];
        if (interpolate) {
            const double a = static_cast<double>(q + 1) / ns, b = 1.0 - a;
            for (int c = 0; c < 12; ++c) g[c] = b * g_old[c] + a * g_new[c];
        } else {
            for (int c = 0; c < 12; ++c) g[c] = g_old[c];
        }
        orc::sgbc_set_ghosts(S, x, g);
        const double h = orc::sgbc_step_size(t0 + q * hh, hh);
        if (h > 0.0) {
            orc::sgbc_factor(S, orc::kSdirkGamma * h);
            orc::sgbc_sdirk(S, x, h);
        }
    }
}
int64_t orc_sgbc_stack_iface(void* s, int right)
{
    auto& S = *static_cast<orc::SgbcStack*>(s);
    return right ? S.idx_right() : S.idx_left();
}

}  // extern "C"
