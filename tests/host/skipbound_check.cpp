// Host check of the TF/SF skip-test bounds (dgtd_gb300/csrc/skipbound.hpp) against the exact
// sum the reference evaluates (GlobalEvolution.cpp:587-598): for random node clouds, waves and
// times, a decided flag must agree with sum_n ||0.5 pw(x_n, t)||^2 < 1e-16. Prints
// "decided <n> undecided <m> wrong <k>" and exits non-zero if any decision is wrong.
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "skipbound.hpp"

int main()
{
    std::mt19937_64 rng(20261204);
    std::uniform_real_distribution<double> U(-1.0, 1.0);
    std::normal_distribution<double> G(0.0, 1.0);
    long decided = 0, undecided = 0, wrong = 0;
    for (int trial = 0; trial < 200; ++trial) {
        const int Np = 10, K = 1 + static_cast<int>(rng() % 50);
        std::vector<double> x(K * Np), y(K * Np), z(K * Np);
        const double scale = 0.2 + 2.0 * (U(rng) + 1.0);
        for (int i = 0; i < K * Np; ++i) { x[i] = scale * U(rng); y[i] = scale * U(rng); z[i] = scale * U(rng); }
        std::vector<int32_t> elems;
        for (int e = 0; e < K; ++e)
            if (rng() % 3) elems.push_back(e);
        if (elems.empty()) elems.push_back(0);
        dgtd::PlaneWaveDev w{};
        double k[3] = {G(rng), G(rng), G(rng)}, g[3] = {G(rng), G(rng), G(rng)};
        const double kn = std::sqrt(k[0] * k[0] + k[1] * k[1] + k[2] * k[2]);
        for (double& v : k) v /= kn;
        const double gk = g[0] * k[0] + g[1] * k[1] + g[2] * k[2];
        double p[3] = {g[0] - gk * k[0], g[1] - gk * k[1], g[2] - gk * k[2]};
        const double pn = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        for (int c = 0; c < 3; ++c) { w.k[c] = k[c]; w.pol[c] = p[c] / pn; }
        w.kxp[0] = w.k[1] * w.pol[2] - w.k[2] * w.pol[1];
        w.kxp[1] = w.k[2] * w.pol[0] - w.k[0] * w.pol[2];
        w.kxp[2] = w.k[0] * w.pol[1] - w.k[1] * w.pol[0];
        w.spread = 0.02 + 0.3 * (U(rng) + 1.0);
        w.mean = 3.0 * U(rng);
        w.freq = 0.0;
        const dgtd::TfsfSkipBound bound(x, y, z, elems, Np, w);
        for (int q = 0; q < 400; ++q) {
            const double t = 8.0 * U(rng);
            double sum = 0.0;
            for (int32_t e : elems)
                for (int i = 0; i < Np; ++i) {
                    const size_t n = static_cast<size_t>(e) * Np + i;
                    const double a = x[n] * w.k[0] + y[n] * w.k[1] + z[n] * w.k[2] - t - w.mean;
                    const double gg = std::exp(-a * a / (2.0 * w.spread * w.spread));
                    for (int c = 0; c < 3; ++c) {
                        const double pe = 0.5 * gg * w.pol[c], ph = 0.5 * gg * w.kxp[c];
                        sum += pe * pe + ph * ph;
                    }
                }
            const int d = bound.decide(t);
            if (d < 0) { ++undecided; continue; }
            ++decided;
            if (d != (sum < 1e-16 ? 1 : 0)) ++wrong;
        }
    }
    std::printf("decided %ld undecided %ld wrong %ld\n", decided, undecided, wrong);
    return wrong == 0 && decided > 0 ? 0 : 1;
}
