// Host-side bounds for the TF/SF skip test of one incidence driven by one unmodulated
// Gaussian plane wave.
//
// The reference skips the TF/SF source term of a stage while the sum over the TF/SF-submesh
// nodes of ||0.5 pw(x, t)||^2 is below 1e-16 (GlobalEvolution.cpp:587-598). For one plane
// wave with unit polarisation p and propagation k, node n contributes
// 0.25 g_n^2 (1 + |k x p|^2), between 0.25 g_n^2 and 0.5 g_n^2, where
// g_n = exp(-(x_n.k - t - mean)^2 / (2 spread^2)). The node nearest the pulse centre
// t + mean (in x.k) therefore bounds the sum from below by one term and from above by
// (node count) terms. `decide` returns 0 (source applied) or 1 (skipped) when the bound is
// a factor 10 clear of the threshold, and -1 when the exact device test must run.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

#include "kernels.hpp"

namespace dgtd {

class TfsfSkipBound {
public:
    TfsfSkipBound() = default;

    // x, y, z: node coordinates [K*Np]; elems: TF/SF-submesh elements.
    TfsfSkipBound(const std::vector<double>& x, const std::vector<double>& y, const std::vector<double>& z,
                  const std::vector<int32_t>& elems, int Np, const PlaneWaveDev& w)
        : mean_(w.mean), spread_(w.spread)
    {
        if (w.freq != 0.0 || elems.empty()) return;
        proj_.reserve(elems.size() * static_cast<size_t>(Np));
        for (int32_t e : elems)
            for (int i = 0; i < Np; ++i) {
                const size_t g = static_cast<size_t>(e) * Np + i;
                proj_.push_back(x[g] * w.k[0] + y[g] * w.k[1] + z[g] * w.k[2]);
            }
        std::sort(proj_.begin(), proj_.end());
    }

    bool usable() const { return !proj_.empty(); }

    int decide(double t) const
    {
        if (proj_.empty()) return -1;
        const double centre = t + mean_;
        auto it = std::lower_bound(proj_.begin(), proj_.end(), centre);
        double d = std::numeric_limits<double>::infinity();
        if (it != proj_.end()) d = std::min(d, *it - centre);
        if (it != proj_.begin()) d = std::min(d, centre - *(it - 1));
        const double g2 = std::exp(-d * d / (spread_ * spread_));
        const double lower = 0.25 * g2, upper = 0.5 * static_cast<double>(proj_.size()) * g2;
        if (lower > 1e-15) return 0;
        if (upper < 1e-17) return 1;
        return -1;
    }

private:
    std::vector<double> proj_;   // sorted x.k of the TF/SF-submesh nodes
    double mean_ = 0.0, spread_ = 1.0;
};

}  // namespace dgtd
