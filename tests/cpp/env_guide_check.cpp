// Checks the environment map's guided inverse-CDF search
// (ohao_engine_gb300/csrc/env_guide.hpp) against the whole-row binary search
// of the reference's sampler on CDF rows built to be awkward: flat runs
// (zero-weight texels), a single spike, the last entry reached early, rows of
// 1-3 entries and rows that are not a power of two long; at every guide
// boundary j / m, its float neighbours, every CDF value and its neighbours,
// and seeded uniform draws. Prints "ok" and exits 0 when every search agrees.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <random>
#include <vector>

#include "env_guide.hpp"

namespace eg = ohao_env_guide;

static int full_search(const std::vector<float>& cdf, float u) {
    int lo = 0, hi = static_cast<int>(cdf.size()) - 1;
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (cdf[mid] < u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Normalised running sum of the weights, as ohao_env_cdf_build forms a row.
static std::vector<float> cdf_of(const std::vector<float>& wgt) {
    std::vector<float> c(wgt.size());
    float total = 0.0f;
    for (size_t i = 0; i < wgt.size(); ++i) { total += wgt[i]; c[i] = total; }
    for (float& x : c) x = total > 0.0f ? x / total : 0.0f;
    return c;
}

int main() {
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    std::vector<std::vector<float>> rows;
    for (uint32_t n : {1u, 2u, 3u, 7u, 64u, 512u, 1000u, 1024u, 1025u}) {
        std::vector<float> w(n);
        for (auto& x : w) x = U(rng);
        rows.push_back(cdf_of(w));                                   // dense
        for (auto& x : w) x = U(rng) < 0.7f ? 0.0f : U(rng);
        rows.push_back(cdf_of(w));                                   // flat runs
        std::fill(w.begin(), w.end(), 0.0f);
        w[n / 2] = 1.0f;
        rows.push_back(cdf_of(w));                                   // one spike
        for (uint32_t i = 0; i < n; ++i) w[i] = i < n / 3 ? 1.0f : 0.0f;
        rows.push_back(cdf_of(w));                                   // reaches 1 early
        for (uint32_t i = 0; i < n; ++i) w[i] = std::exp(40.0f * (U(rng) - 1.0f));
        rows.push_back(cdf_of(w));                                   // heavy dynamic range
        std::fill(w.begin(), w.end(), 0.0f);
        rows.push_back(cdf_of(w));                                   // all zero
    }
    long checked = 0, bad = 0;
    for (const auto& cdf : rows) {
        const uint32_t n = static_cast<uint32_t>(cdf.size());
        if (!eg::monotone(cdf.data(), n)) { std::printf("row of %u not monotone\n", n); return 1; }
        const uint32_t m = eg::cells_for(n);
        std::vector<uint16_t> g(m + 1);
        eg::build(cdf.data(), n, m, g.data());
        std::vector<float> us = {0.0f, 1.0f, std::nextafter(1.0f, 0.0f), std::nextafter(0.0f, 1.0f)};
        for (uint32_t j = 0; j <= m; ++j) {
            const float b = static_cast<float>(j) / static_cast<float>(m);
            us.push_back(b);
            us.push_back(std::nextafter(b, 0.0f));
            us.push_back(std::nextafter(b, 2.0f));
        }
        for (float c : cdf) {
            us.push_back(c);
            us.push_back(std::nextafter(c, 0.0f));
            us.push_back(std::nextafter(c, 2.0f));
        }
        for (int k = 0; k < 2000; ++k) us.push_back(U(rng));
        for (float u : us) {
            if (u < 0.0f || u > 1.0f) continue;
            const int want = full_search(cdf, u);
            const int got = eg::search([&](int i) { return cdf[static_cast<size_t>(i)]; },
                                       [&](uint32_t j) { return static_cast<int>(g[j]); }, m, u);
            ++checked;
            if (got != want) {
                if (++bad < 10) std::printf("n %u u %.9g: guided %d, full %d\n", n, static_cast<double>(u), got, want);
            }
        }
    }
    const float dec[4] = {0.1f, 0.5f, 0.4f, 1.0f};
    const float nan[3] = {0.1f, NAN, 1.0f};
    if (eg::monotone(dec, 4) || eg::monotone(nan, 3)) { std::printf("non-monotone row accepted\n"); return 1; }
    std::printf("%ld searches, %ld differ\n", checked, bad);
    if (bad) return 1;
    std::printf("ok\n");
    return 0;
}
