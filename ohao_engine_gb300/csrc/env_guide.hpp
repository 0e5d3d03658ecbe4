// Guide tables for the environment map's inverse-CDF sampling (the cutpoint
// method of Chen and Asau, 1974).
//
// The sampler inverts a marginal CDF over rows and a conditional CDF per row
// with a binary search over the whole row (env_sampling.glsl:15-37 of the
// reference): for u it returns the first index i in [0, n-2] with
// cdf[i] >= u, else n - 1. For a non-decreasing CDF that index is a
// non-decreasing function a(u) of u. A guide table of m + 1 entries (m a power
// of two, so u * m is exact in float) stores g[j] = a(j / m) and g[m] = n - 1;
// for j = floor(u * m), a(u) lies in [g[j], g[j + 1]], and the same search
// run between those two bounds returns the same index in about one or two
// steps instead of log2(n) dependent loads. Only non-decreasing rows (no NaN)
// get a guide; the caller keeps the full search for any other CDF.
#pragma once

#include <cmath>
#include <cstdint>

#ifdef __CUDACC__
#define OHAO_EG_HD __host__ __device__ __forceinline__
#else
#define OHAO_EG_HD inline
#endif

namespace ohao_env_guide {

constexpr uint32_t kMaxEntries = 65536;   // indices must fit the uint16 entries

// Guide cells for a row of n entries: the smallest power of two >= n.
inline uint32_t cells_for(uint32_t n) {
    uint32_t m = 1;
    while (m < n) m <<= 1;
    return m;
}

// True if cdf[0..n) is non-decreasing and holds no NaN.
inline bool monotone(const float* cdf, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i)
        if (cdf[i] != cdf[i]) return false;
    for (uint32_t i = 0; i + 1 < n; ++i)
        if (!(cdf[i] <= cdf[i + 1])) return false;
    return true;
}

// g[j] = a(j / m) for j < m, g[m] = n - 1 (n in [1, kMaxEntries]; cdf
// non-decreasing): one merge pass over the row.
inline void build(const float* cdf, uint32_t n, uint32_t m, uint16_t* g) {
    uint32_t i = 0;
    for (uint32_t j = 0; j < m; ++j) {
        const float u = static_cast<float>(j) / static_cast<float>(m);
        while (i + 1 < n && cdf[i] < u) ++i;
        g[j] = static_cast<uint16_t>(i);
    }
    g[m] = static_cast<uint16_t>(n - 1);
}

// a(u) for u in [0, 1], searched between the guide's bounds; cdf_at(i) and
// guide_at(j) load the row's entries.
template <class CdfAt, class GuideAt>
OHAO_EG_HD int search(CdfAt cdf_at, GuideAt guide_at, uint32_t m, float u) {
    uint32_t j = u > 0.0f ? static_cast<uint32_t>(fminf(u, 1.0f) * static_cast<float>(m)) : 0u;
    j = j < m ? j : m - 1;
    int lo = guide_at(j), hi = guide_at(j + 1);
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (cdf_at(mid) < u) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

}  // namespace ohao_env_guide
