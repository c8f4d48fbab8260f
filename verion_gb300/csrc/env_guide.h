// Guide tables of the environment map's CDF searches (the cutpoint method), host side. The CDF
// search is pt_core.slang:274-306's: the first of n entries >= u, the last when none is. For K
// buckets (K a power of two, so u K is exact in float) entry k of a guide is that search's answer
// for u = k / K, k = 0..K; the CDFs are non-decreasing, so every u with floor(u K) = k has its
// answer between entries k and k + 1, and a search started on that range ends at the same entry.
// The device form of guided_search is envSample (pt_device.cuh).
#pragma once
#include <stdint.h>

#include <algorithm>

namespace envg {

inline uint32_t cdf_search(const float* cdf, uint32_t n, float u)
{
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (cdf[mid] >= u)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// K + 1 entries for one CDF of n entries.
inline void build_guide(const float* cdf, uint32_t n, uint32_t K, uint32_t* out)
{
    for (uint32_t k = 0; k <= K; k++)
        out[k] = cdf_search(cdf, n, (float)k / (float)K);
}

// The search started from the guide's range for u's bucket (u in [0, 1)).
inline uint32_t guided_search(const float* cdf, const uint32_t* guide, uint32_t K, float u)
{
    uint32_t k = std::min((uint32_t)(u * (float)K), K - 1);
    uint32_t lo = guide[k], hi = guide[k + 1];
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (cdf[mid] >= u)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

} // namespace envg
