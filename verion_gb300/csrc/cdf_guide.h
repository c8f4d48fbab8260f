// Guide tables of the inverse-CDF searches (the cutpoint method of Chen and Asau, 1974), host
// side: the environment map's marginal and conditional CDFs (pt_core.slang:274-306) and the
// emitter CDF (pt_core.slang:1343-1352, and the ReSTIR DI candidates at :759-882). Each search is
// the reference's: the first of n entries >= u, the last when none is. For K buckets (K a power of
// two, so u K is exact in float) entry k of a guide is that search's answer for u = k / K,
// k = 0..K; a non-decreasing CDF then has the answer for every u with floor(u K) = k between
// entries k and k + 1, and a search started on that range ends at the same entry.
//
// A CDF that is not non-decreasing (negative or NaN weights from the caller) gets the guide
// K, K - 1, ..., 0: every bucket's range is then empty-and-reversed (lo > hi), which the search
// reads as "search all n entries", the reference's own search.
//
// The device form of guided_search is guidedCdf (pt_device.cuh).
#pragma once
#include <stdint.h>

#include <algorithm>

namespace cdfg {

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

inline bool non_decreasing(const float* cdf, uint32_t n)
{
    for (uint32_t i = 0; i + 1 < n; i++)
        if (!(cdf[i] <= cdf[i + 1]))
            return false;
    return n == 0 || cdf[n - 1] == cdf[n - 1];
}

// K + 1 entries for one CDF of n entries.
inline void build_guide(const float* cdf, uint32_t n, uint32_t K, uint32_t* out)
{
    if (!non_decreasing(cdf, n)) {
        for (uint32_t k = 0; k <= K; k++)
            out[k] = K - k;
        return;
    }
    for (uint32_t k = 0; k <= K; k++)
        out[k] = cdf_search(cdf, n, (float)k / (float)K);
}

// The search started from the guide's range for u's bucket (u in [0, 1)).
inline uint32_t guided_search(const float* cdf, uint32_t n, const uint32_t* guide, uint32_t K, float u)
{
    uint32_t k = std::min((uint32_t)(u * (float)K), K - 1);
    uint32_t lo = guide[k], hi = guide[k + 1];
    if (lo > hi) {
        lo = 0;
        hi = n - 1;
    }
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (cdf[mid] >= u)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// Buckets of the emitter CDF's guide for n emitters: the power of two at or above 2 n, at least 2
// and at most 2^20 (one u32 per bucket).
inline uint32_t emitter_guide_buckets(uint32_t n)
{
    uint32_t k = 2;
    while (k < 2u * n && k < (1u << 20))
        k <<= 1;
    return k;
}

} // namespace cdfg
