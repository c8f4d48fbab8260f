"""Guide tables of the inverse-CDF searches (verion_gb300/csrc/cdf_guide.h): the search started
from a guide's range finds the entry the full search finds (pt_core.slang:274-306, 1343-1352) for
environment-sized guides (256 and 1024 buckets) and emitter-sized ones (the power of two at or
above twice the entry count), for non-decreasing CDFs with flat runs, spikes, all-zero rows and a
last entry below 1, for CDFs that decrease or hold NaN (negative or broken weights: the guide then
falls back to the full search), and for u at the bucket edges, just below them, on the CDF's own
values and at random. Compiled with g++ from the header the library uses."""
import shutil
import subprocess
from pathlib import Path

import pytest

CSRC = Path(__file__).resolve().parent.parent / "verion_gb300" / "csrc"

HARNESS = r"""
#include "cdf_guide.h"
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

int main()
{
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> uni(0.0f, 1.0f);
    const uint32_t sizes[] = {1, 2, 3, 17, 64, 1024, 2048, 4096};
    long checked = 0, fallbacks = 0;
    for (int trial = 0; trial < 560; trial++) {
        uint32_t n = sizes[rng() % 8];
        std::vector<float> w(n);
        int kind = trial % 7;
        for (uint32_t i = 0; i < n; i++) {
            float x = uni(rng);
            if (kind == 0)
                w[i] = x;                                  // smooth
            else if (kind == 1)
                w[i] = (rng() % 50 == 0) ? 1.0e4f * x : 1.0e-3f * x; // a few spikes (a sun)
            else if (kind == 2)
                w[i] = ((i / 7) % 2) ? x : 0.0f;             // flat runs
            else if (kind == 3)
                w[i] = 0.0f;                                 // an all-zero row
            else if (kind == 4)
                w[i] = x * x * x * x;                        // strongly skewed
            else if (kind == 5)
                w[i] = x - 0.3f;                             // negative weights: the CDF decreases
            else
                w[i] = (i == n / 2) ? NAN : x;               // a broken weight
        }
        std::vector<float> cdf(n);
        double total = 0.0;
        for (float x : w)
            total += x;
        float run = 0.0f;
        for (uint32_t i = 0; i < n; i++) {
            run += w[i];
            cdf[i] = total > 0.0 ? (float)(run / total) : 0.0f;
            if (kind < 5 && i > 0 && cdf[i] < cdf[i - 1])
                cdf[i] = cdf[i - 1]; // keep it non-decreasing, as the packer's is
        }
        if (trial % 3 == 0 && n > 0 && total > 0.0)
            cdf[n - 1] = std::nextafter(1.0f, 0.0f); // last entry just below 1
        const uint32_t buckets[] = {256, 1024, cdfg::emitter_guide_buckets(n)};
        for (uint32_t K : buckets) {
            std::vector<uint32_t> g(K + 1);
            cdfg::build_guide(cdf.data(), n, K, g.data());
            if (!cdfg::non_decreasing(cdf.data(), n))
                fallbacks++;
            std::vector<float> us;
            for (uint32_t k = 0; k < K; k++) {
                float e = (float)k / (float)K;
                us.push_back(e);
                if (k > 0)
                    us.push_back(std::nextafter(e, 0.0f));
            }
            for (float c : cdf)
                if (c < 1.0f) {
                    us.push_back(c);
                    us.push_back(std::nextafter(c, 0.0f));
                    us.push_back(std::nextafter(c, 1.0f));
                }
            for (int r = 0; r < 2000; r++)
                us.push_back(uni(rng));
            us.push_back(0.0f);
            us.push_back(1.0e-30f);
            us.push_back(std::nextafter(1.0f, 0.0f));
            for (float u : us) {
                if (!(u >= 0.0f && u < 1.0f))
                    continue;
                uint32_t a = cdfg::cdf_search(cdf.data(), n, u);
                uint32_t b = cdfg::guided_search(cdf.data(), n, g.data(), K, u);
                if (a != b) {
                    std::printf("mismatch n=%u K=%u u=%.9g full=%u guided=%u\n", n, K, u, a, b);
                    return 1;
                }
                checked++;
            }
        }
    }
    if (fallbacks == 0) {
        std::printf("no CDF took the full-search fallback\n");
        return 1;
    }
    std::printf("ok %ld\n", checked);
    return 0;
}
"""


def test_guided_search_finds_the_full_searchs_entry(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "guide.cpp"
    src.write_text(HARNESS)
    exe = tmp_path / "guide"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(CSRC), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("ok"), out.stdout
