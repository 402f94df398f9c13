// TEST INFRASTRUCTURE ONLY: what the stand-in kernels (fake_kernels.cpp)
// produce for a whole request, computed on the host, and seeded test signals.
#pragma once
#include "../../include/occastft_gb300.h"

#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

namespace fake {

// Frame f reads samples [f*hop, f*hop + N), zeros past the signal; output
// float k of the frame's row takes sample k mod N (rows of N, 2N, N/2+1 or
// N+2 floats for power, half-complex, dense power, dense half-complex; the
// reference half-complex layout ends at 2*OHalfSize floats).  Floats no frame
// writes stay NaN.  Empty on a geometry error.
inline std::vector<float> expected_out(const float* x, uint64_t n, int exp, float ov, const std::string& opts)
{
    ocs_geometry g;
    if (ocs_geometry_get(n, exp, ov, opts.c_str(), &g) != OCS_OK) return {};
    const uint64_t N = 1ull << exp;
    const bool half = opts.find("--half_complex_return") != std::string::npos;
    const bool dense = opts.find("--layout=dense") != std::string::npos;
    const uint64_t row = dense ? (N / 2 + 1) * (half ? 2 : 1) : (half ? 2 * N : N);
    std::vector<float> out(g.out_floats, std::nanf(""));
    for (uint64_t f = 0; f < g.frames; ++f)
        for (uint64_t k = 0; k < row; ++k) {
            const uint64_t idx = f * row + k;
            if (idx >= g.out_floats) break;
            const uint64_t s = f * g.hop + k % N;
            out[idx] = s < n ? x[s] : 0.0f;
        }
    return out;
}

// seeded samples in [1, 2): never zero, so zero padding stays visible
inline std::vector<float> make_signal(uint64_t n, uint32_t seed)
{
    std::vector<float> x(n);
    uint32_t v = seed * 2654435761u + 1;
    for (auto& s : x) {
        v = v * 1664525u + 1013904223u;
        s = (float)(v >> 8) * (1.0f / 16777216.0f) + 1.0f;
    }
    return x;
}

}  // namespace fake
