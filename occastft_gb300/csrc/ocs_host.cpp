// Host-side request parsing: option grammar, geometry, window tables.
// Compiled with -ffp-contract=off: the window formulas must round exactly as
// the reference's serial build does (no fused multiply-add).
#include "ocs_host.h"

#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <thread>

namespace ocs {

static const double kPi = 3.14159265358979323846;  // M_PI

std::string parse_options(const char* options, Options& o)
{
    o = Options{};
    const std::string s = options ? options : "";
    static const char* kWin[] = {"--hanning_window",          "--hamming_window",         "--blackman_window",
                                 "--nuttall_window",          "--blackman_nuttall_window", "--blackman_harris_window",
                                 "--flattop_window"};
    for (int i = 0; i < 7; ++i) {
        if (s.find(kWin[i]) != std::string::npos) {
            o.window = i + 1;
            break;
        }
    }
    if (o.window == WIN_NONE) {
        const size_t gpos = s.find("--gaussian_window=");
        const size_t spos = s.find("<<sigma");
        if (gpos != std::string::npos && spos != std::string::npos) {
            // sigma text starts 19 characters after an 18-character prefix:
            // the reference skips the first sigma character (RunnerCommon.cpp:228)
            const size_t p1 = gpos + 19;
            if (p1 > s.size()) return "--gaussian_window";
            const size_t cnt = spos >= p1 ? spos - p1 : std::string::npos;
            const std::string sig = s.substr(p1, cnt);
            // std::stof semantics: no conversion or ERANGE -> failure
            const char* b = sig.c_str();
            char* e = nullptr;
            errno = 0;
            const float v = std::strtof(b, &e);
            if (e == b || errno == ERANGE) return "--gaussian_window";
            if (v > 0) {
                o.window = WIN_GAUSSIAN;
                o.sigma = v;
            }
        }
    }
    o.remove_dc = s.find("--remove_dc") != std::string::npos;
    o.half_complex = s.find("--half_complex_return") != std::string::npos;
    o.dense = s.find("--layout=dense") != std::string::npos;
    o.serial_power = s.find("--serial_power") != std::string::npos;
    if (s.find("--precision=tc-fp16") != std::string::npos) o.precision = 1;
    if (s.find("--precision=tc-bf16x2") != std::string::npos) o.precision = 2;
    if (s.find("--precision=tc-bf16x3") != std::string::npos) o.precision = 3;
    return "OK";
}

std::string make_geometry(uint64_t n, int exp, float overlap, const Options& o, Geometry& g)
{
    if (exp < 6) return "Operation not supported";
    // the reference's window size is an int: 2^31 overflows it, and at 2^30
    // OFullSize = qt * N < 2^32 already allows at most three frames
    if (exp > 30) return "Operation not supported: window sizes above 2^30";
    if (n == 0) return "empty input signal";
    if (n > 0xffffffffull) return "signal longer than 2^32-1 samples";
    if (!(overlap < 1.0f) || std::isnan(overlap)) return "overlap ratio must be below 1";
    const uint32_t win = 1u << exp;
    const float hopf = (float)win * (1.0f - overlap);  // CudaImpl.cpp:421
    if (!(hopf >= 1.0f) || hopf >= 4294967296.0f) return "frame advance (OMove) below one sample";
    const float full = (float)(uint32_t)n;
    float qf;
    if (overlap == 0.0f) {
        qf = full / (float)win + 1.0f;
    } else {
        qf = full / ((float)win * (1.0f - overlap)) + 1.0f;
    }
    if (!(qf < 2147483648.0f)) return "frame count overflows";
    const int qt = (int)qf;
    const uint64_t ofull = (uint64_t)(uint32_t)qt * (uint64_t)win;
    if (qt <= 0 || ofull >= 4294967296ull) return "OFullSize overflows 32 bits";
    g.qt = (uint32_t)qt;
    g.hop = (uint32_t)hopf;
    g.ofull = (uint32_t)ofull;
    g.ohalf = (uint32_t)(ofull / 2);
    g.n_window = (uint32_t)win;
    if (o.dense) {
        g.out_floats = (uint64_t)g.qt * (win / 2 + 1) * (o.half_complex ? 2u : 1u);
        g.frames = g.qt;
    } else {
        g.out_floats = g.ofull;
        // compat half-complex is a flat copy of the first OHalfSize bins:
        // only the first ceil(qt/2) frames contribute
        g.frames = o.half_complex ? ((uint64_t)g.ohalf + win - 1) / win : g.qt;
    }
    return "OK";
}

std::vector<float> window_table(int kind, int nwin, float sigma)
{
    std::vector<float> w;
    if (kind == WIN_NONE) return w;
    w.resize(nwin);
    // every entry is the same float/double expression, so tables of windows
    // of millions of samples fill in parallel without changing a bit
    auto fill = [&](int i0, int i1) {
    for (int i = i0; i < i1; ++i) {
        float v = 1.0f;
        switch (kind) {
        case WIN_HANNING: {
            const float a = (float)(2.0 * kPi * i / (double)(float)(nwin - 1));
            v = (float)(0.5 * (1.0 - (double)cosf(a)));
            break;
        }
        case WIN_HAMMING: {
            const float a = (float)(2.0 * kPi * i / (double)(float)(nwin - 1));
            v = (float)(0.54 - (0.46 * (double)cosf(a)));
            break;
        }
        case WIN_BLACKMAN: {
            const float f = (float)(2.0 * kPi * i / (double)(float)nwin);
            const float s = (float)((double)f * 2.0);
            v = (float)(0.42 - 0.5 * (double)cosf(f) + 0.08 * (double)cosf(s));
            break;
        }
        case WIN_NUTTALL: {
            const float f = (float)(2.0 * kPi * i / (double)(float)nwin);
            const float s = (float)((double)f * 2.0), t = (float)((double)f * 3.0);
            v = (float)(0.355768 - 0.487396 * (double)cosf(f) + 0.144232 * (double)cosf(s) -
                        0.012604 * (double)cosf(t));
            break;
        }
        case WIN_BLACKMAN_NUTTALL: {
            const float f = (float)(2.0 * kPi * i / (double)(float)nwin);
            const float s = (float)((double)f * 2.0), t = (float)((double)f * 3.0);
            v = (float)(0.3635819 - 0.4891775 * (double)cosf(f) + 0.1365995 * (double)cosf(s) -
                        0.0106411 * (double)cosf(t));
            break;
        }
        case WIN_BLACKMAN_HARRIS: {
            const float f = (float)(2.0 * kPi * i / (double)(float)nwin);
            const float s = (float)((double)f * 2.0), t = (float)((double)f * 3.0);
            v = (float)(0.35875 - 0.48829 * (double)cosf(f) + 0.14128 * (double)cosf(s) -
                        0.01168 * (double)cosf(t));
            break;
        }
        case WIN_FLATTOP: {
            const float f = (float)(2.0 * kPi * i / (double)(float)nwin);
            const float s = (float)((double)f * 2.0), t = (float)((double)f * 3.0);
            const float u = (float)((double)f * 4.0);
            v = (float)(0.21557895 - 0.41663158 * (double)cosf(f) + 0.277263158 * (double)cosf(s) -
                        0.083578947 * (double)cosf(t) + 0.006947368 * (double)cosf(u));
            break;
        }
        case WIN_GAUSSIAN: {
            const int h = nwin >> 1;
            float a = (float)(i - h) / ((float)h * sigma);
            a = a * a;
            a = (float)((double)a * -0.5);
            v = expf(a);
            break;
        }
        default:
            break;
        }
        w[i] = v;
    }
    };
    const unsigned hw = std::thread::hardware_concurrency();
    const int parts = (nwin >= (1 << 20) && hw > 1) ? (int)(hw < 64 ? hw : 64) : 1;
    if (parts == 1) {
        fill(0, nwin);
    } else {
        std::vector<std::thread> th;
        const int per = (nwin + parts - 1) / parts;
        for (int p = 0; p < parts; ++p) {
            const int i0 = p * per, i1 = i0 + per < nwin ? i0 + per : nwin;
            if (i0 < i1) th.emplace_back(fill, i0, i1);
        }
        for (auto& t : th) t.join();
    }
    return w;
}

}  // namespace ocs
