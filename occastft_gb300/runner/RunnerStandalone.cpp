// Common runner code for using the GB300 runner outside the reference tree:
// Runner construction / destruction and runnerFunction::Default_Pipeline.
// Inside StandAlone/cross_gpgpu the reference's GLOBAL/RunnerCommon.cpp
// provides these (with its WebSocket server); this file restates the
// pipeline's stage order and option handling (RunnerCommon.cpp:166-316) so the
// hooks can be driven stage by stage here too.
#include "gb300Struct.hpp"
#include "occastft_runner.hpp"

Runner::Runner(const int& portNumber)
{
    (void)portNumber;  // no server in the standalone build
    InitEnv();
    BuildKernel();
}

Runner::~Runner()
{
    UnInit();
    delete env;
    delete kens;
}

namespace {
bool has(const std::string& s, const char* opt) { return s.find(opt) != std::string::npos; }
}  // namespace

std::string runnerFunction::Default_Pipeline(void* userStruct, void* origin, void* real, void* imag, void* subreal,
                                             void* subimag, void* out, CUI FullSize, CUI windowSize, CUI qtConst,
                                             CUI OFullSize, CUI OHalfSize, CUI OMove, const std::string& options,
                                             const int windowSizeEXP, const float overlapRatio)
{
    (void)overlapRatio;
    Overlap(userStruct, origin, OFullSize, FullSize, windowSizeEXP, OMove, real);
    struct W {
        const char* opt;
        bool (*fn)(void*, void*, CUI, CUI);
    } const wins[] = {{"--hanning_window", Hanning},          {"--hamming_window", Hamming},
                      {"--blackman_window", Blackman},        {"--nuttall_window", Nuttall},
                      {"--blackman_nuttall_window", Blackman_Nuttall},
                      {"--blackman_harris_window", Blackman_Harris}, {"--flattop_window", FlatTop}};
    bool windowed = false;
    for (const W& w : wins) {
        if (has(options, w.opt)) {
            if (!w.fn(userStruct, real, OFullSize, windowSize)) return w.opt;
            windowed = true;
            break;
        }
    }
    if (!windowed && has(options, "--gaussian_window=") && has(options, "<<sigma")) {
        const size_t p1 = options.find("--gaussian_window=") + 19;  // skips the first sigma character
        const size_t p2 = options.find("<<sigma");
        float sigma = -1.0f;
        if (p1 > options.size()) return "--gaussian_window";
        try {
            sigma = std::stof(options.substr(p1, p2 - p1));
        } catch (const std::exception&) {
            return "--gaussian_window";
        }
        if (sigma > 0 && !Gaussian(userStruct, real, OFullSize, windowSize, sigma)) return "--gaussian_window";
    }
    if (has(options, "--remove_dc") && !RemoveDC(userStruct, real, qtConst, OFullSize, windowSize))
        return "--remove_dc";
    if (windowSizeEXP < 6) return "Operation not supported";
    bool ok;
    switch (windowSizeEXP) {
    case 6: ok = EXP6(userStruct, real, imag, OHalfSize); break;
    case 7: ok = EXP7(userStruct, real, imag, OHalfSize); break;
    case 8: ok = EXP8(userStruct, real, imag, OHalfSize); break;
    case 9: ok = EXP9(userStruct, real, imag, OHalfSize); break;
    case 10: ok = EXP10(userStruct, real, imag, OHalfSize); break;
    case 11: ok = EXP11(userStruct, real, imag, OHalfSize); break;
    default:
        ok = EXPC(userStruct, real, imag, subreal, subimag, out, windowSize >> 1, windowSizeEXP, OFullSize, real, imag);
    }
    if (!ok) return "Err On Stockham";
    if (has(options, "--half_complex_return")) {
        if (!HalfComplex(userStruct, out, real, imag, OHalfSize, windowSizeEXP)) return "--half_complex_return";
    } else {
        ToPower(userStruct, out, real, imag, OFullSize);
    }
    return "OK";
}
