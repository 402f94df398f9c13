// occastft_gb300 — the reference's runner contract for the GB300 runner.
//
// These declarations have to match OCCAstft's vendor contract so that the
// GB300 runner drops into StandAlone/cross_gpgpu in place of the CUDA runner:
// the same type aliases, toQuot, the runnerFunction hook signatures and the
// Runner members (StandAlone/cross_gpgpu/GLOBAL/RunnerInterface.hpp:13-131).
// What differs: no IXWebSocket / FFTStruct includes (the server lives in the
// reference's GLOBAL/RunnerCommon.cpp, which a maintainer links instead of
// occastft_gb300/runner/RunnerStandalone.cpp), and Runner keeps the status of
// its last pipeline run in `last_status`.
#pragma once
#include <optional>
#include <string>
#include <vector>

using VECF = std::vector<float>;
using MAYBE_DATA = std::optional<VECF>;
using BIN = std::string;
using CUI = const unsigned int;
using UI = unsigned int;
struct Genv;
struct Gcodes;

struct cplx_t {
    float real;
    float imag;
};

// frame count in float arithmetic, truncated (RunnerInterface.hpp:26-35)
inline int toQuot(float fullSize, float overlapRatio, float windowSize)
{
    if (overlapRatio == 0.0f) {
        return fullSize / windowSize + 1;
    }
    return ((fullSize) / (windowSize * (1.0f - overlapRatio))) + 1;
}

// Per-stage hooks.  The void* data arguments point at device pointers
// (float**), as the reference's CUDA runner passes CUdeviceptr*; userStruct
// points at a GB300Data (occastft_gb300/runner/gb300Struct.hpp).
namespace runnerFunction {

bool Overlap(void* userStruct, void* origin, CUI OFullSize, CUI FullSize, CUI windowSizeEXP, CUI OMove, void* Realout);
bool Hanning(void* userStruct, void* data, CUI OFullSize, CUI windowSize);
bool Hamming(void* userStruct, void* data, CUI OFullSize, CUI windowSize);
bool Blackman(void* userStruct, void* data, CUI OFullSize, CUI windowSize);
bool Nuttall(void* userStruct, void* data, CUI OFullSize, CUI windowSize);
bool Blackman_Nuttall(void* userStruct, void* data, CUI OFullSize, CUI windowSize);
bool Blackman_Harris(void* userStruct, void* data, CUI OFullSize, CUI windowSize);
bool FlatTop(void* userStruct, void* data, CUI OFullSize, CUI windowSize);
bool Gaussian(void* userStruct, void* data, CUI OFullSize, CUI windowSize, const float sigma);

bool RemoveDC(void* userStruct, void* data, CUI qtConst, CUI OFullSize, CUI windowSize);

bool EXP6(void* userStruct, void* Real, void* Imag, CUI OHalfSize);
bool EXP7(void* userStruct, void* Real, void* Imag, CUI OHalfSize);
bool EXP8(void* userStruct, void* Real, void* Imag, CUI OHalfSize);
bool EXP9(void* userStruct, void* Real, void* Imag, CUI OHalfSize);
bool EXP10(void* userStruct, void* Real, void* Imag, CUI OHalfSize);
bool EXP11(void* userStruct, void* Real, void* Imag, CUI OHalfSize);

bool EXPC(void* userStruct, void* real, void* imag, void* subreal, void* subimag, void* out, CUI HWindowSize,
          CUI windowSizeEXP, CUI OFullSize, void* realResult, void* imagResult);

bool HalfComplex(void* userStruct, void* out, void* realResult, void* imagResult, CUI OHalfSize, CUI windowSizeEXP);

bool ToPower(void* userStruct, void* out, void* realResult, void* imagResult, CUI OFullSize);

std::string Default_Pipeline(void* userStruct, void* origin, void* real, void* imag, void* subreal, void* subimag,
                             void* out, CUI FullSize, CUI windowSize, CUI qtConst, CUI OFullSize, CUI OHalfSize,
                             CUI OMove, const std::string& options, const int windowSizeEXP,
                             const float overlapRatio);

};  // namespace runnerFunction

struct Runner {
private:
    void InitEnv();
    void BuildKernel();
    void UnInit();
    Genv* env = nullptr;
    Gcodes* kens = nullptr;

public:
    [[nodiscard]] MAYBE_DATA ActivateSTFT(VECF& inData, const int& windowSizeEXP, const float& overlapRatio,
                                          const std::string& options);
    std::string last_status = "OK";
    Runner(const int& portNumber);
    ~Runner();
};
