// Host-side request parsing shared by the C ABI and the C++ runner: option
// grammar, frame geometry and window tables, each as the reference defines them.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace ocs {

enum WindowKind : int {
    WIN_NONE = 0,
    WIN_HANNING = 1,
    WIN_HAMMING = 2,
    WIN_BLACKMAN = 3,
    WIN_NUTTALL = 4,
    WIN_BLACKMAN_NUTTALL = 5,
    WIN_BLACKMAN_HARRIS = 6,
    WIN_FLATTOP = 7,
    WIN_GAUSSIAN = 8
};

struct Options {
    int window = WIN_NONE;
    float sigma = -1.0f;
    bool remove_dc = false;
    bool half_complex = false;
    bool dense = false;
    bool serial_power = false;
    // 0 plain FP32; tensor cores with split operands: 1 fp16 hi/lo
    // (--precision=tc-fp16), 2 bf16 hi/lo (tc-bf16x2), 3 bf16 hi/mid/lo (tc-bf16x3)
    int precision = 0;
};

struct Geometry {
    uint32_t qt = 0, hop = 0, ofull = 0, ohalf = 0, n_window = 0;
    uint64_t out_floats = 0;
    uint64_t frames = 0;
};

// Parses the option string as runnerFunction::Default_Pipeline does
// (RunnerCommon.cpp:216-248).  Returns "OK" or the reference's status string.
std::string parse_options(const char* options, Options& o);

// Frame geometry (RunnerInterface.hpp:26-35, CudaImpl.cpp:416-421).  Returns
// "OK" or a status message; exp < 6 gives the reference's
// "Operation not supported" (RunnerCommon.cpp:250-253).
std::string make_geometry(uint64_t n, int exp, float overlap, const Options& o, Geometry& g);

// Window coefficients exactly as the reference's serial kernels compute them
// (OKL/kernel.okl:33-127): angle in double stored to float, single-precision
// cosine, double combine rounded to float.  Empty for WIN_NONE.
std::vector<float> window_table(int kind, int n_window, float sigma);

// Sets the message ocs_last_error() returns on this thread.
void set_last_error(const std::string& msg);

}  // namespace ocs
