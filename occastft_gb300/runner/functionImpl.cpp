// runnerFunction hooks of the GB300 runner (the reference's CUDA versions are
// StandAlone/cross_gpgpu/CUDA/src/functionImpl.cpp:15-683).  Data arguments
// point at device pointers (float**), userStruct at a GB300Data.  Each hook
// launches one unfused stage kernel through the C ABI on the GB300Data stream
// and returns false on a failed launch, as the reference's hooks do.
//
// EXPC writes the finished spectrum back into real/imag for every exponent,
// so a caller that keeps reading `real` after it (Default_Pipeline does) gets
// the full transform also for odd exponents >= 13.
#include "gb300Struct.hpp"
#include "occastft_gb300.h"
#include "occastft_runner.hpp"

namespace {
void* stream_of(void* userStruct) { return userStruct ? static_cast<GB300Data*>(userStruct)->stream : nullptr; }
float* dptr(void* p) { return *static_cast<float**>(p); }
bool window(void* userStruct, int kind, void* data, CUI OFullSize, CUI windowSize, float sigma)
{
    return ocs_stage_window(kind, dptr(data), OFullSize, windowSize, sigma, stream_of(userStruct)) == OCS_OK;
}
bool fft(void* userStruct, void* Real, void* Imag, CUI OHalfSize, unsigned exp)
{
    return ocs_stage_fft(dptr(Real), dptr(Imag), OHalfSize, exp, stream_of(userStruct)) == OCS_OK;
}
}  // namespace

bool runnerFunction::Overlap(void* userStruct, void* origin, CUI OFullSize, CUI FullSize, CUI windowSizeEXP,
                             CUI OMove, void* Realout)
{
    return ocs_stage_overlap(dptr(origin), OFullSize, FullSize, windowSizeEXP, OMove, dptr(Realout),
                             stream_of(userStruct)) == OCS_OK;
}

bool runnerFunction::Hanning(void* u, void* d, CUI o, CUI w) { return window(u, 1, d, o, w, -1.0f); }
bool runnerFunction::Hamming(void* u, void* d, CUI o, CUI w) { return window(u, 2, d, o, w, -1.0f); }
bool runnerFunction::Blackman(void* u, void* d, CUI o, CUI w) { return window(u, 3, d, o, w, -1.0f); }
bool runnerFunction::Nuttall(void* u, void* d, CUI o, CUI w) { return window(u, 4, d, o, w, -1.0f); }
bool runnerFunction::Blackman_Nuttall(void* u, void* d, CUI o, CUI w) { return window(u, 5, d, o, w, -1.0f); }
bool runnerFunction::Blackman_Harris(void* u, void* d, CUI o, CUI w) { return window(u, 6, d, o, w, -1.0f); }
bool runnerFunction::FlatTop(void* u, void* d, CUI o, CUI w) { return window(u, 7, d, o, w, -1.0f); }
bool runnerFunction::Gaussian(void* u, void* d, CUI o, CUI w, const float sigma) { return window(u, 8, d, o, w, sigma); }

bool runnerFunction::RemoveDC(void* userStruct, void* data, CUI qtConst, CUI OFullSize, CUI windowSize)
{
    return ocs_stage_remove_dc(dptr(data), qtConst, OFullSize, windowSize, stream_of(userStruct)) == OCS_OK;
}

bool runnerFunction::EXP6(void* u, void* r, void* i, CUI h) { return fft(u, r, i, h, 6); }
bool runnerFunction::EXP7(void* u, void* r, void* i, CUI h) { return fft(u, r, i, h, 7); }
bool runnerFunction::EXP8(void* u, void* r, void* i, CUI h) { return fft(u, r, i, h, 8); }
bool runnerFunction::EXP9(void* u, void* r, void* i, CUI h) { return fft(u, r, i, h, 9); }
bool runnerFunction::EXP10(void* u, void* r, void* i, CUI h) { return fft(u, r, i, h, 10); }
bool runnerFunction::EXP11(void* u, void* r, void* i, CUI h) { return fft(u, r, i, h, 11); }

bool runnerFunction::EXPC(void* userStruct, void* real, void* imag, void* subreal, void* subimag, void* out,
                          CUI HWindowSize, CUI windowSizeEXP, CUI OFullSize, void* realResult, void* imagResult)
{
    (void)subreal;
    (void)subimag;
    (void)out;
    (void)HWindowSize;
    (void)realResult;
    (void)imagResult;
    return fft(userStruct, real, imag, OFullSize / 2, windowSizeEXP);
}

bool runnerFunction::HalfComplex(void* userStruct, void* out, void* realResult, void* imagResult, CUI OHalfSize,
                                 CUI windowSizeEXP)
{
    return ocs_stage_half_complex(dptr(out), dptr(realResult), dptr(imagResult), OHalfSize, windowSizeEXP,
                                  stream_of(userStruct)) == OCS_OK;
}

bool runnerFunction::ToPower(void* userStruct, void* out, void* realResult, void* imagResult, CUI OFullSize)
{
    return ocs_stage_to_power(dptr(out), dptr(realResult), dptr(imagResult), OFullSize, stream_of(userStruct)) ==
           OCS_OK;
}
