// TEST INFRASTRUCTURE ONLY — C entry points over the reference's own Serial /
// OpenMP runner code, compiled from the reference's sources by
// oracle/build_ref.sh into oracle/_ref/.  Used only by tests and by the CPU
// timing legs; never shipped.
//
// ref_activate mirrors the sizing and buffer set-up of the Serial runner's
// ActivateSTFT (StandAlone/cross_gpgpu/Serial/src/SerialImpl.cpp:30-75) and
// then calls the reference's own runnerFunction::Default_Pipeline
// (StandAlone/cross_gpgpu/GLOBAL/RunnerCommon.cpp:184-316).
#include "RunnerInterface.hpp"

#include <cstring>

extern "C" void Overlap_Common(float*, CUI&, CUI&, CUI&, CUI&, float*);
extern "C" void Window_Hanning(float*, CUI&, CUI&);
extern "C" void Window_Hamming(float*, CUI&, CUI&);
extern "C" void Window_Blackman(float*, CUI&, CUI&);
extern "C" void Window_Nuttall(float*, CUI&, CUI&);
extern "C" void Window_Blackman_Nuttall(float*, CUI&, CUI&);
extern "C" void Window_Blackman_harris(float*, CUI&, CUI&);
extern "C" void Window_FlatTop(float*, CUI&, CUI&);
extern "C" void Window_Gaussian(float*, CUI&, CUI&, const float&);
extern "C" void DCRemove_Common(float*, CUI&, CUI&);

extern "C" {

int ref_geometry(unsigned int n, int exp, float ov, unsigned int* qt, unsigned int* hop,
                 unsigned int* ofull, unsigned int* ohalf)
{
    const int windowSize = 1 << exp;
    const int qtConst = toQuot(n, ov, windowSize);
    *qt = (unsigned)qtConst;
    *ofull = (unsigned)qtConst * (unsigned)windowSize;
    *ohalf = *ofull / 2;
    *hop = windowSize * (1.0f - ov);
    return 0;
}

// Runs the reference pipeline; out must hold OFullSize floats.  Returns the
// length written, or -1 when the pipeline status is not "OK" (status copied
// into status_out).
long long ref_activate(const float* in, unsigned int n, int exp, float ov, const char* options,
                       float* out, char* status_out, int status_cap)
{
    VECF inData(in, in + n);
    const unsigned int FullSize = inData.size();
    const int windowSize = 1 << exp;
    const int qtConst = toQuot(FullSize, ov, windowSize);
    const unsigned int OFullSize = qtConst * windowSize;
    const unsigned int OHalfSize = OFullSize / 2;
    const unsigned int OMove = windowSize * (1.0f - ov);
    std::vector<float> Real(OFullSize);
    std::vector<float> subReal;
    std::vector<float> Imag(OFullSize);
    std::vector<float> subImag;
    std::vector<float> outMem(OFullSize);
    std::string st = runnerFunction::Default_Pipeline(
        nullptr, &inData, &Real, &Imag, &subReal, &subImag, &outMem, FullSize, windowSize,
        qtConst, OFullSize, OHalfSize, OMove, std::string(options), exp, ov);
    if (status_out && status_cap > 0) {
        std::strncpy(status_out, st.c_str(), status_cap - 1);
        status_out[status_cap - 1] = 0;
    }
    std::memcpy(out, outMem.data(), sizeof(float) * OFullSize);
    return st == "OK" ? (long long)OFullSize : -1;
}

// Reference overlap + one window kernel (kind as in orc_window kinds 1..8).
void ref_overlap_window(const float* in, unsigned int n, int exp, float ov, int kind, float sigma,
                        int remove_dc, float* out)
{
    unsigned qt, hop, ofull, ohalf;
    ref_geometry(n, exp, ov, &qt, &hop, &ofull, &ohalf);
    const unsigned int fs = n, e = exp, N = 1u << exp;
    Overlap_Common(const_cast<float*>(in), ofull, fs, e, hop, out);
    switch (kind) {
    case 1: Window_Hanning(out, ofull, N); break;
    case 2: Window_Hamming(out, ofull, N); break;
    case 3: Window_Blackman(out, ofull, N); break;
    case 4: Window_Nuttall(out, ofull, N); break;
    case 5: Window_Blackman_Nuttall(out, ofull, N); break;
    case 6: Window_Blackman_harris(out, ofull, N); break;
    case 7: Window_FlatTop(out, ofull, N); break;
    case 8: Window_Gaussian(out, ofull, N, sigma); break;
    default: break;
    }
    if (remove_dc) DCRemove_Common(out, ofull, N);
}

}  // extern "C"
