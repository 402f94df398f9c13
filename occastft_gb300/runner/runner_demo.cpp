// Command-line driver of the C++ runner (no server): reads a raw float32
// signal, runs Runner::ActivateSTFT (fused path) or Default_Pipeline over the
// runnerFunction hooks (stage path), and writes the raw float32 result.
//   ocs_runner_demo <in.f32> <out.f32> <windowSizeEXP> <overlapRatio> <options> [stages]
#include "gb300Struct.hpp"
#include "occastft_gb300.h"
#include "occastft_runner.hpp"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>

int main(int argc, char** argv)
{
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s in.f32 out.f32 windowSizeEXP overlapRatio options [stages]\n", argv[0]);
        return 2;
    }
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    std::fseek(f, 0, SEEK_END);
    const long bytes = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    VECF in(bytes / 4);
    if (std::fread(in.data(), 4, in.size(), f) != in.size()) return 3;
    std::fclose(f);
    const int exp = std::atoi(argv[3]);
    const float ov = (float)std::atof(argv[4]);
    const std::string options = argv[5];
    const bool stages = argc > 6 && std::strcmp(argv[6], "stages") == 0;
    Runner runner(0);
    VECF out;
    if (!stages) {
        MAYBE_DATA r = runner.ActivateSTFT(in, exp, ov, options);
        if (!r) {
            std::fprintf(stderr, "ActivateSTFT: %s\n", runner.last_status.c_str());
            return 1;
        }
        out = std::move(*r);
    } else {
        // the reference's sizing block (CudaImpl.cpp:416-421) and buffers
        const unsigned FullSize = in.size();
        const unsigned windowSize = 1u << exp;
        const unsigned qtConst = toQuot(FullSize, ov, windowSize);
        const unsigned OFullSize = qtConst * windowSize;
        const unsigned OHalfSize = OFullSize / 2;
        const unsigned OMove = windowSize * (1.0f - ov);
        float *dIn, *dR, *dI, *dO;
        cudaMalloc(&dIn, 4ull * FullSize);
        cudaMalloc(&dR, 4ull * OFullSize);
        cudaMalloc(&dI, 4ull * OFullSize);
        cudaMalloc(&dO, 4ull * OFullSize);
        cudaMemset(dI, 0, 4ull * OFullSize);
        cudaMemcpy(dIn, in.data(), 4ull * FullSize, cudaMemcpyHostToDevice);
        GB300Data ud;
        const std::string st = runnerFunction::Default_Pipeline(&ud, &dIn, &dR, &dI, nullptr, nullptr, &dO, FullSize,
                                                                windowSize, qtConst, OFullSize, OHalfSize, OMove,
                                                                options, exp, ov);
        out.resize(OFullSize);
        cudaMemcpy(out.data(), dO, 4ull * OFullSize, cudaMemcpyDeviceToHost);
        cudaFree(dIn);
        cudaFree(dR);
        cudaFree(dI);
        cudaFree(dO);
        if (st != "OK") {
            std::fprintf(stderr, "Default_Pipeline: %s\n", st.c_str());
            return 1;
        }
    }
    FILE* o = std::fopen(argv[2], "wb");
    if (!o) return 4;
    std::fwrite(out.data(), 4, out.size(), o);
    std::fclose(o);
    return 0;
}
