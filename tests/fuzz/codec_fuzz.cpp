// TEST INFRASTRUCTURE ONLY: mutation fuzzing of the runner's RequestCapnp
// decoder (occastft_gb300/standalone/request_codec.cpp), which reads bytes a
// network peer sends.  Built with AddressSanitizer and UndefinedBehavior-
// Sanitizer: every mutated message sits in a buffer of exactly its length, so
// a read past the message, or past a segment into the next allocation, stops
// the run.  A message that decodes has every field and every data element
// read back, so the pointers the decoder hands out are checked as well.
//
//   codec_fuzz <iterations per seed> <seed file>...
// Prints "decoded ok: <n> of <m>" and exits 0 when no sanitizer fired.
#include "request_codec.hpp"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iterator>
#include <random>
#include <string>
#include <vector>

using ocs_standalone::Request;

namespace {

volatile uint64_t g_sink = 0;

void touch(const Request& r)
{
    uint64_t h = r.sharedMemory.size() + r.mappedID.size() + r.options.size();
    for (char c : r.sharedMemory) h = h * 31 + (unsigned char)c;
    for (char c : r.mappedID) h = h * 31 + (unsigned char)c;
    for (char c : r.options) h = h * 31 + (unsigned char)c;
    if (r.data) {
        uint32_t v;
        for (uint64_t i = 0; i < r.dataCount; ++i) {
            std::memcpy(&v, r.data + i, 4);
            h += v;
        }
    }
    g_sink = g_sink + h + r.memPTR + r.dataLength + r.overlapdataLength + r.windowRadix;
}

const uint64_t kSpecial[] = {0,
                             ~0ull,
                             1ull << 31,
                             (1ull << 32) - 1,
                             0x00000000FFFFFFFCull,  // struct pointer, offset -1
                             0x0004000600000000ull,  // struct pointer, 6 data words, 4 pointers
                             0xFFFFFFF800000001ull,  // list pointer, huge count
                             0x000000FF00000002ull,  // far pointer to segment 255
                             0x0000000100000006ull,  // double-far pointer to segment 1
                             0x7FFFFFFFFFFFFFFFull};

std::vector<uint8_t> mutate(const std::vector<uint8_t>& seed, std::mt19937_64& rng)
{
    std::vector<uint8_t> m = seed;
    const int edits = 1 + (int)(rng() % 6);
    for (int e = 0; e < edits; ++e) {
        switch (rng() % 6) {
        case 0:  // flip bits of a byte
            if (!m.empty()) m[rng() % m.size()] ^= (uint8_t)(1u << (rng() % 8));
            break;
        case 1:  // random byte
            if (!m.empty()) m[rng() % m.size()] = (uint8_t)rng();
            break;
        case 2:  // an aligned word set to a special or random value
            if (m.size() >= 8) {
                const size_t w = (rng() % (m.size() / 8)) * 8;
                const uint64_t v = (rng() % 2) ? kSpecial[rng() % (sizeof kSpecial / sizeof kSpecial[0])] : rng();
                std::memcpy(m.data() + w, &v, 8);
            }
            break;
        case 3:  // truncate
            if (!m.empty()) m.resize(rng() % m.size());
            break;
        case 4:  // append random bytes
            for (int i = 0, n = (int)(rng() % 64); i < n; ++i) m.push_back((uint8_t)rng());
            break;
        case 5:  // segment-table entry (first 4..4+4k bytes) set to a random count
            if (m.size() >= 8) {
                const uint32_t v = (rng() % 2) ? (uint32_t)(rng() % 64) : (uint32_t)rng();
                std::memcpy(m.data() + 4 * (1 + rng() % std::min<size_t>(4, m.size() / 4 - 1)), &v, 4);
            }
            break;
        }
    }
    return m;
}

}  // namespace

int main(int argc, char** argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: codec_fuzz <iterations> <seed>...\n");
        return 2;
    }
    const long iters = std::atol(argv[1]);
    std::mt19937_64 rng(20260101);
    long ok = 0, total = 0;
    for (int a = 2; a < argc; ++a) {
        std::ifstream f(argv[a], std::ios::binary);
        const std::vector<uint8_t> seed((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
        // the seed itself must decode
        {
            std::vector<uint8_t> copy = seed;
            Request r;
            std::vector<float> scratch;
            if (!ocs_standalone::decode_request(copy.data(), copy.size(), r, scratch).empty()) {
                std::printf("seed %s does not decode\n", argv[a]);
                return 1;
            }
            touch(r);
        }
        for (long i = 0; i < iters; ++i) {
            const std::vector<uint8_t> m = mutate(seed, rng);
            // exactly m.size() bytes, 16-byte aligned (operator new): any overread is outside the block
            uint8_t* buf = new uint8_t[m.size() ? m.size() : 1];
            if (!m.empty()) std::memcpy(buf, m.data(), m.size());
            Request r;
            std::vector<float> scratch;
            const std::string e = ocs_standalone::decode_request(buf, m.size(), r, scratch);
            if (e.empty()) {
                touch(r);
                ++ok;
            }
            ++total;
            delete[] buf;
        }
    }
    std::printf("decoded ok: %ld of %ld\n", ok, total);
    return 0;
}
