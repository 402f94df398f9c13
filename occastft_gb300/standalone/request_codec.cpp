// RequestCapnp codec: see request_codec.hpp.  Encoding rules followed here
// (Cap'n Proto encoding specification):
//  * flat array: u32 (segments - 1), u32 size in words per segment, padding
//    to 8 bytes, then the segments back to back;
//  * the root pointer is the first word of segment 0;
//  * struct pointer: bits 0-1 = 0, bits 2-31 signed word offset from the end
//    of the pointer, bits 32-47 data words, bits 48-63 pointer count;
//  * list pointer: bits 0-1 = 1, bits 2-31 offset, bits 32-34 element size
//    (2 = byte, 4 = four bytes), bits 35-63 element count;
//  * far pointer: bits 0-1 = 2, bit 2 double-far, bits 3-31 landing-pad word
//    offset, bits 32-63 segment id.  A single-far pad is an ordinary pointer
//    located in the target segment; a double-far pad is a far pointer to the
//    content followed by a tag word (struct or list pointer, offset ignored);
//  * text is a byte list that includes its NUL terminator.
// All values are little-endian (both hosts this runs on are).
#include "request_codec.hpp"

#include <cstring>

namespace ocs_standalone {
namespace {

struct Msg {
    const uint8_t* base = nullptr;
    std::vector<const uint8_t*> seg;  // segment starts
    std::vector<uint64_t> words;      // segment sizes in words
};

uint64_t word_at(const Msg& m, uint32_t s, uint64_t w)
{
    uint64_t v;
    std::memcpy(&v, m.seg[s] + w * 8, 8);
    return v;
}

int64_t sext30(uint64_t ptr) { return (int64_t)(int32_t)(uint32_t)ptr >> 2; }

// A resolved pointer: where the object starts, in which segment, and the
// pointer word that describes it (its offset field no longer matters).
struct Target {
    uint32_t seg = 0;
    uint64_t word = 0;  // object start (word index in seg)
    uint64_t tag = 0;   // struct or list pointer describing the object
    bool null = true;
};

std::string resolve(const Msg& m, uint32_t s, uint64_t at, Target& t)
{
    if (s >= m.seg.size() || at >= m.words[s]) return "pointer outside its segment";
    const uint64_t p = word_at(m, s, at);
    t = Target{};
    if (p == 0) return "";
    const uint32_t kind = (uint32_t)(p & 3u);
    if (kind == 0 || kind == 1) {
        const int64_t start = (int64_t)at + 1 + sext30(p);
        if (start < 0 || (uint64_t)start > m.words[s]) return "pointer target outside its segment";
        t.seg = s;
        t.word = (uint64_t)start;
        t.tag = p;
        t.null = false;
        return "";
    }
    if (kind != 2) return "capability pointers are not part of this schema";
    const bool dbl = (p >> 2) & 1u;
    const uint64_t pad = (p >> 3) & 0x1FFFFFFFu;
    const uint32_t ps = (uint32_t)(p >> 32);
    if (ps >= m.seg.size()) return "far pointer to a missing segment";
    if (!dbl) {
        if (pad >= m.words[ps]) return "far pointer landing pad outside its segment";
        const uint64_t q = word_at(m, ps, pad);
        if ((q & 3u) > 1u) return "far landing pad is not a struct or list pointer";
        const int64_t start = (int64_t)pad + 1 + sext30(q);
        if (start < 0 || (uint64_t)start > m.words[ps]) return "far target outside its segment";
        t.seg = ps;
        t.word = (uint64_t)start;
        t.tag = q;
        t.null = false;
        return "";
    }
    if (pad + 1 >= m.words[ps]) return "double-far landing pad outside its segment";
    const uint64_t f = word_at(m, ps, pad);
    const uint64_t tag = word_at(m, ps, pad + 1);
    if ((f & 3u) != 2u || ((f >> 2) & 1u)) return "double-far pad does not hold a single far pointer";
    const uint32_t cs = (uint32_t)(f >> 32);
    const uint64_t cw = (f >> 3) & 0x1FFFFFFFu;
    if (cs >= m.seg.size() || cw > m.words[cs]) return "double-far content outside its segment";
    if ((tag & 3u) > 1u) return "double-far tag is not a struct or list pointer";
    t.seg = cs;
    t.word = cw;
    t.tag = tag;
    t.null = false;
    return "";
}

std::string read_text(const Msg& m, uint32_t s, uint64_t at, std::string& out)
{
    Target t;
    std::string e = resolve(m, s, at, t);
    if (!e.empty()) return e;
    out.clear();
    if (t.null) return "";
    if ((t.tag & 3u) != 1u || ((t.tag >> 32) & 7u) != 2u) return "text field is not a byte list";
    const uint64_t n = t.tag >> 35;
    if (n == 0) return "";
    if (t.word * 8 + n > m.words[t.seg] * 8) return "text runs past its segment";
    const char* c = reinterpret_cast<const char*>(m.seg[t.seg] + t.word * 8);
    out.assign(c, c + n - 1);  // drop the NUL terminator
    return "";
}

}  // namespace

std::string decode_request(const uint8_t* msg, size_t len, Request& req, std::vector<float>& scratch)
{
    req = Request{};
    if (len < 8) return "message shorter than a segment table";
    uint32_t nseg_m1;
    std::memcpy(&nseg_m1, msg, 4);
    const uint64_t nseg = (uint64_t)nseg_m1 + 1;
    if (nseg > 512) return "too many segments";
    const uint64_t table = ((4 * (1 + nseg)) + 7) / 8 * 8;
    if (table > len) return "segment table runs past the message";
    Msg m;
    m.base = msg;
    uint64_t off = table;
    for (uint64_t i = 0; i < nseg; ++i) {
        uint32_t w;
        std::memcpy(&w, msg + 4 + 4 * i, 4);
        if (off + (uint64_t)w * 8 > len) return "segment runs past the message";
        m.seg.push_back(msg + off);
        m.words.push_back(w);
        off += (uint64_t)w * 8;
    }
    if (m.words[0] == 0) return "empty first segment";
    Target root;
    std::string e = resolve(m, 0, 0, root);
    if (!e.empty()) return e;
    if (root.null || (root.tag & 3u) != 0u) return "root is not a struct";
    const uint64_t dw = (root.tag >> 32) & 0xFFFFu, pc = (root.tag >> 48) & 0xFFFFu;
    if (root.word + dw + pc > m.words[root.seg]) return "root struct runs past its segment";
    auto dword = [&](uint64_t i) -> uint64_t { return i < dw ? word_at(m, root.seg, root.word + i) : 0; };
    req.memPTR = dword(0);
    req.posixFileDes = (int64_t)dword(1);
    req.windowsHandlePTR = dword(2);
    const uint64_t w3 = dword(3);
    req.windowRadix = (uint32_t)w3;
    const uint32_t ob = (uint32_t)(w3 >> 32);
    std::memcpy(&req.overlapRatio, &ob, 4);
    req.dataLength = dword(4);
    req.overlapdataLength = dword(5);
    const uint64_t pbase = root.word + dw;
    if (pc > 0 && !(e = read_text(m, root.seg, pbase + 0, req.sharedMemory)).empty()) return "sharedMemory: " + e;
    if (pc > 2 && !(e = read_text(m, root.seg, pbase + 2, req.mappedID)).empty()) return "mappedID: " + e;
    if (pc > 3 && !(e = read_text(m, root.seg, pbase + 3, req.options)).empty()) return "options: " + e;
    if (pc > 1) {
        Target t;
        e = resolve(m, root.seg, pbase + 1, t);
        if (!e.empty()) return "data: " + e;
        if (!t.null) {
            if ((t.tag & 3u) != 1u || ((t.tag >> 32) & 7u) != 4u) return "data is not a list of 32-bit values";
            const uint64_t n = t.tag >> 35;
            if (t.word * 8 + n * 4 > m.words[t.seg] * 8) return "data list runs past its segment";
            const uint8_t* p = m.seg[t.seg] + t.word * 8;
            req.dataCount = n;
            if ((reinterpret_cast<uintptr_t>(p) & 3u) == 0) {
                req.data = reinterpret_cast<const float*>(p);
            } else {
                scratch.resize(n);
                std::memcpy(scratch.data(), p, n * 4);
                req.data = scratch.data();
            }
        }
    }
    return "";
}

namespace {
uint64_t text_words(const std::string& s) { return s.empty() ? 0 : (s.size() + 1 + 7) / 8; }
uint64_t list_ptr(uint64_t at, uint64_t target, uint32_t esize, uint64_t count)
{
    const int64_t off = (int64_t)target - (int64_t)at - 1;
    return 1u | ((uint64_t)(uint32_t)(off << 2) & 0xFFFFFFFCu) | ((uint64_t)esize << 32) | (count << 35);
}
}  // namespace

size_t encoded_size(const Request& req)
{
    const uint64_t words = 1 + 6 + 4 + text_words(req.sharedMemory) + text_words(req.mappedID) +
                           text_words(req.options) + (req.dataCount * 4 + 7) / 8;
    return 8 + words * 8;
}

void encode_request(const Request& req, uint8_t* out, float** data_slot)
{
    const size_t total = encoded_size(req);
    std::memset(out, 0, total);
    const uint32_t nseg_m1 = 0, segw = (uint32_t)((total - 8) / 8);
    std::memcpy(out, &nseg_m1, 4);
    std::memcpy(out + 4, &segw, 4);
    uint8_t* seg = out + 8;
    auto put = [&](uint64_t w, uint64_t v) { std::memcpy(seg + w * 8, &v, 8); };
    // root struct right after the root pointer: offset 0, 6 data words, 4 pointers
    put(0, (uint64_t)6 << 32 | (uint64_t)4 << 48);
    put(1, req.memPTR);
    put(2, (uint64_t)req.posixFileDes);
    put(3, req.windowsHandlePTR);
    uint32_t ob;
    std::memcpy(&ob, &req.overlapRatio, 4);
    put(4, (uint64_t)req.windowRadix | (uint64_t)ob << 32);
    put(5, req.dataLength);
    put(6, req.overlapdataLength);
    uint64_t next = 11;  // first word after the pointer section (words 7..10)
    auto text = [&](uint64_t slot, const std::string& s) {
        if (s.empty()) return;
        put(slot, list_ptr(slot, next, 2, s.size() + 1));
        std::memcpy(seg + next * 8, s.data(), s.size());
        next += text_words(s);
    };
    text(7 + 0, req.sharedMemory);
    text(7 + 2, req.mappedID);
    text(7 + 3, req.options);
    float* slot = nullptr;
    if (req.dataCount) {
        put(7 + 1, list_ptr(7 + 1, next, 4, req.dataCount));
        slot = reinterpret_cast<float*>(seg + next * 8);
        if (req.data) std::memcpy(slot, req.data, req.dataCount * 4);
        next += (req.dataCount * 4 + 7) / 8;
    }
    if (data_slot) *data_slot = slot;
}

}  // namespace ocs_standalone
