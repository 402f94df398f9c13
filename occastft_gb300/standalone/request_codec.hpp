// RequestCapnp on the wire, without the Cap'n Proto library.
//
// The reference's proxy and runners exchange one Cap'n Proto struct per
// WebSocket binary message (StandAlone/include/FFTcapnp.capnp:1-16), written
// with capnp::messageToFlatArray (StandAlone/src/FFTStruct.cpp:41-53): a
// segment table followed by the segments.  This codec reads any such message
// (several segments, single- and double-far pointers, data or pointer
// sections shorter than the schema's) and writes single-segment messages,
// following the published Cap'n Proto encoding.  Field placement is the one
// the capnp compiler assigns to the schema (6 data words, 4 pointers):
//   data word 0 memPTR, 1 posixFileDes, 2 windowsHandlePTR,
//   word 3 low half windowRadix, word 3 high half overlapRatio,
//   word 4 dataLength, word 5 overlapdataLength;
//   pointer 0 sharedMemory, 1 data, 2 mappedID, 3 options.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace ocs_standalone {

struct Request {
    std::string sharedMemory;
    std::string mappedID;
    std::string options;
    uint64_t memPTR = 0;
    int64_t posixFileDes = 0;
    uint64_t windowsHandlePTR = 0;
    uint32_t windowRadix = 0;
    float overlapRatio = 0.0f;
    uint64_t dataLength = 0;
    uint64_t overlapdataLength = 0;
    // data list: points into the decoded message buffer (no copy); on encode,
    // `data` (when non-null) is written as the list
    const float* data = nullptr;
    uint64_t dataCount = 0;
};

// Decodes a flat-array message.  Returns "" on success, else what is wrong.
// `msg` must stay alive while req.data is used; it must be 4-byte aligned for
// req.data to be read as floats in place (otherwise the list is copied into
// `scratch`).
std::string decode_request(const uint8_t* msg, size_t len, Request& req, std::vector<float>& scratch);

// Size in bytes of the single-segment message encode_request writes.
size_t encoded_size(const Request& req);

// Writes a single-segment flat-array message into out (encoded_size bytes,
// 8-byte aligned).  If data_slot is non-null it receives where the data
// list's floats start in out, so a caller may fill them later (req.data may
// then be null with req.dataCount set).
void encode_request(const Request& req, uint8_t* out, float** data_slot);

}  // namespace ocs_standalone
