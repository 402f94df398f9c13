// POSIX shared-memory payloads, the runner's side.
//
// A proxy that runs next to the runner puts the signal into a POSIX shared
// memory object named "/STFT<mappedID>SHAREDMEM", sized to the page-rounded
// byte length of overlapdataLength floats, and sends only its name
// (StandAlone/src/FFTStruct_linux.cpp:5-65).  The runner maps the same object
// read-write, reads dataLength floats, writes the result over it and unmaps
// it; unlinking stays with the proxy (FFTStruct_linux.cpp:112-160).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

namespace ocs_standalone {

struct ShmMapping {
    void* ptr = nullptr;
    size_t bytes = 0;
    int fd = -1;
};

// Whether `name` has the protocol's form "/STFT<mappedID>SHAREDMEM" (no other
// '/').  The runner maps only such objects: a peer cannot point it at, and
// have it overwrite, any other shared-memory object its user can open.
bool protocol_shm_name(const std::string& name);

// page-rounded byte size of `floats` floats (FFTStruct.hpp:151-157)
size_t page_rounded_bytes(uint64_t floats);

// Opens and maps an existing object; `populate` builds the mapping's page
// tables up front.  Returns "" or the error.
std::string shm_map(const std::string& name, uint64_t overlap_floats, ShmMapping& m, bool populate);

void shm_unmap(ShmMapping& m);

}  // namespace ocs_standalone
