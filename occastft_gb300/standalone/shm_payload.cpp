// POSIX shared-memory payloads: see shm_payload.hpp.
#include "shm_payload.hpp"

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdint>
#include <cstring>

namespace ocs_standalone {

bool protocol_shm_name(const std::string& name)
{
    static const std::string head = "/STFT", tail = "SHAREDMEM";
    return name.size() > head.size() + tail.size() && name.compare(0, head.size(), head) == 0 &&
           name.compare(name.size() - tail.size(), tail.size(), tail) == 0 && name.find('/', 1) == std::string::npos;
}

size_t page_rounded_bytes(uint64_t floats)
{
    const uint64_t page = (uint64_t)sysconf(_SC_PAGESIZE);
    if (floats > (UINT64_MAX - page) / sizeof(float)) return 0;  // no such region: refused by the caller
    const uint64_t bytes = floats * sizeof(float);
    return (size_t)((bytes + page - 1) / page * page);
}

std::string shm_map(const std::string& name, uint64_t overlap_floats, ShmMapping& m, bool populate)
{
    m = ShmMapping{};
    const size_t bytes = page_rounded_bytes(overlap_floats);
    if (bytes == 0) return "shared memory region of zero bytes or beyond the address space";
    const int fd = shm_open(name.c_str(), O_RDWR, 0666);
    if (fd < 0) return "shm_open " + name + ": " + std::strerror(errno);
    // the mapping must not reach past the object: a store there would fault
    struct stat st;
    if (fstat(fd, &st) != 0 || (uint64_t)st.st_size < bytes) {
        close(fd);
        return "shared memory object " + name + " is smaller than overlapdataLength floats";
    }
    // MAP_POPULATE: build the page tables now, in one pass, instead of one
    // fault per page while the copies to and from the device run over it
    void* p = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_SHARED | (populate ? MAP_POPULATE : 0), fd, 0);
    if (p == MAP_FAILED) {
        const std::string e = std::strerror(errno);
        close(fd);
        return "mmap " + name + ": " + e;
    }
    m.ptr = p;
    m.bytes = bytes;
    m.fd = fd;
    return "";
}

void shm_unmap(ShmMapping& m)
{
    if (m.ptr) munmap(m.ptr, m.bytes);
    if (m.fd >= 0) close(m.fd);
    m = ShmMapping{};
}

}  // namespace ocs_standalone
