// TEST INFRASTRUCTURE ONLY: mutation fuzzing of the runner's WebSocket server
// (occastft_gb300/standalone/ws_server.cpp), which parses bytes a network
// peer sends.  The real server listens on a loopback port in this process,
// built with AddressSanitizer and UndefinedBehaviorSanitizer.  Each case
// connects, completes the opening handshake, sends a mutated stream of valid
// client frames (masked text, fragmented binary, ping, close) and hangs up;
// the handler reads every byte of every message it is given.  At the end a
// clean client must still be served.  Prints "cases: <n>, messages: <m>" and
// exits 0 when no sanitizer fired.
//
//   ws_fuzz <cases>
#include "ws_server.hpp"

#include <arpa/inet.h>
#include <netinet/in.h>
#include <sys/socket.h>
#include <sys/time.h>
#include <unistd.h>

#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

using namespace ocs_standalone;

namespace {

std::atomic<long> g_messages{0};
volatile uint64_t g_sink = 0;

void frame(std::vector<uint8_t>& out, int op, bool fin, const std::vector<uint8_t>& payload, std::mt19937_64& rng)
{
    out.push_back((uint8_t)((fin ? 0x80 : 0) | op));
    const size_t n = payload.size();
    if (n < 126) {
        out.push_back((uint8_t)(0x80 | n));
    } else if (n <= 0xFFFF) {
        out.push_back(0x80 | 126);
        out.push_back((uint8_t)(n >> 8));
        out.push_back((uint8_t)n);
    } else {
        out.push_back(0x80 | 127);
        for (int i = 7; i >= 0; --i) out.push_back((uint8_t)((uint64_t)n >> (8 * i)));
    }
    uint8_t key[4];
    for (auto& k : key) k = (uint8_t)rng();
    out.insert(out.end(), key, key + 4);
    for (size_t i = 0; i < n; ++i) out.push_back(payload[i] ^ key[i & 3]);
}

std::vector<uint8_t> stream(std::mt19937_64& rng)
{
    std::vector<uint8_t> s;
    auto bytes = [&](size_t n) {
        std::vector<uint8_t> v(n);
        for (auto& b : v) b = (uint8_t)rng();
        return v;
    };
    frame(s, 1, true, bytes(rng() % 40), rng);         // text
    frame(s, 2, false, bytes(rng() % 300), rng);       // binary, first fragment
    frame(s, 9, true, bytes(rng() % 20), rng);         // ping inside the fragmented message
    frame(s, 0, false, bytes(rng() % 70000), rng);     // continuation (16-bit or 64-bit length)
    frame(s, 0, true, bytes(rng() % 10), rng);         // last fragment
    frame(s, 8, true, {0x03, 0xE8}, rng);              // close
    const int edits = 1 + (int)(rng() % 8);
    for (int e = 0; e < edits && !s.empty(); ++e) {
        switch (rng() % 4) {
        case 0: s[rng() % s.size()] ^= (uint8_t)(1u << (rng() % 8)); break;
        case 1: s[rng() % std::min<size_t>(s.size(), 64)] = (uint8_t)rng(); break;  // mostly headers
        case 2: s.resize(rng() % s.size()); break;
        case 3: s[rng() % s.size()] = (uint8_t)rng(); break;
        }
    }
    return s;
}

int connect_to(int port)
{
    const int fd = ::socket(AF_INET, SOCK_STREAM, 0);
    sockaddr_in a{};
    a.sin_family = AF_INET;
    a.sin_port = htons((uint16_t)port);
    a.sin_addr.s_addr = htonl(INADDR_LOOPBACK);
    if (::connect(fd, reinterpret_cast<sockaddr*>(&a), sizeof a) != 0) {
        ::close(fd);
        return -1;
    }
    timeval tv{2, 0};
    ::setsockopt(fd, SOL_SOCKET, SO_RCVTIMEO, &tv, sizeof tv);
    return fd;
}

bool handshake(int fd)
{
    const char* req = "GET / HTTP/1.1\r\nHost: x\r\nUpgrade: websocket\r\nConnection: Upgrade\r\n"
                      "Sec-WebSocket-Key: dGhlIHNhbXBsZSBub25jZQ==\r\nSec-WebSocket-Version: 13\r\n\r\n";
    if (::send(fd, req, std::strlen(req), MSG_NOSIGNAL) < 0) return false;
    std::string resp;
    char buf[512];
    while (resp.find("\r\n\r\n") == std::string::npos) {
        const ssize_t k = ::recv(fd, buf, sizeof buf, 0);
        if (k <= 0) return false;
        resp.append(buf, (size_t)k);
    }
    return resp.compare(0, 12, "HTTP/1.1 101") == 0;
}

void drain(int fd)
{
    char buf[4096];
    while (::recv(fd, buf, sizeof buf, 0) > 0) {
    }
}

}  // namespace

int main(int argc, char** argv)
{
    const long cases = argc > 1 ? std::atol(argv[1]) : 1000;
    WsServer server;
    if (!server.listen(0).empty()) return 2;
    std::thread srv([&] {
        server.run([](Connection& c, const Message& m) {
            uint64_t h = 0;
            const uint8_t* p = m.data();
            for (size_t i = 0; i < m.size; ++i) h = h * 131 + p[i];
            g_sink = g_sink + h;
            ++g_messages;
            if (m.binary) c.send_binary(p, m.size < 16 ? m.size : 16);
        });
    });
    std::mt19937_64 rng(424242);
    long done = 0;
    for (long i = 0; i < cases; ++i) {
        const int fd = connect_to(server.port());
        if (fd < 0) continue;
        if (handshake(fd)) {
            const std::vector<uint8_t> s = stream(rng);
            ::send(fd, s.data(), s.size(), MSG_NOSIGNAL);
            ::shutdown(fd, SHUT_WR);
            drain(fd);
        }
        ::close(fd);
        ++done;
    }
    // a clean client is still served
    bool served = false;
    const int fd = connect_to(server.port());
    if (fd >= 0 && handshake(fd)) {
        std::vector<uint8_t> s;
        frame(s, 9, true, {'o', 'k'}, rng);
        ::send(fd, s.data(), s.size(), MSG_NOSIGNAL);
        uint8_t r[4];
        served = ::recv(fd, r, 4, MSG_WAITALL) == 4 && r[0] == 0x8A && r[1] == 2 && r[2] == 'o' && r[3] == 'k';
    }
    if (fd >= 0) ::close(fd);
    server.stop();
    srv.join();
    std::printf("cases: %ld, messages: %ld, clean client served: %s\n", done, g_messages.load(), served ? "yes" : "no");
    return served ? 0 : 1;
}
