// Minimal WebSocket server: see ws_server.hpp.
#include "ws_server.hpp"

#include <arpa/inet.h>
#include <netinet/in.h>
#include <netinet/tcp.h>
#include <poll.h>
#include <sys/socket.h>
#include <unistd.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <chrono>
#include <cstring>
#include <exception>
#include <memory>
#include <mutex>
#include <new>
#include <set>
#include <thread>

namespace ocs_standalone {

// ------------------------------------------------------------ SHA-1, base64
namespace {
inline uint32_t rotl(uint32_t x, int n) { return (x << n) | (x >> (32 - n)); }
}  // namespace

void sha1(const uint8_t* data, size_t len, uint8_t out[20])
{
    uint32_t h[5] = {0x67452301u, 0xEFCDAB89u, 0x98BADCFEu, 0x10325476u, 0xC3D2E1F0u};
    std::vector<uint8_t> m(data, data + len);
    m.push_back(0x80);
    while (m.size() % 64 != 56) m.push_back(0);
    const uint64_t bits = (uint64_t)len * 8;
    for (int i = 7; i >= 0; --i) m.push_back((uint8_t)(bits >> (8 * i)));
    for (size_t c = 0; c < m.size(); c += 64) {
        uint32_t w[80];
        for (int t = 0; t < 16; ++t)
            w[t] = (uint32_t)m[c + 4 * t] << 24 | (uint32_t)m[c + 4 * t + 1] << 16 | (uint32_t)m[c + 4 * t + 2] << 8 |
                   (uint32_t)m[c + 4 * t + 3];
        for (int t = 16; t < 80; ++t) w[t] = rotl(w[t - 3] ^ w[t - 8] ^ w[t - 14] ^ w[t - 16], 1);
        uint32_t a = h[0], b = h[1], cc = h[2], d = h[3], e = h[4];
        for (int t = 0; t < 80; ++t) {
            uint32_t f, k;
            if (t < 20) {
                f = (b & cc) | (~b & d);
                k = 0x5A827999u;
            } else if (t < 40) {
                f = b ^ cc ^ d;
                k = 0x6ED9EBA1u;
            } else if (t < 60) {
                f = (b & cc) | (b & d) | (cc & d);
                k = 0x8F1BBCDCu;
            } else {
                f = b ^ cc ^ d;
                k = 0xCA62C1D6u;
            }
            const uint32_t tmp = rotl(a, 5) + f + e + k + w[t];
            e = d;
            d = cc;
            cc = rotl(b, 30);
            b = a;
            a = tmp;
        }
        h[0] += a;
        h[1] += b;
        h[2] += cc;
        h[3] += d;
        h[4] += e;
    }
    for (int i = 0; i < 5; ++i)
        for (int j = 0; j < 4; ++j) out[4 * i + j] = (uint8_t)(h[i] >> (24 - 8 * j));
}

std::string base64(const uint8_t* d, size_t n)
{
    static const char* A = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
    std::string o;
    for (size_t i = 0; i < n; i += 3) {
        const uint32_t v = (uint32_t)d[i] << 16 | (i + 1 < n ? (uint32_t)d[i + 1] << 8 : 0u) |
                           (i + 2 < n ? (uint32_t)d[i + 2] : 0u);
        o.push_back(A[(v >> 18) & 63]);
        o.push_back(A[(v >> 12) & 63]);
        o.push_back(i + 1 < n ? A[(v >> 6) & 63] : '=');
        o.push_back(i + 2 < n ? A[v & 63] : '=');
    }
    return o;
}

std::string websocket_accept(const std::string& key)
{
    const std::string s = key + "258EAFA5-E914-47DA-95CA-C5AB0DC85B11";  // RFC 6455 section 1.3
    uint8_t dg[20];
    sha1(reinterpret_cast<const uint8_t*>(s.data()), s.size(), dg);
    return base64(dg, 20);
}

// ------------------------------------------------------------ socket helpers
namespace {

bool send_all(int fd, const uint8_t* p, size_t n)
{
    while (n) {
        const ssize_t k = ::send(fd, p, n, MSG_NOSIGNAL);
        if (k < 0) {
            if (errno == EINTR) continue;
            return false;
        }
        p += k;
        n -= (size_t)k;
    }
    return true;
}

bool recv_all(int fd, uint8_t* p, size_t n)
{
    while (n) {
        const ssize_t k = ::recv(fd, p, n, 0);
        if (k == 0) return false;
        if (k < 0) {
            if (errno == EINTR) continue;
            return false;
        }
        p += k;
        n -= (size_t)k;
    }
    return true;
}

std::string lower(std::string s)
{
    for (char& c : s) c = (char)std::tolower((unsigned char)c);
    return s;
}

std::string trim(const std::string& s)
{
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

// the opening handshake; false when the peer is not a WebSocket client or
// has not sent its whole opening request by `deadline` (one limit for all
// reads, so a peer that trickles bytes cannot stretch it)
bool handshake(int fd, std::chrono::steady_clock::time_point deadline)
{
    std::string req;
    char buf[1024];
    while (req.find("\r\n\r\n") == std::string::npos) {
        if (req.size() > 16384) return false;
        const auto left = std::chrono::duration_cast<std::chrono::milliseconds>(
                              deadline - std::chrono::steady_clock::now())
                              .count();
        if (left <= 0) return false;
        pollfd p{fd, POLLIN, 0};
        const int r = ::poll(&p, 1, (int)std::min<long long>(left, 1000));
        if (r < 0 && errno == EINTR) continue;
        if (r < 0) return false;
        if (r == 0) continue;  // the loop re-checks the deadline
        const ssize_t k = ::recv(fd, buf, sizeof buf, 0);
        if (k < 0 && errno == EINTR) continue;
        if (k <= 0) return false;
        req.append(buf, (size_t)k);
    }
    // bytes after the header block would be frames; a client waits for the
    // 101 answer before sending any, so none are expected here
    std::string key;
    bool upgrade = false;
    size_t pos = req.find("\r\n");
    const std::string first = req.substr(0, pos);
    while (pos != std::string::npos) {
        const size_t nx = req.find("\r\n", pos + 2);
        if (nx == std::string::npos || nx == pos + 2) break;
        const std::string line = req.substr(pos + 2, nx - pos - 2);
        const size_t c = line.find(':');
        if (c != std::string::npos) {
            const std::string name = lower(trim(line.substr(0, c)));
            const std::string val = trim(line.substr(c + 1));
            if (name == "sec-websocket-key") key = val;
            if (name == "upgrade" && lower(val).find("websocket") != std::string::npos) upgrade = true;
        }
        pos = nx;
    }
    if (first.compare(0, 4, "GET ") != 0 || key.empty() || !upgrade) {
        static const char* bad = "HTTP/1.1 400 Bad Request\r\nContent-Length: 0\r\nConnection: close\r\n\r\n";
        send_all(fd, reinterpret_cast<const uint8_t*>(bad), std::strlen(bad));
        return false;
    }
    const std::string resp = "HTTP/1.1 101 Switching Protocols\r\nUpgrade: websocket\r\nConnection: Upgrade\r\n"
                             "Sec-WebSocket-Accept: " +
                             websocket_accept(key) + "\r\n\r\n";
    return send_all(fd, reinterpret_cast<const uint8_t*>(resp.data()), resp.size());
}

constexpr uint64_t kMaxMessage = 1ull << 36;
constexpr int kHandshakeSeconds = 5;  // a peer that has not sent its opening request by then is dropped
constexpr uint64_t kRecvStep = 64ull << 20;  // payload bytes received per buffer growth

}  // namespace

// ------------------------------------------------------------ frames
bool Connection::send_frame(int opcode, const uint8_t* p, size_t n)
{
    uint8_t h[10];
    size_t hl = 2;
    h[0] = (uint8_t)(0x80 | opcode);
    if (n < 126) {
        h[1] = (uint8_t)n;
    } else if (n <= 0xFFFF) {
        h[1] = 126;
        h[2] = (uint8_t)(n >> 8);
        h[3] = (uint8_t)n;
        hl = 4;
    } else {
        h[1] = 127;
        for (int i = 0; i < 8; ++i) h[2 + i] = (uint8_t)((uint64_t)n >> (56 - 8 * i));
        hl = 10;
    }
    return send_all(fd_, h, hl) && (n == 0 || send_all(fd_, p, n));
}

bool Connection::send_text(const std::string& s)
{
    return send_frame(1, reinterpret_cast<const uint8_t*>(s.data()), s.size());
}

bool Connection::send_binary(const uint8_t* p, size_t n) { return send_frame(2, p, n); }

// ------------------------------------------------------------ server
namespace {
std::mutex g_conn_mu;
std::set<int> g_conns;
}  // namespace

std::string WsServer::listen(int port)
{
    lfd_ = ::socket(AF_INET, SOCK_STREAM, 0);
    if (lfd_ < 0) return std::string("socket: ") + std::strerror(errno);
    int one = 1;
    ::setsockopt(lfd_, SOL_SOCKET, SO_REUSEADDR, &one, sizeof one);
    sockaddr_in a{};
    a.sin_family = AF_INET;
    a.sin_port = htons((uint16_t)port);
    a.sin_addr.s_addr = htonl(INADDR_ANY);
    if (::bind(lfd_, reinterpret_cast<sockaddr*>(&a), sizeof a) != 0 || ::listen(lfd_, 64) != 0) {
        const std::string e = std::strerror(errno);
        ::close(lfd_);
        lfd_ = -1;
        return "bind/listen on port " + std::to_string(port) + ": " + e;
    }
    socklen_t al = sizeof a;
    ::getsockname(lfd_, reinterpret_cast<sockaddr*>(&a), &al);
    port_ = ntohs(a.sin_port);
    return "";
}

void WsServer::stop()
{
    stopping_ = true;
    std::lock_guard<std::mutex> lk(g_conn_mu);
    for (int fd : g_conns) ::shutdown(fd, SHUT_RDWR);
}

void WsServer::run(const Handler& on_message)
{
    // connection threads, joined as they finish so a long-running server
    // does not accumulate them
    struct Worker {
        std::thread t;
        std::shared_ptr<std::atomic<bool>> done;
    };
    std::vector<Worker> workers;
    auto reap = [&workers] {
        for (auto it = workers.begin(); it != workers.end();) {
            if (it->done->load()) {
                it->t.join();
                it = workers.erase(it);
            } else {
                ++it;
            }
        }
    };
    while (!stopping_) {
        reap();
        pollfd p{lfd_, POLLIN, 0};
        const int r = ::poll(&p, 1, 100);
        if (r <= 0 || !(p.revents & POLLIN)) continue;
        const int fd = ::accept(lfd_, nullptr, nullptr);
        if (fd < 0) continue;
        const auto accepted = std::chrono::steady_clock::now();
        if (workers.size() >= (size_t)kMaxConnections) {  // at the cap: refused at once
            ::close(fd);
            continue;
        }
        int one = 1;
        ::setsockopt(fd, IPPROTO_TCP, TCP_NODELAY, &one, sizeof one);
        {
            std::lock_guard<std::mutex> lk(g_conn_mu);
            g_conns.insert(fd);
        }
        auto done = std::make_shared<std::atomic<bool>>(false);
        try {
            workers.push_back(Worker{std::thread([this, fd, accepted, &on_message, done] {
                                         serve(fd, accepted, on_message);
                                         done->store(true);
                                     }),
                                     done});
        } catch (const std::exception&) {  // no thread for it: drop the connection
            {
                std::lock_guard<std::mutex> lk(g_conn_mu);
                g_conns.erase(fd);
            }
            ::close(fd);
        }
    }
    ::close(lfd_);
    lfd_ = -1;
    for (auto& w : workers) w.t.join();
}

void WsServer::serve(int fd, std::chrono::steady_clock::time_point accepted, const Handler& on_message)
{
    Connection conn(fd);
    // the whole opening handshake must arrive within kHandshakeSeconds of
    // the accept; afterwards reads wait as long as the peer keeps the
    // connection open (a client such as the reference's proxy holds one
    // connection and sends requests on it whenever it has one)
    const bool upgraded =
        handshake(fd, accepted + std::chrono::seconds(kHandshakeSeconds));
    if (upgraded) {
        Message msg;
        bool in_msg = false;
        uint64_t have = 0;
        while (!stopping_) {
            uint8_t h[2];
            if (!recv_all(fd, h, 2)) break;
            const bool fin = h[0] & 0x80;
            const int op = h[0] & 0x0F;
            const bool masked = h[1] & 0x80;
            uint64_t len = h[1] & 0x7F;
            if (len == 126) {
                uint8_t e[2];
                if (!recv_all(fd, e, 2)) break;
                len = (uint64_t)e[0] << 8 | e[1];
            } else if (len == 127) {
                uint8_t e[8];
                if (!recv_all(fd, e, 8)) break;
                len = 0;
                for (int i = 0; i < 8; ++i) len = len << 8 | e[i];
            }
            uint8_t key[4] = {0, 0, 0, 0};
            if (masked && !recv_all(fd, key, 4)) break;
            if ((h[0] & 0x70) || !masked) {  // no extension negotiated; clients must mask (RFC 6455 5.1)
                const uint8_t code[2] = {0x03, 0xEA};  // 1002 protocol error
                conn.send_frame(8, code, 2);
                break;
            }
            if (op >= 8) {  // control frame: at most 125 bytes, never fragmented
                if (!fin || len > 125) break;
                uint8_t pl[125];
                if (len && !recv_all(fd, pl, (size_t)len)) break;
                for (uint64_t i = 0; i < len; ++i) pl[i] ^= key[i & 3];
                if (op == 9) {
                    conn.send_frame(10, pl, (size_t)len);  // pong with the ping's payload
                } else if (op == 8) {
                    conn.send_frame(8, pl, len >= 2 ? 2 : 0);  // echo the status code
                    break;
                }
                continue;  // pong: nothing to do
            }
            if (op == 1 || op == 2) {
                if (in_msg) break;  // a new message inside a fragmented one
                msg = Message{};
                msg.binary = (op == 2);
                have = 0;
                in_msg = true;
            } else if (op != 0 || !in_msg) {
                break;
            }
            // have <= kMaxMessage here, so the subtraction cannot wrap (a sum
            // with a 64-bit frame length could); an allocation the host
            // cannot make is answered like a message that is too big
            bool fits = len <= kMaxMessage && have <= kMaxMessage - len;
            // The buffer grows with the bytes that arrive, not with the
            // length a header states: a header alone allocates nothing.
            // Capacity doubles, capped at the frame's end, so the copies on
            // growth stay within twice the message.
            bool lost = false;
            for (uint64_t got = 0; fits && got < len;) {
                const uint64_t step = std::min<uint64_t>(len - got, kRecvStep);
                const size_t words = (size_t)((have + got + step + 7) / 8);
                try {
                    if (words > msg.store.capacity())
                        msg.store.reserve(std::max<size_t>(
                            words, std::min<size_t>(2 * msg.store.capacity(), (size_t)((have + len + 7) / 8))));
                    msg.store.resize(words);
                } catch (const std::bad_alloc&) {
                    fits = false;
                    break;
                }
                if (!recv_all(fd, reinterpret_cast<uint8_t*>(msg.store.data()) + have + got, (size_t)step)) {
                    lost = true;
                    break;
                }
                got += step;
            }
            if (!fits) {
                const uint8_t code[2] = {0x03, 0xF1};  // 1009 message too big
                conn.send_frame(8, code, 2);
                break;
            }
            if (lost) break;
            uint8_t* dst = reinterpret_cast<uint8_t*>(msg.store.data()) + have;
            // unmask; the key repeats every 4 bytes of the frame payload
            uint64_t i = 0;
            uint32_t k32;
            std::memcpy(&k32, key, 4);
            const uint64_t k64 = (uint64_t)k32 << 32 | k32;
            for (; i + 8 <= len; i += 8) {
                uint64_t v;
                std::memcpy(&v, dst + i, 8);
                v ^= k64;
                std::memcpy(dst + i, &v, 8);
            }
            for (; i < len; ++i) dst[i] ^= key[i & 3];
            have += len;
            if (fin) {
                msg.size = (size_t)have;
                in_msg = false;
                try {
                    on_message(conn, msg);
                } catch (const std::exception&) {  // the handler failed: end this connection only
                    const uint8_t code[2] = {0x03, 0xF3};  // 1011 internal error
                    conn.send_frame(8, code, 2);
                    break;
                }
                msg = Message{};
            }
        }
    }
    {
        std::lock_guard<std::mutex> lk(g_conn_mu);
        g_conns.erase(fd);
    }
    ::close(fd);
}

}  // namespace ocs_standalone
