// Minimal WebSocket server (RFC 6455) for the runner executable.
//
// The reference's runners serve through IXWebSocket on 0.0.0.0:<port>
// (StandAlone/cross_gpgpu/GLOBAL/RunnerCommon.cpp:62-140): binary messages
// carry RequestCapnp requests, the text message "CLOSE_REQUEST" stops the
// runner.  This is the part of that server the protocol needs: the opening
// handshake (Sec-WebSocket-Accept), masked client frames, fragmented
// messages, ping/pong, close, and unmasked server frames.  Extensions that a
// client offers (permessage-deflate) are declined by not echoing them, which
// RFC 7692 allows; the client then sends uncompressed frames.  One thread
// per connection; messages of one connection are handled in order.  At most
// kMaxConnections connections are open at once (more are closed at
// accept), and a peer must complete its opening handshake within a few
// seconds of the accept (one limit for all its reads).
#pragma once
#include <atomic>
#include <chrono>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <string>
#include <vector>

namespace ocs_standalone {

constexpr int kMaxConnections = 256;

// SHA-1 (FIPS 180-4) and base64 (RFC 4648), as the handshake needs them.
void sha1(const uint8_t* data, size_t len, uint8_t out[20]);
std::string base64(const uint8_t* data, size_t len);
// Sec-WebSocket-Accept for a client's Sec-WebSocket-Key
std::string websocket_accept(const std::string& key);

class Connection {
public:
    explicit Connection(int fd) : fd_(fd) {}
    bool send_text(const std::string& s);
    bool send_binary(const uint8_t* p, size_t n);
    int fd() const { return fd_; }

private:
    friend class WsServer;
    bool send_frame(int opcode, const uint8_t* p, size_t n);
    int fd_;
};

// A received message.  Binary payloads are stored 8-byte aligned (a
// RequestCapnp flat array is read in place).
struct Message {
    bool binary = false;
    std::vector<uint64_t> store;
    size_t size = 0;
    const uint8_t* data() const { return reinterpret_cast<const uint8_t*>(store.data()); }
    std::string text() const { return std::string(reinterpret_cast<const char*>(store.data()), size); }
};

class WsServer {
public:
    using Handler = std::function<void(Connection&, const Message&)>;
    // Binds 0.0.0.0:port.  Returns "" or the error.
    std::string listen(int port);
    // Accepts connections and serves them until stop(); returns when every
    // connection thread has ended.
    void run(const Handler& on_message);
    // Asks run() to return: closes the listening socket and every connection.
    void stop();
    int port() const { return port_; }

private:
    // accepted: when the connection was accepted (the handshake deadline counts from it)
    void serve(int fd, std::chrono::steady_clock::time_point accepted, const Handler& on_message);
    int lfd_ = -1;
    int port_ = 0;
    std::atomic<bool> stopping_{false};
};

}  // namespace ocs_standalone
