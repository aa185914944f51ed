// Stand-in for the absent core/tcp_adaptor.hpp (single process, no network).
#pragma once
#include <string>
struct TCP_Adaptor {
    void send(int, int, const std::string &) {}
    std::string recv(int) { return std::string(); }
};
