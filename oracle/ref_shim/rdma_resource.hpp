// Stand-in for core/rdma_resource.hpp in a one-server harness: remote reads
// are never taken (global_num_servers == 1), and Mem is a plain host arena
// with the accessors core/gstore.hpp uses (core/mem.hpp keeps kvstore first).
#pragma once
#include <cstdint>
#include <cstdlib>
#include <cstring>
struct RDMA {
    struct Dev { int RdmaRead(int, int, char *, uint64_t, uint64_t) { return 0; } };
    Dev dev_;
    Dev *dev = &dev_;
    static RDMA &get_rdma() { static RDMA r; return r; }
};
class Mem {
    char *kvs_;
    uint64_t kvs_sz_;
    char *buf_;
public:
    explicit Mem(uint64_t kvs_sz) : kvs_sz_(kvs_sz) {
        kvs_ = (char *)calloc(kvs_sz, 1);
        buf_ = (char *)calloc(1 << 20, 1);
    }
    ~Mem() { free(kvs_); free(buf_); }
    char *kvstore() { return kvs_; }
    uint64_t kvstore_size() { return kvs_sz_; }
    char *buffer(int) { return buf_; }
};
