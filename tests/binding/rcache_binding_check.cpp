// Compiles the reference-side binding (include/wk_rcache_binding.hpp) against
// the reference's own request_or_reply (core/query.hpp) and config globals
// (core/config.hpp), links libwkgpu.so, and drives it on a host-only context:
// the store builds, a history loads, and every op reports the host-only
// context as an exception.  Test infrastructure: built and run by
// tests/test_binding.py, never shipped.
#include <cstdio>
#include <exception>
#include <vector>

#include "query.hpp"
#include "wk_rcache_binding.hpp"

static int expect_throw(const char *what, void (*f)(RCache &, request_or_reply &), RCache &rc,
                        request_or_reply &req) {
    try {
        f(rc, req);
    } catch (const std::exception &e) {
        std::printf("%s threw: %s\n", what, e.what());
        return 0;
    }
    std::printf("%s did not throw\n", what);
    return 1;
}

int main() {
    const int32_t base = 1 << 17;
    // <v0 p2 v1> <v1 p2 v2> <v0 type C> with C = id 3
    std::vector<int32_t> s{base, base + 1, base}, p{2, 2, 1}, o{base + 1, base + 2, 3};
    global_gpu_memstore_size_gb = 0;   // whole store resident
    RCache rc(-1, s.data(), p.data(), o.data(), (int64_t)s.size(), 3);
    request_or_reply req;
    req.cmd_chains = {base, 2, 1, -1, -1, 2, 1, -2};
    req.step = 1;
    req.col_num = 1;
    const int32_t hist[2] = {base, base + 1};
    int bad = 0;
    try {
        rc.load_history(req, hist, 2);
        std::printf("history loaded\n");
    } catch (const std::exception &e) {
        std::printf("load_history threw: %s\n", e.what());
    }
    bad += expect_throw("known_to_unknown", [](RCache &r, request_or_reply &q) { r.known_to_unknown(q, -1, 1, 2); },
                        rc, req);
    bad += expect_throw("known_to_known", [](RCache &r, request_or_reply &q) { r.known_to_known(q, -1, 1, 2, -1); },
                        rc, req);
    bad += expect_throw("known_to_const", [](RCache &r, request_or_reply &q) { r.known_to_const(q, -1, 1, 2, base); },
                        rc, req);
    bad += expect_throw("index_to_unknown", [](RCache &r, request_or_reply &q) { r.index_to_unknown(q, 2, 0); }, rc,
                        req);
    std::printf("binding check %s\n", bad ? "FAILED" : "done");
    return bad;
}
