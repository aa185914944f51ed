/*
 * wk_rcache_binding.hpp -- the reference-side binding of this library.
 *
 * A replacement for the reference's RCache (core/rcache.hpp:73-963) that keeps
 * the four per-pattern member functions GPU_Engine calls
 * (core/gpu_engine.hpp:208, :231, :254, :280) and forwards them to the C ABI
 * of wukong_gpu.h.  A maintainer includes it in the reference's tree in place
 * of core/rcache.hpp, after core/query.hpp (request_or_reply) and
 * core/config.hpp (the global_gpu_* knobs), and links libwkgpu.so.
 *
 * request_or_reply keeps its fields: the library's wk_history mirrors
 * gpu_history_ptr / gpu_history_table_size / col_num (core/query.hpp:63-65).
 * A step that is not the query's last leaves the new table on the device for
 * the next step (core/rcache.hpp:389-400); the last one is brought home
 * (core/rcache.hpp:402-408).  Errors become exceptions carrying
 * wk_last_error() where the reference asserts.
 */
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "wukong_gpu.h"

class RCache {
    wk_ctx *ctx_ = nullptr;

    static void check(int st) {
        if (st != WK_OK) throw std::runtime_error(std::string(wk_status_str(st)) + ": " + wk_last_error());
    }

    static wk_history hist_of(request_or_reply &req) {
        wk_history h;
        wk_history_init(&h);
        h.data = reinterpret_cast<int32_t *>(req.gpu_history_ptr);
        h.size = req.gpu_history_table_size;
        h.col_num = req.get_col_num();
        h.step = req.step;
        return h;
    }

    std::vector<int> finish(request_or_reply &req, wk_history &h) {
        if (!req.is_last_handler()) {
            req.gpu_history_ptr = reinterpret_cast<char *>(h.data);
            req.gpu_history_table_size = static_cast<int>(h.size);
            return {};
        }
        std::vector<int> out(static_cast<size_t>(h.size));
        check(wk_history_download(ctx_, &h, out.data(), h.size));
        req.gpu_history_ptr = nullptr;
        req.gpu_history_table_size = 0;
        return out;
    }

public:
    /* devid: the CUDA device (-1 gives a host-only context, whose ops all
     * fail with WK_EDEVICE); s/p/o: the loader's ID triples. */
    RCache(int devid, const int32_t *s, const int32_t *p, const int32_t *o, int64_t n, int num_ids) {
        wk_config cfg;
        wk_config_default(&cfg);
        cfg.device = devid;
        cfg.cache_budget_mb = global_gpu_memstore_size_gb * 1024;   // the store's device budget
        cfg.enable_prefetch = global_gpu_enable_pipeline;
        check(wk_ctx_create(&cfg, &ctx_));
        const int st = wk_store_build(ctx_, s, p, o, n, num_ids);
        if (st != WK_OK) {
            const std::string msg = std::string(wk_status_str(st)) + ": " + wk_last_error();
            wk_ctx_destroy(ctx_);
            throw std::runtime_error(msg);
        }
    }
    RCache(const RCache &) = delete;
    RCache &operator=(const RCache &) = delete;
    ~RCache() { wk_ctx_destroy(ctx_); }

    /* GPU::load_history_data (core/gpu.hpp:79-88) */
    void load_history(request_or_reply &req, const int32_t *host, int64_t size) {
        wk_history h = hist_of(req);
        check(wk_history_upload(ctx_, &h, host, size, req.get_col_num()));
        req.gpu_history_ptr = reinterpret_cast<char *>(h.data);
        req.gpu_history_table_size = static_cast<int>(h.size);
    }

    std::vector<int> known_to_unknown(request_or_reply &req, int start, int direction, int predict) {
        wk_history h = hist_of(req);
        check(wk_known_to_unknown(ctx_, &h, start, direction, predict));
        return finish(req, h);
    }
    std::vector<int> known_to_known(request_or_reply &req, int start, int direction, int predict, int end) {
        wk_history h = hist_of(req);
        check(wk_known_to_known(ctx_, &h, start, direction, predict, end));
        return finish(req, h);
    }
    std::vector<int> known_to_const(request_or_reply &req, int start, int direction, int predict, int end) {
        wk_history h = hist_of(req);
        check(wk_known_to_const(ctx_, &h, start, direction, predict, end));
        return finish(req, h);
    }
    std::vector<int> index_to_unknown(request_or_reply &req, int index_vertex, int direction) {
        wk_history h = hist_of(req);
        h.col_num = 0;
        check(wk_index_to_unknown(ctx_, &h, index_vertex, direction));
        return finish(req, h);
    }
};
