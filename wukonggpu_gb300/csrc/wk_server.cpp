// Request loop: admission, continuous batching, overlap, latency accounting.
//
// Requests carry a scheduled arrival time (seconds after wk_server_start):
// the loop sees a request only once the server clock has passed it, which is
// how an open-loop arrival process is replayed.  Two modes:
//
//   mode 0  query-at-a-time: one worker runs every arrived request through
//           wk_execute in arrival order, one query on the GPU at a time (the
//           reference's GPU engine discipline, core/gpu.hpp:49-61).
//   mode 1  serving: light requests (constant start, <= max_steps patterns)
//           are packed into batches as they arrive.  Two batch objects, each
//           on its own stream, alternate: while one batch runs, the next is
//           formed from whatever has arrived and launched as soon as a batch
//           object is free, and finished batches are unpacked while the
//           device works (continuous batching at batch granularity).  A batch
//           admits requests in arrival order while the sum of their projected
//           history bytes stays within the light budget and slots remain.
//           Heavy requests (index start or longer) run on worker contexts
//           that share the store and have their own streams, so they overlap
//           the light batches on the device.  A batch that overflows its
//           capacity is re-run one request at a time.
//
// Planning (plan = 1): each request is planned at submission by the
// statistics planner (wk_plan); a request the statistics prove empty is
// completed with zero rows without device work.  A request whose plan comes
// back empty runs as written.
//
// Projected bytes of a request: along its patterns, rows grow by the average
// degree of (predicate, direction) -- triples/subjects for OUT,
// triples/objects for IN -- and each step's table is rows x columns x 4.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "wk_runtime.h"

extern "C" {
struct wk_batch;
int wk_batch_create(wk_ctx *, int32_t, int32_t, int64_t, wk_batch **);
int wk_batch_destroy(wk_batch *);
int wk_batch_launch(wk_batch *, const int64_t *, const int32_t *, int32_t, int32_t);
int wk_batch_ready(wk_batch *);
int wk_batch_wait(wk_batch *);
int wk_batch_result(wk_batch *, int32_t, int64_t *, int32_t *, int64_t *);
int wk_batch_download(wk_batch *, int32_t *, int64_t, int64_t *);
}

namespace {

using clk = std::chrono::steady_clock;

struct Req {
    int64_t id = 0;
    std::vector<int64_t> cmd;
    int npat = 0;
    double arrival = 0.0;
    bool heavy = false;      // the request's class, by shape (the same in both modes)
    int32_t type = -1;       // the template it was made from (wk_server_submit_typed)
    double proj_bytes = 0.0;
    // 0 waiting, 1 running, 2 done, 3 failed, 4 refused at admission, 5 cancelled
    std::atomic<int> state{0};
    int status = 0;
    std::vector<int32_t> result;
    int64_t rows = 0;
    int32_t cols = 0;
    double done_t = 0.0;
};

// Latency at rate q of a sorted sample by the reference Logger's rule
// (core/logger.hpp:197-305): element floor(n q), the last one for q = 1.
double rank_at(const std::vector<double> &sorted, double q) {
    if (sorted.empty()) return 0.0;
    size_t i = (size_t)((double)sorted.size() * q);
    if (i >= sorted.size()) i = sorted.size() - 1;
    return sorted[i];
}

double pct(std::vector<double> v, double q) {
    std::sort(v.begin(), v.end());
    return rank_at(v, q);
}

// The Logger's 25 CDF rates: 0.01, 0.05 .. 0.95 by 0.05, 0.96 .. 1.00 by 0.01
// (core/logger.hpp print_cdf).
double cdf_rate(int k) { return k == 0 ? 0.01 : (k < 20 ? 0.05 * k : 0.95 + 0.01 * (k - 19)); }

}  // namespace

struct wk_server {
    wk_ctx *ctx = nullptr;
    wk_server_config cfg{};
    std::vector<wk_ctx *> workers;      // heavy workers (mode 1) / the single worker (mode 0)
    wk_ctx *solo = nullptr;             // overflow re-runs of light requests
    wk_batch *batch[2] = {nullptr, nullptr};
    int32_t *h_res = nullptr;           // pinned download buffer of a batch
    std::deque<std::unique_ptr<Req>> all;
    std::deque<Req *> light_q;          // light requests waiting for a batch (mode 1)
    std::deque<Req *> single_q;         // requests the workers run one at a time
    std::mutex mu;
    std::condition_variable cv;
    std::vector<std::thread> threads;
    clk::time_point t0;
    std::atomic<bool> started{false}, stopping{false};
    std::atomic<int64_t> done_count{0}, failed{0}, batches{0}, batched_reqs{0}, device_launches{0};
    std::atomic<int64_t> rejected{0}, cancelled{0};
    int64_t submitted = 0;

    double now() const { return std::chrono::duration<double>(clk::now() - t0).count(); }
};

namespace {

void finish(wk_server *s, Req *r, int status) {
    r->status = status;
    r->done_t = s->now();
    r->state.store(status == WK_OK ? 2 : 3);
    if (status != WK_OK) s->failed++;
    s->done_count++;
    s->cv.notify_all();
}

// run one request alone on `ctx` (wk_execute + download)
void run_single(wk_server *s, wk_ctx *ctx, Req *r) {
    wk_history h;
    wk_history_init(&h);
    int st = wk_execute(ctx, r->cmd.data(), r->npat, &h, nullptr);
    if (st == WK_OK) {
        r->rows = h.col_num ? h.size / h.col_num : 0;
        r->cols = h.col_num;
        if (s->cfg.keep_results) {
            r->result.resize((size_t)h.size);
            st = wk_history_download(ctx, &h, r->result.data(), h.size);
        } else {
            st = wk_sync(ctx);
        }
    }
    finish(s, r, st);
}

// next arrived request of queue q (caller holds the lock)
Req *pop_arrived(wk_server *s, std::deque<Req *> &q, double t) {
    if (q.empty() || q.front()->arrival > t) return nullptr;
    Req *r = q.front();
    q.pop_front();
    return r;
}

void single_loop(wk_server *s, wk_ctx *ctx, std::deque<Req *> *q) {
    while (!s->stopping.load()) {
        Req *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            r = pop_arrived(s, *q, s->now());
            if (!r) {
                const double wait = q->empty() ? 1e-3 : std::max(0.0, q->front()->arrival - s->now());
                s->cv.wait_for(lk, std::chrono::duration<double>(std::min(wait, 1e-3)));
                continue;
            }
        }
        r->state.store(1);
        run_single(s, ctx, r);
    }
}

struct InFlight {
    std::vector<Req *> reqs;
    bool busy = false;
};

void unpack(wk_server *s, int i, InFlight &f) {
    wk_batch *b = s->batch[i];
    int st = wk_batch_wait(b);
    if (st == WK_EOVERFLOW) {
        for (Req *r : f.reqs) run_single(s, s->solo, r);   // one at a time
        f.reqs.clear();
        f.busy = false;
        return;
    }
    int64_t tot = 0;
    if (st == WK_OK && s->cfg.keep_results) st = wk_batch_download(b, s->h_res, s->cfg.batch_capacity_ints, &tot);
    for (size_t k = 0; k < f.reqs.size(); ++k) {
        Req *r = f.reqs[k];
        if (st == WK_OK) {
            int64_t rows = 0, off = 0;
            int32_t cols = 0;
            wk_batch_result(b, (int32_t)k, &rows, &cols, &off);
            r->rows = rows;
            r->cols = cols;
            if (s->cfg.keep_results) r->result.assign(s->h_res + off, s->h_res + off + rows * cols);
        }
        finish(s, r, st);
    }
    f.reqs.clear();
    f.busy = false;
}

void batch_loop(wk_server *s) {
    InFlight inflight[2];
    std::vector<int64_t> cmd;
    std::vector<int32_t> npat;
    const double budget = (double)s->cfg.light_budget_bytes;
    const double window = 1e-6 * (double)std::max(0, s->cfg.batch_window_us);
    while (true) {
        // retire finished batches
        for (int i = 0; i < 2; ++i)
            if (inflight[i].busy && wk_batch_ready(s->batch[i])) unpack(s, i, inflight[i]);
        const bool idle = !inflight[0].busy && !inflight[1].busy;
        if (s->stopping.load() && idle) break;
        int freeb = !inflight[0].busy ? 0 : (!inflight[1].busy ? 1 : -1);
        std::vector<Req *> take;
        if (freeb >= 0) {
            std::lock_guard<std::mutex> lk(s->mu);
            const double t = s->now();
            // the batching window: wait for more arrivals while the oldest
            // request has waited less than the window and the batch is not full
            bool ready = !s->light_q.empty() && s->light_q.front()->arrival <= t;
            if (ready && window > 0.0 && t - s->light_q.front()->arrival < window) {
                double pb = 0.0;
                int n = 0;
                for (Req *r : s->light_q) {
                    if (r->arrival > t || n >= s->cfg.max_batch) break;
                    pb += r->proj_bytes;
                    ++n;
                }
                ready = n >= s->cfg.max_batch || pb > budget;
            }
            double bytes = 0.0;
            while (ready && !s->light_q.empty() && (int)take.size() < s->cfg.max_batch) {
                Req *r = s->light_q.front();
                if (r->arrival > t) break;
                if (!take.empty() && bytes + r->proj_bytes > budget) break;
                bytes += r->proj_bytes;
                take.push_back(r);
                s->light_q.pop_front();
            }
        }
        if (!take.empty()) {
            cmd.clear();
            npat.clear();
            for (Req *r : take) {
                r->state.store(1);
                cmd.insert(cmd.end(), r->cmd.begin(), r->cmd.end());
                npat.push_back(r->npat);
            }
            int st = wk_batch_launch(s->batch[freeb], cmd.data(), npat.data(), (int32_t)take.size(), 1);
            if (st != WK_OK) {
                for (Req *r : take) finish(s, r, st);
                continue;
            }
            inflight[freeb].reqs = std::move(take);
            inflight[freeb].busy = true;
            s->batches++;
            s->batched_reqs += (int64_t)inflight[freeb].reqs.size();
            continue;
        }
        // nothing to launch: sleep until the next arrival (at most 1 ms when
        // idle, 20 us while a batch runs) rather than polling the device,
        // which would contend for the driver with the heavy workers
        std::unique_lock<std::mutex> lk(s->mu);
        double wait = idle ? 1e-3 : 2e-5;
        if (!s->light_q.empty()) {
            const double a0 = s->light_q.front()->arrival, t = s->now();
            const double next = a0 <= t ? a0 + window : a0;   // window end, or the next arrival
            wait = std::min(wait, std::max(0.0, next - t));
        }
        if (wait > 0) s->cv.wait_for(lk, std::chrono::duration<double>(wait));
    }
}

double projected_bytes(wk_ctx *ctx, const std::vector<int64_t> &cmd, int n) {
    const wk::HostStore &hs = *ctx->store->hs;
    double rows = 1.0, bytes = 0.0;
    int cols = 0;
    for (int i = 0; i < n; ++i) {
        const int64_t st = cmd[4 * i], p = cmd[4 * i + 1], d = cmd[4 * i + 2], en = cmd[4 * i + 3];
        double deg = 1.0;
        if (i == 0 && st > 1 && st < WK_VID_BASE) {
            const wk::PredSeg &sg = hs.segs[(size_t)st];   // index: its list length
            deg = (double)(sg.subjects > 0 ? sg.subjects : 1);
            rows = deg;
            cols = 1;
            bytes += rows * 4.0;
            continue;
        }
        if (p >= 1 && p <= hs.num_ids) {
            const wk::PredSeg &sg = hs.segs[(size_t)p];
            const double denom = (double)(d == WK_DIR_OUT ? sg.subjects : sg.objects);
            deg = denom > 0 ? (double)sg.triples / denom : 0.0;
        }
        const bool expands = en < 0 && -en > cols;
        if (expands) { rows *= deg; ++cols; }
        else rows *= std::min(1.0, deg);
        bytes += rows * 4.0 * (double)std::max(cols, 1);
    }
    return bytes;
}

// the batch accepts: `<const> p d -1` or an index start first, then k2u
// binding the next column, k2k, or k2c (mirrors fill_desc in wk_batch.cu)
bool batch_compatible(const std::vector<int64_t> &cmd, int n, int max_steps, int num_ids) {
    if (n < 1 || n > max_steps || cmd[3] != -1) return false;
    const bool index_start = cmd[0] > 1 && cmd[0] < WK_VID_BASE && cmd[0] <= num_ids &&
                             ((cmd[1] == WK_TYPE_ID && cmd[2] == WK_DIR_IN) ||
                              (cmd[1] == WK_PREDICATE_ID && (cmd[2] == 0 || cmd[2] == 1)));
    if (!index_start && (cmd[0] < WK_VID_BASE || cmd[0] > 0x7fffffffll)) return false;
    int col = 1;
    for (int i = 1; i < n; ++i) {
        const int64_t st = cmd[4 * i], en = cmd[4 * i + 3];
        if (!(st < 0 && -st <= col)) return false;
        if (en < 0 && -en > col) {
            if (-en - 1 != col) return false;
            ++col;
        } else if (en > 0x7fffffffll) {
            return false;
        }
    }
    return true;
}

void stop_threads(wk_server *s) {
    s->stopping.store(true);
    s->cv.notify_all();
    for (auto &t : s->threads)
        if (t.joinable()) t.join();
    s->threads.clear();
}

}  // namespace

using namespace wk;

// Worker contexts reserve their per-op scratch for steps of this many input
// rows up front: growing a buffer later frees the old one, and cudaFree
// synchronises the device, stalling the light batches.
constexpr int64_t kWorkerRows = 16ll << 20;

extern "C" void wk_server_config_default(wk_server_config *c) {
    if (!c) return;
    std::memset(c, 0, sizeof(*c));
    c->mode = 1;
    c->max_batch = 4096;
    c->max_steps = 4;
    c->heavy_workers = 1;
    c->batch_capacity_ints = 1ll << 26;
    c->light_budget_bytes = 1ll << 27;
    c->plan = 1;
    c->keep_results = 1;
}

extern "C" int wk_server_create(wk_ctx *ctx, const wk_server_config *cfg, wk_server **out) {
    if (!ctx || !cfg || !out) return set_error(WK_EINVAL, "wk_server_create: null");
    if (!ctx->store) return set_error(WK_ENOSTORE, "wk_server_create: no store built");
    if (ctx->device < 0) return set_error(WK_EDEVICE, "wk_server_create: host-only context");
    if (cfg->mode < 0 || cfg->mode > 1 || cfg->max_batch < 1 || cfg->max_steps < 1 || cfg->heavy_workers < 0 ||
        cfg->heavy_workers > 8 || cfg->batch_capacity_ints < 1)
        return set_error(WK_EINVAL, "wk_server_create: bad configuration");
    wk_server *s = new wk_server();
    s->ctx = ctx;
    s->cfg = *cfg;
    const int nworkers = cfg->mode == 0 ? 1 : std::max(1, cfg->heavy_workers);
    int st = WK_OK;
    for (int i = 0; i < nworkers && st == WK_OK; ++i) {
        wk_config wc;
        wk_config_default(&wc);
        wc.device = ctx->device;
        wk_ctx *w = nullptr;
        if ((st = wk_ctx_create(&wc, &w)) == WK_OK && (st = wk_ctx_share_store(w, ctx)) == WK_OK &&
            (st = wk::reserve_op_scratch(w, kWorkerRows)) == WK_OK)
            s->workers.push_back(w);
        else if (w) wk_ctx_destroy(w);
    }
    if (st == WK_OK && cfg->mode == 1) {
        wk_config wc;
        wk_config_default(&wc);
        wc.device = ctx->device;
        if ((st = wk_ctx_create(&wc, &s->solo)) == WK_OK) st = wk_ctx_share_store(s->solo, ctx);
        for (int i = 0; i < 2 && st == WK_OK; ++i)
            st = wk_batch_create(ctx, cfg->max_batch, cfg->max_steps, cfg->batch_capacity_ints, &s->batch[i]);
        if (st == WK_OK && cfg->keep_results &&
            cudaHostAlloc((void **)&s->h_res, 4 * (size_t)cfg->batch_capacity_ints, 0) != cudaSuccess) {
            cudaGetLastError();
            st = set_error(WK_ENOMEM, "wk_server_create: pinned result buffer");
        }
    }
    if (st != WK_OK) {
        wk_server_destroy(s);
        return st;
    }
    *out = s;
    return WK_OK;
}

extern "C" int64_t wk_server_submit(wk_server *s, const int64_t *cmd, int32_t npat, double arrival_s) {
    return wk_server_submit_typed(s, cmd, npat, arrival_s, -1);
}

extern "C" int64_t wk_server_submit_typed(wk_server *s, const int64_t *cmd, int32_t npat, double arrival_s,
                                          int32_t type) {
    if (!s || !cmd || npat < 1 || npat > 16) return set_error(WK_EINVAL, "wk_server_submit: bad arguments");
    std::unique_ptr<Req> r(new Req());
    r->cmd.assign(cmd, cmd + (size_t)npat * 4);
    r->npat = npat;
    r->arrival = arrival_s;
    r->type = type;
    bool empty = false;
    if (s->cfg.plan) {
        std::vector<int64_t> out((size_t)(npat + 2) * 4);
        int32_t nout = npat + 2, pe = 0;
        double cost = 0;
        if (wk_plan(s->ctx, r->cmd.data(), npat, out.data(), &nout, &cost, &pe) == WK_OK) {
            if (pe) empty = true;
            else if (nout > 0) {
                r->cmd.assign(out.begin(), out.begin() + (size_t)nout * 4);
                r->npat = nout;
            }
        }
    }
    // the class, by shape in both modes: light is a constant start the batch
    // accepts, heavy everything else (index starts, longer queries); where it
    // runs is separate -- mode 0 runs every request on the single worker
    r->heavy = r->cmd[0] < WK_VID_BASE ||
               !batch_compatible(r->cmd, r->npat, s->cfg.max_steps, s->ctx->store->hs->num_ids);
    r->proj_bytes = projected_bytes(s->ctx, r->cmd, r->npat);
    // admission by projected history bytes: a request over the cap is refused
    const bool refuse = s->cfg.max_request_bytes > 0 && r->proj_bytes > (double)s->cfg.max_request_bytes;
    Req *raw = r.get();
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = (int64_t)s->all.size();
    s->all.push_back(std::move(r));
    s->submitted++;
    if (refuse) {
        raw->status = WK_EREJECTED;
        raw->done_t = raw->arrival;
        raw->state.store(4);
        s->rejected++;
        s->done_count++;
        return raw->id;
    }
    if (empty) {
        raw->rows = 0;
        raw->cols = 0;
        raw->state.store(1);
        raw->done_t = raw->arrival;   // answered from the statistics at arrival
        raw->state.store(2);
        s->done_count++;
        return raw->id;
    }
    auto &q = (s->cfg.mode == 0 || raw->heavy) ? s->single_q : s->light_q;
    auto it = std::upper_bound(q.begin(), q.end(), raw, [](Req *a, Req *b) { return a->arrival < b->arrival; });
    q.insert(it, raw);
    s->cv.notify_all();
    return raw->id;
}

extern "C" int wk_server_start(wk_server *s) {
    if (!s) return set_error(WK_EINVAL, "wk_server_start: null");
    if (s->started.exchange(true)) return set_error(WK_EINVAL, "wk_server_start: already started");
    s->t0 = clk::now();
    if (s->cfg.mode == 0) {
        s->threads.emplace_back(single_loop, s, s->workers[0], &s->single_q);
    } else {
        s->threads.emplace_back(batch_loop, s);
        for (wk_ctx *w : s->workers) s->threads.emplace_back(single_loop, s, w, &s->single_q);
    }
    return WK_OK;
}

extern "C" int wk_server_drain(wk_server *s, double timeout_s) {
    if (!s) return set_error(WK_EINVAL, "wk_server_drain: null");
    std::unique_lock<std::mutex> lk(s->mu);
    const auto dl = clk::now() + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(timeout_s));
    while (s->done_count.load() < s->submitted) {
        if (s->cv.wait_until(lk, dl) == std::cv_status::timeout && s->done_count.load() < s->submitted)
            return set_error(WK_ETIMEDOUT, "wk_server_drain: %lld of %lld requests done",
                             (long long)s->done_count.load(), (long long)s->submitted);
    }
    return WK_OK;
}

extern "C" int wk_server_result(wk_server *s, int64_t id, int64_t *rows, int32_t *cols, int32_t *host, int64_t cap,
                                double *latency_s, int32_t *status) {
    if (!s || !rows || !cols) return set_error(WK_EINVAL, "wk_server_result: null");
    Req *r;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (id < 0 || id >= (int64_t)s->all.size()) return set_error(WK_EINVAL, "wk_server_result: id %lld", (long long)id);
        r = s->all[(size_t)id].get();
    }
    const int stt = r->state.load();
    if (stt < 2) return set_error(WK_EINVAL, "wk_server_result: request %lld not finished", (long long)id);
    *rows = r->rows;
    *cols = r->cols;
    if (latency_s) *latency_s = r->done_t - r->arrival;
    if (status) *status = r->status;
    if (host) {
        if (cap < (int64_t)r->result.size()) return set_error(WK_EOVERFLOW, "wk_server_result: room for %lld", (long long)cap);
        std::memcpy(host, r->result.data(), r->result.size() * 4);
    }
    return WK_OK;
}

extern "C" int wk_server_get_stats(wk_server *s, wk_server_stats *out) {
    if (!s || !out) return set_error(WK_EINVAL, "wk_server_get_stats: null");
    std::memset(out, 0, sizeof(*out));
    std::vector<double> all, light, heavy;
    double first = 1e300, last = 0.0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &r : s->all) {
            const int stt = r->state.load();
            if (stt != 2 && stt != 3) continue;   // waiting, running, refused or cancelled
            const double lat = r->done_t - r->arrival;
            all.push_back(lat);
            (r->heavy ? heavy : light).push_back(lat);
            first = std::min(first, r->arrival);
            last = std::max(last, r->done_t);
        }
    }
    out->completed = (int64_t)all.size();
    out->light = (int64_t)light.size();
    out->heavy = (int64_t)heavy.size();
    out->failed = s->failed.load();
    out->batches = s->batches.load();
    out->mean_batch = s->batches.load() ? (double)s->batched_reqs.load() / (double)s->batches.load() : 0.0;
    out->span_s = all.empty() ? 0.0 : last - first;
    out->qps = out->span_s > 0 ? (double)all.size() / out->span_s : 0.0;
    out->p50_ms = pct(all, 0.50) * 1e3;
    out->p99_ms = pct(all, 0.99) * 1e3;
    out->light_p50_ms = pct(light, 0.50) * 1e3;
    out->light_p99_ms = pct(light, 0.99) * 1e3;
    out->heavy_p50_ms = pct(heavy, 0.50) * 1e3;
    out->heavy_p99_ms = pct(heavy, 0.99) * 1e3;
    out->rejected = s->rejected.load();
    out->cancelled = s->cancelled.load();
    return WK_OK;
}

extern "C" int wk_server_type_stats(wk_server *s, int32_t type, wk_type_stats *out) {
    if (!s || !out) return set_error(WK_EINVAL, "wk_server_type_stats: null");
    std::memset(out, 0, sizeof(*out));
    std::vector<double> v;
    double first = 1e300, last = 0.0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &r : s->all) {
            const int stt = r->state.load();
            if (stt != 2 && stt != 3) continue;
            first = std::min(first, r->arrival);
            last = std::max(last, r->done_t);
            if (r->type != type) continue;
            v.push_back(r->done_t - r->arrival);
            if (stt == 3) out->failed++;
        }
    }
    std::sort(v.begin(), v.end());
    out->completed = (int64_t)v.size();
    out->qps = last > first ? (double)v.size() / (last - first) : 0.0;
    out->p50_ms = rank_at(v, 0.50) * 1e3;
    out->p99_ms = rank_at(v, 0.99) * 1e3;
    for (int k = 0; k < WK_CDF_POINTS; ++k) out->cdf_ms[k] = rank_at(v, cdf_rate(k)) * 1e3;
    return WK_OK;
}

extern "C" int wk_server_cancel(wk_server *s, int64_t id) {
    if (!s) return set_error(WK_EINVAL, "wk_server_cancel: null");
    std::lock_guard<std::mutex> lk(s->mu);
    if (id < 0 || id >= (int64_t)s->all.size()) return set_error(WK_EINVAL, "wk_server_cancel: id %lld", (long long)id);
    Req *r = s->all[(size_t)id].get();
    // a request still in a queue has not started: the loops take requests
    // out of their queue under this lock before they run them
    for (std::deque<Req *> *q : {&s->light_q, &s->single_q}) {
        auto it = std::find(q->begin(), q->end(), r);
        if (it == q->end()) continue;
        q->erase(it);
        r->status = WK_ECANCELED;
        r->done_t = s->started.load() ? s->now() : r->arrival;
        r->state.store(5);
        s->cancelled++;
        s->done_count++;
        s->cv.notify_all();
        return WK_OK;
    }
    return set_error(WK_EINVAL, "wk_server_cancel: request %lld is running or finished", (long long)id);
}

extern "C" int wk_server_inject_alloc_failure(wk_server *s, int32_t worker, int32_t n) {
    if (!s || n < 0 || worker < -1 || worker >= (int32_t)s->workers.size())
        return set_error(WK_EINVAL, "wk_server_inject_alloc_failure: bad arguments");
    wk_ctx *c = worker < 0 ? s->solo : s->workers[(size_t)worker];
    if (!c) return set_error(WK_EINVAL, "wk_server_inject_alloc_failure: no such context in this mode");
    return wk_ctx_inject_alloc_failure(c, n);
}

extern "C" int wk_server_latency_cdf(wk_server *s, int32_t cls, double *out_ms) {
    if (!s || !out_ms || cls < 0 || cls > 2) return set_error(WK_EINVAL, "wk_server_latency_cdf: bad arguments");
    std::vector<double> v;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto &r : s->all) {
            const int stt = r->state.load();
            if (stt != 2 && stt != 3) continue;
            if (cls == 1 && r->heavy) continue;
            if (cls == 2 && !r->heavy) continue;
            v.push_back(r->done_t - r->arrival);
        }
    }
    std::sort(v.begin(), v.end());
    for (int k = 0; k < WK_CDF_POINTS; ++k) out_ms[k] = rank_at(v, cdf_rate(k)) * 1e3;
    return WK_OK;
}

extern "C" int wk_server_destroy(wk_server *s) {
    if (!s) return WK_OK;
    stop_threads(s);
    for (int i = 0; i < 2; ++i)
        if (s->batch[i]) wk_batch_destroy(s->batch[i]);
    if (s->h_res) cudaFreeHost(s->h_res);
    if (s->solo) wk_ctx_destroy(s->solo);
    for (wk_ctx *w : s->workers) wk_ctx_destroy(w);
    delete s;
    return WK_OK;
}
