// Seeded synthetic RDF graphs in ID form.
//
// Id encoding follows datagen/generate_data.cpp:88-98: ids below 2^17 are
// predicates and types (0 = predicate index, 1 = rdf:type), vertices start at
// 2^17.  Predicates take ids 2.. in group order, classes follow them.
//
// Every random draw comes from a counter-based stream keyed by
// (seed, predicate, subject), so the graph does not depend on the thread
// count, and all floating point is +,-,*,/ on doubles with contraction
// disabled (this file is compiled with -ffp-contract=off) so that x86_64 and
// aarch64 produce the same triples.
#include "wk_internal.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

namespace wk {

static inline uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(splitmix64(seed)) {}
    uint64_t next() { s += 0x9E3779B97F4A7C15ull; return splitmix64(s); }
    // uniform integer in [0, n) by multiply-shift
    uint64_t below(uint64_t n) { return (uint64_t)(((unsigned __int128)next() * n) >> 64); }
    // uniform double in [0, 1) from 53 bits
    double unit() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// ln(x) for x > 0: x = m * 2^e, m in [1,2), ln m by the atanh series.
static double det_log(double x) {
    int e = 0;
    double m = std::frexp(x, &e);   // m in [0.5, 1)
    m *= 2.0; e -= 1;               // m in [1, 2)
    double t = (m - 1.0) / (m + 1.0), t2 = t * t, term = t, sum = 0.0;
    for (int k = 1; k < 80; k += 2) { sum += term / (double)k; term *= t2; }
    return 2.0 * sum + (double)e * 0.69314718055994530942;
}

// exp(y): y = k ln2 + r with |r| <= ln2/2, Taylor series for exp(r).
static double det_exp(double y) {
    const double ln2 = 0.69314718055994530942;
    double kf = std::floor(y / ln2 + 0.5);
    double r = y - kf * ln2, term = 1.0, sum = 1.0;
    for (int k = 1; k < 30; ++k) { term = term * r / (double)k; sum += term; }
    return std::ldexp(sum, (int)kf);
}

struct ZipfTable {
    std::vector<double> cdf;   // cdf[k-1] = sum_{j<=k} j^-s
    double mean = 0.0;
    ZipfTable(double s, int cap) : cdf((size_t)cap) {
        double acc = 0.0, m = 0.0;
        for (int k = 1; k <= cap; ++k) {
            double w = det_exp(-s * det_log((double)k));
            acc += w; m += w * (double)k;
            cdf[(size_t)k - 1] = acc;
        }
        mean = m / acc;
    }
    int sample(Rng &r) const {
        double u = r.unit() * cdf.back();
        size_t k = (size_t)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
        if (k >= cdf.size()) k = cdf.size() - 1;
        return (int)k + 1;
    }
};

static uint64_t gcd_u64(uint64_t a, uint64_t b) { while (b) { uint64_t t = a % b; a = b; b = t; } return a; }

// affine bijection i -> (a*i + b) mod n
struct Affine {
    uint64_t a = 1, b = 0, n = 1;
    Affine() {}
    Affine(uint64_t seed, uint64_t n_) : n(n_) {
        Rng r(seed);
        a = 1 + r.below(n - 1 > 0 ? n - 1 : 1);
        while (gcd_u64(a, n) != 1) a = (a + 1) % n ? (a + 1) % n : 1;
        b = r.below(n);
    }
    uint64_t operator()(uint64_t i) const {
        return (uint64_t)(((unsigned __int128)a * i + b) % n);
    }
};

struct PredPlan {
    int32_t pid;
    int32_t kind;
    double q;
    const ZipfTable *zipf;
    Affine perm;   // functional: the bijection
};

}  // namespace wk

using namespace wk;

struct wk_graph {
    std::vector<int32_t> s, p, o;
    int32_t num_ids = 0;
    int32_t first_class = 0;
};

extern "C" int wk_graph_generate(const wk_graph_spec *spec, int32_t n_threads, wk_graph **out) {
    if (!spec || !out) return wk::set_error(WK_EINVAL, "wk_graph_generate: null argument");
    if (spec->n_entities <= 0 || spec->n_entities > (int64_t)INT32_MAX - WK_VID_BASE ||
        spec->n_classes < 0 || spec->n_groups < 0 || spec->n_groups > 4)
        return wk::set_error(WK_EINVAL, "wk_graph_generate: bad spec sizes");
    const uint64_t n = (uint64_t)spec->n_entities;
    const uint64_t seed = spec->seed;

    int32_t npred = 0;
    for (int g = 0; g < spec->n_groups; ++g) {
        const wk_pred_group &G = spec->groups[g];
        if (G.count < 0 || G.kind < 0 || G.kind > 2 || G.participation < 0.0 || G.participation > 1.0)
            return wk::set_error(WK_EINVAL, "wk_graph_generate: bad predicate group");
        if (G.kind == 0 && (G.zipf_cap < 1 || (uint64_t)G.zipf_cap > n))
            return wk::set_error(WK_EINVAL, "wk_graph_generate: bad zipf cap");
        npred += G.count;
    }
    const int32_t first_class = 2 + npred;
    const int32_t num_ids = first_class + spec->n_classes - 1;
    if (num_ids >= WK_VID_BASE) return wk::set_error(WK_EINVAL, "wk_graph_generate: too many ids");

    std::vector<ZipfTable *> tables;
    std::vector<PredPlan> plans;
    int32_t pid = 2;
    for (int g = 0; g < spec->n_groups; ++g) {
        const wk_pred_group &G = spec->groups[g];
        ZipfTable *zt = nullptr;
        if (G.kind == 0) { zt = new ZipfTable(G.zipf_s, G.zipf_cap); tables.push_back(zt); }
        for (int c = 0; c < G.count; ++c, ++pid) {
            PredPlan pp;
            pp.pid = pid; pp.kind = G.kind; pp.q = G.participation; pp.zipf = zt;
            if (G.kind == 1) pp.perm = Affine(seed ^ (0xF00Dull * (uint64_t)pid), n);
            plans.push_back(pp);
        }
    }
    // hub set shared by every many-to-one predicate
    double hub_frac = 0.01;
    for (int g = 0; g < spec->n_groups; ++g)
        if (spec->groups[g].kind == 2 && spec->groups[g].hub_frac > 0) hub_frac = spec->groups[g].hub_frac;
    uint64_t n_hub = (uint64_t)((double)n * hub_frac);
    if (n_hub < 1) n_hub = 1;
    Affine hub_perm(seed ^ 0x4B1Bull, n);

    // tasks: (plan index or -1 for type triples) x entity chunk
    const uint64_t CH = 1 << 16;
    const uint64_t nchunks = (n + CH - 1) / CH;
    const size_t ntasks = (plans.size() + 1) * nchunks;
    std::vector<std::vector<int32_t>> task_s(ntasks), task_o(ntasks);
    std::atomic<size_t> next{0};
    const uint64_t PMUL = 0xD6E8FEB86659FD93ull;

    auto worker = [&]() {
        std::vector<uint64_t> objs;
        for (;;) {
            size_t t = next.fetch_add(1);
            if (t >= ntasks) break;
            size_t pi = t / nchunks;          // 0 = type triples, else plans[pi-1]
            uint64_t c0 = (t % nchunks) * CH, c1 = std::min(n, c0 + CH);
            std::vector<int32_t> &S = task_s[t], &O = task_o[t];
            if (pi == 0) {
                if (spec->n_classes == 0) continue;
                S.reserve(c1 - c0); O.reserve(c1 - c0);
                for (uint64_t i = c0; i < c1; ++i) {
                    Rng r(seed ^ (i * PMUL) ^ 0x7E57ull);
                    S.push_back((int32_t)(WK_VID_BASE + i));
                    O.push_back(first_class + (int32_t)r.below((uint64_t)spec->n_classes));
                }
                continue;
            }
            const PredPlan &pp = plans[pi - 1];
            const uint64_t thr = pp.q >= 1.0 ? ~0ull : (uint64_t)(pp.q * 18446744073709551616.0);
            for (uint64_t i = c0; i < c1; ++i) {
                Rng r(seed ^ (i * PMUL) ^ ((uint64_t)pp.pid << 40) ^ 0xA5A5ull);
                if (pp.q < 1.0 && r.next() >= thr) continue;
                const int32_t sv = (int32_t)(WK_VID_BASE + i);
                if (pp.kind == 1) {
                    S.push_back(sv); O.push_back((int32_t)(WK_VID_BASE + pp.perm(i)));
                } else if (pp.kind == 2) {
                    S.push_back(sv);
                    O.push_back((int32_t)(WK_VID_BASE + hub_perm(r.below(n_hub))));
                } else {
                    int d = pp.zipf->sample(r);
                    objs.clear();
                    while ((int)objs.size() < d) {
                        while ((int)objs.size() < d) objs.push_back(r.below(n));
                        std::sort(objs.begin(), objs.end());
                        objs.erase(std::unique(objs.begin(), objs.end()), objs.end());
                    }
                    for (uint64_t x : objs) { S.push_back(sv); O.push_back((int32_t)(WK_VID_BASE + x)); }
                }
            }
        }
    };
    int nt = n_threads > 0 ? n_threads : (int)std::max(1u, std::thread::hardware_concurrency());
    std::vector<std::thread> th;
    for (int i = 1; i < nt; ++i) th.emplace_back(worker);
    worker();
    for (auto &x : th) x.join();
    for (auto *z : tables) delete z;

    size_t total = 0;
    for (auto &v : task_s) total += v.size();
    wk_graph *G = new (std::nothrow) wk_graph();
    if (!G) return wk::set_error(WK_ENOMEM, "wk_graph_generate: out of host memory");
    try {
        G->s.resize(total); G->p.resize(total); G->o.resize(total);
    } catch (...) { delete G; return wk::set_error(WK_ENOMEM, "wk_graph_generate: out of host memory"); }
    size_t at = 0;
    for (size_t t = 0; t < ntasks; ++t) {
        size_t pi = t / nchunks;
        int32_t p = pi == 0 ? WK_TYPE_ID : plans[pi - 1].pid;
        size_t m = task_s[t].size();
        if (!m) continue;
        std::memcpy(&G->s[at], task_s[t].data(), m * 4);
        std::memcpy(&G->o[at], task_o[t].data(), m * 4);
        std::fill(G->p.begin() + at, G->p.begin() + at + m, p);
        at += m;
        std::vector<int32_t>().swap(task_s[t]);
        std::vector<int32_t>().swap(task_o[t]);
    }
    G->num_ids = num_ids;
    G->first_class = first_class;
    *out = G;
    return WK_OK;
}

extern "C" int64_t wk_graph_size(const wk_graph *g) { return g ? (int64_t)g->s.size() : 0; }
extern "C" int32_t wk_graph_num_ids(const wk_graph *g) { return g ? g->num_ids : 0; }
extern "C" int32_t wk_graph_first_class(const wk_graph *g) { return g ? g->first_class : 0; }
extern "C" const int32_t *wk_graph_s(const wk_graph *g) { return g ? g->s.data() : nullptr; }
extern "C" const int32_t *wk_graph_p(const wk_graph *g) { return g ? g->p.data() : nullptr; }
extern "C" const int32_t *wk_graph_o(const wk_graph *g) { return g ? g->o.data() : nullptr; }
extern "C" void wk_graph_free(wk_graph *g) { delete g; }
