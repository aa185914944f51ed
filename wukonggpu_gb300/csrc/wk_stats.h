// Planner statistics shared by the statistics planner and the learned one.
#pragma once

#include <unordered_map>
#include <vector>

#include "wk_internal.h"

namespace wk {

struct FourNum {
    int64_t out_out = 0, out_in = 0, in_in = 0, in_out = 0;
};

// The reference's global_* maps after the one-server gather
// (core/data_statistic.hpp:41-52, :150-156).
struct Stats {
    int32_t num_ids = 0;
    std::unordered_map<int, int64_t> pt, ps, po, tys;
    std::vector<FourNum> pp;   // (num_ids+1)^2, index p1*(n+1)+p2
    FourNum &pair(int a, int b) { return pp[(size_t)a * (size_t)(num_ids + 1) + (size_t)b]; }
    const FourNum *pair_c(int a, int b) const {
        if (a < 0 || b < 0 || a > num_ids || b > num_ids) return nullptr;
        return &pp[(size_t)a * (size_t)(num_ids + 1) + (size_t)b];
    }
    double get(const std::unordered_map<int, int64_t> &m, int k) const {
        auto it = m.find(k);
        return it == m.end() ? 0.0 : (double)it->second;
    }
};

Stats &stats_of(wk_ctx *ctx);   // built on first use

}  // namespace wk
