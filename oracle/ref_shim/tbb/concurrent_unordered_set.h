#pragma once
#include <unordered_set>
namespace tbb { template <class K> using concurrent_unordered_set = std::unordered_set<K>; }
