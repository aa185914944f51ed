#pragma once
#include <unordered_map>
namespace tbb { template <class K, class V> using concurrent_unordered_map = std::unordered_map<K, V>; }
