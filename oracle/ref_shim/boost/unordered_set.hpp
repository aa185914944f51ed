#pragma once
#include <unordered_set>
namespace boost { template <class K, class H = std::hash<K>> using unordered_set = std::unordered_set<K, H>; }
