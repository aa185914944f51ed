// Stand-in for the tbb::concurrent_hash_map API used by core/gstore.hpp:
// insert(accessor&, key), accessor->second, range-for, swap, size, empty.
// An accessor holds the map's mutex while bound, which serialises the
// reference's concurrent push_backs exactly as TBB's element lock does.
#pragma once
#include <map>
#include <mutex>
#include <memory>
namespace tbb {
template <class K, class V>
class concurrent_hash_map {
    std::map<K, V> m_;
    std::unique_ptr<std::recursive_mutex> mu_{new std::recursive_mutex};
public:
    typedef std::pair<const K, V> value_type;
    class accessor {
        friend class concurrent_hash_map;
        value_type *p_ = nullptr;
        std::unique_lock<std::recursive_mutex> lk_;
    public:
        value_type *operator->() const { return p_; }
        value_type &operator*() const { return *p_; }
    };
    bool insert(accessor &a, const K &k) {
        a.lk_ = std::unique_lock<std::recursive_mutex>(*mu_);
        auto r = m_.emplace(k, V());
        a.p_ = &*r.first;
        return r.second;
    }
    typename std::map<K, V>::iterator begin() { return m_.begin(); }
    typename std::map<K, V>::iterator end() { return m_.end(); }
    typename std::map<K, V>::const_iterator begin() const { return m_.begin(); }
    typename std::map<K, V>::const_iterator end() const { return m_.end(); }
    size_t size() const { return m_.size(); }
    bool empty() const { return m_.empty(); }
    void swap(concurrent_hash_map &o) { m_.swap(o.m_); }
};
}  // namespace tbb
