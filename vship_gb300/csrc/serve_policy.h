// serve_policy.h -- host-side policy of the serving runtime (serve.cu): admission by charged
// device bytes, an LRU cache of per-source device state with pinning, and FIFO continuous
// batching. Plain C++ without CUDA, so that the policy is unit-tested on any host.
#pragma once

#include <cstddef>
#include <cstdint>
#include <deque>
#include <list>
#include <unordered_map>
#include <utility>
#include <vector>

namespace vship {

enum : int { SERVE_SSIMU2 = 0, SERVE_BUTTERAUGLI = 1 };

// Charged device bytes per active pair of w x h pixels: 12 FP32 planes for SSIMULACRA2, 31 for
// Butteraugli (the planes the reference holds per pair).
inline uint64_t serve_charge_per_pair(int metric, int64_t w, int64_t h) {
    return (metric == SERVE_SSIMU2 ? 48ull : 124ull) * (uint64_t)w * (uint64_t)h;
}

// Bytes charged against a budget; a charge either fits whole or waits.
class Admission {
public:
    explicit Admission(uint64_t budget = 0) : budget_(budget) {}
    bool fits_alone(uint64_t b) const { return b <= budget_; }
    bool try_charge(uint64_t b) {
        if (used_ + b > budget_) return false;
        used_ += b;
        if (used_ > peak_) peak_ = used_;
        return true;
    }
    void release(uint64_t b) { used_ = b > used_ ? 0 : used_ - b; }
    uint64_t used() const { return used_; }
    uint64_t peak() const { return peak_; }
    uint64_t budget() const { return budget_; }

private:
    uint64_t budget_ = 0, used_ = 0, peak_ = 0;
};

struct SourceKey {
    int metric = 0, res = 0;
    uint64_t key = 0;
    bool operator==(const SourceKey& o) const { return metric == o.metric && res == o.res && key == o.key; }
};
struct SourceKeyHash {
    size_t operator()(const SourceKey& k) const {
        uint64_t x = k.key * 0x9E3779B97F4A7C15ull ^ ((uint64_t)k.metric << 56) ^ ((uint64_t)k.res << 48);
        x ^= x >> 31;
        return (size_t)x;
    }
};

// LRU cache of source state. `V` is the caller's handle to the state (a device pointer); the
// cache never frees anything itself: entries it drops are handed back through `evicted`, and an
// entry with pin count > 0 (in use by a batch in flight) is never dropped.
template <typename V>
class SourceCache {
public:
    explicit SourceCache(uint64_t capacity_bytes = 0) : cap_(capacity_bytes) {}

    // Hit: moves the entry to the front, pins it once and returns its value.
    bool acquire(const SourceKey& k, V* out) {
        auto it = map_.find(k);
        if (it == map_.end()) {
            misses_++;
            return false;
        }
        hits_++;
        lru_.splice(lru_.begin(), lru_, it->second);
        it->second->pins++;
        *out = it->second->value;
        return true;
    }
    // Insert (pinned once), dropping unpinned entries from the back until `bytes` fit. Returns
    // false, changing nothing, when the pinned entries leave no room (or bytes > capacity).
    bool insert(const SourceKey& k, V value, uint64_t bytes, std::vector<V>* evicted) {
        if (bytes > cap_ || map_.count(k)) return false;
        uint64_t freeable = 0;
        for (const Node& n : lru_)
            if (n.pins == 0) freeable += n.bytes;
        if (used_ + bytes > cap_ && used_ - freeable + bytes > cap_) return false;
        // walk from the least recently used end, dropping unpinned entries
        auto it = lru_.end();
        while (used_ + bytes > cap_ && it != lru_.begin()) {
            --it;
            if (it->pins == 0) {
                used_ -= it->bytes;
                evicted->push_back(it->value);
                map_.erase(it->key);
                it = lru_.erase(it);
                evictions_++;
            }
        }
        lru_.push_front(Node{k, value, bytes, 1});
        map_[k] = lru_.begin();
        used_ += bytes;
        return true;
    }
    // Remove one entry whatever its pins (its state never became valid); its value goes to `out`.
    bool erase(const SourceKey& k, V* out) {
        auto it = map_.find(k);
        if (it == map_.end()) return false;
        *out = it->second->value;
        used_ -= it->second->bytes;
        lru_.erase(it->second);
        map_.erase(it);
        return true;
    }
    void unpin(const SourceKey& k) {
        auto it = map_.find(k);
        if (it != map_.end() && it->second->pins > 0) it->second->pins--;
    }
    // Drop every entry (all must be unpinned); their values go to `out`.
    void clear(std::vector<V>* out) {
        for (const Node& n : lru_) out->push_back(n.value);
        lru_.clear();
        map_.clear();
        used_ = 0;
    }
    int pins(const SourceKey& k) const {
        auto it = map_.find(k);
        return it == map_.end() ? -1 : it->second->pins;
    }
    uint64_t bytes() const { return used_; }
    size_t size() const { return map_.size(); }
    uint64_t hits() const { return hits_; }
    uint64_t misses() const { return misses_; }
    uint64_t evictions() const { return evictions_; }

private:
    struct Node {
        SourceKey key;
        V value;
        uint64_t bytes;
        int pins;
    };
    uint64_t cap_ = 0, used_ = 0, hits_ = 0, misses_ = 0, evictions_ = 0;
    std::list<Node> lru_;  // front = most recently used
    std::unordered_map<SourceKey, typename std::list<Node>::iterator, SourceKeyHash> map_;
};

// Continuous batching: take requests from the front of the queue, in arrival order, while each
// one's charge fits the admission budget and the batch stays within max_pairs pairs. A request
// that does not fit ends the batch (no overtaking, so no request starves). `charge(r)` and
// `pairs(r)` read a request.
template <typename R, typename ChargeFn, typename PairsFn>
std::vector<R*> form_batch(std::deque<R*>& queue, Admission& adm, int max_pairs, ChargeFn charge, PairsFn pairs) {
    std::vector<R*> batch;
    int np = 0;
    while (!queue.empty()) {
        R* r = queue.front();
        const int p = pairs(r);
        if (!batch.empty() && np + p > max_pairs) break;
        if (!adm.try_charge(charge(r))) break;
        queue.pop_front();
        batch.push_back(r);
        np += p;
    }
    return batch;
}

}  // namespace vship
