// Free-extent bookkeeping of one contiguous region (the server's pinned result
// reserve): best-fit allocation in multiples of a grain, and freed extents merged
// with their free neighbours, so that the region is one extent again once every
// block is back.  Offsets and lengths only: no memory is touched, and the caller
// holds whatever lock guards it.
#pragma once

#include <cstddef>
#include <map>

namespace ooc {

class Extents {
 public:
  // The region [0, bytes) is free; blocks are rounded up to multiples of `grain`.
  void reset(size_t bytes, size_t grain) {
    by_off_.clear();
    by_size_.clear();
    grain_ = grain;
    total_ = bytes;
    if (bytes) add(0, bytes);
  }
  // Best fit: the smallest free extent that holds n bytes (rounded up to the grain).
  // Returns false when none does; otherwise the block's offset and its length `cap`.
  bool take(size_t n, size_t& off, size_t& cap) {
    const size_t want = (n + grain_ - 1) / grain_ * grain_;
    auto it = by_size_.lower_bound(want ? want : grain_);
    if (it == by_size_.end()) return false;
    const size_t o = it->second, len = it->first;
    remove(o, len);
    cap = want ? want : grain_;
    if (len > cap) add(o + cap, len - cap);
    off = o;
    return true;
  }
  // Returns block [off, off + cap), merging it with the free extents on either side.
  void put(size_t off, size_t cap) {
    size_t len = cap;
    auto next = by_off_.lower_bound(off);
    if (next != by_off_.end() && next->first == off + len) {  // merge with the extent after
      len += next->second;
      remove(next->first, next->second);
    }
    auto prev = by_off_.lower_bound(off);
    if (prev != by_off_.begin()) {
      --prev;
      if (prev->first + prev->second == off) {  // and the one before
        off = prev->first;
        len += prev->second;
        remove(prev->first, prev->second);
      }
    }
    add(off, len);
  }
  size_t free_bytes() const {
    size_t f = 0;
    for (const auto& kv : by_off_) f += kv.second;
    return f;
  }
  size_t extents() const { return by_off_.size(); }
  size_t total() const { return total_; }

 private:
  void add(size_t off, size_t len) {
    by_off_[off] = len;
    by_size_.emplace(len, off);
  }
  void remove(size_t off, size_t len) {
    by_off_.erase(off);
    auto range = by_size_.equal_range(len);
    for (auto it = range.first; it != range.second; ++it)
      if (it->second == off) {
        by_size_.erase(it);
        break;
      }
  }
  size_t grain_ = 1, total_ = 0;
  std::map<size_t, size_t> by_off_;        // free extents: offset -> length
  std::multimap<size_t, size_t> by_size_;  // the same extents: length -> offset
};

}  // namespace ooc
