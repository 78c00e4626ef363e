// Stand-in for ankerl::unordered_dense::map (martinus/unordered_dense; the
// reference's submodule pin is not available). Observable behaviour kept:
// entries live in a dense vector of std::pair<Key, T>, iteration visits them
// in insertion order, find/operator[] are average O(1). Written from the
// library's documented interface; no code of the library is used.
#pragma once
#include <cstddef>
#include <cstdint>
#include <functional>
#include <utility>
#include <vector>

namespace ankerl {
namespace unordered_dense {

template <class Key, class T, class Hash = std::hash<Key>, class KeyEqual = std::equal_to<Key>>
class map {
 public:
  using value_type = std::pair<Key, T>;
  using iterator = typename std::vector<value_type>::iterator;
  using const_iterator = typename std::vector<value_type>::const_iterator;

  map() = default;
  explicit map(std::size_t bucket_count) { reserve(bucket_count); }

  iterator begin() { return values_.begin(); }
  iterator end() { return values_.end(); }
  const_iterator begin() const { return values_.begin(); }
  const_iterator end() const { return values_.end(); }
  std::size_t size() const { return values_.size(); }
  bool empty() const { return values_.empty(); }

  void clear() {
    values_.clear();
    for (auto &b : buckets_) b = 0;
  }
  void reserve(std::size_t n) {
    values_.reserve(n);
    if (n * 2 > buckets_.size()) rehash(n * 2);
  }
  iterator find(const Key &k) {
    if (buckets_.empty()) return end();
    std::size_t m = buckets_.size() - 1, h = slot_of(k) & m;
    for (;;) {
      uint32_t s = buckets_[h];
      if (!s) return end();
      if (KeyEqual()(values_[s - 1].first, k)) return values_.begin() + (s - 1);
      h = (h + 1) & m;
    }
  }
  const_iterator find(const Key &k) const { return const_cast<map *>(this)->find(k); }
  T &operator[](const Key &k) {
    auto it = find(k);
    if (it != end()) return it->second;
    if ((values_.size() + 1) * 2 > buckets_.size()) rehash((values_.size() + 1) * 2);
    values_.emplace_back(k, T());
    place(values_.size() - 1);
    return values_.back().second;
  }

 private:
  std::vector<value_type> values_;
  std::vector<uint32_t> buckets_;  // value index + 1, 0 = empty

  static std::size_t slot_of(const Key &k) {
    uint64_t z = uint64_t(Hash()(k)) + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return std::size_t(z ^ (z >> 31));
  }
  void place(std::size_t idx) {
    std::size_t m = buckets_.size() - 1, h = slot_of(values_[idx].first) & m;
    while (buckets_[h]) h = (h + 1) & m;
    buckets_[h] = uint32_t(idx + 1);
  }
  void rehash(std::size_t want) {
    std::size_t c = 8;
    while (c < want) c <<= 1;
    buckets_.assign(c, 0);
    for (std::size_t i = 0; i < values_.size(); i++) place(i);
  }
};

}  // namespace unordered_dense
}  // namespace ankerl
