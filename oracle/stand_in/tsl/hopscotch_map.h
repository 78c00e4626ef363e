// Stand-in for tsl::hopscotch_map (Tessil/hopscotch-map). Like the library,
// its value_type is std::pair<Key, T> (the key is not const) and its iterators
// have `value()`. Entries live in a vector in insertion order, found through
// a std::unordered_map of positions. Only the reference's non-hot code paths
// use it (Tensor::multiply); it must compile and give the same entries, its
// speed does not matter.
#pragma once
#include <cstddef>
#include <functional>
#include <unordered_map>
#include <utility>
#include <vector>

namespace tsl {
template <class Key, class T, class Hash = std::hash<Key>, class KeyEqual = std::equal_to<Key>>
class hopscotch_map {
  using entries = std::vector<std::pair<Key, T>>;
  entries e_;
  std::unordered_map<Key, std::size_t, Hash, KeyEqual> pos_;

 public:
  using value_type = std::pair<Key, T>;
  template <class It>
  struct iter {
    It it;
    decltype(auto) operator*() const { return *it; }
    auto operator->() const { return &*it; }
    decltype(auto) value() const { return (it->second); }
    iter &operator++() {
      ++it;
      return *this;
    }
    bool operator==(const iter &o) const { return it == o.it; }
    bool operator!=(const iter &o) const { return it != o.it; }
  };
  using iterator = iter<typename entries::iterator>;
  using const_iterator = iter<typename entries::const_iterator>;
  iterator begin() { return {e_.begin()}; }
  iterator end() { return {e_.end()}; }
  const_iterator begin() const { return {e_.begin()}; }
  const_iterator end() const { return {e_.end()}; }
  iterator find(const Key &k) {
    auto p = pos_.find(k);
    return p == pos_.end() ? end() : iterator{e_.begin() + std::ptrdiff_t(p->second)};
  }
  const_iterator find(const Key &k) const {
    auto p = pos_.find(k);
    return p == pos_.end() ? end() : const_iterator{e_.begin() + std::ptrdiff_t(p->second)};
  }
  T &operator[](const Key &k) {
    auto p = pos_.find(k);
    if (p != pos_.end()) return e_[p->second].second;
    pos_.emplace(k, e_.size());
    e_.emplace_back(k, T());
    return e_.back().second;
  }
  std::size_t size() const { return e_.size(); }
  std::size_t overflow_size() const { return 0; }  // the library's overflow list: none here
  void clear() {
    e_.clear();
    pos_.clear();
  }
  void reserve(std::size_t n) {
    e_.reserve(n);
    pos_.reserve(n);
  }
  std::pair<iterator, bool> insert(const value_type &v) {
    auto p = pos_.find(v.first);
    if (p != pos_.end()) return {iterator{e_.begin() + std::ptrdiff_t(p->second)}, false};
    pos_.emplace(v.first, e_.size());
    e_.push_back(v);
    return {iterator{e_.end() - 1}, true};
  }
};
}  // namespace tsl
