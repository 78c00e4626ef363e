// Stand-in for tsl::hopscotch_map (Tessil/hopscotch-map): a std::unordered_map
// with the library's iterator extension `it.value()`. Only the reference's
// non-hot code paths use it; it must compile, its speed does not matter.
#pragma once
#include <functional>
#include <unordered_map>
#include <utility>

namespace tsl {
template <class Key, class T, class Hash = std::hash<Key>, class KeyEqual = std::equal_to<Key>>
class hopscotch_map {
  using base = std::unordered_map<Key, T, Hash, KeyEqual>;
  base m_;

 public:
  template <class It>
  struct iter {
    It it;
    decltype(auto) operator*() const { return *it; }
    auto operator->() const { return &*it; }
    decltype(auto) value() const { return (it->second); }
    iter &operator++() { ++it; return *this; }
    bool operator==(const iter &o) const { return it == o.it; }
    bool operator!=(const iter &o) const { return it != o.it; }
  };
  using iterator = iter<typename base::iterator>;
  using const_iterator = iter<typename base::const_iterator>;
  iterator begin() { return {m_.begin()}; }
  iterator end() { return {m_.end()}; }
  const_iterator begin() const { return {m_.begin()}; }
  const_iterator end() const { return {m_.end()}; }
  iterator find(const Key &k) { return {m_.find(k)}; }
  const_iterator find(const Key &k) const { return {m_.find(k)}; }
  T &operator[](const Key &k) { return m_[k]; }
  std::size_t size() const { return m_.size(); }
  void clear() { m_.clear(); }
  void reserve(std::size_t n) { m_.reserve(n); }
  template <class... A> auto insert(A &&...a) { return m_.insert(std::forward<A>(a)...); }
};
}  // namespace tsl
