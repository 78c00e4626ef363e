// Stand-in for tsl::hopscotch_set (Tessil/hopscotch-map): std::unordered_set.
#pragma once
#include <functional>
#include <unordered_set>

namespace tsl {
template <class Key, class Hash = std::hash<Key>, class KeyEqual = std::equal_to<Key>>
using hopscotch_set = std::unordered_set<Key, Hash, KeyEqual>;
}
