// Stand-in for emhash8::HashMap (ktprime/emhash): std::unordered_map. Only
// class templates of the reference that the contraction never instantiates
// name it.
#pragma once
#include <functional>
#include <unordered_map>

namespace emhash8 {
template <class Key, class T, class Hash = std::hash<Key>, class KeyEqual = std::equal_to<Key>>
using HashMap = std::unordered_map<Key, T, Hash, KeyEqual>;
}
