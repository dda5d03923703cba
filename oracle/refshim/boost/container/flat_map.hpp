// Stand-in for boost::container::flat_map as an ordered std::map: the
// reference's Resource arena keeps its destructor registry in one (test
// infrastructure; nothing on the checked paths uses it).
#pragma once
#include <map>
namespace boost {
namespace container {
template <typename K, typename V>
using flat_map = std::map<K, V>;
}  // namespace container
}  // namespace boost
