// Stand-in for oneTBB's parallel_sort: a stable sort, so elements with equal
// keys keep their input order (TBB does not specify that order; test
// infrastructure).
#pragma once
#include <algorithm>
namespace tbb {
template <typename It, typename Compare>
void parallel_sort(It first, It last, const Compare &comp) {
  std::stable_sort(first, last, comp);
}
template <typename It>
void parallel_sort(It first, It last) {
  std::stable_sort(first, last);
}
}  // namespace tbb
