// Stand-in for oneTBB's parallel_for: runs the body once over the whole range
// on the calling thread (test infrastructure).
#pragma once
#include "blocked_range.h"
namespace tbb {
template <typename Range, typename Body>
void parallel_for(const Range &r, const Body &body) {
  body(r);
}
}  // namespace tbb
