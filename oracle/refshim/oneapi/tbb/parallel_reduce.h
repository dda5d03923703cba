// Stand-in for oneTBB's functional parallel_reduce: one sequential chunk,
// then the join with the identity (test infrastructure).
#pragma once
#include "blocked_range.h"
namespace tbb {
template <typename Range, typename Value, typename RealBody, typename Reduction>
Value parallel_reduce(const Range &r, const Value &identity, const RealBody &body,
                      const Reduction &join) {
  return join(identity, body(r, identity));
}
}  // namespace tbb
