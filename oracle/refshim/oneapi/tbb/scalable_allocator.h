// Stand-in for oneTBB's scalable_memory_resource: the default new/delete
// resource (test infrastructure).
#pragma once
#include <memory_resource>
#include "cache_aligned_allocator.h"
namespace tbb {
inline std::pmr::memory_resource *scalable_memory_resource() { return std::pmr::new_delete_resource(); }
}  // namespace tbb
namespace oneapi {
namespace tbb {
using ::tbb::cache_aligned_resource;
using ::tbb::scalable_memory_resource;
}  // namespace tbb
}  // namespace oneapi
