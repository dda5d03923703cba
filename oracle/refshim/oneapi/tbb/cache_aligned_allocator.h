// Stand-in for oneTBB's cache_aligned_resource: a memory_resource that returns
// 64-byte aligned blocks from its upstream, zero-filled.  The reference
// allocates its radix-tree nodes without constructing them and counts refit
// arrivals in them, relying on fresh memory being zero (test infrastructure).
#pragma once
#include <cstddef>
#include <cstring>
#include <memory_resource>
namespace tbb {
class cache_aligned_resource : public std::pmr::memory_resource {
 public:
  cache_aligned_resource() : up_(std::pmr::get_default_resource()) {}
  explicit cache_aligned_resource(std::pmr::memory_resource *up) : up_(up) {}

 private:
  static std::size_t al(std::size_t a) { return a < 64 ? 64 : a; }
  void *do_allocate(std::size_t bytes, std::size_t align) override {
    void *p = up_->allocate(bytes, al(align));
    std::memset(p, 0, bytes);
    return p;
  }
  void do_deallocate(void *p, std::size_t bytes, std::size_t align) override {
    up_->deallocate(p, bytes, al(align));
  }
  bool do_is_equal(const std::pmr::memory_resource &o) const noexcept override { return this == &o; }
  std::pmr::memory_resource *up_;
};
}  // namespace tbb
