// Stand-in for oneTBB's blocked_range (test infrastructure).
#pragma once
#include <cstddef>
namespace tbb {
template <typename T>
class blocked_range {
 public:
  blocked_range(T b, T e) : b_(b), e_(e) {}
  T begin() const { return b_; }
  T end() const { return e_; }
  std::size_t size() const { return std::size_t(e_ - b_); }
  bool empty() const { return !(b_ < e_); }

 private:
  T b_, e_;
};
}  // namespace tbb
