// Serial stand-in for TBB's blocked_range (the pin library runs the
// reference's parallel loops on one thread; their bodies are independent
// per index, so the order does not change any result).
#pragma once
namespace tbb {
template <class T>
class blocked_range {
 public:
  blocked_range(T b, T e) : b_(b), e_(e) {}
  T begin() const { return b_; }
  T end() const { return e_; }

 private:
  T b_, e_;
};
}  // namespace tbb
