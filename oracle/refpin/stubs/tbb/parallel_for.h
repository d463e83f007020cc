// Serial stand-in for tbb::parallel_for: the body runs once over the whole range.
#pragma once
#include "blocked_range.h"
namespace tbb {
template <class Range, class Body>
void parallel_for(const Range& r, const Body& body) {
  body(r);
}
}  // namespace tbb
