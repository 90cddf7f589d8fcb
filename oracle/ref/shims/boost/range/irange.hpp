// Minimal stand-in for boost::irange (half-open integer range).
#pragma once
#include <vector>
namespace boost {
template <class T>
std::vector<T> irange(T first, T last) {
  std::vector<T> r;
  for (T i = first; i < last; ++i) r.push_back(i);
  return r;
}
}  // namespace boost
