// Minimal stand-in for boost::push_back(container, range).
#pragma once
namespace boost {
template <class C, class R>
C& push_back(C& c, const R& r) {
  for (const auto& v : r) c.push_back(v);
  return c;
}
}  // namespace boost
