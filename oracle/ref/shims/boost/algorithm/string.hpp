// Minimal stand-in for the Boost string algorithms the reference uses:
// iequals, to_lower, to_lower_copy. Only for building the oracle.
#pragma once
#include <cctype>
#include <string>

namespace boost {
namespace algorithm {
inline void to_lower(std::string& s) {
  for (auto& c : s) c = (char)std::tolower((unsigned char)c);
}
inline std::string to_lower_copy(std::string s) {
  to_lower(s);
  return s;
}
inline bool iequals(const std::string& a, const std::string& b) {
  if (a.size() != b.size()) return false;
  for (size_t i = 0; i < a.size(); ++i)
    if (std::tolower((unsigned char)a[i]) != std::tolower((unsigned char)b[i])) return false;
  return true;
}
}  // namespace algorithm
using algorithm::iequals;
using algorithm::to_lower;
using algorithm::to_lower_copy;
}  // namespace boost
