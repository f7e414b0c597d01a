// boost::algorithm::ends_with for relativity.cc
#pragma once
#include <string>
namespace boost {
namespace algorithm {
inline bool ends_with(const std::string& s, const std::string& suffix) {
  return s.size() >= suffix.size() && s.compare(s.size() - suffix.size(), suffix.size(), suffix) == 0;
}
}  // namespace algorithm
}  // namespace boost
