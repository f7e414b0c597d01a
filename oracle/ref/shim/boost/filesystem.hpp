// boost::filesystem subset used by network.cc (exists, create_directories)
#pragma once
#include <filesystem>
#include <string>
namespace boost {
namespace filesystem {
inline bool exists(const std::string& p) { return std::filesystem::exists(p); }
inline bool create_directories(const std::string& p) { return std::filesystem::create_directories(p); }
}  // namespace filesystem
}  // namespace boost
