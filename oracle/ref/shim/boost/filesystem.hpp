// Stand-in for the one boost::filesystem call the reference makes (fworkdir.hpp): exists().
#pragma once
#include <filesystem>
namespace boost {
namespace filesystem {
inline bool exists(const std::string &p) { return std::filesystem::exists(p); }
}  // namespace filesystem
}  // namespace boost
