// split.hpp -- tbsla::utils::io::split (src/cpp/include/tbsla/cpp/utils/split.hpp,
// src/cpp/utils/split.cpp): the pieces of `str` between occurrences of
// `delim`, empty pieces dropped.
#ifndef SPLIT_HPP
#define SPLIT_HPP
#include <string>
#include <vector>

namespace tbsla { namespace utils { namespace io {

  std::vector<std::string> split(const std::string& str, const std::string& delim);

}}}
#endif
