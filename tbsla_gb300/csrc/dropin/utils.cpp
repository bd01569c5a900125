// dropin/utils.cpp -- TBSLA's utility functions (src/cpp/utils/vector.cpp,
// range.cpp, csr.cpp, values_generation.cpp, InputParser.cpp, split.cpp,
// cpuset_to_cstr.cpp) for the drop-in headers.
#include <algorithm>
#include <cmath>
#include <iomanip>

#include <string>

#include <tbsla/cpp/utils/InputParser.hpp>
#include <tbsla/cpp/utils/cpuset_to_cstr.hpp>
#include <tbsla/cpp/utils/csr.hpp>
#include <tbsla/cpp/utils/range.hpp>
#include <tbsla/cpp/utils/split.hpp>
#include <tbsla/cpp/utils/values_generation.hpp>
#include <tbsla/cpp/utils/vector.hpp>

#include "common.h"

namespace {

// the product of the cdiag matrix (ones at (i, i - c) and (i, i + c); one
// diagonal when c = 0) with v, row by row
std::vector<double> cdiag_product(int nr, int nc, int c, const std::vector<double> &v) {
  std::vector<double> r((size_t)std::max(nr, 0), 0.0);
  for (long i = 0; i < nr; ++i) {
    if (c == 0) {
      r[(size_t)i] = i < nc ? v[(size_t)i] : 0.0;
      continue;
    }
    const bool lo = i - c >= 0 && i - c < nc, hi = i + c < nc;
    if (lo && hi) r[(size_t)i] = v[(size_t)(i + c)] + v[(size_t)(i - c)];
    else if (hi) r[(size_t)i] = v[(size_t)(i + c)];
    else if (lo) r[(size_t)i] = v[(size_t)(i - c)];
  }
  return r;
}

// compares r with the expected vector band by band; the codes are the
// reference's (vector.cpp:30-49)
int compare_bands(int nr, int nc, int c, const std::vector<double> &r, const std::vector<double> &e, bool debug) {
  for (long i = 0; i < nr; ++i) {
    if (debug) std::cout << "i = " << i << " r[i] = " << r[(size_t)i] << " exp " << e[(size_t)i] << std::endl;
    if (r[(size_t)i] != e[(size_t)i]) {
      if (i < std::min(c, nr)) return 10;
      if (i < std::min(nr, nc - c)) return 12;
      return 14;
    }
  }
  return 0;
}

}  // namespace

namespace tbsla { namespace utils { namespace vector {

int test_spmv_cdiag(int nr, int nc, int c, std::vector<double> &v, std::vector<double> &r, bool debug) {
  return compare_bands(nr, nc, c, r, cdiag_product(nr, nc, c, v), debug);
}

int test_a_axpx__cdiag(int nr, int nc, int c, std::vector<double> &v, std::vector<double> &r, bool debug) {
  if (nr != nc) return 111;
  std::vector<double> e = cdiag_product(nr, nc, c, v);
  for (size_t i = 0; i < e.size(); ++i) e[i] += v[i];
  e = cdiag_product(nr, nc, c, e);
  return compare_bands(nr, nc, c, r, e, debug);
}

// fixed-point table: as many decimals as the widest integer part (at least 1)
void print_dense_matrix(int nr, int nc, const std::vector<double> &m, std::ostream &os) {
  int digits = 1;
  for (long i = 0; i < (long)nr * nc; ++i) {
    const double a = std::fabs(m[(size_t)i]);
    if (a > 0 && std::isfinite(a)) digits = std::max(digits, (int)(std::log10(a) + 1));
  }
  os << std::fixed;
  os.precision(digits);
  for (long i = 0; i < nr; ++i) {
    for (long j = 0; j < nc; ++j) os << std::setw(digits + 3) << m[(size_t)(i * nc + j)] << "  ";
    os << std::endl;
  }
}

int compare_vectors(std::vector<double> v1, std::vector<double> v2) {
  if (v1.size() != v2.size()) return -1;
  int worst = 0;
  for (size_t i = 0; i < v1.size(); ++i) {
    const double d = v1[i] - v2[i];
    worst = std::max(worst, (int)(d * d));
  }
  return worst;
}

}}}  // namespace tbsla::utils::vector

namespace tbsla { namespace utils { namespace range {

size_t lnv(size_t size, int local_pos, int number_pos) {
  return size / (size_t)number_pos + ((size_t)local_pos < size % (size_t)number_pos ? 1 : 0);
}

size_t pflv(size_t size, int local_pos, int number_pos) {
  const size_t rem = size % (size_t)number_pos;
  return lnv(size, local_pos, number_pos) * (size_t)local_pos + ((size_t)local_pos >= rem ? rem : 0);
}

}}}  // namespace tbsla::utils::range

namespace tbsla { namespace cpp { namespace utils { namespace csr {

bool compare_row(const std::vector<int> &row, const std::vector<int> &col, unsigned i, unsigned j) {
  return row[i] != row[j] ? row[i] < row[j] : col[i] < col[j];
}

}}}}  // namespace tbsla::cpp::utils::csr

namespace tbsla { namespace utils { namespace values_generation {

std::tuple<std::size_t, std::size_t, double, std::size_t> cdiag_value(std::size_t i, std::size_t, std::size_t,
                                                                      std::size_t nc, std::size_t cdiag) {
  int64_t r = 0, c = 0;
  int tag = 0;
  tbsla::cdiag_entry_tagged((int64_t)i, (int64_t)nc, (int64_t)cdiag, r, c, tag);
  return std::make_tuple((std::size_t)r, (std::size_t)c, 1.0, (std::size_t)tag);
}

std::tuple<std::size_t, std::size_t, double, std::size_t> cqmat_value(std::size_t i, std::size_t nr, std::size_t nc,
                                                                      std::size_t c, double q,
                                                                      unsigned int seed_mult) {
  int64_t r = 0, col = 0;
  int tag = 0;
  tbsla::cqmat_entry_tagged(i, nr, nc, c, q, seed_mult, r, col, tag);
  return std::make_tuple((std::size_t)r, (std::size_t)col, 1.0, (std::size_t)tag);
}

std::vector<double> cqmat_sum_columns(std::size_t nr, std::size_t nc, std::size_t c, double q,
                                      unsigned int seed_mult) {
  std::vector<double> s = tbsla::cqmat_column_sums((int)nr, (int)nc, (int)c, q, seed_mult);
  s.resize(nc);
  return s;
}

}}}  // namespace tbsla::utils::values_generation

// ------------------------------------------------ driver-program utilities
// InputParser (src/cpp/utils/InputParser.cpp:4-21)
InputParser::InputParser(int &argc, char **argv) {
  for (int i = 1; i < argc; ++i) params.emplace_back(argv[i]);
}

std::string InputParser::get_opt(const std::string &option, const std::string default_opt) const {
  for (std::size_t i = 0; i < params.size(); ++i)
    if (params[i] == option) return i + 1 < params.size() ? params[i + 1] : default_opt;
  return default_opt;
}

bool InputParser::has_opt(const std::string &option) const {
  return std::find(params.begin(), params.end(), option) != params.end();
}

namespace tbsla { namespace utils { namespace io {

// the non-empty pieces of str between occurrences of delim (an empty delim
// leaves str whole)
std::vector<std::string> split(const std::string &str, const std::string &delim) {
  std::vector<std::string> out;
  if (delim.empty()) {
    if (!str.empty()) out.push_back(str);
    return out;
  }
  std::size_t start = 0;
  while (start <= str.size()) {
    const std::size_t hit = str.find(delim, start);
    const std::size_t end = hit == std::string::npos ? str.size() : hit;
    if (end > start) out.push_back(str.substr(start, end - start));
    if (hit == std::string::npos) break;
    start = hit + delim.size();
  }
  return out;
}

}}}  // namespace tbsla::utils::io

namespace tbsla { namespace cpp { namespace utils {

char *cpuset_to_cstr(cpu_set_t *mask, char *str) {
  std::string out;
  for (int i = 0; i < CPU_SETSIZE; ++i) {
    if (!CPU_ISSET(i, mask)) continue;
    int j = i;
    while (j + 1 < CPU_SETSIZE && CPU_ISSET(j + 1, mask)) ++j;
    if (!out.empty()) out += ',';
    if (j - i >= 2) out += std::to_string(i) + "-" + std::to_string(j);
    else if (j == i + 1) out += std::to_string(i) + "," + std::to_string(j);
    else out += std::to_string(i);
    i = j;
  }
  std::copy(out.begin(), out.end(), str);
  str[out.size()] = '\0';
  return str;
}

}}}  // namespace tbsla::cpp::utils
