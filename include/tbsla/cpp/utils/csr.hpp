// tbsla/cpp/utils/csr.hpp -- drop-in for TBSLA's conversion helpers
// (src/cpp/include/tbsla/cpp/utils/csr.hpp, src/cpp/utils/csr.cpp).
#ifndef TBSLA_CPP_UTILS_CSR
#define TBSLA_CPP_UTILS_CSR

#include <cassert>
#include <vector>

namespace tbsla { namespace cpp { namespace utils { namespace csr {

// t permuted by order: result[i] = t[order[i]]
template <typename T>
std::vector<T> applyPermutation(const std::vector<int> &order, const std::vector<T> &t) {
  assert(order.size() == t.size());
  std::vector<T> st(t.size());
  for (std::size_t i = 0; i < t.size(); ++i) st[i] = t[(std::size_t)order[i]];
  return st;
}

// (row, col) lexicographic "less" of entries i and j
bool compare_row(const std::vector<int> &row, const std::vector<int> &col, unsigned i, unsigned j);

}}}}

#endif
