// tbsla/cpp/utils/vector.hpp -- drop-in for TBSLA's vector helpers
// (src/cpp/include/tbsla/cpp/utils/vector.hpp, src/cpp/utils/vector.cpp):
// printing, the closed-form checks of cdiag products and the vector
// comparison the reference's tests use.
#ifndef TBSLA_CPP_UTILS
#define TBSLA_CPP_UTILS

#include <iostream>
#include <string>
#include <vector>

namespace tbsla { namespace utils { namespace vector {

// "name : v0, v1, ..., vn"
template <class myType>
void streamvector(std::ostream &os, const std::string name, const std::vector<myType> &v) {
  os << name << " : ";
  for (std::size_t i = 0; i < v.size(); ++i) {
    if (i) os << ", ";
    os << v[i];
  }
}

// 0 when r equals the cdiag product of v (cdiag offset c, nr x nc), else a
// code naming the failing band: 10 (rows < c), 12 (middle), 14 (tail)
int test_spmv_cdiag(int nr, int nc, int c, std::vector<double> &v, std::vector<double> &r, bool debug);
// the same for a_axpx_ (square only, 111 otherwise)
int test_a_axpx__cdiag(int nr, int nc, int c, std::vector<double> &v, std::vector<double> &r, bool debug);
void print_dense_matrix(int nr, int nc, const std::vector<double> &m, std::ostream &os);
// -1 on a size mismatch, else the largest squared difference truncated to int
int compare_vectors(std::vector<double> v1, std::vector<double> v2);

}}}

#endif
