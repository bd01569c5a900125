// tbsla/cpp/utils/values_generation.hpp -- drop-in for TBSLA's generator
// entry functions (src/cpp/include/tbsla/cpp/utils/values_generation.hpp,
// src/cpp/utils/values_generation.cpp).  Each returns (row, column, value,
// tag); the tag names the branch that produced the entry, as the reference's.
#ifndef TBSLA_CPP_VALUES_GENERATION
#define TBSLA_CPP_VALUES_GENERATION

#include <cstddef>
#include <tuple>
#include <vector>

namespace tbsla { namespace utils { namespace values_generation {
std::tuple<std::size_t, std::size_t, double, std::size_t> cdiag_value(std::size_t i, std::size_t nv, std::size_t nr,
                                                                      std::size_t nc, std::size_t cdiag);
std::tuple<std::size_t, std::size_t, double, std::size_t> cqmat_value(std::size_t i, std::size_t nr, std::size_t nc,
                                                                      std::size_t c, double q,
                                                                      unsigned int seed_mult);
std::vector<double> cqmat_sum_columns(std::size_t nr, std::size_t nc, std::size_t c, double q, unsigned int seed_mult);
}}}

#endif
