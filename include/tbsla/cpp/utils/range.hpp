// tbsla/cpp/utils/range.hpp -- drop-in for TBSLA's block split
// (src/cpp/include/tbsla/cpp/utils/range.hpp, src/cpp/utils/range.cpp).
#ifndef TBSLA_CPP_RANGE
#define TBSLA_CPP_RANGE

#include <cstddef>

namespace tbsla { namespace utils { namespace range {
// number of the size values held by part local_pos of number_pos parts
size_t lnv(size_t size, int local_pos, int number_pos);
// index of that part's first value
size_t pflv(size_t size, int local_pos, int number_pos);
}}}

#endif
