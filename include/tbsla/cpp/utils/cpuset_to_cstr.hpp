// cpuset_to_cstr.hpp -- tbsla::cpp::utils::cpuset_to_cstr
// (src/cpp/include/tbsla/cpp/utils/cpuset_to_cstr.hpp): writes the CPUs of
// `mask` to `str` as a list such as "0-3,6,8,9" (runs of three or more as
// ranges) and returns `str`; `str` needs room for the longest list.
#ifndef CPUSET_TO_CSTR_HPP
#define CPUSET_TO_CSTR_HPP
#include <sched.h>

namespace tbsla { namespace cpp { namespace utils {

  char *cpuset_to_cstr(cpu_set_t *mask, char *str);

}}}
#endif
