// The drop-in's driver-program utilities on known answers: split
// (src/cpp/utils/split.cpp), cpuset_to_cstr (src/cpp/utils/cpuset_to_cstr.cpp)
// and InputParser (src/cpp/utils/InputParser.cpp).  Exit code = failures.
#include <iostream>
#include <string>
#include <vector>

#include <tbsla/cpp/utils/InputParser.hpp>
#include <tbsla/cpp/utils/cpuset_to_cstr.hpp>
#include <tbsla/cpp/utils/split.hpp>

static int failures = 0;
static void expect(bool ok, const std::string &what) {
  if (!ok) {
    ++failures;
    std::cout << "FAIL " << what << std::endl;
  }
}

int main() {
  using V = std::vector<std::string>;
  using tbsla::utils::io::split;
  expect(split("a,b,,c", ",") == V({"a", "b", "c"}), "split drops empty pieces");
  expect(split(",a,", ",") == V({"a"}), "split leading and trailing delimiters");
  expect(split("", ",").empty(), "split empty string");
  expect(split("abc", ",") == V({"abc"}), "split without delimiter");
  expect(split("x::y::::z", "::") == V({"x", "y", "z"}), "split multi-character delimiter");
  expect(split("key: value", ": ") == V({"key", "value"}), "split key/value");

  cpu_set_t m;
  CPU_ZERO(&m);
  for (int c : {0, 1, 2, 3, 6, 8, 9, 12, 13, 14}) CPU_SET(c, &m);
  char buf[7 * CPU_SETSIZE];
  expect(std::string(tbsla::cpp::utils::cpuset_to_cstr(&m, buf)) == "0-3,6,8,9,12-14", "cpuset_to_cstr runs");
  CPU_ZERO(&m);
  expect(std::string(tbsla::cpp::utils::cpuset_to_cstr(&m, buf)) == "", "cpuset_to_cstr empty set");
  CPU_SET(5, &m);
  expect(std::string(tbsla::cpp::utils::cpuset_to_cstr(&m, buf)) == "5", "cpuset_to_cstr one CPU");

  char a0[] = "app", a1[] = "--format", a2[] = "CSR", a3[] = "--print-infos", a4[] = "--format", a5[] = "ELL",
       a6[] = "--C";
  char *argv[] = {a0, a1, a2, a3, a4, a5, a6};
  int argc = 7;
  InputParser in(argc, argv);
  expect(in.get_opt("--format") == "CSR", "get_opt takes the first occurrence");
  expect(in.has_opt("--print-infos") && !in.has_opt("--op"), "has_opt");
  expect(in.get_opt("--C", "8") == "8", "get_opt of a last option gives the default");
  expect(in.get_opt("--Q", "0.1") == "0.1", "get_opt of an absent option gives the default");
  expect(in.get_opt("app", "none") == "none", "argv[0] is not an argument");
  std::cout << (failures ? "FAILED " : "OK ") << failures << std::endl;
  return failures;
}
