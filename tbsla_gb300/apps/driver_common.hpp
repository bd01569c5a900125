// driver_common.hpp -- shared pieces of the driver programs: the
// reference's one-line JSON report (src/cpp/apps/tbsla_perf.cpp:145-192: a
// std::map of string keys and string values printed in key order as
// {"key":"value",...}), wall-clock time, the format chooser, and the
// algorithmic byte counts used for the GB/s figures.
#pragma once

#include <chrono>
#include <cstdint>
#include <iostream>
#include <map>
#include <memory>
#include <string>

#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>
#include <tbsla_gb300.h>

namespace driver {

inline double seconds() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

inline void print_report(const std::map<std::string, std::string> &out) {
  std::cout << "{";
  bool first = true;
  for (const auto &kv : out) {
    std::cout << (first ? "" : ",") << "\"" << kv.first << "\":\"" << kv.second << "\"";
    first = false;
  }
  std::cout << "}\n";
}

// an empty matrix of the named format (either case), or nullptr
inline std::unique_ptr<tbsla::cpp::Matrix> make_matrix(const std::string &format) {
  if (format == "COO" || format == "coo") return std::make_unique<tbsla::cpp::MatrixCOO>();
  if (format == "SCOO" || format == "scoo") return std::make_unique<tbsla::cpp::MatrixSCOO>();
  if (format == "CSR" || format == "csr") return std::make_unique<tbsla::cpp::MatrixCSR>();
  if (format == "ELL" || format == "ell") return std::make_unique<tbsla::cpp::MatrixELL>();
  if (format == "DENSE" || format == "dense") return std::make_unique<tbsla::cpp::MatrixDENSE>();
  return nullptr;
}

// a COO matrix converted to the named format (the reference's conversion
// constructors), or the COO itself
inline std::unique_ptr<tbsla::cpp::Matrix> convert(const tbsla::cpp::MatrixCOO &coo, const std::string &format) {
  if (format == "SCOO" || format == "scoo") return std::make_unique<tbsla::cpp::MatrixSCOO>(coo);
  if (format == "CSR" || format == "csr") return std::make_unique<tbsla::cpp::MatrixCSR>(coo);
  if (format == "ELL" || format == "ell") return std::make_unique<tbsla::cpp::MatrixELL>(coo);
  if (format == "DENSE" || format == "dense") return std::make_unique<tbsla::cpp::MatrixDENSE>(coo);
  return std::make_unique<tbsla::cpp::MatrixCOO>(coo);
}

// algorithmic bytes of one FP64 product: the stored entries with their
// indices (CSR: + row pointer; ELL and DENSE: every slot), x read once and
// y written once
inline double product_bytes(const tbsla_matrix_info_t &i) {
  const double vec = 8.0 * ((double)i.n_col + (double)i.n_row);
  switch (i.format) {
  case TBSLA_FMT_CSR: return 12.0 * (double)i.stored + 4.0 * ((double)i.rows + 1) + vec;
  case TBSLA_FMT_ELL: return 12.0 * (double)i.stored + vec;
  case TBSLA_FMT_DENSE: return 8.0 * (double)i.stored + vec;
  default: return 16.0 * (double)i.stored + vec;  // COO, SCOO
  }
}

inline std::string device_name_and_peak(double *peak_gbs) {
  char name[256] = {0};
  int dev = 0;
  *peak_gbs = 0;
  if (tbsla_device_describe(dev, name, (int)sizeof name, peak_gbs, nullptr) != TBSLA_OK) return "unknown";
  return name;
}

}  // namespace driver
