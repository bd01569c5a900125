// dropin/common.h -- helpers shared by the drop-in classes: status checks,
// the device copy record, the reference's binary layout and text output.
#pragma once

#include <cstdint>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include <tbsla/cpp/Matrix.hpp>

#include "../../../include/tbsla_gb300.h"
#include "../host_gen.h"

namespace tbsla { namespace cpp { namespace detail {

// Throws std::runtime_error with the library's message on failure.
inline void check(tbsla_status_t s) {
  if (s != TBSLA_OK) throw std::runtime_error(std::string("tbsla_gb300: ") + tbsla_last_error());
}

// Device handle of a matrix plus the identity of the host arrays it was
// built from (data pointers, sizes, geometry).
struct DeviceCopy {
  tbsla_matrix_t *h = nullptr;
  const void *ptr[3] = {nullptr, nullptr, nullptr};
  std::size_t size[3] = {0, 0, 0};
  long geom[12] = {0};
  ~DeviceCopy() {
    if (h) tbsla_matrix_destroy(h);
  }
};

// Geometry block of the binary layout (MatrixCSR.cpp:179-190 and the
// matching lines of every format): n_row n_col ln_row ln_col f_row f_col
// nnz(long) pr pc NR NC.
struct Geometry {
  int n_row, n_col, ln_row, ln_col, f_row, f_col;
  long int nnz;
  int pr, pc, NR, NC;
};

template <typename T> void put(std::ostream &os, const T &v) {
  os.write(reinterpret_cast<const char *>(&v), sizeof(T));
}
template <typename T> void get(std::istream &is, T &v) { is.read(reinterpret_cast<char *>(&v), sizeof(T)); }

inline void write_geometry(std::ostream &os, const Geometry &g) {
  put(os, g.n_row); put(os, g.n_col); put(os, g.ln_row); put(os, g.ln_col); put(os, g.f_row); put(os, g.f_col);
  put(os, g.nnz); put(os, g.pr); put(os, g.pc); put(os, g.NR); put(os, g.NC);
}
inline void read_geometry(std::istream &is, Geometry &g) {
  get(is, g.n_row); get(is, g.n_col); get(is, g.ln_row); get(is, g.ln_col); get(is, g.f_row); get(is, g.f_col);
  get(is, g.nnz); get(is, g.pr); get(is, g.pc); get(is, g.NR); get(is, g.NC);
}

// An array as (size_t count, elements).
template <typename T> void write_array(std::ostream &os, const std::vector<T> &v) {
  const std::size_t n = v.size();
  put(os, n);
  if (n) os.write(reinterpret_cast<const char *>(v.data()), n * sizeof(T));
}
template <typename T> void read_array(std::istream &is, std::vector<T> &v) {
  std::size_t n = 0;
  get(is, n);
  if (!is) { v.clear(); return; }
  v.resize(n);
  if (n) is.read(reinterpret_cast<char *>(v.data()), n * sizeof(T));
}

// The header lines of Matrix*::print (e.g. MatrixCSR.cpp:80-95).
void print_geometry(std::ostream &os, const char *title, const Geometry &g);

// r[0:n) of a product from the device; `accumulate` adds into r (the COO,
// SCOO and DENSE Ax), otherwise rows [0, rows) are overwritten (CSR, ELL).
void device_product(tbsla_matrix_t *h, std::vector<double> &r, const std::vector<double> &v, int vect_incr,
                    int n_row, bool accumulate, long rows);

// Row-major (row, col) order of triplets, ties in input order: the order of
// the reference's conversions (utils/csr.cpp:3-8; its std::sort leaves the
// order of equal (row, col) pairs unspecified).
std::vector<int64_t> row_col_order(const std::vector<int> &row, const std::vector<int> &col, int n_row);

}}}  // namespace tbsla::cpp::detail

// Member-wise geometry moves used inside the format classes (the fields are
// protected members of tbsla::cpp::Matrix).
#define TBSLA_GEOMETRY() \
  (tbsla::cpp::detail::Geometry{n_row, n_col, ln_row, ln_col, f_row, f_col, nnz, pr, pc, NR, NC})
#define TBSLA_SET_GEOMETRY(g)                                                                   \
  do {                                                                                          \
    n_row = (g).n_row; n_col = (g).n_col; ln_row = (g).ln_row; ln_col = (g).ln_col;             \
    f_row = (g).f_row; f_col = (g).f_col; nnz = (g).nnz; pr = (g).pr; pc = (g).pc;              \
    NR = (g).NR; NC = (g).NC;                                                                   \
    invalidate_device();                                                                        \
  } while (0)
// geometry of generated arrays (host_gen.h); nnz only where the reference
// sets it
// A stored array takes a fill's result the way the reference refills it
// (clear, then reserve or resize to the new size): its capacity never
// shrinks, which print() shows.  The generated array is moved in when the old
// capacity is smaller and the new array is exactly sized.
template <typename T> inline void refill(std::vector<T> &dst, std::vector<T> &&src) {
  if (dst.capacity() < src.size() && src.capacity() == src.size()) {
    dst = std::move(src);
    return;
  }
  dst.clear();
  dst.reserve(src.size());
  dst.insert(dst.end(), src.begin(), src.end());
}

// The cqmat fills of COO, SCOO and CSR end with shrink_to_fit in the
// reference: their arrays are exactly sized.
template <typename T> inline void refill_exact(std::vector<T> &dst, std::vector<T> &&src) {
  dst = std::move(src);
  dst.shrink_to_fit();
}

#define TBSLA_TAKE_GENERATED(o)                                                                 \
  do {                                                                                          \
    n_row = (o).geom[0]; n_col = (o).geom[1]; ln_row = (o).geom[2]; ln_col = (o).geom[3];       \
    f_row = (o).geom[4]; f_col = (o).geom[5]; pr = (o).geom[6]; pc = (o).geom[7];               \
    NR = (o).geom[8]; NC = (o).geom[9];                                                         \
    if ((o).nnz_set) nnz = (long int)(o).nnz;                                                   \
    invalidate_device();                                                                        \
  } while (0)
