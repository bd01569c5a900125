// dropin/matrix_ell_dense.cpp -- tbsla::cpp::MatrixELL and MatrixDENSE
// (src/cpp/matrix/MatrixELL.cpp, MatrixDENSE.cpp) with their products on the
// GPU (tbsla_ell_create / tbsla_dense_create + tbsla_spmv_host).
#include <algorithm>

#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/utils/vector.hpp>

#include "common.h"

namespace tbsla { namespace cpp {

// ------------------------------------------------------------------ ELL
// MatrixELL(const MatrixCOO&) (MatrixELL.cpp:12-54): entries in (row, col)
// order, each row left-aligned in max_col slots, padding (column 0, value 0)
MatrixELL::MatrixELL(const MatrixCOO &m) : values(0), columns(0), max_col(0) {
  n_row = ln_row = m.get_n_row();
  n_col = ln_col = m.get_n_col();
  f_row = m.get_f_row(); f_col = m.get_f_col();
  pr = m.get_pr(); pc = m.get_pc(); NR = m.get_NR(); NC = m.get_NC();
  nnz = m.get_nnz();
  if (m.get_values().empty()) {
    max_col = 0;
    nnz = 0;
    return;
  }
  const auto &r = m.get_row(), &c = m.get_col();
  const auto &v = m.get_values();
  const std::vector<int64_t> p = detail::row_col_order(r, c, n_row);
  std::vector<int> count((size_t)n_row, 0);
  for (int x : r) ++count[(size_t)x];
  max_col = *std::max_element(count.begin(), count.end());
  values.assign((size_t)n_row * max_col, 0.0);
  columns.assign((size_t)n_row * max_col, 0);
  size_t k = 0;
  for (int i = 0; i < n_row; ++i)
    for (int j = 0; j < count[(size_t)i]; ++j, ++k) {
      values[(size_t)i * max_col + j] = v[(size_t)p[k]];
      columns[(size_t)i * max_col + j] = c[(size_t)p[k]];
    }
}

std::ostream &operator<<(std::ostream &os, const MatrixELL &m) { return m.print(os); }

// rows the reference's loops visit: min(ln_row or n_row, values / max_col)
static long ell_rows(long lim, size_t n_values, int max_col) {
  return max_col > 0 ? std::min<long>(lim, (long)(n_values / (size_t)max_col)) : 0;
}

std::ostream &MatrixELL::print(std::ostream &os) const {
  detail::print_geometry(os, "------ ELL ------", TBSLA_GEOMETRY());
  os << "maximum number of columns  -  max_col : " << max_col << std::endl;
  tbsla::utils::vector::streamvector<double>(os, "val", values);
  os << std::endl;
  tbsla::utils::vector::streamvector<int>(os, "col", columns);
  os << std::endl;
  os << "-----------------" << std::endl << std::flush;
  return os;
}

std::ostream &MatrixELL::print_as_dense(std::ostream &os) {
  std::vector<double> d((size_t)n_row * n_col, 0.0);
  const long rows = ell_rows(n_row, values.size(), max_col);
  for (long i = 0; i < rows; ++i)
    for (int j = 0; j < max_col; ++j)
      d[(size_t)i * n_col + columns[(size_t)i * max_col + j]] += values[(size_t)i * max_col + j];
  tbsla::utils::vector::print_dense_matrix(n_row, n_col, d, os);
  return os;
}

std::vector<double> MatrixELL::spmv(const std::vector<double> &v, int vect_incr) const {
  std::vector<double> r(n_row, 0.0);
  Ax(r, v, vect_incr);
  return r;
}

// MatrixELL::Ax (MatrixELL.cpp:101-114): nothing when nnz or max_col is 0;
// r[i] = row i's sum for i < min(ln_row, values/max_col); columns below
// f_col read v[0]
void MatrixELL::Ax(std::vector<double> &r, const std::vector<double> &v, int vect_incr) const {
  if (product_is_zero()) return;
  const long rows = ell_rows(ln_row, values.size(), max_col);
  tbsla_matrix_t *h = device_matrix();
  if (rows >= n_row && r.size() == (size_t)n_row) {
    detail::check(tbsla_spmv_host(h, v.data(), (int64_t)v.size(), r.data(), (int64_t)r.size(), vect_incr));
    return;
  }
  detail::device_product(h, r, v, vect_incr, n_row, false, rows);
}

tbsla_matrix *MatrixELL::upload() const {
  const long rows = ell_rows(ln_row, values.size(), max_col);
  if ((long long)columns.size() < (long long)rows * max_col)
    throw std::invalid_argument("tbsla_gb300: MatrixELL columns shorter than values");
  tbsla_matrix_t *h = nullptr;
  detail::check(tbsla_ell_create(n_row, n_col, f_col, (int)rows, max_col, columns.data(), values.data(),
                                 TBSLA_STORE_F64, &h));
  return h;
}

bool MatrixELL::product_is_zero() const { return nnz == 0 || max_col == 0; }

void MatrixELL::array_identity(const void *ptr[3], std::size_t size[3]) const {
  ptr[0] = values.data(); size[0] = values.size();
  ptr[1] = columns.data(); size[1] = columns.size();
  ptr[2] = nullptr; size[2] = (size_t)max_col;
}

std::ostream &MatrixELL::print_infos(std::ostream &os) {
  os << "-----------------" << std::endl;
  os << "------ ELL ------" << std::endl;
  os << "--- general   ---" << std::endl;
  os << "n_row : " << n_row << std::endl;
  os << "n_col : " << n_col << std::endl;
  os << "nnz : " << nnz << std::endl;
  os << "max_col : " << max_col << std::endl;
  os << "--- capacity  ---" << std::endl;
  os << "values : " << values.capacity() << std::endl;
  os << "columns : " << columns.capacity() << std::endl;
  os << "--- size      ---" << std::endl;
  os << "values : " << values.size() << std::endl;
  os << "columns : " << columns.size() << std::endl;
  os << "-----------------" << std::endl;
  return os;
}

// the reference prints zero counts for ELL (MatrixELL.cpp:133-139)
std::ostream &MatrixELL::print_stats(std::ostream &os) {
  os << "upper values : " << 0 << std::endl;
  os << "lower values : " << 0 << std::endl;
  os << "diag  values : " << 0 << std::endl;
  return os;
}

// binary layout: geometry, max_col, values, columns (MatrixELL.cpp:141-190)
std::ostream &MatrixELL::write(std::ostream &os) {
  detail::write_geometry(os, TBSLA_GEOMETRY());
  detail::put(os, max_col);
  detail::write_array(os, values);
  detail::write_array(os, columns);
  return os;
}

std::istream &MatrixELL::read(std::istream &is, std::size_t, std::size_t) {
  detail::Geometry g{};
  detail::read_geometry(is, g);
  TBSLA_SET_GEOMETRY(g);
  detail::get(is, max_col);
  detail::read_array(is, values);
  detail::read_array(is, columns);
  return is;
}

void MatrixELL::fill_cdiag(int n_row_, int n_col_, int cdiag, int pr_, int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_ELL, 1, n_row_, n_col_, cdiag, 0.0, 0, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  max_col = o.geom[10];
  refill(values, std::move(o.values)); refill(columns, std::move(o.idx0));
}

void MatrixELL::fill_cqmat(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_, int pc_,
                           int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_ELL, 0, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  max_col = o.geom[10];
  refill(values, std::move(o.values)); refill(columns, std::move(o.idx0));
}

void MatrixELL::fill_cqmat_stochastic(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_,
                                      int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_ELL, 2, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  max_col = o.geom[10];
  refill(values, std::move(o.values)); refill(columns, std::move(o.idx0));
}

// MatrixELL::normalize_columns (MatrixELL.cpp:406-423): padding slots count
// toward column 0's sum, as in the reference
void MatrixELL::normalize_columns() {
  std::vector<double> sum((size_t)std::max(ln_col, 0), 0.0);
  const long rows = ell_rows(ln_row, values.size(), max_col);
  for (int pass = 0; pass < 2; ++pass)
    for (long i = 0; i < rows; ++i)
      for (int j = 0; j < max_col; ++j) {
        const size_t k = (size_t)i * max_col + j;
        long idx = (long)columns[k] - f_col;
        if (idx < 0) idx = 0;
        if (pass == 0) sum[(size_t)idx] += values[k];
        else values[k] /= sum[(size_t)idx];
      }
  invalidate_device();
}

// ---------------------------------------------------------------- DENSE
// MatrixDENSE(const MatrixCOO&) (MatrixDENSE.cpp:11-28): duplicates summed
// in the COO's order
MatrixDENSE::MatrixDENSE(const MatrixCOO &m) : values(0) {
  n_row = ln_row = m.get_n_row();
  n_col = ln_col = m.get_n_col();
  f_row = m.get_f_row(); f_col = m.get_f_col();
  pr = m.get_pr(); pc = m.get_pc(); NR = m.get_NR(); NC = m.get_NC();
  nnz = m.get_nnz();
  values.assign((size_t)ln_row * ln_col, 0.0);
  const auto &r = m.get_row(), &c = m.get_col();
  const auto &v = m.get_values();
  for (size_t k = 0; k < v.size(); ++k) values[(size_t)r[k] * ln_col + c[k]] += v[k];
}

std::ostream &operator<<(std::ostream &os, const MatrixDENSE &m) { return m.print(os); }

std::ostream &MatrixDENSE::print(std::ostream &os) const {
  detail::print_geometry(os, "----- DENSE -----", TBSLA_GEOMETRY());
  tbsla::utils::vector::print_dense_matrix(ln_row, ln_col, values, os);
  os << "-----------------" << std::endl << std::flush;
  return os;
}

std::ostream &MatrixDENSE::print_as_dense(std::ostream &os) { return print(os); }

std::vector<double> MatrixDENSE::spmv(const std::vector<double> &v, int vect_incr) const {
  std::vector<double> r(n_row, 0.0);
  if (product_is_zero()) return r;
  detail::check(tbsla_spmv_host(device_matrix(), v.data(), (int64_t)v.size(), r.data(), (int64_t)r.size(),
                                vect_incr));
  return r;
}

// MatrixDENSE::Ax (MatrixDENSE.cpp:64-73): r[i] += row i . v; nothing when
// nnz is 0
void MatrixDENSE::Ax(std::vector<double> &r, const std::vector<double> &v, int vect_incr) const {
  if (product_is_zero()) return;
  detail::device_product(device_matrix(), r, v, vect_incr, n_row, true, 0);
}

tbsla_matrix *MatrixDENSE::upload() const {
  if ((long long)values.size() < (long long)ln_row * ln_col)
    throw std::invalid_argument("tbsla_gb300: MatrixDENSE values shorter than ln_row * ln_col");
  tbsla_matrix_t *h = nullptr;
  detail::check(tbsla_dense_create(n_row, n_col, ln_row, ln_col, values.data(), TBSLA_STORE_F64, &h));
  return h;
}

bool MatrixDENSE::product_is_zero() const { return nnz == 0 || values.empty(); }

void MatrixDENSE::array_identity(const void *ptr[3], std::size_t size[3]) const {
  ptr[0] = values.data(); size[0] = values.size();
  ptr[1] = ptr[2] = nullptr; size[1] = size[2] = 0;
}

std::ostream &MatrixDENSE::print_infos(std::ostream &os) {
  os << "-----------------" << std::endl;
  os << "----- DENSE -----" << std::endl;
  os << "--- general   ---" << std::endl;
  os << "n_row : " << n_row << std::endl;
  os << "n_col : " << n_col << std::endl;
  os << "nnz : " << nnz << std::endl;
  os << "--- capacity  ---" << std::endl;
  os << "values : " << values.capacity() << std::endl;
  os << "--- size      ---" << std::endl;
  os << "values : " << values.size() << std::endl;
  os << "-----------------" << std::endl;
  return os;
}

std::ostream &MatrixDENSE::print_stats(std::ostream &os) {
  os << "upper values : " << 0 << std::endl;
  os << "lower values : " << 0 << std::endl;
  os << "diag  values : " << 0 << std::endl;
  return os;
}

// binary layout: geometry, values (MatrixDENSE.cpp:98-135)
std::ostream &MatrixDENSE::write(std::ostream &os) {
  detail::write_geometry(os, TBSLA_GEOMETRY());
  detail::write_array(os, values);
  return os;
}

std::istream &MatrixDENSE::read(std::istream &is, std::size_t, std::size_t) {
  detail::Geometry g{};
  detail::read_geometry(is, g);
  TBSLA_SET_GEOMETRY(g);
  detail::read_array(is, values);
  return is;
}

void MatrixDENSE::fill_cdiag(int n_row_, int n_col_, int cdiag, int pr_, int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_DENSE, 1, n_row_, n_col_, cdiag, 0.0, 0, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill(values, std::move(o.values));
}

void MatrixDENSE::fill_cqmat(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_, int pc_,
                             int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_DENSE, 0, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill(values, std::move(o.values));
}

void MatrixDENSE::fill_cqmat_stochastic(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_,
                                        int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_DENSE, 2, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill(values, std::move(o.values));
}

// MatrixDENSE::normalize_columns (MatrixDENSE.cpp:288-300)
void MatrixDENSE::normalize_columns() {
  std::vector<double> sum((size_t)std::max(ln_col, 0), 0.0);
  for (long i = 0; i < ln_row; ++i)
    for (long j = 0; j < ln_col; ++j) sum[(size_t)j] += values[(size_t)i * ln_col + j];
  for (long i = 0; i < ln_row; ++i)
    for (long j = 0; j < ln_col; ++j) values[(size_t)i * ln_col + j] /= sum[(size_t)j];
  invalidate_device();
}

}}  // namespace tbsla::cpp
