// dropin/matrix_csr.cpp -- tbsla::cpp::MatrixCSR (src/cpp/matrix/MatrixCSR.cpp)
// with its product on the GPU (tbsla_csr_create + tbsla_spmv_host).
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/utils/vector.hpp>

#include "common.h"

namespace tbsla { namespace cpp {

// MatrixCSR(n_row, n_col, values, rowptr, colidx) (MatrixCSR.cpp:13-27).
// The reference leaves nnz uninitialised here; it is the stored count.
MatrixCSR::MatrixCSR(int n_row_, int n_col_, std::vector<double> &values_, std::vector<int> &rowptr_,
                     std::vector<int> &colidx_)
    : values(values_), rowptr(rowptr_), colidx(colidx_) {
  nnz = (long int)values.size();
  n_row = ln_row = n_row_;
  n_col = ln_col = n_col_;
  f_row = f_col = 0;
  pr = pc = 0;
  NR = NC = 1;
}

// MatrixCSR(const MatrixCOO&) (MatrixCSR.cpp:29-74): entries in (row, col)
// order, rowptr by counting
MatrixCSR::MatrixCSR(const MatrixCOO &m) {
  n_row = ln_row = m.get_n_row();
  n_col = ln_col = m.get_n_col();
  f_row = m.get_f_row(); f_col = m.get_f_col();
  pr = m.get_pr(); pc = m.get_pc(); NR = m.get_NR(); NC = m.get_NC();
  nnz = m.get_nnz();
  const auto &r = m.get_row(), &c = m.get_col();
  const auto &v = m.get_values();
  const std::vector<int64_t> p = detail::row_col_order(r, c, n_row);
  values.resize(p.size());
  colidx.resize(p.size());
  rowptr.assign((size_t)n_row + 1, 0);
  for (size_t k = 0; k < p.size(); ++k) {
    values[k] = v[(size_t)p[k]];
    colidx[k] = c[(size_t)p[k]];
    ++rowptr[(size_t)r[(size_t)p[k]] + 1];
  }
  for (int i = 0; i < n_row; ++i) rowptr[(size_t)i + 1] += rowptr[(size_t)i];
}

std::ostream &operator<<(std::ostream &os, const MatrixCSR &m) { return m.print(os); }

std::ostream &MatrixCSR::print(std::ostream &os) const {
  detail::print_geometry(os, "------ CSR ------", TBSLA_GEOMETRY());
  tbsla::utils::vector::streamvector<double>(os, "values", values);
  os << std::endl;
  tbsla::utils::vector::streamvector<int>(os, "rowptr", rowptr);
  os << std::endl;
  tbsla::utils::vector::streamvector<int>(os, "colidx", colidx);
  os << std::endl;
  os << "-----------------" << std::endl << std::flush;
  return os;
}

std::ostream &MatrixCSR::print_as_dense(std::ostream &os) {
  std::vector<double> d((size_t)n_row * n_col, 0.0);
  if (!values.empty() && !rowptr.empty()) {
    const int base = rowptr.front();
    for (size_t i = 0; i + 1 < rowptr.size(); ++i)
      for (int j = rowptr[i] - base; j < rowptr[i + 1] - base; ++j) d[i * n_col + colidx[(size_t)j]] += values[(size_t)j];
  }
  tbsla::utils::vector::print_dense_matrix(n_row, n_col, d, os);
  return os;
}

std::vector<double> MatrixCSR::spmv(const std::vector<double> &v, int vect_incr) const {
  std::vector<double> r(n_row, 0.0);
  Ax(r, v, vect_incr);
  return r;
}

// MatrixCSR::Ax (MatrixCSR.cpp:129-140): r[i] = row i's sum for the rows of
// rowptr; nothing when there are no values
void MatrixCSR::Ax(std::vector<double> &r, const std::vector<double> &v, int vect_incr) const {
  if (product_is_zero()) return;
  const long rows = rowptr.empty() ? 0 : (long)rowptr.size() - 1;
  tbsla_matrix_t *h = device_matrix();
  if (rows >= n_row && r.size() == (size_t)n_row) {
    detail::check(tbsla_spmv_host(h, v.data(), (int64_t)v.size(), r.data(), (int64_t)r.size(), vect_incr));
    return;
  }
  detail::device_product(h, r, v, vect_incr, n_row, false, rows);
}

tbsla_matrix *MatrixCSR::upload() const {
  const int rows = rowptr.empty() ? 0 : (int)rowptr.size() - 1;
  if (rows > 0) {
    const long long need = (long long)rowptr.back() - rowptr.front();
    if (need < 0 || (long long)colidx.size() < need || (long long)values.size() < need)
      throw std::invalid_argument("tbsla_gb300: MatrixCSR arrays shorter than rowptr says");
  }
  tbsla_matrix_t *h = nullptr;
  detail::check(tbsla_csr_create(n_row, n_col, f_col, rows, rowptr.data(), colidx.data(), values.data(),
                                 TBSLA_STORE_F64, &h));
  return h;
}

bool MatrixCSR::product_is_zero() const { return values.empty(); }

void MatrixCSR::array_identity(const void *ptr[3], std::size_t size[3]) const {
  ptr[0] = values.data(); size[0] = values.size();
  ptr[1] = rowptr.data(); size[1] = rowptr.size();
  ptr[2] = colidx.data(); size[2] = colidx.size();
}

std::ostream &MatrixCSR::print_infos(std::ostream &os) {
  os << "-----------------" << std::endl;
  os << "------ CSR ------" << std::endl;
  os << "--- general   ---" << std::endl;
  os << "n_row : " << n_row << std::endl;
  os << "n_col : " << n_col << std::endl;
  os << "--- capacity  ---" << std::endl;
  os << "values : " << values.capacity() << std::endl;
  os << "rowptr : " << rowptr.capacity() << std::endl;
  os << "colidx : " << colidx.capacity() << std::endl;
  os << "--- size      ---" << std::endl;
  os << "values : " << values.size() << std::endl;
  os << "rowptr : " << rowptr.size() << std::endl;
  os << "colidx : " << colidx.size() << std::endl;
  os << "-----------------" << std::endl;
  return os;
}

// entries above / below / on the diagonal (MatrixCSR.cpp:161-177; the
// reference prints the count of col > row as "lower")
std::ostream &MatrixCSR::print_stats(std::ostream &os) {
  long s = 0, u = 0, d = 0;
  if (!rowptr.empty()) {
    const int base = rowptr.front();
    for (size_t i = 0; i + 1 < rowptr.size(); ++i)
      for (int j = rowptr[i] - base; j < rowptr[i + 1] - base; ++j) {
        if ((int)i < colidx[(size_t)j]) ++s;
        else if ((int)i > colidx[(size_t)j]) ++u;
        else ++d;
      }
  }
  os << "upper values : " << u << std::endl;
  os << "lower values : " << s << std::endl;
  os << "diag  values : " << d << std::endl;
  return os;
}

// binary layout of MatrixCSR::write / read (MatrixCSR.cpp:179-232)
std::ostream &MatrixCSR::write(std::ostream &os) {
  detail::write_geometry(os, TBSLA_GEOMETRY());
  detail::write_array(os, values);
  detail::write_array(os, rowptr);
  detail::write_array(os, colidx);
  return os;
}

std::istream &MatrixCSR::read(std::istream &is, std::size_t, std::size_t) {
  detail::Geometry g{};
  detail::read_geometry(is, g);
  TBSLA_SET_GEOMETRY(g);
  detail::read_array(is, values);
  detail::read_array(is, rowptr);
  detail::read_array(is, colidx);
  return is;
}

void MatrixCSR::fill_cdiag(int n_row_, int n_col_, int cdiag, int pr_, int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_CSR, 1, n_row_, n_col_, cdiag, 0.0, 0, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill(values, std::move(o.values)); refill(rowptr, std::move(o.idx0)); refill(colidx, std::move(o.idx1));
}

void MatrixCSR::fill_cqmat(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_, int pc_,
                           int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_CSR, 0, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill_exact(values, std::move(o.values)); refill_exact(rowptr, std::move(o.idx0)); refill_exact(colidx, std::move(o.idx1));
}

void MatrixCSR::fill_cqmat_stochastic(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_,
                                      int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_CSR, 2, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill_exact(values, std::move(o.values)); refill_exact(rowptr, std::move(o.idx0)); refill_exact(colidx, std::move(o.idx1));
}

// MatrixCSR::normalize_columns (MatrixCSR.cpp:423-435): each value divided by
// its column's sum (column index relative to f_col), summed row by row over
// the raw rowptr ranges
void MatrixCSR::normalize_columns() {
  std::vector<double> sum((size_t)std::max(ln_col, 0), 0.0);
  for (int pass = 0; pass < 2; ++pass)
    for (size_t i = 0; i + 1 < rowptr.size(); ++i)
      for (long j = rowptr[i]; j < rowptr[i + 1]; ++j) {
        const size_t c = (size_t)(colidx[(size_t)j] - f_col);
        if (pass == 0) sum[c] += values[(size_t)j];
        else values[(size_t)j] /= sum[c];
      }
  invalidate_device();
}

}}  // namespace tbsla::cpp
