// dropin/matrix_coo.cpp -- tbsla::cpp::MatrixCOO and MatrixSCOO
// (src/cpp/matrix/MatrixCOO.cpp, MatrixSCOO.cpp) with their products on the
// GPU (tbsla_coo_create + tbsla_spmv_host), Matrix Market input included.
#include <sstream>
#include <string>

#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>
#include <tbsla/cpp/utils/vector.hpp>

#include "common.h"

namespace tbsla { namespace cpp {

namespace {

template <typename Fn> void stats(const std::vector<int> &row, const std::vector<int> &col, std::ostream &os, Fn) {
  long s = 0, u = 0, d = 0;
  if (row.size() != col.size()) {
    std::cerr << "Err \n";
    return;
  }
  for (size_t i = 0; i < row.size(); ++i) {
    if (row[i] < col[i]) ++s;
    else if (row[i] > col[i]) ++u;
    else ++d;
  }
  os << "upper values : " << u << std::endl;
  os << "lower values : " << s << std::endl;
  os << "diag  values : " << d << std::endl;
}

void triplet_infos(std::ostream &os, const char *title, int n_row, int n_col, const std::vector<double> &values,
                   const std::vector<int> &row, const std::vector<int> &col) {
  os << "-----------------" << std::endl;
  os << title << std::endl;
  os << "--- general   ---" << std::endl;
  os << "n_row : " << n_row << std::endl;
  os << "n_col : " << n_col << std::endl;
  os << "--- capacity  ---" << std::endl;
  os << "values : " << values.capacity() << std::endl;
  os << "row : " << row.capacity() << std::endl;
  os << "col : " << col.capacity() << std::endl;
  os << "--- size      ---" << std::endl;
  os << "values : " << values.size() << std::endl;
  os << "row : " << row.size() << std::endl;
  os << "col : " << col.size() << std::endl;
  os << "-----------------" << std::endl;
}

void triplet_print(std::ostream &os, const std::vector<double> &values, const std::vector<int> &row,
                   const std::vector<int> &col) {
  tbsla::utils::vector::streamvector<double>(os, "val", values);
  os << std::endl;
  tbsla::utils::vector::streamvector<int>(os, "row", row);
  os << std::endl;
  tbsla::utils::vector::streamvector<int>(os, "col", col);
  os << std::endl;
  os << "-----------------" << std::endl << std::flush;
}

void triplet_dense(std::ostream &os, int n_row, int n_col, const std::vector<double> &values,
                   const std::vector<int> &row, const std::vector<int> &col) {
  std::vector<double> d((size_t)n_row * n_col, 0.0);
  for (size_t i = 0; i < row.size(); ++i) d[(size_t)row[i] * n_col + col[i]] += values[i];
  tbsla::utils::vector::print_dense_matrix(n_row, n_col, d, os);
}

tbsla_matrix_t *triplet_upload(int n_row, int n_col, int f_row, int f_col, const std::vector<double> &values,
                               const std::vector<int> &row, const std::vector<int> &col) {
  if (row.size() < values.size() || col.size() < values.size())
    throw std::invalid_argument("tbsla_gb300: COO index arrays shorter than the values");
  tbsla_matrix_t *h = nullptr;
  detail::check(tbsla_coo_create(n_row, n_col, f_row, f_col, (int64_t)values.size(), row.data(), col.data(),
                                 values.data(), TBSLA_STORE_F64, &h));
  return h;
}

}  // namespace

// ------------------------------------------------------------------ COO
void MatrixCOO::init(int n_row_, int n_col_, long int n_values) {
  n_row = ln_row = n_row_;
  n_col = ln_col = n_col_;
  f_row = f_col = 0;
  pr = pc = 0;
  NR = NC = 1;
  values.reserve((size_t)n_values);
  row.reserve((size_t)n_values);
  col.reserve((size_t)n_values);
}

// the reference leaves nnz uninitialised in the array constructors; it is
// the stored count here
MatrixCOO::MatrixCOO(int n_row_, int n_col_, std::vector<double> &values_, std::vector<int> &row_,
                     std::vector<int> &col_)
    : values(values_), row(row_), col(col_) {
  init(n_row_, n_col_, 0);
  nnz = (long int)values.size();
}

MatrixCOO::MatrixCOO(int n_row_, int n_col_, long int n_values) { init(n_row_, n_col_, n_values); }

MatrixCOO::MatrixCOO(int n_row_, int n_col_) { init(n_row_, n_col_, 0); }

std::ostream &operator<<(std::ostream &os, const MatrixCOO &m) { return m.print(os); }

std::ostream &MatrixCOO::print(std::ostream &os) const {
  detail::print_geometry(os, "------ COO ------", TBSLA_GEOMETRY());
  triplet_print(os, values, row, col);
  return os;
}

std::ostream &MatrixCOO::print_as_dense(std::ostream &os) {
  triplet_dense(os, n_row, n_col, values, row, col);
  return os;
}

std::ostream &MatrixCOO::print_infos(std::ostream &os) {
  triplet_infos(os, "------ COO ------", n_row, n_col, values, row, col);
  return os;
}

std::ostream &MatrixCOO::print_stats(std::ostream &os) {
  stats(row, col, os, 0);
  return os;
}

std::vector<double> MatrixCOO::spmv(const std::vector<double> &v, int vect_incr) const {
  std::vector<double> r(n_row, 0.0);
  if (product_is_zero()) return r;
  detail::check(tbsla_spmv_host(device_matrix(), v.data(), (int64_t)v.size(), r.data(), (int64_t)r.size(),
                                vect_incr));
  return r;
}

// MatrixCOO::Ax (MatrixCOO.cpp:107-116): r[row + vect_incr] += value * v[col]
void MatrixCOO::Ax(std::vector<double> &r, const std::vector<double> &v, int vect_incr) const {
  if (product_is_zero()) return;
  detail::device_product(device_matrix(), r, v, vect_incr, n_row, true, 0);
}

tbsla_matrix *MatrixCOO::upload() const { return triplet_upload(n_row, n_col, 0, 0, values, row, col); }

bool MatrixCOO::product_is_zero() const { return values.empty(); }

void MatrixCOO::array_identity(const void *ptr[3], std::size_t size[3]) const {
  ptr[0] = values.data(); size[0] = values.size();
  ptr[1] = row.data(); size[1] = row.size();
  ptr[2] = col.data(); size[2] = col.size();
}

// MatrixCOO::push_back (MatrixCOO.cpp:118-126): out-of-range entries are
// dropped silently
void MatrixCOO::push_back(int r, int c, double v) {
  if (r >= n_row || r < 0) return;
  if (c >= n_col || c < 0) return;
  values.push_back(v);
  row.push_back(r);
  col.push_back(c);
}

void MatrixCOO::update_nnz() {
  values.shrink_to_fit();
  col.shrink_to_fit();
  row.shrink_to_fit();
  nnz = (long int)values.size();
}

std::ostream &MatrixCOO::write(std::ostream &os) {
  detail::write_geometry(os, TBSLA_GEOMETRY());
  detail::write_array(os, values);
  detail::write_array(os, row);
  detail::write_array(os, col);
  return os;
}

std::istream &MatrixCOO::read(std::istream &is, std::size_t, std::size_t) {
  detail::Geometry g{};
  detail::read_geometry(is, g);
  TBSLA_SET_GEOMETRY(g);
  detail::read_array(is, values);
  detail::read_array(is, row);
  detail::read_array(is, col);
  return is;
}

// MatrixCOO::readMM (MatrixCOO.cpp:230-292): "%%MatrixMarket matrix
// coordinate real general|symmetric"; 1-based entries, symmetric files add
// the mirror of each off-diagonal entry; the banner and size lines are echoed
// to stdout; other kinds throw MatrixFormatReadException.  A file that
// cannot be opened leaves the matrix unchanged.
void MatrixCOO::readMM(std::string name) {
  std::ifstream is(name);
  if (!is.is_open()) return;
  std::string line;
  std::getline(is, line);
  std::vector<std::string> w;
  {
    // fields split on single spaces, as utils/split.cpp does
    size_t a = 0;
    while (true) {
      const size_t b = line.find(' ', a);
      w.push_back(line.substr(a, b == std::string::npos ? std::string::npos : b - a));
      if (b == std::string::npos) break;
      a = b + 1;
    }
  }
  std::cout << line << "\n";
  const bool coord = w.size() >= 4 && w[0] == "%%MatrixMarket" && w[1] == "matrix" && w[2] == "coordinate" &&
                     w[3] == "real";
  const bool general = coord && w.size() >= 5 && w[4] == "general";
  const bool symmetric = coord && w.size() >= 5 && w[4] == "symmetric";
  if (!general && !symmetric) throw MatrixFormatReadException();
  while (line.rfind("%", 0) == 0) std::getline(is, line);
  std::cout << line << "\n";
  std::stringstream ss(line);
  int nr = 0, nc = 0, nv = 0;
  ss >> nr >> nc >> nv;
  // like the reference, entries already held are kept (init only reserves)
  init(nr, nc, symmetric ? 2L * nv : (long)nv);
  int r = 0, c = 0;
  double v = 0;
  for (int i = 0; i < nv && !is.eof(); ++i) {
    is >> r >> c >> v;
    push_back(r - 1, c - 1, v);
    if (symmetric && r != c) push_back(c - 1, r - 1, v);
  }
  update_nnz();
}

void MatrixCOO::fill_cdiag(int n_row_, int n_col_, int cdiag, int pr_, int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_COO, 1, n_row_, n_col_, cdiag, 0.0, 0, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill(values, std::move(o.values)); refill(row, std::move(o.idx0)); refill(col, std::move(o.idx1));
}

void MatrixCOO::fill_cqmat(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_, int pc_,
                           int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_COO, 0, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill_exact(values, std::move(o.values)); refill_exact(row, std::move(o.idx0)); refill_exact(col, std::move(o.idx1));
}

void MatrixCOO::fill_cqmat_stochastic(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_,
                                      int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_COO, 2, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill_exact(values, std::move(o.values)); refill_exact(row, std::move(o.idx0)); refill_exact(col, std::move(o.idx1));
}

// MatrixCOO::normalize_columns (MatrixCOO.cpp:385-393): global columns
void MatrixCOO::normalize_columns() {
  std::vector<double> sum((size_t)std::max(n_col, 0), 0.0);
  for (size_t k = 0; k < values.size(); ++k) sum[(size_t)col[k]] += values[k];
  for (size_t k = 0; k < values.size(); ++k) values[k] /= sum[(size_t)col[k]];
  invalidate_device();
}

// ----------------------------------------------------------------- SCOO
// MatrixSCOO constructors (MatrixSCOO.cpp:14-68).  The reference leaves
// ln_row / ln_col unset in the (n_row, n_col[, n_values]) forms; they are
// n_row / n_col here.
MatrixSCOO::MatrixSCOO(int n_row_, int n_col_, std::vector<double> &values_, std::vector<int> &row_,
                       std::vector<int> &col_)
    : values(values_), row(row_), col(col_) {
  n_row = ln_row = n_row_;
  n_col = ln_col = n_col_;
  f_row = f_col = 0;
  pr = pc = 0;
  NR = NC = 1;
  nnz = (long int)values.size();
}

MatrixSCOO::MatrixSCOO(int n_row_, int n_col_, int n_values) : MatrixSCOO(n_row_, n_col_) {
  values.reserve((size_t)std::max(n_values, 0));
  row.reserve((size_t)std::max(n_values, 0));
  col.reserve((size_t)std::max(n_values, 0));
}

MatrixSCOO::MatrixSCOO(int n_row_, int n_col_) {
  n_row = ln_row = n_row_;
  n_col = ln_col = n_col_;
  f_row = f_col = 0;
  pr = pc = 0;
  NR = NC = 1;
}

MatrixSCOO::MatrixSCOO(const MatrixCOO &m) : values(m.get_values()), row(m.get_row()), col(m.get_col()) {
  n_row = ln_row = m.get_n_row();
  n_col = ln_col = m.get_n_col();
  f_row = m.get_f_row(); f_col = m.get_f_col();
  pr = m.get_pr(); pc = m.get_pc(); NR = m.get_NR(); NC = m.get_NC();
  nnz = m.get_nnz();
}

std::ostream &operator<<(std::ostream &os, const MatrixSCOO &m) { return m.print(os); }

std::ostream &MatrixSCOO::print(std::ostream &os) const {
  detail::print_geometry(os, "----- SCOO ------", TBSLA_GEOMETRY());
  triplet_print(os, values, row, col);
  return os;
}

std::ostream &MatrixSCOO::print_as_dense(std::ostream &os) {
  triplet_dense(os, n_row, n_col, values, row, col);
  return os;
}

std::ostream &MatrixSCOO::print_infos(std::ostream &os) {
  triplet_infos(os, "----- SCOO ------", n_row, n_col, values, row, col);
  return os;
}

std::ostream &MatrixSCOO::print_stats(std::ostream &os) {
  stats(row, col, os, 0);
  return os;
}

std::vector<double> MatrixSCOO::spmv(const std::vector<double> &v, int vect_incr) const {
  std::vector<double> r(n_row, 0.0);
  if (product_is_zero()) return r;
  detail::check(tbsla_spmv_host(device_matrix(), v.data(), (int64_t)v.size(), r.data(), (int64_t)r.size(),
                                vect_incr));
  return r;
}

// MatrixSCOO::Ax (MatrixSCOO.cpp:114-123): r[row + vect_incr - f_row] +=
// value * v[col - f_col]
void MatrixSCOO::Ax(std::vector<double> &r, const std::vector<double> &v, int vect_incr) const {
  if (product_is_zero()) return;
  detail::device_product(device_matrix(), r, v, vect_incr, n_row, true, 0);
}

tbsla_matrix *MatrixSCOO::upload() const { return triplet_upload(n_row, n_col, f_row, f_col, values, row, col); }

bool MatrixSCOO::product_is_zero() const { return values.empty(); }

void MatrixSCOO::array_identity(const void *ptr[3], std::size_t size[3]) const {
  ptr[0] = values.data(); size[0] = values.size();
  ptr[1] = row.data(); size[1] = row.size();
  ptr[2] = col.data(); size[2] = col.size();
}

void MatrixSCOO::push_back(int r, int c, double v) {
  if (r >= n_row || r < 0) return;
  if (c >= n_col || c < 0) return;
  values.push_back(v);
  row.push_back(r);
  col.push_back(c);
}

std::ostream &MatrixSCOO::write(std::ostream &os) {
  detail::write_geometry(os, TBSLA_GEOMETRY());
  detail::write_array(os, values);
  detail::write_array(os, row);
  detail::write_array(os, col);
  return os;
}

std::istream &MatrixSCOO::read(std::istream &is, std::size_t, std::size_t) {
  detail::Geometry g{};
  detail::read_geometry(is, g);
  TBSLA_SET_GEOMETRY(g);
  detail::read_array(is, values);
  detail::read_array(is, row);
  detail::read_array(is, col);
  return is;
}

void MatrixSCOO::fill_cdiag(int n_row_, int n_col_, int cdiag, int pr_, int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_SCOO, 1, n_row_, n_col_, cdiag, 0.0, 0, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill(values, std::move(o.values)); refill(row, std::move(o.idx0)); refill(col, std::move(o.idx1));
}

void MatrixSCOO::fill_cqmat(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_, int pc_,
                            int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_SCOO, 0, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill_exact(values, std::move(o.values)); refill_exact(row, std::move(o.idx0)); refill_exact(col, std::move(o.idx1));
}

void MatrixSCOO::fill_cqmat_stochastic(int n_row_, int n_col_, int c, double q, unsigned int seed_mult, int pr_,
                                       int pc_, int NR_, int NC_) {
  GenArrays o;
  detail::check(generate_arrays(TBSLA_FMT_SCOO, 2, n_row_, n_col_, c, q, seed_mult, pr_, pc_, NR_, NC_, o));
  TBSLA_TAKE_GENERATED(o);
  refill_exact(values, std::move(o.values)); refill_exact(row, std::move(o.idx0)); refill_exact(col, std::move(o.idx1));
}

// MatrixSCOO::normalize_columns (MatrixSCOO.cpp:401-409): columns relative to
// f_col
void MatrixSCOO::normalize_columns() {
  std::vector<double> sum((size_t)std::max(ln_col, 0), 0.0);
  for (size_t k = 0; k < values.size(); ++k) sum[(size_t)(col[k] - f_col)] += values[k];
  for (size_t k = 0; k < values.size(); ++k) values[k] /= sum[(size_t)(col[k] - f_col)];
  invalidate_device();
}

}}  // namespace tbsla::cpp
