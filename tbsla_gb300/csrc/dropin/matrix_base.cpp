// dropin/matrix_base.cpp -- tbsla::cpp::Matrix (src/cpp/matrix/Matrix.cpp):
// the device copy, a_axpx_ and both PageRank drivers on the GPU, and the
// helpers shared by the formats.
#include <algorithm>
#include <mutex>
#include <numeric>

#include "common.h"

namespace tbsla { namespace cpp {

namespace {
// guards the lazily built device copies (products are const and may run
// from several threads; the C ABI serialises each handle's host calls)
std::mutex g_device_mu;
}  // namespace

Matrix::~Matrix() = default;

void Matrix::invalidate_device() const {
  std::lock_guard<std::mutex> lk(g_device_mu);
  device_.reset();
}

tbsla_matrix *Matrix::device_matrix() const {
  std::lock_guard<std::mutex> lk(g_device_mu);
  const void *ptr[3];
  std::size_t size[3];
  array_identity(ptr, size);
  const long geom[12] = {n_row, n_col, f_row, f_col, ln_row, ln_col, pr, pc, NR, NC, nnz, 0};
  if (device_) {
    bool same = true;
    for (int k = 0; k < 3; ++k) same = same && device_->ptr[k] == ptr[k] && device_->size[k] == size[k];
    for (int k = 0; k < 12; ++k) same = same && device_->geom[k] == geom[k];
    if (same) return device_->h;
  }
  auto d = std::make_shared<detail::DeviceCopy>();
  d->h = upload();
  std::copy(ptr, ptr + 3, d->ptr);
  std::copy(size, size + 3, d->size);
  std::copy(geom, geom + 12, d->geom);
  device_ = d;
  return d->h;
}

// Matrix::a_axpx_ (Matrix.cpp:6-11): r = A v; r += v; r = A r.  Square
// matrices take one device call with the "+ v" fused into the first product;
// others compose the two products as the reference does.
std::vector<double> Matrix::a_axpx_(const std::vector<double> &v, int vect_incr) const {
  if (product_is_zero()) return std::vector<double>(n_row, 0.0);
  if (n_row != n_col) {
    std::vector<double> r = spmv(v, vect_incr);
    for (std::size_t i = 0; i < r.size(); ++i) r[i] += v[i];
    return spmv(r, vect_incr);
  }
  std::vector<double> r(n_row, 0.0);
  tbsla_matrix_t *h = device_matrix();
  detail::check(tbsla_a_axpx_host(h, v.data(), (int64_t)v.size(), r.data(), (int64_t)r.size(), vect_incr));
  return r;
}

// Matrix::page_rank (Matrix.cpp:13-61): max-normalised power iteration from
// b = 1, stop when sum |b - b_prev| < epsilon, result divided by its sum.
std::vector<double> Matrix::page_rank(double epsilon, double beta, int max_iteration, int &nb_iterations_done) {
  tbsla_pagerank_params_t p{};
  p.beta = beta;
  p.tol = epsilon;
  p.max_iter = max_iteration;
  p.mode = TBSLA_PR_REFERENCE;
  p.precision = TBSLA_F64;
  tbsla_pagerank_result_t res{};
  std::vector<double> b(n_col, 0.0);
  detail::check(tbsla_pagerank_host(device_matrix(), &p, b.data(), (int64_t)b.size(), &res));
  nb_iterations_done = res.iterations;
  return b;
}

// Matrix::personalized_page_rank (Matrix.cpp:63-114)
std::vector<double> Matrix::personalized_page_rank(double epsilon, double beta, int max_iteration,
                                                   std::vector<int> personalized_nodes, int &nb_iterations_done) {
  tbsla_pagerank_params_t p{};
  p.beta = beta;
  p.tol = epsilon;
  p.max_iter = max_iteration;
  p.mode = TBSLA_PR_REFERENCE;
  p.precision = TBSLA_F64;
  tbsla_pagerank_result_t res{};
  std::vector<double> b(n_col, 0.0);
  detail::check(tbsla_personalized_pagerank_host(device_matrix(), &p, personalized_nodes.data(),
                                                 (int)personalized_nodes.size(), b.data(), (int64_t)b.size(), &res));
  nb_iterations_done = res.iterations;
  return b;
}

namespace detail {

void print_geometry(std::ostream &os, const char *title, const Geometry &g) {
  os << "-----------------" << std::endl;
  os << title << std::endl;
  os << "-----------------" << std::endl;
  os << "number of rows             -  n_row   : " << g.n_row << std::endl;
  os << "number of columns          -  n_col   : " << g.n_col << std::endl;
  os << "local number of rows       -  ln_row  : " << g.ln_row << std::endl;
  os << "local number of columns    -  ln_col  : " << g.ln_col << std::endl;
  os << "first row                  -  f_row   : " << g.f_row << std::endl;
  os << "first column               -  f_col   : " << g.f_col << std::endl;
  os << "number of non-zero elts    -  nnz     : " << g.nnz << std::endl;
  os << "block position (row)       -  pr      : " << g.pr << std::endl;
  os << "block position (column)    -  pc      : " << g.pc << std::endl;
  os << "number of blocks (row)     -  NR      : " << g.NR << std::endl;
  os << "number of blocks (column)  -  NC      : " << g.NC << std::endl;
}

void device_product(tbsla_matrix_t *h, std::vector<double> &r, const std::vector<double> &v, int vect_incr,
                    int n_row, bool accumulate, long rows) {
  const std::size_t n = std::max<std::size_t>(r.size(), (std::size_t)std::max(n_row, 0));
  std::vector<double> t(n, 0.0);
  check(tbsla_spmv_host(h, v.data(), (int64_t)v.size(), t.data(), (int64_t)n, vect_incr));
  if (accumulate) {
    for (std::size_t i = 0; i < r.size(); ++i) r[i] += t[i];
  } else {
    const std::size_t m = std::min<std::size_t>(r.size(), (std::size_t)std::max(rows, 0L));
    std::copy(t.begin(), t.begin() + m, r.begin());
  }
}

std::vector<int64_t> row_col_order(const std::vector<int> &row, const std::vector<int> &col, int n_row) {
  const int64_t n = (int64_t)row.size();
  for (int64_t k = 0; k < n; ++k)
    if (row[k] < 0 || row[k] >= n_row)
      throw std::out_of_range("tbsla_gb300: COO row index " + std::to_string(row[k]) + " outside [0, " +
                              std::to_string(n_row) + ")");
  // counting sort by row (stable), then a stable sort by column per row
  std::vector<int64_t> start((size_t)n_row + 1, 0);
  for (int64_t k = 0; k < n; ++k) ++start[(size_t)row[k] + 1];
  std::partial_sum(start.begin(), start.end(), start.begin());
  std::vector<int64_t> p((size_t)n), next(start.begin(), start.end() - 1);
  for (int64_t k = 0; k < n; ++k) p[(size_t)next[(size_t)row[k]]++] = k;
  #pragma omp parallel for schedule(dynamic, 4096)
  for (int64_t i = 0; i < (int64_t)n_row; ++i) {
    auto b = p.begin() + start[(size_t)i], e = p.begin() + start[(size_t)i + 1];
    if (e - b > 1) std::stable_sort(b, e, [&](int64_t x, int64_t y) { return col[(size_t)x] < col[(size_t)y]; });
  }
  return p;
}

}  // namespace detail
}}  // namespace tbsla::cpp
