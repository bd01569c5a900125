// Drop-in C++ API on the GPU: the tbsla::cpp classes and the C_CPP_* ABI,
// checked the way TBSLA's own tests check the reference
// (src/cpp/tests/csr.cpp, coo.cpp, test_spmv_cdiag.cpp,
// test_a_axpx__cdiag.cpp, test_spmv_cqmat.cpp, test_page_rank.cpp,
// test_personalized_page_rank.cpp): known answers, closed-form cdiag
// products, exact cross-format equality on integer-valued products, PageRank
// across formats; plus binary and Matrix Market round trips.
// Usage: test_dropin <scratch dir>.  Prints one line per failure; exit code
// = number of failures.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <functional>
#include <iostream>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include <tbsla/cpp/MatrixCOO.h>
#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.h>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>
#include <tbsla/cpp/Vector.h>
#include <tbsla/cpp/utils/vector.hpp>

using namespace tbsla::cpp;

static int failures = 0;
static void expect(bool ok, const std::string &what) {
  if (!ok) {
    ++failures;
    std::cout << "FAIL " << what << std::endl;
  }
}

static std::vector<double> iota_vec(int n, double start = 0) {
  std::vector<double> v((size_t)n);
  for (int i = 0; i < n; ++i) v[(size_t)i] = start + i;
  return v;
}

// every format of one matrix: filled directly (fill) and converted from COO
static std::vector<std::pair<std::string, std::unique_ptr<Matrix>>> all_formats(
    const std::function<void(Matrix &)> &fill) {
  std::vector<std::pair<std::string, std::unique_ptr<Matrix>>> out;
  auto coo = std::make_unique<MatrixCOO>();
  fill(*coo);
  out.emplace_back("SCOO<-COO", std::make_unique<MatrixSCOO>(*coo));
  out.emplace_back("CSR<-COO", std::make_unique<MatrixCSR>(*coo));
  out.emplace_back("ELL<-COO", std::make_unique<MatrixELL>(*coo));
  out.emplace_back("DENSE<-COO", std::make_unique<MatrixDENSE>(*coo));
  std::unique_ptr<Matrix> f[5] = {std::make_unique<MatrixSCOO>(), std::make_unique<MatrixCSR>(),
                                  std::make_unique<MatrixELL>(), std::make_unique<MatrixDENSE>(), nullptr};
  const char *names[4] = {"SCOO", "CSR", "ELL", "DENSE"};
  for (int k = 0; k < 4; ++k) {
    fill(*f[k]);
    out.emplace_back(names[k], std::move(f[k]));
  }
  out.emplace_back("COO", std::move(coo));
  return out;
}

static void known_answers() {
  // the 5 x 5 matrix of src/cpp/tests/csr.cpp and coo.cpp, x = 1..5
  std::vector<double> values{1, 2, 3, 4, 5, 6, 7, 8, 9, 10};
  std::vector<int> rowptr{0, 3, 4, 5, 7, 10};
  std::vector<int> colidx{0, 1, 4, 2, 1, 1, 3, 0, 2, 4};
  std::vector<double> x{1, 2, 3, 4, 5}, expected{20, 12, 10, 40, 85};
  MatrixCSR csr(5, 5, values, rowptr, colidx);
  expect(csr.spmv(x) == expected, "known answer CSR");
  // the same entries as unsorted triplets
  std::vector<double> tv{10, 4, 1, 7, 3, 8, 2, 6, 9, 5};
  std::vector<int> tr{4, 1, 0, 3, 0, 4, 0, 3, 4, 2};
  std::vector<int> tc{4, 2, 0, 3, 4, 0, 1, 1, 2, 1};
  MatrixCOO coo(5, 5, tv, tr, tc);
  coo.update_nnz();
  expect(coo.spmv(x) == expected, "known answer COO");
  expect(MatrixCSR(coo).spmv(x) == expected, "known answer CSR(COO)");
  expect(MatrixELL(coo).spmv(x) == expected, "known answer ELL(COO)");
  expect(MatrixSCOO(coo).spmv(x) == expected, "known answer SCOO(COO)");
  expect(MatrixDENSE(coo).spmv(x) == expected, "known answer DENSE(COO)");
  // CSR(COO) gives the reference's sorted arrays
  std::ostringstream a, b;
  MatrixCSR(coo).print(a);
  MatrixCSR sorted(5, 5, values, rowptr, colidx);
  sorted.print(b);
  expect(a.str().find("values : 1, 2, 3, 4, 5, 6, 7, 8, 9, 10") != std::string::npos, "CSR(COO) values order");
  expect(a.str().find("colidx : 0, 1, 4, 2, 1, 1, 3, 0, 2, 4") != std::string::npos, "CSR(COO) colidx order");
  // Ax accumulates for COO and overwrites for CSR
  std::vector<double> r(5, 1.0);
  coo.Ax(r, x);
  expect(r == std::vector<double>({21, 13, 11, 41, 86}), "COO Ax accumulates");
  r.assign(5, 1.0);
  csr.Ax(r, x);
  expect(r == expected, "CSR Ax overwrites");
  // COO push_back drops out-of-range entries
  MatrixCOO p(3, 3);
  p.push_back(0, 0, 1.0);
  p.push_back(3, 0, 1.0);
  p.push_back(0, -1, 1.0);
  p.update_nnz();
  expect(p.get_nnz() == 1, "push_back range filter");
}

static void cdiag_closed_forms() {
  const int shapes[6][2] = {{10, 10}, {5, 10}, {10, 5}, {30, 30}, {20, 30}, {30, 20}};
  for (auto &s : shapes)
    for (int c = 0; c <= 12; ++c) {
      auto ms = all_formats([&](Matrix &m) { m.fill_cdiag(s[0], s[1], c); });
      for (auto &nm : ms) {
        Matrix &m = *nm.second;
        std::vector<double> v = iota_vec(m.get_n_col());
        std::vector<double> r = m.spmv(v);
        const int rc = tbsla::utils::vector::test_spmv_cdiag(m.get_n_row(), m.get_n_col(), c, v, r, false);
        expect(rc == 0, "cdiag spmv " + nm.first + " " + std::to_string(s[0]) + "x" + std::to_string(s[1]) +
                            " c=" + std::to_string(c) + " code " + std::to_string(rc));
        if (s[0] == s[1]) {
          std::vector<double> w(v.size());
          for (size_t i = 0; i < v.size(); ++i) w[i] = 2.0 * (double)i + 1.0;
          std::vector<double> ra = m.a_axpx_(w);
          const int ra_rc = tbsla::utils::vector::test_a_axpx__cdiag(m.get_n_row(), m.get_n_col(), c, w, ra, false);
          expect(ra_rc == 0, "cdiag a_axpx_ " + nm.first + " n=" + std::to_string(s[0]) + " c=" + std::to_string(c));
        }
      }
    }
}

static void cqmat_cross_format() {
  const int shapes[4][3] = {{100, 100, 10}, {150, 100, 12}, {100, 150, 7}, {1000, 1000, 16}};
  for (auto &s : shapes)
    for (int seed : {0, 1, 11}) {
      auto ms = all_formats([&](Matrix &m) { m.fill_cqmat(s[0], s[1], s[2], 0.1, (unsigned)seed); });
      std::vector<double> v = iota_vec(s[1]);
      const std::vector<double> ref = ms.back().second->spmv(v);  // COO
      for (auto &nm : ms)
        expect(nm.second->spmv(v) == ref, "cqmat cross-format " + nm.first + " " + std::to_string(s[0]) + "x" +
                                              std::to_string(s[1]) + " seed " + std::to_string(seed));
    }
}

static double l1(const std::vector<double> &a, const std::vector<double> &b) {
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i) s += std::fabs(a[i] - b[i]);
  return s;
}

static void pagerank_cross_format() {
  for (int n : {100, 1000}) {
    auto ms = all_formats([&](Matrix &m) { m.fill_cqmat_stochastic(n, n, 8, 0.1, 3); });
    int it_ref = 0, pit_ref = 0;
    const std::vector<double> ref = ms.back().second->page_rank(1e-10, 0.85, 500, it_ref);
    const std::vector<int> nodes{1, 5, 5, n - 1};
    const std::vector<double> pref = ms.back().second->personalized_page_rank(1e-10, 0.85, 500, nodes, pit_ref);
    double sum = 0;
    for (double x : ref) sum += x;
    expect(std::fabs(sum - 1.0) < 1e-12 && it_ref > 1, "page_rank normalised n=" + std::to_string(n));
    for (auto &nm : ms) {
      int it = 0, pit = 0;
      const std::vector<double> b = nm.second->page_rank(1e-10, 0.85, 500, it);
      const std::vector<double> pb = nm.second->personalized_page_rank(1e-10, 0.85, 500, nodes, pit);
      // formats sum in different orders: the stopping test may cross 1e-10
      // one sweep apart, which moves the vector by about that much
      const double tb = it == it_ref ? 1e-12 : 1e-9, tp = pit == pit_ref ? 1e-12 : 1e-9;
      expect(std::abs(it - it_ref) <= 1 && l1(b, ref) < tb, "page_rank " + nm.first + " n=" + std::to_string(n));
      expect(std::abs(pit - pit_ref) <= 1 && l1(pb, pref) < tp, "personalized_page_rank " + nm.first);
    }
  }
}

static void binary_round_trip(const std::string &dir) {
  auto ms = all_formats([&](Matrix &m) { m.fill_cqmat(300, 250, 9, 0.2, 5); });
  const std::vector<double> v = iota_vec(250);
  for (auto &nm : ms) {
    const std::string path = dir + "/m_" + nm.first.substr(0, nm.first.find('<')) + ".bin";
    std::remove(path.c_str());
    {
      std::ofstream os(path, std::ofstream::binary);
      nm.second->write(os);
    }
    std::unique_ptr<Matrix> back;
    const std::string f = nm.first.substr(0, nm.first.find('<'));
    if (f == "COO") back = std::make_unique<MatrixCOO>();
    else if (f == "SCOO") back = std::make_unique<MatrixSCOO>();
    else if (f == "CSR") back = std::make_unique<MatrixCSR>();
    else if (f == "ELL") back = std::make_unique<MatrixELL>();
    else back = std::make_unique<MatrixDENSE>();
    std::ifstream is(path, std::ifstream::binary);
    back->read(is);
    std::ostringstream a, b;
    nm.second->print(a);
    back->print(b);
    expect(a.str() == b.str(), "binary round trip arrays " + nm.first);
    expect(back->spmv(v) == nm.second->spmv(v), "binary round trip product " + nm.first);
    expect(back->get_nnz() == nm.second->get_nnz(), "binary round trip nnz " + nm.first);
  }
}

static void matrix_market(const std::string &dir) {
  const std::string g = dir + "/general.mtx", s = dir + "/symmetric.mtx", bad = dir + "/array.mtx";
  {
    std::ofstream o(g);
    o << "%%MatrixMarket matrix coordinate real general\n% comment\n3 4 4\n1 1 2.5\n3 4 -1\n2 2 4\n1 4 1\n";
    std::ofstream p(s);
    p << "%%MatrixMarket matrix coordinate real symmetric\n3 3 3\n1 1 2\n3 1 5\n2 2 1\n";
    std::ofstream q(bad);
    q << "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n";
  }
  MatrixCOO a;
  a.readMM(g);
  expect(a.get_n_row() == 3 && a.get_n_col() == 4 && a.get_nnz() == 4, "readMM general shape");
  expect(a.spmv({1, 2, 3, 4}) == std::vector<double>({6.5, 8, -4}), "readMM general product");
  MatrixCOO b;
  b.readMM(s);
  expect(b.get_nnz() == 4, "readMM symmetric mirrors off-diagonal entries");
  expect(MatrixCSR(b).spmv({1, 1, 1}) == std::vector<double>({7, 1, 5}), "readMM symmetric product");
  bool thrown = false;
  try {
    MatrixCOO c;
    c.readMM(bad);
  } catch (const MatrixFormatReadException &) {
    thrown = true;
  }
  expect(thrown, "readMM rejects array files");
}

static void c_abi(const std::string &dir) {
  C_CPP_MatrixCSR_t *m = C_CPP_MatrixCSR_create();
  C_CPP_MatrixCSR_fill_cqmat(m, 200, 200, 10, 0.1, 1, 0, 0, 1, 1);
  C_CPP_Vector_t *v = C_CPP_Vector_create();
  C_CPP_Vector_fill(v, 200, 0);
  C_CPP_Vector_t *r = C_CPP_MatrixCSR_spmv(m, v);
  MatrixCOO coo;
  coo.fill_cqmat(200, 200, 10, 0.1, 1);
  const std::vector<double> expected = coo.spmv(iota_vec(200));
  expect(*static_cast<std::vector<double> *>(r->obj) == expected, "C_CPP_MatrixCSR_spmv");
  const std::string path = dir + "/c_abi.bin";
  std::remove(path.c_str());
  std::vector<char> name(path.begin(), path.end());
  name.push_back('\0');
  expect(C_CPP_MatrixCSR_write(m, name.data()), "C_CPP_MatrixCSR_write");
  C_CPP_MatrixCSR_t *m2 = C_CPP_MatrixCSR_create();
  expect(C_CPP_MatrixCSR_read(m2, name.data(), 0), "C_CPP_MatrixCSR_read");
  C_CPP_Vector_t *r2 = C_CPP_MatrixCSR_spmv(m2, v);
  expect(*static_cast<std::vector<double> *>(r2->obj) == expected, "C_CPP read back product");
  C_CPP_Vector_t *e = C_CPP_MatrixCSR_spmv(nullptr, v);
  expect(static_cast<std::vector<double> *>(e->obj)->empty(), "C_CPP NULL matrix gives an empty vector");
  expect(!C_CPP_MatrixCSR_read(nullptr, name.data(), 0), "C_CPP NULL read is false");
  C_CPP_Vector_t *s = C_CPP_Vector_create();
  C_CPP_Vector_fill(s, 3, 5);
  C_CPP_Vector_t *t = C_CPP_Vector_create();
  C_CPP_Vector_fill(t, 4, 1);
  C_CPP_Vector_add_incr(s, t, 1);
  expect(*static_cast<std::vector<double> *>(s->obj) == std::vector<double>({7, 9, 11}), "C_CPP_Vector_add_incr");
  C_CPP_Vector_gather(s, t);
  expect(static_cast<std::vector<double> *>(s->obj)->size() == 7, "C_CPP_Vector_gather");
  for (C_CPP_Vector_t *x : {v, r, r2, e, s, t}) C_CPP_Vector_destroy(x);
  C_CPP_MatrixCSR_destroy(m);
  C_CPP_MatrixCSR_destroy(m2);
}

static void mutation_rebuilds_device_copy() {
  MatrixCSR m;
  m.fill_cqmat(500, 500, 8, 0.1, 2);
  const std::vector<double> v = iota_vec(500);
  const std::vector<double> before = m.spmv(v);
  m.normalize_columns();  // in place: the device copy must follow
  MatrixCOO c;
  c.fill_cqmat(500, 500, 8, 0.1, 2);
  c.normalize_columns();
  const std::vector<double> after = m.spmv(v), ref = c.spmv(v);
  expect(after != before, "normalize_columns changes the product");
  expect(l1(after, ref) < 1e-9, "normalize_columns CSR vs COO");
  m.fill_cqmat(300, 300, 4, 0.0, 1);  // refill with other sizes
  expect(m.spmv(iota_vec(300)).size() == 300, "refill rebuilds the device copy");
}

// A second fill or read of the same shape reuses the arrays' buffers (same
// data pointers and sizes); the product after it must be the new matrix's,
// equal to a fresh object's holding the same fill.
static std::unique_ptr<Matrix> make_format(const std::string &f) {
  if (f == "COO") return std::make_unique<MatrixCOO>();
  if (f == "SCOO") return std::make_unique<MatrixSCOO>();
  if (f == "CSR") return std::make_unique<MatrixCSR>();
  if (f == "ELL") return std::make_unique<MatrixELL>();
  return std::make_unique<MatrixDENSE>();
}

static void refill_same_shape(const std::string &dir) {
  const std::vector<double> v = iota_vec(400);
  using Fill = std::function<void(Matrix &)>;
  const std::pair<const char *, Fill> fills[] = {
      {"cqmat seed 1", [](Matrix &m) { m.fill_cqmat(400, 400, 8, 0.1, 1); }},
      {"cqmat seed 2", [](Matrix &m) { m.fill_cqmat(400, 400, 8, 0.1, 2); }},
      {"cqmat_stochastic seed 2", [](Matrix &m) { m.fill_cqmat_stochastic(400, 400, 8, 0.1, 2); }},
      {"cdiag 3", [](Matrix &m) { m.fill_cdiag(400, 400, 3); }},
      {"cdiag 5", [](Matrix &m) { m.fill_cdiag(400, 400, 5); }},
      {"cqmat seed 3", [](Matrix &m) { m.fill_cqmat(400, 400, 8, 0.1, 3); }}};
  for (const char *f : {"COO", "SCOO", "CSR", "ELL", "DENSE"}) {
    auto m = make_format(f);
    std::vector<double> prev;
    for (const auto &fl : fills) {
      fl.second(*m);
      const std::vector<double> got = m->spmv(v);
      auto fresh = make_format(f);
      fl.second(*fresh);
      expect(got == fresh->spmv(v), std::string("refill ") + f + " " + fl.first);
      expect(got != prev, std::string("refill changes the product ") + f + " " + fl.first);
      prev = got;
    }
    // read() of two files of the same shape into one object
    const std::string p1 = dir + "/refill_a_" + f + ".bin", p2 = dir + "/refill_b_" + f + ".bin";
    auto a = make_format(f), b = make_format(f);
    a->fill_cqmat(400, 400, 8, 0.1, 4);
    b->fill_cqmat(400, 400, 8, 0.1, 5);
    for (auto &pm : {std::make_pair(&p1, a.get()), std::make_pair(&p2, b.get())}) {
      std::remove(pm.first->c_str());
      std::ofstream os(*pm.first, std::ofstream::binary);
      pm.second->write(os);
    }
    auto r = make_format(f);
    {
      std::ifstream is(p1, std::ifstream::binary);
      r->read(is);
    }
    expect(r->spmv(v) == a->spmv(v), std::string("read first file ") + f);
    {
      std::ifstream is(p2, std::ifstream::binary);
      r->read(is);
    }
    expect(r->spmv(v) == b->spmv(v), std::string("read second file of the same shape ") + f);
  }
}

int main(int argc, char **argv) {
  const std::string dir = argc > 1 ? argv[1] : ".";
  const std::pair<const char *, std::function<void()>> sections[] = {
      {"known_answers", known_answers},
      {"cdiag_closed_forms", cdiag_closed_forms},
      {"cqmat_cross_format", cqmat_cross_format},
      {"pagerank_cross_format", pagerank_cross_format},
      {"binary_round_trip", [&] { binary_round_trip(dir); }},
      {"matrix_market", [&] { matrix_market(dir); }},
      {"c_abi", [&] { c_abi(dir); }},
      {"mutation_rebuilds_device_copy", mutation_rebuilds_device_copy},
      {"refill_same_shape", [&] { refill_same_shape(dir); }}};
  for (const auto &sec : sections) {
    try {
      sec.second();
    } catch (const std::exception &ex) {
      std::cout << "FAIL " << sec.first << " exception: " << ex.what() << std::endl;
      ++failures;
    }
  }
  std::cout << (failures ? "FAILED " : "OK ") << failures << std::endl;
  return failures > 255 ? 255 : failures;
}
