// ref_harness.cpp -- extern "C" access to the TBSLA reference classes.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// the reference's own sources (src/cpp/matrix/*.cpp and src/cpp/utils/*.cpp,
// read where they lie, never copied) into oracle/_ref/libtbsla_ref.so.  The
// tests use it to pin the C restatement in tbsla_oracle.c, and
// tests/golden/make_golden.py uses it to write the golden vectors.  Matrices
// are handed back through the reference's own binary writer
// (Matrix*::write, e.g. src/cpp/matrix/MatrixCSR.cpp:179-204).
#include <tbsla/cpp/Matrix.hpp>
#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>

#include <cstring>
#include <sstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using tbsla::cpp::Matrix;

namespace {
enum { COO = 0, SCOO = 1, CSR = 2, ELL = 3, DENSE = 4 };

Matrix *make(int fmt) {
  switch (fmt) {
  case COO: return new tbsla::cpp::MatrixCOO();
  case SCOO: return new tbsla::cpp::MatrixSCOO();
  case CSR: return new tbsla::cpp::MatrixCSR();
  case ELL: return new tbsla::cpp::MatrixELL();
  case DENSE: return new tbsla::cpp::MatrixDENSE();
  }
  return nullptr;
}
}  // namespace

extern "C" {

void ref_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : 1);
#else
  (void)n;
#endif
}

void *ref_new(int fmt) { return make(fmt); }
// Matrix has no virtual destructor and is a virtual base, so objects are
// deleted through their concrete type.
void ref_delete(void *p, int fmt) {
  Matrix *m = static_cast<Matrix *>(p);
  switch (fmt) {
  case COO: delete dynamic_cast<tbsla::cpp::MatrixCOO *>(m); break;
  case SCOO: delete dynamic_cast<tbsla::cpp::MatrixSCOO *>(m); break;
  case CSR: delete dynamic_cast<tbsla::cpp::MatrixCSR *>(m); break;
  case ELL: delete dynamic_cast<tbsla::cpp::MatrixELL *>(m); break;
  case DENSE: delete dynamic_cast<tbsla::cpp::MatrixDENSE *>(m); break;
  }
}

void ref_fill_cqmat(void *m, int nr, int nc, int c, double q, unsigned s, int pr, int pc, int NR, int NC) {
  static_cast<Matrix *>(m)->fill_cqmat(nr, nc, c, q, s, pr, pc, NR, NC);
}
void ref_fill_cqmat_stochastic(void *m, int nr, int nc, int c, double q, unsigned s, int pr, int pc,
                               int NR, int NC) {
  static_cast<Matrix *>(m)->fill_cqmat_stochastic(nr, nc, c, q, s, pr, pc, NR, NC);
}
void ref_fill_cdiag(void *m, int nr, int nc, int cd, int pr, int pc, int NR, int NC) {
  static_cast<Matrix *>(m)->fill_cdiag(nr, nc, cd, pr, pc, NR, NC);
}
void ref_normalize_columns(void *m) { static_cast<Matrix *>(m)->normalize_columns(); }

// MatrixCOO / MatrixSCOO (values,row,col) and MatrixCSR (values,rowptr,colidx)
void *ref_from_arrays(int fmt, int nr, int nc, const double *v, long nv, const int *a, long na,
                      const int *b, long nb) {
  std::vector<double> vv(v, v + nv);
  std::vector<int> aa(a, a + na), bb(b, b + nb);
  // every handle is a Matrix* (the virtual base sits at an offset)
  Matrix *m = nullptr;
  switch (fmt) {
  case COO: m = new tbsla::cpp::MatrixCOO(nr, nc, vv, aa, bb); break;
  case SCOO: m = new tbsla::cpp::MatrixSCOO(nr, nc, vv, aa, bb); break;
  case CSR: m = new tbsla::cpp::MatrixCSR(nr, nc, vv, aa, bb); break;
  }
  return m;
}
void ref_update_nnz(void *coo) { dynamic_cast<tbsla::cpp::MatrixCOO *>(static_cast<Matrix *>(coo))->update_nnz(); }

void *ref_convert(void *coo, int fmt) {
  const tbsla::cpp::MatrixCOO &c = *dynamic_cast<tbsla::cpp::MatrixCOO *>(static_cast<Matrix *>(coo));
  Matrix *m = nullptr;
  switch (fmt) {
  case SCOO: m = new tbsla::cpp::MatrixSCOO(c); break;
  case CSR: m = new tbsla::cpp::MatrixCSR(c); break;
  case ELL: m = new tbsla::cpp::MatrixELL(c); break;
  case DENSE: m = new tbsla::cpp::MatrixDENSE(c); break;
  }
  return m;
}

// Serialises with the reference's writer; returns the byte count and copies
// at most cap bytes into buf.
long ref_serialize(void *m, char *buf, long cap) {
  std::ostringstream os(std::ios::binary);
  static_cast<Matrix *>(m)->write(os);
  std::string s = os.str();
  if (buf && cap > 0) std::memcpy(buf, s.data(), (size_t)std::min<long>(cap, (long)s.size()));
  return (long)s.size();
}

// Reads the reference binary format (Matrix*::read) into a new matrix.
void *ref_deserialize(int fmt, const char *buf, long n) {
  Matrix *m = make(fmt);
  std::istringstream is(std::string(buf, (size_t)n), std::ios::binary);
  m->read(is);
  return m;
}

// MatrixCOO::readMM (MatrixCOO.cpp:230-292) into a new COO matrix; NULL when
// the reader throws (kinds it refuses)
void *ref_read_mm(const char *path) {
  auto *m = new tbsla::cpp::MatrixCOO();
  try {
    m->readMM(path);
  } catch (...) {
    delete m;
    return nullptr;
  }
  return static_cast<Matrix *>(m);
}

long ref_get_nnz(void *m) { return static_cast<Matrix *>(m)->get_nnz(); }
int ref_get_n_row(void *m) { return static_cast<Matrix *>(m)->get_n_row(); }
int ref_get_n_col(void *m) { return static_cast<Matrix *>(m)->get_n_col(); }

void ref_spmv(void *m, const double *v, long nv, double *r, int vect_incr) {
  std::vector<double> vv(v, v + nv);
  std::vector<double> rr = static_cast<Matrix *>(m)->spmv(vv, vect_incr);
  std::memcpy(r, rr.data(), rr.size() * sizeof(double));
}

void ref_a_axpx(void *m, const double *v, long nv, double *r) {
  std::vector<double> vv(v, v + nv);
  std::vector<double> rr = static_cast<Matrix *>(m)->a_axpx_(vv, 0);
  std::memcpy(r, rr.data(), rr.size() * sizeof(double));
}

int ref_page_rank(void *m, double epsilon, double beta, int max_it, double *out) {
  int it = 0;
  std::vector<double> b = static_cast<Matrix *>(m)->page_rank(epsilon, beta, max_it, it);
  std::memcpy(out, b.data(), b.size() * sizeof(double));
  return it;
}

int ref_personalized_page_rank(void *m, double epsilon, double beta, int max_it, const int *nodes,
                               int n_nodes, double *out) {
  int it = 0;
  std::vector<int> nn(nodes, nodes + n_nodes);
  std::vector<double> b = static_cast<Matrix *>(m)->personalized_page_rank(epsilon, beta, max_it, nn, it);
  std::memcpy(out, b.data(), b.size() * sizeof(double));
  return it;
}

}  // extern "C"
