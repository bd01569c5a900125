// dropin/c_interface.cpp -- the C_CPP_* C ABI of TBSLA
// (src/cpp/interface/c/matrix/*.cpp) over the GPU-backed drop-in classes.
// Exceptions do not cross the C boundary: a failing product prints the
// library's message on stderr and returns an empty vector.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <numeric>
#include <string>

#include <tbsla/cpp/MatrixCOO.h>
#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.h>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.h>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.h>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.h>
#include <tbsla/cpp/MatrixSCOO.hpp>
#include <tbsla/cpp/Vector.h>
#include <tbsla/cpp/utils/vector.hpp>

namespace {
std::vector<double> *vec(C_CPP_Vector_t *v) { return static_cast<std::vector<double> *>(v->obj); }
}  // namespace

// ---------------------------------------------------------------- vectors
extern "C" {

C_CPP_Vector_t *C_CPP_Vector_create() {
  C_CPP_Vector_t *v = static_cast<C_CPP_Vector_t *>(std::malloc(sizeof(C_CPP_Vector_t)));
  v->obj = new std::vector<double>();
  return v;
}

void C_CPP_Vector_destroy(C_CPP_Vector_t *v) {
  if (!v) return;
  delete vec(v);
  std::free(v);
}

void C_CPP_Vector_print(C_CPP_Vector_t *v) {
  if (!v) {
    std::printf("C_CPP_Vector_print : input vector is NULL\n");
    return;
  }
  tbsla::utils::vector::streamvector<double>(std::cout, "v", *vec(v));
  std::cout << std::endl << std::flush;
}

void C_CPP_Vector_set(C_CPP_Vector_t *v, void *obj) {
  if (v) v->obj = obj;
}

void C_CPP_Vector_copy(C_CPP_Vector_t *v, void *obj) {
  if (!v) return;
  *vec(v) = *static_cast<std::vector<double> *>(obj);
}

void C_CPP_Vector_fill(C_CPP_Vector_t *v, int n, int s) {
  if (!v) return;
  std::vector<double> &x = *vec(v);
  x.assign((size_t)std::max(n, 0), 0.0);
  std::iota(x.begin(), x.end(), (double)s);
}

bool C_CPP_Vector_read(C_CPP_Vector_t *v, char *filename, int seek) {
  if (!v) return false;
  std::ifstream is(filename, std::ifstream::binary);
  if (!is.is_open()) return false;
  is.seekg(seek, is.beg);
  size_t n = 0;
  is.read(reinterpret_cast<char *>(&n), sizeof(n));
  vec(v)->resize(n);
  is.read(reinterpret_cast<char *>(vec(v)->data()), (std::streamsize)(n * sizeof(double)));
  return true;
}

bool C_CPP_Vector_write(C_CPP_Vector_t *v, char *filename) {
  if (!v) return false;
  std::ofstream os(filename, std::ofstream::binary | std::ofstream::app);
  if (!os.is_open()) return false;
  const size_t n = vec(v)->size();
  os.write(reinterpret_cast<const char *>(&n), sizeof(n));
  os.write(reinterpret_cast<const char *>(vec(v)->data()), (std::streamsize)(n * sizeof(double)));
  return true;
}

bool C_CPP_Vector_add(C_CPP_Vector_t *v1, C_CPP_Vector_t *v2) {
  if (!v1 || !v2) return false;
  std::vector<double> &a = *vec(v1);
  const std::vector<double> &b = *vec(v2);
  for (size_t i = 0; i < a.size(); ++i) a[i] += b[i];
  return true;
}

bool C_CPP_Vector_add_incr(C_CPP_Vector_t *v1, C_CPP_Vector_t *v2, int incr) {
  if (!v1 || !v2) return false;
  std::vector<double> &a = *vec(v1);
  const std::vector<double> &b = *vec(v2);
  for (size_t i = 0; i < a.size(); ++i) a[i] += b[i + (size_t)incr];
  return true;
}

bool C_CPP_Vector_gather(C_CPP_Vector_t *v1, C_CPP_Vector_t *v2) {
  if (!v1 || !v2) return false;
  vec(v1)->insert(vec(v1)->end(), vec(v2)->begin(), vec(v2)->end());
  return true;
}

}  // extern "C"

// ---------------------------------------------------------------- matrices
#define TBSLA_C_MATRIX(F)                                                                                 \
  struct C_CPP_Matrix##F {                                                                                \
    void *obj;                                                                                            \
  };                                                                                                      \
  extern "C" {                                                                                            \
  C_CPP_Matrix##F##_t *C_CPP_Matrix##F##_create() {                                                       \
    C_CPP_Matrix##F##_t *m = static_cast<C_CPP_Matrix##F##_t *>(std::malloc(sizeof(C_CPP_Matrix##F##_t))); \
    m->obj = new tbsla::cpp::Matrix##F();                                                                 \
    return m;                                                                                             \
  }                                                                                                       \
  void C_CPP_Matrix##F##_destroy(C_CPP_Matrix##F##_t *m) {                                                \
    if (!m) return;                                                                                       \
    delete static_cast<tbsla::cpp::Matrix##F *>(m->obj);                                                  \
    std::free(m);                                                                                         \
  }                                                                                                       \
  void C_CPP_Matrix##F##_fill_cdiag(C_CPP_Matrix##F##_t *m, int n_row, int n_col, int cdiag, int pr,       \
                                    int pc, int NR, int NC) {                                             \
    if (m) static_cast<tbsla::cpp::Matrix##F *>(m->obj)->fill_cdiag(n_row, n_col, cdiag, pr, pc, NR, NC);  \
  }                                                                                                       \
  void C_CPP_Matrix##F##_fill_cqmat(C_CPP_Matrix##F##_t *m, int n_row, int n_col, int c, double q,         \
                                    unsigned int seed_mult, int pr, int pc, int NR, int NC) {             \
    if (m)                                                                                                \
      static_cast<tbsla::cpp::Matrix##F *>(m->obj)->fill_cqmat(n_row, n_col, c, q, seed_mult, pr, pc, NR, \
                                                                NC);                                      \
  }                                                                                                       \
  bool C_CPP_Matrix##F##_read(C_CPP_Matrix##F##_t *m, char *filename, int seek) {                         \
    if (!m) return false;                                                                                 \
    std::ifstream is(filename, std::ifstream::binary);                                                    \
    if (!is.is_open()) return false;                                                                      \
    is.seekg(seek, is.beg);                                                                               \
    static_cast<tbsla::cpp::Matrix##F *>(m->obj)->read(is);                                               \
    return true;                                                                                          \
  }                                                                                                       \
  bool C_CPP_Matrix##F##_write(C_CPP_Matrix##F##_t *m, char *filename) {                                  \
    if (!m) return false;                                                                                 \
    std::ofstream os(filename, std::ofstream::binary | std::ofstream::app);                               \
    if (!os.is_open()) return false;                                                                      \
    static_cast<tbsla::cpp::Matrix##F *>(m->obj)->write(os);                                              \
    return true;                                                                                          \
  }                                                                                                       \
  void C_CPP_Matrix##F##_print(C_CPP_Matrix##F##_t *m) {                                                  \
    if (!m) return;                                                                                       \
    tbsla::cpp::Matrix##F *o = static_cast<tbsla::cpp::Matrix##F *>(m->obj);                              \
    o->print_infos(std::cerr);                                                                            \
    std::cerr << *o << std::endl;                                                                         \
  }                                                                                                       \
  C_CPP_Vector_t *C_CPP_Matrix##F##_spmv(C_CPP_Matrix##F##_t *m, C_CPP_Vector_t *v) {                     \
    C_CPP_Vector_t *r = C_CPP_Vector_create();                                                            \
    if (!m || !v) return r;                                                                               \
    try {                                                                                                 \
      *vec(r) = static_cast<tbsla::cpp::Matrix##F *>(m->obj)->spmv(*vec(v), 0);                           \
    } catch (const std::exception &e) {                                                                   \
      std::fprintf(stderr, "C_CPP_Matrix" #F "_spmv: %s\n", e.what());                                    \
      vec(r)->clear();                                                                                    \
    }                                                                                                     \
    return r;                                                                                             \
  }                                                                                                       \
  }

TBSLA_C_MATRIX(COO)
TBSLA_C_MATRIX(SCOO)
TBSLA_C_MATRIX(CSR)
TBSLA_C_MATRIX(ELL)
TBSLA_C_MATRIX(DENSE)
