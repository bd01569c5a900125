// dropin/io.cpp -- files straight into device handles: the reference's binary
// matrix layout (Matrix*::read, e.g. MatrixCSR.cpp:206-232) and Matrix
// Market files (MatrixCOO::readMM, MatrixCOO.cpp:230-292), converted to the
// requested format as the reference's constructors do (MatrixCSR(COO),
// MatrixELL(COO), MatrixSCOO(COO), MatrixDENSE(COO)).
#include <fstream>

#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>

#include "common.h"

namespace tbsla {
tbsla_status_t fail(tbsla_status_t s, const char *fmt, ...);
}

namespace {

using namespace tbsla::cpp;

// each format's device handle from its host arrays (the classes' upload)
template <typename M> struct Handle : M {
  using M::M;
  tbsla_matrix_t *make() const { return this->upload(); }
};

template <typename M> tbsla_status_t from_file(std::istream &is, tbsla_matrix_t **out) {
  Handle<M> m;
  m.read(is);
  if (is.fail()) return tbsla::fail(TBSLA_ERR_INVALID_ARG, "the file ends inside the matrix");
  *out = m.make();
  return TBSLA_OK;
}

template <typename M> tbsla_status_t from_coo(const MatrixCOO &c, tbsla_matrix_t **out) {
  Handle<M> m(c);
  *out = m.make();
  return TBSLA_OK;
}

struct CooHandle : MatrixCOO {
  tbsla_matrix_t *make() const { return this->upload(); }
};

}  // namespace

extern "C" {

tbsla_status_t tbsla_matrix_read_file(const char *path, int format, int64_t seek, tbsla_matrix_t **out) {
  if (!path || !out) return tbsla_status_t(TBSLA_ERR_INVALID_ARG);
  *out = nullptr;
  std::ifstream is(path, std::ifstream::binary);
  if (!is.is_open()) return tbsla::fail(TBSLA_ERR_INVALID_ARG, "cannot open %s", path);
  is.seekg(seek, is.beg);
  try {
    switch (format) {
    case TBSLA_FMT_COO: return from_file<MatrixCOO>(is, out);
    case TBSLA_FMT_SCOO: return from_file<MatrixSCOO>(is, out);
    case TBSLA_FMT_CSR: return from_file<MatrixCSR>(is, out);
    case TBSLA_FMT_ELL: return from_file<MatrixELL>(is, out);
    case TBSLA_FMT_DENSE: return from_file<MatrixDENSE>(is, out);
    default: return tbsla::fail(TBSLA_ERR_INVALID_ARG, "unknown format %d", format);
    }
  } catch (const std::exception &e) {
    return tbsla::fail(TBSLA_ERR_INVALID_ARG, "%s: %s", path, e.what());
  }
}

tbsla_status_t tbsla_matrix_read_mm(const char *path, int format, tbsla_matrix_t **out) {
  if (!path || !out) return tbsla_status_t(TBSLA_ERR_INVALID_ARG);
  *out = nullptr;
  {
    std::ifstream probe(path);
    if (!probe.is_open()) return tbsla::fail(TBSLA_ERR_INVALID_ARG, "cannot open %s", path);
  }
  try {
    CooHandle c;
    c.readMM(path);
    switch (format) {
    case TBSLA_FMT_COO: *out = c.make(); return TBSLA_OK;
    case TBSLA_FMT_SCOO: return from_coo<MatrixSCOO>(c, out);
    case TBSLA_FMT_CSR: return from_coo<MatrixCSR>(c, out);
    case TBSLA_FMT_ELL: return from_coo<MatrixELL>(c, out);
    case TBSLA_FMT_DENSE: return from_coo<MatrixDENSE>(c, out);
    default: return tbsla::fail(TBSLA_ERR_INVALID_ARG, "unknown format %d", format);
    }
  } catch (const MatrixFormatReadException &e) {
    return tbsla::fail(TBSLA_ERR_UNSUPPORTED, "%s: %s", path, e.what());
  } catch (const std::exception &e) {
    return tbsla::fail(TBSLA_ERR_INVALID_ARG, "%s: %s", path, e.what());
  }
}

}  // extern "C"
