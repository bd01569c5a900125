// The drop-in classes' host side without a GPU: fill a matrix with the
// reference generators, write it in the reference's binary layout
// (Matrix*::write), read the file back into a new object (Matrix*::read) and
// write that object again.  Nothing here builds a device copy.
//
//   dropin_files <FMT> <gen: cqmat|cdiag|stochastic> <n_row> <n_col> <c> <q> <seed> <pr> <pc> <NR> <NC>
//                <first.bin> <second.bin>
//   dropin_files MM <file.mtx> <out.bin>   MatrixCOO::readMM, then write (exit 6: the reader refused)
//   dropin_files CONV <FMT> <n_row> <n_col> <c> <q> <seed> <normalize 0|1> <out.bin>
//                a COO cqmat fill (normalize_columns first when asked), converted to FMT by the
//                constructor from MatrixCOO, then written
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <fstream>
#include <memory>
#include <string>

#include <tbsla/cpp/MatrixCOO.hpp>
#include <tbsla/cpp/MatrixCSR.hpp>
#include <tbsla/cpp/MatrixDENSE.hpp>
#include <tbsla/cpp/MatrixELL.hpp>
#include <tbsla/cpp/MatrixSCOO.hpp>

static std::unique_ptr<tbsla::cpp::Matrix> make(const std::string &fmt) {
  if (fmt == "COO") return std::make_unique<tbsla::cpp::MatrixCOO>();
  if (fmt == "SCOO") return std::make_unique<tbsla::cpp::MatrixSCOO>();
  if (fmt == "CSR") return std::make_unique<tbsla::cpp::MatrixCSR>();
  if (fmt == "ELL") return std::make_unique<tbsla::cpp::MatrixELL>();
  if (fmt == "DENSE") return std::make_unique<tbsla::cpp::MatrixDENSE>();
  return nullptr;
}

int main(int argc, char **argv) {
  if (argc == 4 && std::string(argv[1]) == "MM") {
    tbsla::cpp::MatrixCOO m;
    try {
      m.readMM(argv[2]);
    } catch (const std::exception &) {
      return 6;
    }
    std::ofstream os(argv[3], std::ios::binary);
    m.write(os);
    return os ? 0 : 5;
  }
  if (argc == 10 && std::string(argv[1]) == "CONV") {
    const std::string fmt = argv[2];
    tbsla::cpp::MatrixCOO coo;
    coo.fill_cqmat(std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]), std::atof(argv[6]),
                   (unsigned)std::strtoul(argv[7], nullptr, 10));
    if (std::atoi(argv[8])) coo.normalize_columns();
    std::unique_ptr<tbsla::cpp::Matrix> m;
    if (fmt == "CSR") m = std::make_unique<tbsla::cpp::MatrixCSR>(coo);
    else if (fmt == "ELL") m = std::make_unique<tbsla::cpp::MatrixELL>(coo);
    else if (fmt == "SCOO") m = std::make_unique<tbsla::cpp::MatrixSCOO>(coo);
    else if (fmt == "DENSE") m = std::make_unique<tbsla::cpp::MatrixDENSE>(coo);
    else return 2;
    std::ofstream os(argv[9], std::ios::binary);
    m->write(os);
    return os ? 0 : 5;
  }
  if (argc != 14) {
    std::fprintf(stderr, "usage: %s FMT GEN n_row n_col c q seed pr pc NR NC first.bin second.bin\n", argv[0]);
    return 2;
  }
  const std::string fmt = argv[1], gen = argv[2];
  const int n_row = std::atoi(argv[3]), n_col = std::atoi(argv[4]), c = std::atoi(argv[5]);
  const double q = std::atof(argv[6]);
  const unsigned seed = (unsigned)std::strtoul(argv[7], nullptr, 10);
  const int pr = std::atoi(argv[8]), pc = std::atoi(argv[9]), NR = std::atoi(argv[10]), NC = std::atoi(argv[11]);
  auto m = make(fmt);
  auto back = make(fmt);
  if (!m || !back) return 2;
  if (gen == "cqmat") m->fill_cqmat(n_row, n_col, c, q, seed, pr, pc, NR, NC);
  else if (gen == "cdiag") m->fill_cdiag(n_row, n_col, c, pr, pc, NR, NC);
  else if (gen == "stochastic") m->fill_cqmat_stochastic(n_row, n_col, c, q, seed, pr, pc, NR, NC);
  else return 2;
  {
    std::ofstream os(argv[12], std::ios::binary);
    m->write(os);
    if (!os) return 3;
  }
  {
    std::ifstream is(argv[12], std::ios::binary);
    back->read(is);
    if (!is) return 4;
  }
  std::ofstream os(argv[13], std::ios::binary);
  back->write(os);
  return os ? 0 : 5;
}
