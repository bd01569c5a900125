// tbsla/cpp/MatrixDENSE.hpp -- drop-in for TBSLA's MatrixDENSE
// (src/cpp/include/tbsla/cpp/MatrixDENSE.hpp): row-major ln_row x ln_col.
#ifndef TBSLA_CPP_MatrixDENSE
#define TBSLA_CPP_MatrixDENSE

#include <iostream>
#include <vector>

#include <tbsla/cpp/Matrix.hpp>
#include <tbsla/cpp/MatrixCOO.hpp>

namespace tbsla { namespace cpp {

class MatrixDENSE : public virtual Matrix {
  public:
    MatrixDENSE() : values(0) {}
    MatrixDENSE(const tbsla::cpp::MatrixCOO & m);
    friend std::ostream & operator<<(std::ostream &os, const MatrixDENSE &m);
    std::vector<double> spmv(const std::vector<double> &v, int vect_incr = 0) const override;
    void Ax(std::vector<double> &r, const std::vector<double> &v, int vect_incr = 0) const override;
    using tbsla::cpp::Matrix::a_axpx_;
    std::ostream & print_stats(std::ostream &os) override;
    std::ostream & print_infos(std::ostream &os) override;
    std::ostream & print_as_dense(std::ostream &os) override;
    std::ostream & write(std::ostream &os) override;
    std::istream & read(std::istream &is, std::size_t pos = 0, std::size_t n = 1) override;
    std::ostream & print(std::ostream &os) const override;
    void fill_cdiag(int n_row, int n_col, int cdiag, int pr = 0, int pc = 0, int NR = 1, int NC = 1) override;
    void fill_cqmat(int n_row, int n_col, int c, double q, unsigned int seed_mult = 1, int pr = 0, int pc = 0,
                    int NR = 1, int NC = 1) override;
    void fill_cqmat_stochastic(int n_row, int n_col, int c, double q, unsigned int seed_mult = 1, int pr = 0,
                               int pc = 0, int NR = 1, int NC = 1) override;
    void normalize_columns() override;

  protected:
    std::vector<double> values;
    struct tbsla_matrix *upload() const override;
    void array_identity(const void *ptr[3], std::size_t size[3]) const override;
    bool product_is_zero() const override;
};

}}

#endif
