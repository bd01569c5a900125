// tbsla/cpp/MatrixCOO.hpp -- drop-in for TBSLA's MatrixCOO
// (src/cpp/include/tbsla/cpp/MatrixCOO.hpp): unsorted triplets with global
// indices.  spmv / Ax run the GPU COO product (rows sorted once on upload).
#ifndef TBSLA_CPP_MatrixCOO
#define TBSLA_CPP_MatrixCOO

#include <iostream>
#include <string>
#include <vector>

#include <tbsla/cpp/Matrix.hpp>

namespace tbsla { namespace cpp {

class MatrixCOO : public virtual Matrix {
  public:
    friend std::ostream & operator<<(std::ostream &os, const MatrixCOO &m);
    MatrixCOO(int n_row, int n_col, std::vector<double> & values, std::vector<int> & row, std::vector<int> & col);
    MatrixCOO(int n_row, int n_col, long int n_values);
    MatrixCOO(int n_row, int n_col);
    MatrixCOO() : values(0), row(0), col(0) {}
    const std::vector<double>& get_values() const { return values; }
    const std::vector<int>& get_row() const { return row; }
    const std::vector<int>& get_col() const { return col; }
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
    void push_back(int r, int c, double v);
    void update_nnz();
    void readMM(std::string name);

  protected:
    std::vector<double> values;
    std::vector<int> row;
    std::vector<int> col;
    struct tbsla_matrix *upload() const override;
    void array_identity(const void *ptr[3], std::size_t size[3]) const override;
    bool product_is_zero() const override;

  private:
    void init(int n_row, int n_col, long int n_values);
};

}}

#endif
