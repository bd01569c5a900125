// tbsla/cpp/Matrix.hpp -- drop-in for TBSLA's abstract matrix
// (src/cpp/include/tbsla/cpp/Matrix.hpp:9-47).  Same class, members and
// signatures; products and PageRank run on the GPU through the C ABI of
// tbsla_gb300.h.  Each object keeps its arrays in host std::vectors, as the
// reference does, and a device copy built on first use (shared between
// copies of the object, rebuilt when the arrays are reallocated or a
// mutating member function runs).  CUDA failures throw std::runtime_error.
#ifndef TBSLA_CPP_Matrix
#define TBSLA_CPP_Matrix

#include <cstddef>
#include <exception>
#include <fstream>
#include <memory>
#include <vector>

struct tbsla_matrix;

namespace tbsla { namespace cpp {

namespace detail { struct DeviceCopy; }

class Matrix {
  public:
    friend std::ostream & operator<<(std::ostream &os, const Matrix &m) { return m.print(os); }
    virtual ~Matrix();
    virtual std::vector<double> spmv(const std::vector<double> &v, int vect_incr = 0) const = 0;
    virtual void Ax(std::vector<double> &r, const std::vector<double> &v, int vect_incr = 0) const = 0;
    std::vector<double> a_axpx_(const std::vector<double> &v, int vect_incr = 0) const;
    std::vector<double> & saxpy(const std::vector<double> &x, std::vector<double> &y);
    std::vector<double> page_rank(double epsilon, double beta, int max_iteration, int& nb_iterations_done);
    std::vector<double> personalized_page_rank(double epsilon, double beta, int max_iteration,
                                               std::vector<int> personalized_nodes, int& nb_iterations_done);
    int get_n_row() const { return n_row; }
    int get_n_col() const { return n_col; }
    int get_f_row() const { return f_row; }
    int get_f_col() const { return f_col; }
    int get_ln_row() const { return ln_row; }
    int get_ln_col() const { return ln_col; }
    int get_pr() const { return pr; }
    int get_pc() const { return pc; }
    int get_NR() const { return NR; }
    int get_NC() const { return NC; }
    long int get_nnz() const { return nnz; }

    virtual std::ostream & print_stats(std::ostream &os) = 0;
    virtual std::ostream & print_infos(std::ostream &os) = 0;
    virtual std::ostream & write(std::ostream &os) = 0;
    virtual std::istream & read(std::istream &is, std::size_t pos = 0, std::size_t n = 1) = 0;
    virtual std::ostream & print(std::ostream &os) const = 0;
    virtual std::ostream & print_as_dense(std::ostream &os) = 0;

    virtual void fill_cdiag(int n_row, int n_col, int cdiag, int pr = 0, int pc = 0, int NR = 1, int NC = 1) = 0;
    virtual void fill_cqmat(int n_row, int n_col, int c, double q, unsigned int seed_mult = 1, int pr = 0,
                            int pc = 0, int NR = 1, int NC = 1) = 0;
    virtual void fill_cqmat_stochastic(int n_row, int n_col, int c, double q, unsigned int seed_mult = 1,
                                       int pr = 0, int pc = 0, int NR = 1, int NC = 1) = 0;

    virtual void normalize_columns() = 0;

    // The device handle (tbsla_gb300.h) holding this matrix, built or
    // rebuilt as needed; for callers mixing this class with the C ABI.
    struct tbsla_matrix *device_matrix() const;

  protected:
    int n_row = 0, n_col = 0, f_row = 0, f_col = 0, ln_row = 0, ln_col = 0, pr = 0, pc = 0, NR = 1, NC = 1;
    long int nnz = 0;

    // A subclass that writes the stored arrays in place calls this before
    // the next product; reallocations are noticed without it.
    void invalidate_device() const;
    // Uploads the arrays as a new device handle (one per format).
    virtual struct tbsla_matrix *upload() const = 0;
    // Identity of the arrays behind the device copy: data pointers and sizes.
    virtual void array_identity(const void *ptr[3], std::size_t size[3]) const = 0;
    // True where the format's Ax returns without touching r (no values, or
    // nnz / max_col of 0): the product is zero and nothing is uploaded.
    virtual bool product_is_zero() const = 0;

  private:
    mutable std::shared_ptr<detail::DeviceCopy> device_;
};

struct MatrixFormatReadException : public std::exception {
  const char *what() const noexcept override { return "This Matrix format import is not implemented!"; }
};

}}

#endif
