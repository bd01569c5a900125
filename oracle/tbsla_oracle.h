/*
 * tbsla_oracle.h -- CPU restatement of TBSLA's SpMV / PageRank path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker that the parity tests,
 * __graft_entry__.smoke() and the bench's CPU-baseline leg compare the CUDA
 * path against.  The product library (tbsla_gb300) never links, loads or
 * calls anything in this directory.
 *
 * Every function restates the reference algorithm at the file:line cited in
 * its comment (paths relative to the TBSLA source tree).  The restatement is
 * pinned against the reference itself (compiled from its own sources into
 * oracle/_ref by oracle/Makefile) and against the committed golden vectors in
 * tests/golden/ (generated by tests/golden/make_golden.py from that build).
 *
 * Floating point: the file is compiled with -ffp-contract=off so that
 * `acc += a * b` is a rounded multiply followed by a rounded add on every
 * host, exactly as the reference's x86-64 build evaluates it.
 */
#ifndef TBSLA_ORACLE_H
#define TBSLA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_COO = 0, ORC_SCOO = 1, ORC_CSR = 2, ORC_ELL = 3, ORC_DENSE = 4 };

/* One matrix in the reference's own storage layout (Matrix.hpp:43-45 plus the
 * per-format arrays of Matrix{COO,SCOO,CSR,ELL,DENSE}.hpp). */
typedef struct {
  int fmt;
  int n_row, n_col, ln_row, ln_col, f_row, f_col, pr, pc, NR, NC;
  int64_t nnz;          /* the reference's nnz field, quirks included        */
  int max_col;          /* ELL only                                          */
  int64_t n_values;     /* length of values                                  */
  double *values;
  int64_t n_idx0;       /* COO/SCOO: row, CSR: rowptr, ELL: columns          */
  int *idx0;
  int64_t n_idx1;       /* COO/SCOO: col, CSR: colidx                        */
  int *idx1;
} orc_matrix;

void orc_matrix_init(orc_matrix *m, int fmt);
void orc_matrix_free(orc_matrix *m);

/* per-entry generators (utils/values_generation.cpp) */
void orc_cqmat_value(uint64_t i, uint64_t nr, uint64_t nc, uint64_t c, double q,
                     unsigned int seed_mult, int64_t *row, int64_t *col, double *val);
void orc_cdiag_value(uint64_t i, uint64_t nv, uint64_t nr, uint64_t nc, uint64_t cdiag,
                     int64_t *row, int64_t *col, double *val);
void orc_cqmat_sum_columns(uint64_t nr, uint64_t nc, uint64_t c, double q,
                           unsigned int seed_mult, double *sum /* nc */);

/* fills (Matrix*::fill_cdiag / fill_cqmat / fill_cqmat_stochastic) */
void orc_fill_cdiag(orc_matrix *m, int n_row, int n_col, int cdiag, int pr, int pc, int NR, int NC);
void orc_fill_cqmat(orc_matrix *m, int n_row, int n_col, int c, double q, unsigned int seed_mult,
                    int pr, int pc, int NR, int NC);
void orc_fill_cqmat_stochastic(orc_matrix *m, int n_row, int n_col, int c, double q,
                               unsigned int seed_mult, int pr, int pc, int NR, int NC);
void orc_normalize_columns(orc_matrix *m);

/* array constructors: MatrixCOO(n_row, n_col, values, row, col) and friends */
void orc_from_arrays(orc_matrix *m, int fmt, int n_row, int n_col, const double *values,
                     int64_t n_values, const int *idx0, int64_t n_idx0, const int *idx1,
                     int64_t n_idx1);
/* MatrixCOO::update_nnz (MatrixCOO.cpp:128-133) */
void orc_update_nnz(orc_matrix *m);
/* conversions from COO: MatrixCSR(COO), MatrixELL(COO), MatrixSCOO(COO), MatrixDENSE(COO) */
void orc_convert(orc_matrix *dst, int fmt, const orc_matrix *coo);

/* spmv: r (n_row, zeroed here) = A * v.  threads<=1 runs the loop in order.  */
void orc_spmv(const orc_matrix *m, const double *v, double *r, int vect_incr, int threads);
/* Matrix::a_axpx_ (Matrix.cpp:6-11) */
void orc_a_axpx(const orc_matrix *m, const double *v, double *r, int vect_incr, int threads);
/* Matrix::page_rank (Matrix.cpp:13-61); returns iterations done, b has n_col */
int orc_page_rank(const orc_matrix *m, double epsilon, double beta, int max_iteration,
                  double *b, int threads);
/* Matrix::personalized_page_rank (Matrix.cpp:63-114) */
int orc_personalized_page_rank(const orc_matrix *m, double epsilon, double beta,
                               int max_iteration, const int *nodes, int n_nodes, double *b,
                               int threads);

/* PageRank with uniform redistribution of dangling mass and a sum-normalised
 * L1 stopping rule (no reference counterpart: the reference's page_rank has
 * no dangling term).  A is CSR; dangling[j]!=0 marks nodes without out-edges.
 * x0 = 1/n.  Each sweep: y = A x;  d = sum_{dangling} x;  s = sum x;
 * x' = beta*y + (beta*d + (1-beta)*s)/n;  stop when ||x'-x||_1 < tol.
 * Returns sweeps done; *resid gets the last L1 change. */
int orc_page_rank_dangling(int n, const int *rowptr, const int *colidx, const double *values,
                           const unsigned char *dangling, double beta, double tol, int max_it,
                           double *x, double *resid, int threads);
/* affine (teleport) PageRank and its adjoint; no reference counterpart */
int orc_pagerank_teleport(int n, const int *rowptr, const int *colidx, const double *values,
                          const unsigned char *dangling, const double *v, double beta, double tol,
                          int max_it, double *x, double *resid);
int orc_pagerank_adjoint(int n, const int *rowptr, const int *colidx, const double *values,
                         const unsigned char *dangling, const double *v, const double *x, const double *w,
                         double beta, double tol, int max_it, double *grad_values, double *grad_v);

/* R-MAT edge list (Chakrabarti, Zhan, Faloutsos 2004): recursive quadrant
 * choice per bit with probabilities (a,b,c,1-a-b-c), counter-based uniform
 * numbers (tbsla_rmat_uniform).  Writes src[e], dst[e] for e in [0, m). */
void orc_rmat_edges(int scale, int64_t m, double a, double b, double c, uint64_t seed,
                    int *src, int *dst);

/* FNV-1a over bytes: array fingerprints for golden fixtures */
uint64_t orc_fnv1a(const void *data, size_t nbytes);

#ifdef __cplusplus
}
#endif
#endif
