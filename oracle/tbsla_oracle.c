/*
 * tbsla_oracle.c -- CPU restatement of TBSLA's SpMV / PageRank path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference legs load this code.  See
 * tbsla_oracle.h for the contract.  Paths in citations are relative to the
 * TBSLA source tree (src/cpp/...).
 *
 * The loops below follow the reference's loops one for one, including its
 * quirks (integer division in the tail-row coin flip, nnz counted over padded
 * rows, COO's ln_row=NR, ...), because the product is checked against the
 * arrays those quirks produce.
 */
#define _DEFAULT_SOURCE
#include "tbsla_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int64_t imin(int64_t a, int64_t b) { return a < b ? a : b; }
static int64_t imax(int64_t a, int64_t b) { return a > b ? a : b; }
static uint64_t umin(uint64_t a, uint64_t b) { return a < b ? a : b; }

/* ------------------------------------------------------------------------ */
/* growable arrays                                                          */
/* ------------------------------------------------------------------------ */
typedef struct { double *p; int64_t n, cap; } dvec;
typedef struct { int *p; int64_t n, cap; } ivec;

static void dpush(dvec *v, double x) {
  if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 64; v->p = (double *)realloc(v->p, v->cap * sizeof(double)); }
  v->p[v->n++] = x;
}
static void ipush(ivec *v, int x) {
  if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 64; v->p = (int *)realloc(v->p, v->cap * sizeof(int)); }
  v->p[v->n++] = x;
}

void orc_matrix_init(orc_matrix *m, int fmt) {
  memset(m, 0, sizeof(*m));
  m->fmt = fmt;
  m->NR = m->NC = 1;
}

void orc_matrix_free(orc_matrix *m) {
  free(m->values); free(m->idx0); free(m->idx1);
  m->values = NULL; m->idx0 = m->idx1 = NULL;
  m->n_values = m->n_idx0 = m->n_idx1 = 0;
}

static void set_arrays(orc_matrix *m, dvec *v, ivec *a, ivec *b) {
  free(m->values); free(m->idx0); free(m->idx1);
  m->values = v ? v->p : NULL; m->n_values = v ? v->n : 0;
  m->idx0 = a ? a->p : NULL; m->n_idx0 = a ? a->n : 0;
  m->idx1 = b ? b->p : NULL; m->n_idx1 = b ? b->n : 0;
}

/* range::lnv / range::pflv (utils/range.cpp:7-26) */
static int64_t lnv(int64_t size, int pos, int npos) {
  int64_t n = size / npos, mod = size % npos;
  if (pos < mod) n++;
  return n;
}
static int64_t pflv(int64_t size, int pos, int npos) {
  int64_t mod = size % npos;
  int64_t n = lnv(size, pos, npos) * pos;
  if (pos >= mod) n += mod;
  return n;
}

/* ------------------------------------------------------------------------ */
/* generators                                                               */
/* ------------------------------------------------------------------------ */

/* values_generation::cqmat_value (utils/values_generation.cpp:26-45).
 * Entry i of the band matrix: full rows hold c consecutive entries starting at
 * the diagonal, the last c-1 rows a shrinking triangle; each entry moves to a
 * rand_r column with probability q.  The seed is seed_mult*i (i when
 * seed_mult==0) truncated to 32 bits; glibc rand_r is called as the
 * reference calls it. */
void orc_cqmat_value(uint64_t i, uint64_t nr, uint64_t nc, uint64_t c_in, double q,
                     unsigned int seed_mult, int64_t *row, int64_t *col, double *val) {
  unsigned int seed = (unsigned int)(seed_mult > 0 ? (uint64_t)seed_mult * i : i);
  uint64_t c = umin(nc, c_in);
  uint64_t n_full = umin(nc - c + 1, nr);
  *val = 1.0;
  if (i < c * n_full) {
    *row = (int64_t)(i / c);
    double u = (double)rand_r(&seed) / RAND_MAX;
    *col = u < q ? (int64_t)((uint64_t)rand_r(&seed) % nc) : (int64_t)(i / c + i % c);
    return;
  }
  uint64_t it = i - c * n_full;
  uint64_t cur = 1;
  while (cur < nr - n_full && it >= c - cur) {
    it -= c - cur;
    cur++;
  }
  cur += n_full - 1;
  *row = (int64_t)cur;
  /* the reference divides two ints here, so the draw is 0 except when
   * rand_r returns RAND_MAX (values_generation.cpp:43) */
  double u = (double)(rand_r(&seed) / RAND_MAX);
  *col = u < q ? (int64_t)((uint64_t)rand_r(&seed) % nc) : (int64_t)(cur + it);
}

/* values_generation::cdiag_value (utils/values_generation.cpp:4-24) */
void orc_cdiag_value(uint64_t i, uint64_t nv, uint64_t nr, uint64_t nc, uint64_t cdiag,
                     int64_t *row, int64_t *col, double *val) {
  (void)nv; (void)nr;
  int64_t inc = (int64_t)nc, icd = (int64_t)cdiag, ii = (int64_t)i;
  *val = 1.0;
  if (cdiag == 0) { *row = ii; *col = ii; return; }
  if (ii < imax(imin(inc - icd, icd), 0)) { *row = ii; *col = ii + icd; return; }
  if (ii < imax(icd + 2 * (inc - 2 * icd), 0)) {
    int64_t it = (ii + icd) / 2;
    *row = it;
    *col = (i % 2 == 0) ? it - icd : it + icd;
    return;
  }
  int64_t it = ii - (inc - 2 * icd);
  if (icd > inc) it -= icd - inc;
  *row = it; *col = it - icd;
}

static uint64_t cqmat_global_count(uint64_t nr, uint64_t nc, uint64_t c) {
  uint64_t cc = umin(c, nc), g = 0;
  uint64_t nfull = umin(nc - cc + 1, nr);
  for (uint64_t i = 0; i < nfull; i++) g += cc;
  uint64_t mn = umin(nr, nc);
  for (uint64_t i = 0; i + nfull < mn; i++) g += cc - i - 1;
  return g;
}

/* values_generation::cqmat_sum_columns (utils/values_generation.cpp:47-62) */
void orc_cqmat_sum_columns(uint64_t nr, uint64_t nc, uint64_t c, double q,
                           unsigned int seed_mult, double *sum) {
  uint64_t gnv = cqmat_global_count(nr, nc, c);
  for (uint64_t j = 0; j < nc; j++) sum[j] = 0;
  for (uint64_t i = 0; i < gnv; i++) {
    int64_t r, cl; double v;
    orc_cqmat_value(i, nr, nc, c, q, seed_mult, &r, &cl, &v);
    sum[cl] += v;
  }
}

static void set_geometry(orc_matrix *m, int n_row, int n_col, int pr, int pc, int NR, int NC) {
  m->n_row = n_row; m->n_col = n_col; m->pr = pr; m->pc = pc; m->NR = NR; m->NC = NC;
  m->ln_row = (int)lnv(n_row, pr, NR); m->f_row = (int)pflv(n_row, pr, NR);
  m->ln_col = (int)lnv(n_col, pc, NC); m->f_col = (int)pflv(n_col, pc, NC);
}

static int in_window(const orc_matrix *m, int64_t r, int64_t c) {
  return r >= m->f_row && r < m->f_row + m->ln_row && c >= m->f_col && c < m->f_col + m->ln_col;
}

/* COO/SCOO push_back: entries outside the global shape are dropped
 * (MatrixCOO.cpp:118-126, MatrixSCOO.cpp:125-133) */
static void coo_push(const orc_matrix *m, dvec *v, ivec *r, ivec *c, int64_t ri, int64_t ci, double x) {
  int rr = (int)ri, cc = (int)ci; /* the reference passes these through int */
  if (rr >= m->n_row || rr < 0) return;
  if (cc >= m->n_col || cc < 0) return;
  dpush(v, x); ipush(r, rr); ipush(c, cc);
}

/* fill_cdiag: COO (MatrixCOO.cpp:294-330), CSR (MatrixCSR.cpp:234-297),
 * ELL (MatrixELL.cpp:192-260), SCOO (MatrixSCOO.cpp:230-286),
 * DENSE (MatrixDENSE.cpp:137-190) */
void orc_fill_cdiag(orc_matrix *m, int n_row, int n_col, int cdiag, int pr, int pc, int NR, int NC) {
  dvec v = {0}; ivec a = {0}, b = {0};
  if (m->fmt == ORC_COO) {
    m->n_row = n_row; m->n_col = n_col; m->pr = pr; m->pc = pc; m->NR = NR; m->NC = NC;
    m->ln_row = NR; m->ln_col = NC; m->f_row = 0; m->f_col = 0;
    int64_t gnv = imax(imin(n_row, (int64_t)n_col - cdiag), 0) + imax(imin((int64_t)n_row - cdiag, n_col), 0);
    if (cdiag == 0) gnv /= 2;
    m->nnz = 0;
    set_arrays(m, NULL, NULL, NULL);
    if (gnv == 0) return;
    int64_t s = pflv(gnv, pr * NC + pc, NR * NC), n = lnv(gnv, pr * NC + pc, NR * NC);
    m->nnz = n;
    for (int64_t i = s; i < s + n; i++) {
      int64_t r, c; double x;
      orc_cdiag_value((uint64_t)i, (uint64_t)gnv, n_row, n_col, (uint64_t)cdiag, &r, &c, &x);
      coo_push(m, &v, &a, &b, r, c, x);
    }
    set_arrays(m, &v, &a, &b);
    return;
  }
  set_geometry(m, n_row, n_col, pr, pc, NR, NC);
  set_arrays(m, NULL, NULL, NULL);
  int64_t nv = 0;
  for (int64_t i = m->f_row; i < m->f_row + m->ln_row; i++) {
    if (in_window(m, i, i - cdiag)) nv++;
    if (cdiag != 0 && in_window(m, i, i + cdiag)) nv++;
  }
  if (nv == 0) { if (m->fmt == ORC_ELL) m->max_col = cdiag == 0 ? 1 : 2; return; }
  switch (m->fmt) {
  case ORC_CSR: {
    m->nnz = nv; /* the reference leaves this field unset; the stored count is recorded here */
    ipush(&a, 0);
    int64_t k = 0;
    for (int64_t i = m->f_row; i < m->f_row + m->ln_row; i++) {
      if (in_window(m, i, i - cdiag)) { ipush(&b, (int)(i - cdiag)); dpush(&v, 1); k++; }
      if (cdiag != 0 && in_window(m, i, i + cdiag)) { ipush(&b, (int)(i + cdiag)); dpush(&v, 1); k++; }
      ipush(&a, (int)k);
    }
    set_arrays(m, &v, &a, &b);
    break;
  }
  case ORC_ELL: {
    m->max_col = cdiag == 0 ? 1 : 2;
    m->nnz = nv;
    for (int64_t i = m->f_row; i < m->f_row + m->ln_row; i++) {
      if (in_window(m, i, i - cdiag)) { ipush(&a, (int)(i - cdiag)); dpush(&v, 1); }
      else { ipush(&a, 0); dpush(&v, 0); }
      if (cdiag != 0) {
        if (in_window(m, i, i + cdiag)) { ipush(&a, (int)(i + cdiag)); dpush(&v, 1); }
        else { ipush(&a, 0); dpush(&v, 0); }
      }
    }
    set_arrays(m, &v, &a, NULL);
    break;
  }
  case ORC_SCOO: {
    m->nnz = nv;
    for (int64_t i = m->f_row; i < m->f_row + m->ln_row; i++) {
      if (in_window(m, i, i - cdiag)) coo_push(m, &v, &a, &b, i, i - cdiag, 1);
      if (cdiag != 0 && in_window(m, i, i + cdiag)) coo_push(m, &v, &a, &b, i, i + cdiag, 1);
    }
    set_arrays(m, &v, &a, &b);
    break;
  }
  case ORC_DENSE: {
    m->nnz = nv;
    int64_t sz = (int64_t)m->ln_col * m->ln_row;
    double *d = (double *)calloc(sz ? sz : 1, sizeof(double));
    for (int64_t i = m->f_row; i < m->f_row + m->ln_row; i++) {
      if (in_window(m, i, i - cdiag)) d[(i - m->f_row) * m->ln_col + (i - cdiag - m->f_col)] = 1;
      if (cdiag != 0 && in_window(m, i, i + cdiag)) d[(i - m->f_row) * m->ln_col + (i + cdiag - m->f_col)] = 1;
    }
    m->values = d; m->n_values = sz;
    break;
  }
  }
}

/* fill_cqmat: COO (MatrixCOO.cpp:332-375), CSR (MatrixCSR.cpp:299-409),
 * ELL (MatrixELL.cpp:262-392), SCOO (MatrixSCOO.cpp:288-391),
 * DENSE (MatrixDENSE.cpp:192-271) */
void orc_fill_cqmat(orc_matrix *m, int n_row, int n_col, int c, double q, unsigned int seed_mult,
                    int pr, int pc, int NR, int NC) {
  dvec v = {0}; ivec a = {0}, b = {0};
  int64_t r, cl; double x;
  if (m->fmt == ORC_COO) {
    m->n_row = n_row; m->n_col = n_col; m->pr = pr; m->pc = pc; m->NR = NR; m->NC = NC;
    m->ln_row = NR; m->ln_col = NC; m->f_row = 0; m->f_col = 0;
    set_arrays(m, NULL, NULL, NULL);
    int64_t gnv = (int64_t)cqmat_global_count(n_row, n_col, c < 0 ? 0 : c);
    if (gnv == 0) return;
    int64_t s = pflv(gnv, pr * NC + pc, NR * NC), n = lnv(gnv, pr * NC + pc, NR * NC);
    m->nnz = n;
    for (int64_t i = s; i < s + n; i++) {
      orc_cqmat_value((uint64_t)i, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
      coo_push(m, &v, &a, &b, r, cl, x);
    }
    set_arrays(m, &v, &a, &b);
    return;
  }
  set_geometry(m, n_row, n_col, pr, pc, NR, NC);
  set_arrays(m, NULL, NULL, NULL);
  const int64_t cc = imin(c, n_col);
  const int64_t min_ = imin((int64_t)n_col - cc + 1, n_row);
  const int64_t fr = m->f_row, lr = m->ln_row;
  int64_t incr = 0, nv = 0;
  for (int64_t i = 0; i < min_; i++) {
    if (i < fr) incr += cc;
    if (i >= fr && i < fr + lr) nv += cc;
    if (i >= fr + lr) break;
  }
  for (int64_t i = 0; i < imin(n_row, n_col) - min_; i++) {
    if (i + min_ < fr) incr += cc - i - 1;
    if (i + min_ >= fr && i + min_ < fr + lr) nv += cc - i - 1;
    if (i + min_ >= fr + lr) break;
  }
  const int64_t incr_save = incr;
  const int64_t end_all = imin(imin(n_row, n_col), fr + lr);

  if (m->fmt == ORC_CSR || m->fmt == ORC_SCOO) {
    /* nnz counts min(c,n_col) draws for every row, tail rows included */
    m->nnz = 0;
    for (int64_t i = fr; i < end_all; i++)
      for (int64_t j = 0; j < cc; j++) {
        orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
        if (in_window(m, r, cl)) m->nnz++;
        incr++;
      }
    incr = incr_save;
    if (nv == 0) return;
    int64_t k = 0, i;
    if (m->fmt == ORC_CSR) ipush(&a, 0);
    for (i = fr; i < imin(min_, fr + lr); i++) {
      for (int64_t j = 0; j < cc; j++) {
        orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
        if (in_window(m, r, cl)) {
          if (m->fmt == ORC_CSR) { ipush(&b, (int)cl); dpush(&v, x); k++; }
          else coo_push(m, &v, &a, &b, r, cl, x);
        }
        incr++;
      }
      if (m->fmt == ORC_CSR) ipush(&a, (int)k);
    }
    for (; i < end_all; i++) {
      for (int64_t j = 0; j < cc - i + min_ - 1; j++) {
        orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
        if (in_window(m, r, cl)) {
          if (m->fmt == ORC_CSR) { ipush(&b, (int)cl); dpush(&v, x); k++; }
          else coo_push(m, &v, &a, &b, r, cl, x);
        }
        incr++;
      }
      if (m->fmt == ORC_CSR) ipush(&a, (int)k);
    }
    set_arrays(m, &v, &a, &b);
    return;
  }

  if (m->fmt == ORC_ELL) {
    m->nnz = 0;
    m->max_col = 0;
    int64_t i;
    for (i = fr; i < imin(min_, fr + lr); i++) {
      int nbc = 0;
      for (int64_t j = 0; j < cc; j++) {
        orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
        if (in_window(m, r, cl)) { m->nnz++; nbc++; }
        incr++;
      }
      if (nbc > m->max_col) m->max_col = nbc;
    }
    for (; i < end_all; i++) {
      int nbc = 0;
      int64_t j = 0;
      for (; j < cc - i + min_ - 1; j++) {
        orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
        if (in_window(m, r, cl)) { nbc++; m->nnz++; }
        incr++;
      }
      /* the reference compares the slot index with the column window here
       * (MatrixELL.cpp:338-342) */
      for (; j < cc; j++)
        if (j >= m->f_col && j < m->f_col + m->ln_col) nbc++;
      if (nbc > m->max_col) m->max_col = nbc;
    }
    if (nv == 0) return;
    incr = incr_save;
    for (i = fr; i < imin(min_, fr + lr); i++) {
      int64_t k = 0;
      for (int64_t j = 0; j < cc; j++) {
        orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
        if (in_window(m, r, cl)) { ipush(&a, (int)cl); dpush(&v, x); k++; }
        incr++;
      }
      for (int64_t j = k; j < m->max_col; j++) { ipush(&a, 0); dpush(&v, 0); }
    }
    for (; i < imin(n_row, fr + lr); i++) {
      int64_t k = 0;
      for (int64_t j = 0; j < cc - i + min_ - 1; j++) {
        orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
        if (in_window(m, r, cl)) { ipush(&a, (int)cl); dpush(&v, x); k++; }
        incr++;
      }
      for (int64_t j = k; j < m->max_col; j++) { ipush(&a, 0); dpush(&v, 0); }
    }
    set_arrays(m, &v, &a, NULL);
    return;
  }

  /* DENSE */
  if (nv == 0) return;
  m->nnz = 0;
  int64_t sz = (int64_t)m->ln_col * m->ln_row;
  double *d = (double *)calloc(sz ? sz : 1, sizeof(double));
  int64_t i;
  for (i = fr; i < imin(min_, fr + lr); i++)
    for (int64_t j = 0; j < cc; j++) {
      orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
      if (in_window(m, r, cl)) { d[(r - fr) * m->ln_col + (cl - m->f_col)] += x; m->nnz++; }
      incr++;
    }
  for (; i < imin(n_row, fr + lr); i++)
    for (int64_t j = 0; j < cc - i + min_ - 1; j++) {
      orc_cqmat_value((uint64_t)incr, n_row, n_col, c, q, seed_mult, &r, &cl, &x);
      if (in_window(m, r, cl)) { d[(r - fr) * m->ln_col + (cl - m->f_col)] += x; m->nnz++; }
      incr++;
    }
  m->values = d; m->n_values = sz;
}

/* fill_cqmat_stochastic: COO (MatrixCOO.cpp:377-383), CSR (MatrixCSR.cpp:411-421),
 * ELL (MatrixELL.cpp:394-404), SCOO (MatrixSCOO.cpp:393-399),
 * DENSE (MatrixDENSE.cpp:273-286) */
void orc_fill_cqmat_stochastic(orc_matrix *m, int n_row, int n_col, int c, double q,
                               unsigned int seed_mult, int pr, int pc, int NR, int NC) {
  orc_fill_cqmat(m, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC);
  if ((m->fmt == ORC_CSR || m->fmt == ORC_ELL || m->fmt == ORC_DENSE) && m->n_values == 0) return;
  double *sum = (double *)malloc((n_col > 0 ? n_col : 1) * sizeof(double));
  orc_cqmat_sum_columns(n_row, n_col, c, q, seed_mult, sum);
  switch (m->fmt) {
  case ORC_COO: case ORC_SCOO:
    for (int64_t k = 0; k < m->n_values; k++) m->values[k] /= sum[m->idx1[k]];
    break;
  case ORC_CSR:
    for (int64_t i = 0; i + 1 < m->n_idx0; i++)
      for (int64_t k = m->idx0[i]; k < m->idx0[i + 1]; k++) m->values[k] /= sum[m->idx1[k]];
    break;
  case ORC_ELL: {
    int64_t rows = imin(m->ln_row, m->n_values / m->max_col);
    for (int64_t i = 0; i < rows; i++)
      for (int64_t j = 0; j < m->max_col; j++) {
        int64_t k = i * m->max_col + j;
        if (m->values[k] != 0) m->values[k] /= sum[m->idx0[k]];
      }
    break;
  }
  case ORC_DENSE:
    for (int j = 0; j < n_col; j++) if (sum[j] == 0) sum[j] = 1;
    for (int64_t i = 0; i < m->ln_row; i++)
      for (int64_t j = 0; j < m->ln_col; j++) m->values[i * m->ln_col + j] /= sum[m->f_col + j];
    break;
  }
  free(sum);
}

/* normalize_columns: COO (MatrixCOO.cpp:385-393), CSR (MatrixCSR.cpp:423-435),
 * ELL (MatrixELL.cpp:406-422), SCOO (MatrixSCOO.cpp:401-409),
 * DENSE (MatrixDENSE.cpp:288-300) */
void orc_normalize_columns(orc_matrix *m) {
  int64_t ncol = m->fmt == ORC_COO ? m->n_col : m->ln_col;
  double *sum = (double *)calloc(ncol > 0 ? ncol : 1, sizeof(double));
  switch (m->fmt) {
  case ORC_COO:
    for (int64_t k = 0; k < m->n_values; k++) sum[m->idx1[k]] += m->values[k];
    for (int64_t k = 0; k < m->n_values; k++) m->values[k] /= sum[m->idx1[k]];
    break;
  case ORC_SCOO:
    for (int64_t k = 0; k < m->n_values; k++) sum[m->idx1[k] - m->f_col] += m->values[k];
    for (int64_t k = 0; k < m->n_values; k++) m->values[k] /= sum[m->idx1[k] - m->f_col];
    break;
  case ORC_CSR:
    for (int64_t i = 0; i + 1 < m->n_idx0; i++)
      for (int64_t k = m->idx0[i]; k < m->idx0[i + 1]; k++) sum[m->idx1[k] - m->f_col] += m->values[k];
    for (int64_t i = 0; i + 1 < m->n_idx0; i++)
      for (int64_t k = m->idx0[i]; k < m->idx0[i + 1]; k++) m->values[k] /= sum[m->idx1[k] - m->f_col];
    break;
  case ORC_ELL: {
    if (m->max_col == 0) break;
    int64_t rows = imin(m->ln_row, m->n_values / m->max_col);
    for (int pass = 0; pass < 2; pass++)
      for (int64_t i = 0; i < rows; i++)
        for (int64_t j = 0; j < m->max_col; j++) {
          int64_t k = i * m->max_col + j;
          int64_t idx = m->idx0[k] - m->f_col;
          if (idx < 0) idx = 0;
          if (pass == 0) sum[idx] += m->values[k]; else m->values[k] /= sum[idx];
        }
    break;
  }
  case ORC_DENSE:
    for (int64_t i = 0; i < m->ln_row; i++)
      for (int64_t j = 0; j < m->ln_col; j++) sum[j] += m->values[i * m->ln_col + j];
    for (int64_t i = 0; i < m->ln_row; i++)
      for (int64_t j = 0; j < m->ln_col; j++) m->values[i * m->ln_col + j] /= sum[j];
    break;
  }
  free(sum);
}

/* ------------------------------------------------------------------------ */
/* construction from arrays and conversions                                 */
/* ------------------------------------------------------------------------ */
static void *dupmem(const void *p, size_t n) {
  void *q = malloc(n ? n : 1);
  if (n) memcpy(q, p, n);
  return q;
}

void orc_from_arrays(orc_matrix *m, int fmt, int n_row, int n_col, const double *values,
                     int64_t n_values, const int *idx0, int64_t n_idx0, const int *idx1,
                     int64_t n_idx1) {
  orc_matrix_free(m);
  orc_matrix_init(m, fmt);
  m->n_row = m->ln_row = n_row; m->n_col = m->ln_col = n_col;
  m->values = (double *)dupmem(values, n_values * sizeof(double)); m->n_values = n_values;
  m->idx0 = (int *)dupmem(idx0, n_idx0 * sizeof(int)); m->n_idx0 = n_idx0;
  m->idx1 = (int *)dupmem(idx1, n_idx1 * sizeof(int)); m->n_idx1 = n_idx1;
  /* the array constructors leave nnz unset (MatrixCOO.cpp:30-44,
   * MatrixCSR.cpp:13-27); the stored count is recorded here */
  m->nnz = n_values;
}

void orc_update_nnz(orc_matrix *m) { m->nnz = m->n_values; }

/* the (row, col) lexicographic order of utils/csr.cpp:3-8 used by the
 * conversions; ties keep their input order (stable merge sort) */
static const int *g_row, *g_col;
static int cmp_rc(int64_t i, int64_t j) {
  if (g_row[i] != g_row[j]) return g_row[i] < g_row[j] ? -1 : 1;
  if (g_col[i] != g_col[j]) return g_col[i] < g_col[j] ? -1 : 1;
  return 0;
}
static void msort(int64_t *p, int64_t *tmp, int64_t n) {
  if (n < 2) return;
  int64_t h = n / 2;
  msort(p, tmp, h); msort(p + h, tmp, n - h);
  int64_t i = 0, j = h, k = 0;
  while (i < h && j < n) tmp[k++] = cmp_rc(p[j], p[i]) < 0 ? p[j++] : p[i++];
  while (i < h) tmp[k++] = p[i++];
  while (j < n) tmp[k++] = p[j++];
  memcpy(p, tmp, n * sizeof(int64_t));
}

/* MatrixCSR(const MatrixCOO&) (MatrixCSR.cpp:29-74), MatrixELL(COO)
 * (MatrixELL.cpp:12-54), MatrixSCOO(COO) (MatrixSCOO.cpp:53-68),
 * MatrixDENSE(COO) (MatrixDENSE.cpp:11-28).  The reference sorts with an
 * unstable std::sort; tied (row, col) pairs are ordered stably here, which
 * equals the reference whenever tied entries carry equal values. */
void orc_convert(orc_matrix *d, int fmt, const orc_matrix *coo) {
  orc_matrix_free(d);
  orc_matrix_init(d, fmt);
  d->n_row = coo->n_row; d->n_col = coo->n_col;
  d->ln_row = coo->n_row; d->ln_col = coo->n_col;
  d->f_row = coo->f_row; d->f_col = coo->f_col;
  d->pr = coo->pr; d->pc = coo->pc; d->NR = coo->NR; d->NC = coo->NC;
  d->nnz = coo->nnz;
  int64_t n = coo->n_values;
  if (fmt == ORC_SCOO) {
    d->values = (double *)dupmem(coo->values, n * sizeof(double)); d->n_values = n;
    d->idx0 = (int *)dupmem(coo->idx0, n * sizeof(int)); d->n_idx0 = n;
    d->idx1 = (int *)dupmem(coo->idx1, n * sizeof(int)); d->n_idx1 = n;
    return;
  }
  if (fmt == ORC_DENSE) {
    int64_t sz = (int64_t)d->ln_row * d->ln_col;
    d->values = (double *)calloc(sz ? sz : 1, sizeof(double)); d->n_values = sz;
    for (int64_t k = 0; k < n; k++) d->values[(int64_t)coo->idx0[k] * d->ln_col + coo->idx1[k]] += coo->values[k];
    return;
  }
  int64_t *p = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t));
  int64_t *tmp = (int64_t *)malloc((n ? n : 1) * sizeof(int64_t));
  for (int64_t k = 0; k < n; k++) p[k] = k;
  g_row = coo->idx0; g_col = coo->idx1;
  msort(p, tmp, n);
  free(tmp);
  if (fmt == ORC_CSR) {
    d->n_idx0 = (int64_t)d->n_row + 1;
    d->idx0 = (int *)calloc(d->n_idx0, sizeof(int));
    d->values = (double *)malloc((n ? n : 1) * sizeof(double)); d->n_values = n;
    d->idx1 = (int *)malloc((n ? n : 1) * sizeof(int)); d->n_idx1 = n;
    for (int64_t k = 0; k < n; k++) {
      d->values[k] = coo->values[p[k]];
      d->idx1[k] = coo->idx1[p[k]];
      d->idx0[coo->idx0[p[k]] + 1]++;
    }
    /* the reference's rowptr walk (MatrixCSR.cpp:53-72) is a prefix count */
    for (int64_t i = 0; i < d->n_row; i++) d->idx0[i + 1] += d->idx0[i];
  } else { /* ELL */
    if (n == 0) { d->max_col = 0; d->nnz = 0; free(p); return; }
    int *cnt = (int *)calloc(d->n_row > 0 ? d->n_row : 1, sizeof(int));
    for (int64_t k = 0; k < n; k++) cnt[coo->idx0[k]]++;
    int mx = 0;
    for (int i = 0; i < d->n_row; i++) if (cnt[i] > mx) mx = cnt[i];
    d->max_col = mx;
    int64_t sz = (int64_t)d->n_row * mx;
    d->values = (double *)calloc(sz ? sz : 1, sizeof(double)); d->n_values = sz;
    d->idx0 = (int *)calloc(sz ? sz : 1, sizeof(int)); d->n_idx0 = sz;
    int64_t k = 0;
    for (int64_t i = 0; i < d->n_row; i++)
      for (int j = 0; j < cnt[i]; j++, k++) {
        d->values[i * mx + j] = coo->values[p[k]];
        d->idx0[i * mx + j] = coo->idx1[p[k]];
      }
    free(cnt);
  }
  free(p);
}

/* ------------------------------------------------------------------------ */
/* products                                                                 */
/* ------------------------------------------------------------------------ */

/* Ax for each format: COO (MatrixCOO.cpp:107-116), SCOO (MatrixSCOO.cpp:114-123),
 * CSR (MatrixCSR.cpp:129-140), ELL (MatrixELL.cpp:101-114),
 * DENSE (MatrixDENSE.cpp:64-73).  spmv zero-fills r first (e.g.
 * MatrixCSR.cpp:123-127). */
void orc_spmv(const orc_matrix *m, const double *v, double *r, int vect_incr, int threads) {
  for (int64_t i = 0; i < m->n_row; i++) r[i] = 0;
#ifdef _OPENMP
  if (threads < 1) threads = 1;
#else
  (void)threads;
#endif
  switch (m->fmt) {
  case ORC_COO:
    for (int64_t k = 0; k < m->n_values; k++) r[m->idx0[k] + vect_incr] += m->values[k] * v[m->idx1[k]];
    break;
  case ORC_SCOO:
    for (int64_t k = 0; k < m->n_values; k++)
      r[m->idx0[k] + vect_incr - m->f_row] += m->values[k] * v[m->idx1[k] - m->f_col];
    break;
  case ORC_CSR: {
    if (m->n_values == 0) break;
    const int *rp = m->idx0;
    const int base = rp[0];
    const int64_t rows = m->n_idx0 - 1;
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static)
#endif
    for (int64_t i = 0; i < rows; i++) {
      double t = 0;
      for (int64_t k = rp[i] - base; k < rp[i + 1] - base; k++) t += m->values[k] * v[m->idx1[k] - m->f_col];
      r[i] = t;
    }
    break;
  }
  case ORC_ELL: {
    if (m->nnz == 0 || m->max_col == 0) break;
    int64_t rows = imin(m->ln_row, m->n_values / m->max_col);
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static)
#endif
    for (int64_t i = 0; i < rows; i++) {
      double t = 0;
      for (int64_t j = 0; j < m->max_col; j++) {
        int64_t idx = m->idx0[i * m->max_col + j] - m->f_col;
        if (idx < 0) idx = 0;
        t += m->values[i * m->max_col + j] * v[idx];
      }
      r[i] = t;
    }
    break;
  }
  case ORC_DENSE: {
    if (m->nnz == 0 || m->n_values == 0) break;
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static)
#endif
    for (int64_t i = 0; i < m->ln_row; i++)
      for (int64_t j = 0; j < m->ln_col; j++) r[i] += m->values[i * m->ln_col + j] * v[j];
    break;
  }
  }
}

void orc_a_axpx(const orc_matrix *m, const double *v, double *r, int vect_incr, int threads) {
  double *t = (double *)malloc((m->n_row > 0 ? m->n_row : 1) * sizeof(double));
  orc_spmv(m, v, t, vect_incr, threads);
  for (int64_t i = 0; i < m->n_row; i++) t[i] += v[i];
  orc_spmv(m, t, r, vect_incr, threads);
  free(t);
}

/* Matrix::page_rank (Matrix.cpp:13-61) */
int orc_page_rank(const orc_matrix *m, double epsilon, double beta, int max_iteration,
                  double *b, int threads) {
  const int n = m->n_col;
  double *bt = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
  double *y = (double *)malloc(((m->n_row > n ? m->n_row : n) + 1) * sizeof(double));
  for (int i = 0; i < n; i++) b[i] = 1.0;
  int it = 0, conv = 0;
  while (!conv && it < max_iteration) {
    double tele = 0.0;
    memcpy(bt, b, n * sizeof(double));
    orc_spmv(m, bt, y, 0, threads);
    memcpy(b, y, n * sizeof(double));
    for (int i = 0; i < n; i++) tele += bt[i];
    tele *= (1 - beta) / n;
    b[0] = beta * b[0] + tele;
    double mx = b[0];
    for (int i = 1; i < n; i++) {
      b[i] = beta * b[i] + tele;
      if (mx < b[i]) mx = b[i];
    }
    double err = 0.0;
    for (int i = 0; i < n; i++) {
      b[i] = b[i] / mx;
      err += fabs(b[i] - bt[i]);
    }
    if (err < epsilon) conv = 1;
    it++;
  }
  double s = b[0];
  for (int i = 1; i < n; i++) s += b[i];
  for (int i = 0; i < n; i++) b[i] = b[i] / s;
  free(bt); free(y);
  return it;
}

/* Matrix::personalized_page_rank (Matrix.cpp:63-114) */
int orc_personalized_page_rank(const orc_matrix *m, double epsilon, double beta,
                               int max_iteration, const int *nodes, int n_nodes, double *b,
                               int threads) {
  const int n = m->n_col;
  double *bt = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
  double *y = (double *)malloc(((m->n_row > n ? m->n_row : n) + 1) * sizeof(double));
  unsigned char *mark = (unsigned char *)calloc(n > 0 ? n : 1, 1);
  for (int k = 0; k < n_nodes; k++) if (nodes[k] >= 0 && nodes[k] < n) mark[nodes[k]] = 1;
  for (int i = 0; i < n; i++) b[i] = 0.25;
  int it = 0, conv = 0;
  while (!conv && it < max_iteration) {
    double tele = 0.0;
    memcpy(bt, b, n * sizeof(double));
    orc_spmv(m, bt, y, 0, threads);
    memcpy(b, y, n * sizeof(double));
    for (int i = 0; i < n; i++) tele += bt[i];
    tele *= (1 - beta) / n_nodes;
    for (int i = 0; i < n; i++) {
      b[i] = beta * b[i];
      if (mark[i]) b[i] += tele;
    }
    double mx = b[0];
    for (int i = 1; i < n; i++) if (mx < b[i]) mx = b[i];
    double err = 0.0;
    for (int i = 0; i < n; i++) {
      b[i] = b[i] / mx;
      err += fabs(b[i] - bt[i]);
    }
    if (err < epsilon) conv = 1;
    it++;
  }
  double s = b[0];
  for (int i = 1; i < n; i++) s += b[i];
  for (int i = 0; i < n; i++) b[i] = b[i] / s;
  free(bt); free(y); free(mark);
  return it;
}

int orc_page_rank_dangling(int n, const int *rowptr, const int *colidx, const double *values,
                           const unsigned char *dangling, double beta, double tol, int max_it,
                           double *x, double *resid, int threads) {
  double *xn = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
#ifndef _OPENMP
  (void)threads;
#else
  if (threads < 1) threads = 1;
#endif
  for (int i = 0; i < n; i++) x[i] = 1.0 / n;
  int it = 0;
  double res = INFINITY;
  while (it < max_it) {
    double d = 0, s = 0;
    for (int j = 0; j < n; j++) { s += x[j]; if (dangling[j]) d += x[j]; }
    const double add = (beta * d + (1 - beta) * s) / n;
    res = 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(threads) schedule(static) reduction(+ : res)
#endif
    for (int i = 0; i < n; i++) {
      double t = 0;
      for (int k = rowptr[i]; k < rowptr[i + 1]; k++) t += values[k] * x[colidx[k]];
      xn[i] = beta * t + add;
      res += fabs(xn[i] - x[i]);
    }
    memcpy(x, xn, n * sizeof(double));
    it++;
    if (res < tol) break;
  }
  free(xn);
  if (resid) *resid = res;
  return it;
}

/* ------------------------------------------------------------------------ */
/* R-MAT                                                                    */
/* ------------------------------------------------------------------------ */
/* splitmix64 finaliser (Steele, Lea, Flood 2014) */
static uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* Edge e draws its bits from the 64-bit words mix64(mix64(seed) + 32*e + w),
 * w = 0..; level l uses the high (l even) or low (l odd) 32 bits of word l/2,
 * scaled by 2^-32.  Level 0 picks the most significant bit.  Quadrant
 * a -> (0,0), b -> (0,1), c -> (1,0), d -> (1,1) as (src bit, dst bit). */
void orc_rmat_edges(int scale, int64_t m, double a, double b, double c, uint64_t seed,
                    int *src, int *dst) {
  const double ta = a, tb = a + b, tc = a + b + c;
  const uint64_t key = mix64(seed);
  for (int64_t e = 0; e < m; e++) {
    uint32_t s = 0, d = 0;
    uint64_t h = 0;
    for (int l = 0; l < scale; l++) {
      if ((l & 1) == 0) h = mix64(key + 32ull * (uint64_t)e + (uint64_t)(l >> 1));
      uint32_t bits = (l & 1) ? (uint32_t)h : (uint32_t)(h >> 32);
      double u = (double)bits * (1.0 / 4294967296.0);
      uint32_t rb, cb;
      if (u < ta) { rb = 0; cb = 0; }
      else if (u < tb) { rb = 0; cb = 1; }
      else if (u < tc) { rb = 1; cb = 0; }
      else { rb = 1; cb = 1; }
      s = (s << 1) | rb;
      d = (d << 1) | cb;
    }
    src[e] = (int)s;
    dst[e] = (int)d;
  }
}

uint64_t orc_fnv1a(const void *data, size_t nbytes) {
  const unsigned char *p = (const unsigned char *)data;
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < nbytes; i++) { h ^= p[i]; h *= 1099511628211ull; }
  return h;
}

/* ------------------------------------------------------------------------ */
/* PageRank in affine (teleport) form and its adjoint.  No reference         */
/* counterpart: the fixed point x = beta*A x + (beta*d.x + 1 - beta) v, with */
/* d the dangling columns, and lambda = beta*A^T lambda + beta*d*(v.lambda) */
/* + w, the adjoint of L(x*) with w = dL/dx*.  Gradients:                    */
/*   dL/dA[k] = beta*lambda[row(k)]*x[col(k)],                               */
/*   dL/dv    = (beta*d.x + 1 - beta)*lambda.                                */
/* Jacobi sweeps from x0 = v / lambda0 = w; max_it sweeps at most, stop when */
/* the L1 change is below tol.  v NULL means uniform 1/n.                    */
/* ------------------------------------------------------------------------ */
static double tele_v(const double *v, int i, int n) { return v ? v[i] : 1.0 / n; }

int orc_pagerank_teleport(int n, const int *rowptr, const int *colidx, const double *values,
                          const unsigned char *dangling, const double *v, double beta, double tol,
                          int max_it, double *x, double *resid) {
  double *xn = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
  for (int i = 0; i < n; i++) x[i] = tele_v(v, i, n);
  int it = 0;
  double res = INFINITY;
  while (it < max_it) {
    double d = 0;
    for (int j = 0; j < n; j++) if (dangling[j]) d += x[j];
    const double a = beta * d + (1 - beta);
    res = 0;
    for (int i = 0; i < n; i++) {
      double t = 0;
      for (int k = rowptr[i]; k < rowptr[i + 1]; k++) t += values[k] * x[colidx[k]];
      xn[i] = beta * t + a * tele_v(v, i, n);
      res += fabs(xn[i] - x[i]);
    }
    memcpy(x, xn, n * sizeof(double));
    it++;
    if (res < tol) break;
  }
  free(xn);
  if (resid) *resid = res;
  return it;
}

int orc_pagerank_adjoint(int n, const int *rowptr, const int *colidx, const double *values,
                         const unsigned char *dangling, const double *v, const double *x, const double *w,
                         double beta, double tol, int max_it, double *grad_values, double *grad_v) {
  double *lam = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
  double *t = (double *)malloc((n > 0 ? n : 1) * sizeof(double));
  memcpy(lam, w, n * sizeof(double));
  int it = 0;
  while (it < max_it) {
    double vl = 0;
    for (int j = 0; j < n; j++) vl += tele_v(v, j, n) * lam[j];
    for (int j = 0; j < n; j++) t[j] = 0;
    for (int i = 0; i < n; i++)
      for (int k = rowptr[i]; k < rowptr[i + 1]; k++) t[colidx[k]] += values[k] * lam[i];
    double res = 0;
    for (int j = 0; j < n; j++) {
      const double nl = beta * t[j] + w[j] + (dangling[j] ? beta * vl : 0.0);
      res += fabs(nl - lam[j]);
      lam[j] = nl;
    }
    it++;
    if (res < tol) break;
  }
  double dx = 0;
  for (int j = 0; j < n; j++) if (dangling[j]) dx += x[j];
  if (grad_v)
    for (int j = 0; j < n; j++) grad_v[j] = (beta * dx + 1 - beta) * lam[j];
  if (grad_values)
    for (int i = 0; i < n; i++)
      for (int k = rowptr[i]; k < rowptr[i + 1]; k++) grad_values[k] = beta * lam[i] * x[colidx[k]];
  free(lam);
  free(t);
  return it;
}
