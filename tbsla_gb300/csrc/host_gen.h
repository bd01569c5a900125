// host_gen.h -- C++ interface of the synthetic-matrix builders, used by the
// drop-in classes (arrays straight into their std::vectors) and by
// tbsla_generate / tbsla_generate_matrix.
#pragma once

#include <cstdint>
#include <vector>

#include "../../include/tbsla_gb300.h"

namespace tbsla {

struct GenArrays {
  int format = 0;
  // n_row n_col ln_row ln_col f_row f_col pr pc NR NC max_col
  int geom[11] = {0};
  int64_t nnz = 0;
  bool nnz_set = false;  // false where the reference leaves nnz unset
  std::vector<double> values;
  std::vector<int> idx0, idx1;
};

// gen: 0 = cqmat, 1 = cdiag (c is the diagonal offset), 2 = cqmat_stochastic,
// 3 = cqmat_baseline (whole matrix only; see tbsla_generate)
tbsla_status_t generate_arrays(int format, int gen, int n_row, int n_col, int c, double q,
                               unsigned int seed_mult, int pr, int pc, int NR, int NC,
                               GenArrays &out);

// entry i of the global generators (values_generation.cpp:4-45): row,
// column and the reference's branch tag (cqmat: 30 full rows, 31 tail rows;
// cdiag: 10 main diagonal, 30 / 31 / 32 / 33 by band segment)
void cqmat_entry_tagged(uint64_t i, uint64_t nr, uint64_t nc, uint64_t c, double q, unsigned int seed_mult,
                        int64_t &row, int64_t &col, int &tag);
void cdiag_entry_tagged(int64_t i, int64_t nc, int64_t cd, int64_t &row, int64_t &col, int &tag);

// column sums of the global cqmat (values_generation.cpp:47-62)
std::vector<double> cqmat_column_sums(int n_row, int n_col, int c, double q, unsigned int seed_mult);

}  // namespace tbsla
