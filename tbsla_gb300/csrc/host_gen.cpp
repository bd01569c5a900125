// host_gen.cpp -- builders of TBSLA's synthetic matrices (cdiag, cqmat,
// cqmat_stochastic) in the reference's array layouts, parallel over rows.
//
// The arrays must equal the reference's element for element, quirks
// included, because the drop-in classes hand them back through the same
// getters and binary writer.  The per-entry generator follows
// src/cpp/utils/values_generation.cpp:4-62; the per-format fills follow
// Matrix{COO,SCOO,CSR,ELL,DENSE}::fill_cdiag / fill_cqmat /
// fill_cqmat_stochastic (file:line at each function below).  glibc rand_r
// is called exactly where the reference calls it.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "host_gen.h"

namespace tbsla {
tbsla_status_t fail(tbsla_status_t s, const char *fmt, ...);
}

namespace {

using i64 = int64_t;
using u64 = uint64_t;

// ---------------------------------------------------------------- entries
// cqmat entry i: (row, col), value 1 (values_generation.cpp:26-45)
struct Entry { i64 row, col; };

inline Entry cqmat_entry(u64 i, u64 nr, u64 nc, u64 c_in, double q, unsigned seed_mult) {
  unsigned int seed = (unsigned int)(seed_mult > 0 ? (u64)seed_mult * i : i);
  const u64 c = std::min(nc, c_in);
  const u64 nfull = std::min(nc - c + 1, nr);
  if (i < c * nfull) {
    const double u = (double)rand_r(&seed) / RAND_MAX;
    const i64 col = u < q ? (i64)((u64)rand_r(&seed) % nc) : (i64)(i / c + i % c);
    return {(i64)(i / c), col};
  }
  u64 it = i - c * nfull, cur = 1;
  while (cur < nr - nfull && it >= c - cur) {
    it -= c - cur;
    ++cur;
  }
  cur += nfull - 1;
  // integer division in the reference: nonzero only for rand_r == RAND_MAX
  const double u = (double)(rand_r(&seed) / RAND_MAX);
  const i64 col = u < q ? (i64)((u64)rand_r(&seed) % nc) : (i64)(cur + it);
  return {(i64)cur, col};
}

// cdiag entry i (values_generation.cpp:4-24), used by MatrixCOO::fill_cdiag
inline Entry cdiag_entry(i64 i, i64 nc, i64 cd) {
  if (cd == 0) return {i, i};
  if (i < std::max(std::min(nc - cd, cd), (i64)0)) return {i, i + cd};
  if (i < std::max(cd + 2 * (nc - 2 * cd), (i64)0)) {
    const i64 it = (i + cd) / 2;
    return {it, (i % 2 == 0) ? it - cd : it + cd};
  }
  i64 it = i - (nc - 2 * cd);
  if (cd > nc) it -= cd - nc;
  return {it, it - cd};
}

// range::lnv / range::pflv (utils/range.cpp:7-26)
inline i64 lnv(i64 size, int pos, int npos) {
  i64 n = size / npos;
  if (pos < size % npos) ++n;
  return n;
}
inline i64 pflv(i64 size, int pos, int npos) {
  const i64 mod = size % npos;
  i64 n = lnv(size, pos, npos) * pos;
  if (pos >= mod) n += mod;
  return n;
}

using Out = tbsla::GenArrays;

struct Block {
  i64 nr, nc, fr, lr, fc, lc;
  bool in(i64 r, i64 c) const { return r >= fr && r < fr + lr && c >= fc && c < fc + lc; }
};

void set_block(Out &o, Block &b, int n_row, int n_col, int pr, int pc, int NR, int NC) {
  b.nr = n_row; b.nc = n_col;
  b.lr = lnv(n_row, pr, NR); b.fr = pflv(n_row, pr, NR);
  b.lc = lnv(n_col, pc, NC); b.fc = pflv(n_col, pc, NC);
  int *g = o.geom;
  g[0] = n_row; g[1] = n_col; g[2] = (int)b.lr; g[3] = (int)b.lc; g[4] = (int)b.fr; g[5] = (int)b.fc;
  g[6] = pr; g[7] = pc; g[8] = NR; g[9] = NC;
}

// ------------------------------------------------------------- cqmat
// Row layout of the band: rows [0, min_) hold cc entries, row min_+k holds
// cc-k-1; entries are numbered row by row.
struct Band {
  i64 cc, min_, mn;
  i64 start(i64 i) const {
    if (i <= min_) return i * cc;
    const i64 m = i - min_;
    return min_ * cc + m * (cc - 1) - m * (m - 1) / 2;
  }
  i64 count(i64 i) const { return i < min_ ? cc : cc - (i - min_) - 1; }
};

// Per-row in-window entries of rows [r0, r1) (generation order), two
// parallel passes: count, then fill at prefix offsets.
void band_rows(const Band &bd, const Block &b, i64 r0, i64 r1, u64 c, double q, unsigned s,
               std::vector<i64> &off, std::vector<int> *cols, std::vector<int> *rowsv) {
  const i64 R = std::max<i64>(r1 - r0, 0);
  off.assign((size_t)R + 1, 0);
#pragma omp parallel for schedule(static)
  for (i64 k = 0; k < R; ++k) {
    const i64 i = r0 + k, st = bd.start(i), n = std::max<i64>(bd.count(i), 0);
    i64 cnt = 0;
    for (i64 j = 0; j < n; ++j) {
      const Entry e = cqmat_entry((u64)(st + j), (u64)b.nr, (u64)b.nc, c, q, s);
      if (b.in(e.row, e.col)) ++cnt;
    }
    off[k + 1] = cnt;
  }
  for (i64 k = 0; k < R; ++k) off[k + 1] += off[k];
  if (cols) cols->resize((size_t)off[R]);
  if (rowsv) rowsv->resize((size_t)off[R]);
#pragma omp parallel for schedule(static)
  for (i64 k = 0; k < R; ++k) {
    const i64 i = r0 + k, st = bd.start(i), n = std::max<i64>(bd.count(i), 0);
    i64 p = off[k];
    for (i64 j = 0; j < n; ++j) {
      const Entry e = cqmat_entry((u64)(st + j), (u64)b.nr, (u64)b.nc, c, q, s);
      if (b.in(e.row, e.col)) {
        if (cols) (*cols)[p] = (int)e.col;
        if (rowsv) (*rowsv)[p] = (int)e.row;
        ++p;
      }
    }
  }
}

// in-window draws over the index range [a, b)
i64 count_range(const Block &bl, i64 a, i64 e, u64 c, double q, unsigned s) {
  i64 cnt = 0;
#pragma omp parallel for schedule(static) reduction(+ : cnt)
  for (i64 i = a; i < e; ++i) {
    const Entry en = cqmat_entry((u64)i, (u64)bl.nr, (u64)bl.nc, c, q, s);
    if (bl.in(en.row, en.col)) ++cnt;
  }
  return cnt;
}

tbsla_status_t fill_cqmat(Out &o, int n_row, int n_col, int c, double q, unsigned s, int pr, int pc,
                          int NR, int NC) {
  Block b;
  set_block(o, b, n_row, n_col, pr, pc, NR, NC);
  o.values.clear(); o.idx0.clear(); o.idx1.clear();
  const i64 cc = std::min<i64>(c, n_col);
  Band bd{cc, std::min<i64>((i64)n_col - cc + 1, n_row), std::min<i64>(n_row, n_col)};

  if (o.format == TBSLA_FMT_COO) {
    // MatrixCOO::fill_cqmat (MatrixCOO.cpp:332-375): a share of the global
    // entry list, global indices, ln_row = NR and ln_col = NC as the
    // reference sets them
    o.geom[2] = NR; o.geom[3] = NC; o.geom[4] = 0; o.geom[5] = 0;
    const i64 gnv = bd.start(bd.mn);
    if (gnv == 0) return TBSLA_OK;
    const i64 s0 = pflv(gnv, pr * NC + pc, NR * NC), n = lnv(gnv, pr * NC + pc, NR * NC);
    o.nnz = n; o.nnz_set = true;
    o.values.assign((size_t)n, 1.0);
    o.idx0.resize((size_t)n);
    o.idx1.resize((size_t)n);
    bool dropped = false;
#pragma omp parallel for schedule(static) reduction(|| : dropped)
    for (i64 k = 0; k < n; ++k) {
      const Entry e = cqmat_entry((u64)(s0 + k), (u64)n_row, (u64)n_col, (u64)c, q, s);
      const int r = (int)e.row, cl = (int)e.col;  // push_back takes ints (MatrixCOO.cpp:118-126)
      const bool ok = r >= 0 && r < n_row && cl >= 0 && cl < n_col;
      o.idx0[(size_t)k] = ok ? r : -1;
      o.idx1[(size_t)k] = cl;
      dropped = dropped || !ok;
    }
    if (dropped) {  // push_back drops entries outside the shape
      size_t w = 0;
      for (size_t k = 0; k < (size_t)n; ++k)
        if (o.idx0[k] >= 0) { o.idx0[w] = o.idx0[k]; o.idx1[w] = o.idx1[k]; ++w; }
      o.idx0.resize(w); o.idx1.resize(w); o.values.resize(w);
    }
    return TBSLA_OK;
  }

  const i64 fr = b.fr, lr = b.lr;
  // entry rows [fr, gen_end): CSR/SCOO stop at min(n_row, n_col); ELL and
  // DENSE run to min(n_row, fr+lr) (rows past n_col have no entries)
  const i64 gen_end_csr = std::min(std::min<i64>(n_row, n_col), fr + lr);
  i64 nv = 0;
  for (i64 i = fr; i < std::min(bd.min_, fr + lr); ++i) nv += cc;
  for (i64 i = std::max(fr, bd.min_); i < gen_end_csr; ++i) nv += bd.count(i);

  if (o.format == TBSLA_FMT_CSR || o.format == TBSLA_FMT_SCOO) {
    // nnz: min(c,n_col) draws per row for every row, tail rows included
    // (MatrixCSR.cpp:343-358, MatrixSCOO.cpp:331-347)
    std::vector<i64> off;
    const bool any = nv != 0;
    band_rows(bd, b, fr, std::max(fr, gen_end_csr), (u64)c, q, s, off,
              any ? &o.idx1 : nullptr, (any && o.format == TBSLA_FMT_SCOO) ? &o.idx0 : nullptr);
    const i64 rows_counted = std::max<i64>(gen_end_csr - fr, 0);
    const i64 full_end = std::min(std::max(fr, std::min(bd.min_, fr + lr)), fr + rows_counted);
    i64 nnz = off[(size_t)(full_end - fr)];
    const i64 e = bd.start(std::min(fr, bd.mn)) + rows_counted * cc;
    // draws of the counting loop past the full rows
    const i64 cnt_from = bd.start(std::min(fr, bd.mn)) + (full_end - fr) * cc;
    if (e > cnt_from) nnz += count_range(b, cnt_from, e, (u64)c, q, s);
    o.nnz = nnz; o.nnz_set = true;
    if (!any) { o.idx0.clear(); o.idx1.clear(); return TBSLA_OK; }
    o.values.assign(o.idx1.size(), 1.0);
    if (o.format == TBSLA_FMT_CSR) {
      o.idx0.resize(off.size());
      for (size_t k = 0; k < off.size(); ++k) o.idx0[k] = (int)off[k];
    } else {
      // SCOO push_back drops entries outside the global shape (never the case
      // for in-window entries)
    }
    return TBSLA_OK;
  }

  if (o.format == TBSLA_FMT_ELL) {
    // MatrixELL::fill_cqmat (MatrixELL.cpp:262-392)
    const i64 fill_end = std::min<i64>(n_row, fr + lr);
    std::vector<i64> off;
    std::vector<int> cols;
    band_rows(bd, b, fr, std::max(fr, gen_end_csr), (u64)c, q, s, off, &cols, nullptr);
    i64 nnz = off.back();
    int max_col = 0;
    for (i64 i = fr; i < gen_end_csr; ++i) {
      i64 nbc = off[(size_t)(i - fr + 1)] - off[(size_t)(i - fr)];
      if (i >= bd.min_) {
        // the reference compares the slot index with the column window for
        // the slots a tail row does not draw (MatrixELL.cpp:338-342)
        for (i64 j = std::max<i64>(bd.count(i), 0); j < cc; ++j)
          if (j >= b.fc && j < b.fc + b.lc) ++nbc;
      }
      max_col = std::max<int>(max_col, (int)nbc);
    }
    o.nnz = nnz; o.nnz_set = true;
    o.geom[10] = max_col;
    if (nv == 0) return TBSLA_OK;
    const i64 rows_out = std::max<i64>(fill_end - fr, 0);
    o.values.assign((size_t)(rows_out * max_col), 0.0);
    o.idx0.assign((size_t)(rows_out * max_col), 0);
#pragma omp parallel for schedule(static)
    for (i64 k = 0; k < rows_out; ++k) {
      if (fr + k >= gen_end_csr) continue;
      const i64 a = off[(size_t)k], e = off[(size_t)k + 1];
      for (i64 p = a; p < e; ++p) {
        o.idx0[(size_t)(k * max_col + (p - a))] = cols[(size_t)p];
        o.values[(size_t)(k * max_col + (p - a))] = 1.0;
      }
    }
    return TBSLA_OK;
  }

  // DENSE (MatrixDENSE.cpp:192-271): duplicates accumulate
  if (nv == 0) return TBSLA_OK;
  std::vector<i64> off;
  std::vector<int> cols, rowsv;
  band_rows(bd, b, fr, std::max(fr, gen_end_csr), (u64)c, q, s, off, &cols, &rowsv);
  o.nnz = off.back(); o.nnz_set = true;
  const i64 lc = b.lc;
  o.values.assign((size_t)(lr * lc), 0.0);
  const i64 R = std::max<i64>(gen_end_csr - fr, 0);
#pragma omp parallel for schedule(static)
  for (i64 k = 0; k < R; ++k)
    for (i64 p = off[(size_t)k]; p < off[(size_t)k + 1]; ++p)
      o.values[(size_t)((rowsv[(size_t)p] - fr) * lc + (cols[(size_t)p] - b.fc))] += 1.0;
  return TBSLA_OK;
}

// column sums of the global cqmat (values_generation.cpp:47-62); every
// value is 1, so the sum of a column is its entry count
std::vector<double> cqmat_colsum(int n_row, int n_col, int c, double q, unsigned s) {
  const i64 cc = std::min<i64>(c, n_col);
  Band bd{cc, std::min<i64>((i64)n_col - cc + 1, n_row), std::min<i64>(n_row, n_col)};
  const i64 gnv = bd.start(bd.mn);
  std::vector<int> cnt((size_t)std::max(n_col, 1), 0);
#pragma omp parallel for schedule(static)
  for (i64 i = 0; i < gnv; ++i) {
    const Entry e = cqmat_entry((u64)i, (u64)n_row, (u64)n_col, (u64)c, q, s);
    __atomic_fetch_add(&cnt[(size_t)e.col], 1, __ATOMIC_RELAXED);
  }
  std::vector<double> sum((size_t)std::max(n_col, 1));
  for (int j = 0; j < n_col; ++j) sum[j] = (double)cnt[j];
  return sum;
}

tbsla_status_t fill_cqmat_stochastic(Out &o, int n_row, int n_col, int c, double q, unsigned s, int pr,
                                     int pc, int NR, int NC) {
  tbsla_status_t st = fill_cqmat(o, n_row, n_col, c, q, s, pr, pc, NR, NC);
  if (st != TBSLA_OK) return st;
  const bool has = !o.values.empty();
  if (!has && o.format != TBSLA_FMT_COO && o.format != TBSLA_FMT_SCOO) return TBSLA_OK;
  std::vector<double> sum = cqmat_colsum(n_row, n_col, c, q, s);
  switch (o.format) {
  case TBSLA_FMT_COO:
  case TBSLA_FMT_SCOO:
  case TBSLA_FMT_CSR:  // (MatrixCSR.cpp:411-421)
    for (size_t k = 0; k < o.values.size(); ++k) o.values[k] /= sum[(size_t)o.idx1[k]];
    break;
  case TBSLA_FMT_ELL: {  // (MatrixELL.cpp:394-404)
    for (size_t k = 0; k < o.values.size(); ++k)
      if (o.values[k] != 0) o.values[k] /= sum[(size_t)o.idx0[k]];
    break;
  }
  case TBSLA_FMT_DENSE: {  // (MatrixDENSE.cpp:273-286)
    for (auto &v : sum) if (v == 0) v = 1;
    const i64 lr = o.geom[2], lc = o.geom[3], fc = o.geom[5];
    for (i64 i = 0; i < lr; ++i)
      for (i64 j = 0; j < lc; ++j) o.values[(size_t)(i * lc + j)] /= sum[(size_t)(fc + j)];
    break;
  }
  }
  return TBSLA_OK;
}

// ------------------------------------------------------------- cdiag
tbsla_status_t fill_cdiag(Out &o, int n_row, int n_col, int cd, int pr, int pc, int NR, int NC) {
  Block b;
  set_block(o, b, n_row, n_col, pr, pc, NR, NC);
  o.values.clear(); o.idx0.clear(); o.idx1.clear();
  if (o.format == TBSLA_FMT_COO) {
    // MatrixCOO::fill_cdiag (MatrixCOO.cpp:294-330)
    o.geom[2] = NR; o.geom[3] = NC; o.geom[4] = 0; o.geom[5] = 0;
    i64 gnv = std::max<i64>(std::min<i64>(n_row, (i64)n_col - cd), 0) +
              std::max<i64>(std::min<i64>((i64)n_row - cd, n_col), 0);
    if (cd == 0) gnv /= 2;
    o.nnz = 0; o.nnz_set = true;
    if (gnv == 0) return TBSLA_OK;
    const i64 s0 = pflv(gnv, pr * NC + pc, NR * NC), n = lnv(gnv, pr * NC + pc, NR * NC);
    o.nnz = n;
    for (i64 i = s0; i < s0 + n; ++i) {
      const Entry e = cdiag_entry(i, n_col, cd);
      const int r = (int)e.row, cl = (int)e.col;
      if (r < 0 || r >= n_row || cl < 0 || cl >= n_col) continue;
      o.values.push_back(1.0); o.idx0.push_back(r); o.idx1.push_back(cl);
    }
    return TBSLA_OK;
  }
  // CSR (MatrixCSR.cpp:234-297), ELL (MatrixELL.cpp:192-260),
  // SCOO (MatrixSCOO.cpp:230-286), DENSE (MatrixDENSE.cpp:137-190)
  i64 nv = 0;
  for (i64 i = b.fr; i < b.fr + b.lr; ++i) {
    if (b.in(i, i - cd)) ++nv;
    if (cd != 0 && b.in(i, i + cd)) ++nv;
  }
  if (o.format == TBSLA_FMT_ELL) o.geom[10] = cd == 0 ? 1 : 2;
  if (nv == 0) return TBSLA_OK;
  // CSR and SCOO leave nnz unset in the reference; the stored count is given
  o.nnz = nv; o.nnz_set = true;
  switch (o.format) {
  case TBSLA_FMT_CSR: {
    o.idx0.reserve((size_t)b.lr + 1);
    o.idx0.push_back(0);
    int k = 0;
    for (i64 i = b.fr; i < b.fr + b.lr; ++i) {
      if (b.in(i, i - cd)) { o.idx1.push_back((int)(i - cd)); o.values.push_back(1); ++k; }
      if (cd != 0 && b.in(i, i + cd)) { o.idx1.push_back((int)(i + cd)); o.values.push_back(1); ++k; }
      o.idx0.push_back(k);
    }
    break;
  }
  case TBSLA_FMT_SCOO:
    for (i64 i = b.fr; i < b.fr + b.lr; ++i) {
      if (b.in(i, i - cd)) { o.values.push_back(1); o.idx0.push_back((int)i); o.idx1.push_back((int)(i - cd)); }
      if (cd != 0 && b.in(i, i + cd)) { o.values.push_back(1); o.idx0.push_back((int)i); o.idx1.push_back((int)(i + cd)); }
    }
    break;
  case TBSLA_FMT_ELL:
    for (i64 i = b.fr; i < b.fr + b.lr; ++i) {
      const bool lo = b.in(i, i - cd);
      o.idx0.push_back(lo ? (int)(i - cd) : 0); o.values.push_back(lo ? 1 : 0);
      if (cd != 0) {
        const bool hi = b.in(i, i + cd);
        o.idx0.push_back(hi ? (int)(i + cd) : 0); o.values.push_back(hi ? 1 : 0);
      }
    }
    break;
  case TBSLA_FMT_DENSE:
    o.values.assign((size_t)(b.lr * b.lc), 0.0);
    for (i64 i = b.fr; i < b.fr + b.lr; ++i) {
      if (b.in(i, i - cd)) o.values[(size_t)((i - b.fr) * b.lc + (i - cd - b.fc))] = 1;
      if (cd != 0 && b.in(i, i + cd)) o.values[(size_t)((i - b.fr) * b.lc + (i + cd - b.fc))] = 1;
    }
    break;
  }
  return TBSLA_OK;
}

// ---------------------------------------------------------- cqmat_baseline
// The cqmat matrix of the benchmark configuration n = 1e5, c = 10, q = 0.1:
// the reference's pattern (fill_cqmat, seed_mult as given), duplicates merged
// (each row's columns sorted, repeats kept once), values drawn uniform in
// (0, 1].  No reference counterpart beyond the pattern.  Value k (in (row,
// column) order) is 1 - u(seed_mult, 1, k) with u the SplitMix64 generator
// (Steele, Lea, Flood, OOPSLA 2014) started at state (stream << 32) | seed:
// output k = mix(state + (k + 1) * 0x9e3779b97f4a7c15), u = (output >> 11) *
// 2^-53.  Callers draw x from stream 2 the same way.
inline u64 splitmix64_at(u64 state, u64 k) {
  u64 z = state + (k + 1) * 0x9e3779b97f4a7c15ULL;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

tbsla_status_t fill_cqmat_baseline(Out &o, int n_row, int n_col, int c, double q, unsigned s, int pr, int pc,
                                   int NR, int NC) {
  if (pr != 0 || pc != 0 || NR != 1 || NC != 1)
    return tbsla::fail(TBSLA_ERR_INVALID_ARG, "cqmat_baseline is built for the whole matrix (block 0,0 of 1x1)");
  const int format = o.format;
  Out csr;
  csr.format = TBSLA_FMT_CSR;
  tbsla_status_t st = fill_cqmat(csr, n_row, n_col, c, q, s, 0, 0, 1, 1);
  if (st != TBSLA_OK) return st;
  // the fill's rowptr stops after the last row that can hold entries; the
  // merged matrix has every row (rows past it empty)
  const i64 filled = csr.idx0.empty() ? 0 : (i64)csr.idx0.size() - 1, rows = n_row;
  // merge: per row sort the columns, keep each once
  std::vector<i64> kept((size_t)rows + 1, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (i64 i = 0; i < filled; ++i) {
    int *b = csr.idx1.data() + csr.idx0[(size_t)i], *e = csr.idx1.data() + csr.idx0[(size_t)i + 1];
    std::sort(b, e);
    kept[(size_t)i + 1] = std::unique(b, e) - b;
  }
  for (i64 i = 0; i < rows; ++i) kept[(size_t)i + 1] += kept[(size_t)i];
  const i64 nnz = kept[(size_t)rows];
  std::vector<int> rowptr((size_t)rows + 1), colidx((size_t)nnz), rowof((size_t)nnz);
  std::vector<double> values((size_t)nnz);
  const u64 state = ((u64)1 << 32) | (u64)s;
  int longest = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(max : longest)
  for (i64 i = 0; i < rows; ++i) {
    const i64 b = kept[(size_t)i], len = kept[(size_t)i + 1] - b;
    rowptr[(size_t)i] = (int)b;
    if (len == 0) continue;
    for (i64 j = 0; j < len; ++j) {
      colidx[(size_t)(b + j)] = csr.idx1[(size_t)(csr.idx0[(size_t)i] + j)];
      rowof[(size_t)(b + j)] = (int)i;
      values[(size_t)(b + j)] = 1.0 - (double)(splitmix64_at(state, (u64)(b + j)) >> 11) * 0x1.0p-53;
    }
    longest = std::max(longest, (int)len);
  }
  rowptr[(size_t)rows] = (int)nnz;
  o = Out();
  o.format = format;
  Block b;
  set_block(o, b, n_row, n_col, 0, 0, 1, 1);
  o.nnz = nnz;
  o.nnz_set = true;
  switch (format) {
  case TBSLA_FMT_CSR:
    o.values = std::move(values); o.idx0 = std::move(rowptr); o.idx1 = std::move(colidx);
    break;
  case TBSLA_FMT_COO:
  case TBSLA_FMT_SCOO:
    o.values = std::move(values); o.idx0 = std::move(rowof); o.idx1 = std::move(colidx);
    break;
  case TBSLA_FMT_ELL: {  // as MatrixELL(const MatrixCOO&): padding (column 0, value 0)
    o.geom[10] = longest;
    o.values.assign((size_t)(b.lr * longest), 0.0);
    o.idx0.assign((size_t)(b.lr * longest), 0);
    for (i64 i = 0; i < rows; ++i)
      for (i64 k = rowptr[(size_t)i]; k < rowptr[(size_t)i + 1]; ++k) {
        const size_t slot = (size_t)(i * longest + (k - rowptr[(size_t)i]));
        o.values[slot] = values[(size_t)k];
        o.idx0[slot] = colidx[(size_t)k];
      }
    break;
  }
  default:  // DENSE, as MatrixDENSE(const MatrixCOO&)
    o.values.assign((size_t)(b.lr * b.lc), 0.0);
    for (i64 i = 0; i < rows; ++i)
      for (i64 k = rowptr[(size_t)i]; k < rowptr[(size_t)i + 1]; ++k)
        o.values[(size_t)(i * b.lc + colidx[(size_t)k])] += values[(size_t)k];
    break;
  }
  return TBSLA_OK;
}

}  // namespace

namespace tbsla {

tbsla_status_t generate_arrays(int format, int gen, int n_row, int n_col, int c, double q,
                               unsigned int seed_mult, int pr, int pc, int NR, int NC,
                               GenArrays &o) {
  if (format < TBSLA_FMT_COO || format > TBSLA_FMT_DENSE)
    return fail(TBSLA_ERR_INVALID_ARG, "unknown format %d", format);
  if (n_row < 0 || n_col < 0 || NR < 1 || NC < 1 || pr < 0 || pc < 0 || pr >= NR || pc >= NC)
    return fail(TBSLA_ERR_INVALID_ARG, "bad geometry");
  if (gen != 1 && c < 0) return fail(TBSLA_ERR_INVALID_ARG, "c must be >= 0");
  o = GenArrays();
  o.format = format;
  if (gen == 0) return fill_cqmat(o, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC);
  if (gen == 1) return fill_cdiag(o, n_row, n_col, c, pr, pc, NR, NC);
  if (gen == 2) return fill_cqmat_stochastic(o, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC);
  if (gen == 3) return fill_cqmat_baseline(o, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC);
  return fail(TBSLA_ERR_INVALID_ARG, "unknown generator %d", gen);
}

void cqmat_entry_tagged(uint64_t i, uint64_t nr, uint64_t nc, uint64_t c, double q, unsigned int seed_mult,
                        int64_t &row, int64_t &col, int &tag) {
  const Entry e = cqmat_entry(i, nr, nc, c, q, seed_mult);
  const u64 cc = std::min(nc, c);
  tag = i < cc * std::min(nc - cc + 1, nr) ? 30 : 31;
  row = e.row;
  col = e.col;
}

void cdiag_entry_tagged(int64_t i, int64_t nc, int64_t cd, int64_t &row, int64_t &col, int &tag) {
  const Entry e = cdiag_entry(i, nc, cd);
  if (cd == 0) tag = 10;
  else if (i < std::max(std::min(nc - cd, cd), (i64)0)) tag = 30;
  else if (i < std::max(cd + 2 * (nc - 2 * cd), (i64)0)) tag = (i % 2 == 0) ? 31 : 32;
  else tag = 33;
  row = e.row;
  col = e.col;
}

std::vector<double> cqmat_column_sums(int n_row, int n_col, int c, double q, unsigned int seed_mult) {
  return cqmat_colsum(n_row, n_col, c, q, seed_mult);
}

}  // namespace tbsla

extern "C" tbsla_status_t tbsla_generate(int format, int gen, int n_row, int n_col, int c, double q,
                                         unsigned int seed_mult, int pr, int pc, int NR, int NC,
                                         int64_t sizes[3], int geom[11], int64_t *nnz,
                                         double *values, int *idx0, int *idx1) {
  if (!sizes) return tbsla::fail(TBSLA_ERR_INVALID_ARG, "sizes is NULL");
  // The arrays are regenerated for the second call: the call stays
  // stateless.  tbsla_generate_matrix builds a handle in one pass.
  Out o;
  tbsla_status_t st = tbsla::generate_arrays(format, gen, n_row, n_col, c, q, seed_mult, pr, pc, NR, NC, o);
  if (st != TBSLA_OK) return st;
  if (!values && !idx0 && !idx1) {
    sizes[0] = (int64_t)o.values.size();
    sizes[1] = (int64_t)o.idx0.size();
    sizes[2] = (int64_t)o.idx1.size();
  } else {
    if (sizes[0] < (int64_t)o.values.size() || sizes[1] < (int64_t)o.idx0.size() ||
        sizes[2] < (int64_t)o.idx1.size())
      return tbsla::fail(TBSLA_ERR_INVALID_ARG, "output arrays too small");
    if (values && !o.values.empty()) std::memcpy(values, o.values.data(), o.values.size() * sizeof(double));
    if (idx0 && !o.idx0.empty()) std::memcpy(idx0, o.idx0.data(), o.idx0.size() * sizeof(int));
    if (idx1 && !o.idx1.empty()) std::memcpy(idx1, o.idx1.data(), o.idx1.size() * sizeof(int));
  }
  if (geom) std::memcpy(geom, o.geom, sizeof o.geom);
  if (nnz) *nnz = o.nnz_set ? o.nnz : 0;
  return TBSLA_OK;
}

extern "C" tbsla_status_t tbsla_generate_matrix(int format, int gen, int n_row, int n_col, int c,
                                                double q, unsigned int seed_mult, int stores,
                                                tbsla_matrix_t **out) {
  if (!out) return tbsla::fail(TBSLA_ERR_INVALID_ARG, "out is NULL");
  *out = nullptr;
  Out o;
  tbsla_status_t st = tbsla::generate_arrays(format, gen, n_row, n_col, c, q, seed_mult, 0, 0, 1, 1, o);
  if (st != TBSLA_OK) return st;
  const int *g = o.geom;
  switch (format) {
  case TBSLA_FMT_CSR: {
    static const int zero = 0;
    const int rows = o.idx0.empty() ? 0 : (int)o.idx0.size() - 1;
    return tbsla_csr_create(g[0], g[1], g[5], rows, o.idx0.empty() ? &zero : o.idx0.data(), o.idx1.data(),
                            o.values.data(), stores, out);
  }
  case TBSLA_FMT_ELL: {
    const int mc = g[10];
    const int rows = mc ? (int)std::min<int64_t>(g[2], (int64_t)o.values.size() / mc) : 0;
    return tbsla_ell_create(g[0], g[1], g[5], rows, mc, o.idx0.data(), o.values.data(), stores, out);
  }
  case TBSLA_FMT_COO:
  case TBSLA_FMT_SCOO:
    return tbsla_coo_create(g[0], g[1], format == TBSLA_FMT_SCOO ? g[4] : 0, format == TBSLA_FMT_SCOO ? g[5] : 0,
                            (int64_t)o.values.size(), o.idx0.data(), o.idx1.data(), o.values.data(), stores, out);
  default:
    return tbsla_dense_create(g[0], g[1], o.values.empty() ? 0 : g[2], g[3], o.values.data(), stores, out);
  }
}
