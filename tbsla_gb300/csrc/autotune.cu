// autotune.cu -- choices made by measurement on the operands at hand.
//
// Each tuner times its candidates with CUDA events on a private stream
// (after one untimed run of each, so first-touch costs do not count), keeps
// the fastest, and stores it where the library reads it: the CSR product's
// kernel variant, staged short-row kernel and x L2-keep fraction
// (tbsla_matrix_set_variant / TBSLA_TUNE_SHORT_ROWS / TBSLA_TUNE_X_L2_KEEP),
// the persistent grid of a matrix batch
// (tbsla_batch_tune), the tile width of batched PageRank (used when
// tbsla_ppr_batched is called with tile 0).  Results never depend on these
// choices, only times do.
#include <vector>

#include "common.cuh"

extern "C" tbsla_status_t tbsla_ppr_batched(const tbsla_matrix_t *A, const tbsla_pagerank_params_t *p, int k,
                                            const int *nodes, const int *offsets, int tile, double *d_out,
                                            int *iterations, double *residuals, void *stream);

using namespace tbsla;

namespace {

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  Timer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  ~Timer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

template <typename F> tbsla_status_t time_ms(cudaStream_t s, int reps, F run, float *ms) {
  Timer t;
  TB_TRY(run());  // untimed
  TB_CUDA(cudaStreamSynchronize(s));
  TB_CUDA(cudaEventRecord(t.a, s));
  for (int r = 0; r < reps; ++r) TB_TRY(run());
  TB_CUDA(cudaEventRecord(t.b, s));
  TB_CUDA(cudaEventSynchronize(t.b));
  TB_CUDA(cudaEventElapsedTime(ms, t.a, t.b));
  *ms /= reps;
  return TBSLA_OK;
}

}  // namespace

extern "C" {

tbsla_status_t tbsla_autotune_spmv(tbsla_matrix_t *A, tbsla_dtype_t store, tbsla_autotune_result_t *res) {
  TB_CHECK(A, "matrix is NULL");
  TB_CHECK(A->values[store == TBSLA_F64 ? 0 : store == TBSLA_F32 ? 1 : 2], "the value store is not present");
  TB_CUDA(cudaSetDevice(A->device));
  const tbsla_dtype_t vt = store == TBSLA_F64 ? TBSLA_F64 : TBSLA_F32;
  const size_t el = vt == TBSLA_F64 ? 8 : 4;
  void *x = nullptr, *y = nullptr;
  TB_CUDA(cudaMalloc(&x, std::max<size_t>((size_t)A->n_col, 1) * el));
  if (cudaMalloc(&y, std::max<size_t>((size_t)A->n_row, 1) * el) != cudaSuccess) {
    cudaFree(x);
    return fail(TBSLA_ERR_OOM, "autotune vectors");
  }
  cudaMemset(x, 0, std::max<size_t>((size_t)A->n_col, 1) * el);
  cudaStream_t s;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  const float keeps[] = {0.0f, 0.3f, 0.6f, 1.0f};
  // kernels: 0 direct, 1 row blocks (CSR), 2 direct with the staged
  // short-row kernel (every row at most 32 entries), 3 direct with two lanes
  // per short row, 4 direct with warp tiles of tiny rows (every row at most
  // kTinyRow entries, in order: the default rule, TBSLA_TUNE_SHORT_ROWS -1),
  // 5 the ELL-layout copy (TBSLA_TUNE_SHORT_ROWS 3; F64 / F32 stores of
  // handles that keep one)
  const bool csr = A->format == TBSLA_FMT_CSR;
  const bool tiny = A->n_short > 0 && A->short_rows == nullptr && A->short_max <= kTinyRow;
  const bool sliced = A->sell_width > 0 && store != TBSLA_BF16 && A->sell_vals[store == TBSLA_F64 ? 0 : 1];
  auto mode_of = [](int v) { return v == 2 ? 1 : v == 3 ? 2 : v == 4 ? -1 : v == 5 ? 3 : 0; };
  float best = 1e30f;
  int best_v = A->csr_variant == 1 ? 1 : A->short_mode == 1 ? 2 : A->short_mode == 2 ? 3
               : (A->short_mode < 0 || A->short_mode == 3) && sliced ? 5
               : (A->short_mode < 0 && tiny) ? 4 : 0;
  const int mode_in = A->short_mode;
  float best_k = A->x_keep;
  tbsla_status_t st = TBSLA_OK;
  int tried = 0;
  for (int v = 0; v < 6 && st == TBSLA_OK; ++v) {
    if (v == 1 && !csr) continue;
    if (v == 2 && A->stage_cap == 0) continue;
    if (v == 3 && A->n_short == 0) continue;
    if (v == 4 && !tiny) continue;
    if (v == 5 && !sliced) continue;
    for (float k : keeps) {
      if (csr) A->csr_variant = v == 1 ? 1 : 0;
      A->short_mode = mode_of(v);
      A->x_keep = k;
      float ms = 0;
      st = time_ms(s, 5, [&] { return tbsla_spmv_ex(A, store, vt, x, vt, y, 0, s); }, &ms);
      if (st != TBSLA_OK) break;
      ++tried;
      if (ms < best) { best = ms; best_v = v; best_k = k; }
      if (v == 1) break;  // the row-block kernel does not read x_keep
    }
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  cudaFree(x);
  cudaFree(y);
  if (csr) A->csr_variant = best_v == 1 ? 1 : 0;
  A->short_mode = mode_of(best_v);
  if (tried == 0) A->short_mode = mode_in;
  if (A->pr_relabel) A->pr_relabel->short_mode = A->short_mode;
  A->x_keep = best_k;
  if (res) {
    res->candidates = tried;
    res->best_ms = best;
    res->choice = best_v;
    res->value = best_k;
  }
  return st;
}

tbsla_status_t tbsla_autotune_batch(tbsla_batch_t *B, tbsla_autotune_result_t *res) {
  TB_CHECK(B, "batch is NULL");
  cudaStream_t s;
  TB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const int cands[] = {2, 4, 6, 8, 12, 16, 24, 32};
  float best = 1e30f;
  int best_c = 6, tried = 0;
  tbsla_status_t st = TBSLA_OK;
  for (int c : cands) {
    st = tbsla_batch_tune(B, c);
    float ms = 0;
    if (st == TBSLA_OK) st = time_ms(s, 5, [&] { return tbsla_batch_spmv(B, s); }, &ms);
    if (st != TBSLA_OK) break;
    ++tried;
    if (ms < best) { best = ms; best_c = c; }
  }
  cudaStreamSynchronize(s);
  cudaStreamDestroy(s);
  if (st == TBSLA_OK) st = tbsla_batch_tune(B, best_c);
  if (res) {
    res->candidates = tried;
    res->best_ms = best;
    res->choice = best_c;
    res->value = best_c;
  }
  return st;
}

tbsla_status_t tbsla_autotune_ppr(tbsla_matrix_t *A, int k, tbsla_dtype_t precision, tbsla_autotune_result_t *res) {
  TB_CHECK(A && k > 0, "bad argument");
  TB_CHECK(precision == TBSLA_F64 || precision == TBSLA_F32, "precision must be TBSLA_F64 or TBSLA_F32");
  TB_CUDA(cudaSetDevice(A->device));
  // k single-seed vectors spread over the graph, 3 sweeps each
  std::vector<int> nodes((size_t)k), offsets((size_t)k + 1);
  for (int c = 0; c < k; ++c) {
    nodes[(size_t)c] = (int)(((long long)c * 7919 + 13) % A->n_row);
    offsets[(size_t)c] = c;
  }
  offsets[(size_t)k] = k;
  double *out = nullptr;
  TB_CUDA(cudaMalloc(&out, (size_t)k * A->n_row * sizeof(double)));
  tbsla_pagerank_params_t p{};
  p.beta = 0.85;
  p.tol = 0.0;
  p.max_iter = 3;
  p.mode = TBSLA_PR_TELEPORT;
  p.precision = precision;
  p.check_every = 3;
  // narrow tiles keep a tile's iterates in L2 (n * KT values), wide ones
  // stream the matrix fewer times per vector
  const int tiles[] = {2, 4, 8, 16, 32};
  float best = 1e30f;
  int best_t = 32, tried = 0;
  tbsla_status_t st = TBSLA_OK;
  Timer t;
  for (int tile : tiles) {
    if (tile > 8 && tile > k) break;
    st = tbsla_ppr_batched(A, &p, k, nodes.data(), offsets.data(), tile, out, nullptr, nullptr, nullptr);
    if (st != TBSLA_OK) break;
    cudaEventRecord(t.a, nullptr);
    st = tbsla_ppr_batched(A, &p, k, nodes.data(), offsets.data(), tile, out, nullptr, nullptr, nullptr);
    cudaEventRecord(t.b, nullptr);
    cudaEventSynchronize(t.b);
    float ms = 0;
    cudaEventElapsedTime(&ms, t.a, t.b);
    if (st != TBSLA_OK) break;
    ++tried;
    if (ms < best) { best = ms; best_t = tile; }
  }
  cudaFree(out);
  if (st == TBSLA_OK) A->ppr_tile[precision == TBSLA_F64 ? 0 : 1] = best_t;
  if (res) {
    res->candidates = tried;
    res->best_ms = best;
    res->choice = best_t;
    res->value = best_t;
  }
  return st;
}

}  // extern "C"
