// batch.cu -- many CSR matrices multiplied in one persistent launch.
//
// A batch holds a device table of its members (CSR handles: rowptr, colidx,
// values of one store, bound x and y) and a list of work items, each at most
// kBatchRows rows of one member.  One kernel launch walks the items with a
// static stride (block b takes items b, b + grid, ...), so the order of every
// sum is fixed and the launch needs no counter to reset: it can be replayed
// from a CUDA graph as is.  A row is summed by one thread in its stored
// order (the thread-per-row loads of csr_direct.cuh: the single products'
// arithmetic with TBSLA_TUNE_SHORT_ROWS = 0).  Members that keep the
// ELL-layout copy (csr_sell_kernel's arrays) for the bound store are read
// from it, two rows per thread (items of 2 * kBatchRows rows): the same sums,
// coalesced loads.  An optional device mask skips members (per-instance
// convergence masking for iterative callers).
#include <algorithm>
#include <vector>

#include "product.cuh"

namespace tbsla {

struct BatchMember {
  const int *rowptr;
  const int *colidx;
  const void *values;
  const void *x;
  void *y;
  int f_col, rows, n_row, sell_width;
  const int *sell_cols;     // the ELL-layout copy (NULL: none)
  const void *sell_vals;    // its values for the bound store (NULL: read the CSR arrays)
  int64_t sell_stride;
};

constexpr int kBatchRows = 256;

// The block-uniform item loop carries the next item's descriptor and member
// entry (and its mask flag) one iteration ahead: their dependent loads
// overlap the current rows' sums instead of preceding them.
template <typename V, typename T>
__global__ void __launch_bounds__(256) batch_spmv_kernel(const BatchMember *__restrict__ members,
                                                        const int4 *__restrict__ items, int n_items,
                                                        const int *__restrict__ mask) {
  using Acc = typename AccOf<T>::type;
  const uint64_t keep = policy_keep(0.6f);
  int i = blockIdx.x;
  if (i >= n_items) return;
  int4 w = items[i];
  BatchMember m = members[w.x];
  bool on = !mask || mask[w.x] != 0;
  for (; i < n_items; i += gridDim.x) {
    const int in = i + gridDim.x;
    int4 wn = w;
    BatchMember mn = m;
    bool onn = on;
    if (in < n_items) {
      wn = items[in];
      mn = members[wn.x];
      onn = !mask || mask[wn.x] != 0;
    }
    if (on) {  // `on` is uniform across the block
      T *y = static_cast<T *>(m.y);
      const T *x = static_cast<const T *>(m.x);
      const int ra = w.y + (int)threadIdx.x, rb = ra + kBatchRows;
      if (m.sell_vals) {
        // rows ra and rb from the ELL-layout copy, slot by slot (padding and
        // rows past m.rows hold column -1 or are not read)
        const V *sv = static_cast<const V *>(m.sell_vals);
        const bool ha = ra < w.z && ra < m.rows, hb = rb < w.z && rb < m.rows;
        Acc sa = 0, sb = 0;
        #pragma unroll 4
        for (int j = 0; j < m.sell_width; ++j) {
          const size_t off = (size_t)j * m.sell_stride;
          const int ca = ha ? ld_ell<false>(m.sell_cols + off + ra) : -1;
          const int cb = hb ? ld_ell<false>(m.sell_cols + off + rb) : -1;
          const V va = ha ? ld_ell<false>(sv + off + ra) : V(0);
          const V vb = hb ? ld_ell<false>(sv + off + rb) : V(0);
          if (ca >= 0) sa = fma_acc(to_acc(va, Acc()), to_acc(ld_keep(x + (ca - m.f_col), keep), Acc()), sa);
          if (cb >= 0) sb = fma_acc(to_acc(vb, Acc()), to_acc(ld_keep(x + (cb - m.f_col), keep), Acc()), sb);
        }
        if (ra < w.z) __stcs(y + ra, (T)sa);
        if (rb < w.z) __stcs(y + rb, (T)sb);
      } else {
        for (int r = ra; r < w.z; r += kBatchRows) {
          if (r >= m.rows) {
            y[r] = T(0);
          } else {
            const int a = __ldg(m.rowptr + r), b = __ldg(m.rowptr + r + 1);
            const Acc s = row_sum_thread<V, T, Acc>(m.colidx, static_cast<const V *>(m.values), x, m.f_col, a,
                                                    b, keep);
            __stcs(y + r, (T)s);
          }
        }
      }
    }
    w = wn;
    m = mn;
    on = onn;
  }
}

}  // namespace tbsla

using namespace tbsla;

struct tbsla_batch {
  int device = 0;
  std::vector<const tbsla_matrix *> members;
  std::vector<BatchMember> table;    // host copy of the member table
  BatchMember *d_table = nullptr;
  int4 *d_items = nullptr;
  int n_items = 0;
  const int *d_mask = nullptr;       // caller's mask or NULL
  int blocks_per_sm = 6;             // persistent grid: 152 x blocks_per_sm (tbsla_batch_tune)
  tbsla_dtype_t store = TBSLA_F64;   // value store chosen by tbsla_batch_bind
  bool bound = false;
  cudaGraphExec_t graph = nullptr;   // tbsla_batch_spmv_graph
  ~tbsla_batch() {
    if (graph) cudaGraphExecDestroy(graph);
    if (d_table) cudaFree(d_table);
    if (d_items) cudaFree(d_items);
  }
};

static tbsla_status_t batch_launch(tbsla_batch *B, tbsla_dtype_t store, cudaStream_t s) {
  if (B->n_items == 0) return TBSLA_OK;
  const int grid = std::max(1, std::min(B->n_items, 152 * B->blocks_per_sm));
  if (store == TBSLA_F64)
    batch_spmv_kernel<double, double><<<grid, 256, 0, s>>>(B->d_table, B->d_items, B->n_items, B->d_mask);
  else if (store == TBSLA_F32)
    batch_spmv_kernel<float, float><<<grid, 256, 0, s>>>(B->d_table, B->d_items, B->n_items, B->d_mask);
  else
    batch_spmv_kernel<__nv_bfloat16, float><<<grid, 256, 0, s>>>(B->d_table, B->d_items, B->n_items, B->d_mask);
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

extern "C" {

tbsla_status_t tbsla_batch_create(int count, const tbsla_matrix_t *const *members, tbsla_batch_t **out) {
  TB_CHECK(out, "out is NULL");
  *out = nullptr;
  TB_CHECK(count > 0 && members, "empty batch");
  tbsla_batch *B = new tbsla_batch();
  B->device = members[0]->device;
  std::vector<int4> items;
  for (int m = 0; m < count; ++m) {
    const tbsla_matrix *A = members[m];
    if (!A || A->format != TBSLA_FMT_CSR || A->device != B->device) {
      delete B;
      return fail(TBSLA_ERR_INVALID_ARG, "batch member %d is not a CSR handle on device %d", m, B->device);
    }
    B->members.push_back(A);
    BatchMember d{};
    d.rowptr = A->idx0;
    d.colidx = A->idx1;
    d.f_col = A->f_col;
    d.rows = A->rows;
    d.n_row = A->n_row;
    d.sell_width = A->sell_width;
    d.sell_cols = A->sell_cols;
    d.sell_stride = A->sell_stride;
    B->table.push_back(d);
    // members with the ELL-layout copy: items of two rows per thread
    const int span = A->sell_width ? 2 * kBatchRows : kBatchRows;
    for (int r = 0; r < A->n_row; r += span) items.push_back(make_int4(m, r, std::min(r + span, A->n_row), 0));
  }
  B->n_items = (int)items.size();
  cudaSetDevice(B->device);
  if (cudaMalloc(&B->d_table, sizeof(BatchMember) * count) != cudaSuccess ||
      cudaMalloc(&B->d_items, sizeof(int4) * std::max<size_t>(items.size(), 1)) != cudaSuccess ||
      (!items.empty() &&
       cudaMemcpy(B->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice) != cudaSuccess)) {
    cudaGetLastError();
    delete B;
    return fail(TBSLA_ERR_OOM, "batch tables");
  }
  *out = B;
  return TBSLA_OK;
}

tbsla_status_t tbsla_batch_bind(tbsla_batch_t *B, tbsla_dtype_t store, const void *const *d_x, void *const *d_y) {
  TB_CHECK(B && d_x && d_y, "NULL argument");
  TB_CHECK(store == TBSLA_F64 || store == TBSLA_F32 || store == TBSLA_BF16, "bad store");
  const int si = store_index(store);
  for (size_t m = 0; m < B->members.size(); ++m) {
    const tbsla_matrix *A = B->members[m];
    TB_CHECK(A->values[si], "batch member %zu lacks the requested value store", m);
    TB_CHECK(d_y[m] || A->n_row == 0, "y of member %zu is NULL", m);
    TB_CHECK(d_x[m] || A->stored == 0, "x of member %zu is NULL", m);
    B->table[m].values = A->values[si];
    B->table[m].sell_vals = A->sell_width && si < 2 ? A->sell_vals[si] : nullptr;
    B->table[m].x = d_x[m];
    B->table[m].y = d_y[m];
  }
  TB_CUDA(cudaSetDevice(B->device));
  TB_CUDA(cudaMemcpy(B->d_table, B->table.data(), sizeof(BatchMember) * B->table.size(), cudaMemcpyHostToDevice));
  B->bound = true;
  if (B->store != store && B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
  B->store = store;  // the graph holds the table's address, not its contents: rebinding keeps it valid
  return TBSLA_OK;
}

tbsla_status_t tbsla_batch_set_mask(tbsla_batch_t *B, const int *d_mask) {
  TB_CHECK(B, "batch is NULL");
  B->d_mask = d_mask;
  if (B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
  return TBSLA_OK;
}

tbsla_status_t tbsla_batch_tune(tbsla_batch_t *B, int blocks_per_sm) {
  TB_CHECK(B, "batch is NULL");
  TB_CHECK(blocks_per_sm >= 1 && blocks_per_sm <= 64, "blocks per SM %d outside [1, 64]", blocks_per_sm);
  B->blocks_per_sm = blocks_per_sm;
  if (B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
  return TBSLA_OK;
}

tbsla_status_t tbsla_batch_spmv(tbsla_batch_t *B, void *stream) {
  TB_CHECK(B && B->bound, "batch is NULL or has no bound vectors");
  TB_CUDA(cudaSetDevice(B->device));
  return batch_launch(B, B->store, (cudaStream_t)stream);
}

tbsla_status_t tbsla_batch_spmv_graph(tbsla_batch_t *B, void *stream) {
  TB_CHECK(B && B->bound, "batch is NULL or has no bound vectors");
  TB_CUDA(cudaSetDevice(B->device));
  cudaStream_t s = (cudaStream_t)stream;
  const tbsla_dtype_t store = B->store;
  if (!B->graph) {
    cudaStream_t cs;
    TB_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g = nullptr;
    tbsla_status_t st = TBSLA_OK;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) st = fail(TBSLA_ERR_CUDA, "capture");
    if (st == TBSLA_OK) st = batch_launch(B, store, cs);
    const cudaError_t e = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (st != TBSLA_OK) { if (g) cudaGraphDestroy(g); return st; }
    if (e != cudaSuccess) return fail(TBSLA_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    const cudaError_t ie = cudaGraphInstantiate(&B->graph, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return fail(TBSLA_ERR_CUDA, "cudaGraphInstantiate: %s", cudaGetErrorString(ie));
  }
  TB_CUDA(cudaGraphLaunch(B->graph, s));
  return TBSLA_OK;
}

tbsla_status_t tbsla_batch_destroy(tbsla_batch_t *B) {
  if (B) {
    cudaSetDevice(B->device);
    delete B;
  }
  return TBSLA_OK;
}

}  // extern "C"
