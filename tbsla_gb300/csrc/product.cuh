// product.cuh -- launches of the SpMV kernels of every format with an
// epilogue functor (shared by the plain products and PageRank).
//
// Every epilogue provides:
//   active()             false once its computation is finished (PageRank
//                        sweeps after convergence): kernels return at once;
//   emit(row, v, state)  receives each finished row exactly once;
//   block_done / fixup_done(state, block)  per-block reduction hooks;
//   set_part_base(k)     offset of the launch's blocks in a partials array.
#pragma once

#include <algorithm>

#include "common.cuh"
#include "csr_direct.cuh"
#include "csr_rows.cuh"
#include "spmv_kernels.cuh"

namespace tbsla {

// grids of the grid-stride CSR kernels.  Plain products take one row (one
// warp item) per thread (warp): the most loads in flight.  Epilogues that
// reduce per block cap the grid at kStrideBlocks blocks, so that each
// block's reduction covers many rows and the partials stay few.
constexpr int kStrideBlocks = 152 * 16;
inline int short_grid(int n_short, bool reduces) {
  const int g = (int)(((int64_t)n_short + 255) / 256);
  return std::max(1, reduces ? std::min(g, kStrideBlocks) : g);
}
inline int group_grid(int n_items, int lanes, bool reduces) {
  const int per_block = 256 / lanes;
  const int g = (int)(((int64_t)n_items + per_block - 1) / per_block);
  return std::max(1, reduces ? std::min(g, kStrideBlocks) : g);
}
inline int fixup_grid(int n) { return std::max(1, (n + 127) / 128); }

template <typename Acc> inline Carry<Acc> carry_of(const tbsla_matrix *A);
template <> inline Carry<double> carry_of<double>(const tbsla_matrix *A) {
  return Carry<double>{A->tile_head_row, A->tile_head_val, A->tile_tail_val, A->tile_emitted};
}
template <> inline Carry<float> carry_of<float>(const tbsla_matrix *A) {
  return Carry<float>{A->tile_head_row, A->tile_head_val32, A->tile_tail_val32, A->tile_emitted};
}

// ------------------------------------------------------------ launches
// Dynamic shared memory of csr_rows_kernel (set once per instantiation).
template <typename V, typename XT, typename Epi> size_t csr_rows_setup() {
  constexpr size_t smem = csr_rows_smem<typename Epi::Acc>();
  static bool done = false;
  if (!done) {
    cudaFuncSetAttribute(csr_rows_kernel<V, XT, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    done = true;
  }
  return smem;
}

template <typename Acc> inline Acc *huge_partials_of(const tbsla_matrix *A);
template <> inline double *huge_partials_of<double>(const tbsla_matrix *A) { return A->huge_partials; }
template <> inline float *huge_partials_of<float>(const tbsla_matrix *A) { return A->huge_partials32; }
template <typename Acc> inline Acc *chunk_partials_of(const tbsla_matrix *A);
template <> inline double *chunk_partials_of<double>(const tbsla_matrix *A) { return A->chunk_partials; }
template <> inline float *chunk_partials_of<float>(const tbsla_matrix *A) { return A->chunk_partials32; }

// The handle's L2 policy on the gathered vector (x of type XT).  The range
// form needs the vector's bytes in 32 bits; larger vectors keep a fraction.
template <typename XT> inline XKeep xkeep_of(const tbsla_matrix *A) {
  XKeep k{A->x_keep, 0u};
  const int64_t bytes = A->x_extent * (int64_t)sizeof(XT);
  if (A->x_keep_range && bytes > 0 && bytes <= (int64_t)0xffffffffll) k.range = (uint32_t)bytes;
  return k;
}

// Reducing epilogues take the short list's tiny head (n_tiny rows of at most
// kTinyRow entries) in warp tiles when the short-row kernel is the default.
template <typename Epi> inline bool tiny_split(const tbsla_matrix *A) {
  return Epi::kReduces && A->n_tiny > 0 && A->short_rows != nullptr && A->short_mode <= 0;
}
// the partial slots the short-row launches of a reducing epilogue write
inline int short_parts_reducing(const tbsla_matrix *A) {
  if (A->n_short == 0) return 0;
  if (A->n_tiny > 0 && A->short_rows != nullptr && A->short_mode <= 0) {
    const int rest = A->n_short - A->n_tiny;
    return tiny_list_grid(A->n_tiny, true) + (rest > 0 ? short_grid(rest, true) : 0);
  }
  return short_grid(A->n_short, true);
}

// The staged kernel applies when every row is short (stage_cap > 0) and the
// handle's stage mode (tbsla_matrix_tune) is on.
inline bool stage_on(const tbsla_matrix *A) {
  return A->stage_cap > 0 && A->short_rows == nullptr && A->short_mode == 1 &&
         A->stage_cap <= kStageCapMax;
}
// dynamic shared memory of csr_stage_kernel (the attribute is raised once per
// instantiation to the largest capacity)
template <typename V, typename XT, typename Epi> size_t csr_stage_setup(int cap) {
  static bool done = false;
  if (!done) {
    cudaFuncSetAttribute(csr_stage_kernel<V, XT, Epi>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)csr_stage_smem<V>(kStageCapMax));
    done = true;
  }
  return csr_stage_smem<V>(cap);
}

// Rows per thread of csr_sell_kernel: the handle's setting, else 2 (cqmat
// 7e4 to 1.6e7 rows, c 8 to 32, FP32 and FP64: 2 the fastest or within 3 %;
// the 2^24 FP64 product 0.625 ms against 0.646 with 4 and more with 1)
inline int sell_rows_per_thread(const tbsla_matrix *A) {
  return A->sell_rows > 0 ? A->sell_rows : 2;
}

// The sliced copy of the value store `vals` (csr_sell_kernel), when the
// handle has one and plain products take it: the default short-row mode, or
// mode 3; F64 and F32 stores (BF16 slots load 64 bytes per warp instruction:
// cqmat 2^24 0.366 ms against 0.334 with one thread per row)
template <typename V, typename Epi> inline const V *sell_vals_for(const tbsla_matrix *A, const V *vals) {
  if constexpr (sizeof(V) < 4) {
    return nullptr;  // BF16: the copy is not kept
  } else {
    if (Epi::kReduces || !A->sell_width || !(A->short_mode == -1 || A->short_mode == 3)) return nullptr;
    for (int k = 0; k < 2; ++k)
      if (A->values[k] == static_cast<const void *>(vals)) return static_cast<const V *>(A->sell_vals[k]);
    return nullptr;
  }
}

// The direct CSR launches (row bins of the handle) over rowptr / colidx:
// the CSR arrays of a CSR handle, or the derived row pointer of a row-sorted
// COO handle.
template <typename V, typename XT, typename Epi>
tbsla_status_t launch_csr_direct(const tbsla_matrix *A, const int *rowptr, const int *colidx, const V *vals,
                                 const XT *x, Epi epi, cudaStream_t s) {
  using Acc = typename Epi::Acc;
  KernelTimer kt(A, s);
  int base = 0;
  if (const V *sv = sell_vals_for<V, Epi>(A, vals)) {
    // every row short, the ELL-layout copy: one warp per 32 R rows
    const int R = sell_rows_per_thread(A);
    const int64_t threads = A->sell_stride / (32 * R) * 32;
    const int grid = (int)((threads + 255) / 256);
    if (R == 4)
      csr_sell_kernel<4, V, XT, Epi><<<grid, 256, 0, s>>>(A->sell_cols, sv, A->sell_stride, A->sell_width, x,
                                                          A->f_col, A->rows, xkeep_of<XT>(A), epi);
    else if (R == 2)
      csr_sell_kernel<2, V, XT, Epi><<<grid, 256, 0, s>>>(A->sell_cols, sv, A->sell_stride, A->sell_width, x,
                                                          A->f_col, A->rows, xkeep_of<XT>(A), epi);
    else
      csr_sell_kernel<1, V, XT, Epi><<<grid, 256, 0, s>>>(A->sell_cols, sv, A->sell_stride, A->sell_width, x,
                                                          A->f_col, A->rows, xkeep_of<XT>(A), epi);
    kt.stop();
    return TBSLA_OK;
  }
  if (A->n_short > 0 && stage_on(A)) {
    // all rows short: the staged kernel (reducing epilogues: the same grid as
    // the short-row kernel, so that every partial slot is written)
    const size_t smem = csr_stage_setup<V, XT, Epi>(A->stage_cap);
    const int tiles = (A->n_short + 31) / 32;
    const int grid = Epi::kReduces ? short_grid(A->n_short, true)
                                   : std::max(1, std::min((tiles + kStageWarps - 1) / kStageWarps, kStrideBlocks));
    epi.set_part_base(base);
    base += short_grid(A->n_short, Epi::kReduces);
    csr_stage_kernel<V, XT, Epi><<<grid, kStageWarps * 32, smem, s>>>(A->n_short, rowptr, colidx, vals, x, A->f_col,
                                                                     xkeep_of<XT>(A), A->stage_cap, epi);
  } else if (A->n_short > 0 && A->short_rows == nullptr && A->short_mode < 0 && !Epi::kReduces &&
             A->short_max <= kTinyRow) {
    // every row in order and tiny: warp tiles of 32 * 8 / T rows
    const int T = A->short_max <= 2 ? 2 : 4;
    const int64_t warps = ((int64_t)A->n_short + 32 * (8 / T) - 1) / (32 * (8 / T));
    const int grid = (int)((warps * 32 + 255) / 256);
    epi.set_part_base(base);
    base += short_grid(A->n_short, Epi::kReduces);
    if (T == 2)
      csr_tiny_kernel<2, V, XT, Epi><<<grid, 256, 0, s>>>(A->n_short, rowptr, colidx, vals, x, A->f_col,
                                                          xkeep_of<XT>(A), epi);
    else
      csr_tiny_kernel<4, V, XT, Epi><<<grid, 256, 0, s>>>(A->n_short, rowptr, colidx, vals, x, A->f_col,
                                                          xkeep_of<XT>(A), epi);
  } else if (A->n_short > 0 && tiny_split<Epi>(A)) {
    // the tiny head in warp tiles, the rest one thread per row
    const int grid = tiny_list_grid(A->n_tiny, true);
    epi.set_part_base(base);
    base += grid;
    csr_tiny_list_kernel<V, XT, Epi><<<grid, 256, 0, s>>>(A->short_rows, A->n_tiny, rowptr, colidx, vals, x,
                                                          A->f_col, xkeep_of<XT>(A), epi);
    const int rest = A->n_short - A->n_tiny;
    if (rest > 0) {
      epi.set_part_base(base);
      base += short_grid(rest, true);
      csr_short_kernel<V, XT, Epi><<<short_grid(rest, true), 256, 0, s>>>(
          A->short_rows + A->n_tiny, rest, rowptr, colidx, vals, x, A->f_col, xkeep_of<XT>(A), epi);
    }
  } else if (A->n_short > 0 && (A->short_mode == 2 || (A->short_mode < 0 && sizeof(V) == 8 && !Epi::kReduces &&
                                                       A->short_nnz >= (int64_t)kPairMinRow * A->n_short))) {
    // two lanes per row: twice the threads of the one-lane grid (reducing
    // epilogues: the same capped grid, so every partial slot is written)
    const int grid = Epi::kReduces ? short_grid(A->n_short, true) : short_grid(2 * A->n_short, false);
    epi.set_part_base(base);
    base += short_grid(A->n_short, Epi::kReduces);
    csr_pair_kernel<V, XT, Epi><<<grid, 256, 0, s>>>(A->short_rows, A->n_short, rowptr, colidx, vals, x, A->f_col,
                                                     xkeep_of<XT>(A), epi);
  } else if (A->n_short > 0) {
    epi.set_part_base(base);
    base += short_grid(A->n_short, Epi::kReduces);
    csr_short_kernel<V, XT, Epi><<<short_grid(A->n_short, Epi::kReduces), 256, 0, s>>>(
        A->short_rows, A->n_short, rowptr, colidx, vals, x, A->f_col, xkeep_of<XT>(A), epi);
  }
  for (int c = 0; c < kGroupClasses; ++c) {
    const int first = A->item_class_start[c], count = A->item_class_start[c + 1] - first;
    if (count == 0) continue;
    const int grid = group_grid(count, kGroupLanes[c], Epi::kReduces);
    epi.set_part_base(base);
    base += grid;
    const int4 *items = A->warp_items + first;
    Acc *parts = chunk_partials_of<Acc>(A);
    switch (kGroupLanes[c]) {
    case 4:
      csr_group_kernel<4, V, XT, Epi><<<grid, 256, 0, s>>>(items, count, colidx, vals, x, A->f_col, xkeep_of<XT>(A), parts, epi);
      break;
    case 8:
      csr_group_kernel<8, V, XT, Epi><<<grid, 256, 0, s>>>(items, count, colidx, vals, x, A->f_col, xkeep_of<XT>(A), parts, epi);
      break;
    case 16:
      csr_group_kernel<16, V, XT, Epi><<<grid, 256, 0, s>>>(items, count, colidx, vals, x, A->f_col, xkeep_of<XT>(A), parts, epi);
      break;
    default:
      csr_group_kernel<32, V, XT, Epi><<<grid, 256, 0, s>>>(items, count, colidx, vals, x, A->f_col, xkeep_of<XT>(A), parts, epi);
      break;
    }
  }
  kt.stop();
  if (A->n_chunk_rows > 0) {
    epi.set_part_base(base);
    csr_chunk_fixup_kernel<Epi><<<fixup_grid(A->n_chunk_rows), 128, 0, s>>>(
        A->chunk_rows, A->n_chunk_rows, chunk_partials_of<Acc>(A), epi);
  }
  return TBSLA_OK;
}

template <typename V, typename XT, typename Epi>
tbsla_status_t launch_product(const tbsla_matrix *A, const V *vals, const XT *x, Epi epi,
                              cudaStream_t s) {
  using Acc = typename Epi::Acc;
  switch (A->format) {
  case TBSLA_FMT_CSR:
    if (A->rows > 0 && A->csr_variant == 0) {
      TB_TRY(launch_csr_direct<V, XT>(A, A->idx0, A->idx1, vals, x, epi, s));
    } else if (A->rows > 0) {
      const size_t smem = csr_rows_setup<V, XT, Epi>();
      KernelTimer kt(A, s);
      csr_rows_kernel<V, XT, Epi><<<A->num_blocks, kRowsNT, smem, s>>>(
          A->row_blocks, A->idx0, A->idx1, vals, x, A->f_col, huge_partials_of<Acc>(A), epi);
      kt.stop();
      if (A->num_huge > 0)
        csr_huge_fixup_kernel<Epi><<<(A->num_huge + 127) / 128, 128, 0, s>>>(A->huge_rows, A->num_huge,
                                                                            huge_partials_of<Acc>(A), epi);
    }
    break;
  case TBSLA_FMT_COO:
  case TBSLA_FMT_SCOO:
    if (A->stored > 0 && A->coo_rowptr && A->csr_variant == 0) {
      TB_TRY(launch_csr_direct<V, XT>(A, A->coo_rowptr, A->idx1, vals, x, epi, s));
    } else if (A->stored > 0) {
      KernelTimer kt(A, s);
      coo_merge_kernel<kMergeThreads, kMergeItems, V, XT, Epi><<<A->num_tiles, kMergeThreads, 0, s>>>(
          A->idx0, A->idx1, vals, x, A->f_col, A->stored, carry_of<Acc>(A), epi);
      kt.stop();
      merge_fixup_kernel<Epi><<<(A->num_tiles + 255) / 256, 256, 0, s>>>(A->num_tiles, carry_of<Acc>(A), epi);
    }
    break;
  case TBSLA_FMT_ELL:
    if (A->rows > 0 && A->max_col > 0) {
      const bool cs = A->x_extent * (int64_t)sizeof(XT) <= (64ll << 20);
      KernelTimer kt(A, s);
      if (A->csr_variant == 0) {
        // warp tiles of 32 R rows (the default), R rows per thread
        // (TBSLA_TUNE_SELL_ROWS)
        const int R = sell_rows_per_thread(A);
        const int64_t threads = ((int64_t)A->rows + 32 * R - 1) / (32 * R) * 32;
        const int grid = (int)((threads + 255) / 256);
        const XKeep k = xkeep_of<XT>(A);
        if (cs && R == 4)
          ell_warp_kernel<V, XT, Epi, true, 4><<<grid, 256, 0, s>>>(A->idx0, vals, x, A->f_col, A->rows,
                                                                    A->rows_pad, A->max_col, k, epi);
        else if (cs && R == 2)
          ell_warp_kernel<V, XT, Epi, true, 2><<<grid, 256, 0, s>>>(A->idx0, vals, x, A->f_col, A->rows,
                                                                    A->rows_pad, A->max_col, k, epi);
        else if (cs)
          ell_warp_kernel<V, XT, Epi, true, 1><<<grid, 256, 0, s>>>(A->idx0, vals, x, A->f_col, A->rows,
                                                                    A->rows_pad, A->max_col, k, epi);
        else if (R == 4)
          ell_warp_kernel<V, XT, Epi, false, 4><<<grid, 256, 0, s>>>(A->idx0, vals, x, A->f_col, A->rows,
                                                                     A->rows_pad, A->max_col, k, epi);
        else if (R == 2)
          ell_warp_kernel<V, XT, Epi, false, 2><<<grid, 256, 0, s>>>(A->idx0, vals, x, A->f_col, A->rows,
                                                                     A->rows_pad, A->max_col, k, epi);
        else
          ell_warp_kernel<V, XT, Epi, false, 1><<<grid, 256, 0, s>>>(A->idx0, vals, x, A->f_col, A->rows,
                                                                     A->rows_pad, A->max_col, k, epi);
      } else {
        // four consecutive rows per thread
        const int threads = (A->rows + 3) / 4;
        if (cs)
          ell_kernel<V, XT, Epi, true><<<(threads + 255) / 256, 256, 0, s>>>(A->idx0, vals, x, A->f_col, A->rows,
                                                                             A->rows_pad, A->max_col, xkeep_of<XT>(A), epi);
        else
          ell_kernel<V, XT, Epi, false><<<(threads + 255) / 256, 256, 0, s>>>(A->idx0, vals, x, A->f_col, A->rows,
                                                                              A->rows_pad, A->max_col, xkeep_of<XT>(A), epi);
      }
      kt.stop();
    }
    break;
  case TBSLA_FMT_DENSE:
    if (A->rows > 0 && A->cols > 0) {
      const int warps = (A->rows + 3) / 4;
      KernelTimer kt(A, s);
      dense_kernel<V, XT, Epi><<<(warps + 7) / 8, 256, 0, s>>>(vals, x, A->rows, A->cols, epi);
      kt.stop();
    }
    break;
  default:
    return fail(TBSLA_ERR_INVALID_ARG, "unknown format %d", A->format);
  }
  TB_CUDA(cudaGetLastError());
  return TBSLA_OK;
}

}  // namespace tbsla
