"""torch.autograd shims over the library's kernels.

``csr_spmv(A, values, x)`` is y = A x for a CSR handle whose stored values are
``values``; ``pagerank(A, values, v)`` is the teleport-form PageRank fixed
point x = beta A x + (beta d.x + 1 - beta) v (TBSLA_PR_TELEPORT).  Both are
differentiable with respect to the values and to x / v.  The backward passes
are the library's own kernels: the transposed product and the values
gradient for the SpMV, the adjoint fixed-point solve for PageRank.  torch only
carries the tensors and the stream; the forward writes ``values`` into the
handle (tbsla_matrix_set_values), so one handle serves every evaluation.
"""
from __future__ import annotations

import torch

from . import capi


def _code(dtype: torch.dtype) -> int:
    if dtype == torch.float64:
        return capi.F64
    if dtype == torch.float32:
        return capi.F32
    raise TypeError(f"unsupported dtype {dtype}")


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


class CsrSpMV(torch.autograd.Function):
    """y = A x; dL/dvalues[k] = dL/dy[row(k)] x[col(k)], dL/dx = A^T dL/dy."""

    @staticmethod
    def forward(ctx, values: torch.Tensor, x: torch.Tensor, matrix: "capi.DeviceMatrix"):
        if not (values.is_cuda and x.is_cuda) or values.dtype != x.dtype:
            raise ValueError("values and x must be CUDA tensors of one dtype")
        dt = _code(values.dtype)
        vals = values.detach().contiguous()
        xx = x.detach().contiguous()
        matrix.set_values(dt, vals.data_ptr(), _stream())
        info = matrix.info()
        y = torch.empty(info.n_row, dtype=x.dtype, device=x.device)
        matrix.spmv_ex(dt, dt, xx.data_ptr(), dt, y.data_ptr(), 0, _stream())
        ctx.matrix = matrix
        ctx.dt = dt
        ctx.shape = (int(info.stored), int(info.n_col))
        ctx.save_for_backward(xx)
        return y

    @staticmethod
    def backward(ctx, gy: torch.Tensor):
        (x,) = ctx.saved_tensors
        m, dt = ctx.matrix, ctx.dt
        nnz, n_col = ctx.shape
        gy = gy.contiguous()
        gvals = gx = None
        if ctx.needs_input_grad[0]:
            gvals = torch.empty(nnz, dtype=x.dtype, device=x.device)
            m.grad_values(dt, gy.data_ptr(), x.data_ptr(), 1.0, gvals.data_ptr(), _stream())
        if ctx.needs_input_grad[1]:
            gx = torch.empty(n_col, dtype=x.dtype, device=x.device)
            m.spmv_transpose_ex(dt, dt, gy.data_ptr(), dt, gx.data_ptr(), _stream())
        return gvals, gx, None


class PageRankTeleport(torch.autograd.Function):
    """x* of x = beta A x + (beta d.x + 1 - beta) v; gradients by the adjoint
    solve lambda = beta A^T lambda + beta d (v.lambda) + dL/dx*.  Both solves
    use Anderson acceleration unless accel = 0 (same fixed points and
    stopping rules, several times fewer sweeps for the adjoint)."""

    @staticmethod
    def forward(ctx, values, v, matrix, beta=0.85, tol=1e-14, max_iter=10000, accel=1):
        if values.dtype != torch.float64 or v.dtype != torch.float64:
            raise TypeError("PageRank runs in FP64")
        vals = values.detach().contiguous()
        vv = v.detach().contiguous()
        matrix.set_values(capi.F64, vals.data_ptr(), _stream())
        n = matrix.info().n_col
        x = torch.empty(n, dtype=torch.float64, device=v.device)
        matrix.pagerank_teleport(vv.data_ptr(), x.data_ptr(), beta, tol, max_iter, _stream(), accel=accel)
        ctx.matrix = matrix
        ctx.params = (beta, tol, max_iter, int(matrix.info().stored), accel)
        ctx.save_for_backward(vv, x)
        return x

    @staticmethod
    def backward(ctx, gx):
        vv, x = ctx.saved_tensors
        beta, tol, max_iter, nnz, accel = ctx.params
        gx = gx.contiguous()
        gvals = torch.empty(nnz, dtype=torch.float64, device=x.device) if ctx.needs_input_grad[0] else None
        gv = torch.empty_like(x) if ctx.needs_input_grad[1] else None
        # lambda is O(|dL/dx|) per entry: the L1 tolerance scales with n
        adj_tol = max(tol, 1e-15) * x.numel()
        ctx.matrix.pagerank_adjoint(vv.data_ptr(), x.data_ptr(), gx.data_ptr(),
                                    None if gvals is None else gvals.data_ptr(),
                                    None if gv is None else gv.data_ptr(), beta, adj_tol, max_iter, _stream(),
                                    accel=accel)
        return gvals, gv, None, None, None, None, None


def csr_spmv(matrix, values: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    return CsrSpMV.apply(values, x, matrix)


def pagerank(matrix, values: torch.Tensor, v: torch.Tensor, beta: float = 0.85, tol: float = 1e-14,
             max_iter: int = 10000, accel: int = 1) -> torch.Tensor:
    return PageRankTeleport.apply(values, v, matrix, beta, tol, max_iter, accel)
