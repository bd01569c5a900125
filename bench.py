"""Benchmark of the TBSLA SpMV / PageRank path on GB300 (one JSON line on stdout).

Headline (``value``): CSR FP64 SpMV y = A x on the cqmat matrix n = 2^24, c = 16,
q = 0.1, seed 0 (268,435,336 stored entries, 3.56 GB of algorithmic traffic per
product), in GB/s of algorithmic bytes over device time with the matrix and x
resident in HBM.  Every section runs with 32-byte L2 fetches
(tbsla_set_l2_fetch_granularity); the headline and the format sweep keep x
evict-last in a 64 MiB persisting L2 set-aside (tbsla_set_l2_persisting), the
other sections run with the context's set-aside (the values gradient and the
transposed product: both).  A "step" is one product, read from the handle's
ELL-layout copy when it keeps one (csr_sell_kernel; the CSR-array pair kernel
is timed beside it, ``csr_pair_kernel``).  ``e2e`` is the same metric through
the C ABI's host-vector call (tbsla_spmv_host) on pinned host vectors: x is
copied into HBM and the product writes y into host memory over NVLink-C2C,
both inside the timed region; the host link's copy rates for the same vectors,
timed in the run, give its floor (``transfer_floor_ms``).

Also reported (single-GPU runs): the format sweep of the same configuration
(CSR/ELL/COO/SCOO FP64 SpMV and a_axpx_, CSR FP32/BF16 stores, DENSE n = 32768,
cdiag n = 2^26), the 64-vector DENSE product on the tensor cores, PageRank on
the R-MAT graph 2^24 nodes / 2^28 edge draws, (a,b,c,d) = (0.57, 0.19, 0.19,
0.05), seed 1, damping 0.85, dangling mass redistributed, stopped at L1
residual 1e-10: time to tolerance in FP64 and with FP32 / BF16 stored values
plus FP64 refinement (plain or Anderson-accelerated), each result's L1 distance
to an FP64 solve at 1e-13 and to the oracle's, with the oracle's own times on
the host cores; batching (64 matrices in one launch, 256 personalized PageRank
vectors plain / accelerated / refined, k vectors through one matrix); and
differentiation (the adjoint PageRank against finite differences on 1000
edges of R-MAT 2^22, the backward of y = A x at 2^24).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the reference's CPU product (MatrixCSR::Ax, OpenMP
over rows, src/cpp/matrix/MatrixCSR.cpp:129-140) as restated in oracle/ on all
host cores (the reference's own sources are not on the GPU host).  Under
torchrun every rank runs an independent replica on its own GPU (the path has no
data exchange); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_HEADLINE = 1 << 24
C_HEADLINE = 16
Q_HEADLINE = 0.1
L2_FETCH_BYTES = 32  # L2 fetch granularity of the whole run (tbsla_set_l2_fetch_granularity)
L2_PERSIST_BYTES = 64 << 20  # persisting L2 set-aside of the headline (tbsla_set_l2_persisting)
# the headline and the format sweep load as much of x evict-last as the
# 67.8 MB set-aside holds, the same lines every product (range policy:
# TBSLA_TUNE_X_L2_KEEP with TBSLA_TUNE_X_L2_RANGE 1): the first 45 % of an
# FP64 x of 2^24 entries (60 MB), all of an FP32 one (64 MiB)
X_KEEP_HEADLINE = 0.45
X_RANGE_HEADLINE = 1
X_KEEP_FP32 = 1.0
# the headline's timed products rotate over this many x vectors of different
# content, so that no evict-last line of one product's x is the next one's
X_BUFFERS = 4
METRIC = "SpMV GB/s (% HBM peak); PageRank time-to-L1 1e-10, mixed vs FP64 GPU"
WORKLOAD = "cqmat CSR FP64 SpMV n=2^{log2n} c=16 q=0.1 seed=0"
# DRAM bytes (read + write) of one csr_sell_kernel launch on the 2^24
# workload with x rotated (the launch after one with another x), from the
# one-kernel, one-launch ncu capture summarised in
# profiles/csr_sell_kernel_cqmat_2p24.md
NCU_TRAFFIC_BYTES = 3_898_083_328


def csr_bytes(n_row, n_col, nnz, val_bytes=8, vec_bytes=8):
    """Algorithmic bytes of one CSR product: nnz*(value+index) + rowptr +
    x read once + y written once."""
    return nnz * (val_bytes + 4) + (n_row + 1) * 4 + n_col * vec_bytes + n_row * vec_bytes


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev, self.rows, self.proc, self.thread = device_index, [], None, None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None
        sm = [num(r[1]) for r in self.rows if num(r[1]) is not None]
        mx = [num(r[2]) for r in self.rows if num(r[2]) is not None]
        pw = [num(r[3]) for r in self.rows if num(r[3]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({nm for r in self.rows for k, nm in enumerate(names) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "reasons": reasons, "samples": len(self.rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v: float) -> float:
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_spmv_baseline(m, n_row, n_col, nnz, steps: int, threads: int):
    """The reference's CSR product restated in oracle/ (OpenMP over rows) on
    the full matrix m (an oracle matrix); returns (GB/s, seconds per
    product)."""
    x = np.random.default_rng(1).uniform(-1, 1, n_col)
    m.spmv(x, threads=threads)  # first touch
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        m.spmv(x, threads=threads)
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    return csr_bytes(n_row, n_col, nnz) / t / 1e9, t


def headline_config(log2n: int, nnz: int, world: int) -> dict:
    """The headline workload's config, the same for both arms."""
    n = 1 << log2n
    return {"workload": WORKLOAD.format(log2n=log2n), "n": n, "nnz": nnz, "format": "CSR",
            "algorithmic_bytes": csr_bytes(n, n, nnz), "parallelism": f"replicas{world}",
            "l2": f"inputs larger than L2: {csr_bytes(n, n, nnz) / 1e9:.2f} GB streamed per step, no flush needed",
            "x_buffers": X_BUFFERS,
            "l2_fetch_granularity_bytes": L2_FETCH_BYTES, "l2_persisting_bytes_requested": L2_PERSIST_BYTES,
            "x_evict_last": f"first {X_KEEP_HEADLINE:.0%} of x's addresses (range policy)"}


def run_reference(args, world, rank):
    """The reference's CPU product on the machine's host cores: the cqmat matrix
    built by the oracle's generators (bit-identical to the reference's
    fill_cqmat) and multiplied by the oracle's CSR loop; nothing of the
    product library is loaded."""
    if rank != 0:
        return
    from oracle.oracle import Oracle
    from oracle.oracle import build as obuild
    obuild(ref=False)
    threads = os.cpu_count() or 1
    n = 1 << args.log2n
    m = Oracle().fill_cqmat("CSR", n, n, C_HEADLINE, Q_HEADLINE, 0)
    nnz = int(m.h.s.n_values)
    gbs, t = cpu_spmv_baseline(m, n, n, nnz, max(args.steps, 1), threads)
    line = {"impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": headline_config(args.log2n, nnz, world),
            "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                             "sample": f"full matrix, median of {max(args.steps, 1)} products (oracle CSR loop, "
                                       f"OpenMP over rows; matrix from the oracle's fill_cqmat)"},
            "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_product(capi, A, store, vt, n_row, n_col, reps=10):
    """Device time of one product (CUDA events on the launching stream)."""
    import torch
    tdt = torch.float64 if vt == capi.F64 else torch.float32
    x = torch.rand(n_col, dtype=tdt, device="cuda")
    y = torch.empty(n_row, dtype=tdt, device="cuda")
    s = torch.cuda.current_stream()
    for _ in range(3):
        A.spmv_ex(store, vt, x.data_ptr(), vt, y.data_ptr(), 0, s.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        A.spmv_ex(store, vt, x.data_ptr(), vt, y.data_ptr(), 0, s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def time_axpx(capi, A, n, reps=10):
    """Device time of one a_axpx_ (r = A (A x + x), tbsla_a_axpx, FP64)."""
    import torch
    x = torch.rand(n, dtype=torch.float64, device="cuda")
    r = torch.empty(n, dtype=torch.float64, device="cuda")
    tmp = torch.empty(n, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    for _ in range(3):
        A.a_axpx(x.data_ptr(), r.data_ptr(), tmp.data_ptr(), 0, s.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        A.a_axpx(x.data_ptr(), r.data_ptr(), tmp.data_ptr(), 0, s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def format_sweep(capi, peak, log2n=24):
    """Every format / store of the configuration, device GB/s.  As the
    headline: a 64 MiB persisting L2 set-aside (restored after; every case
    starts with it cleared) holding the first addresses of x, as much as
    fits."""
    import torch
    L = capi.lib()
    sa0, sa_max = C.c_size_t(), C.c_size_t()
    capi.check(L.tbsla_get_l2_persisting(C.byref(sa0), C.byref(sa_max)))
    capi.check(L.tbsla_set_l2_persisting(min(L2_PERSIST_BYTES, sa_max.value)))
    sa_set = C.c_size_t()
    capi.check(L.tbsla_get_l2_persisting(C.byref(sa_set), None))
    out = {"l2": {"persisting_bytes": int(sa_set.value), "x_evict_last": f"first {X_KEEP_HEADLINE:.0%} of an FP64 x's addresses, all of an FP32 x"}}
    n = 1 << log2n
    nd = 32768 if log2n >= 24 else 8192  # DENSE order (small cases stay a few GB)
    cases = [("CSR_f64", "CSR", "cqmat", n, 16, 1, capi.F64, capi.F64),
             ("CSR_f32", "CSR", "cqmat", n, 16, 2, capi.F32, capi.F32),
             ("CSR_bf16", "CSR", "cqmat", n, 16, 4, capi.BF16, capi.F32),
             ("ELL_f64", "ELL", "cqmat", n, 16, 1, capi.F64, capi.F64),
             ("COO_f64", "COO", "cqmat", n, 16, 1, capi.F64, capi.F64),
             ("SCOO_f64", "SCOO", "cqmat", n, 16, 1, capi.F64, capi.F64),
             (f"DENSE_f64_{nd}", "DENSE", "cqmat", nd, 16, 1, capi.F64, capi.F64),
             (f"CSR_f64_cdiag_2^{log2n + 2}", "CSR", "cdiag", 4 * n, 1, 1, capi.F64, capi.F64)]
    for (key, fmt, gen, nn, c, stores, store, vt) in cases:
        # a cleared set-aside: no persisting lines of the previous case's x
        capi.check(L.tbsla_set_l2_persisting(min(L2_PERSIST_BYTES, sa_max.value)))
        if gen == "cdiag":  # built on the device (tbsla_generate_device), the host fill's arrays
            A = capi.DeviceMatrix.generate_device(fmt, gen, nn, nn, c, 0.0, 0, stores=stores)
        else:
            A = capi.DeviceMatrix.generate(fmt, gen, nn, nn, c, Q_HEADLINE, 0, stores=stores)
        A.tune(capi.TUNE_X_L2_KEEP, X_KEEP_HEADLINE if vt == capi.F64 else X_KEEP_FP32)
        A.tune(capi.TUNE_X_L2_RANGE, X_RANGE_HEADLINE)
        i = A.info()
        ms = time_product(capi, A, store, vt, i.n_row, i.n_col)
        vb = {capi.F64: 8, capi.F32: 4, capi.BF16: 2}[store]
        xb = 8 if vt == capi.F64 else 4
        if fmt == "CSR":
            algo = csr_bytes(i.n_row, i.n_col, i.stored, vb, xb)
        elif fmt == "ELL":
            algo = i.stored * (vb + 4) + 2 * nn * xb
        elif fmt in ("COO", "SCOO"):
            algo = i.stored * (vb + 8) + 2 * nn * xb
        else:
            algo = i.stored * vb + 2 * nn * xb
        gbs = algo / (ms * 1e-3) / 1e9
        out[key] = {"ms": round(ms, 4), "GB_s": round(gbs, 1), "frac_hbm": round(gbs / peak, 3),
                    "stored": int(i.stored), "gflops": round(2 * i.stored / (ms * 1e-3) / 1e9, 1)}
        if fmt in ("COO", "SCOO"):
            # the direct kernels read a derived row pointer, not the row array:
            # the bytes they move are the CSR product's
            read = csr_bytes(i.n_row, i.n_col, i.stored, vb, xb)
            out[key]["GB_s_of_bytes_read"] = round(read / (ms * 1e-3) / 1e9, 1)
            out[key]["frac_hbm_of_bytes_read"] = round(read / (ms * 1e-3) / 1e9 / peak, 3)
        if gen == "cqmat" and fmt in ("CSR", "ELL", "COO", "SCOO") and store == capi.F64:
            # a_axpx_ (Matrix.cpp:6-11): two products and the "+ x" (fused
            # into the first product's epilogue); bytes 2 x the matrix + 5 n-vectors
            ax_ms = time_axpx(capi, A, nn)
            ax = 2 * (algo - 2 * nn * xb) + 5 * nn * 8
            out[key]["a_axpx"] = {"ms": round(ax_ms, 4), "GB_s": round(ax / (ax_ms * 1e-3) / 1e9, 1),
                                  "frac_hbm": round(ax / (ax_ms * 1e-3) / 1e9 / peak, 3)}
        A.close()
        torch.cuda.empty_cache()
    out[f"DENSE_multi_vector_{nd}_k64"] = dense_multi(capi, nd, 64)
    capi.check(L.tbsla_set_l2_persisting(sa0.value))
    return out


def cfg1_bench(capi, peak):
    """The CPU-runnable configuration as stated: cqmat n = 100000, c = 10,
    q = 0.1, duplicates merged, values U(0,1] (generator cqmat_baseline,
    seed 0), x U[0,1): each format's product and a_axpx_ on the device (the
    14 MB matrix stays in L2: a latency case, not a roofline one) beside the
    oracle's products on the host cores."""
    import torch
    from oracle.oracle import Oracle, splitmix64_u01
    n = 100000
    threads = os.cpu_count() or 1
    out = {"workload": "cqmat_baseline n=100000 c=10 q=0.1 seed=0 (duplicates merged, values U(0,1])",
           "l2": "matrix and vectors L2-resident (14 MB)"}
    x = splitmix64_u01(0, 2, n)
    orc = Oracle()
    for fmt in ("CSR", "ELL", "COO", "SCOO"):
        A = capi.DeviceMatrix.generate(fmt, "cqmat_baseline", n, n, 10, 0.1, 0)
        i = A.info()
        ms = time_product(capi, A, capi.F64, capi.F64, n, n, reps=200)
        ax_ms = time_axpx(capi, A, n, reps=200)
        if fmt == "CSR":
            algo = csr_bytes(n, n, i.stored)
        elif fmt == "ELL":
            algo = i.stored * 12 + 2 * n * 8
        else:
            algo = i.stored * 16 + 2 * n * 8
        g = capi.generate(fmt, "cqmat_baseline", n, n, 10, 0.1, 0)
        om = orc.from_layout(fmt, g.geom, g.nnz, g.values, g.idx0, g.idx1)
        om.spmv(x, threads=threads)
        ts = []
        for _ in range(20):
            t0 = time.perf_counter()
            om.spmv(x, threads=threads)
            ts.append(time.perf_counter() - t0)
        cpu_ms = float(np.median(ts)) * 1e3
        # the drop-in's own call: host vectors in, host vector out
        A.spmv_host(x)
        t0 = time.perf_counter()
        for _ in range(50):
            A.spmv_host(x)
        host_ms = (time.perf_counter() - t0) / 50 * 1e3
        out[fmt] = {"stored": int(i.stored), "ms": round(ms, 4), "GB_s": round(algo / ms / 1e6, 1),
                    "a_axpx_ms": round(ax_ms, 4), "spmv_host_ms": round(host_ms, 4),
                    "cpu_ms": round(cpu_ms, 3),
                    "cpu_threads": threads if fmt in ("CSR", "ELL") else 1}
        A.close()
    torch.cuda.empty_cache()
    return out


def dense_multi(capi, n, k):
    """Y = A X for k vectors: the library's tensor-core kernel (tcgen05, TMA)
    for the BF16 and F32 (TF32) stores, cuBLAS DGEMM for F64; beside it the
    same BF16 GEMM through cuBLAS (torch.matmul) and the K-split sweep."""
    import torch
    peak, _ = peaks()
    A = capi.DeviceMatrix.generate("DENSE", "cqmat", n, n, 16, Q_HEADLINE, 0,
                                   stores=capi.STORE_F64 | capi.STORE_F32 | capi.STORE_BF16)
    res = {"n": n, "k": k}
    s = torch.cuda.current_stream().cuda_stream

    def timed(fn, reps=10):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = _events()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    for name, store, tdt, vb in (("f64", capi.F64, torch.float64, 8), ("f32_tf32", capi.F32, torch.float32, 4),
                                 ("bf16", capi.BF16, torch.float32, 2)):
        X = torch.rand((k, n), dtype=tdt, device="cuda")
        Y = torch.empty((k, n), dtype=tdt, device="cuda")
        ms = timed(lambda: A.dense_spmm(store, k, X.data_ptr(), n, Y.data_ptr(), n, s), 3 if vb == 8 else 10)
        algo = n * n * vb + 2 * n * k * (8 if vb == 8 else 4)
        res[name] = {"ms": round(ms, 4), "TFLOP_s": round(2.0 * n * n * k / ms / 1e9, 1),
                     "GB_s": round(algo / ms / 1e6, 1), "frac_hbm": round(algo / ms / 1e6 / peak, 3)}
        if store != capi.F64:
            sweep = {}
            for split in (1, 2, 4, 8, 16):
                A.tune(capi.TUNE_TC_SPLIT, split)
                sweep[str(split)] = round(timed(lambda: A.dense_spmm(store, k, X.data_ptr(), n, Y.data_ptr(), n, s)), 4)
            A.tune(capi.TUNE_TC_SPLIT, 0)
            res[name]["ms_by_k_split"] = sweep
        del X, Y
    res["device_status"] = A.device_status()
    A.close()
    torch.cuda.empty_cache()
    # the same BF16 GEMM through cuBLAS, for comparison
    Ab = torch.rand((n, n), device="cuda").to(torch.bfloat16)
    Xb = torch.rand((n, k), device="cuda").to(torch.bfloat16)
    ms = timed(lambda: torch.matmul(Ab, Xb))
    res["cublas_bf16_torch_matmul_ms"] = round(ms, 4)
    del Ab, Xb
    torch.cuda.empty_cache()
    return res


def pagerank_bench(capi, scale=24, cpu=True):
    """R-MAT 2^scale (16 draws per vertex) PageRank to L1 residual 1e-10:
    FP64 vs FP32/BF16 + FP64 refinement; the reference mode at 1e-9; with
    cpu, the oracle's solves on the host cores beside them."""
    import torch
    t0 = time.time()
    A = capi.DeviceMatrix.rmat_pagerank(scale, 16 << scale, 0.57, 0.19, 0.19, seed=1,
                                        stores=capi.STORE_F64 | capi.STORE_F32 | capi.STORE_BF16)
    setup = time.time() - t0
    info = A.info()
    n = info.n_row
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    ref = torch.empty(n, dtype=torch.float64, device="cuda")
    r = A.pagerank(ref.data_ptr(), tol=1e-13, max_iter=2000, precision=capi.F64)
    res = {"graph": f"R-MAT scale {scale}, 2^{scale + 4} draws, (0.57,0.19,0.19,0.05), seed 1", "n": n,
           "edges": int(info.stored), "setup_s": round(setup, 1), "tol": 1e-10,
           "reference_solve": {"tol": 1e-13, "sweeps": r.iterations, "converged": bool(r.converged)}}
    times, gpu_vectors = {}, {}
    for name, prec, acc in (("fp64", capi.F64, 0), ("fp32_refined", capi.F32, 0), ("bf16_refined", capi.BF16, 0),
                            ("fp64_anderson", capi.F64, 1), ("fp32_refined_anderson", capi.F32, 1),
                            ("bf16_refined_anderson", capi.BF16, 1)):
        A.pagerank(out.data_ptr(), tol=1e-10, max_iter=2000, precision=prec, accel=acc)  # warm: workspace + graphs
        torch.cuda.synchronize()
        ts = []
        for _ in range(3):
            t1 = time.perf_counter()
            r = A.pagerank(out.data_ptr(), tol=1e-10, max_iter=2000, precision=prec, accel=acc)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t1)
        err = float((out - ref).abs().sum().item())
        gpu_vectors[name] = out.cpu().numpy()
        times[name] = min(ts)
        res[name] = {"ms": round(min(ts) * 1e3, 2), "sweeps": r.iterations, "fp64_sweeps": r.iterations_f64,
                     "residual": r.residual, "converged": bool(r.converged), "l1_vs_fp64_1e-13": err}
    res["bf16_over_fp64_time"] = round(times["bf16_refined"] / times["fp64"], 3)
    res["anderson_over_fp64_time"] = round(times["fp64_anderson"] / times["fp64"], 3)
    res["fp32_over_fp64_time"] = round(times["fp32_refined"] / times["fp64"], 3)
    # the precision form with accelerated correction solves, against the plain
    # FP64 solve (the ratio the target names) and the accelerated FP64 one
    res["fp32_anderson_refined_over_fp64_time"] = round(times["fp32_refined_anderson"] / times["fp64"], 3)
    res["bf16_anderson_refined_over_fp64_time"] = round(times["bf16_refined_anderson"] / times["fp64"], 3)
    res["fp32_anderson_refined_over_fp64_anderson_time"] = round(times["fp32_refined_anderson"] /
                                                                  times["fp64_anderson"], 3)
    # Matrix::page_rank (reference mode: max-normalised, no dangling term) at
    # the reference's epsilon 1e-9 on the same graph
    A.pagerank(out.data_ptr(), beta=0.85, tol=1e-9, max_iter=1000, mode=capi.PR_REFERENCE)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    r = A.pagerank(out.data_ptr(), beta=0.85, tol=1e-9, max_iter=1000, mode=capi.PR_REFERENCE)
    torch.cuda.synchronize()
    res["reference_mode_1e-9"] = {"ms": round((time.perf_counter() - t1) * 1e3, 2), "iterations": r.iterations,
                                  "converged": bool(r.converged)}
    ref_mode_gpu = out.cpu().numpy()
    if cpu:
        res["cpu_baseline"] = pagerank_cpu_baseline(A, gpu_vectors, ref_mode_gpu, res)
    A.close()
    torch.cuda.empty_cache()
    return res


def pagerank_cpu_baseline(A, gpu_vectors, ref_mode_gpu, res):
    """The oracle's PageRank on the host cores, on the graph the GPU solved:
    the reference's page_rank (Matrix.cpp:13-61, epsilon 1e-9) and the
    dangling-mode restatement to L1 1e-10, timed; the dangling solve run on
    to 1e-13 is the anchor each GPU result is compared with (l1_vs_oracle)."""
    import math
    from oracle.oracle import Oracle
    threads = os.cpu_count() or 1
    orc = Oracle()
    rp, ci, va = A.csr_download()
    n = rp.size - 1
    dang = (np.bincount(ci, minlength=n) == 0).astype(np.uint8)
    out = {"cores": threads, "kind": "port"}
    t0 = time.perf_counter()
    xd, it_d, res_d = orc.page_rank_dangling(rp, ci, va, dang, 0.85, 1e-10, 5000, threads=threads)
    out["dangling_1e-10"] = {"s": round(time.perf_counter() - t0, 3), "sweeps": it_d, "residual": res_d}
    xo, it_o, res_o = orc.page_rank_dangling(rp, ci, va, dang, 0.85, 1e-13, 5000, threads=threads)
    xo = xo / math.fsum(xo)
    out["anchor"] = {"tol": 1e-13, "sweeps": it_o, "residual": res_o}
    for name, x in gpu_vectors.items():
        res[name]["l1_vs_oracle"] = float(np.abs(x - xo).sum())
    om = orc.from_arrays("CSR", n, n, va, rp, ci)
    del rp, ci, va
    t0 = time.perf_counter()
    b, it = om.page_rank(1e-9, 0.85, 1000, threads=threads)
    out["reference_mode_1e-9"] = {"s": round(time.perf_counter() - t0, 3), "iterations": it,
                                  "gpu_iterations_equal": it == res["reference_mode_1e-9"]["iterations"],
                                  "l1_gpu_vs_oracle": float(np.abs(ref_mode_gpu - b).sum())}
    out["gpu_speedup_dangling_fp64"] = round(out["dangling_1e-10"]["s"] * 1e3 / res["fp64"]["ms"], 1)
    out["gpu_speedup_reference_mode"] = round(out["reference_mode_1e-9"]["s"] * 1e3 /
                                              res["reference_mode_1e-9"]["ms"], 1)
    return out


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def batching_bench(capi, ppr_scale=22, ppr_vectors=256):
    """64 cqmat matrices (n log-uniform 1e3..1e6, c 8..32, q 0.1, FP32) in one
    launch vs 64 launches; 256 personalized PageRank vectors (|P| log-uniform
    1..100) on R-MAT 2^22 solved together vs one at a time."""
    import torch
    dev = torch.device("cuda")
    rng = np.random.default_rng(4)
    out = {}
    # ---- multi-matrix batch
    members, algo = [], 0
    for m in range(64):
        n = int(np.exp(rng.uniform(np.log(1e3), np.log(1e6))))
        c = int(rng.integers(8, 33))
        A = capi.DeviceMatrix.generate("CSR", "cqmat", n, n, c, 0.1, m + 1, stores=capi.STORE_F32)
        members.append(A)
        i = A.info()
        algo += i.stored * 8 + (i.rows + 1) * 4 + i.n_col * 4 + i.n_row * 4
    xs = [torch.rand(A.info().n_col, dtype=torch.float32, device=dev) for A in members]
    ys = [torch.empty(A.info().n_row, dtype=torch.float32, device=dev) for A in members]
    B = capi.Batch(members)
    B.bind(capi.F32, [x.data_ptr() for x in xs], [y.data_ptr() for y in ys])
    tuned = B.autotune()
    s = torch.cuda.current_stream()
    for _ in range(3):
        B.spmv(s.cuda_stream, graph=True)
    reps = 20
    e0, e1 = _events()
    e0.record(s)
    for _ in range(reps):
        B.spmv(s.cuda_stream, graph=True)
    e1.record(s)
    torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1) / reps
    e0.record(s)
    for _ in range(reps):
        for A, x, y in zip(members, xs, ys):
            A.spmv_ex(capi.F32, capi.F32, x.data_ptr(), capi.F32, y.data_ptr(), 0, s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    single_ms = e0.elapsed_time(e1) / reps
    out["multi_matrix"] = {
        "matrices": 64, "stored": int(sum(A.info().stored for A in members)), "dtype": "f32",
        "one_launch_ms": round(batch_ms, 4), "one_launch_GB_s": round(algo / batch_ms / 1e6, 1),
        "64_launches_ms": round(single_ms, 4), "speedup": round(single_ms / batch_ms, 2),
        "autotuned_blocks_per_sm": tuned.choice}
    B.close()
    del members, xs, ys
    torch.cuda.empty_cache()
    # ---- 256 personalized PageRank vectors
    G = capi.DeviceMatrix.rmat_pagerank(ppr_scale, 16 << ppr_scale, seed=1, stores=capi.STORE_F64 | capi.STORE_F32)
    n = G.info().n_row
    k = ppr_vectors
    sets = [rng.integers(0, n, int(np.exp(rng.uniform(0, np.log(100))))) for _ in range(k)]
    res = {"graph": f"R-MAT scale {ppr_scale}, 2^{ppr_scale + 4} draws, seed 1", "vectors": k, "tol": 1e-10}
    ref = torch.empty(k * n, dtype=torch.float64, device=dev)
    buf = torch.empty(k * n, dtype=torch.float64, device=dev)
    # plain and Anderson-accelerated solves; FP32 iterates alone (to 1e-6),
    # and FP32 sweeps with FP64 defect correction (tbsla_ppr_batched_refined)
    # to the FP64 tolerance; distances to the FP64 batched solve (itself at
    # 1e-10)
    for name, prec, tol, refined, accel in (("fp64", capi.F64, 1e-10, False, 0), ("fp32", capi.F32, 1e-6, False, 0),
                                            ("fp32_refined", capi.F32, 1e-10, True, 0),
                                            ("fp64_anderson", capi.F64, 1e-10, False, 1),
                                            ("fp32_refined_anderson", capi.F32, 1e-10, True, 1)):
        t = G.autotune_ppr(k, prec)
        out_buf = ref if name == "fp64" else buf
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        its, rs = capi.ppr_batched(G, sets, out_buf.data_ptr(), tol=tol, max_iter=1000, precision=prec,
                                   refined=refined, accel=accel)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        entry = {"tile": t.choice, "s": round(dt, 3), "ms_per_vector": round(dt * 1e3 / k, 3),
                 "sweeps_min_median_max": [int(its.min()), int(np.median(its)), int(its.max())],
                 "converged": int((rs < tol).sum())}
        if name != "fp64":
            entry["max_l1_vs_fp64"] = float((buf.view(k, n) - ref.view(k, n)).abs().sum(dim=1).max().item())
        res[name] = entry
    for name in ("fp32_refined", "fp64_anderson", "fp32_refined_anderson"):
        res[name + "_over_fp64_time"] = round(res[name]["s"] / res["fp64"]["s"], 3)
    del buf
    # one vector at a time (teleport form, same stopping rule)
    v = torch.zeros(n, dtype=torch.float64, device=dev)
    seeds = np.unique(sets[0])
    v[torch.from_numpy(seeds).to(dev)] = 1.0 / seeds.size
    x = torch.empty(n, dtype=torch.float64, device=dev)
    G.pagerank_teleport(v.data_ptr(), x.data_ptr(), 0.85, 1e-10, 1000)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = G.pagerank_teleport(v.data_ptr(), x.data_ptr(), 0.85, 1e-10, 1000)
    torch.cuda.synchronize()
    one = time.perf_counter() - t0
    res["one_vector_fp64"] = {"ms": round(one * 1e3, 3), "sweeps": r.iterations,
                              "l1_vs_batched": float((x - ref.view(k, n)[0]).abs().sum().item())}
    res["batched_speedup_per_vector_fp64"] = round(one * 1e3 / res["fp64"]["ms_per_vector"], 2)
    out["ppr_256"] = res
    G.close()
    torch.cuda.empty_cache()
    # ---- k vectors through one CSR matrix (tbsla_spmm) vs k products, cqmat 2^22
    N = 1 << 22
    A = capi.DeviceMatrix.generate("CSR", "cqmat", N, N, C_HEADLINE, Q_HEADLINE, 0,
                                   stores=capi.STORE_F64 | capi.STORE_F32)
    st = int(A.info().stored)
    s = torch.cuda.current_stream().cuda_stream
    sp = {}
    for store, tdt, vb in ((capi.F64, torch.float64, 8), (capi.F32, torch.float32, 4)):
        for k in (8, 32):
            X = torch.rand((N, k), dtype=tdt, device=dev)
            Y = torch.empty((N, k), dtype=tdt, device=dev)
            xs = [torch.rand(N, dtype=tdt, device=dev) for _ in range(k)]
            y1 = torch.empty(N, dtype=tdt, device=dev)

            def singles():
                for xv in xs:
                    A.spmv_ex(store, store, xv.data_ptr(), store, y1.data_ptr(), 0, s)
            A.spmm(store, k, X.data_ptr(), k, Y.data_ptr(), k, s)
            singles()
            e0, e1 = _events()
            e0.record()
            for _ in range(5):
                A.spmm(store, k, X.data_ptr(), k, Y.data_ptr(), k, s)
            e1.record()
            torch.cuda.synchronize()
            mm_ms = e0.elapsed_time(e1) / 5
            e0.record()
            for _ in range(5):
                singles()
            e1.record()
            torch.cuda.synchronize()
            single_ms = e0.elapsed_time(e1) / 5
            algo = st * (vb + 4) + (N + 1) * 4 + 2 * N * k * vb
            sp[f"{'f64' if store == capi.F64 else 'f32'}_k{k}"] = {
                "spmm_ms": round(mm_ms, 4), "spmm_GB_s": round(algo / mm_ms / 1e6, 1),
                "fma_per_s_T": round(st * k / mm_ms / 1e9, 3),
                "k_products_ms": round(single_ms, 4), "speedup": round(single_ms / mm_ms, 2)}
            del X, Y, xs
    out["csr_spmm_cqmat_2^22"] = sp
    A.close()
    torch.cuda.empty_cache()
    return out


FD_EDGES = 1000


def fd_check_edges(capi, G, v, w, gvals, n_edges, seed=7, sweeps=30):
    """Central fourth-order finite differences of L = w . x*(values) on
    n_edges random stored entries of G, each through the GPU forward solve
    (teleport form, Anderson-accelerated, a fixed `sweeps` sweeps with no
    stopping test, which reaches FP64 rounding: the same count for every
    perturbation keeps L a smooth function of the step), against the adjoint's
    gradient gvals.

    Perturbing one entry is a rank-one change of the fixed point's system, so
    L(t) = L0 + g t / (1 - c t) exactly, and the differences
    (8(L(h) - L(-h)) - (L(2h) - L(-2h))) / 12h equal g (1 - 4 c^4 h^4).  L
    carries about one unit in the last place of rounding (~2e-18 here), so a
    step of 3e-3 of the entry drowns the smallest gradients (2e-9: 4e-5
    relative); the step is that, raised where needed to make |g| h reach
    2e-10, at most a quarter of the entry.  Also reported: the rank-one
    estimate g = 2 / (h (1/(L(h) - L0) - 1/(L(-h) - L0))), exact for any
    step, from the same solves and one unperturbed solve.  Returns the
    relative errors' summary."""
    import torch
    dev = torch.device("cuda")
    _, _, vals = G.csr_download()
    base = torch.from_numpy(vals).to(dev)
    xx = torch.empty_like(v)
    rng = np.random.default_rng(seed)
    edges = rng.choice(vals.size, n_edges, replace=False)

    def loss():
        G.set_values(capi.F64, base.data_ptr())
        G.pagerank_teleport(v.data_ptr(), xx.data_ptr(), 0.85, 0.0, sweeps, accel=1)
        return float(torch.dot(w, xx).item())

    t0 = time.perf_counter()
    l0 = loss()
    rel, rel_rank1, steps = [], [], []
    for e in edges:
        e = int(e)
        a = vals[e]
        h = max(3e-3 * a, min(0.25 * a, 2e-10 / max(abs(gvals[e]), 1e-300)))
        steps.append(h / a)
        f = []
        for s_ in (1, -1, 2, -2):
            base[e] = a + s_ * h
            f.append(loss())
        base[e] = a
        fd = (8 * (f[0] - f[1]) - (f[2] - f[3])) / (12 * h)
        rel.append(abs(gvals[e] - fd) / max(abs(fd), 1e-300))
        r1 = 2.0 / (h * (1.0 / (f[0] - l0) - 1.0 / (f[1] - l0)))
        rel_rank1.append(abs(gvals[e] - r1) / max(abs(r1), 1e-300))
    G.set_values(capi.F64, base.data_ptr())
    rel, rel_rank1 = np.array(rel), np.array(rel_rank1)
    return {"edges": int(n_edges), "order": 4, "forward_sweeps": sweeps,
            "step_over_entry_min_median_max": [float(np.min(steps)), float(np.median(steps)), float(np.max(steps))],
            "rel_err_max": float(rel.max()), "rel_err_median": float(np.median(rel)),
            "edges_above_1e-6": int((rel > 1e-6).sum()),
            "rank_one_estimate_rel_err_max": float(rel_rank1.max()),
            "s": round(time.perf_counter() - t0, 1)}


def differentiation_bench(capi, scale=22):
    """Adjoint PageRank gradients on R-MAT 2^22 (w ~ N(0,1), seed 2) with a
    finite-difference check on 1000 random edges; backward of y = A x for
    cqmat 2^24 in FP32 (values gradient and transposed product)."""
    import torch
    dev = torch.device("cuda")
    out = {}
    G = capi.DeviceMatrix.rmat_pagerank(scale, 16 << scale, seed=1)
    info = G.info()
    n, nnz = info.n_row, int(info.stored)
    w = torch.from_numpy(np.random.default_rng(2).standard_normal(n)).to(dev)
    v = torch.full((n,), 1.0 / n, dtype=torch.float64, device=dev)
    x = torch.empty(n, dtype=torch.float64, device=dev)
    gvals = torch.empty(nnz, dtype=torch.float64, device=dev)
    gv = torch.empty(n, dtype=torch.float64, device=dev)
    G.pagerank_teleport(v.data_ptr(), x.data_ptr(), 0.85, 1e-15, 2000)
    G.pagerank_adjoint(v.data_ptr(), x.data_ptr(), w.data_ptr(), gvals.data_ptr(), gv.data_ptr(), 0.85, n * 1e-15,
                       2000)  # warm: transposed copy, buffers
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rf = G.pagerank_teleport(v.data_ptr(), x.data_ptr(), 0.85, 1e-15, 2000)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    ra = G.pagerank_adjoint(v.data_ptr(), x.data_ptr(), w.data_ptr(), gvals.data_ptr(), gv.data_ptr(), 0.85,
                            n * 1e-15, 2000)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    # the same two solves with Anderson acceleration
    xa = torch.empty_like(x)
    gvals_a, gv_a = torch.empty_like(gvals), torch.empty_like(gv)
    G.pagerank_teleport(v.data_ptr(), xa.data_ptr(), 0.85, 1e-15, 2000, accel=1)
    G.pagerank_adjoint(v.data_ptr(), xa.data_ptr(), w.data_ptr(), gvals_a.data_ptr(), gv_a.data_ptr(), 0.85,
                       n * 1e-15, 2000, accel=1)  # warm: graphs, ring buffers
    torch.cuda.synchronize()
    t3 = time.perf_counter()
    rfa = G.pagerank_teleport(v.data_ptr(), xa.data_ptr(), 0.85, 1e-15, 2000, accel=1)
    torch.cuda.synchronize()
    t4 = time.perf_counter()
    raa = G.pagerank_adjoint(v.data_ptr(), xa.data_ptr(), w.data_ptr(), gvals_a.data_ptr(), gv_a.data_ptr(), 0.85,
                             n * 1e-15, 2000, accel=1)
    torch.cuda.synchronize()
    t5 = time.perf_counter()
    accel_grad_diff = float((gvals_a - gvals).abs().max() / gvals.abs().max())
    # fourth-order differences of the GPU forward solve on 1000 random edges
    fd = fd_check_edges(capi, G, v, w, gvals.cpu().numpy(), FD_EDGES, seed=7)
    out["pagerank_adjoint"] = {
        "graph": f"R-MAT scale {scale}, 2^{scale + 4} draws, seed 1", "edges": nnz,
        "forward_ms": round((t1 - t0) * 1e3, 2), "forward_sweeps": rf.iterations,
        "adjoint_ms": round((t2 - t1) * 1e3, 2), "adjoint_sweeps": ra.iterations,
        "anderson": {"forward_ms": round((t4 - t3) * 1e3, 2), "forward_sweeps": rfa.iterations,
                     "adjoint_ms": round((t5 - t4) * 1e3, 2), "adjoint_sweeps": raa.iterations,
                     "values_gradient_max_rel_diff_to_plain": accel_grad_diff},
        "finite_differences": fd}
    G.close()
    torch.cuda.empty_cache()
    # backward of y = A x, cqmat 2^24, FP32; the values gradient and the
    # transposed product with the format sweep's L2 settings (64 MiB set-aside
    # holding all of the FP32 vector they gather; restored after), the
    # gradient also with the context's set-aside
    N = N_HEADLINE
    L = capi.lib()
    sa0, sa_max = C.c_size_t(), C.c_size_t()
    capi.check(L.tbsla_get_l2_persisting(C.byref(sa0), C.byref(sa_max)))
    A = capi.DeviceMatrix.generate("CSR", "cqmat", N, N, C_HEADLINE, Q_HEADLINE, 0,
                                   stores=capi.STORE_F64 | capi.STORE_F32)
    A.tune(capi.TUNE_X_L2_KEEP, X_KEEP_FP32)  # before the transposed copy is built: it inherits them
    A.tune(capi.TUNE_X_L2_RANGE, X_RANGE_HEADLINE)
    st = int(A.info().stored)
    gy = torch.rand(N, dtype=torch.float32, device=dev)
    xv = torch.rand(N, dtype=torch.float32, device=dev)
    gx = torch.empty(N, dtype=torch.float32, device=dev)
    gval = torch.empty(st, dtype=torch.float32, device=dev)
    t0 = time.perf_counter()
    A.spmv_transpose_ex(capi.F32, capi.F32, gy.data_ptr(), capi.F32, gx.data_ptr())
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    s = torch.cuda.current_stream().cuda_stream
    for _ in range(3):
        A.grad_values(capi.F32, gy.data_ptr(), xv.data_ptr(), 1.0, gval.data_ptr(), s)
        A.spmv_transpose_ex(capi.F32, capi.F32, gy.data_ptr(), capi.F32, gx.data_ptr(), s)
    reps = 10

    def grad_ms():
        for _ in range(3):
            A.grad_values(capi.F32, gy.data_ptr(), xv.data_ptr(), 1.0, gval.data_ptr(), s)
        e0, e1 = _events()
        e0.record()
        for _ in range(reps):
            A.grad_values(capi.F32, gy.data_ptr(), xv.data_ptr(), 1.0, gval.data_ptr(), s)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps
    gv_ctx_ms = grad_ms()  # the context's set-aside
    capi.check(L.tbsla_set_l2_persisting(min(L2_PERSIST_BYTES, sa_max.value)))
    gv_ms = grad_ms()  # 64 MiB set-aside, the gathered FP32 vector evict-last
    e0, e1 = _events()
    for _ in range(3):
        A.spmv_transpose_ex(capi.F32, capi.F32, gy.data_ptr(), capi.F32, gx.data_ptr(), s)
    e0.record()
    for _ in range(reps):
        A.spmv_transpose_ex(capi.F32, capi.F32, gy.data_ptr(), capi.F32, gx.data_ptr(), s)
    e1.record()
    torch.cuda.synchronize()
    tr_ms = e0.elapsed_time(e1) / reps
    gv_bytes = st * 8 + (N + 1) * 4 + 2 * N * 4   # colidx in, gradient out, dL/dy and x once
    tr_bytes = st * 8 + (N + 1) * 4 + 2 * N * 4
    out["spmv_backward_cqmat_2^24_f32"] = {
        "stored": st, "grad_values_ms": round(gv_ms, 4), "grad_values_GB_s": round(gv_bytes / gv_ms / 1e6, 1),
        "grad_values_context_setaside_ms": round(gv_ctx_ms, 4),
        "transpose_product_ms": round(tr_ms, 4), "transpose_product_GB_s": round(tr_bytes / tr_ms / 1e6, 1),
        "transpose_build_s": round(build_s, 2),
        "l2": "values gradient and transposed product: 64 MiB persisting set-aside, all of the gathered FP32 "
              "vector evict-last"}
    A.close()
    capi.check(L.tbsla_set_l2_persisting(sa0.value))
    torch.cuda.empty_cache()
    return out


def run_gb300(args, world, rank, local, pg):
    from tbsla_gb300 import build, capi
    build.build()
    L = capi.lib()
    capi.check(L.tbsla_set_device(local))
    import torch
    torch.cuda.set_device(local)

    n = 1 << args.log2n
    # every section runs with 32-byte L2 fetches: the random gathers of x
    # bring one sector, the kernels' streams ask for 256-byte prefetches
    capi.check(L.tbsla_set_l2_fetch_granularity(L2_FETCH_BYTES))
    # the headline (device and end-to-end products) keeps 45 % of x evict-last
    # in a 64 MiB persisting L2 set-aside; the context's set-aside is restored
    # after it (PageRank sweeps lose 2 % with the larger one)
    sa0, sa_max = C.c_size_t(), C.c_size_t()
    capi.check(L.tbsla_get_l2_persisting(C.byref(sa0), C.byref(sa_max)))
    capi.check(L.tbsla_set_l2_persisting(min(L2_PERSIST_BYTES, sa_max.value)))
    sa_set = C.c_size_t()
    capi.check(L.tbsla_get_l2_persisting(C.byref(sa_set), None))
    t0 = time.time()
    g = capi.generate("CSR", "cqmat", n, n, C_HEADLINE, Q_HEADLINE, 0)
    A = capi.DeviceMatrix.from_generated(g)
    A.tune(capi.TUNE_X_L2_KEEP, X_KEEP_HEADLINE)
    A.tune(capi.TUNE_X_L2_RANGE, X_RANGE_HEADLINE)
    setup_s = time.time() - t0
    nnz = int(g.values.size)
    algo = csr_bytes(n, n, nnz)
    kernels = A.info().kernels

    stream = torch.cuda.Stream()
    # X_BUFFERS vectors of different content, rotated product by product
    xs_dev = [torch.from_numpy(np.random.default_rng(1 + k).uniform(-1, 1, n)).cuda() for k in range(X_BUFFERS)]
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    sp = stream.cuda_stream
    with torch.cuda.stream(stream):
        for i in range(max(args.warmup, 3)):
            A.spmv(xs_dev[i % X_BUFFERS].data_ptr(), y.data_ptr(), 0, sp)
    torch.cuda.synchronize()

    def timed(rotate: bool):
        A.timing(True)
        A.timing_read()
        barrier(pg)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for i in range(args.steps):
                A.spmv(xs_dev[i % X_BUFFERS if rotate else 0].data_ptr(), y.data_ptr(), 0, sp)
            e1.record(stream)
        torch.cuda.synchronize()
        barrier(pg)
        ms = e0.elapsed_time(e1) / args.steps
        k_ms, k_n = A.timing_read()
        A.timing(False)
        return max_over_ranks(pg, ms), k_ms / max(k_n, 1)

    # the same x every product (reported beside the headline)
    same_step_ms, same_kern_ms = timed(False)
    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)
    step_ms, kern_avg_ms = timed(True)
    clocks = clk.stop()
    sliced = A.info().slices > 0
    # the kernel the rows take without the sliced copy (two lanes per row on
    # the CSR arrays), x rotated the same way, reported beside the headline
    A.tune(capi.TUNE_SHORT_ROWS, 2)
    _, pair_kern_ms = timed(True)
    A.tune(capi.TUNE_SHORT_ROWS, -1)

    # end to end through the C ABI with pinned host vectors
    hx, hy = C.c_void_p(), C.c_void_p()
    capi.check(L.tbsla_host_alloc(C.byref(hx), n * 8))
    capi.check(L.tbsla_host_alloc(C.byref(hy), n * 8))
    xs = np.ctypeslib.as_array(C.cast(hx, C.POINTER(C.c_double)), shape=(n,))
    xs[:] = np.random.default_rng(2).uniform(-1, 1, n)
    for _ in range(2):
        capi.check(L.tbsla_spmv_host(A.h, hx, n, hy, n, 0))
    barrier(pg)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        capi.check(L.tbsla_spmv_host(A.h, hx, n, hy, n, 0))
    e2e_s = max_over_ranks(pg, (time.perf_counter() - t0) / args.steps)
    # the host link's rates for the same vectors (copy engine, pinned host
    # memory): x in and y out can take no less than n*8/h2d + n*8/d2h
    hx_t = torch.empty(n, dtype=torch.float64, pin_memory=True)
    d_t = torch.empty(n, dtype=torch.float64, device="cuda")
    link = {}
    for name, (dst, src) in (("h2d", (d_t, hx_t)), ("d2h", (hx_t, d_t))):
        for _ in range(2):
            dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            dst.copy_(src, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        link[name] = e0.elapsed_time(e1) / 5
    del hx_t, d_t
    L.tbsla_host_free(hx)
    L.tbsla_host_free(hy)
    capi.check(L.tbsla_set_l2_persisting(sa0.value))
    A.close()
    del xs_dev
    torch.cuda.empty_cache()

    if rank != 0:
        return
    peak, peak_kind = peaks()
    value = world * algo / (step_ms * 1e-3) / 1e9
    achieved = algo / (kern_avg_ms * 1e-3) / 1e9
    threads = os.cpu_count() or 1
    from oracle.oracle import Oracle
    om = Oracle().from_layout("CSR", g.geom, g.nnz, g.values, g.idx0, g.idx1)
    del g
    cpu_gbs, cpu_t = cpu_spmv_baseline(om, n, n, nnz, 5, threads)
    del om
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(args.log2n, nnz, world),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": NCU_TRAFFIC_BYTES if args.log2n == 24 and sliced else None,
                     "kernel": "csr_sell_kernel" if sliced else "csr_pair_kernel",
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "kernel_ms": round(kern_avg_ms, 4), "l2_persisting_bytes_set": int(sa_set.value)},
        "same_x_every_step": {"value": round(world * algo / (same_step_ms * 1e-3) / 1e9, 2),
                              "kernel_GB_s": round(algo / (same_kern_ms * 1e-3) / 1e9, 2),
                              "frac": round(algo / (same_kern_ms * 1e-3) / 1e9 / peak, 4)},
        "csr_pair_kernel": {"kernel_ms": round(pair_kern_ms, 4),
                            "kernel_GB_s": round(algo / (pair_kern_ms * 1e-3) / 1e9, 2),
                            "frac": round(algo / (pair_kern_ms * 1e-3) / 1e9 / peak, 4)},
        "cpu_baseline": {"value": round(cpu_gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": "full matrix, median of 5 products (oracle CSR loop, OpenMP over rows)"},
        "e2e": {"value": round(algo / e2e_s / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": n * 8,
                "d2h_bytes_per_step": n * 8, "ms_per_step": round(e2e_s * 1e3, 3),
                "host_link_GB_s": {k: round(n * 8 / (v * 1e-3) / 1e9, 1) for k, v in link.items()},
                "transfer_floor_ms": round(link["h2d"] + link["d2h"], 3),
                "of_transfer_floor": round((link["h2d"] + link["d2h"]) / (e2e_s * 1e3), 3)},
        "gpu_launches": kernels * args.steps,
        "clocks": clocks,
        "setup_s": round(setup_s, 2),
    }
    if world == 1 and not args.headline_only:
        line["cfg1"] = cfg1_bench(capi, peak)
        line["formats"] = format_sweep(capi, peak)
        line["pagerank"] = pagerank_bench(capi)
        line["batching"] = batching_bench(capi)
        line["differentiation"] = differentiation_bench(capi)
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--headline-only", action="store_true", help="skip the format sweep and PageRank")
    ap.add_argument("--log2n", type=int, default=24, help="headline matrix size 2^log2n (profiling cases)")
    ap.add_argument("--pagerank-only", action="store_true", help="only the R-MAT PageRank timings (profiling)")
    ap.add_argument("--rmat-scale", type=int, default=24, help="R-MAT graph of 2^scale vertices (profiling cases)")
    ap.add_argument("--dense-k", type=int, default=64, help="vectors of the DENSE multi-vector section")
    ap.add_argument("--ppr-vectors", type=int, default=256, help="personalized PageRank vectors of the batching "
                    "section (profiling cases)")
    ap.add_argument("--section", choices=["pagerank", "batching", "differentiation", "formats", "cfg1", "dense"],
                    default=None,
                    help="only one section of the full report (profiling cases)")
    args = ap.parse_args()
    world, rank, local, pg = dist_setup()
    if args.pagerank_only or args.section:
        from tbsla_gb300 import build, capi
        build.build()
        capi.check(capi.lib().tbsla_set_l2_fetch_granularity(L2_FETCH_BYTES))
        if args.pagerank_only or args.section == "pagerank":
            print(json.dumps({"pagerank": pagerank_bench(capi, args.rmat_scale)}), flush=True)
        elif args.section == "batching":
            print(json.dumps({"batching": batching_bench(capi, args.rmat_scale if args.rmat_scale != 24 else 22,
                                                         args.ppr_vectors)}), flush=True)
        elif args.section == "dense":
            nd = 32768 if args.log2n >= 24 else 1 << (args.log2n - 9)
            print(json.dumps({"dense": dense_multi(capi, nd, args.dense_k)}), flush=True)
        elif args.section == "cfg1":
            print(json.dumps({"cfg1": cfg1_bench(capi, peaks()[0])}), flush=True)
        elif args.section == "formats":
            print(json.dumps({"formats": format_sweep(capi, peaks()[0], args.log2n)}), flush=True)
        elif args.section == "differentiation":
            print(json.dumps({"differentiation": differentiation_bench(capi)}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gb300(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
