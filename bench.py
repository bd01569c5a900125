"""Benchmark of the TBSLA SpMV path on GB300 (one JSON line on stdout).

Headline workload: CSR FP64 SpMV y = A x on the cqmat matrix n = 2^24,
c = 16, q = 0.1, seed 0 (268,435,336 stored entries, 3.56 GB of
algorithmic traffic per product).  A "step" is one product over the resident
matrix.  ``value`` is achieved GB/s (algorithmic bytes / device time, inputs
resident in HBM); ``e2e`` is the same metric through the C ABI's host-vector
call (tbsla_spmv_host: pinned x in, y out, copies inside the timed region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

``--impl reference`` times the reference's CPU path (MatrixCSR::Ax with
OpenMP over rows, src/cpp/matrix/MatrixCSR.cpp:129-140) as restated in
oracle/ (the reference's sources are not on the GPU host) on all host cores.
Under torchrun each rank runs an independent replica on its own GPU
(the path has no data exchange); rank 0 prints the line.
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
METRIC = "SpMV GB/s (% HBM peak)"
# DRAM bytes per launch of csr_merge_kernel on this workload from the ncu
# capture summarised in profiles/csr_merge_kernel_cqmat_2p24.md (None until
# captured)
NCU_TRAFFIC_BYTES = None


def csr_bytes(n_row, n_col, nnz, val_bytes=8, vec_bytes=8):
    """Algorithmic bytes of one CSR product: nnz*(value+index) + rowptr +
    x read once + y written once."""
    return nnz * (val_bytes + 4) + (n_row + 1) * 4 + n_col * vec_bytes + n_row * vec_bytes


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.rows = []
        self.proc = None
        self.thread = None

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
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


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


def cpu_spmv_baseline(g, steps: int, threads: int):
    """The reference's CSR product restated in oracle/ (OpenMP over rows) on
    the full matrix; returns (GB/s, seconds per product)."""
    from oracle.oracle import Oracle
    orc = Oracle()
    m = orc.from_layout("CSR", g.geom, g.nnz, g.values, g.idx0, g.idx1)
    x = np.random.default_rng(1).uniform(-1, 1, g.n_col)
    m.spmv(x, threads=threads)  # first touch
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        m.spmv(x, threads=threads)
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    return csr_bytes(g.n_row, g.n_col, g.values.size) / t / 1e9, t


def run_reference(args, world, rank, pg):
    if rank != 0:
        return
    from tbsla_gb300 import build, capi
    build.build()
    from oracle.oracle import build as obuild
    obuild(ref=False)
    threads = os.cpu_count() or 1
    t0 = time.time()
    g = capi.generate("CSR", "cqmat", N_HEADLINE, N_HEADLINE, C_HEADLINE, Q_HEADLINE, 0)
    gen_s = time.time() - t0
    for _ in range(args.warmup):
        pass
    gbs, t = cpu_spmv_baseline(g, max(args.steps, 1), threads)
    line = {"impl": "reference", "metric": METRIC, "value": round(gbs, 3), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "cqmat CSR FP64 SpMV n=2^24 c=16 q=0.1 seed=0", "n": N_HEADLINE,
                       "nnz": int(g.values.size), "format": "CSR"},
            "cpu_baseline": {"value": round(gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                             "sample": f"full matrix, median of {max(args.steps, 1)} products"},
            "e2e": {"value": round(gbs, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "setup_s": round(gen_s, 2)}
    print(json.dumps(line), flush=True)


def run_gb300(args, world, rank, local, pg):
    from tbsla_gb300 import build, capi
    build.build()
    L = capi.lib()
    capi.check(L.tbsla_set_device(local))

    n = N_HEADLINE
    t0 = time.time()
    g = capi.generate("CSR", "cqmat", n, n, C_HEADLINE, Q_HEADLINE, 0)
    A = capi.DeviceMatrix.from_generated(g)
    setup_s = time.time() - t0
    nnz = int(g.values.size)
    algo = csr_bytes(n, n, nnz)

    # device vectors and a stream of our own (events are recorded on it)
    import torch
    torch.cuda.set_device(local)
    stream = torch.cuda.Stream()
    x = torch.from_numpy(np.random.default_rng(1).uniform(-1, 1, n)).cuda()
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    sp = stream.cuda_stream
    launches_per_step = 2  # csr_merge_kernel + merge_fixup_kernel

    with torch.cuda.stream(stream):
        for _ in range(max(args.warmup, 3)):
            A.spmv(x.data_ptr(), y.data_ptr(), 0, sp)
    torch.cuda.synchronize()
    A.timing(True)
    A.timing_read()

    clk = ClockSampler(local)
    clk.start()
    time.sleep(0.3)
    barrier(pg)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        for _ in range(args.steps):
            A.spmv(x.data_ptr(), y.data_ptr(), 0, sp)
        e1.record(stream)
    torch.cuda.synchronize()
    barrier(pg)
    step_ms = e0.elapsed_time(e1) / args.steps
    kern_ms, kern_n = A.timing_read()
    A.timing(False)
    clocks = clk.stop()
    step_ms = max_over_ranks(pg, step_ms)
    kern_avg_ms = kern_ms / max(kern_n, 1)

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
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = max_over_ranks(pg, e2e_s)
    L.tbsla_host_free(hx)
    L.tbsla_host_free(hy)

    if rank != 0:
        return
    peak, peak_kind = peaks()
    value = world * algo / (step_ms * 1e-3) / 1e9
    achieved = algo / (kern_avg_ms * 1e-3) / 1e9
    threads = os.cpu_count() or 1
    cpu_gbs, cpu_t = cpu_spmv_baseline(g, 5, threads)
    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "cqmat CSR FP64 SpMV n=2^24 c=16 q=0.1 seed=0", "n": n, "nnz": nnz,
                   "format": "CSR", "algorithmic_bytes": algo, "parallelism": f"replicas{world}",
                   "l2": "inputs larger than L2 (3.56 GB streamed per step)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": NCU_TRAFFIC_BYTES,
                     "kernel": "csr_merge_kernel", "peak_source": peak_kind,
                     "kernel_ms": round(kern_avg_ms, 4)},
        "hbm_frac_of_measured": round(value / peak, 4),
        "cpu_baseline": {"value": round(cpu_gbs, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": "full matrix, median of 5 products (oracle CSR loop, OpenMP over rows)"},
        "e2e": {"value": round(algo / e2e_s / 1e9, 3), "unit": "GB/s", "h2d_bytes_per_step": n * 8,
                "d2h_bytes_per_step": n * 8, "ms_per_step": round(e2e_s * 1e3, 3)},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "setup_s": round(setup_s, 2),
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    args = ap.parse_args()
    world, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank, pg)
    else:
        run_gb300(args, world, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
