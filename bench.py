#!/usr/bin/env python
"""Assembly throughput benchmark.

Workload: FP64 P2-tetrahedron anisotropic diffusion dot(mul(A, grad u),
grad v) on the 64^3 x 6 cube (1,572,864 tets, 2,146,689 DOFs, 60,859,905
nonzeros), interior vertices jittered by U(-0.2h, 0.2h)^3, per-element SPD
A = Q diag(exp(N(0, 0.5^2))) Q^T, 4-point quadrature (seeded synthetic data).

  value  assembled CSR nonzeros per second, inputs resident in HBM (both
         kernels of the fused affine path, CUDA events on the launching
         stream); inputs (~670 MB per step) exceed the 129 MB L2.
  e2e    same metric through the assembler's host-facing API: per step the
         coefficient A (3,3,E) goes host->device from page-locked memory and
         the CSR values come back device->host into the page-locked buffer
         that backs the returned scipy matrix.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU oracle (a restatement of the reference's
threaded C++ assembly) on the host cores, on a bounded sample of the same
workload.  Under torchrun each rank assembles its own replica (weak scaling;
the path has no exchange step).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "scikit-fem-native_gb300"))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

N_CELLS = 64
SEED = 2
METRIC = "assembled CSR nnz/s (FP64 P2-tet anisotropic diffusion)"
UNIT = "nnz/s"
CONFIG = {
    "workload": "P2-tet anisotropic diffusion, 64^3x6 jittered cube (1,572,864 tets), 4-point rule, FP64",
    "elements": 1572864, "dofs": 2146689, "nnz": 60859905, "quadrature_points": 4,
    "l2": "inputs larger than L2 (~670 MB touched per step vs 129 MB L2)",
}


def spd_tensors(E, rng):
    G = rng.standard_normal((E, 3, 3))
    Q, R = np.linalg.qr(G)
    Q = Q * np.sign(np.diagonal(R, axis1=1, axis2=2))[:, None, :]
    lam = np.exp(rng.normal(0.0, 0.5, size=(E, 3)))
    return np.einsum("eij,ej,ekj->eik", Q, lam, Q)


def jittered_cube(n, rng, mesh_tensor):
    p, t = mesh_tensor(*(np.linspace(0.0, 1.0, n + 1),) * 3)
    h = 1.0 / n
    inner = np.all((p > 1e-12) & (p < 1 - 1e-12), axis=0)
    p = p.copy()
    p[:, inner] += rng.uniform(-0.2 * h, 0.2 * h, size=(3, int(inner.sum())))
    return p, t


def rule4():
    a, b = 0.5854101966249685, 0.1381966011250105
    return np.array([[a, b, b, b], [b, a, b, b], [b, b, a, b]]), np.full(4, 1.0 / 24.0)


# ----------------------------------------------------------------- clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in getattr(self, "lines", []):
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- CPU side

class OracleSample:
    """The workload at n^3 x 6 on the CPU oracle (threaded colored assembly,
    the reference's multi-thread scheme); set up once, one assembly per step."""

    def __init__(self, n, threads):
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O

        self.O = O
        self.threads = threads
        rng = np.random.default_rng(np.random.SeedSequence(SEED))
        p, t = jittered_cube(n, rng, O.mesh_tet_tensor)
        p2, t2 = O.mesh_tet2_from_mesh(p, t)
        X, W = rule4()
        self.basis = O.make_basis(p2, t2, True, quadrature=(X, W), threads=threads)
        E, Q = self.basis.dx.shape
        A = spd_tensors(E, rng)
        self.T = O.anisotropic_tensor(np.broadcast_to(np.moveaxis(A, (1, 2), (0, 1))[..., None], (3, 3, E, Q)),
                                      (E, Q))
        dofs = self.basis.dofs3.reshape(E, -1)
        self.pattern = O.Pattern(dofs, dofs)
        self.nnz, self.E = self.pattern.nnz, E
        self.desc = (f"P2 anisotropic {n}^3x6 jittered cube ({E} tets, nnz {self.nnz}), "
                     f"threaded colored assembly on {threads} threads")

    def step(self):
        t0 = time.perf_counter()
        self.O.cross_gradient_tensor_assemble(self.basis, self.T, threads=self.threads, pattern=self.pattern)
        return time.perf_counter() - t0


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


REFERENCE_SAMPLE_CELLS = 32


def run_reference(args, rank):
    if rank != 0:
        return
    threads = host_threads()
    sample = OracleSample(REFERENCE_SAMPLE_CELLS, threads)
    for _ in range(args.warmup):
        sample.step()
    times = [sample.step() for _ in range(args.steps)]
    elapsed = sum(times)
    value = sample.nnz * args.steps / elapsed
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(CONFIG, sample=sample.desc),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample.desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU side

def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per launch of the row pass from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "k_affine_rows_p2_aniso_64.txt")
    try:
        for ln in open(path):
            if ln.startswith("dram_bytes_per_launch_full:"):
                return float(ln.split(":")[1])
    except OSError:
        pass
    return None


def run_gpu(args, rank, world):
    import torch

    import skfemntv_gb300 as sk
    from skfemntv_gb300 import _device as dev
    from skfemntv_gb300._native import call
    from skfemntv_gb300.assembly import NativeTensorForm
    import ctypes

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rng = np.random.default_rng(np.random.SeedSequence(SEED))
    p, t = jittered_cube(N_CELLS, rng, lambda *a: (lambda m: (m.p, m.t))(sk.MeshTet.init_tensor(*a)))
    m2 = sk.MeshTet2.from_mesh(sk.MeshTet(p, t))
    X, W = rule4()
    basis = sk.Basis(m2, sk.ElementVector(sk.ElementTetP2(), dim=1), quadrature=(X, W))
    E, Q = basis._coefficient_shape
    A = spd_tensors(E, rng)
    A_cf = np.ascontiguousarray(np.moveaxis(A, (1, 2), (0, 1)))  # (3,3,E) public component-first
    A_pub = np.broadcast_to(A_cf[..., None], (3, 3, E, Q))      # public layout, broadcast over points
    form = NativeTensorForm(basis)
    nnz = form.pattern.nnz
    dA = dev.to_device(A_cf, np.float64)
    prec = {"fp64": 0, "split_fp32": 1, "fp64_emulated": 2}
    stream = torch.cuda.current_stream()

    def step_device(mode):
        form.assemble_device(None, precision=mode, tensor_device=dA, tensor_kind=2)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if world > 1:
            tt = torch.tensor([x], device="cuda")
            torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
            return float(tt.item())
        return x

    def time_mode(mode):
        for _ in range(max(3, args.warmup)):
            step_device(mode)
        barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(torch.cuda.current_device()) as clocks:
            barrier()
            ev0.record(stream)
            for _ in range(args.steps):
                step_device(mode)
            ev1.record(stream)
            barrier()
        ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps)
        kms = (ctypes.c_float * 2)()
        k_el, k_rows = [], []
        for _ in range(args.steps):
            call("skg_h1_assemble_affine_profiled", form.pattern.h, dev.ptr(m2._dev("p")), m2.p.shape[1],
                 dev.ptr(m2._dev("t")), 10, E, dev.ptr(basis._dev_dofs()), Q, dev.hptr(basis.X), dev.hptr(basis.W),
                 2, dev.ptr(dA), prec[mode], dev.ptr(form.target.d_values), kms, dev.stream_ptr())
            k_el.append(kms[0])
            k_rows.append(kms[1])
        return ms, statistics.mean(k_el), statistics.mean(k_rows), clocks.summary()

    results = {}
    reference_values = None
    for mode in ("fp64", "fp64_emulated", "split_fp32"):
        ms, t_el, t_rows, clk = time_mode(mode)
        vals = form.target.d_values[:nnz].clone()
        if reference_values is None:
            reference_values = vals
            err = 0.0
        else:
            err = float((vals - reference_values).abs().max() / reference_values.abs().max())
        results[mode] = {"value": world * nnz / (ms * 1e-3), "ms_per_step": ms,
                         "kernel_ms": {"element_pass": t_el, "row_pass": t_rows},
                         "max_rel_err_vs_fp64": err, "clocks": clk}
    head = results["fp64"]
    ms, t_el, t_rows = head["ms_per_step"], head["kernel_ms"]["element_pass"], head["kernel_ms"]["row_pass"]
    value = head["value"]

    # ---- e2e (native FP64): host (page-locked) A in, host CSR values out, through the assembler API
    for _ in range(2):
        form.assemble_device(A_pub)
        form.target.download()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        form.assemble_device(A_pub)
        form.target.download()
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    e2e_value = world * nnz / e2e_s

    # ---- roofline of the dominant kernel (headline mode)
    peak, peak_kind = measured_peak()
    npts_vertex = (N_CELLS + 1) ** 3
    bytes_elem = 24 * npts_vertex + 16 * E + 72 * E     # vertex coords + 4 vertex ids + A
    bytes_rows = 40 * E + 8 * nnz                       # 10 dof ids per element + CSR values
    dominant = ("k_rows_group", bytes_rows, t_rows) if t_rows >= t_el else ("k_elem_fp64", bytes_elem, t_el)
    achieved = dominant[1] / (dominant[2] * 1e-3) / 1e9
    traffic = profiled_traffic() if dominant[0] == "k_rows_group" else None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered cube, seeded SPD tensors)",
        "config": dict(CONFIG, parallelism=f"replicas x{world}" if world > 1 else "single GPU"),
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(A_cf.nbytes),
                "d2h_bytes_per_step": int(8 * nnz), "ms_per_step": 1e3 * e2e_s},
        "roofline": {"bound": "hbm", "kernel": dominant[0], "achieved": achieved, "peak": peak,
                     "peak_kind": f"{peak_kind} hbm_gbs", "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algorithmic_bytes_per_launch": dominant[1],
                     "whole_assembly_hbm_frac": (bytes_elem + bytes_rows) / ((t_el + t_rows) * 1e-3) / 1e9 / peak},
        "precision_variants": results,
        "gpu_launches": 2 * args.steps,
        "clocks": head["clocks"],
    }
    if rank == 0 and not args.no_cpu_baseline:
        sample = OracleSample(REFERENCE_SAMPLE_CELLS, host_threads())
        sample.step()
        times = [sample.step() for _ in range(3)]
        line["cpu_baseline"] = {
            "value": sample.nnz * len(times) / sum(times), "unit": UNIT, "cores": sample.threads, "kind": "port",
            "sample": sample.desc + ", 3 timed assemblies",
        }
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        torch.distributed.init_process_group("nccl")
    try:
        run_gpu(args, rank, world)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
