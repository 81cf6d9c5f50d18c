#!/usr/bin/env python
"""Assembly throughput benchmark.

Workload: FP64 P2-tetrahedron anisotropic diffusion dot(mul(A, grad u),
grad v) on the 64^3 x 6 cube (1,572,864 tets, 2,146,689 DOFs, 60,859,905
nonzeros), interior vertices jittered by U(-0.2h, 0.2h)^3, per-element SPD
A = Q diag(exp(N(0, 0.5^2))) Q^T, 4-point quadrature (seeded synthetic data).

  value  assembled CSR nonzeros per second, inputs resident in HBM (both
         kernels of the fused affine path, CUDA events on the launching
         stream); inputs (~670 MB per step) exceed the 129 MB L2.
  e2e    same metric through the assembler's host-facing API
         (NativeTensorForm.assemble): per step the coefficient A (3,3,E) is
         read from host memory (by the element kernel over NVLink-C2C on
         Grace-Blackwell) and the CSR values land in the page-locked buffer
         behind the returned scipy matrix, copied in row chunks while the
         row pass runs.

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
        self.samples = []

    def _reader(self):
        for ln in self.proc.stdout:
            if ln.strip():
                self.samples.append((time.perf_counter(), ln))

    def __enter__(self):
        """Starts sampling every 50 ms and returns once the first sample is in,
        so that the sampler is live when the timed region starts."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return self
        self.thread = threading.Thread(target=self._reader, daemon=True)
        self.thread.start()
        t_end = time.perf_counter() + 5.0
        while not self.samples and time.perf_counter() < t_end and self.proc.poll() is None:
            time.sleep(0.01)
        self.t_start = time.perf_counter()
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            # a timed region shorter than the sampling period: keep the sampler
            # until one sample from after its start is in (at most 0.5 s)
            t_end = time.perf_counter() + 0.5
            while (not any(t >= self.t_start for t, _ in self.samples) and time.perf_counter() < t_end
                   and self.proc.poll() is None):
                time.sleep(0.005)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.proc.wait()
            self.thread.join(timeout=5)
            self.lines = [ln for t, ln in self.samples if t >= self.t_start]

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
    """The workload at n^3 x 6 on the CPU oracle (the reference's assembly
    algorithm: per-point contributions summed into the CSR slots, threaded by
    element coloring as bilinear_form_assembler.cpp:62-70 does); set up once,
    one assembly per step."""

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
        self.nnz, self.E, self.n = self.pattern.nnz, E, n
        self.values = None

    def desc(self, threads):
        return (f"P2 anisotropic {self.n}^3x6 jittered cube ({self.E} tets, nnz {self.nnz}), "
                f"colored assembly on {threads} thread{'s' if threads > 1 else ''}")

    def step(self, threads=None):
        t0 = time.perf_counter()
        self.values, _, _ = self.O.cross_gradient_tensor_assemble(self.basis, self.T, threads=threads or self.threads,
                                                                  pattern=self.pattern)
        return time.perf_counter() - t0


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_baseline_of(sample, reps):
    """All host cores over `reps` timed assemblies (after one warm-up), and one
    timed single-thread assembly (the reference's default thread count,
    cpp/src/runtime.cpp:10)."""
    sample.step()
    times = [sample.step() for _ in range(reps)]
    t_one = sample.step(threads=1)
    return {"value": sample.nnz * len(times) / sum(times), "unit": UNIT, "cores": sample.threads, "kind": "port",
            "sample": sample.desc(sample.threads) + f", {reps} timed assemblies",
            "same_config": sample.n == N_CELLS,
            "one_thread": {"value": sample.nnz / t_one, "unit": UNIT, "cores": 1, "seconds": t_one,
                           "sample": sample.desc(1) + ", 1 timed assembly"}}


def run_reference(args, rank):
    if rank != 0:
        return
    threads = host_threads()
    if args.workload != "p2_aniso":
        cb = aux_cpu_baseline(args.workload, threads, reps=max(1, args.steps))
        line = {"impl": "reference", "metric": AUX_METRIC[args.workload], "value": cb["value"], "unit": cb["unit"],
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": args.workload, "sample": cb["sample"]}, "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    # the full workload (same mesh, tensors and rule as the GPU arm), every
    # step one complete assembly on all host cores
    sample = OracleSample(args.cells, threads)
    for _ in range(args.warmup):
        sample.step()
    times = [sample.step() for _ in range(args.steps)]
    t_one = sample.step(threads=1)
    elapsed = sum(times)
    value = sample.nnz * args.steps / elapsed
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(CONFIG, sample=sample.desc(threads), cells=args.cells),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample.desc(threads) + f", {args.steps} timed assemblies",
                         "same_config": args.cells == N_CELLS,
                         "one_thread": {"value": sample.nnz / t_one, "unit": UNIT, "cores": 1, "seconds": t_one,
                                        "sample": sample.desc(1) + ", 1 timed assembly"}},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- GPU side

def reduce_max(x, world, device="cuda"):
    """Largest value over the ranks (the slowest rank's time); identity for one rank."""
    if world <= 1:
        return x
    import torch

    tt = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# Counters behind the FP64 roofline, kept as data (measured, not recomputed
# here): FP64 thread instructions (DFMA + DMUL + DADD, ncu
# smsp__sass_thread_inst_executed_op_{dfma,dmul,dadd}_pred_on.sum of one
# launch divided by the elements) and DRAM bytes (dram__bytes_read.sum +
# dram__bytes_write.sum of one launch at 48^3, scaled to 64^3 by the element
# count) of each FP64 pass of the headline workload.
FP64_PROFILE = {
    "source": "ncu --metrics ... --clock-control none on python bench.py --cells 32 (instructions) / --cells 48 "
              "(DRAM) --steps 2 --warmup 3 --no-cpu-baseline --modes fp64, GB300",
    "commit": "a327ee2",
    "ops_per_element": {"k_elem_ke_fp64_exact": 163.0, "k_rows_ke": 95.3},
    "dram_bytes_64": {"k_elem_ke_fp64_exact": 1262200000.0, "k_rows_ke": 2229800000.0},
}
# The plain neo-Hookean call: element matrices k_nh_ke + row pass k_rows_ke<12>.
NH_FP64_OPS_PER_ELEMENT = 535.1 + 180.0


def fp64_roof(call, passes, elements):
    """FP64 pipe roof of the FP64 passes: the device's FMA rate measured now
    (skg_fp64_fma_rate) against each pass's FP64 instructions per second."""
    import ctypes

    rate = ctypes.c_double()
    call("skg_fp64_fma_rate", ctypes.byref(rate), None)
    out = {"peak_gops": rate.value, "peak_source": "skg_fp64_fma_rate: independent FMA chains, measured in this run",
           "counts": {k: FP64_PROFILE[k] for k in ("source", "commit")}, "passes": {}}
    for name, _, _, ms in passes:
        ops = FP64_PROFILE["ops_per_element"].get(name)
        if ops is None or ms <= 0:
            continue
        achieved = ops * elements / (ms * 1e-3) / 1e9
        out["passes"][name] = {"ops_per_element": ops, "achieved_gops": achieved, "frac": achieved / rate.value}
    return out


def oracle_errors(sample, mode_values):
    """Largest error of each precision mode's values relative to the largest
    oracle entry, on the full workload (the oracle assembled it last)."""
    ref = sample.values
    scale = float(np.max(np.abs(ref)))
    return {m: float(np.max(np.abs(v - ref)) / scale) for m, v in mode_values.items()}


def run_gpu(args, rank, world):
    import torch

    import skfemntv_gb300 as sk
    from skfemntv_gb300 import _device as dev
    from skfemntv_gb300._native import call
    from skfemntv_gb300.assembly import NativeTensorForm
    import ctypes

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rng = np.random.default_rng(np.random.SeedSequence(SEED))
    p, t = jittered_cube(args.cells, rng, lambda *a: (lambda m: (m.p, m.t))(sk.MeshTet.init_tensor(*a)))
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
        return reduce_max(x, world)

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
                 dev.ptr(m2._dev("t")), 10, E, Q, dev.hptr(basis.X), dev.hptr(basis.W),
                 2, dev.ptr(dA), prec[mode], dev.ptr(form.target.d_values), kms, dev.stream_ptr())
            k_el.append(kms[0])
            k_rows.append(kms[1])
        return ms, statistics.mean(k_el), statistics.mean(k_rows), clocks.summary()

    results = {}
    reference_values = None
    mode_values = {}  # host copies for the comparison with the oracle
    for mode in args.modes:
        ms, t_el, t_rows, clk = time_mode(mode)
        vals = form.target.d_values[:nnz].clone()
        mode_values[mode] = vals.cpu().numpy()
        if reference_values is None:
            reference_values = vals
            err = 0.0
        else:
            err = float((vals - reference_values).abs().max() / reference_values.abs().max())
        results[mode] = {"value": world * nnz / (ms * 1e-3), "ms_per_step": ms,
                         "kernel_ms": {"element_pass": t_el, "row_pass": t_rows},
                         "max_rel_err_vs_fp64": err, "clocks": clk}
    head = results[args.modes[0]]
    ms, t_el, t_rows = head["ms_per_step"], head["kernel_ms"]["element_pass"], head["kernel_ms"]["row_pass"]
    value = head["value"]

    # ---- e2e (native FP64) through the assembler's host API: A from host memory in,
    # the CSR values out into the host matrix (chunked copies overlapping the row pass)
    for _ in range(2):
        form.assemble(A_pub, copy=False)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        form.assemble(A_pub, copy=False)
    barrier()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / args.steps)
    e2e_value = world * nnz / e2e_s

    # ---- roofline of the dominant kernel (headline mode)
    peak, peak_kind = measured_peak()
    npts_vertex = (args.cells + 1) ** 3
    # compulsory bytes, each counted once: vertex coordinates, 10 int32 DOF
    # ids per element (4 vertex ids read by the element pass, 6 edge ids
    # charged to the row pass), A (9 float64 per element), the CSR values
    bytes_elem = 24 * npts_vertex + 16 * E + 72 * E
    bytes_rows = 24 * E + 8 * nnz
    head_mode = args.modes[0]
    # the workload's 4-point rule integrates quadratics exactly: the integer-factor element kernel runs
    names = {"fp64": ("k_elem_ke_fp64_exact", "k_rows_ke"), "fp64_emulated": ("k_elem_ke_df64_packed", "k_rows_ke_df"),
             "split_fp32": ("k_elem_ke_split", "k_rows_ke_f32")}[head_mode]
    passes = [q for q in [(names[0], "element", bytes_elem, t_el), (names[1], "row", bytes_rows, t_rows)] if q[3] > 0]
    dominant = max(passes, key=lambda q: q[3])
    achieved = dominant[2] / (dominant[3] * 1e-3) / 1e9
    traffic = (FP64_PROFILE["dram_bytes_64"].get(dominant[0])
               if head_mode == "fp64" and args.cells == N_CELLS else None)

    config = dict(CONFIG, cells=args.cells, parallelism=f"replicas x{world}" if world > 1 else "single GPU")
    if args.cells != N_CELLS:
        config.update(workload=f"P2-tet anisotropic diffusion, {args.cells}^3x6 jittered cube (profiling size)",
                      elements=E, dofs=basis.N, nnz=nnz)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered cube, seeded SPD tensors)",
        "config": config,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(A_cf.nbytes),
                "d2h_bytes_per_step": int(8 * nnz), "ms_per_step": 1e3 * e2e_s},
        "roofline": {"bound": "hbm", "kernel": dominant[0], "achieved": achieved, "peak": peak,
                     "peak_kind": f"{peak_kind} hbm_gbs", "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "algorithmic_bytes_per_launch": dominant[2],
                     "limiter": ("FP64 pipe in the element pass; load latency and the FP64 pipe in the row pass"
                                 if head_mode == "fp64" else "load latency of the row pass"),
                     "passes": {q[0]: {"ms": q[3], "algorithmic_bytes": q[2],
                                       "achieved_gbs": q[2] / (q[3] * 1e-3) / 1e9} for q in passes},
                     "whole_assembly_bytes": bytes_elem + bytes_rows,
                     "whole_assembly_hbm_frac": (bytes_elem + bytes_rows) / ((t_el + t_rows) * 1e-3) / 1e9 / peak,
                     "fp64_pipe": fp64_roof(call, passes, E) if head_mode == "fp64" else None},
        "precision_variants": results,
        "gpu_launches": 3 * args.steps,  # element pass + one row pass per group class
        "clocks": head["clocks"],
    }
    if rank == 0 and not args.no_cpu_baseline:
        sample = OracleSample(args.cells, host_threads())
        line["cpu_baseline"] = cpu_baseline_of(sample, 3)
        sample.step()  # all cores, leaves the oracle's values for the comparison
        for mode, err in oracle_errors(sample, mode_values).items():
            results[mode]["max_rel_err_vs_oracle"] = err
    if rank == 0:
        print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- other rows of the path
#
# --workload selects one of the other assembly paths; each prints one JSON
# line with the same keys.  Algorithmic bytes per call are the inputs read
# plus the outputs written once (coordinates, connectivity, coefficients,
# result values); the roofline is taken over the whole call.

X1 = np.array([[0.25], [0.25], [0.25]])
W1 = np.array([1.0 / 6.0])
AUX_METRIC = {
    "p1_laplace": "assembled CSR nnz/s (FP64 P1-tet Laplace)",
    "n1_maxwell": "assembled CSR nnz/s (FP64 Nedelec N1 Maxwell)",
    "p1_adjoint": "adjoint elements/s (J = u^T K(kappa) v with dJ/dkappa, dJ/dx, dJ/du, dJ/dv, P1)",
    "nh": "neo-Hookean residual+tangent elements/s (FP64 plain law)",
    "vp1_elasticity": "assembled CSR nnz/s (FP64 vector P1 elasticity)",
}


def _timer(args, world):
    import torch

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    flush_buf = []

    def timed(fn, flush_l2=False):
        """Mean device time of one call.  flush_l2 (workloads whose inputs fit in
        L2): before every timed call a 256 MiB buffer is written, outside the
        events around the call."""
        for _ in range(max(3, args.warmup)):
            fn()
        barrier()
        stream = torch.cuda.current_stream()
        if flush_l2 and not flush_buf:
            flush_buf.append(torch.empty(256 << 20, dtype=torch.uint8, device="cuda"))
        with ClockSampler(torch.cuda.current_device()) as clocks:
            barrier()
            if flush_l2:
                pairs = []
                for _ in range(args.steps):
                    flush_buf[0].fill_(1)
                    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    ev0.record(stream)
                    fn()
                    ev1.record(stream)
                    pairs.append((ev0, ev1))
                barrier()
                total = sum(a.elapsed_time(b) for a, b in pairs)
            else:
                ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ev0.record(stream)
                for _ in range(args.steps):
                    fn()
                ev1.record(stream)
                barrier()
                total = ev0.elapsed_time(ev1)
        ms = reduce_max(total / args.steps, world)
        return ms, clocks.summary()

    def wall(fn):
        for _ in range(2):
            fn()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        barrier()
        return reduce_max((time.perf_counter() - t0) / args.steps, world)

    return timed, wall


def _roofline(alg_bytes, ms):
    peak, kind = measured_peak()
    achieved = alg_bytes / (ms * 1e-3) / 1e9
    return {"bound": "hbm", "kernel": "whole call", "achieved": achieved, "peak": peak,
            "peak_kind": f"{kind} hbm_gbs", "unit": "GB/s", "frac": achieved / peak, "traffic": None,
            "algorithmic_bytes_per_launch": alg_bytes}


def _relerr(a, b):
    return float((a - b).abs().max() / b.abs().max())


def sine_displacement(doflocs, seed=5, amplitude=0.05, wavevectors="unit"):
    """Vector P1 displacement: 8 modes amplitude * d_m sin(pi k_m . x + phi_m)
    with seeded unit directions d_m, phases phi_m and wavevectors k_m =
    +-e_axis ("unit") or drawn from {-1, 0, 1}^3 without 0 ("int3") (node-major
    DOFs, component fastest)."""
    rng = np.random.default_rng(np.random.SeedSequence(seed))
    n = doflocs.shape[1]
    u = np.zeros(n)
    comp = np.arange(n) % 3
    for _ in range(8):
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        if wavevectors == "unit":
            kv = np.zeros(3)
            kv[rng.integers(0, 3)] = rng.choice([-1.0, 1.0])
        else:
            kv = np.zeros(3)
            while not kv.any():
                kv = rng.integers(-1, 2, size=3).astype(np.float64)
        ph = rng.uniform(0, 2 * np.pi)
        u += amplitude * d[comp] * np.sin(np.pi * (kv @ doflocs) + ph)
    return u


def _p1_mesh(sk, n, comp=1):
    m = sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, n + 1),) * 3)
    return m, sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=comp), quadrature=(X1, W1))


def wl_p1_laplace(args, world, timed, wall):
    """Plain P1 Laplace a(u,v) = grad u . grad v, 32^3 x 6 cube, 1-point rule, coefficient 1."""
    import skfemntv_gb300 as sk
    from skfemntv_gb300.assembly import NativeBilinearForm

    n = args.cells or 32
    m, b = _p1_mesh(sk, n)
    form = NativeBilinearForm(b)
    nnz, E = form.pattern.nnz, m.nelements
    variants, ref = {}, None
    for mode in ("fp64", "fp64_emulated", "split_fp32"):
        ms, clk = timed(lambda: form.assemble_device(gradient=1.0, precision=mode), flush_l2=True)
        vals = form.target.d_values[:nnz].clone()
        ref = vals if ref is None else ref
        variants[mode] = {"value": world * nnz / (ms * 1e-3), "ms_per_step": ms,
                          "max_rel_err_vs_fp64": _relerr(vals, ref), "clocks": clk}

    # the same FP64 assembly replayed from a CUDA graph (per-element kappa on the device)
    import torch

    kappa = torch.ones(E, dtype=torch.float64, device="cuda")
    graph = form.capture_gradient(kappa)
    ms_g, clk_g = timed(graph.replay, flush_l2=True)
    graph_err = _relerr(form.target.d_values[:nnz], ref)

    @sk.BilinearForm
    def lap(u, v, w):
        return sk.ddot(sk.grad(u), sk.grad(v))

    e2e_s = wall(lambda: sk.asm(lap, b))
    alg = 24 * m.p.shape[1] + 16 * E + 8 * nnz
    head = variants["fp64"]
    return dict(
        metric=AUX_METRIC["p1_laplace"], unit="nnz/s", value=head["value"],
        ms_per_step=head["ms_per_step"], dtype="f64", clocks=head["clocks"],
        config={"workload": f"P1-tet Laplace, {n}^3x6 cube ({E} tets), 1-point rule, coefficient 1",
                "elements": E, "dofs": b.N, "nnz": nnz, "l2": "inputs (8 MB) fit in L2: a 256 MiB buffer is written before every timed call"},
        e2e={"value": world * nnz / e2e_s, "unit": "nnz/s", "h2d_bytes_per_step": 0,
             "d2h_bytes_per_step": 8 * nnz, "ms_per_step": 1e3 * e2e_s},
        roofline=_roofline(alg, head["ms_per_step"]), precision_variants=variants,
        cuda_graph={"value": world * nnz / (ms_g * 1e-3), "ms_per_step": ms_g, "max_rel_err_vs_fp64": graph_err,
                    "clocks": clk_g, "note": "NativeBilinearForm.capture_gradient, replay() per step"},
        gpu_launches=3 * args.steps)


def wl_n1_maxwell(args, world, timed, wall):
    """Nedelec N1 curl-curl + mass, 48^3 x 6 cube with seeded vertex relabelling,
    mu_e = exp(N(0, 0.3^2)), curl coefficient 1/mu_e, mass coefficient 1."""
    import skfemntv_gb300 as sk
    from skfemntv_gb300 import _device as dev
    from skfemntv_gb300._native import call

    n = args.cells or 48
    rng = np.random.default_rng(np.random.SeedSequence(3))
    m0 = sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, n + 1),) * 3)
    perm = rng.permutation(m0.p.shape[1])
    inv = np.argsort(perm)
    mesh = sk.MeshTet(np.ascontiguousarray(m0.p[:, inv]), perm[m0.t].astype(m0.t.dtype))
    mu = np.exp(rng.normal(0.0, 0.3, mesh.nelements))
    nb = sk.AffineTetN1Basis(mesh)
    asmb = sk.TetN1Assembler(nb)
    E, Q = nb.mesh.nelements, len(nb.W)
    nnz = asmb.pattern.nnz
    dnu = dev.to_device(1.0 / mu, np.float64)

    def step():
        call("skg_n1_assemble", asmb.pattern.h, dev.ptr(nb.mesh._dev("p")), nb.mesh.p.shape[1], dev.ptr(nb._t4),
             dev.ptr(nb._ee_dev), dev.ptr(nb._signs_dev), E, Q, dev.hptr(nb.X), dev.hptr(nb.W), None, dev.ptr(dnu),
             1, 1, 0, dev.ptr(asmb.target.d_values), dev.stream_ptr())

    ms, clk = timed(step, flush_l2=True)
    ref = asmb.target.d_values[:nnz].clone()

    def step_split():
        call("skg_n1_assemble", asmb.pattern.h, dev.ptr(nb.mesh._dev("p")), nb.mesh.p.shape[1], dev.ptr(nb._t4),
             dev.ptr(nb._ee_dev), dev.ptr(nb._signs_dev), E, Q, dev.hptr(nb.X), dev.hptr(nb.W), None, dev.ptr(dnu),
             1, 1, 1, dev.ptr(asmb.target.d_values), dev.stream_ptr())

    ms_s, clk_s = timed(step_split, flush_l2=True)
    err_s = _relerr(asmb.target.d_values[:nnz], ref)
    curl = (1.0 / mu)[:, None]
    e2e_s = wall(lambda: asmb.assemble_maxwell(mass_coefficient=1.0, curl_coefficient=curl))
    alg = 24 * mesh.p.shape[1] + 16 * E + 24 * E + 8 * E + 8 * nnz
    return dict(
        metric=AUX_METRIC["n1_maxwell"], unit="nnz/s", value=world * nnz / (ms * 1e-3),
        ms_per_step=ms, dtype="f64", clocks=clk,
        config={"workload": f"N1 curl-curl + mass, {n}^3x6 cube ({E} tets), relabelled vertices, "
                            f"{Q}-point Duffy rule, curl coefficient 1/mu_e, mass 1",
                "elements": E, "dofs": nb.N, "nnz": nnz, "l2": "inputs fit in L2: a 256 MiB buffer is written before every timed call"},
        e2e={"value": world * nnz / e2e_s, "unit": "nnz/s", "h2d_bytes_per_step": 8 * E,
             "d2h_bytes_per_step": 8 * nnz, "ms_per_step": 1e3 * e2e_s},
        roofline=_roofline(alg, ms),
        precision_variants={"fp64": {"value": world * nnz / (ms * 1e-3), "ms_per_step": ms},
                            "split_fp32": {"value": world * nnz / (ms_s * 1e-3), "ms_per_step": ms_s,
                                           "max_rel_err_vs_fp64": err_s, "clocks": clk_s}},
        gpu_launches=3 * args.steps)


def wl_p1_adjoint(args, world, timed, wall):
    """J = u^T K(kappa) v on P1, 64^3 x 6 cube: J and dJ/dkappa, dJ/dx, dJ/du, dJ/dv."""
    import torch

    import skfemntv_gb300 as sk

    n = args.cells or 64
    rng = np.random.default_rng(np.random.SeedSequence(4))
    m, b = _p1_mesh(sk, n)
    E, npts = m.nelements, m.p.shape[1]
    op = sk.P1Energy(b)
    f64 = dict(dtype=torch.float64, device="cuda")
    kappa = torch.as_tensor(np.exp(rng.standard_normal(E)), **f64)
    coords = torch.as_tensor(m.p, **f64).contiguous()
    u = torch.as_tensor(rng.standard_normal(b.N), **f64)
    v = torch.as_tensor(rng.standard_normal(b.N), **f64)

    def step():  # what the autograd forward runs when inputs require gradients
        op.energy_and_gradients(kappa, coords, u, v)

    ms, clk = timed(step, flush_l2=True)
    hk, hu, hv = (x.cpu().numpy() for x in (kappa, u, v))
    pin = [torch.empty(x.shape, dtype=torch.float64, pin_memory=True) for x in (hk, hu, hv)]
    for dst, src in zip(pin, (hk, hu, hv)):
        dst.numpy()[:] = src

    def e2e():
        k = pin[0].to("cuda", non_blocking=True).requires_grad_(True)
        x = coords.detach().clone().requires_grad_(True)
        J = op(k, x, pin[1].to("cuda", non_blocking=True), pin[2].to("cuda", non_blocking=True))
        J.backward()
        return float(J), k.grad.cpu(), x.grad.cpu()

    e2e_s = wall(e2e)
    alg = 24 * npts + 16 * E + 8 * E + 16 * b.N + 8 * E + 24 * npts
    return dict(
        metric=AUX_METRIC["p1_adjoint"], unit="elements/s",
        value=world * E / (ms * 1e-3), ms_per_step=ms, dtype="f64", clocks=clk,
        config={"workload": f"P1 energy adjoint, {n}^3x6 cube ({E} tets), kappa_e = exp(N(0,1)), u, v ~ N(0,1)",
                "elements": E, "dofs": b.N, "l2": "inputs (68 MB) fit in L2: a 256 MiB buffer is written before every timed call"},
        e2e={"value": world * E / e2e_s, "unit": "elements/s", "h2d_bytes_per_step": 8 * (E + 2 * b.N),
             "d2h_bytes_per_step": 8 * (E + 3 * npts), "ms_per_step": 1e3 * e2e_s},
        roofline=_roofline(alg, ms), gpu_launches=3 * args.steps)  # element pass, energy sum, gather


def _nh_fp64(elements, ms):
    peak = _fp64_rate()
    achieved = NH_FP64_OPS_PER_ELEMENT * elements / (ms * 1e-3) / 1e9
    return {"ops_per_element": NH_FP64_OPS_PER_ELEMENT, "achieved_gops": achieved, "peak_gops": peak,
            "frac": achieved / peak, "peak_source": "skg_fp64_fma_rate, measured in this run"}


def _fp64_rate():
    import ctypes

    from skfemntv_gb300._native import call

    rate = ctypes.c_double()
    call("skg_fp64_fma_rate", ctypes.byref(rate), None)
    return rate.value


def wl_nh(args, world, timed, wall):
    """Vector P1 neo-Hookean residual + tangent, 64^3 x 6 cube, mu = 1, lambda = 10:
    plain FP64 law against the GPU-trained MLP energy surrogate."""
    import torch

    import skfemntv_gb300 as sk
    from skfemntv_gb300 import _device as dev

    n = args.cells or 64
    m, b = _p1_mesh(sk, n, comp=3)
    E = m.nelements
    nh = sk.NeoHookean(b, 1.0, 10.0)
    nnz = nh.pattern.nnz
    u = sine_displacement(b.doflocs)
    du = dev.to_device(u, np.float64)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    if args.quick_train:  # profiling runs: a short schedule (accuracy not representative)
        sur = sk.EnergySurrogate.train(mu=1.0, lmbda=10.0, sigma=0.1, n_samples=200_000, steps=300, refine_iters=300,
                                       refine_samples=65536, seed=1)
    else:
        sur = sk.EnergySurrogate.train(mu=1.0, lmbda=10.0, sigma=0.1, seed=1)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    ms_plain, clk = timed(lambda: nh.assemble_device(du), flush_l2=True)
    r0 = nh.d_res[: b.N].clone()
    k0 = nh.target.d_values[:nnz].clone()
    ms_sur, clk_s = timed(lambda: nh.assemble_device(du, surrogate=sur, tol=1e-2, count_fallback=False),
                          flush_l2=True)
    nh.assemble_device(du, surrogate=sur, tol=1e-2)
    fallback = nh.last_fallback
    err_r = _relerr(nh.d_res[: b.N], r0)
    err_k = _relerr(nh.target.d_values[:nnz], k0)
    # the same law and network on the other displacement recipe (integer
    # wavevectors in {-1, 0, 1}^3): deformation gradients farther from the
    # training distribution, so some elements take the plain-law fallback
    u_int = sine_displacement(b.doflocs, wavevectors="int3")
    du_int = dev.to_device(u_int, np.float64)
    ms_plain_i, _ = timed(lambda: nh.assemble_device(du_int), flush_l2=True)
    r0i = nh.d_res[: b.N].clone()
    k0i = nh.target.d_values[:nnz].clone()
    ms_sur_i, _ = timed(lambda: nh.assemble_device(du_int, surrogate=sur, tol=1e-2, count_fallback=False),
                        flush_l2=True)
    nh.assemble_device(du_int, surrogate=sur, tol=1e-2)
    int3 = {"tol_1e-2": {"fallback_elements": nh.last_fallback, "fallback_fraction": nh.last_fallback / E,
                         "plain_ms": ms_plain_i, "surrogate_ms": ms_sur_i, "speedup_vs_plain": ms_plain_i / ms_sur_i,
                         "max_rel_err_residual": _relerr(nh.d_res[: b.N], r0i),
                         "max_rel_err_tangent": _relerr(nh.target.d_values[:nnz], k0i)}}
    # a tighter stress check sends more of these elements to the plain law
    ms_sur_t, _ = timed(lambda: nh.assemble_device(du_int, surrogate=sur, tol=1e-4, count_fallback=False),
                        flush_l2=True)
    nh.assemble_device(du_int, surrogate=sur, tol=1e-4)
    int3["tol_1e-4"] = {"fallback_elements": nh.last_fallback, "fallback_fraction": nh.last_fallback / E,
                        "surrogate_ms": ms_sur_t, "speedup_vs_plain": ms_plain_i / ms_sur_t,
                        "max_rel_err_residual": _relerr(nh.d_res[: b.N], r0i),
                        "max_rel_err_tangent": _relerr(nh.target.d_values[:nnz], k0i)}
    del du_int, r0i, k0i
    hu = torch.empty(b.N, dtype=torch.float64, pin_memory=True)
    hu.numpy()[:] = u
    e2e_s = wall(lambda: nh.assemble(hu.numpy()))
    alg = 24 * m.p.shape[1] + 16 * E + 2 * 8 * b.N + 8 * nnz
    return dict(
        metric=AUX_METRIC["nh"], unit="elements/s",
        value=world * E / (ms_plain * 1e-3), ms_per_step=ms_plain, dtype="f64", clocks=clk,
        config={"workload": f"vector P1 neo-Hookean, {n}^3x6 cube ({E} tets), 8 sine modes amplitude 0.05, "
                            "unit wavevectors, mu=1, lambda=10, 1-point rule",
                "training": "short profiling schedule" if args.quick_train else
                            "2M samples, 3000 Adam steps, L-BFGS on 524,288 samples",
                "elements": E, "dofs": b.N, "nnz": nnz, "l2": "inputs fit in L2: a 256 MiB buffer is written before every timed call"},
        e2e={"value": world * E / e2e_s, "unit": "elements/s", "h2d_bytes_per_step": 8 * b.N,
             "d2h_bytes_per_step": 8 * (b.N + nnz), "ms_per_step": 1e3 * e2e_s},
        roofline=dict(_roofline(alg, ms_plain), fp64_pipe=_nh_fp64(E, ms_plain)),
        learned_closure={"value": world * E / (ms_sur * 1e-3), "ms_per_step": ms_sur,
                         "speedup_vs_plain": ms_plain / ms_sur, "max_rel_err_residual": err_r,
                         "max_rel_err_tangent": err_k, "fallback_elements": fallback,
                         "training_seconds": t_train, "training_history": sur.history[-2:],
                         "roofline": _roofline(alg, ms_sur), "clocks": clk_s,
                         "integer_wavevectors": int3},
        gpu_launches=3 * args.steps)


def wl_vp1_elasticity(args, world, timed, wall):
    """Vector P1 linear elasticity 2 mu eps(u):eps(v) + lambda div u div v + rho u.v (mu = 1, lambda = 10,
    rho = 0.5) on a 48^3 x 6 cube with the reference's default 4-point rule (value, symmetric-gradient and
    divergence kinds, bilinear_form_assembler.cpp:79-105): constant coefficients through the fused affine P1
    kernel, and the same form with per-point coefficients through the tabulated kernels."""
    import skfemntv_gb300 as sk
    from skfemntv_gb300.assembly import NativeBilinearForm

    n = args.cells or 48
    m = sk.MeshTet.init_tensor(*(np.linspace(0.0, 1.0, n + 1),) * 3)
    b = sk.Basis(m, sk.ElementVector(sk.ElementTetP1(), dim=3))
    form = NativeBilinearForm(b)
    nnz, E = form.pattern.nnz, m.nelements
    ms, clk = timed(lambda: form.assemble_device(value=0.5, symmetric_gradient=2.0, divergence=10.0), flush_l2=True)
    # the same form with the coefficients given per point (device (E, Q) arrays): the tabulated kernels
    import torch

    Qn = len(b.W)
    pts = {k: torch.full((E, Qn), v, dtype=torch.float64, device="cuda")
           for k, v in (("value", 0.5), ("symmetric_gradient", 2.0), ("divergence", 10.0))}
    ms_tab, _ = timed(lambda: form.assemble_device(**pts), flush_l2=True)
    fused = form.assemble_device(value=0.5, symmetric_gradient=2.0, divergence=10.0)[:nnz].clone()
    tab_err = _relerr(form.assemble_device(**pts)[:nnz], fused)
    del pts

    @sk.BilinearForm
    def elast(u, v, w):
        return 2.0 * sk.ddot(sk.sym_grad(u), sk.sym_grad(v)) + 10.0 * sk.div(u) * sk.div(v) + 0.5 * sk.dot(u, v)

    e2e_s = wall(lambda: sk.asm(elast, b))
    Q = len(b.W)
    alg = 24 * m.p.shape[1] + 48 * E + 8 * nnz
    return dict(
        metric=AUX_METRIC["vp1_elasticity"], unit="nnz/s", value=world * nnz / (ms * 1e-3), ms_per_step=ms,
        dtype="f64", clocks=clk,
        config={"workload": f"vector P1 elasticity, {n}^3x6 cube ({E} tets), {Q}-point rule, "
                            "mu=1, lambda=10, rho=0.5, constant coefficients (fused affine P1 path)",
                "elements": E, "dofs": b.N, "nnz": nnz, "l2": "inputs fit in L2: a 256 MiB buffer is written before every timed call"},
        per_point_tabulated={"ms_per_step": ms_tab, "value": world * nnz / (ms_tab * 1e-3),
                             "max_rel_err_vs_fused": tab_err,
                             "note": "same form, coefficients as device (E, Q) arrays: tabulated kernels"},
        e2e={"value": world * nnz / e2e_s, "unit": "nnz/s", "h2d_bytes_per_step": 0,
             "d2h_bytes_per_step": 8 * nnz, "ms_per_step": 1e3 * e2e_s},
        roofline=_roofline(alg, ms), gpu_launches=3 * args.steps)  # element pass + one row pass per group class


AUX_WORKLOADS = {"p1_laplace": wl_p1_laplace, "n1_maxwell": wl_n1_maxwell, "p1_adjoint": wl_p1_adjoint,
                 "nh": wl_nh, "vp1_elasticity": wl_vp1_elasticity}


def run_aux(args, rank, world):
    import torch

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    timed, wall = _timer(args, world)
    r = AUX_WORKLOADS[args.workload](args, world, timed, wall)
    line = {"metric": r.pop("metric"), "value": r.pop("value"), "unit": r.pop("unit"), "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": r.pop("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": r.pop("dtype"),
            "data": "synthetic (seeded)"}
    line.update(r)
    line["config"]["parallelism"] = f"replicas x{world}" if world > 1 else "single GPU"
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = aux_cpu_baseline(args.workload, host_threads())
    if rank == 0:
        print(json.dumps(line), flush=True)


def aux_cpu_baseline(workload, threads, reps=3):
    """The oracle (CPU restatement of the reference's assembly) on a bounded
    sample of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    def mesh(n):
        return O.mesh_tet_tensor(*(np.linspace(0.0, 1.0, n + 1),) * 3)

    if workload == "p1_laplace":
        n = 32
        p, t = mesh(n)
        b = O.make_basis(p, t, False, quadrature=(X1, W1), threads=threads)
        dofs = b.dofs3.reshape(b.dofs3.shape[0], -1)
        pat = O.Pattern(dofs, dofs)
        grad = np.ones(b.dx.shape)
        run = lambda: O.bilinear_assemble(b, gradient=grad, threads=threads, pattern=pat)  # noqa: E731
        units, unit, desc = pat.nnz, "nnz/s", f"P1 Laplace {n}^3x6 (full size), threaded colored assembly"
    elif workload == "n1_maxwell":
        n = 24
        p, t = mesh(n)
        b = O.make_n1_basis(p, t)
        pat = O.Pattern(np.ascontiguousarray(b.element_dofs.T), nrows=b.N, coloring=False)
        curl = np.ones(b.dx.shape)
        run = lambda: O.n1_assemble_maxwell(b, 1.0, curl, threads=threads, pattern=pat)  # noqa: E731
        units, unit, desc = pat.nnz, "nnz/s", f"N1 Maxwell {n}^3x6 sample, threaded element integration + scatter"
    elif workload == "p1_adjoint":
        n = 32
        p, t = mesh(n)
        rng = np.random.default_rng(4)
        b = O.make_basis(p, t, False, quadrature=(X1, W1), threads=threads)
        E = t.shape[1]
        kappa = np.exp(rng.standard_normal(E))
        u, v = rng.standard_normal(b.N), rng.standard_normal(b.N)
        dofs = b.dofs3.reshape(E, -1)
        pat = O.Pattern(dofs, dofs)

        def run():
            data, indptr, indices = O.bilinear_assemble(b, gradient=kappa[:, None], threads=threads, pattern=pat)
            import scipy.sparse as sp
            J = u @ (sp.csr_matrix((data, indices, indptr), shape=(b.N, b.N)) @ v)
            gu = np.einsum("ea,eaj->ej", u[dofs], b.grad[:, 0])
            gv = np.einsum("ea,eaj->ej", v[dofs], b.grad[:, 0])
            return J, np.einsum("ej,ej->e", gu, gv) * b.dx[:, 0]

        units, unit, desc = E, "elements/s", (f"P1 {n}^3x6 sample: J via assembled K and dJ/dkappa "
                                              "(no coordinate gradient)")
    elif workload == "vp1_elasticity":
        n = 24
        p, t = mesh(n)
        X, W = O.tet_quadrature_p1()
        b = O.make_basis(p, t, False, comp=3, quadrature=(X, W), threads=threads)
        dofs = b.dofs3.reshape(b.dofs3.shape[0], -1)
        pat = O.Pattern(dofs, dofs)
        run = lambda: O.bilinear_assemble(b, value=0.5, symmetric_gradient=2.0, divergence=10.0,  # noqa: E731
                                          threads=threads, pattern=pat)
        units, unit, desc = pat.nnz, "nnz/s", f"vector P1 elasticity {n}^3x6 sample, threaded colored assembly"
    else:
        n = 24
        p, t = mesh(n)
        b = O.make_basis(p, t, False, comp=3, quadrature=(X1, W1), threads=threads)
        u = sine_displacement(np.repeat(p, 3, axis=1))
        dofs = b.dofs3.reshape(b.dofs3.shape[0], -1)
        pat = O.Pattern(dofs, dofs)

        def run():
            Gu = O.displacement_gradient(b, u)
            r = O.linear_assemble(b, gradient=O.nh_first_piola(Gu, 1.0, 10.0))
            return r, O.cross_gradient_tensor_assemble(b, O.nh_tangent(Gu, 1.0, 10.0), threads=threads,
                                                       pattern=pat)

        units, unit, desc = t.shape[1], "elements/s", f"neo-Hookean {n}^3x6 sample: numpy law + oracle assembly"
    run()
    t0 = time.perf_counter()
    for _ in range(reps):
        run()
    dt = (time.perf_counter() - t0) / reps
    return {"value": units / dt, "unit": unit, "cores": threads, "kind": "port", "sample": f"{desc}, {reps} runs"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="p2_aniso", choices=["p2_aniso"] + sorted(AUX_WORKLOADS),
                    help="p2_aniso (headline) or another row of the assembly path")
    ap.add_argument("--cells", type=int, default=None, help="cube cells per side (smaller cases for profiling)")
    ap.add_argument("--quick-train", action="store_true",
                    help="nh workload: short surrogate training (profiling runs only)")
    ap.add_argument("--modes", default="fp64,fp64_emulated,split_fp32",
                    help="precision modes to time; the first is the headline")
    args = ap.parse_args()
    args.modes = [m for m in args.modes.split(",") if m]
    if args.workload == "p2_aniso" and args.cells is None:
        args.cells = N_CELLS
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
        if args.workload == "p2_aniso":
            run_gpu(args, rank, world)
        else:
            run_aux(args, rank, world)
    finally:
        if world > 1:
            import torch

            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
