"""Benchmark of the Laplace/diffusion assembly hot path (one step = one whole-mesh assembly).

Workload: 128^3 trilinear hexahedra on the unit cube (E = 2,097,152, N = 2,146,689 nodes,
nnz = 57,066,625), 2x2x2 Gauss, interior nodes jittered uniformly by +-0.1h and per-element
conductivity log-uniform in [0.1, 10] (seeded synthetic inputs).  The headline `value` is
assembled elements/s with inputs resident in HBM; `e2e` is the same metric through the C ABI with
host buffers (coordinates and conductivities copied in, the assembled CSR values copied out,
inside the timed region).  The solve (Jacobi-CG to relative residual 1e-12, FP64 and mixed
refinement) is reported beside it.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl gfe|reference] [--n 128]

--impl reference times the CPU restatement of Iron's element loop (the oracle, Iron's own
algorithm: per-element gather, Gauss loop, bisection insert into CSR) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L2_BYTES = 129 * 1024 * 1024
WORKLOAD = "laplace_diffusion_trilinear_hex"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gfe", choices=["gfe", "reference"])
    ap.add_argument("--n", type=int, default=128, help="elements per side")
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed_df", "mixed"])
    ap.add_argument("--workload", default="laplace",
                    choices=["laplace", "laplace_bases", "mr", "mr_newton", "mr_adjoint", "serve"],
                    help="laplace: the headline assembly workload; laplace_bases: higher-order Lagrange, "
                         "Hermite and simplex Laplace assembly; mr: Mooney-Rivlin Q2/Q1 residual + Jacobian "
                         "assembly (32^3); mr_newton: load-stepped Newton solve of the uniaxial stretch (32^3); "
                         "mr_adjoint: batched residual adjoint (16^3 x 64); serve: request stream")
    ap.add_argument("--path", default="auto", choices=["auto", "regular", "general"],
                    help="assembly kernel: regular-mesh tiled kernel (auto for generated meshes) or colour scatter")
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the Mooney-Rivlin keys of the headline line (for profiling runs)")
    ap.add_argument("--serve-requests", type=int, default=2000, help="serve workload: requests in the stream")
    ap.add_argument("--serve-workers", type=int, default=8, help="serve workload: concurrent request slots")
    ap.add_argument("--serve-rate", type=float, default=200.0, help="serve workload: Poisson arrival rate (1/s)")
    ap.add_argument("--headline-serve-requests", type=int, default=200,
                    help="requests of the below-capacity stream in the headline line (0: none)")
    ap.add_argument("--headline-serve-rate", type=float, default=20.0,
                    help="arrival rate (1/s) of the below-capacity stream in the headline line")
    ap.add_argument("--cpu-sample-n", type=int, default=48, help="side of the single-core CPU-baseline sample mesh")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def make_problem(n: int, seed: int = 0):
    from iron_gb300 import mesh as M

    m = M.RegularMesh((n, n, n))
    m.jitter_interior(seed)
    kappa = np.exp(np.random.default_rng(seed + 1).uniform(np.log(0.1), np.log(10.0), m.n_elements))
    return m, kappa


def algorithmic_bytes(E: int, N: int, nnz: int) -> int:
    # E*(8*4 connectivity + 8 conductivity) + N*(3*8 coordinates + 8 rhs) + nnz*8 (values written once)
    return E * (8 * 4 + 8) + N * (3 * 8 + 8) + nnz * 8


def algorithmic_flops(E: int) -> int:
    # per element: ng*(18 nen + 45 + 18 nen + 6 nen^2) with nen = 8, ng = 8
    return E * 8 * (18 * 8 + 45 + 18 * 8 + 6 * 64)


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic_per_unit(kernel: str):
    """DRAM bytes (read + write) per element of `kernel` (e.g. "laplace_regular_kernel<f2>") from
    the committed ncu summary profiles/laplace_kernels_traffic.txt, if it lists the kernel."""
    p = ROOT / "profiles" / "laplace_kernels_traffic.txt"
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        parts = ln.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def cpu_baseline(n_sample: int, threads: int, structure=None):
    """The oracle (Iron's algorithm restated in C++) timed on an n_sample^3 mesh of the workload on
    `threads` host cores.  Returns (elements/s, seconds, elements, oracle values, (row_ptr, col_idx))."""
    import oracle

    m, kappa = make_problem(n_sample, seed=0)
    rp, ci = structure if structure is not None else oracle.csr_structure(m.elem_nodes, m.n_nodes)
    # the timing build: the compiler's default FMA contraction, as a normal build of Iron would have
    prev = oracle.use_build("timing")
    try:
        oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], m.elem_nodes[:64], m.coords, kappa[:64], rp, ci, 1)
        t0 = time.perf_counter()
        vals, _ = oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], m.elem_nodes, m.coords, kappa, rp, ci, threads)
        dt = time.perf_counter() - t0
    finally:
        oracle.use_build(prev)
    return m.n_elements / dt, dt, m.n_elements, vals, (rp, ci)


def cpu_baseline_bases(interp, ngauss, elem_params, params, scale, kappa):
    """The oracle's basis-generic Laplace assembly timed on one sample mesh on all host cores."""
    import oracle

    threads = os.cpu_count() or 1
    rp, ci = oracle.csr_structure(elem_params, params.shape[1])
    prev = oracle.use_build("timing")
    try:
        t0 = time.perf_counter()
        oracle.laplace_assemble_scaled(3, interp, ngauss, elem_params, params, scale, kappa, rp, ci, threads)
        dt = time.perf_counter() - t0
    finally:
        oracle.use_build(prev)
    E = elem_params.shape[0]
    return E / dt, dt, E, threads


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle

    threads = os.cpu_count() or 1
    n = args.n
    m, _ = make_problem(n, seed=0)
    structure = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    del m
    vals = []
    E = n ** 3
    for i in range(args.warmup + args.steps):
        v, dt, E, _, _ = cpu_baseline(n, threads, structure)
        if i >= args.warmup:
            vals.append(v)
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": "assembled_elements_per_s", "value": value, "unit": "elements/s",
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "elements_per_side": n, "elements": E, "gauss": "2x2x2",
                   "conductivity": "log-uniform [0.1,10] seeded", "jitter": "+-0.1h seeded"},
        "cpu_baseline": {"value": value, "unit": "elements/s", "cores": threads, "kind": "port",
                         "sample": f"the whole {n}^3 = {E} element workload per step; Iron's algorithm restated in "
                                   f"C++ (oracle/), Iron itself cannot be built here (Fortran+MPI+PETSc)"},
        "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gfe(args):
    import torch

    from iron_gb300 import _lib, replicas
    from iron_gb300.laplace import LaplaceAssembly

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local if ws > 1 else 0)
    torch.cuda.set_device(dev)
    _lib.load()

    log(f"mesh {args.n}^3")
    m, kappa = make_problem(args.n, seed=rank)
    log("structure + device upload")
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kappa, device=dev)
    E, N, nnz = A.n_elements, A.n_nodes, A.nnz
    ncol = len(A.colour_ptr) - 1
    stream = torch.cuda.current_stream(dev)

    path = args.path
    # element-matrix accuracy of each precision against the FP64 assembly
    v64 = A.assemble("fp64", path=path).clone()
    precisions = ["fp64", "mixed_df", "mixed"]
    asm_err = {}
    for prec in precisions[1:]:
        v = A.assemble(prec, path=path)
        asm_err[prec] = float((v - v64).abs().max() / v64.abs().max())
    del v64
    timings = {}
    log("timed assembly")
    for prec in precisions:
        for _ in range(args.warmup):
            A.assemble(prec, check=False, path=path)
        torch.cuda.synchronize()
        _lib.profile_enable(True)
        _lib.profile_read(_lib.STAGE_LAPLACE_ELEMENTS, reset=True)
        replicas.barrier()
        with ClockSampler(dev.index) as clk:
            torch.cuda.synchronize()
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(args.steps):
                A.assemble(prec, check=False, path=path)
            t1.record(stream)
            torch.cuda.synchronize()
        _lib.profile_enable(False)
        kern_ms, launches = _lib.profile_read(_lib.STAGE_LAPLACE_ELEMENTS, reset=True)
        _lib.raise_device_errors("bench assembly")
        ms = replicas.max_over_replicas(t0.elapsed_time(t1) / args.steps, dev)
        timings[prec] = {"ms_per_step": ms, "kernel_ms_total": kern_ms, "launches": launches,
                         "clocks": clk.summary()}

    log("end-to-end timing")
    # end to end through the C ABI with host buffers: H2D geometry + conductivity, D2H values
    coords_h = torch.from_numpy(m.coords).pin_memory()
    kappa_h = torch.from_numpy(kappa).pin_memory()
    vals_h = torch.empty(nnz, dtype=torch.float64).pin_memory()
    e2e = {}
    for prec in precisions:
        # on the regular mesh every precision uses the native slab pipeline (inputs uploaded slab by
        # slab, device-to-host copies overlapping later slabs); otherwise copy in, assemble, copy out
        pipelined = A.regular is not None and path in ("regular", "auto")
        for i in range(args.warmup + args.steps):
            if i == args.warmup:
                torch.cuda.synchronize()
                replicas.barrier()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
            if pipelined:
                A.assemble_to_host(vals_h, prec, coords_host=coords_h, kappa_host=kappa_h, stream=stream)
            else:
                A.coords.copy_(coords_h, non_blocking=True)
                A.kappa.copy_(kappa_h, non_blocking=True)
                A.assemble(prec, check=False, path=path)
                vals_h.copy_(A.values, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e[prec] = replicas.max_over_replicas(e0.elapsed_time(e1) / args.steps, dev)
        if pipelined:
            # the host copy equals the device-resident assembly of the same precision
            A.assemble(prec, check=False, path="regular")
            torch.cuda.synchronize()
            if not torch.equal(vals_h, A.values.cpu()):
                raise RuntimeError(f"slab-pipelined host values differ from the device assembly ({prec})")
    _lib.raise_device_errors("bench e2e")
    h2d = int(coords_h.numel() * 8 + kappa_h.numel() * 8)
    d2h = int(nnz * 8)

    solve = None
    if not args.no_solve:
        fixed = torch.zeros(N, dtype=torch.uint8, device=dev)
        x0 = torch.zeros(N, dtype=torch.float64, device=dev)
        left, right = torch.from_numpy(m.face_nodes(0, 0)).to(dev), torch.from_numpy(m.face_nodes(0, 1)).to(dev)
        fixed[left] = 1
        fixed[right] = 1
        x0[right] = 1.0
        solve = {}
        xs = {}
        for prec in precisions:
            log(f"solve {prec}")
            A.assemble(prec, path=path, fp32_copy=prec != "fp64")
            x = x0.clone()
            torch.cuda.synchronize()
            s0 = time.perf_counter()
            info = A.solve(fixed, x, rtol=1e-12, precision=prec)
            torch.cuda.synchronize()
            solve[prec] = {"ms": (time.perf_counter() - s0) * 1e3, "iterations": info.iterations,
                           "rel_residual": info.relative_residual}
            xs[prec] = x
            # Iron's path: the solver system (fixed DOFs removed, their coupling in the right-hand
            # side), built once per set of fixed DOFs, reduced per assembly, solved, copied back
            torch.cuda.synchronize()
            s0 = time.perf_counter()
            S = A.solver_system(fixed) if A.regular is not None else A.solver_system(fixed, col_listed=None)
            torch.cuda.synchronize()
            s1 = time.perf_counter()
            xr = x0.clone()
            info_r = A.solve_reduced(fixed, xr, rtol=1e-12, precision=prec, system=S)
            torch.cuda.synchronize()
            s2 = time.perf_counter()
            solve[prec]["reduced"] = {"structure_ms": (s1 - s0) * 1e3, "reduce_and_solve_ms": (s2 - s1) * 1e3,
                                      "iterations": info_r.iterations, "rel_residual": info_r.relative_residual,
                                      "n_free": S.n_free, "nnz": S.nnz,
                                      "max_diff_vs_full_space": float((xr - x).abs().max())}
        for prec in precisions[1:]:
            solve[prec]["rel_err_vs_fp64"] = float((xs[prec] - xs["fp64"]).abs().max() / xs["fp64"].abs().max())
        solve["note"] = ("Jacobi-CG, u=0 at x=0 and u=1 at x=1, rtol 1e-12 on the assembled FP64 matrix; mixed "
                         "precisions = FP32 inner CG + FP64 refinement; rel_err vs the FP64 assembly+solve; "
                         "'reduced' = Iron's solver system (Dirichlet rows/columns removed) solved the same way")

    # headline: the fastest precision whose solution meets the 1e-10 accuracy bar vs FP64 plain
    head = "fp64"
    if args.precision != "auto":
        head = args.precision
    elif solve is not None:
        for prec in precisions[1:]:
            if solve[prec].get("rel_err_vs_fp64", 1.0) <= 1e-10 and \
                    timings[prec]["ms_per_step"] < timings[head]["ms_per_step"]:
                head = prec
    T = timings[head]
    if path == "auto":
        used_path = "general" if (head == "fp64" or A.regular is None) else "regular"
    else:
        used_path = path
    value = replicas.job_throughput(E, T["ms_per_step"], ws)
    bytes_per_elem = algorithmic_bytes(E, N, nnz) / E
    peak, peak_kind = measured_peaks()
    if used_path == "regular" and head == "mixed_df":
        # float-float on the regular mesh: three kernels per assembly (Gauss-point metrics,
        # contraction, row gather); the roofline is that of the whole assembly
        knames = ["laplace_metric_kernel<f2>", "laplace_contract_kernel<f2>", "laplace_gather_kernel<f2>"]
        per_launch_ms = T["kernel_ms_total"] / max(args.steps, 1)
        units_per_launch = E
    else:
        knames = [("laplace_regular_kernel" if used_path == "regular" else "laplace_assemble_color") +
                  "<%s>" % {"fp64": "double", "mixed_df": "f2", "mixed": "float"}[head]]
        per_launch_ms = T["kernel_ms_total"] / max(T["launches"], 1)
        units_per_launch = E / max(T["launches"] // max(args.steps, 1), 1)
    achieved = bytes_per_elem * units_per_launch / (per_launch_ms * 1e-3) / 1e9
    kname = " + ".join(knames)
    parts = [profile_traffic_per_unit(k) for k in knames]
    tpu = None if any(t is None for t in parts) else sum(parts)
    line = {
        "metric": "assembled_elements_per_s", "value": value, "unit": "elements/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": T["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "mixed_df": "f32x2+f64acc", "mixed": "f32+f64acc"}[head],
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "elements_per_side": args.n, "elements": E, "nodes": N, "nnz": nnz,
                   "gauss": "2x2x2", "conductivity": "log-uniform [0.1,10] seeded", "jitter": "+-0.1h seeded",
                   "precision": head, "l2": "inputs larger than L2 (CSR values %.0f MB > 129 MB)" % (nnz * 8 / 1e6),
                   "parallelism": "replicas" if ws > 1 else "single"},
        "clocks": T["clocks"],
        "e2e": {"value": replicas.job_throughput(E, e2e[head], ws), "unit": "elements/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        # element kernel launches + one coordinate split (regular path) or FP32 copy (colour path)
        # per step for the FP32-pipe precisions
        "gpu_launches": int(T["launches"]) + (args.steps if head != "fp64" else 0),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "traffic": None if tpu is None else tpu * units_per_launch,
                     "kernel": kname,
                     "per_launch_ms": per_launch_ms, "units_per_launch": units_per_launch,
                     "algorithmic_bytes_per_element": bytes_per_elem},
        "precisions": {p: {"ms_per_step": timings[p]["ms_per_step"],
                           "elements_per_s": replicas.job_throughput(E, timings[p]["ms_per_step"], ws),
                           "e2e_ms": e2e[p], "kernel_ms_per_launch": timings[p]["kernel_ms_total"] /
                           max(timings[p]["launches"], 1)} for p in precisions},
        "assembly_rel_err_vs_fp64": asm_err,
        "path": used_path,
    }
    log("fma probes")
    try:
        line["fp64_pipe_gflops"] = _lib.probe_fma_rate(_lib.GFE_FP64)
        line["fp32_pipe_gflops"] = _lib.probe_fma_rate(_lib.GFE_MIXED)
        fl = algorithmic_flops(E) / (T["ms_per_step"] * 1e-3) / 1e9
        line["flops"] = {"algorithmic_gflops_per_s": fl, "formula": "E*8*(18*8+45+18*8+6*64)"}
        # the element arithmetic, not memory, bounds the headline kernel: its algorithmic flops are
        # FP64-accurate (float-float on the FP32 pipes), so the natural roof is GB300's FP64 pipe
        fp64_peak = line["fp64_pipe_gflops"]
        line["compute_roofline"] = {
            "bound": "fp32_pipe" if head != "fp64" else "fp64_pipe",
            "achieved_fp64_equivalent_gflops": fl,
            "fp64_pipe_peak_gflops": fp64_peak, "vs_fp64_pipe_peak": fl / fp64_peak if fp64_peak else None,
            "fp32_pipe_peak_gflops": line["fp32_pipe_gflops"],
            "note": "algorithmic flops per second against the probed FMA-chain rates; float-float "
                    "costs several FP32 instructions per FP64-accurate flop"}
    except Exception as exc:  # diagnostic only
        line["probe_error"] = str(exc)
    if solve is not None:
        line["solve"] = solve
    if rank == 0:
        threads = os.cpu_count() or 1
        log("cpu baseline: the oracle on the whole workload")
        v, dt, Es, ovals, _ = cpu_baseline(args.n, threads)
        line["cpu_baseline"] = {"value": v, "unit": "elements/s", "cores": threads, "kind": "port",
                                "sample": f"the whole {args.n}^3 = {Es} element workload, one assembly ({dt:.2f} s)"}
        # the assembled values of the GPU kernels against the oracle's at full size
        scale = float(np.abs(ovals).max())
        acc = {}
        for prec in precisions:
            pth = "general" if prec == "fp64" else path
            g = A.assemble(prec, path=pth).cpu().numpy()
            acc[prec] = float(np.abs(g - ovals).max() / scale)
        line["assembly_rel_err_vs_oracle"] = acc
        del ovals
        n1 = args.cpu_sample_n
        log(f"cpu baseline: one core on a {n1}^3 sample")
        v1, dt1, E1, _, _ = cpu_baseline(n1, 1)
        line["cpu_baseline_single_core"] = {"value": v1, "unit": "elements/s", "cores": 1, "kind": "port",
                                            "sample": f"{n1}^3 = {E1} elements, one assembly ({dt1:.2f} s); one "
                                                      "core matches one Iron MPI rank"}
        if solve is not None:
            log("solution against the oracle's FP64 solve (48^3)")
            line["solve_vs_oracle_48"] = solution_vs_oracle(48, dev)
        if not args.headline_only:
            log("Mooney-Rivlin 32^3 Jacobians and 16^3 x 64 adjoint")
            from iron_gb300 import benchmarks

            line["mooney_rivlin_32"] = benchmarks.mr_measure(32, 5, 3, ClockSampler, log)
            line["mooney_rivlin_adjoint_16x64"] = benchmarks.mr_adjoint_measure(16, 64, 5, 3, ClockSampler, log)
            if args.headline_serve_requests > 0:
                from iron_gb300 import serving

                rate = args.headline_serve_rate
                log(f"serving: {args.headline_serve_requests} requests at {rate:g}/s")
                reqs = serving.request_stream(n_requests=args.headline_serve_requests, rate=rate, seed=1,
                                              mr_n_hi=serving.MR_SERVE_N_HI)
                for r in reqs:
                    serving.make_inputs(r)
                m = serving.measure_stream(reqs, args.serve_workers, ClockSampler, log)
                line["serve_stream_below_capacity"] = {
                    "config": serving.stream_config(reqs, rate, 64, serving.MR_SERVE_N_HI, args.serve_workers), **m}
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def solution_vs_oracle(n: int, dev) -> dict:
    """The benchmark's problem at n^3 (u = 0 at x = 0, u = 1 at x = 1) solved on the GPU (FP64 and
    float-float assembly with FP32-refined CG, rtol 1e-12) against the oracle's FP64 assembly and CG
    (rtol 1e-13): max |u - u_oracle| / max |u_oracle| per precision."""
    import torch

    import oracle
    from iron_gb300.laplace import LaplaceAssembly

    m, kappa = make_problem(n, seed=2)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kappa, device=dev)
    rp, ci = oracle.csr_structure(m.elem_nodes, m.n_nodes)
    ov, _ = oracle.laplace_assemble(3, [1, 1, 1], [2, 2, 2], m.elem_nodes, m.coords, kappa, rp, ci,
                                    os.cpu_count() or 1)
    fixed = np.zeros(m.n_nodes, np.uint8)
    x0 = np.zeros(m.n_nodes)
    fixed[m.face_nodes(0, 0)] = 1
    fixed[m.face_nodes(0, 1)] = 1
    x0[m.face_nodes(0, 1)] = 1.0
    uo, _, _ = oracle.cg_dirichlet(rp, ci, ov, None, fixed, x0, rtol=1e-13)
    out = {}
    for prec in ("fp64", "mixed_df"):
        A.assemble(prec, fp32_copy=prec != "fp64")
        x = torch.from_numpy(x0).to(dev)
        A.solve(torch.from_numpy(fixed).to(dev), x, rtol=1e-12, precision=prec)
        out[prec] = float(np.abs(x.cpu().numpy() - uo).max() / np.abs(uo).max())
    return out


def log(msg: str) -> None:
    """Progress on stderr (the JSON result line is the only stdout output)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def main():
    import faulthandler

    faulthandler.enable()
    args = parse()
    if args.workload != "laplace":
        from iron_gb300 import benchmarks

        args.hbm_peak = measured_peaks()
        return benchmarks.run(args, log=log, clock_sampler=ClockSampler,
                              cpu_bases=cpu_baseline_bases if args.workload == "laplace_bases" else None)
    if args.impl == "reference":
        return run_reference(args)
    return run_gfe(args)


if __name__ == "__main__":
    sys.exit(main())
