"""Secondary benchmark workloads of bench.py (the default workload, Laplace assembly, lives there).

mr:         Mooney-Rivlin mixed u-p (triquadratic u, trilinear p) residual, Iron's analytic
            Jacobian and the consistent tangent assembled on a 32^3 mesh, c10 = 2, c01 = 6, at a 10 %
            uniaxial stretch state with a small seeded perturbation.
mr_adjoint: residual and its hand-written adjoint for a batch of 64 parameter sets on a 16^3 mesh
            (c10, c01 log-uniform in [0.5, 10], displacement perturbation N(0, (0.01 h)^2), seeded).
laplace_bases: the basis-generic Laplace assembly (triquadratic and tricubic Lagrange hexahedra,
            tricubic Hermite with arc-length scale factors, linear, quadratic and cubic tetrahedra) on
            jittered meshes with log-uniform conductivity, FP64 / float-float / FP32, against the
            oracle on a sample of each mesh.
serve:      the request stream of iron_gb300.serving.

Each prints one JSON line.
"""
from __future__ import annotations

import json
import time

import numpy as np
import torch

from . import _lib
from .elasticity import MooneyRivlinAssembly


def _events_time(fn, steps, warmup, stream):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def stretched_state(A: MooneyRivlinAssembly, lam: float, c10: float, c01: float, seed: int, amp: float):
    """z = uniaxial isochoric stretch of x plus N(0, (amp h)^2); p = traction-free lateral value."""
    rng = np.random.default_rng(seed)
    x = A.xg.cpu().numpy()
    z = x * np.array([lam, lam ** -0.5, lam ** -0.5])[:, None]
    h = 1.0 / A.mesh.nelem[0]
    z = z + rng.normal(0.0, amp * h, z.shape)
    F = np.diag([lam, lam ** -0.5, lam ** -0.5])
    Cb = F.T @ F
    S = -2 * c01 * Cb + 2 * (c10 + np.trace(Cb) * c01) * np.eye(3)
    sb = F @ S @ F.T
    p = np.trace(sb) / 3 - sb[1, 1]
    return np.r_[z.ravel(), np.full(A.n_lin, p)]


def mr_measure(n: int, steps: int, warmup: int, clock_sampler, log) -> dict:
    """Residual, Jacobians (Iron's analytic in FP64 / FP32 CUDA-core / tensor-core contraction, the
    consistent tangent, Iron's FD Jacobian) of the n^3 Q2/Q1 mesh at a 10 % stretched, perturbed state:
    times, errors against FP64 and algorithmic rates."""
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    log(f"MR Q2/Q1 mesh {n}^3: structure + slot map")
    A = MooneyRivlinAssembly.from_regular_mesh((n, n, n), device=dev)
    c = torch.tensor([2.0, 6.0], dtype=torch.float64, device=dev)
    dep = torch.from_numpy(stretched_state(A, 1.10, 2.0, 6.0, 0, 0.01)).to(dev)
    R = torch.empty_like(dep)
    E, ndof, nnz = A.n_elements, A.ndof, A.nnz
    res = {}
    with clock_sampler(dev.index) as clk:
        log("timing residual")
        res["residual_ms"] = _events_time(lambda: A.residual(dep, c, out=R, check=False), steps, warmup, stream)
        for prec in ("fp64", "mixed", "tf32x3", "tf32"):
            log(f"timing analytic Jacobian ({prec})")
            res[f"jacobian_{prec}_ms"] = _events_time(lambda: A.jacobian(dep, c, precision=prec, check=False),
                                                      steps, warmup, stream)
            log(f"timing consistent tangent ({prec})")
            res[f"tangent_{prec}_ms"] = _events_time(lambda: A.tangent(dep, c, precision=prec, check=False),
                                                     steps, warmup, stream)
        log("timing Iron's FD Jacobian")
        res["jacobian_fd_ms"] = _events_time(lambda: A.jacobian_fd(dep, c, check=False), max(1, steps // 2), 1,
                                             stream)
        res["jacobian_ms"] = res["jacobian_fp64_ms"]
        # accuracy of the reduced-precision contractions against FP64
        v64 = A.jacobian(dep, c, precision="fp64").clone()
        res_err = {}
        for prec in ("mixed", "tf32x3", "tf32"):
            vmx = A.jacobian(dep, c, precision=prec)
            res_err[prec] = float((vmx - v64).abs().max() / v64.abs().max())
        t64 = A.tangent(dep, c, precision="fp64").clone()
        tan_err = {}
        for prec in ("mixed", "tf32x3"):
            tmx = A.tangent(dep, c, precision=prec)
            tan_err[prec] = float((tmx - t64).abs().max() / t64.abs().max())
        del v64, t64
    _lib.raise_device_errors("bench mr")
    jac_bytes = E * (27 * 4 + 8 * 4) + A.n_q2 * (3 * 8 * 2) + A.n_lin * 8 * 2 + nnz * 8
    res_bytes = E * (27 * 4 + 8 * 4) + A.n_q2 * (3 * 8 * 2) + A.n_lin * 8 * 2 + ndof * 8
    jac_flop = 27 * (2 * 81 * 81 * 9 + 2 * 81 * 36 + 4 * 81 * 8) * E
    return {
        "config": {"workload": "mooney_rivlin_q2p1", "elements_per_side": n, "elements": E, "dofs": ndof,
                   "jacobian_nnz": nnz, "gauss": "3x3x3", "c10": 2.0, "c01": 6.0,
                   "state": "10% uniaxial stretch + N(0,(0.01h)^2), traction-free p"},
        "times_ms": res,
        "jacobian_rel_err_vs_fp64": res_err,
        "tangent_rel_err_vs_fp64": tan_err,
        "elements_per_s": {k.replace("_ms", ""): E / (v * 1e-3) for k, v in res.items()},
        "dofs_per_s": {k.replace("_ms", ""): ndof / (v * 1e-3) for k, v in res.items()},
        "algorithmic": {"jacobian_bytes": jac_bytes, "residual_bytes": res_bytes, "jacobian_flop": jac_flop,
                        "jacobian_GBps": jac_bytes / (res["jacobian_ms"] * 1e-3) / 1e9},
        "clocks": clk.summary(),
    }


def bench_mr(args, log, clock_sampler):
    n = 32 if args.n == 128 else args.n
    r = mr_measure(n, args.steps, args.warmup, clock_sampler, log)
    E = r["config"]["elements"]
    line = {"metric": "mr_jacobian_assembled_elements_per_s", "value": E / (r["times_ms"]["jacobian_ms"] * 1e-3),
            "unit": "elements/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic"}
    line.update(r)
    print(json.dumps(line), flush=True)
    return 0


def mr_adjoint_measure(n: int, B: int, steps: int, warmup: int, clock_sampler, log) -> dict:
    """Residual and its reverse-mode adjoint for B parameter sets on the n^3 Q2/Q1 mesh (c10, c01
    log-uniform in [0.5, 10], displacement perturbation N(0, (0.01 h)^2)), with a directional check
    of one gradient against central differences."""
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    log(f"MR adjoint {n}^3 x {B}")
    A = MooneyRivlinAssembly.from_regular_mesh((n, n, n), device=dev, build_jacobian=False)
    rng = np.random.default_rng(7)
    cs = np.exp(rng.uniform(np.log(0.5), np.log(10.0), (B, 2)))
    deps = np.stack([stretched_state(A, 1.0, cs[b, 0], cs[b, 1], 100 + b, 0.01) for b in range(B)])
    dep = torch.from_numpy(deps).to(dev)
    c = torch.from_numpy(cs).to(dev)
    v = torch.from_numpy(rng.normal(0, 1, deps.shape)).to(dev)
    R = torch.empty_like(dep)
    with clock_sampler(dev.index) as clk:
        fwd = _events_time(lambda: A.residual(dep, c, out=R, check=False), steps, warmup, stream)
        bwd = _events_time(lambda: A.residual_vjp(dep, c, v), steps, warmup, stream)
    _lib.raise_device_errors("bench mr adjoint")
    du, dc = A.residual_vjp(dep[:1], c[:1], v[:1])
    d = torch.from_numpy(rng.normal(0, 1, deps.shape[1])).to(dev)
    h = 1e-6
    Rp = A.residual(dep[0] + h * d, c[0])
    Rm = A.residual(dep[0] - h * d, c[0])
    fd = float((v[0] * (Rp - Rm)).sum() / (2 * h))
    an = float((du[0] * d).sum())
    return {"config": {"workload": "mooney_rivlin_q2p1_adjoint", "elements_per_side": n, "batch": B,
                       "params": "c10,c01 log-uniform [0.5,10] kPa", "perturbation": "N(0,(0.01h)^2)"},
            "forward_ms": fwd, "backward_ms": bwd, "backward_over_forward": bwd / fwd,
            "element_problems_per_s": A.n_elements * B / ((fwd + bwd) * 1e-3),
            "directional_check": {"adjoint": an, "central_fd": fd, "rel_diff": abs(an - fd) / max(abs(fd), 1e-300)},
            "clocks": clk.summary()}


def bench_mr_adjoint(args, log, clock_sampler):
    n = 16 if args.n == 128 else args.n
    r = mr_adjoint_measure(n, 64, args.steps, args.warmup, clock_sampler, log)
    line = {"metric": "mr_residual_adjoint_element_problems_per_s", "value": r["element_problems_per_s"],
            "unit": "element-problems/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic"}
    line.update(r)
    print(json.dumps(line), flush=True)
    return 0


# (name, mesh builder, bench size, CPU sample size, Gauss points per direction or simplex order)
BASES = [
    ("lagrange_q2_hex", "q2", 48, 16, 3),
    ("lagrange_q3_hex", "q3", 24, 10, 4),
    ("hermite_cubic_hex", "hermite", 32, 12, 4),
    ("simplex_p1_tet", "tet1", 96, 48, 1),
    ("simplex_p2_tet", "tet2", 40, 24, 3),
    ("simplex_p3_tet", "tet3", 24, 8, 4),
]
SIMPLEX_POINTS = {1: 1, 2: 4, 3: 5, 4: 11, 5: 14}


def _bases_problem(kind: str, n: int, ng: int, seed: int = 0, device=None):
    """Jittered mesh of side n and its LaplaceAssembly (conductivity log-uniform in [0.1, 10]);
    returns (assembly or None when device is None, interp codes, elem_params, params, scale, kappa)."""
    from . import mesh as M
    from .laplace import LaplaceAssembly

    rng = np.random.default_rng(seed + 1)
    if kind in ("q2", "q3"):
        o = 2 if kind == "q2" else 3
        m = M.RegularMesh((n, n, n), order=o)
        m.jitter_interior(seed)
        kap = np.exp(rng.uniform(np.log(0.1), np.log(10.0), m.n_elements))
        A = LaplaceAssembly.from_regular_mesh(m, kappa=kap, n_gauss=ng, device=device) if device else None
        return A, [o] * 3, m.elem_nodes, m.coords, None, kap
    if kind == "hermite":
        m = M.HermiteMesh((n, n, n), extent=(1.0, 1.0, 1.0), scaling="arc_length")
        m.jitter_interior(seed)
        kap = np.exp(rng.uniform(np.log(0.1), np.log(10.0), m.n_elements))
        A = LaplaceAssembly.from_hermite_mesh(m, kappa=kap, n_gauss=ng, device=device) if device else None
        return A, [4] * 3, m.elem_params, m.params, m.scale, kap
    o = int(kind[-1])
    m = M.TetMesh((n, n, n), order=o)
    m.jitter_interior(seed)
    kap = np.exp(rng.uniform(np.log(0.1), np.log(10.0), m.n_elements))
    A = LaplaceAssembly.from_tet_mesh(m, kappa=kap, n_gauss=ng, device=device) if device else None
    return A, [6 + o] * 3, m.elem_nodes, m.coords, None, kap


def bench_laplace_bases(args, log, clock_sampler, cpu_fn=None):
    """Per basis: assembly time in each precision (CUDA events, inputs resident, values larger
    than L2 except where noted), error against the FP64 assembly, algorithmic flops and bytes,
    the fraction of the FP64-pipe and HBM peaks, and the oracle's rate on a sample of the same
    mesh kind (cpu_fn, supplied by bench.py)."""
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    fp64_peak = _lib.probe_fma_rate(_lib.GFE_FP64)
    hbm_peak, hbm_source = getattr(args, "hbm_peak", (6800.0, "fallback"))
    cases = {}
    with clock_sampler(dev.index) as clk:
        for name, kind, n, n_cpu, ng in BASES:
            log(f"{name}: {n}^3 mesh")
            A, interp, ep, params, scale, kap = _bases_problem(kind, n, ng, device=dev)
            E, nns = ep.shape
            ndof, nnz = params.shape[1], A.nnz
            pts = SIMPLEX_POINTS[ng] if kind.startswith("tet") else ng ** 3
            flop = E * pts * (18 * nns + 45 + 18 * nns + 6 * nns * nns)
            in_bytes = E * (nns * 4 + 8) + ndof * (3 * 8 + 8) + (E * nns * 8 if scale is not None else 0)
            res = {}
            v64 = None
            precs = ("fp64", "mixed_df", "mixed") + (() if kind.startswith("tet") else ("tf32x3",))
            for prec in precs:
                ms = _events_time(lambda: A.assemble(prec, check=False), args.steps, args.warmup, stream)
                A.assemble(prec)
                if prec == "fp64":
                    v64 = A.values.clone()
                    err = 0.0
                else:
                    err = float((A.values - v64).abs().max() / v64.abs().max())
                byts = in_bytes + nnz * (8 if prec == "fp64" else 12)
                res[prec] = {"ms": ms, "elements_per_s": E / (ms * 1e-3), "dofs_per_s": ndof / (ms * 1e-3),
                             "rel_err_vs_fp64": err, "algorithmic_bytes": byts,
                             "hbm_frac": byts / (ms * 1e-3) / 1e9 / hbm_peak,
                             "fp64_equiv_gflops": flop / (ms * 1e-3) / 1e9}
                if prec == "fp64":
                    # only the FP64 kernel runs on the FP64 pipe; the float-float and FP32 kernels run
                    # on the FP32 pipes, where a fraction of the FP64 FMA rate would mean nothing
                    res[prec]["fp64_pipe_frac"] = flop / (ms * 1e-3) / 1e9 / fp64_peak
                else:
                    res[prec]["speedup_vs_fp64"] = res["fp64"]["ms"] / ms
                if prec == "tf32x3":
                    # the contraction K = C B on the tensor cores: 2 nen (3 points) nen flops an element
                    res[prec]["tensor_gflops"] = 2.0 * E * nns * 3 * pts * nns * 3 / (ms * 1e-3) / 1e9
            del v64
            cpu = None
            if cpu_fn is not None:
                _, interp_s, ep_s, params_s, scale_s, kap_s = _bases_problem(kind, n_cpu, ng)
                rate, dt, E_s, threads = cpu_fn(interp_s, [ng] * 3, ep_s, params_s, scale_s, kap_s)
                cpu = {"value": rate, "unit": "elements/s", "cores": threads, "kind": "port",
                       "sample": f"{n_cpu}^3 {kind} mesh = {E_s} elements, one assembly ({dt:.2f} s)"}
            cases[name] = {"elements_per_side": n, "elements": E, "dofs": ndof, "nnz": nnz,
                           "element_dofs": nns, "gauss_points": pts, "flop_per_element": flop // E,
                           "values_MB": nnz * 8 / 1e6, "precisions": res, "cpu_baseline": cpu}
            del A
            torch.cuda.empty_cache()
    _lib.raise_device_errors("bench laplace bases")
    head = cases["lagrange_q2_hex"]["precisions"]["mixed_df"]
    line = {
        "metric": "assembled_elements_per_s", "value": head["elements_per_s"], "unit": "elements/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "dtype": "f64 (float-float element arithmetic)", "data": "synthetic",
        "config": {"workload": "laplace_bases", "headline_case": "lagrange_q2_hex, mixed_df",
                   "conductivity": "log-uniform [0.1,10] seeded", "jitter": "interior nodes, seeded",
                   "l2": "CSR values larger than L2 except simplex_p1_tet (110 MB)"},
        "fp64_pipe_gflops": fp64_peak, "hbm_gbs": hbm_peak, "hbm_peak_source": hbm_source,
        "flop_formula": "E*points*(18*nen + 45 + 18*nen + 6*nen^2)",
        "byte_formula": "E*(nen*4 + 8) + N*(3*8 + 8) [+ E*nen*8 scale factors] + nnz*8 [+ nnz*4 FP32 copy]",
        "cases": cases, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def bench_mr_newton(args, log, clock_sampler):
    """Uniaxial stretch of the Mooney-Rivlin box to lambda = 1.1 in 5 load steps (Iron's increment
    rule), roller conditions, Newton with the consistent tangent and MINRES; FP64 plain against
    mixed precision (tensor-core contraction + FP32 MINRES inside FP64 refinement, FP64 residual)."""
    from .newton import NewtonSolver, uniaxial_exact_state, uniaxial_roller_conditions

    n = 32 if args.n == 128 else args.n
    lam, steps = 1.10, 5
    dev = torch.device("cuda", 0)
    log(f"MR Newton {n}^3: structure + slot map")
    A = MooneyRivlinAssembly.from_regular_mesh((n, n, n), device=dev)
    fixed, full = uniaxial_roller_conditions(A, lam)
    exact = uniaxial_exact_state(A, lam, 2.0, 6.0)
    # untimed warm-up of both arms' code paths on a 4^3 mesh: the first use of a library kernel in a
    # process can take seconds (its code is paged in), which would otherwise land in the first arm
    log("warm-up (4^3, both precisions)")
    Aw = MooneyRivlinAssembly.from_regular_mesh((4, 4, 4), device=dev)
    fw, fullw = uniaxial_roller_conditions(Aw, lam)
    for prec in ("fp64", "mixed"):
        NewtonSolver(Aw, [2.0, 6.0], precision=prec, linear_relative_tolerance=1e-6).solve(
            Aw.initial_state(0.0), fw, fullw, load_increments=1)
    torch.cuda.synchronize()
    del Aw
    res, states = {}, {}
    with clock_sampler(dev.index) as clk:
        for prec in ("fp64", "mixed"):
            dep = A.initial_state(0.0)
            solver = NewtonSolver(A, [2.0, 6.0], precision=prec, absolute_tolerance=1e-12,
                                  relative_tolerance=1e-12, solution_tolerance=0.0,
                                  linear_relative_tolerance=1e-6)
            log(f"Newton ({prec})")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            infos = solver.solve(dep, fixed, full, load_increments=steps,
                                 callback=lambda s, i: log(f"  step {s}: {i.iterations} its, "
                                                           f"|R| {i.residual_norms[-1]:.3e}, "
                                                           f"linear {i.linear_iterations}"))
            torch.cuda.synchronize()
            res[prec] = {"seconds": time.perf_counter() - t0,
                         "newton_iterations": [i.iterations for i in infos],
                         "linear_iterations": [i.linear_iterations for i in infos],
                         "final_residual": infos[-1].residual_norms[-1]}
            states[prec] = dep
    _lib.raise_device_errors("bench mr newton")
    scale = float(states["fp64"].abs().max())
    err_mixed = float((states["mixed"] - states["fp64"]).abs().max()) / scale
    err_exact = {p: float((states[p] - exact).abs().max()) / scale for p in states}
    best = min(res, key=lambda p: res[p]["seconds"])
    E = A.n_elements
    line = {
        "metric": "mr_newton_load_stepped_elements_per_s", "value": E * steps / res[best]["seconds"],
        "unit": "element-load-steps/s", "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": True,
        "dtype": "f64" if best == "fp64" else "f32/f64", "data": "synthetic",
        "config": {"workload": "mooney_rivlin_q2p1_uniaxial_newton", "elements_per_side": n, "elements": E,
                   "dofs": A.ndof, "jacobian_nnz": A.nnz, "lambda": lam, "load_steps": steps, "c10": 2.0,
                   "c01": 6.0, "bcs": "rollers on x=0,y=0,z=0; z1=lambda on x=1",
                   "jacobian": "consistent tangent", "linear_solver": "MINRES + saddle diagonal"},
        "headline_precision": best, "runs": res,
        "mixed_rel_err_vs_fp64": err_mixed, "rel_err_vs_exact": err_exact,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run(args, log, clock_sampler, cpu_bases=None):
    _lib.load()
    if args.workload == "laplace_bases":
        return bench_laplace_bases(args, log, clock_sampler, cpu_bases)
    if args.workload == "mr":
        return bench_mr(args, log, clock_sampler)
    if args.workload == "mr_newton":
        return bench_mr_newton(args, log, clock_sampler)
    if args.workload == "mr_adjoint":
        return bench_mr_adjoint(args, log, clock_sampler)
    if args.workload == "serve":
        from . import serving

        return serving.bench(args, log, clock_sampler)
    raise ValueError(args.workload)
