"""Newton solve of the static finite-elasticity problem with load increments.

This is the caller of the residual and Jacobian kernels on Iron's side:
Problem_SolverEquationsStaticNonlinearSolve drives PETSc SNES (newtonls) through the residual and
Jacobian callbacks (src/problem_routines.F90:1132, 1264, 3801, 4109), and the control loop applies
incremented Dirichlet conditions before each load step
(EQUATIONS_SET_BOUNDARY_CONDITIONS_INCREMENT, src/equations_set_routines.F90:6261-6360).

Defaults mirror Iron's Newton solver (src/solver_routines.F90:17960-18032, 18942-18991):
absolute tolerance 1e-10 and relative tolerance 1e-5 on the residual norm, solution tolerance
1e-5 on the step, 50 iterations, backtracking line search with cubic interpolation and
alpha = 1e-4.  Iron's default Jacobian is its one-sided finite-difference Jacobian
(jacobian="fd", gfe_mr_jacobian_fd, step 1e-6 as Iron's); here the default is the consistent
tangent (the exact derivative of the residual, which the FD Jacobian approximates), and Iron's
analytic Jacobian is selectable (jacobian="analytic").  The linear solve of each Newton step
replaces PETSc KSP: preconditioned MINRES for the consistent tangent (symmetric indefinite) and
restarted GMRES (Iron's default Krylov method) for the FD and analytic Jacobians, which are not
symmetric; all are preconditioned by the diagonal of gfe_saddle_preconditioner.

Precision 'mixed': the Jacobian's basis-gradient contraction on the tensor cores (tcgen05, TF32
in three passes, about FP32 accuracy; `contraction` selects "fp32" for the CUDA-core FP32
contraction or "tf32" for one pass) with FP32 kinematics, and FP32 Krylov iterations (FP32 matrix
copy and vectors) inside FP64 refinement residuals; the nonlinear residual, its norm, the line
search and the convergence test stay in FP64, so the converged state is set by the FP64 residual
alone.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._lib import GfeError


@dataclass
class LinearSolveInfo:
    iterations: int
    relative_residual: float
    nodal: bool = False  # MINRES ran the node-grouped sparse product


def saddle_preconditioner(row_ptr, col_idx, values, n_u: int, fixed=None, out=None, stream=None) -> torch.Tensor:
    """Inverse diagonal preconditioner of a u-p saddle-point matrix (gfe_saddle_preconditioner)."""
    n = row_ptr.numel() - 1
    minv = out if out is not None else torch.empty(n, dtype=torch.float64, device=values.device)
    _lib.call("gfe_saddle_preconditioner", n, int(n_u), _lib.ptr(row_ptr), _lib.ptr(col_idx), _lib.ptr(values),
              _lib.ptr(fixed), _lib.ptr(minv), _lib.stream_handle(stream))
    return minv


def minres_solve(row_ptr, col_idx, values, f, fixed, x, minv=None, values32=None, rtol: float = 1e-5,
                 max_iters: int = 20000, precision: str = "fp64", stream=None, n_node: int = 0,
                 n_comp: int = 3) -> LinearSolveInfo:
    """Solve K x = f (K symmetric, possibly indefinite) with x fixed where fixed != 0 by
    preconditioned MINRES (gfe_minres_solve).  x: Dirichlet values on entry, solution on exit.
    n_node > 0: the first n_comp * n_node rows are a vector field's components in separated
    component order (the u rows of the u-p system, n_node = n_q2); the sparse products then group
    each node's rows (gfe_minres_solve_nodal) where they share a column list."""
    n = row_ptr.numel() - 1
    prec = _lib.GFE_FP64 if precision == "fp64" else _lib.GFE_MIXED
    if prec == _lib.GFE_MIXED and values32 is None:
        raise GfeError(-1, "mixed-precision MINRES needs the FP32 copy of the matrix")
    it = C.c_int32(0)
    rel = C.c_double(0.0)
    v32 = _lib.ptr(values32 if prec == _lib.GFE_MIXED else None)
    if n_node > 0:
        used = C.c_int32(0)
        _lib.call("gfe_minres_solve_nodal", n, int(n_node), int(n_comp), _lib.ptr(row_ptr), _lib.ptr(col_idx),
                  _lib.ptr(values), v32, _lib.ptr(minv), _lib.ptr(f), _lib.ptr(fixed), _lib.ptr(x), float(rtol),
                  int(max_iters), prec, C.byref(it), C.byref(rel), C.byref(used), _lib.stream_handle(stream))
        return LinearSolveInfo(int(it.value), float(rel.value), bool(used.value))
    _lib.call("gfe_minres_solve", n, _lib.ptr(row_ptr), _lib.ptr(col_idx), _lib.ptr(values), v32, _lib.ptr(minv),
              _lib.ptr(f), _lib.ptr(fixed), _lib.ptr(x), float(rtol), int(max_iters), prec, C.byref(it),
              C.byref(rel), _lib.stream_handle(stream))
    return LinearSolveInfo(int(it.value), float(rel.value))


def gmres_solve(row_ptr, col_idx, values, f, fixed, x, minv=None, values32=None, rtol: float = 1e-5,
                max_iters: int = 20000, restart: int = 30, precision: str = "fp64", stream=None) -> LinearSolveInfo:
    """Solve K x = f (K general) with x fixed where fixed != 0 by right-preconditioned restarted
    GMRES (gfe_gmres_solve).  x: Dirichlet values on entry, solution on exit."""
    n = row_ptr.numel() - 1
    prec = _lib.GFE_FP64 if precision == "fp64" else _lib.GFE_MIXED
    if prec == _lib.GFE_MIXED and values32 is None:
        raise GfeError(-1, "mixed-precision GMRES needs the FP32 copy of the matrix")
    it = C.c_int32(0)
    rel = C.c_double(0.0)
    _lib.call("gfe_gmres_solve", n, _lib.ptr(row_ptr), _lib.ptr(col_idx), _lib.ptr(values),
              _lib.ptr(values32 if prec == _lib.GFE_MIXED else None), _lib.ptr(minv), _lib.ptr(f), _lib.ptr(fixed),
              _lib.ptr(x), float(rtol), int(max_iters), int(restart), prec, C.byref(it), C.byref(rel),
              _lib.stream_handle(stream))
    return LinearSolveInfo(int(it.value), float(rel.value))


def increment_dirichlet(current: torch.Tensor, full: torch.Tensor, step: int, n_steps: int) -> torch.Tensor:
    """Iron's incremented Dirichlet value for load step `step` of `n_steps` (1-based):
    current + (full - current) / (n_steps - step + 1), and exactly `full` at the last step
    (src/equations_set_routines.F90:6330-6345)."""
    if step == n_steps:
        return full.clone()
    return current + (full - current) / (n_steps - step + 1)


@dataclass
class NewtonInfo:
    converged: bool
    reason: str
    iterations: int
    residual_norms: list = field(default_factory=list)
    linear_iterations: list = field(default_factory=list)
    line_search_steps: list = field(default_factory=list)
    residual_evaluations: int = 0
    jacobian_evaluations: int = 0
    seconds: dict = field(default_factory=dict)


class NewtonSolver:
    """Newton's method with a backtracking (cubic) line search on R(dep) = 0 for a
    MooneyRivlinAssembly, with Dirichlet DOFs eliminated."""

    def __init__(self, asm, c, *, jacobian: str = "consistent", precision: str = "fp64", contraction: str | None = None,
                 fd_step: float = 1e-6,
                 absolute_tolerance: float = 1e-10, relative_tolerance: float = 1e-5,
                 solution_tolerance: float = 1e-5, maximum_iterations: int = 50, linesearch_alpha: float = 1e-4,
                 linear_relative_tolerance: float = 1e-5, linear_maximum_iterations: int = 50000,
                 linear_solver: str | None = None, gmres_restart: int = 30, stream=None):
        if jacobian not in ("consistent", "analytic", "fd"):
            raise GfeError(-1, f"unknown Jacobian type {jacobian!r} (consistent | analytic | fd)")
        if linear_solver is None:
            linear_solver = "minres" if jacobian == "consistent" else "gmres"
        if linear_solver not in ("minres", "gmres"):
            raise GfeError(-1, f"unknown linear solver {linear_solver!r} (minres | gmres)")
        if linear_solver == "minres" and jacobian != "consistent":
            raise GfeError(-1, f"the {jacobian} Jacobian is not symmetric: use linear_solver='gmres'")
        if precision not in ("fp64", "mixed"):
            raise GfeError(-1, f"unknown precision {precision!r} (fp64 | mixed)")
        if contraction is None:
            contraction = "tf32x3" if precision == "mixed" else "fp64"
        contraction = {"fp32": "mixed"}.get(contraction, contraction)
        if contraction not in ("fp64", "mixed", "tf32x3", "tf32") or (precision == "fp64") != (contraction == "fp64"):
            raise GfeError(-1, f"contraction {contraction!r} does not go with precision {precision!r}")
        if asm.row_ptr is None:
            asm.build_structure(stream)
        self.asm = asm
        self.c = torch.as_tensor(c, dtype=torch.float64, device=asm.device).reshape(2)
        self.jacobian = jacobian
        self.fd_step = float(fd_step)
        self.precision = precision
        self.contraction = contraction
        self.atol = float(absolute_tolerance)
        self.rtol = float(relative_tolerance)
        self.stol = float(solution_tolerance)
        self.max_its = int(maximum_iterations)
        self.alpha = float(linesearch_alpha)
        self.lin_rtol = float(linear_relative_tolerance)
        self.lin_max = int(linear_maximum_iterations)
        self.linear_solver = linear_solver
        self.restart = int(gmres_restart)
        self.stream = stream
        dev = asm.device
        n = asm.ndof
        self._R = torch.empty(n, dtype=torch.float64, device=dev)
        self._Rt = torch.empty(n, dtype=torch.float64, device=dev)
        self._du = torch.empty(n, dtype=torch.float64, device=dev)
        self._trial = torch.empty(n, dtype=torch.float64, device=dev)
        self._minv = torch.empty(n, dtype=torch.float64, device=dev)
        self._values32 = None

    # residual with the Dirichlet rows removed; returns its 2-norm.  A state with a non-positive
    # element Jacobian or a non-finite value is outside the residual's domain: its norm is +inf,
    # so the line search backtracks (PETSc's SNESSetFunctionDomainError behaviour).
    def _residual(self, dep, out, fixed_b) -> float:
        self.asm.residual(dep, self.c, out=out, stream=self.stream, check=False)
        bits = _lib.device_errors(self.stream)
        if bits & ~(_lib.DEVERR_JACOBIAN | _lib.DEVERR_NONFINITE):
            raise GfeError(-3, f"Newton residual: device error bits {bits:#x}")
        if bits:
            return math.inf
        out.masked_fill_(fixed_b, 0.0)
        return float(torch.linalg.vector_norm(out))

    def _linear_solve(self, dep, fixed_u8, info: NewtonInfo):
        asm = self.asm
        if self.jacobian == "consistent":
            vals = asm.tangent(dep, self.c, precision=self.contraction, stream=self.stream)
        elif self.jacobian == "fd":
            vals = asm.jacobian_fd(dep, self.c, step=self.fd_step, stream=self.stream)
        else:
            vals = asm.jacobian(dep, self.c, precision=self.contraction, stream=self.stream)
        info.jacobian_evaluations += 1
        saddle_preconditioner(asm.row_ptr, asm.col_idx, vals, 3 * asm.n_q2, fixed_u8, out=self._minv,
                              stream=self.stream)
        v32 = None
        if self.precision == "mixed":
            if self._values32 is None:
                self._values32 = torch.empty(vals.numel(), dtype=torch.float32, device=vals.device)
            self._values32.copy_(vals)
            v32 = self._values32
        # J du = -R, du = 0 on fixed DOFs
        self._du.zero_()
        torch.neg(self._R, out=self._Rt)
        if self.linear_solver == "minres":
            li = minres_solve(asm.row_ptr, asm.col_idx, vals, self._Rt, fixed_u8, self._du, minv=self._minv,
                              values32=v32, rtol=self.lin_rtol, max_iters=self.lin_max, precision=self.precision,
                              stream=self.stream, n_node=asm.n_q2)
        else:
            li = gmres_solve(asm.row_ptr, asm.col_idx, vals, self._Rt, fixed_u8, self._du, minv=self._minv,
                             values32=v32, rtol=self.lin_rtol, max_iters=self.lin_max, restart=self.restart,
                             precision=self.precision, stream=self.stream)
        info.linear_iterations.append(li.iterations)

    def _line_search(self, dep, fnorm, fixed_b, info: NewtonInfo):
        """Backtracking on f = ||R||^2 / 2 along du: accept lambda when
        f(dep + lambda du) <= f(dep) + alpha lambda slope with slope = -||R||^2 (the Newton direction);
        otherwise a quadratic, then cubic, interpolated step in [0.1, 0.5] lambda."""
        f0 = 0.5 * fnorm * fnorm
        slope = -fnorm * fnorm
        lam, lam_prev, f_prev = 1.0, None, None
        for _ in range(40):
            torch.add(dep, self._du, alpha=lam, out=self._trial)
            fn = self._residual(self._trial, self._Rt, fixed_b)
            info.residual_evaluations += 1
            if not math.isfinite(fn):
                # outside the residual's domain: halve and restart the interpolation
                lam, lam_prev, f_prev = 0.5 * lam, None, None
                if lam < 1e-12:
                    break
                continue
            f1 = 0.5 * fn * fn
            if f1 <= f0 + self.alpha * lam * slope:
                return lam, fn
            if lam_prev is None:
                lt = -slope / (2.0 * (f1 - f0 - slope))
            else:
                t1 = f1 - f0 - lam * slope
                t2 = f_prev - f0 - lam_prev * slope
                d = 1.0 / (lam - lam_prev)
                a = d * (t1 / lam ** 2 - t2 / lam_prev ** 2)
                b = d * (-lam_prev * t1 / lam ** 2 + lam * t2 / lam_prev ** 2)
                if a == 0.0:
                    lt = -slope / (2.0 * b)
                else:
                    disc = max(b * b - 3.0 * a * slope, 0.0)
                    lt = (-b + math.sqrt(disc)) / (3.0 * a)
            lam_prev, f_prev = lam, f1
            lam = min(max(lt, 0.1 * lam), 0.5 * lam)
            if lam < 1e-12:
                break
        raise GfeError(-5, "Newton line search failed to reduce the residual")

    def solve(self, dep: torch.Tensor, fixed: torch.Tensor, full_values: torch.Tensor | None = None,
              load_increments: int = 1, callback=None) -> list[NewtonInfo]:
        """Solve in place.  dep: FP64 dependent vector (the current field values, including the
        current Dirichlet values).  fixed: [ndof] mask of Dirichlet DOFs.  full_values: the full
        Dirichlet values (None: dep's fixed values are final).  Returns one NewtonInfo per load step;
        raises GfeError if a step does not converge."""
        asm = self.asm
        if dep.dtype != torch.float64 or dep.device != asm.device or dep.numel() != asm.ndof:
            raise GfeError(-1, f"dep must be an FP64 [{asm.ndof}] tensor on {asm.device}")
        fixed_u8 = fixed.to(device=asm.device, dtype=torch.uint8).contiguous()
        fixed_b = fixed_u8.bool()
        if full_values is not None:
            full_values = full_values.to(device=asm.device, dtype=torch.float64)
        infos = []
        for step in range(1, load_increments + 1):
            if full_values is not None:
                cur = dep[fixed_b]
                dep[fixed_b] = increment_dirichlet(cur, full_values[fixed_b], step, load_increments)
            info = self._newton(dep, fixed_u8, fixed_b)
            infos.append(info)
            if callback is not None:
                callback(step, info)
            if not info.converged:
                raise GfeError(-5, f"Newton did not converge in load step {step}: {info.reason}")
        return infos

    def _newton(self, dep, fixed_u8, fixed_b) -> NewtonInfo:
        info = NewtonInfo(False, "", 0)
        t0 = time.perf_counter()
        fnorm = self._residual(dep, self._R, fixed_b)
        info.residual_evaluations += 1
        info.residual_norms.append(fnorm)
        fnorm0 = fnorm
        if not math.isfinite(fnorm):
            info.reason = "non-finite residual"
            return info
        if fnorm < self.atol:
            info.converged, info.reason = True, "absolute residual"
            return info
        for it in range(1, self.max_its + 1):
            self._linear_solve(dep, fixed_u8, info)
            lam, fnorm = self._line_search(dep, fnorm, fixed_b, info)
            info.line_search_steps.append(lam)
            # accept the trial state; its residual is in _Rt
            dep.copy_(self._trial)
            self._R, self._Rt = self._Rt, self._R
            info.iterations = it
            info.residual_norms.append(fnorm)
            if fnorm < self.atol:
                info.converged, info.reason = True, "absolute residual"
                break
            if fnorm <= self.rtol * fnorm0:
                info.converged, info.reason = True, "relative residual"
                break
            if self.stol > 0.0:
                snorm = lam * float(torch.linalg.vector_norm(self._du))
                if snorm < self.stol * float(torch.linalg.vector_norm(dep)):
                    info.converged, info.reason = True, "relative step"
                    break
        else:
            info.reason = f"{self.max_its} iterations"
        info.seconds["total"] = time.perf_counter() - t0
        return info


# ---- the homogeneous uniaxial-stretch problem (a known answer) --------------------------------

def uniaxial_roller_conditions(asm, lam: float, tol: float = 1e-12):
    """Dirichlet conditions of a uniaxial stretch of the box [0, X] x [0, Y] x [0, Z]: rollers on the
    three coordinate planes (z_1 = 0 on x = 0, z_2 = 0 on y = 0, z_3 = 0 on z = 0) and z_1 = lam X on
    x = X; the faces y = Y and z = Z are traction free.  Returns (fixed mask, full values)."""
    x = asm.xg.cpu().numpy()
    nq = asm.n_q2
    fixed = np.zeros(asm.ndof, np.uint8)
    vals = np.zeros(asm.ndof)
    ext = x.max(axis=1)
    for comp in range(3):
        on0 = np.abs(x[comp]) <= tol
        fixed[comp * nq:(comp + 1) * nq][on0] = 1
    onX = np.abs(x[0] - ext[0]) <= tol * max(1.0, ext[0])
    fixed[:nq][onX] = 1
    vals[:nq][onX] = lam * x[0][onX]
    dev = asm.device
    return torch.from_numpy(fixed).to(dev), torch.from_numpy(vals).to(dev)


def uniaxial_exact_state(asm, lam: float, c10: float, c01: float) -> torch.Tensor:
    """The exact solution of that problem for the incompressible Mooney-Rivlin material of
    FiniteElasticity_GaussStressTensor (src/finite_elasticity_routines.F90:6985-7110): the
    homogeneous deformation F = diag(lam, lam^-1/2, lam^-1/2) and the uniform pressure that makes the
    lateral stress zero, p = tr(sigma_bar)/3 - sigma_bar_22 with
    sigma_bar = F (2 (c10 + I1 c01) I - 2 c01 C) F^T (J = 1)."""
    F = np.diag([lam, lam ** -0.5, lam ** -0.5])
    Cb = F.T @ F
    S = 2.0 * (c10 + np.trace(Cb) * c01) * np.eye(3) - 2.0 * c01 * Cb
    sb = F @ S @ F.T
    p = np.trace(sb) / 3.0 - sb[1, 1]
    x = asm.xg.cpu().numpy()
    z = x * np.diag(F)[:, None]
    return torch.from_numpy(np.r_[z.ravel(), np.full(asm.n_lin, p)]).to(asm.device)
