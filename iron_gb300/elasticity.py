"""Finite elasticity (Mooney-Rivlin, mixed u-p) residual and Jacobian assembly on the GPU.

`MooneyRivlinAssembly` owns one triquadratic/trilinear (Q2/Q1) mesh on the device: connectivity
of both mesh components, the geometric field, an element colouring, the Iron-identical CSR
structure of the Jacobian (all four components, including the structurally-zero p-p block) and a
per-element slot map into it.  It stands in for Iron's EquationsSet_ResidualEvaluateStaticFEM /
EquationsSet_JacobianEvaluateStaticFEM for the MOONEY_RIVLIN_SUBTYPE equations set.

The dependent vector is Iron's: deformed positions z (3 components over the quadratic nodes),
then the hydrostatic pressure over the linear nodes (separated component order).
"""
from __future__ import annotations

import ctypes as C
import functools

import numpy as np
import torch

from . import _lib
from ._lib import GfeError
from .laplace import csr_structure
from .mesh import RegularMesh, linear_component

# tensor-core contraction of the Jacobian (tcgen05 kind::tf32): three-pass split / one pass
GFE_TC_TF32X3, GFE_TC_TF32 = 3, 4

# Jacobian calculation types, mirroring Iron's CMFE_EQUATIONS_JACOBIAN_*_CALCULATED selectors of
# cmfe_Equations_JacobianCalculationTypeSet (src/opencmiss_iron.F90:25188-25264): "fd" is Iron's
# default for finite elasticity (one-sided differences of the residual), "analytic" Iron's analytic
# Jacobian, "consistent" the exact derivative of the residual (this package's default).
JACOBIAN_TYPES = ("fd", "analytic", "consistent")
FD_STEP_DEFAULT = 1e-6  # Iron's jacobianFiniteDifferenceStepSize default


@functools.lru_cache(maxsize=64)
def _regular_q2_mesh(nelem: tuple, extent: tuple):
    """Host arrays of Iron's regular Q2/Q1 mesh (kept across device-state evictions of a serving
    engine: generating the 64^3 mesh on the host takes about 0.1 s)."""
    m = RegularMesh(nelem, order=2, extent=extent)
    elin, lin2g = linear_component(m.elem_nodes, 2)
    order, ptr = m.colouring()
    return m, elin, lin2g, order, ptr


class MooneyRivlinAssembly:
    def __init__(self, eq2, elin, xg, colour_elems, colour_ptr, n_lin: int, device=None, build_jacobian=True):
        dev = device if device is not None else _lib.require_cuda()
        _lib.load()
        self.device = torch.device(dev)
        eq2 = np.ascontiguousarray(eq2, np.int32)
        elin = np.ascontiguousarray(elin, np.int32)
        xg = np.ascontiguousarray(xg, np.float64)
        if eq2.ndim != 2 or eq2.shape[1] != 27 or elin.shape != (eq2.shape[0], 8):
            raise GfeError(-1, "Q2/Q1 mesh needs eq2 [E][27] and elin [E][8]")
        self.n_elements = eq2.shape[0]
        self.n_q2 = xg.shape[1]
        self.n_lin = int(n_lin)
        self.ndof = 3 * self.n_q2 + self.n_lin
        self.eq2 = torch.from_numpy(eq2).to(self.device)
        self.elin = torch.from_numpy(elin).to(self.device)
        self.xg = torch.from_numpy(xg).to(self.device)
        self.colour_elems = torch.from_numpy(np.ascontiguousarray(colour_elems, np.int32)).to(self.device)
        self.colour_ptr = np.ascontiguousarray(colour_ptr, np.int32)
        nq = self.n_q2
        dofs = np.concatenate([eq2, eq2 + nq, eq2 + 2 * nq, elin + 3 * nq], axis=1)
        self.elem_dofs = torch.from_numpy(np.ascontiguousarray(dofs, np.int32)).to(self.device)
        self.row_ptr = self.col_idx = self.slots = self.values = None
        self.regular = None  # (nx, ny, nz) on Iron's regular generated mesh: closed-form structure
        if build_jacobian:
            self.build_structure()

    @classmethod
    def from_regular_mesh(cls, nelem, extent=(1.0, 1.0, 1.0), device=None, build_jacobian=True):
        m, elin, lin2g, order, ptr = _regular_q2_mesh(tuple(int(v) for v in nelem), tuple(float(v) for v in extent))
        obj = cls(m.elem_nodes, elin, m.coords, order, ptr, len(lin2g), device=device, build_jacobian=False)
        obj.mesh = m
        obj.lin_to_global = lin2g
        obj.regular = tuple(int(v) for v in nelem)
        if build_jacobian:
            obj.build_structure()
        return obj

    def build_structure(self, stream=None):
        """CSR structure (closed form on Iron's regular generated mesh, else sorted from the element
        DOF lists) and the per-element slot map."""
        if getattr(self, "regular", None) is not None:
            nx, ny, nz = self.regular
            rp = torch.empty(self.ndof + 1, dtype=torch.int32, device=self.device)
            nnz = C.c_int64(0)
            st = _lib.stream_handle(stream)
            _lib.call("gfe_mr_regular_structure", nx, ny, nz, _lib.ptr(rp), None, 0, C.byref(nnz), st)
            ci = torch.empty(max(int(nnz.value), 1), dtype=torch.int32, device=self.device)
            _lib.call("gfe_mr_regular_structure", nx, ny, nz, _lib.ptr(rp), _lib.ptr(ci), int(ci.numel()),
                      C.byref(nnz), st)
            self.row_ptr, self.col_idx = rp, ci[: int(nnz.value)]
        else:
            self.row_ptr, self.col_idx = csr_structure(self.elem_dofs, self.ndof, stream)
        self.nnz = int(self.col_idx.numel())
        self.slots = torch.empty((self.n_elements, 89, 89), dtype=torch.int32, device=self.device)
        _lib.call("gfe_mr_slot_map", self.n_elements, _lib.ptr(self.eq2), _lib.ptr(self.elin), self.n_q2,
                  _lib.ptr(self.colour_elems), _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx), _lib.ptr(self.slots),
                  _lib.stream_handle(stream))
        self.values = torch.empty(self.nnz, dtype=torch.float64, device=self.device)

    def initial_state(self, pressure: float = 0.0) -> torch.Tensor:
        """Dependent vector of the undeformed state (z = x) with a uniform pressure."""
        d = torch.empty(self.ndof, dtype=torch.float64, device=self.device)
        d[: 3 * self.n_q2] = self.xg.reshape(-1)
        d[3 * self.n_q2:] = pressure
        return d

    def _cpar(self, c, batch):
        c = torch.as_tensor(c, dtype=torch.float64, device=self.device).reshape(-1, 2)
        if c.shape[0] == 1 and batch > 1:
            c = c.expand(batch, 2)
        return c.contiguous()

    def residual(self, dep: torch.Tensor, c, out: torch.Tensor | None = None, stream=None, check=True):
        """R(dep; c10, c01).  dep: [ndof] or [B][ndof]; c: [2] or [B][2]."""
        dep = dep.to(self.device, torch.float64).contiguous()
        batch = 1 if dep.dim() == 1 else dep.shape[0]
        if dep.numel() != batch * self.ndof:
            raise GfeError(-1, f"dependent vector must have {self.ndof} entries per problem")
        cp = self._cpar(c, batch)
        R = out if out is not None else torch.empty_like(dep)
        cptr = self.colour_ptr
        _lib.call("gfe_mr_residual", self.n_elements, _lib.ptr(self.eq2), _lib.ptr(self.elin), self.n_q2, self.n_lin,
                  _lib.ptr(self.xg), _lib.ptr(self.colour_elems), cptr.ctypes.data_as(C.c_void_p), len(cptr) - 1,
                  batch, _lib.ptr(dep), _lib.ptr(cp), _lib.ptr(R), _lib.stream_handle(stream))
        if check:
            _lib.raise_device_errors("gfe_mr_residual", stream)
        return R

    def _element_jacobians(self, fn: str, dep, c, precision: str, dense: bool, stream, check: bool):
        prec = {"fp64": _lib.GFE_FP64, "mixed": _lib.GFE_MIXED, "tf32x3": GFE_TC_TF32X3, "tf32": GFE_TC_TF32}[precision]
        if not dense and self.slots is None:
            self.build_structure(stream)
        dep = dep.to(self.device, torch.float64).contiguous()
        cp = self._cpar(c, 1)
        cptr = self.colour_ptr
        K = torch.empty((self.n_elements, 89, 89), dtype=torch.float64, device=self.device) if dense else None
        _lib.call(fn, self.n_elements, _lib.ptr(self.eq2), _lib.ptr(self.elin), self.n_q2, self.n_lin,
                  _lib.ptr(self.xg), _lib.ptr(self.colour_elems), cptr.ctypes.data_as(C.c_void_p), len(cptr) - 1,
                  _lib.ptr(dep), _lib.ptr(cp), None if dense else _lib.ptr(self.slots),
                  None if dense else _lib.ptr(self.row_ptr), None if dense else _lib.ptr(self.values),
                  0 if dense else self.nnz, _lib.ptr(K), prec, _lib.stream_handle(stream))
        if check:
            _lib.raise_device_errors(fn, stream)
        return K if dense else self.values

    def jacobian(self, dep: torch.Tensor, c, precision: str = "fp64", stream=None, check=True) -> torch.Tensor:
        """Iron's analytic Jacobian assembled into the CSR values (self.values).  precision 'mixed'
        runs the basis-gradient contraction in FP32 on the CUDA cores, 'tf32x3' / 'tf32' on the
        tensor cores; those three run the Gauss-point kinematics in FP32 with FP64 volume Jacobians.
        The assembled values are FP64 in every mode."""
        return self._element_jacobians("gfe_mr_jacobian", dep, c, precision, False, stream, check)

    def element_jacobians(self, dep: torch.Tensor, c, precision: str = "fp64", stream=None) -> torch.Tensor:
        """Dense element Jacobians [E][89][89] (Iron's analytic form), for parity checks."""
        return self._element_jacobians("gfe_mr_jacobian", dep, c, precision, True, stream, True)

    def tangent(self, dep: torch.Tensor, c, precision: str = "fp64", stream=None, check=True) -> torch.Tensor:
        """Consistent tangent dR/d(dep) assembled into self.values (exact derivative of residual())."""
        return self._element_jacobians("gfe_mr_tangent", dep, c, precision, False, stream, check)

    def element_tangents(self, dep: torch.Tensor, c, precision: str = "fp64", stream=None) -> torch.Tensor:
        return self._element_jacobians("gfe_mr_tangent", dep, c, precision, True, stream, True)

    def jacobian_fd(self, dep: torch.Tensor, c, step: float = FD_STEP_DEFAULT, stream=None, check=True,
                    dense: bool = False) -> torch.Tensor:
        """Iron's finite-difference Jacobian (its default for finite elasticity) assembled into
        self.values, or dense element matrices [E][89][89] with dense=True: column j of every element
        matrix is (R(dep + delta e_j) - R(dep)) / delta with delta = (1 + ||dep||_2) * step
        (src/equations_set_routines.F90:2839-2962).  FP64."""
        if not dense and self.slots is None:
            self.build_structure(stream)
        dep = dep.to(self.device, torch.float64).contiguous()
        cp = self._cpar(c, 1)
        cptr = self.colour_ptr
        K = torch.empty((self.n_elements, 89, 89), dtype=torch.float64, device=self.device) if dense else None
        _lib.call("gfe_mr_jacobian_fd", self.n_elements, _lib.ptr(self.eq2), _lib.ptr(self.elin), self.n_q2,
                  self.n_lin, _lib.ptr(self.xg), _lib.ptr(self.colour_elems), cptr.ctypes.data_as(C.c_void_p),
                  len(cptr) - 1, _lib.ptr(dep), _lib.ptr(cp), float(step), None if dense else _lib.ptr(self.slots),
                  None if dense else _lib.ptr(self.values), 0 if dense else self.nnz, _lib.ptr(K),
                  _lib.stream_handle(stream))
        if check:
            _lib.raise_device_errors("gfe_mr_jacobian_fd", stream)
        return K if dense else self.values

    # -- Iron's Jacobian calculation type selector ---------------------------------------------
    @property
    def jacobian_calculation_type(self) -> str:
        """'fd' | 'analytic' | 'consistent': which Jacobian evaluate_jacobian() assembles
        (cmfe_Equations_JacobianCalculationTypeSet, src/opencmiss_iron.F90:25188-25264)."""
        return getattr(self, "_jac_type", "consistent")

    @jacobian_calculation_type.setter
    def jacobian_calculation_type(self, kind: str) -> None:
        if kind not in JACOBIAN_TYPES:
            raise GfeError(-1, f"Jacobian calculation type must be one of {JACOBIAN_TYPES}, not {kind!r}")
        self._jac_type = kind

    @property
    def jacobian_finite_difference_step_size(self) -> float:
        """Step of the FD Jacobian (cmfe_Equations_JacobianFiniteDifferenceStepSizeSet,
        src/opencmiss_iron.F90:25271-25348); Iron's default 1e-6."""
        return getattr(self, "_fd_step", FD_STEP_DEFAULT)

    @jacobian_finite_difference_step_size.setter
    def jacobian_finite_difference_step_size(self, step: float) -> None:
        if not step > 0.0:
            raise GfeError(-1, "the finite-difference step must be positive")
        self._fd_step = float(step)

    def evaluate_jacobian(self, dep: torch.Tensor, c, precision: str = "fp64", stream=None, check=True,
                          kind: str | None = None) -> torch.Tensor:
        """Assemble the Jacobian of the selected calculation type into self.values.  The FD
        Jacobian is FP64 (differences of FP64 residuals); `precision` applies to the other two."""
        kind = kind or self.jacobian_calculation_type
        if kind == "fd":
            return self.jacobian_fd(dep, c, self.jacobian_finite_difference_step_size, stream, check)
        if kind == "analytic":
            return self.jacobian(dep, c, precision, stream, check)
        if kind == "consistent":
            return self.tangent(dep, c, precision, stream, check)
        raise GfeError(-1, f"Jacobian calculation type must be one of {JACOBIAN_TYPES}, not {kind!r}")

    def residual_vjp(self, dep: torch.Tensor, c, v: torch.Tensor, stream=None):
        """(v^T dR/d dep, v^T dR/d(c10, c01)) for one or a batch of problems."""
        dep = dep.to(self.device, torch.float64).contiguous()
        batch = 1 if dep.dim() == 1 else dep.shape[0]
        cp = self._cpar(c, batch)
        v = v.to(self.device, torch.float64).contiguous()
        du = torch.empty_like(dep)
        dc = torch.empty((batch, 2), dtype=torch.float64, device=self.device)
        cptr = self.colour_ptr
        _lib.call("gfe_mr_residual_vjp", self.n_elements, _lib.ptr(self.eq2), _lib.ptr(self.elin), self.n_q2,
                  self.n_lin, _lib.ptr(self.xg), _lib.ptr(self.colour_elems), cptr.ctypes.data_as(C.c_void_p),
                  len(cptr) - 1, batch, _lib.ptr(dep), _lib.ptr(cp), _lib.ptr(v), _lib.ptr(du), _lib.ptr(dc),
                  _lib.stream_handle(stream))
        return du, dc

    def to_iron_csr(self):
        return self.row_ptr.cpu().numpy(), self.col_idx.cpu().numpy(), self.values.cpu().numpy()


class MooneyRivlinResidual(torch.autograd.Function):
    """R = residual(dep, c) with a hand-written adjoint backward (gfe_mr_residual_vjp).

    forward(asm, dep [B][ndof] or [ndof], c [B][2] or [2]) -> R (same shape as dep); backward
    returns gradients with respect to dep and c."""

    @staticmethod
    def forward(ctx, asm: MooneyRivlinAssembly, dep: torch.Tensor, c: torch.Tensor):
        ctx.asm = asm
        ctx.save_for_backward(dep, c)
        return asm.residual(dep.detach(), c.detach())

    @staticmethod
    def backward(ctx, grad_R):
        dep, c = ctx.saved_tensors
        asm = ctx.asm
        du, dc = asm.residual_vjp(dep.detach(), c.detach(), grad_R.contiguous())
        if dep.dim() == 1:
            du = du.reshape(dep.shape)
        dc = dc.reshape(c.shape) if c.numel() == dc.numel() else dc.sum(0).reshape(c.shape)
        return None, du, dc


def mr_residual(asm: MooneyRivlinAssembly, dep: torch.Tensor, c: torch.Tensor) -> torch.Tensor:
    """Differentiable residual (autograd through the adjoint kernel)."""
    return MooneyRivlinResidual.apply(asm, dep, c)
