"""Iron's solver system of a linear equations set with Dirichlet conditions, on the GPU.

Iron does not solve the equations matrix itself: SOLVER_MATRICES_STATIC_ASSEMBLE
(src/solver_routines.F90:14025-15050) builds a solver matrix without the rows and columns of
fixed DOFs (structure: SOLVER_MATRIX_STRUCTURE_CALCULATE, src/solver_matrices_routines.F90:
1612-2431; values: SOLVER_MATRIX_EQUATIONS_MATRIX_ADD, :806-1023) and a solver right-hand side
that carries the fixed DOFs' coupling, hands them to PETSc, and copies the solution back into the
dependent field.  `SolverSystem` does the same with the kernels of csrc/dirichlet.cu; structure,
values and right-hand side are bit-identical to Iron's (one equations set, one rank).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from ._lib import GfeError


class SolverSystem:
    """Reduced (solver) system of the equations CSR (row_ptr, col_idx, 1-based, n rows) with the
    Dirichlet DOFs `fixed` (n, nonzero = fixed).

    col_listed (optional, n): the fixed DOFs whose coupling Iron moves to the right-hand side.
    Iron's Dirichlet column lists record only DOFs on boundary nodes
    (src/equations_matrices_routines.F90:4531-4561), so a fixed DOF on an interior node adds no
    right-hand-side term there; pass the boundary-node mask to reproduce that, or None to move
    every fixed DOF's coupling.

    Attributes: n, n_free, nnz, solver_of_dof (n, int32: 0-based solver number or -1), row_ptr
    (n_free + 1) and col_idx (nnz), 1-based."""

    def __init__(self, row_ptr: torch.Tensor, col_idx: torch.Tensor, fixed: torch.Tensor,
                 col_listed: torch.Tensor | None = None, stream=None):
        _lib.load()
        self.device = row_ptr.device
        self.n = int(row_ptr.numel()) - 1
        if self.n <= 0:
            raise GfeError(-1, "the equations matrix has no rows")
        if fixed.numel() != self.n or (col_listed is not None and col_listed.numel() != self.n):
            raise GfeError(-1, f"fixed / col_listed must have {self.n} entries")
        self.eq_row_ptr, self.eq_col_idx = row_ptr, col_idx
        self.fixed = fixed.to(device=self.device, dtype=torch.uint8).contiguous()
        self.col_listed = None if col_listed is None else col_listed.to(device=self.device,
                                                                         dtype=torch.uint8).contiguous()
        self.solver_of_dof = torch.empty(self.n, dtype=torch.int32, device=self.device)
        self.row_ptr = torch.empty(self.n + 1, dtype=torch.int32, device=self.device)
        nf, nnz = C.c_int32(0), C.c_int64(0)
        sh = _lib.stream_handle(stream)
        _lib.call("gfe_solver_structure", self.n, _lib.ptr(row_ptr), _lib.ptr(col_idx), _lib.ptr(self.fixed),
                  _lib.ptr(self.solver_of_dof), _lib.ptr(self.row_ptr), None, 0, C.byref(nf), C.byref(nnz), sh)
        self.n_free, self.nnz = int(nf.value), int(nnz.value)
        self.row_ptr = self.row_ptr[: self.n_free + 1]
        self.col_idx = torch.empty(max(self.nnz, 1), dtype=torch.int32, device=self.device)
        _lib.call("gfe_solver_structure", self.n, _lib.ptr(row_ptr), _lib.ptr(col_idx), _lib.ptr(self.fixed),
                  _lib.ptr(self.solver_of_dof), _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx), self.nnz,
                  C.byref(nf), C.byref(nnz), sh)
        self.col_idx = self.col_idx[: self.nnz]

    def matrix(self, values: torch.Tensor, fp32: bool = False, stream=None):
        """Solver matrix values (FP64, nnz) from the equations matrix values; with fp32=True also
        their FP32 roundings.  Returns values or (values, values32)."""
        v = torch.empty(max(self.nnz, 1), dtype=torch.float64, device=self.device)
        v32 = torch.empty(max(self.nnz, 1), dtype=torch.float32, device=self.device) if fp32 else None
        if self.n_free > 0:
            _lib.call("gfe_solver_matrix", self.n, _lib.ptr(self.eq_row_ptr), _lib.ptr(self.eq_col_idx),
                      _lib.ptr(values), _lib.ptr(self.solver_of_dof), _lib.ptr(self.row_ptr), _lib.ptr(v),
                      _lib.ptr(v32), _lib.stream_handle(stream))
        v = v[: self.nnz]
        return (v, v32[: self.nnz]) if fp32 else v

    def rhs(self, values: torch.Tensor, u: torch.Tensor, f: torch.Tensor | None = None, stream=None):
        """Solver right-hand side (n_free) from the equations matrix values, the dependent vector u
        (Dirichlet values at fixed DOFs) and the equations right-hand side f (None = zero)."""
        out = torch.empty(max(self.n_free, 1), dtype=torch.float64, device=self.device)
        if self.n_free > 0:
            _lib.call("gfe_solver_rhs", self.n, _lib.ptr(self.eq_row_ptr), _lib.ptr(self.eq_col_idx),
                      _lib.ptr(values), _lib.ptr(f), _lib.ptr(u), _lib.ptr(self.fixed), _lib.ptr(self.col_listed),
                      _lib.ptr(self.solver_of_dof), _lib.ptr(out), _lib.stream_handle(stream))
        return out[: self.n_free]

    def update_dependent(self, x: torch.Tensor, u: torch.Tensor, stream=None) -> torch.Tensor:
        """u[i] = x[solver number of i] for every free DOF i (fixed DOFs keep their values)."""
        if self.n_free > 0:
            _lib.call("gfe_solver_update_dependent", self.n, _lib.ptr(self.solver_of_dof), _lib.ptr(x), _lib.ptr(u),
                      _lib.stream_handle(stream))
        return u

    def to_iron_csr(self, values: torch.Tensor):
        """Host copy (row_ptr, col_idx, values) of the solver matrix as Iron stores it (1-based)."""
        return self.row_ptr.cpu().numpy(), self.col_idx.cpu().numpy(), values.cpu().numpy()
