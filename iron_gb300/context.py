"""Python handles over the C ABI's context and mesh handles (gfe_ctx, gfe_mesh).

A `Context` owns a CUDA stream binding, its own device error word and a cache of mesh structures
keyed by connectivity; a `MeshHandle` is a trilinear hexahedral mesh registered with it, whose CSR
structure (Iron's, 1-based) and element colouring are built once and shared by every handle of the
same connectivity.  `MeshHandle.assemble_laplace` and `MeshHandle.solve` run the Laplace element
loop and Jacobi-CG on the context's stream and report kernel errors from the context's word.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from ._lib import GfeError

from .laplace import PRECISIONS  # noqa: E402


class Context:
    def __init__(self, stream: torch.cuda.Stream | None = None, device=None):
        dev = device if device is not None else _lib.require_cuda()
        self.device = torch.device(dev)
        self.stream = stream
        _lib.load()
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("gfe_ctx_create", _lib.stream_handle(stream), C.byref(h))
        self.handle = h

    def device_errors(self) -> int:
        bits = C.c_uint32(0)
        with torch.cuda.device(self.device):
            _lib.call("gfe_ctx_device_errors", self.handle, C.byref(bits))
        return int(bits.value)

    def raise_device_errors(self, what: str) -> None:
        bits = self.device_errors()
        if bits:
            names = [n for b, n in ((_lib.DEVERR_SLOT, "missing CSR slot"), (_lib.DEVERR_JACOBIAN,
                                                                                "non-positive Jacobian"),
                                    (_lib.DEVERR_NONFINITE, "non-finite value"),
                                    (_lib.DEVERR_TIMEOUT, "device wait timeout")) if bits & b]
            raise GfeError(-4 if not bits & _lib.DEVERR_SLOT else -3, f"{what}: device reported {', '.join(names)}")

    def cached_meshes(self) -> int:
        n = C.c_int32(0)
        _lib.call("gfe_ctx_cached_meshes", self.handle, C.byref(n))
        return int(n.value)

    def mesh(self, elem_nodes: np.ndarray, n_nodes: int) -> "MeshHandle":
        en = np.ascontiguousarray(elem_nodes, dtype=np.int32)
        if en.ndim != 2:
            raise GfeError(-1, "elem_nodes must be [E][nodes per element]")
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("gfe_mesh_create", self.handle, en.shape[0], en.shape[1], en.ctypes.data_as(C.c_void_p),
                      int(n_nodes), C.byref(h))
        return MeshHandle(self, h, en.shape[0], int(n_nodes))

    def regular_mesh(self, nx: int, ny: int, nz: int) -> "MeshHandle":
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.call("gfe_mesh_create_regular", self.handle, int(nx), int(ny), int(nz), C.byref(h))
        return MeshHandle(self, h, nx * ny * nz, (nx + 1) * (ny + 1) * (nz + 1))

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.call("gfe_ctx_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MeshHandle:
    def __init__(self, ctx: Context, handle, n_elements: int, n_nodes: int):
        self.ctx = ctx
        self.handle = handle
        self.n_elements = n_elements
        self.n_nodes = n_nodes
        rp, ci, nnz, nr = C.c_void_p(), C.c_void_p(), C.c_int64(0), C.c_int32(0)
        _lib.call("gfe_mesh_csr", handle, C.byref(rp), C.byref(ci), C.byref(nnz), C.byref(nr))
        self.nnz = int(nnz.value)
        self._rp, self._ci = rp.value, ci.value

    def csr(self):
        """The cached structure as int32 device tensors (row_ptr, col_idx), 1-based as Iron stores
        them; views of the context's memory, valid while this handle lives."""
        return (_device_view(self._rp, self.n_nodes + 1, self.ctx.device, self),
                _device_view(self._ci, self.nnz, self.ctx.device, self))

    def assemble_laplace(self, coords: torch.Tensor, kappa: torch.Tensor | None, values: torch.Tensor,
                         precision: str = "fp64", values32: torch.Tensor | None = None,
                         rhs: torch.Tensor | None = None, check: bool = True) -> torch.Tensor:
        if values.numel() != self.nnz or values.dtype != torch.float64:
            raise GfeError(-1, f"values must be an FP64 [{self.nnz}] tensor")
        with torch.cuda.device(self.ctx.device):
            _lib.call("gfe_assemble_laplace", self.ctx.handle, self.handle, _lib.ptr(coords), _lib.ptr(kappa),
                      _lib.ptr(values), _lib.ptr(values32), _lib.ptr(rhs), PRECISIONS[precision])
        if check:
            self.ctx.raise_device_errors("gfe_assemble_laplace")
        return values

    def solve(self, values: torch.Tensor, fixed: torch.Tensor, x: torch.Tensor, f: torch.Tensor | None = None,
              rtol: float = 1e-12, max_iters: int = 100000, precision: str = "fp64",
              values32: torch.Tensor | None = None):
        it, rel = C.c_int32(0), C.c_double(0.0)
        with torch.cuda.device(self.ctx.device):
            _lib.call("gfe_solve_laplace", self.ctx.handle, self.handle, _lib.ptr(values), _lib.ptr(values32),
                      _lib.ptr(f), _lib.ptr(fixed), _lib.ptr(x), float(rtol), int(max_iters), PRECISIONS[precision],
                      C.byref(it), C.byref(rel))
        self.ctx.raise_device_errors("gfe_solve_laplace")
        return int(it.value), float(rel.value)

    def close(self) -> None:
        if getattr(self, "handle", None):
            _lib.call("gfe_mesh_destroy", self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _CudaArray:
    """__cuda_array_interface__ of an int32 device array owned by the library."""

    def __init__(self, ptr: int, n: int, owner):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i4", "data": (ptr, False), "version": 3}
        self.owner = owner


def _device_view(ptr: int, n: int, device, owner) -> torch.Tensor:
    with torch.cuda.device(device):
        return torch.as_tensor(_CudaArray(ptr, n, owner), device=device)
