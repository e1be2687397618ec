"""Laplace / diffusion assembly and solve on the GPU (the classical-field half of the hot path).

`LaplaceAssembly` owns, for one mesh, the device-resident connectivity, geometry, colouring and
the Iron-identical CSR structure, and assembles the global stiffness matrix with libgfe's fused
element + scatter kernels.  It stands in for EquationsSet_AssembleStaticLinearFEM
(src/equations_set_routines.F90:1203-1364) for the Laplace equations set; `solve` stands in for
the static linear solve (src/problem_routines.F90:2533 -> PETSc KSP).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import GFE_FP64, GFE_MIXED, GfeError

GFE_MIXED_DF = 2
GFE_TC_TF32X3 = 3
# fp64: FP64 element arithmetic; mixed: FP32 element arithmetic (about 1e-6 relative), FP64
# accumulation; mixed_df: float-float element arithmetic on the FP32 pipes (FP64-level accuracy);
# tf32x3 (hexahedral bases of the basis-generic path): the element contraction on the tensor cores
# (tcgen05, three TF32 products, about FP32 accuracy)
PRECISIONS = {"fp64": GFE_FP64, "mixed": GFE_MIXED, "mixed_df": GFE_MIXED_DF, "tf32x3": GFE_TC_TF32X3}


def csr_structure(elem_dofs: torch.Tensor, n_dofs: int, stream=None):
    """Iron-identical CSR structure (1-based) of an FEM matrix on the GPU.  K3."""
    elem_dofs = elem_dofs.to(torch.int32).contiguous()
    E, ndpe = elem_dofs.shape
    dev = elem_dofs.device
    rp = torch.empty(n_dofs + 1, dtype=torch.int32, device=dev)
    nnz = C.c_int64(0)
    st = _lib.stream_handle(stream)
    _lib.call("gfe_csr_structure", E, ndpe, _lib.ptr(elem_dofs), n_dofs, _lib.ptr(rp), None, 0, C.byref(nnz), st)
    ci = torch.empty(max(int(nnz.value), 1), dtype=torch.int32, device=dev)
    _lib.call("gfe_csr_structure", E, ndpe, _lib.ptr(elem_dofs), n_dofs, _lib.ptr(rp), _lib.ptr(ci),
              int(ci.numel()), C.byref(nnz), st)
    return rp, ci[: int(nnz.value)]


@dataclass
class SolveInfo:
    iterations: int
    relative_residual: float
    precision: str


class LaplaceAssembly:
    """Device-resident Laplace problem on a hexahedral mesh of tensor-product Lagrange elements.

    elem_nodes: [E][nns] int (0-based, Iron local node order, xi1 fastest); coords: [3][N] float64;
    kappa: [E] element conductivity or None (standard Laplace subtype);
    colour_elems / colour_ptr: an element colouring (elements of one colour share no node);
    order: Iron's interpolation per direction (an int or three): 1..3 = Lagrange of that order,
    4 = cubic Hermite; an element has prod(order + 1) parameters for Lagrange directions and 4 per
    Hermite direction (2 nodes x value and slope); 7 / 8 = linear / quadratic tetrahedra (4 / 10
    nodes in Iron's order, n_gauss = the Gauss_Simplex order 1..3);
    n_gauss: Gauss points per direction (1..4; default order + 1, 4 for Hermite);
    scale: [E][nns] element parameter scale factors (Hermite arc-length scaling) or None.
    For Hermite meshes elem_nodes holds element parameter DOFs and coords the geometric parameters
    per DOF (positions and derivatives).
    Trilinear elements with 2x2x2 Gauss points use the sum-factorised kernels (and, on Iron's
    regular generated mesh, the row-owning one); every other basis uses gfe_laplace_assemble_tp.
    slot_map: for the basis-generic path, compute the element slot map (the CSR position of every
    element entry, gfe_laplace_tp_slot_map) once and pass it to every assembly instead of Iron's
    per-entry row search; default for elements of 20 or more nodes (4 nns^2 bytes an element).
    """

    def __init__(self, elem_nodes, coords, kappa=None, colour_elems=None, colour_ptr=None, device=None,
                 structure=None, order=1, n_gauss=None, scale=None, slot_map=None):
        dev = device if device is not None else _lib.require_cuda()
        _lib.load()
        self.device = torch.device(dev)
        self.order = tuple(int(o) for o in (order if np.ndim(order) else (order,) * 3))
        simplex = self.order[0] in (7, 8, 9)
        if simplex:
            # tetrahedra: one simplex interpolation, n_gauss = Gauss_Simplex order (default: exact
            # for straight-sided elements, 1 for linear, 2 for quadratic, 4 for cubic)
            q = int(n_gauss if n_gauss is not None and not np.ndim(n_gauss) else
                    (n_gauss[0] if n_gauss is not None else {7: 1, 8: 2, 9: 4}[self.order[0]]))
            self.n_gauss = (q, q, q)
            nns = {7: 4, 8: 10, 9: 20}[self.order[0]]
        else:
            self.n_gauss = tuple(int(g) for g in (n_gauss if n_gauss is not None and np.ndim(n_gauss) else
                                                  ((n_gauss,) * 3 if n_gauss is not None else
                                                   [min(o + 1, 4) for o in self.order])))
            nns = int(np.prod([4 if o == 4 else o + 1 for o in self.order]))
        self.tensor_product = self.order != (1, 1, 1) or self.n_gauss != (2, 2, 2)
        en = np.ascontiguousarray(elem_nodes, dtype=np.int32)
        if en.ndim != 2 or en.shape[1] != nns:
            raise GfeError(-1, f"Lagrange order {self.order} needs [E][{nns}] connectivity")
        xyz = np.ascontiguousarray(coords, dtype=np.float64)
        if xyz.ndim != 2 or xyz.shape[0] != 3:
            raise GfeError(-1, "coords must be [3][N] (separated components)")
        self.n_elements = en.shape[0]
        self.n_nodes = xyz.shape[1]
        if en.size and (en.min() < 0 or en.max() >= self.n_nodes):
            raise GfeError(-1, "connectivity refers to a node outside coords")
        if colour_elems is None:
            from .mesh import greedy_colouring
            colour_elems, colour_ptr = greedy_colouring(en, self.n_nodes)
        self.colour_ptr = np.ascontiguousarray(colour_ptr, dtype=np.int32)
        self.elem_nodes = torch.from_numpy(en).to(self.device)
        self.coords = torch.from_numpy(xyz).to(self.device)
        self.kappa = None if kappa is None else torch.as_tensor(np.asarray(kappa, np.float64)).to(self.device)
        if scale is not None:
            scale = np.ascontiguousarray(scale, dtype=np.float64)
            if scale.shape != en.shape:
                raise GfeError(-1, f"scale factors must be [E][{nns}] like the element parameters")
            self.tensor_product = True
        self.scale = None if scale is None else torch.from_numpy(scale).to(self.device)
        self.colour_elems = torch.from_numpy(np.ascontiguousarray(colour_elems, dtype=np.int32)).to(self.device)
        if structure is None:
            self.row_ptr, self.col_idx = csr_structure(self.elem_nodes, self.n_nodes)
        else:
            self.row_ptr, self.col_idx = structure
        self.nnz = int(self.col_idx.numel())
        self.values = torch.empty(self.nnz, dtype=torch.float64, device=self.device)
        self.values32 = None
        self.rhs = torch.empty(self.n_nodes, dtype=torch.float64, device=self.device)
        self.regular = None  # (nx, ny, nz) when the mesh is Iron's trilinear regular generated mesh
        self.grid = None     # (nelem, order) of a regular generated mesh of any order
        self.nns = nns
        self._want_slots = (nns >= 20 if slot_map is None else bool(slot_map)) and self.nnz < 2 ** 31
        self.tp_slots = None  # [E][nns][nns] CSR positions (basis-generic path), built on first use

    @classmethod
    def from_tet_mesh(cls, mesh, kappa=None, device=None, n_gauss=None):
        """Tetrahedral mesh (iron_gb300.mesh.TetMesh), greedy element colouring."""
        return cls(mesh.elem_nodes, mesh.coords, kappa=kappa, device=device, order=6 + mesh.order, n_gauss=n_gauss)

    @classmethod
    def from_hermite_mesh(cls, mesh, kappa=None, device=None, n_gauss=4):
        """Tricubic Hermite mesh (iron_gb300.mesh.HermiteMesh): parameters per DOF and, with
        arc-length scaling, its scale factors."""
        order, ptr = mesh.colouring()
        return cls(mesh.elem_params, mesh.params, kappa=kappa, colour_elems=order, colour_ptr=ptr, device=device,
                   order=4, n_gauss=n_gauss, scale=mesh.scale)

    @classmethod
    def from_regular_mesh(cls, mesh, kappa=None, device=None, n_gauss=None, slot_map=None):
        order, ptr = mesh.colouring()
        obj = cls(mesh.elem_nodes, mesh.coords, kappa=kappa, colour_elems=order, colour_ptr=ptr, device=device,
                  order=mesh.order, n_gauss=n_gauss, slot_map=slot_map)
        obj.grid = (tuple(mesh.nelem), mesh.order)
        if mesh.order == 1 and not obj.tensor_product:
            nx, ny, nz = mesh.nelem
            bad = C.c_int64(-1)
            _lib.call("gfe_laplace_regular_check", nx, ny, nz, _lib.ptr(obj.row_ptr), _lib.ptr(obj.col_idx),
                      C.byref(bad), _lib.stream_handle())
            if bad.value == 0:
                obj.regular = (nx, ny, nz)
        return obj

    def assemble(self, precision: str = "fp64", stream=None, check: bool = True, path: str = "auto",
                 fp32_copy: bool | None = None) -> torch.Tensor:
        """Assemble K into self.values (FP64).  path: 'auto' (regular-mesh kernel when the mesh is
        Iron's regular generated mesh, else the colour-scatter kernel), 'regular' or 'general'.
        fp32_copy (default: for the mixed precisions) also fills self.values32."""
        prec = PRECISIONS[precision]
        if fp32_copy is None:
            fp32_copy = prec != GFE_FP64
        if fp32_copy and self.values32 is None:
            self.values32 = torch.empty(self.nnz, dtype=torch.float32, device=self.device)
        v32 = self.values32 if fp32_copy else None
        if self.tensor_product:
            if path == "regular":
                raise GfeError(-1, "the regular-mesh kernel is trilinear with 2x2x2 Gauss points")
            if self._want_slots and self.tp_slots is None and self.n_elements > 0:
                self.tp_slots = torch.empty((self.n_elements, self.nns, self.nns), dtype=torch.int32,
                                            device=self.device)
                _lib.call("gfe_laplace_tp_slot_map", self.n_elements, self.nns, _lib.ptr(self.elem_nodes),
                          _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx), self.nnz, _lib.ptr(self.tp_slots),
                          _lib.stream_handle(stream))
            cp = self.colour_ptr
            _lib.call("gfe_laplace_assemble_tp", (C.c_int32 * 3)(*self.order), (C.c_int32 * 3)(*self.n_gauss),
                      self.n_elements, self.n_nodes, _lib.ptr(self.elem_nodes), _lib.ptr(self.coords),
                      _lib.ptr(self.scale), _lib.ptr(self.kappa), _lib.ptr(self.colour_elems),
                      cp.ctypes.data_as(C.c_void_p), len(cp) - 1,
                      _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx), self.nnz, _lib.ptr(self.tp_slots),
                      _lib.ptr(self.values), _lib.ptr(v32), _lib.ptr(self.rhs), prec, _lib.stream_handle(stream))
            if check:
                _lib.raise_device_errors("gfe_laplace_assemble_tp", stream)
            return self.values
        if path == "regular" and self.regular is None:
            raise GfeError(-1, "the regular-mesh kernel needs Iron's regular generated mesh")
        if path == "auto":
            # FP64 element arithmetic is bound by GB300's FP64 pipe: the colour kernel computes each
            # element once, while the tiled kernel recomputes its halo elements.  The FP32-pipe
            # precisions are bound by memory traffic, which the tiled kernel minimises.
            path = "general" if (prec == GFE_FP64 or self.regular is None) else "regular"
        if path == "regular":
            nx, ny, nz = self.regular
            ws = self._regular_workspace(prec) if prec != GFE_FP64 else None
            _lib.call("gfe_laplace_assemble_regular_ws", nx, ny, nz, _lib.ptr(self.coords), _lib.ptr(self.kappa),
                      _lib.ptr(self.row_ptr), _lib.ptr(self.values), _lib.ptr(v32), _lib.ptr(self.rhs), prec,
                      _lib.ptr(ws), _lib.stream_handle(stream))
        else:
            cp = self.colour_ptr
            _lib.call("gfe_laplace_assemble", self.n_elements, self.n_nodes, _lib.ptr(self.elem_nodes),
                      _lib.ptr(self.coords), _lib.ptr(self.kappa), _lib.ptr(self.colour_elems),
                      cp.ctypes.data_as(C.c_void_p), len(cp) - 1, _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx),
                      self.nnz, _lib.ptr(self.values), _lib.ptr(v32), _lib.ptr(self.rhs), prec,
                      _lib.stream_handle(stream))
        if check:
            _lib.raise_device_errors("gfe_laplace_assemble", stream)
        return self.values

    def assemble_generalised(self, conductivity, fibre=None, stream=None, check: bool = True) -> torch.Tensor:
        """Generalised Laplace (gfe_laplace_assemble_generalised): assemble K into self.values (FP64)
        with a full conductivity tensor per element in a material frame.  conductivity [6][n_elements]
        (K11 K22 K33 K12 K23 K13 in material coordinates); fibre [n_angles][n_nodes] nodal fibre,
        imbrication and sheet angles in radians (1 to 3 rows) or None for no fibre field.  Trilinear
        hexahedra only; the matrix is not symmetric in general."""
        if self.tensor_product:
            raise GfeError(-1, "the generalised Laplace kernel is for trilinear hexahedra")
        cond = torch.as_tensor(conductivity, dtype=torch.float64).to(self.device).contiguous()
        if cond.shape != (6, self.n_elements):
            raise GfeError(-1, f"conductivity must be [6][{self.n_elements}], got {tuple(cond.shape)}")
        fib, n_ang = None, 0
        if fibre is not None:
            fib = torch.as_tensor(fibre, dtype=torch.float64).to(self.device).contiguous()
            if fib.dim() != 2 or fib.shape[1] != self.n_nodes or not 1 <= fib.shape[0] <= 3:
                raise GfeError(-1, f"fibre must be [1..3][{self.n_nodes}], got {tuple(fib.shape)}")
            n_ang = fib.shape[0]
        cp = self.colour_ptr
        _lib.call("gfe_laplace_assemble_generalised", self.n_elements, self.n_nodes, _lib.ptr(self.elem_nodes),
                  _lib.ptr(self.coords), _lib.ptr(cond), _lib.ptr(fib), n_ang, _lib.ptr(self.colour_elems),
                  cp.ctypes.data_as(C.c_void_p), len(cp) - 1, _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx),
                  self.nnz, _lib.ptr(self.values), _lib.ptr(self.rhs), _lib.stream_handle(stream))
        if check:
            _lib.raise_device_errors("gfe_laplace_assemble_generalised", stream)
        return self.values

    def assemble_to_host(self, values_host: torch.Tensor, precision: str = "mixed_df", coords_host=None,
                         kappa_host=None, slab_layers: int = 16, stream=None) -> torch.Tensor:
        """End-to-end assembly with host buffers on Iron's regular generated mesh
        (gfe_laplace_assemble_regular_host): the geometry and conductivity are copied in from the
        pinned host tensors coords_host [3][N] / kappa_host [n_elements] (optional: None keeps the
        device copies), assembled in node-layer slabs (8 layers first, then slab_layers each, a
        multiple of 8), and each slab's CSR values, one contiguous range, are copied to values_host
        (pinned float64 [nnz]) while later slabs compute.  Inputs are uploaded and converted slab
        by slab, so the first copy-out starts after one 8-layer slab.  Returns values_host; all
        work is ordered before later work on `stream`."""
        if self.regular is None:
            raise GfeError(-1, "the slab pipeline needs Iron's regular generated mesh")
        if values_host.numel() != self.nnz or values_host.dtype != torch.float64 or values_host.is_cuda:
            raise GfeError(-1, f"values_host must be a host float64 tensor of {self.nnz} entries")
        for name, h, d in (("coords_host", coords_host, self.coords), ("kappa_host", kappa_host, self.kappa)):
            if h is None:
                continue
            if d is None or h.is_cuda or h.dtype != torch.float64 or h.numel() != d.numel() or not h.is_contiguous():
                raise GfeError(-1, f"{name} must be a contiguous host float64 tensor like the device copy")
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        L = _lib.load()
        nx, ny, nz = self.regular
        prec = PRECISIONS[precision]
        ws = self._regular_workspace(prec)
        _lib.call("gfe_laplace_assemble_regular_host", nx, ny, nz, _lib.host_ptr(coords_host),
                  _lib.host_ptr(kappa_host), _lib.ptr(self.coords), _lib.ptr(self.kappa), _lib.ptr(self.row_ptr),
                  _lib.ptr(self.values), _lib.host_ptr(values_host), _lib.ptr(self.rhs), prec, _lib.ptr(ws),
                  int(slab_layers), _lib.stream_handle(st))
        return values_host

    def _regular_workspace(self, prec: int) -> torch.Tensor:
        """Device workspace of the regular-mesh kernels for precision code `prec`, allocated once per
        precision and kept (the float-float one also holds every element's Gauss-point metrics and
        element matrix: 672 bytes an element)."""
        cache = self.__dict__.setdefault("_ws_cache", {})
        if prec not in cache:
            nx, ny, nz = self.regular
            wb = int(_lib.load().gfe_laplace_regular_workspace_bytes(nx, ny, nz, prec))
            cache[prec] = torch.empty(max(wb, 16), dtype=torch.uint8, device=self.device)
        return cache[prec]

    def element_matrices(self, precision: str = "fp64", stream=None) -> torch.Tensor:
        if self.tensor_product:
            raise GfeError(-1, "element matrices are available for trilinear elements with 2x2x2 Gauss points")
        K = torch.empty((self.n_elements, 8, 8), dtype=torch.float64, device=self.device)
        _lib.call("gfe_laplace_element_matrices", self.n_elements, self.n_nodes, _lib.ptr(self.elem_nodes),
                  _lib.ptr(self.coords), _lib.ptr(self.kappa), _lib.ptr(K), PRECISIONS[precision],
                  _lib.stream_handle(stream))
        return K

    def spmv(self, x: torch.Tensor, fixed: torch.Tensor | None = None, stream=None) -> torch.Tensor:
        y = torch.empty_like(x)
        _lib.call("gfe_csr_spmv", self.n_nodes, _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx),
                  _lib.ptr(self.values), _lib.ptr(x.contiguous()), _lib.ptr(y), _lib.ptr(fixed),
                  _lib.stream_handle(stream))
        return y

    def solve(self, fixed: torch.Tensor, x: torch.Tensor, f: torch.Tensor | None = None, rtol: float = 1e-12,
              max_iters: int = 200000, precision: str = "fp64", stream=None) -> SolveInfo:
        """Solve K x = f with x fixed (Dirichlet) where fixed != 0; x holds the fixed values on
        entry and the solution on exit.  precision 'fp64': FP64 CG; 'mixed' / 'mixed_df': FP32 CG on
        self.values32 inside FP64 iterative refinement with the FP64 matrix."""
        prec = GFE_FP64 if precision == "fp64" else GFE_MIXED
        if prec == GFE_MIXED and self.values32 is None:
            raise GfeError(-1, "mixed-precision solve needs the FP32 copy (assemble with fp32_copy=True)")
        fixed = fixed.to(device=self.device, dtype=torch.uint8).contiguous()
        it = C.c_int32(0)
        rel = C.c_double(0.0)
        _lib.call("gfe_cg_solve", self.n_nodes, _lib.ptr(self.row_ptr), _lib.ptr(self.col_idx),
                  _lib.ptr(self.values), _lib.ptr(self.values32 if prec == GFE_MIXED else None), _lib.ptr(f),
                  _lib.ptr(fixed), _lib.ptr(x), float(rtol), int(max_iters), prec, C.byref(it), C.byref(rel),
                  _lib.stream_handle(stream))
        return SolveInfo(int(it.value), float(rel.value), precision)

    def solver_system(self, fixed: torch.Tensor, col_listed="boundary", stream=None):
        """Iron's solver system (Dirichlet DOFs `fixed` removed, their coupling moved to the
        right-hand side) for this matrix structure; see iron_gb300.solver_system.SolverSystem.
        col_listed: "boundary" (the fixed DOFs on boundary nodes, as Iron's Dirichlet column lists
        record them; on Iron's regular generated mesh), None (all fixed DOFs) or a mask."""
        from .mesh import boundary_node_mask
        from .solver_system import SolverSystem

        if isinstance(col_listed, str):
            if col_listed != "boundary":
                raise GfeError(-1, f"unknown col_listed {col_listed!r}")
            if self.grid is None:
                raise GfeError(-1, "col_listed='boundary' needs Iron's regular generated mesh; pass a mask")
            nelem, order = self.grid
            col_listed = torch.from_numpy(boundary_node_mask(nelem, order).astype("uint8")).to(self.device)
        return SolverSystem(self.row_ptr, self.col_idx, fixed, col_listed, stream=stream)

    def solve_reduced(self, fixed: torch.Tensor, x: torch.Tensor, f: torch.Tensor | None = None, rtol: float = 1e-12,
                      max_iters: int = 200000, precision: str = "fp64", system=None, stream=None) -> SolveInfo:
        """Iron's solve path: build the solver system (SOLVER_MATRICES_STATIC_ASSEMBLE), solve it by
        Jacobi-preconditioned CG (FP64, or FP32 inner solves inside FP64 refinement for the mixed
        precisions), and copy the solution into the free DOFs of x (the dependent-field update).
        x holds the Dirichlet values at fixed DOFs on entry.  system: a SolverSystem of `fixed` to
        reuse (its structure is built once per set of fixed DOFs)."""
        S = system if system is not None else self.solver_system(fixed, stream=stream)
        prec = GFE_FP64 if precision == "fp64" else GFE_MIXED
        if prec == GFE_MIXED:
            sv, sv32 = S.matrix(self.values, fp32=True, stream=stream)
        else:
            sv, sv32 = S.matrix(self.values, stream=stream), None
        b = S.rhs(self.values, x, f, stream=stream)
        xs = torch.zeros(max(S.n_free, 1), dtype=torch.float64, device=self.device)
        it = C.c_int32(0)
        rel = C.c_double(0.0)
        if S.n_free > 0:
            _lib.call("gfe_cg_solve", S.n_free, _lib.ptr(S.row_ptr), _lib.ptr(S.col_idx), _lib.ptr(sv), _lib.ptr(sv32),
                      _lib.ptr(b), None, _lib.ptr(xs), float(rtol), int(max_iters), prec, C.byref(it), C.byref(rel),
                      _lib.stream_handle(stream))
            S.update_dependent(xs, x, stream=stream)
        return SolveInfo(int(it.value), float(rel.value), precision)

    def to_iron_csr(self):
        """Host copy of the CSR matrix exactly as Iron stores it: (row_ptr 1-based, col_idx 1-based,
        values).  Analogue of cmfe_DistributedMatrix_StorageLocationsGet / DataGet
        (src/opencmiss_iron.F90:45823, :45903)."""
        return (self.row_ptr.cpu().numpy(), self.col_idx.cpu().numpy(), self.values.cpu().numpy())
