"""Parity oracle: ctypes bindings of the C++ restatement of Iron's FE assembly hot path.

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py as the checker; the product package iron_gb300 never imports it.

Parity pins: see tests/test_oracle_golden.py (Iron's analytic-Laplace fixture, known-answer
tests).  The linear solve (PETSc KSP in Iron) is not restated and is parity-unpinned.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import build as _build

_HERE = Path(__file__).resolve().parent
_libs = {}
_variant = "parity"


def use_build(variant: str) -> str:
    """Select the library behind every oracle call: "parity" (no FMA contraction, bit-stable across
    hosts; the default) or "timing" (the compiler's default contraction, for the CPU baseline).
    Returns the previous selection."""
    global _variant
    if variant not in ("parity", "timing"):
        raise ValueError(variant)
    prev, _variant = _variant, variant
    return prev

i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def lib():
    if _variant not in _libs:
        _build.build()
        path = _build.LIB if _variant == "parity" else _build.LIB_TIMING
        L = C.CDLL(str(path))
        L.orc_gauss_legendre.argtypes = [C.c_int, f64p, f64p]
        L.orc_tp_basis.argtypes = [C.c_int, i32p, i32p, C.c_void_p, C.c_void_p]
        L.orc_regular_mesh.argtypes = [C.c_int, i32p, C.c_int, i32p]
        L.orc_regular_coords.argtypes = [C.c_int, i32p, C.c_int, f64p, f64p, f64p]
        L.orc_linear_component.argtypes = [C.c_int, C.c_int, C.c_int, i32p, i32p, i32p, i32p]
        L.orc_csr_structure.argtypes = [C.c_int, C.c_int, i32p, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_csr_structure.restype = C.c_int64
        L.orc_csr_location.argtypes = [i32p, i32p, C.c_int, C.c_int]
        L.orc_csr_location.restype = C.c_int64
        L.orc_laplace_element.argtypes = [C.c_int, i32p, i32p, C.c_int, f64p, C.c_double, f64p]
        L.orc_laplace_assemble.argtypes = [C.c_int, i32p, i32p, C.c_int, C.c_int, i32p, f64p, C.c_void_p,
                                           i32p, i32p, f64p, C.c_void_p, C.c_int]
        L.orc_laplace_assemble_scaled.argtypes = [C.c_int, i32p, i32p, C.c_int, C.c_int, i32p, f64p, C.c_void_p,
                                                  C.c_void_p, i32p, i32p, f64p, C.c_void_p, C.c_int]
        L.orc_laplace_generalised_element.argtypes = [C.c_int, i32p, i32p, f64p, f64p, C.c_void_p, C.c_int, f64p]
        L.orc_laplace_generalised_assemble.argtypes = [C.c_int, i32p, i32p, C.c_int, C.c_int, i32p, f64p, f64p,
                                                       C.c_void_p, C.c_int, i32p, i32p, f64p, C.c_void_p]
        L.orc_csr_spmv.argtypes = [C.c_int, i32p, i32p, f64p, f64p, f64p]
        L.orc_solver_system.argtypes = [C.c_int, i32p, i32p, f64p, C.c_void_p, u8p, C.c_void_p, f64p, i32p, i32p,
                                        i32p, f64p, f64p, C.c_int64, C.POINTER(C.c_int32)]
        L.orc_solver_system.restype = C.c_int64
        L.orc_cg_dirichlet.argtypes = [C.c_int, i32p, i32p, f64p, C.c_void_p, u8p, f64p, C.c_double, C.c_int,
                                       C.POINTER(C.c_double)]
        _register_mr(L)
        _libs[_variant] = L
    return _libs[_variant]


def _register_mr(L):
    """Bindings of the finite-elasticity part (present once the oracle provides it)."""
    if hasattr(L, "orc_mr_element_residual"):
        L.orc_mr_element_residual.argtypes = [f64p, f64p, f64p, C.c_double, C.c_double, f64p]
        L.orc_mr_element_residual.restype = C.c_int
    if hasattr(L, "orc_mr_element_jacobian"):
        L.orc_mr_element_jacobian.argtypes = [f64p, f64p, f64p, C.c_double, C.c_double, f64p]
        L.orc_mr_element_jacobian.restype = C.c_int
    if hasattr(L, "orc_mr_element_jacobian_fd"):
        L.orc_mr_element_jacobian_fd.argtypes = [f64p, f64p, f64p, C.c_double, C.c_double, C.c_double, f64p]
        L.orc_mr_element_jacobian_fd.restype = C.c_int
    if hasattr(L, "orc_mr_assemble_residual"):
        L.orc_mr_assemble_residual.argtypes = [C.c_int, i32p, i32p, C.c_int, C.c_int, f64p, f64p, f64p, f64p]
        L.orc_mr_assemble_jacobian.argtypes = [C.c_int, i32p, i32p, C.c_int, C.c_int, f64p, f64p, f64p, i32p, i32p,
                                               f64p, C.c_int, C.c_double]


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def gauss_legendre(n: int):
    x = np.zeros(n)
    w = np.zeros(n)
    if lib().orc_gauss_legendre(n, x, w) != 0:
        raise ValueError(n)
    return x, w


def tp_basis(nxi: int, order, ngauss):
    order = _i32(order)
    ngauss = _i32(ngauss)
    code = lib().orc_tp_basis(nxi, order, ngauss, None, None)
    if code < 0:
        raise ValueError("bad basis")
    nns, ng = divmod(code, 1000)
    tab = np.zeros((ng, nxi + 1, nns))
    wts = np.zeros(ng)
    lib().orc_tp_basis(nxi, order, ngauss, tab.ctypes.data, wts.ctypes.data)
    return tab, wts


def regular_mesh(nelem, order: int):
    nelem = _i32(nelem)
    nxi = len(nelem)
    E = int(np.prod(nelem))
    out = np.zeros((E, (order + 1) ** nxi), np.int32)
    lib().orc_regular_mesh(nxi, nelem, order, out)
    return out


def regular_coords(nelem, order: int, origin, extent):
    nelem = _i32(nelem)
    nxi = len(nelem)
    N = int(np.prod(order * nelem + 1))
    out = np.zeros((nxi, N))
    lib().orc_regular_coords(nxi, nelem, order, _f64(origin), _f64(extent), out)
    return out


def regular_triangle_mesh(nelem):
    """Linear triangles of Iron's regular generated mesh in two dimensions
    (src/generated_mesh_routines.F90:1641-1660): grid squares stepped xi1 fastest, each split into
    the triangles (np, np+1, np+1+NX) and (np, np+1+NX, np+NX), NX = nodes per row.  0-based node
    numbers [2*E][3]; the nodes are those of regular_mesh(nelem, 1)."""
    n1, n2 = int(nelem[0]), int(nelem[1])
    NX = n1 + 1
    out = np.zeros((2 * n1 * n2, 3), np.int32)
    e = 0
    for j in range(n2):
        for i in range(n1):
            p = i + j * NX
            out[e] = (p, p + 1, p + 1 + NX)
            out[e + 1] = (p, p + 1 + NX, p + NX)
            e += 2
    return out


def linear_component(elem_first, nnx_first):
    elem_first = _i32(elem_first)
    nnx = _i32(list(nnx_first) + [1] * (3 - len(nnx_first)))
    nxi = len(nnx_first)
    E, nns = elem_first.shape
    elem_lin = np.zeros((E, 2 ** nxi), np.int32)
    l2g = np.zeros(E * 2 ** nxi, np.int32)
    n_lin = lib().orc_linear_component(nxi, E, nns, nnx, elem_first, elem_lin, l2g)
    return elem_lin, l2g[:n_lin].copy()


def csr_structure(elem_dofs, n_dofs: int):
    elem_dofs = _i32(elem_dofs)
    E, ndpe = elem_dofs.shape
    nnz = lib().orc_csr_structure(E, ndpe, elem_dofs, n_dofs, None, None)
    rp = np.zeros(n_dofs + 1, np.int32)
    ci = np.zeros(nnz, np.int32)
    lib().orc_csr_structure(E, ndpe, elem_dofs, n_dofs, rp.ctypes.data, ci.ctypes.data)
    return rp, ci


def csr_location(rp, ci, row: int, col: int) -> int:
    return int(lib().orc_csr_location(_i32(rp), _i32(ci), row, col))


def laplace_element(nxi, order, ngauss, xe, kappa=1.0):
    xe = _f64(xe)
    nns = xe.shape[1]
    K = np.zeros((nns, nns))
    rc = lib().orc_laplace_element(nxi, _i32(order), _i32(ngauss), xe.shape[0], xe, float(kappa), K)
    if rc != 0:
        raise ValueError("bad element")
    return K


def laplace_generalised_element(nxi, order, ngauss, xe, cond, fibre=None):
    """Generalised Laplace element matrix: cond the element-constant conductivity components
    (3D: K11 K22 K33 K12 K23 K13; 2D: K11 K22 K12), fibre [n_angles][nns] the element's fibre
    angles (radians) or None for no fibre field."""
    xe = _f64(xe)
    nns = xe.shape[1]
    K = np.zeros((nns, nns))
    fe = None if fibre is None else _f64(fibre)
    rc = lib().orc_laplace_generalised_element(nxi, _i32(order), _i32(ngauss), xe, _f64(cond),
                                               None if fe is None else fe.ctypes.data,
                                               0 if fe is None else fe.shape[0], K)
    if rc != 0:
        raise ValueError("bad element")
    return K


def laplace_generalised_assemble(nxi, order, ngauss, elem_nodes, coords, cond, rp, ci, fibre=None):
    """Generalised Laplace assembly: cond [n_elem][3 or 6] element-constant conductivity, fibre
    [n_angles][N] nodal fibre angles or None.  Returns (values, rhs)."""
    elem_nodes = _i32(elem_nodes)
    coords = _f64(coords)
    E = elem_nodes.shape[0]
    N = coords.shape[1]
    vals = np.zeros(int(rp[-1]) - 1)
    rhs = np.zeros(N)
    fib = None if fibre is None else _f64(fibre)
    rc = lib().orc_laplace_generalised_assemble(nxi, _i32(order), _i32(ngauss), E, N, elem_nodes, coords,
                                                _f64(cond), None if fib is None else fib.ctypes.data,
                                                0 if fib is None else fib.shape[0], _i32(rp), _i32(ci), vals,
                                                rhs.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle assembly failed ({rc})")
    return vals, rhs


def laplace_assemble(nxi, order, ngauss, elem_nodes, coords, kappa, rp, ci, n_threads=1):
    elem_nodes = _i32(elem_nodes)
    coords = _f64(coords)
    E = elem_nodes.shape[0]
    N = coords.shape[1]
    vals = np.zeros(int(rp[-1]) - 1)
    rhs = np.zeros(N)
    kap = None if kappa is None else _f64(kappa)
    rc = lib().orc_laplace_assemble(nxi, _i32(order), _i32(ngauss), E, N, elem_nodes, coords,
                                    None if kap is None else kap.ctypes.data, _i32(rp), _i32(ci), vals,
                                    rhs.ctypes.data, n_threads)
    if rc != 0:
        raise RuntimeError(f"oracle assembly failed ({rc})")
    return vals, rhs


def laplace_assemble_scaled(nxi, interp, ngauss, elem_params, params, scale, kappa, rp, ci, n_threads=1):
    """Laplace assembly on a mesh of any tensor-product basis (interp per direction: 1..3 Lagrange
    order, 4 cubic Hermite), with element parameters elem_params [E][nns] (0-based DOFs), the
    geometric parameters per DOF params [nxi][n_dofs] and optional scale factors [E][nns]."""
    elem_params = _i32(elem_params)
    params = _f64(params)
    E = elem_params.shape[0]
    N = params.shape[1]
    vals = np.zeros(int(rp[-1]) - 1)
    sc = None if scale is None else _f64(scale)
    kap = None if kappa is None else _f64(kappa)
    rc = lib().orc_laplace_assemble_scaled(nxi, _i32(interp), _i32(ngauss), E, N, elem_params, params,
                                           None if sc is None else sc.ctypes.data,
                                           None if kap is None else kap.ctypes.data, _i32(rp), _i32(ci), vals, None,
                                           int(n_threads))
    if rc != 0:
        raise RuntimeError(f"oracle assembly failed ({rc})")
    return vals


def spmv(rp, ci, vals, x):
    n = len(rp) - 1
    y = np.zeros(n)
    lib().orc_csr_spmv(n, _i32(rp), _i32(ci), _f64(vals), _f64(x), y)
    return y


def mr_element_residual(xe, ze, pe, c1, c2):
    R = np.zeros(89)
    lib().orc_mr_element_residual(_f64(xe), _f64(ze), _f64(pe), float(c1), float(c2), R)
    return R


def mr_element_jacobian(xe, ze, pe, c1, c2):
    K = np.zeros((89, 89))
    lib().orc_mr_element_jacobian(_f64(xe), _f64(ze), _f64(pe), float(c1), float(c2), K)
    return K


def mr_element_jacobian_fd(xe, ze, pe, c1, c2, delta):
    K = np.zeros((89, 89))
    lib().orc_mr_element_jacobian_fd(_f64(xe), _f64(ze), _f64(pe), float(c1), float(c2), float(delta), K)
    return K


def mr_assemble_residual(eq2, elin, nq2, nlin, xg, dep, c):
    E = eq2.shape[0]
    cc = np.broadcast_to(np.asarray(c, np.float64), (E, 2)) if np.ndim(c) == 1 else np.asarray(c, np.float64)
    R = np.zeros(3 * nq2 + nlin)
    lib().orc_mr_assemble_residual(E, _i32(eq2), _i32(elin), nq2, nlin, _f64(xg), _f64(dep), _f64(cc), R)
    return R


def mr_assemble_jacobian(eq2, elin, nq2, nlin, xg, dep, c, rp, ci, fd_delta=None):
    E = eq2.shape[0]
    cc = np.broadcast_to(np.asarray(c, np.float64), (E, 2)) if np.ndim(c) == 1 else np.asarray(c, np.float64)
    vals = np.zeros(int(rp[-1]) - 1)
    rc = lib().orc_mr_assemble_jacobian(E, _i32(eq2), _i32(elin), nq2, nlin, _f64(xg), _f64(dep), _f64(cc), _i32(rp),
                                        _i32(ci), vals, 0 if fd_delta is None else 1,
                                        0.0 if fd_delta is None else float(fd_delta))
    if rc != 0:
        raise RuntimeError(f"oracle Jacobian assembly failed ({rc})")
    return vals


def cg_dirichlet(rp, ci, vals, f, fixed, x_fixed, rtol=1e-12, max_it=100000):
    n = len(rp) - 1
    x = _f64(x_fixed).copy()
    rel = C.c_double(0.0)
    fv = None if f is None else _f64(f)
    it = lib().orc_cg_dirichlet(n, _i32(rp), _i32(ci), _f64(vals), None if fv is None else fv.ctypes.data,
                                np.ascontiguousarray(fixed, dtype=np.uint8), x, rtol, max_it, C.byref(rel))
    if it < 0:
        raise RuntimeError("oracle CG did not converge")
    return x, it, rel.value


def solver_system(rp, ci, vals, f, fixed, u, col_listed=None):
    """Iron's solver system (reduced CSR, values and right-hand side) of a linear equations set
    with Dirichlet DOFs `fixed` at values u; see orc_solver_system."""
    n = len(rp) - 1
    rp, ci, vals, u = _i32(rp), _i32(ci), _f64(vals), _f64(u)
    fixed = np.ascontiguousarray(fixed, dtype=np.uint8)
    fv = None if f is None else _f64(f)
    cl = None if col_listed is None else np.ascontiguousarray(col_listed, dtype=np.uint8)
    cap = int(rp[-1] - 1)
    sod = np.empty(n, np.int32)
    s_rp = np.empty(n + 1, np.int32)
    s_ci = np.empty(max(cap, 1), np.int32)
    s_v = np.empty(max(cap, 1), np.float64)
    s_rhs = np.empty(max(n, 1), np.float64)
    nf = C.c_int32(0)
    nnz = lib().orc_solver_system(n, rp, ci, vals, None if fv is None else fv.ctypes.data, fixed,
                                  None if cl is None else cl.ctypes.data, u, sod, s_rp, s_ci, s_v, s_rhs, cap,
                                  C.byref(nf))
    if nnz < 0:
        raise RuntimeError("oracle solver system failed")
    k = nf.value
    return {"solver_of_dof": sod, "row_ptr": s_rp[:k + 1].copy(), "col_idx": s_ci[:nnz].copy(),
            "values": s_v[:nnz].copy(), "rhs": s_rhs[:k].copy(), "n_free": k}
