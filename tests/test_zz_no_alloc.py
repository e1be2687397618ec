"""The allocation-free solve entry point against the regular one.

gfe_cg_solve_noalloc exists for callers that cannot call cudaMalloc (a host framework that owns
all device memory through its own pool, a serving process with a fixed memory partition).  It
keeps its working vectors in one static device array of the library, which every call shares and
which keeps the previous call's contents.  These tests call both entry points through the C ABI:

- on assembled systems, the allocation-free solve twice in a row, against gfe_cg_solve, within the
  solve tolerance of the other parity tests (1e-10 relative).  Before each clean pair a call that
  stops early (one iteration, GFE_ERR_NOCONV) leaves a half-finished state in the shared array, and
  the larger system follows the smaller one, so a call that did not start clean would show;
- a zero diagonal entry on a free row: gfe_cg_solve raises GFE_DEVERR_NONFINITE on the device
  error word, the allocation-free solve returns GFE_ERR_NUMERIC;
- a system larger than the fixed capacity is refused with an error instead of touching the array.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from iron_gb300 import _lib
from iron_gb300 import mesh as M
from iron_gb300.laplace import LaplaceAssembly

pytestmark = pytest.mark.gpu

MAX_ROWS = 524288  # GFE_NOALLOC_MAX_ROWS in include/gfe.h
GFE_ERR_ARG, GFE_ERR_NUMERIC, GFE_ERR_NOCONV = -1, -4, -5
GFE_DEVERR_NONFINITE = 4


def _problem(n, seed):
    m = M.RegularMesh((n, n, n))
    m.jitter_interior(seed)
    kap = np.exp(np.random.default_rng(seed + 7).uniform(np.log(0.1), np.log(10.0), m.n_elements))
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    A.assemble("fp64")
    fixed = np.zeros(m.n_nodes, np.uint8)
    x0 = np.zeros(m.n_nodes)
    fixed[m.face_nodes(0, 0)] = 1
    fixed[m.face_nodes(0, 1)] = 1
    x0[m.face_nodes(0, 1)] = 1.0
    return A, torch.from_numpy(fixed).cuda(), torch.from_numpy(x0).cuda()


def _call(L, name, A, fixed, x0, rtol=1e-12, max_iters=100000, values=None):
    x = x0.clone()
    it = C.c_int32(0)
    rel = C.c_double(0.0)
    st = _lib.stream_handle()
    vals = A.values if values is None else values
    if name == "gfe_cg_solve":
        rc = L.gfe_cg_solve(A.n_nodes, _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), _lib.ptr(vals), None, None,
                            _lib.ptr(fixed), _lib.ptr(x), rtol, max_iters, _lib.GFE_FP64, C.byref(it), C.byref(rel),
                            st)
    else:
        rc = L.gfe_cg_solve_noalloc(A.n_nodes, _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), _lib.ptr(vals), None,
                                    _lib.ptr(fixed), _lib.ptr(x), rtol, max_iters, C.byref(it), C.byref(rel), st)
    torch.cuda.synchronize()
    return rc, x.cpu().numpy(), it.value, rel.value


def test_noalloc_solve_matches_regular_solve_twice(gfe_cuda):
    L = _lib.load()
    for n, seed in ((9, 3), (12, 0)):
        A, fixed, x0 = _problem(n, seed)
        rc, ref, _, _ = _call(L, "gfe_cg_solve", A, fixed, x0)
        assert rc == 0, _lib.last_error()
        # an early stop leaves the shared array mid-solve
        rc, _, it, _ = _call(L, "gfe_cg_solve_noalloc", A, fixed, x0, max_iters=1)
        assert rc == GFE_ERR_NOCONV, _lib.last_error()
        for _ in range(2):
            rc, x, _, rel = _call(L, "gfe_cg_solve_noalloc", A, fixed, x0)
            assert rc == 0, _lib.last_error()
            assert rel <= 1e-12
            assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()


def test_noalloc_reports_zero_diagonal_like_regular_solve(gfe_cuda):
    L = _lib.load()
    A, fixed, x0 = _problem(6, 1)
    rp = A.row_ptr.cpu().numpy()
    ci = A.col_idx.cpu().numpy()
    fixed_h = fixed.cpu().numpy()
    row = int(np.flatnonzero(fixed_h == 0)[len(np.flatnonzero(fixed_h == 0)) // 2])
    k = rp[row] - 1 + int(np.flatnonzero(ci[rp[row] - 1:rp[row + 1] - 1] == row + 1)[0])
    bad = A.values.clone()
    bad[k] = 0.0
    _lib.device_errors()  # clear the library word
    _call(L, "gfe_cg_solve", A, fixed, x0, max_iters=50, values=bad)
    assert _lib.device_errors() & GFE_DEVERR_NONFINITE
    rc, _, _, _ = _call(L, "gfe_cg_solve_noalloc", A, fixed, x0, max_iters=50, values=bad)
    assert rc == GFE_ERR_NUMERIC
    assert "diagonal" in _lib.last_error()
    # the next well-posed call is unaffected by the failed one
    rc, ref, _, _ = _call(L, "gfe_cg_solve", A, fixed, x0)
    assert rc == 0, _lib.last_error()
    rc, x, _, _ = _call(L, "gfe_cg_solve_noalloc", A, fixed, x0)
    assert rc == 0, _lib.last_error()
    assert np.abs(x - ref).max() <= 1e-10 * np.abs(ref).max()


def test_noalloc_rejects_systems_above_capacity(gfe_cuda):
    L = _lib.load()
    A, fixed, x0 = _problem(3, 0)
    x = x0.clone()
    it = C.c_int32(0)
    rel = C.c_double(0.0)
    rc = L.gfe_cg_solve_noalloc(MAX_ROWS + 1, _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), _lib.ptr(A.values), None,
                                _lib.ptr(fixed), _lib.ptr(x), 1e-12, 10, C.byref(it), C.byref(rel),
                                _lib.stream_handle())
    assert rc == GFE_ERR_ARG
    assert "capacity" in _lib.last_error()
