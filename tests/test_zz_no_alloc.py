"""The allocation-free solve entry point against the regular one.

gfe_cg_solve_noalloc exists for callers that cannot call cudaMalloc (a host framework that owns
all device memory through its own pool, a serving process with a fixed memory partition).  It
keeps its working vectors in one static device array of the library.  This test calls both entry
points through the C ABI on the same assembled system, twice in a row for the allocation-free one
(the shared array keeps the previous call's contents, so the second call checks that each call
starts clean), and compares the solutions within the solve tolerance used by the other parity
tests (1e-10 relative).  It also checks that a system larger than the fixed capacity is refused
with an error instead of touching the array.
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


def _solve(L, name, A, fixed, x0, rtol=1e-12):
    x = x0.clone()
    it = C.c_int32(0)
    rel = C.c_double(0.0)
    st = _lib.stream_handle()
    if name == "gfe_cg_solve":
        rc = L.gfe_cg_solve(A.n_nodes, _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), _lib.ptr(A.values), None, None,
                            _lib.ptr(fixed), _lib.ptr(x), rtol, 100000, _lib.GFE_FP64, C.byref(it), C.byref(rel), st)
    else:
        rc = L.gfe_cg_solve_noalloc(A.n_nodes, _lib.ptr(A.row_ptr), _lib.ptr(A.col_idx), _lib.ptr(A.values), None,
                                    _lib.ptr(fixed), _lib.ptr(x), rtol, 100000, C.byref(it), C.byref(rel), st)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    return x.cpu().numpy(), it.value, rel.value


def test_noalloc_solve_matches_regular_solve_twice(gfe_cuda):
    L = _lib.load()
    for n, seed in ((12, 0), (9, 3)):
        A, fixed, x0 = _problem(n, seed)
        ref, it_ref, rel_ref = _solve(L, "gfe_cg_solve", A, fixed, x0)
        for _ in range(2):
            x, it, rel = _solve(L, "gfe_cg_solve_noalloc", A, fixed, x0)
            assert rel <= 1e-12
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
    assert rc == -1  # GFE_ERR_ARG
    assert "capacity" in _lib.last_error()
