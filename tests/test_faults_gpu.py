"""Failure detection on host-injected bad inputs (no GPU fault, trap or hang is provoked).

Kernels never trap: they set bits in a device error word and finish, the host reads the word and
raises with a non-zero status, and the context stays usable for the next call.

- an inverted Mooney-Rivlin element (det Z <= 0 at a Gauss point) -> GFE_DEVERR_JACOBIAN;
- a degenerate trilinear element (det GL = 0) -> GFE_DEVERR_JACOBIAN, on every Laplace kernel
  (an inverted trilinear element is integrated like Iron does, with sqrt|det GL| > 0);
- a non-finite conductivity -> GFE_DEVERR_NONFINITE on every Laplace kernel, a non-finite
  material constant -> GFE_DEVERR_NONFINITE in the Mooney-Rivlin residual;
- after each failure a well-posed call on the same objects succeeds;
- a serving request cancelled while queued is never run and the others complete.
"""
import math

import numpy as np
import pytest
import torch

from iron_gb300 import _lib
from iron_gb300 import mesh as M
from iron_gb300.elasticity import MooneyRivlinAssembly
from iron_gb300.laplace import LaplaceAssembly

pytestmark = pytest.mark.gpu


def _raises(fn, match):
    _lib.device_errors()
    with pytest.raises(_lib.GfeError, match=match):
        fn()
    assert _lib.device_errors() == 0  # raised once and cleared


def test_inverted_mooney_rivlin_element(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 2, 2), build_jacobian=False)
    dep = A.initial_state(0.0)
    nq = A.n_q2
    en = A.mesh.elem_nodes[0]
    # mirror element 0 in x about its own centre: det Z < 0 at every Gauss point
    x = A.xg[0, torch.from_numpy(en.astype(np.int64)).cuda()]
    xm = x.min() + x.max() - x
    dep[torch.from_numpy(en.astype(np.int64)).cuda()] = xm
    _raises(lambda: A.residual(dep, [2.0, 6.0]), "non-positive Jacobian")
    R = A.residual(A.initial_state(0.0), [2.0, 6.0])
    assert R.abs().max().item() < 1e-13
    del nq


@pytest.mark.parametrize("precision,path", [("fp64", "general"), ("mixed_df", "regular"), ("mixed", "regular")])
def test_degenerate_and_nonfinite_laplace(gfe_cuda, precision, path):
    m = M.RegularMesh((4, 3, 3))
    kap = np.ones(m.n_elements)
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    good = A.coords.clone()
    en = torch.from_numpy(m.elem_nodes[5].astype(np.int64)).cuda()
    A.coords[:, en[[1, 3, 5, 7]]] = A.coords[:, en[[0, 2, 4, 6]]]
    _raises(lambda: A.assemble(precision, path=path), "non-positive Jacobian")
    A.coords.copy_(good)
    A.kappa[7] = math.nan
    _raises(lambda: A.assemble(precision, path=path), "non-finite")
    A.kappa[7] = 1.0
    A.assemble(precision, path=path)


def test_nonfinite_conductivity_basis_generic_kernel(gfe_cuda):
    m = M.RegularMesh((3, 2, 2), order=2)
    kap = np.ones(m.n_elements)
    kap[3] = math.inf
    A = LaplaceAssembly.from_regular_mesh(m, kappa=kap)
    _raises(lambda: A.assemble("fp64"), "non-finite")


def test_nonfinite_material_constant(gfe_cuda):
    A = MooneyRivlinAssembly.from_regular_mesh((2, 1, 1), build_jacobian=False)
    dep = A.initial_state(0.0)
    dep[: 3 * A.n_q2] *= 1.01
    _raises(lambda: A.residual(dep, [math.nan, 6.0]), "non-finite")
    A.residual(dep, [2.0, 6.0])


def test_serving_request_cancelled_while_queued(gfe_cuda):
    from iron_gb300.serving import Request, ServingEngine, make_inputs

    reqs = [Request(i, "laplace", 6, 100 + i, arrival=0.0 if i < 2 else 0.5) for i in range(4)]
    for r in reqs:
        make_inputs(r)
    reqs[3].cancel()
    eng = ServingEngine(workers=2)
    try:
        summary = eng.serve(reqs, realtime=True)
    finally:
        eng.close()
    assert reqs[3].cancelled and reqs[3].result is None and math.isnan(reqs[3].t_admit)
    for r in reqs[:3]:
        assert r.result is not None and not r.cancelled
    assert summary["cancelled"] == 1 and summary["requests"] == 3
