"""Host-side pieces of the Newton driver (CPU only): Iron's load-increment rule and the
uniaxial-stretch known answer, checked on the oracle's assembled residual."""
from types import SimpleNamespace

import numpy as np
import torch

import oracle
from iron_gb300.mesh import RegularMesh, linear_component
from iron_gb300.newton import increment_dirichlet, uniaxial_exact_state, uniaxial_roller_conditions

C1, C2 = 2.0, 6.0


def test_increment_rule_is_a_linear_ramp():
    full = torch.tensor([1.1, -2.0, 0.0], dtype=torch.float64)
    cur = torch.tensor([1.0, 0.0, 0.0], dtype=torch.float64)
    start = cur.clone()
    N = 5
    for step in range(1, N + 1):
        cur = increment_dirichlet(cur, full, step, N)
        assert torch.allclose(cur, start + (full - start) * step / N, rtol=0, atol=1e-15)
    assert torch.equal(cur, full)


def _q2(ne):
    m = RegularMesh(ne, order=2)
    elin, lin2g = linear_component(m.elem_nodes, 2)
    nq = m.coords.shape[1]
    asm = SimpleNamespace(xg=torch.from_numpy(m.coords), n_q2=nq, n_lin=len(lin2g), ndof=3 * nq + len(lin2g),
                          device=torch.device("cpu"))
    return m, elin, asm


def test_uniaxial_exact_state_is_the_discrete_solution():
    """The oracle's assembled residual vanishes on every free DOF at the exact homogeneous state,
    and the roller conditions hold there."""
    lam = 1.1
    m, elin, asm = _q2((2, 3, 2))
    fixed, full = uniaxial_roller_conditions(asm, lam)
    dep = uniaxial_exact_state(asm, lam, C1, C2).numpy()
    fx = fixed.numpy().astype(bool)
    assert np.array_equal(dep[fx], full.numpy()[fx])
    R = oracle.mr_assemble_residual(m.elem_nodes, elin, asm.n_q2, asm.n_lin, m.coords, dep, [C1, C2])
    scale = np.abs(R).max()  # reaction forces on the pulled face
    assert scale > 0.1
    assert np.abs(R[~fx]).max() <= 1e-13 * scale


def test_roller_conditions_count():
    m, _, asm = _q2((2, 2, 2))
    fixed, full = uniaxial_roller_conditions(asm, 1.2)
    nq = asm.n_q2
    per_face = 5 * 5
    f = fixed.numpy()
    assert f[:nq].sum() == 2 * per_face and f[nq:2 * nq].sum() == per_face and f[2 * nq:3 * nq].sum() == per_face
    assert f[3 * nq:].sum() == 0
    x = m.coords
    onX = np.abs(x[0] - 1.0) < 1e-12
    assert np.allclose(full.numpy()[:nq][onX], 1.2)
