"""CPU checks of the frequency-domain restatement (oracle/complex_ref.py): the
eliminated C_nu + i omega M_sigma is complex symmetric, and the COCG
restatement reaches the SuperLU solution the reference computes."""
import numpy as np
import pytest

import oracle
from oracle import complex_ref as CR
from hephaestus_gb300 import meshes


def _system(n, p, omega, seed=0, bits=0x3F):
    rng = np.random.default_rng(seed)
    ne = n ** 3
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    ref = oracle.Problem.hex(n, n, n, p)
    Cn, M = CR.forms(ref, nu, sigma)
    ess = ref.hex_ess_mask(bits)
    return CR.eliminated(Cn, M, omega, ess), ess, rng


@pytest.mark.parametrize("p", [1, 2])
def test_eliminated_operator_is_complex_symmetric(p):
    J, ess, _ = _system(3, p, 1e3)
    d = (J - J.T).tocoo()
    assert np.abs(d.data).max(initial=0.0) <= 1e-12 * np.abs(J.data).max()
    # identity rows at essential dofs
    idx = np.flatnonzero(ess)
    assert np.allclose(J[idx][:, idx].toarray(), np.eye(len(idx)))


@pytest.mark.parametrize("p,omega", [(1, 1e2), (2, 1e4)])
def test_cocg_restatement_reaches_direct_solution(p, omega):
    J, ess, rng = _system(3, p, omega, seed=p)
    b = rng.standard_normal(J.shape[0]) + 1j * rng.standard_normal(J.shape[0])
    x_lu = CR.direct_solve(J, b)
    x, it = CR.cocg(J, b, rtol=1e-13, maxit=20000)
    assert it > 0
    assert np.linalg.norm(x - x_lu) / np.linalg.norm(x_lu) < 1e-8
