"""CPU tests of the FP64 oracle: pinned on the reference's own known answer
(the A-form MMS convergence test, test/integration/test_aform_source.cpp:130-209)
and on discretisation identities."""
import os

import numpy as np
import pytest

import oracle
from hephaestus_gb300 import meshes
from tests import hexref

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _rate(e, n):
    # EstimateConvergenceRate of test_aform_source.cpp:10-15
    return [np.log(e[i] / e[i - 1]) / np.log((n[i - 1] / n[i]) ** (1.0 / 3.0)) for i in range(1, len(e))]


def test_aform_mms_rate_beam_tet():
    """Same problem as TestAForm: beam-tet.mesh, 0/1/2 uniform refinements,
    ND_3D_P2, mu = 1/(1+0.5 cos(pi x) cos(pi y)), sigma = 1, one backward-Euler
    step dt = 0.05, A x n = 0 on attributes 1,2,3; assert 1.85 < r < 3.0."""
    d = np.load(os.path.join(GOLD, "beam_tet.npz"))
    v, t, bt, ba = d["verts"], d["tets"], d["btris"], d["battr"]
    errs, nd = [], []
    for lev in range(3):
        if lev:
            v, t, bt, ba = meshes.refine_tets(v, t, bt, ba)
        P = oracle.Problem.tet(v, t, 2)
        P.set_coef_mms(0.05, 0.5, 1.0)
        P.assemble()
        m = P.tet_ess_mask(bt, ba, 0b111)
        P.set_ess(m)
        b = P.load_mms(0.05, 0.5, q=6)
        b[m == 1] = 0.0
        x, st, it, rr = P.pcg(b, precond=1, rtol=1e-13, maxit=20000)
        assert st == 0
        errs.append(P.l2err_mms(0.05 * x, 0.05, q=6))  # A_1 = A_0 + dt dA/dt
        nd.append(P.ndof)
    assert nd == [494, 3152, 22256]
    for r in _rate(errs, nd):
        assert 2 - 0.15 < r < 2 + 1.0, (errs, nd)


@pytest.mark.parametrize("p", [1, 2, 3])
def test_hex_mms_converges(p):
    errs, nd = [], []
    for n in (2, 4):
        P = oracle.Problem.hex(n, n, n, p)
        P.set_coef_mms(0.05, 0.5, 1.0)
        P.assemble()
        m = P.hex_ess_mask(0x3F)
        P.set_ess(m)
        b = P.load_mms(0.05, 0.5, q=p + 4)
        b[m == 1] = 0
        x, st, it, rr = P.pcg(b, rtol=1e-13, maxit=20000)
        errs.append(P.l2err_mms(0.05 * x, 0.05, q=p + 4))
        nd.append(P.ndof)
    assert _rate(errs, nd)[0] > p + 0.5


def _sheared(n):
    v = meshes.box_vertices(n, n, n)
    A = np.array([[1.0, 0.2, 0.1], [0.0, 0.9, -0.15], [0.05, 0.0, 1.1]])
    return v @ A.T


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("shear", [False, True])
def test_hex_symmetric_positive(p, shear):
    n = 2
    P = oracle.Problem.hex(n, n, n, p, _sheared(n) if shear else None)
    rng = np.random.default_rng(1)
    P.set_coef(rng.uniform(0.5, 2, P.ne), rng.uniform(0.5, 2, P.ne))
    P.assemble()
    K = P.csr().toarray()
    assert np.abs(K - K.T).max() < 1e-12 * np.abs(K).max()
    assert np.linalg.eigvalsh(K).min() > 0


@pytest.mark.parametrize("p", [1, 2, 3])
def test_hex_curl_of_gradient_vanishes(p):
    """Exact sequence: C_nu G phi = 0 for every Q_p field phi."""
    n = 3
    P = oracle.Problem.hex(n, n, n, p, _sheared(n))
    rng = np.random.default_rng(2)
    P.set_coef(rng.uniform(0.5, 2, P.ne), None)
    P.assemble()
    phi = rng.standard_normal((n * p + 1,) * 3)
    g = hexref.discrete_gradient(n, n, n, p, phi)
    y = P.apply(g)
    assert np.linalg.norm(y) < 1e-11 * np.linalg.norm(g)
    # and the mass is not degenerate on it
    P.set_coef(np.zeros(P.ne), np.ones(P.ne))
    P.assemble()
    assert g @ P.apply(g) > 0


def test_hex_reference_matrix_vs_quadrature():
    """Element matrix from the 12 reference tensors equals direct quadrature."""
    n, p = 2, 2
    P = oracle.Problem.hex(n, n, n, p, _sheared(n))
    P.set_coef_mms(1.0, 0.0, 1.0)  # constant nu = 1, sigma = 1 via quadrature
    Kq = P.element_matrix(3)
    P.set_coef(np.ones(P.ne), np.ones(P.ne))
    Kr = P.element_matrix(3)
    assert np.abs(Kq - Kr).max() < 1e-12 * np.abs(Kr).max()


def test_mass_exact_on_constant_field():
    """Mass energy of the interpolant of a constant field = |c|^2 vol."""
    n, p = 3, 2
    P = oracle.Problem.hex(n, n, n, p)
    P.set_coef(np.zeros(P.ne), np.ones(P.ne))
    P.assemble()
    c = np.array([0.3, -1.2, 0.7])
    # reference-coordinate dofs of a constant physical field on h-scaled cubes
    h = 1.0 / n
    nd = [n * p * (n * p + 1) ** 2] * 3
    u = np.concatenate([np.full(nd[k], c[k] * h) for k in range(3)])
    assert abs(u @ P.apply(u) - c @ c) < 1e-12


def test_chebyshev_preconditioner_is_spd():
    n, p = 3, 1
    P = oracle.Problem.hex(n, n, n, p)
    rng = np.random.default_rng(3)
    P.set_coef(rng.uniform(0.5, 2, P.ne), rng.uniform(0.5, 2, P.ne))
    P.assemble()
    P.set_ess(P.hex_ess_mask(0x3F))
    lm = 1.1 * P.lanczos_lmax(20)
    Z = np.stack([P.cheb_apply(e, 3, lm, 30.0) for e in np.eye(P.ndof)], axis=1)
    assert np.abs(Z - Z.T).max() < 1e-10 * np.abs(Z).max()
    assert np.linalg.eigvalsh(0.5 * (Z + Z.T)).min() > 0


def test_pcg_matches_direct_solve():
    import scipy.sparse.linalg as spla

    n, p = 4, 2
    P = oracle.Problem.hex(n, n, n, p)
    rng = np.random.default_rng(4)
    P.set_coef(0.01 * meshes.loguniform(P.ne, 1, 1e3, rng), meshes.loguniform(P.ne, 1e-2, 1e6, rng))
    P.assemble()
    m = P.hex_ess_mask(0x3F)
    P.set_ess(m)
    b = P.load_coil(q=4)
    b[m == 1] = 0
    J = P.csr().tolil()
    for i in np.nonzero(m)[0]:
        J[i, :] = 0
        J[:, i] = 0
        J[i, i] = 1.0
    xd = spla.spsolve(J.tocsc(), b)
    for pre, kw in ((1, {}), (2, {"cheb_degree": 3})):
        x, st, it, rr = P.pcg(b, precond=pre, rtol=1e-12, maxit=100000, **kw)
        assert st == 0
        assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-8


def test_eliminated_csr_matches_masked_apply():
    n, p = 3, 2
    P = oracle.Problem.hex(n, n, n, p)
    rng = np.random.default_rng(6)
    P.set_coef(rng.uniform(0.5, 2, P.ne), rng.uniform(0.5, 2, P.ne))
    P.assemble()
    P.set_ess(P.hex_ess_mask(0x3F))
    nnz = oracle.lib().orc_build_eliminated(P.h)
    assert 0 < nnz < oracle.lib().orc_nnz(P.h)
    x = rng.standard_normal(P.ndof)
    y = np.empty_like(x)
    oracle.lib().orc_spmv_eliminated(P.h, oracle._p(x), oracle._p(y), 2)
    assert np.allclose(y, P.apply_masked(x), rtol=1e-14, atol=1e-14)
