"""Tet auxiliary-space preconditioner: the discrete gradient G (exact, curl-free,
reproduces gradients of linear functions, checked with the oracle's basis),
and block PCG with Jacobi + (PG) V (PG)^T against the oracle's solutions.
On order-1 meshes Jacobi alone already converges quickly (the correction
neither helps nor hurts much); on order-2 meshes with the log-uniform
coefficient fields it cuts the iteration count several-fold."""
import numpy as np
import pytest

import oracle
from hephaestus_gb300 import GpuHCurlPCGSolver, HCurlOperator, meshes

pytestmark = pytest.mark.gpu


def _mesh_op(n, p, seed=0, fields="loguniform", bits=0x3F):
    v, t, bt, ba = meshes.kuhn_mesh(n, jitter=0.15, seed=seed)
    rng = np.random.default_rng(seed)
    ne = len(t)
    if fields == "loguniform":
        nu, sigma = meshes.loguniform(ne, 1.0, 1e3, rng), meshes.loguniform(ne, 1e-2, 1e6, rng)
    else:
        nu, sigma = np.ones(ne), np.ones(ne)
    op = HCurlOperator.from_tets(v, t, p, nu, sigma, dt=0.01, btris=bt, battr=ba, ess_attr_bits=bits)
    ref = oracle.Problem.tet(v, t, p)
    ref.set_coef(0.01 * nu, sigma)
    ref.assemble()
    ref.set_ess(ref.tet_ess_mask(bt, ba, bits))
    return op, ref, v, t, rng


@pytest.mark.parametrize("p", [1, 2])
def test_gradient_of_linear_function_is_its_gradient(p):
    """u = c.x on the vertices: the Nedelec field G u equals c inside every element."""
    import torch

    op, ref, v, t, rng = _mesh_op(3, p)
    c = np.array([0.3, -1.2, 0.7])
    u = torch.tensor(v @ c, device="cuda")
    y = torch.empty(op.ndof, dtype=torch.float64, device="cuda")
    op.GradientDevice(u, y)
    yh = y.cpu().numpy()
    for e in (0, 7, len(t) // 2, len(t) - 1):
        for xi in ([0.2, 0.3, 0.1], [0.05, 0.05, 0.8]):
            val, curl = ref.eval(yh, e, np.array(xi))
            assert np.abs(val - c).max() < 1e-12
            assert np.abs(curl).max() < 1e-11


@pytest.mark.parametrize("p", [1, 2])
def test_gradient_is_curl_free(p):
    """K_curl G u = 0 for random vertex values (the curl-curl part alone)."""
    import torch

    v, t, bt, ba = meshes.kuhn_mesh(3, jitter=0.15, seed=1)
    ne = len(t)
    op = HCurlOperator.from_tets(v, t, p, np.ones(ne), np.ones(ne), dt=1.0, btris=bt, battr=ba, ess_attr_bits=0)
    ref = oracle.Problem.tet(v, t, p)
    ref.set_coef(np.ones(ne), None)
    ref.assemble()
    u = torch.tensor(np.random.default_rng(2).standard_normal(len(v)), device="cuda")
    y = torch.empty(op.ndof, dtype=torch.float64, device="cuda")
    op.GradientDevice(u, y)
    g = y.cpu().numpy()
    kc = ref.apply(g)
    ref.set_coef(np.zeros(ne), np.ones(ne))
    ref.assemble()
    km = ref.apply(g)
    assert np.linalg.norm(kc) < 1e-11 * np.linalg.norm(km)


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_rr"])
def test_aux_block_solve_matches_oracle(p, prec):
    import torch

    op, ref, v, t, rng = _mesh_op(5, p, seed=3)
    nrhs = 4
    B = np.zeros((op.ndof, nrhs))
    for k in range(nrhs):
        B[:, k] = ref.load_coil(I0=0.5 + 0.5 * k, xc=0.45 + 0.05 * k, yc=0.5, q=4)
    B[op.ess_mask() == 1, :] = 0.0
    Bd = torch.tensor(B, device="cuda")
    res = {}
    X = {}
    for pc in ("jacobi", "aux"):
        Xd = torch.zeros_like(Bd)
        s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 100000, "Precision": prec,
                               "Preconditioner": pc}, op)
        res[pc] = s.MultMultiDevice(Bd, Xd)
        X[pc] = Xd.cpu().numpy()
    for k in range(nrhs):
        assert res["aux"][k]["status"] == "OK", res["aux"][k]
        xr, st, it, rr = ref.pcg(B[:, k], precond=1, rtol=1e-13, maxit=200000)
        assert np.linalg.norm(X["aux"][:, k] - xr) / np.linalg.norm(xr) < 1e-9, k
        true_res = np.linalg.norm(B[:, k] - ref.apply_masked(X["aux"][:, k])) / np.linalg.norm(B[:, k])
        assert true_res < 2e-12
        if p == 2:
            # the edge-bubble gradients are Jacobi's slow modes on order-2 meshes with coefficient jumps
            assert res["aux"][k]["iterations"] < 0.5 * res["jacobi"][k]["iterations"], (res["aux"][k], res["jacobi"][k])


def test_aux_single_rhs_solve_on_tets():
    """hc_solve with HC_PRECOND_AUX on a tet mesh (one-column block PCG) = oracle."""
    op, ref, v, t, rng = _mesh_op(4, 2, seed=5)
    b = ref.load_coil(I0=1.0, q=4)
    b[op.ess_mask() == 1] = 0.0
    x = np.zeros(op.ndof)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 20000, "Precision": "fp64",
                           "Preconditioner": "aux"}, op)
    s.Mult(b, x)
    assert s.result["status"] == "OK"
    xr, st, it, rr = ref.pcg(b, precond=1, rtol=1e-13, maxit=200000)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-9
    assert s.result["iterations"] < it
