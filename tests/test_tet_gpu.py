"""GPU parity of the tetrahedral Nedelec element-matrix path (closed-form FP64
element matrices) against the oracle (quadrature element matrices + CSR)."""
import os

import numpy as np
import pytest

import oracle
from hephaestus_gb300 import GpuHCurlPCGSolver, HCurlOperator, meshes

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _pair(n, p, jitter=0.15, mass=True, seed=0, dt=0.01, bits=0x3F):
    v, t, bt, ba = meshes.kuhn_mesh(n, jitter=jitter, seed=seed)
    rng = np.random.default_rng(seed)
    ne = len(t)
    nu = meshes.loguniform(ne, 1.0, 1e2, rng)
    sigma = meshes.loguniform(ne, 1e-1, 1e3, rng) if mass else None
    op = HCurlOperator.from_tets(v, t, p, nu, sigma, dt=dt, btris=bt, battr=ba, ess_attr_bits=bits)
    ref = oracle.Problem.tet(v, t, p)
    ref.set_coef(dt * nu, sigma)
    ref.assemble()
    m = ref.tet_ess_mask(bt, ba, bits)
    assert np.array_equal(op.ess_mask(), m)
    ref.set_ess(m)
    return op, ref, rng


@pytest.mark.parametrize("p", [1, 2])
def test_tet_element_matrices_match_oracle(p):
    """Closed-form element matrices (device) = quadrature element matrices (oracle)."""
    op, ref, _ = _pair(2, p)
    for e in (0, 5, 17, op.ne - 1):
        K = op.ElementMatrix(e)
        Kr = ref.element_matrix(e)
        assert np.abs(K - Kr).max() < 1e-12 * np.abs(Kr).max(), e


@pytest.mark.parametrize("p", [1, 2])
def test_tet_apply_parity(p):
    op, ref, rng = _pair(3, p)
    assert op.ndof == ref.ndof
    x = rng.standard_normal(op.ndof)
    y = op.Mult(x)
    yr = ref.apply_masked(x)
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < 1e-12
    yf = op.ApplyForm(x)
    yfr = ref.apply(x)
    assert np.linalg.norm(yf - yfr) / np.linalg.norm(yfr) < 1e-12
    d = op.Diagonal()
    assert np.abs(d - ref.diag_masked()).max() < 1e-12 * np.abs(d).max()


@pytest.mark.parametrize("prec,nrhs", [("float64", 16), ("float32", 16), ("float32", 4), ("float32", 8),
                                       ("float32", 32), ("float32", 2)])
def test_tet_multi_rhs_parity(prec, nrhs):
    import torch

    op, ref, rng = _pair(4, 2)
    X = rng.standard_normal((op.ndof, nrhs))
    Xd = torch.tensor(X, dtype=getattr(torch, prec), device="cuda")
    Yd = torch.empty_like(Xd)
    op.MultMultiDevice(Xd, Yd)
    torch.cuda.synchronize()
    Y = Yd.double().cpu().numpy()
    Xr = Xd.double().cpu().numpy()
    tol = 1e-12 if prec == "float64" else 2e-6
    for r in range(nrhs):
        yr = ref.apply_masked(Xr[:, r])
        assert np.linalg.norm(Y[:, r] - yr) / np.linalg.norm(yr) < tol


def test_tet_multi_rhs_bf16_matrices():
    """BF16 element matrices, FP32 vectors and accumulation: within BF16 rounding
    of the FP64 operator (8-bit significand: tolerance 1e-2, relative 2-norm)."""
    import torch

    op, ref, rng = _pair(4, 2)
    nrhs = 16
    X = rng.standard_normal((op.ndof, nrhs))
    Xd = torch.tensor(X, dtype=torch.float32, device="cuda")
    Yd = torch.empty_like(Xd)
    op.MultMultiDevice(Xd, Yd, bf16_matrices=True)
    torch.cuda.synchronize()
    Y = Yd.double().cpu().numpy()
    Xr = Xd.double().cpu().numpy()
    for r in range(nrhs):
        yr = ref.apply_masked(Xr[:, r])
        err = np.linalg.norm(Y[:, r] - yr) / np.linalg.norm(yr)
        assert 1e-7 < err < 1e-2, (r, err)  # really rounded, and only by BF16


def test_tet_beam_mesh_matches_oracle():
    d = np.load(os.path.join(GOLD, "beam_tet.npz"))
    v, t, bt, ba = meshes.refine_tets(d["verts"], d["tets"], d["btris"], d["battr"])
    ne = len(t)
    op = HCurlOperator.from_tets(v, t, 2, np.ones(ne), np.ones(ne), dt=0.05, btris=bt, battr=ba,
                                 ess_attr_bits=0b111)
    ref = oracle.Problem.tet(v, t, 2)
    ref.set_coef(0.05 * np.ones(ne), np.ones(ne))
    ref.assemble()
    ref.set_ess(ref.tet_ess_mask(bt, ba, 0b111))
    x = np.random.default_rng(3).standard_normal(op.ndof)
    yr = ref.apply_masked(x)
    assert op.ndof == 3152
    assert np.linalg.norm(op.Mult(x) - yr) / np.linalg.norm(yr) < 1e-12


@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_rr"])
def test_tet_solve_matches_oracle(prec):
    op, ref, rng = _pair(4, 2)
    b = rng.standard_normal(op.ndof)
    b[op.ess_mask() == 1] = 0.0
    xr, st, it, rr = ref.pcg(b, precond=1, rtol=1e-13, maxit=100000)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "MaxIter": 100000, "Precision": prec}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "OK", s.result
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-9


@pytest.mark.parametrize("prec", ["fp64", "mixed", "mixed_rr"])
@pytest.mark.parametrize("nrhs", [1, 4, 16])
def test_tet_multi_rhs_solve_matches_oracle(prec, nrhs):
    """Block PCG over nrhs columns = the oracle's PCG column by column.  The
    columns have very different scales (and one is zero when nrhs > 1), so
    each column's own stopping test and freezing are exercised."""
    import torch

    op, ref, rng = _pair(4, 2)
    B = rng.standard_normal((op.ndof, nrhs))
    B *= np.logspace(-3, 3, nrhs)[None, :]
    if nrhs > 1:
        B[:, 1] = 0.0
    B[op.ess_mask() == 1, :] = 0.0
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 100000, "Precision": prec}, op)
    Bd = torch.tensor(B, device="cuda")
    Xd = torch.zeros_like(Bd)
    res = s.MultMultiDevice(Bd, Xd)
    X = Xd.cpu().numpy()
    assert len(res) == nrhs
    for r in range(nrhs):
        assert res[r]["status"] == "OK", (r, res[r])
        if not B[:, r].any():
            assert not X[:, r].any() and res[r]["iterations"] == 0
            continue
        xr, st, it, rr = ref.pcg(B[:, r], precond=1, rtol=1e-13, maxit=100000)
        assert np.linalg.norm(X[:, r] - xr) / np.linalg.norm(xr) < 1e-9, r
        res_true = np.linalg.norm(B[:, r] - ref.apply_masked(X[:, r])) / np.linalg.norm(B[:, r])
        assert res_true < 2e-12, (r, res_true)
        if prec == "fp64":
            # same algorithm and stopping test as the oracle's Jacobi PCG
            _, _, it12, _ = ref.pcg(B[:, r], precond=1, rtol=1e-12, maxit=100000)
            assert abs(res[r]["iterations"] - it12) <= max(3, it12 // 20), (r, res[r]["iterations"], it12)


def test_tet_multi_rhs_solve_initial_guess_and_single_column_agree():
    """A nonzero initial guess is honoured, and every column of the block
    solve equals the single-right-hand-side device solve of that column."""
    import torch

    op, ref, rng = _pair(3, 2, seed=4)
    nrhs = 4
    B = rng.standard_normal((op.ndof, nrhs))
    X0 = rng.standard_normal((op.ndof, nrhs))
    m = op.ess_mask() == 1
    B[m, :] = X0[m, :]  # boundary values carried by the essential rows
    prm = {"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 100000, "Precision": "fp64"}
    Xd = torch.tensor(X0, device="cuda")
    res = GpuHCurlPCGSolver(prm, op).MultMultiDevice(torch.tensor(B, device="cuda"), Xd)
    X = Xd.cpu().numpy()
    for r in range(nrhs):
        x1 = X0[:, r].copy()
        s1 = GpuHCurlPCGSolver(prm, op)
        s1.Mult(B[:, r], x1)
        assert res[r]["status"] == "OK" and s1.result["status"] == "OK"
        assert np.linalg.norm(X[:, r] - x1) / np.linalg.norm(x1) < 1e-10, r
        assert np.array_equal(X[m, r], X0[m, r])


@pytest.mark.parametrize("p", [1, 2])
def test_tet_coil_load_matches_oracle(p):
    """Device coil load on tets (collapsed Gauss-Legendre rule) = the oracle's
    load with the same rule, for a shifted coil and two rule sizes."""
    op, ref, _ = _pair(4, p)
    for q in (3, 5):
        b = op.LoadCoil(I0=1.3, xc=0.56, yc=0.45, q=q)
        br = ref.load_coil(I0=1.3, xc=0.56, yc=0.45, q=q)
        assert np.count_nonzero(br) > 0
        assert np.linalg.norm(b - br) <= 1e-13 * np.linalg.norm(br), q


def test_tet_host_block_solve_matches_device_block_solve():
    """hc_solve_multi (host arrays, the MFEM shim's MultBlock) = hc_solve_multi_device."""
    import torch

    op, ref, rng = _pair(3, 2, seed=6)
    B = rng.standard_normal((op.ndof, 4))
    B[op.ess_mask() == 1, :] = 0.0
    prm = {"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 100000, "Precision": "fp64"}
    X = np.zeros_like(B)
    res_h = GpuHCurlPCGSolver(prm, op).MultMulti(B, X)
    Xd = torch.zeros(op.ndof, 4, dtype=torch.float64, device="cuda")
    res_d = GpuHCurlPCGSolver(prm, op).MultMultiDevice(torch.tensor(B, device="cuda"), Xd)
    assert all(r["status"] == "OK" for r in res_h + res_d)
    # both converged to 1e-12; they differ only by the order of floating-point atomics in the apply
    assert np.linalg.norm(X - Xd.cpu().numpy()) <= 1e-8 * np.linalg.norm(X)
