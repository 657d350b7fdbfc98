"""GPU parity of the frequency-domain operator C_nu + i omega M_sigma and its
COCG solve against the CPU restatement (SuperLU direct solve, as the
reference's ComplexMaxwellOperator::Solve), through the C ABI."""
import ctypes as C

import numpy as np
import pytest

import oracle
from oracle import complex_ref as CR
from hephaestus_gb300 import GpuComplexCOCGSolver, HCurlOperator, meshes
from hephaestus_gb300 import _native as N

pytestmark = pytest.mark.gpu

TOL64 = 1e-12   # FP64 apply, relative 2-norm
TOL32 = 2e-6    # FP32 apply, relative 2-norm


def _sheared(n):
    v = meshes.box_vertices(n, n, n)
    A = np.array([[1.0, 0.2, 0.1], [0.0, 0.9, -0.15], [0.05, 0.0, 1.1]])
    return v @ A.T


def _pair(n, p, omega, shear=False, seed=0, dt=0.01, bits=0x3F):
    rng = np.random.default_rng(seed)
    ne = n ** 3
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    verts = _sheared(n) if shear else None
    # dt of the handle only scales its stored curl factor; the complex operator undoes it
    op = HCurlOperator(n, n, n, p, nu, sigma, dt=dt, vertices=verts, ess_attr_bits=bits)
    ref = oracle.Problem.hex(n, n, n, p, verts)
    Cn, M = CR.forms(ref, nu, sigma)
    J = CR.eliminated(Cn, M, omega, op.ess_mask())
    return op, J, rng


def _crandn(rng, n):
    return rng.standard_normal(n) + 1j * rng.standard_normal(n)


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("shear", [False, True])
def test_complex_apply_parity_fp64(p, shear):
    omega = 3.7e3
    op, J, rng = _pair(3, p, omega, shear)
    x = _crandn(rng, op.ndof)
    y = op.MultComplex(omega, x)
    yr = J @ x
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < TOL64


@pytest.mark.parametrize("p", [1, 2, 3])
def test_complex_apply_parity_fp32(p):
    import torch

    omega = 250.0
    op, J, rng = _pair(4, p, omega, seed=3)
    x = _crandn(rng, op.ndof)
    xr = torch.tensor(x.real, dtype=torch.float32, device="cuda")
    xi = torch.tensor(x.imag, dtype=torch.float32, device="cuda")
    yr, yi = torch.empty_like(xr), torch.empty_like(xi)
    op.MultComplexDevice(omega, xr, xi, yr, yi)
    torch.cuda.synchronize()
    y = yr.double().cpu().numpy() + 1j * yi.double().cpu().numpy()
    x32 = xr.double().cpu().numpy() + 1j * xi.double().cpu().numpy()
    yref = J @ x32
    assert np.linalg.norm(y - yref) / np.linalg.norm(yref) < TOL32


def test_complex_apply_omega_zero_is_curlcurl():
    op, J, rng = _pair(3, 2, 0.0, seed=5)
    x = _crandn(rng, op.ndof)
    y = op.MultComplex(0.0, x)
    assert np.linalg.norm(y - J @ x) / np.linalg.norm(J @ x) < TOL64


@pytest.mark.parametrize("p,omega", [(1, 1e2), (2, 1e3), (3, 1e4)])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_rr"])
def test_complex_solve_matches_direct(p, omega, precision):
    op, J, rng = _pair(3, p, omega, seed=10 + p)
    b = _crandn(rng, op.ndof)
    x_lu = CR.direct_solve(J, b)
    s = GpuComplexCOCGSolver({"Tolerance": 1e-12, "MaxIter": 20000, "Precision": precision}, op, omega)
    x = np.zeros(op.ndof, dtype=np.complex128)
    s.Mult(b, x)
    r = s.result
    assert r["status"] == "OK", r
    assert np.linalg.norm(x - x_lu) / np.linalg.norm(x_lu) < 1e-9, r
    assert np.linalg.norm(b - J @ x) / np.linalg.norm(b) < 1e-11, r


def test_complex_solve_device_and_initial_guess():
    import torch

    omega = 5e2
    op, J, rng = _pair(4, 1, omega, seed=21)
    b = _crandn(rng, op.ndof)
    x_lu = CR.direct_solve(J, b)
    s = GpuComplexCOCGSolver({"Tolerance": 1e-12, "MaxIter": 20000}, op, omega)
    br = torch.tensor(b.real, device="cuda")
    bi = torch.tensor(b.imag, device="cuda")
    # start from the exact solution: zero iterations
    xr = torch.tensor(x_lu.real, device="cuda")
    xi = torch.tensor(x_lu.imag, device="cuda")
    s.MultDevice(br, bi, xr, xi)
    assert s.result["status"] == "OK"
    assert s.result["iterations"] <= 1
    xr.zero_()
    xi.zero_()
    s.MultDevice(br, bi, xr, xi)
    x = xr.cpu().numpy() + 1j * xi.cpu().numpy()
    assert np.linalg.norm(x - x_lu) / np.linalg.norm(x_lu) < 1e-9


def test_complex_entry_points_reject_bad_input():
    op, _, _ = _pair(2, 1, 1.0)
    L = N.lib()
    x = np.zeros(2 * op.ndof)
    y = np.zeros(2 * op.ndof)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    assert L.hc_mult_complex(op.h, -1.0, p(x), p(y)) == N.HC_EINVAL
    assert L.hc_mult_complex(op.h, float("nan"), p(x), p(y)) == N.HC_EINVAL
    assert L.hc_mult_complex(op.h, 1.0, None, p(y)) == N.HC_EINVAL
    prm = N.SolveParams()
    prm.precision = N.HC_FP64
    prm.precond = N.HC_PRECOND_CHEBYSHEV
    prm.cheb_degree = 2
    prm.rtol, prm.atol, prm.maxit = 1e-10, 0.0, 10
    info = N.SolveInfo()
    assert L.hc_solve_complex(op.h, C.byref(prm), 1.0, p(x), p(y), C.byref(info)) == N.HC_ENOTSUP
    assert "Jacobi" in N.last_error(op.h)
    v, t, bt, ba = meshes.kuhn_mesh(2)
    top = HCurlOperator.from_tets(v, t, 1, np.ones(len(t)), np.ones(len(t)), btris=bt, battr=ba)
    xt = np.zeros(2 * top.ndof)
    yt = np.zeros(2 * top.ndof)
    assert L.hc_mult_complex(top.h, 1.0, p(xt), p(yt)) == N.HC_ENOTSUP


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_rr"])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_graph_solve_matches_direct_and_reuses_graph(precision, p):
    import torch

    omega = 2e3
    op, J, rng = _pair(3, p, omega, seed=30 + p)
    s = GpuComplexCOCGSolver({"Tolerance": 1e-12, "MaxIter": 20000, "Precision": precision}, op, omega)
    br = torch.empty(op.ndof, dtype=torch.float64, device="cuda")
    bi, xr, xi = torch.empty_like(br), torch.empty_like(br), torch.empty_like(br)
    for rep in range(2):   # second solve replays the same graph with a new right-hand side
        b = _crandn(rng, op.ndof)
        br.copy_(torch.from_numpy(b.real))
        bi.copy_(torch.from_numpy(b.imag))
        xr.zero_()
        xi.zero_()
        s.MultGraph(br, bi, xr, xi)
        r = s.Finish()
        assert r["status"] == "OK", (rep, r)
        x = xr.cpu().numpy() + 1j * xi.cpu().numpy()
        x_lu = CR.direct_solve(J, b)
        assert np.linalg.norm(x - x_lu) / np.linalg.norm(x_lu) < 1e-9, (rep, r)
        assert r["rel_residual"] < 1e-11


def test_graph_solve_stops_at_maxit():
    import torch

    omega = 10.0
    op, J, rng = _pair(4, 2, omega, seed=41)
    b = _crandn(rng, op.ndof)
    for precision in ("fp64", "mixed", "mixed_rr"):
        s = GpuComplexCOCGSolver({"Tolerance": 1e-14, "MaxIter": 7, "Precision": precision}, op, omega)
        br = torch.tensor(b.real, device="cuda")
        bi = torch.tensor(b.imag, device="cuda")
        xr, xi = torch.zeros_like(br), torch.zeros_like(bi)
        s.MultGraph(br, bi, xr, xi)
        r = s.Finish()
        assert r["status"] == "NOT_CONVERGED", r
        assert r["iterations"] <= 7, r


def test_batch_of_uneven_problems_matches_each_alone():
    import torch

    from hephaestus_gb300.operator import solve_complex_batch

    cases = [(3, 1, 50.0), (4, 2, 3e3), (2, 3, 1e4), (5, 1, 7e2)]
    ops, solvers, rhs, sols, refs, streams = [], [], [], [], [], []
    for k, (n, p, omega) in enumerate(cases):
        op, J, rng = _pair(n, p, omega, seed=50 + k)
        st = torch.cuda.Stream()
        op.set_stream(st)
        streams.append(st)
        b = _crandn(rng, op.ndof)
        refs.append(CR.direct_solve(J, b))
        ops.append(op)
        solvers.append(GpuComplexCOCGSolver({"Tolerance": 1e-12, "MaxIter": 20000, "Precision": "mixed"}, op, omega))
        rhs.append((torch.tensor(b.real, device="cuda"), torch.tensor(b.imag, device="cuda")))
        sols.append((torch.zeros(op.ndof, dtype=torch.float64, device="cuda"),
                     torch.zeros(op.ndof, dtype=torch.float64, device="cuda")))
    torch.cuda.synchronize()
    res = solve_complex_batch(solvers, rhs, sols)
    for k in range(len(cases)):
        assert res[k]["status"] == "OK", (k, res[k])
        x = sols[k][0].cpu().numpy() + 1j * sols[k][1].cpu().numpy()
        assert np.linalg.norm(x - refs[k]) / np.linalg.norm(refs[k]) < 1e-9, (k, res[k])


def test_config4_sized_batch_equals_each_member_alone():
    """Members drawn as config 4 draws them (nu = 10^U(0,3), sigma = 10^U(-2,6),
    coil right-hand side), including a 32^3 order-2 member (300 k complex dofs):
    solved together (hc_solve_complex_batch, each on its own stream) and each
    alone (the same graph-driven solve), mixed precision with the
    auxiliary-space preconditioner; the small member is also checked against
    the oracle's SuperLU solve."""
    import torch

    from hephaestus_gb300 import batch as B
    from hephaestus_gb300.operator import solve_complex_batch

    probs = [B.Problem(32, 2, 3.0e4, 101), B.Problem(12, 3, 2.0e3, 102), B.Problem(9, 1, 4.0e2, 103)]
    params = {"Tolerance": 1e-10, "AbsTolerance": 0.0, "MaxIter": 20000, "Precision": "mixed",
              "Preconditioner": "aux", "InnerTolerance": 3e-4}
    db = B.DeviceBatch(probs, params)
    try:
        res = db.solve()
        assert all(r["status"] == "OK" for r in res), res
        together = db.solutions()
        for k in range(len(probs)):
            db.zero()
            res1 = solve_complex_batch([db.solvers[k]], [db.rhs[k]], [db.sols[k]])
            assert res1[0]["status"] == "OK", res1
            xr, xi = db.sols[k]
            ar, ai = together[k]
            d = torch.sqrt(torch.sum((xr - ar) ** 2 + (xi - ai) ** 2)) / torch.sqrt(torch.sum(xr ** 2 + xi ** 2))
            assert float(d) <= 1e-10, (k, float(d))
        # the 9^3 order-1 member against SuperLU on the oracle's matrices
        pb = probs[2]
        rng = np.random.default_rng(pb.seed)
        ne = pb.n ** 3
        nu = meshes.loguniform(ne, 1.0, 1e3, rng)
        sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
        P = oracle.Problem.hex(pb.n, pb.n, pb.n, pb.p)
        Cn, M = CR.forms(P, nu, sigma)
        J = CR.eliminated(Cn, M, pb.omega, db.ops[2].ess_mask())
        b = db.rhs[2][0].cpu().numpy()
        x_ref = CR.direct_solve(J, b)
        x = together[2][0].cpu().numpy() + 1j * together[2][1].cpu().numpy()
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-8
    finally:
        db.close()
