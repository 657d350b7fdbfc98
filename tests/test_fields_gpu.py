"""GPU parity, through the C ABI, of the work around the solve against the
FP64 oracle: source loads (J, w_i) for a caller-supplied J, the
(nu curl A, w_i) load and the H = nu curl A projection, curl on tets,
backward-Euler steps on device state, and the magnetostatic (sigma = 0)
solve."""
import numpy as np
import pytest

import oracle
from hephaestus_gb300 import GpuHCurlPCGSolver, HCurlOperator, meshes
from tests import oracle_ref as R

pytestmark = pytest.mark.gpu

TOL = 1e-12  # loads and curls: same integrals, FP64, relative 2-norm


def _dev(a):
    import torch

    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _host(t):
    import torch

    torch.cuda.synchronize()
    return t.cpu().numpy()


def _sheared(n):
    v = meshes.box_vertices(n, n, n)
    A = np.array([[1.0, 0.2, 0.1], [0.0, 0.9, -0.15], [0.05, 0.0, 1.1]])
    return v @ A.T


def _hex(n, p, shear=False, seed=0, mass=True, dt=0.01, nu_range=(1.0, 1e3), sig_range=(1e-2, 1e6)):
    rng = np.random.default_rng(seed)
    ne = n ** 3
    nu = meshes.loguniform(ne, *nu_range, rng)
    sigma = meshes.loguniform(ne, *sig_range, rng) if mass else None
    verts = _sheared(n) if shear else None
    op = HCurlOperator(n, n, n, p, nu, sigma, dt=dt, vertices=verts, ess_attr_bits=0x3F)
    ref = oracle.Problem.hex(n, n, n, p, verts)
    ref.set_coef(dt * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    return op, ref, nu, rng


def _tet(n, p, seed=0, dt=0.01):
    v, t, bt, ba = meshes.kuhn_mesh(n, jitter=0.15, seed=seed)
    rng = np.random.default_rng(seed)
    ne = len(t)
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    op = HCurlOperator.from_tets(v, t, p, nu, sigma, dt=dt, btris=bt, battr=ba, ess_attr_bits=0x3F)
    ref = oracle.Problem.tet(v, t, p)
    ref.set_coef(dt * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    return op, ref, nu, rng, (v, t)


def _make(kind, p):
    if kind == "hex":
        op, ref, nu, rng = _hex(3, p)
    elif kind == "hex_sheared":
        op, ref, nu, rng = _hex(3, p, shear=True)
    else:
        op, ref, nu, rng, _ = _tet(3, p)
    return op, ref, nu, rng


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


CASES = [("hex", 1), ("hex", 2), ("hex_sheared", 2), ("hex", 3), ("tet", 1), ("tet", 2)]


@pytest.mark.parametrize("kind,p", CASES)
def test_load_field_per_element_matches_oracle(kind, p):
    import torch

    op, ref, _, rng = _make(kind, p)
    J = rng.standard_normal((op.ne, 3))
    q = p + 2
    b = torch.empty(op.ndof, dtype=torch.float64, device="cuda")
    op.LoadFieldDevice(_dev(J), b, q=q)
    assert _rel(_host(b), ref.load_elem_field(J, q=q)) < TOL


@pytest.mark.parametrize("kind,p", CASES)
def test_load_field_at_points_matches_oracle(kind, p):
    """J(x) = a + B x evaluated at the library's quadrature points; the oracle
    integrates the same affine field with its own rule (both exact)."""
    import torch

    op, ref, _, rng = _make(kind, p)
    a, B = rng.standard_normal(3), rng.standard_normal((3, 3))
    q = p + 2
    xyz = op.QuadPointsDevice(q)
    J = _dev(a) + xyz @ _dev(B).T
    b = torch.empty(op.ndof, dtype=torch.float64, device="cuda")
    op.LoadFieldDevice(J.contiguous(), b)
    # (the affine field makes the integral depend on where the points are, so
    # this also checks the points)
    assert _rel(_host(b), ref.load_affine(a, B, q=q)) < TOL


@pytest.mark.parametrize("kind,p", CASES)
def test_curl_load_matches_oracle(kind, p):
    import torch

    op, ref, nu, rng = _make(kind, p)
    A = rng.standard_normal(op.ndof)
    b = torch.empty(op.ndof, dtype=torch.float64, device="cuda")
    op.CurlLoadDevice(_dev(A), b)
    assert _rel(_host(b), ref.curl_load(nu, A, q=p + 3)) < TOL


@pytest.mark.parametrize("kind,p", [("hex", 2), ("hex_sheared", 1), ("tet", 2)])
def test_magnetic_field_projection_matches_oracle(kind, p):
    """H = nu curl A in the Nedelec space: M H = (nu curl A, w), M the
    unit-coefficient mass (the oracle's, solved directly)."""
    import torch

    op, ref, nu, rng = _make(kind, p)
    A = rng.standard_normal(op.ndof)
    H = torch.zeros(op.ndof, dtype=torch.float64, device="cuda")
    res = op.MagneticFieldDevice(_dev(A), H, rtol=1e-13)
    assert res["status"] == "OK", res
    if kind == "tet":
        v, t = _tet(3, p)[4]
        m = oracle.Problem.tet(v, t, p)
    else:
        n = 3
        m = oracle.Problem.hex(n, n, n, p, _sheared(n) if kind == "hex_sheared" else None)
    m.set_coef(np.zeros(op.ne), np.ones(op.ne))
    m.assemble()
    Href = R.direct_solve(m.csr().tocsc(), ref.curl_load(nu, A, q=p + 3))
    assert _rel(_host(H), Href) < 1e-10
    # second call reuses the mass operator and agrees
    H2 = torch.zeros_like(H)
    op.MagneticFieldDevice(_dev(A), H2, rtol=1e-13)
    assert _rel(_host(H2), Href) < 1e-10


@pytest.mark.parametrize("p", [1, 2])
def test_tet_curl_at_points_matches_oracle(p):
    op, ref, _, rng, _ = _tet(3, p)
    A = rng.standard_normal(op.ndof)
    xi = np.array([[0.25, 0.25, 0.25], [0.1, 0.2, 0.3], [0.6, 0.1, 0.1], [0.05, 0.7, 0.2]])
    B = _host(op.TetCurlPointsDevice(_dev(A), xi))
    assert B.shape == (op.ne, 4, 3)
    worst = 0.0
    scale = np.abs(B).max()
    for e in range(0, op.ne, max(1, op.ne // 40)):
        for k in range(len(xi)):
            _, c = ref.eval(A, e, xi[k])
            worst = max(worst, np.abs(B[e, k] - c).max())
    assert worst <= 1e-12 * scale


def test_be_rhs_matches_oracle():
    import torch

    op, ref, _, rng = _hex(4, 2, dt=0.05)
    f = ref.load_coil(q=4)
    A = rng.standard_normal(op.ndof)
    b = torch.empty(op.ndof, dtype=torch.float64, device="cuda")
    op.BeRhsDevice(_dev(f), _dev(A), b)
    br = f - ref.apply_curlcurl(A) / 0.05
    br[op.ess_mask() != 0] = 0.0
    assert _rel(_host(b), br) < TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_be_five_steps_match_oracle(precision):
    """Five backward-Euler steps on device state (hc_be_steps_device) against
    the oracle's five steps with sparse direct solves."""
    import torch

    dt = 0.01
    op, ref, _, rng = _hex(5, 2, dt=dt)
    f = ref.load_coil(q=4)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-13, "AbsTolerance": 0.0, "MaxIter": 20000, "Precision": precision,
                           "Preconditioner": "aux", "InnerTolerance": 1e-4}, op)
    A = torch.zeros(op.ndof, dtype=torch.float64, device="cuda")
    dA = torch.empty_like(A)
    b = torch.empty_like(A)
    steps = s.StepsDevice(_dev(f), A, dA, b, 5)
    assert len(steps) == 5 and all(r["status"] == "OK" for r in steps), steps
    Aref = R.be_steps(ref, f, dt, 5)
    assert _rel(_host(A), Aref) < 1e-10


def test_be_steps_reports_the_failing_step():
    """A 2-iteration budget cannot converge: the loop stops at step 1 and
    reports only that step."""
    import torch

    op, ref, _, _ = _hex(4, 2)
    f = _dev(ref.load_coil(q=4))
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "MaxIter": 2, "Preconditioner": "jacobi"}, op)
    A = torch.zeros(op.ndof, dtype=torch.float64, device="cuda")
    steps = s.StepsDevice(f, A, torch.empty_like(A), torch.empty_like(A), 4)
    assert len(steps) == 1 and steps[0]["status"] == "NOT_CONVERGED"


def test_magnetostatic_sigma0_solve_matches_oracle():
    """sigma = 0 (StaticsOperator::Solve's singular curl-curl, statics_formulation.cpp:131-161)
    with a consistent right-hand side b = J x_true: A is fixed up to discrete
    gradients, so B = curl A is compared -- with curl x_true and with the
    curl of the oracle's PCG solution of the same system."""
    op, ref, nu, rng = _hex(5, 2, mass=False, dt=1.0, nu_range=(1.0, 10.0))
    xt = rng.standard_normal(op.ndof)
    xt[op.ess_mask() != 0] = 0.0
    b = op.Mult(xt)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 20000,
                           "Preconditioner": "jacobi"}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "OK", s.result
    Bt = op.Curl(xt)
    assert _rel(op.Curl(x), Bt) < 1e-8
    xo, st, _, _ = ref.pcg(b, precond=1, rtol=1e-12, maxit=50000)
    assert st == 0
    assert _rel(op.Curl(x), op.Curl(xo)) < 1e-8
    # the solution differs from x_true by a gradient only: same energy
    assert abs(x @ op.ApplyForm(x) - xt @ op.ApplyForm(xt)) <= 1e-8 * (xt @ op.ApplyForm(xt))
