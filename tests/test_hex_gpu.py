"""GPU parity of the structured-hex Nedelec operator and solvers against the
FP64 oracle (CSR assembly + SpMV + textbook PCG), through the C ABI."""
import numpy as np
import pytest

import oracle
from hephaestus_gb300 import GpuHCurlPCGSolver, HCurlOperator, meshes
from tests import hexref

pytestmark = pytest.mark.gpu

TOL64 = 1e-12   # FP64 apply, relative 2-norm
TOL32 = 2e-6    # FP32 apply, relative 2-norm


def _sheared(n):
    v = meshes.box_vertices(n, n, n)
    A = np.array([[1.0, 0.2, 0.1], [0.0, 0.9, -0.15], [0.05, 0.0, 1.1]])
    return v @ A.T


def _pair(n, p, shear=False, mass=True, bits=0x3F, seed=0, dt=0.01):
    rng = np.random.default_rng(seed)
    ne = n ** 3
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng) if mass else None
    verts = _sheared(n) if shear else None
    op = HCurlOperator(n, n, n, p, nu, sigma, dt=dt, vertices=verts, ess_attr_bits=bits)
    ref = oracle.Problem.hex(n, n, n, p, verts)
    ref.set_coef(dt * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    return op, ref, rng


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("shear", [False, True])
def test_apply_parity_fp64(p, shear):
    op, ref, rng = _pair(3, p, shear)
    x = rng.standard_normal(op.ndof)
    y = op.ApplyForm(x)
    yr = ref.apply(x)
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < TOL64
    ym = op.Mult(x)
    ymr = ref.apply_masked(x)
    assert np.linalg.norm(ym - ymr) / np.linalg.norm(ymr) < TOL64


@pytest.mark.parametrize("p", [1, 2, 3])
def test_apply_parity_fp32(p):
    import torch

    op, ref, rng = _pair(4, p)
    x = rng.standard_normal(op.ndof)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.empty_like(xd)
    op.MultDevice(xd, yd)
    torch.cuda.synchronize()
    y = yd.double().cpu().numpy()
    yr = ref.apply_masked(x.astype(np.float32).astype(np.float64))
    assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < TOL32


@pytest.mark.parametrize("p", [1, 2])
def test_diag_parity(p):
    op, ref, _ = _pair(3, p, shear=True)
    d = op.Diagonal()
    dr = ref.diag_masked()
    assert np.abs(d - dr).max() / np.abs(dr).max() < TOL64


def test_ess_mask_matches_oracle_faces():
    for bits in (0x3F, 0b000101, 0b110000):
        op, ref, _ = _pair(3, 2, bits=bits)
        assert np.array_equal(op.ess_mask(), ref.hex_ess_mask(bits))


def test_weak_curlcurl_parity():
    op, ref, rng = _pair(3, 2, mass=True, dt=0.05)
    u = rng.standard_normal(op.ndof)
    lf = rng.standard_normal(op.ndof)
    lf0 = lf.copy()
    op.AddWeakCurlCurl(u, lf, -1.0)
    # C_nu u with the oracle: alpha = nu (no dt), no mass
    ref.set_coef(op._nu, None)
    ref.assemble()
    want = lf0 - ref.apply(u)
    assert np.linalg.norm(lf - want) / np.linalg.norm(want) < TOL64


@pytest.mark.parametrize("p", [1, 2])
def test_curl_of_gradient_vanishes_on_device(p):
    n = 4
    rng = np.random.default_rng(5)
    op = HCurlOperator(n, n, n, p, rng.uniform(0.5, 2, n ** 3), None, dt=1.0, vertices=_sheared(n),
                       ess_attr_bits=0)
    phi = rng.standard_normal((n * p + 1,) * 3)
    g = hexref.discrete_gradient(n, n, n, p, phi)
    y = op.ApplyForm(g)
    assert np.linalg.norm(y) < 1e-11 * np.linalg.norm(g) * np.abs(op._nu).max() * 10


@pytest.mark.parametrize("p", [1, 2])
def test_apply_parity_across_block_boundaries(p):
    """A grid whose apply spans several thread blocks in x (> 32 elements), y
    and z, so that dofs shared between blocks are combined across them:
    masked and unmasked forms, overwrite (y = J x) and accumulate
    (y += P K P x) forms, FP64 and FP32, against the oracle."""
    import torch

    nx, ny, nz = 37, 9, 11
    rng = np.random.default_rng(11)
    ne = nx * ny * nz
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    op = HCurlOperator(nx, ny, nz, p, nu, sigma, dt=0.01, ess_attr_bits=0x2D)
    ref = oracle.Problem.hex(nx, ny, nz, p)
    ref.set_coef(0.01 * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    x = rng.standard_normal(op.ndof)
    yf = ref.apply(x)
    assert np.linalg.norm(op.ApplyForm(x) - yf) / np.linalg.norm(yf) < TOL64
    ym = ref.apply_masked(x)
    assert np.linalg.norm(op.Mult(x) - ym) / np.linalg.norm(ym) < TOL64
    free = op.ess_mask() == 0
    for dt in (torch.float64, torch.float32):
        xd = torch.tensor(x, dtype=dt, device="cuda")
        yd = torch.empty_like(xd)
        op.MultDevice(xd, yd)
        y0 = rng.standard_normal(op.ndof)
        ya = torch.tensor(y0, dtype=dt, device="cuda")
        op.AddMultDevice(xd, ya)  # y0 + P K P x on free rows, y0 on essential rows
        torch.cuda.synchronize()
        tol = TOL64 if dt == torch.float64 else TOL32
        xr = x if dt == torch.float64 else x.astype(np.float32).astype(np.float64)
        want = ref.apply_masked(xr)
        assert np.linalg.norm(yd.double().cpu().numpy() - want) / np.linalg.norm(want) < tol
        want_add = y0 + np.where(free, want, 0.0)
        got = ya.double().cpu().numpy()
        assert np.linalg.norm(got - want_add) / np.linalg.norm(want_add) < tol


def test_symmetry_and_linearity_fp64():
    op, _, rng = _pair(6, 2)
    x, z = rng.standard_normal(op.ndof), rng.standard_normal(op.ndof)
    Jx, Jz = op.Mult(x), op.Mult(z)
    assert abs(z @ Jx - x @ Jz) < 1e-12 * np.linalg.norm(Jx) * np.linalg.norm(z)
    J2 = op.Mult(2.5 * x - z)
    assert np.linalg.norm(J2 - (2.5 * Jx - Jz)) < 1e-12 * np.linalg.norm(J2)


def _rhs(op, ref, p):
    b = ref.load_coil(q=p + 2)
    b[op.ess_mask() == 1] = 0.0
    return b


@pytest.mark.parametrize("precond", ["jacobi", "chebyshev"])
def test_pcg_fp64_matches_oracle(precond):
    op, ref, _ = _pair(5, 2)
    b = _rhs(op, ref, 2)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "MaxIter": 20000, "Preconditioner": precond,
                           "ChebyshevDegree": 3}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "OK", s.result
    xr, st, it, rr = ref.pcg(b, precond=1, rtol=1e-13, maxit=100000)
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-9
    r = b - ref.apply_masked(x)
    assert np.linalg.norm(r) / np.linalg.norm(b) < 5e-12  # recursive vs true residual gap


def test_pcg_iterates_match_oracle_iteration_counts():
    op, ref, _ = _pair(4, 1)
    b = _rhs(op, ref, 1)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-10, "MaxIter": 20000}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    xr, st, it, rr = ref.pcg(b, precond=1, rtol=1e-10, maxit=20000)
    assert abs(s.result["iterations"] - it) <= max(2, it // 50)


def test_mixed_precision_reaches_fp64_accuracy():
    op, ref, _ = _pair(6, 2)
    b = _rhs(op, ref, 2)
    xr, st, it, rr = ref.pcg(b, precond=1, rtol=1e-14, maxit=200000)
    s = GpuHCurlPCGSolver({"Precision": "mixed", "Tolerance": 1e-12, "MaxIter": 200000,
                           "InnerTolerance": 1e-4}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "OK", s.result
    assert s.result["outer_iterations"] >= 2
    assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-10


@pytest.mark.parametrize("precond", ["jacobi", "aux"])
def test_residual_replacement_reaches_fp64_accuracy(precond):
    """One FP32 PCG with FP64 residual replacement: the solution matches the
    oracle's FP64 PCG to 1e-10, it replaced its residual more than once, and
    its iteration count stays within 1.5x of the FP64 solve's (the Krylov
    space is not restarted; FP32 rounding still costs iterations on this
    problem's 4,000-iteration Jacobi solve)."""
    op, ref, _ = _pair(6, 2)
    b = _rhs(op, ref, 2)
    xr, st, it, rr = ref.pcg(b, precond=1, rtol=1e-14, maxit=200000)
    res = {}
    for prec in ("fp64", "mixed_rr"):
        s = GpuHCurlPCGSolver({"Precision": prec, "Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 200000,
                               "Preconditioner": precond}, op)
        x = np.zeros(op.ndof)
        s.Mult(b, x)
        assert s.result["status"] == "OK", s.result
        assert np.linalg.norm(x - xr) / np.linalg.norm(xr) < 1e-10, prec
        res[prec] = s.result
    assert res["mixed_rr"]["outer_iterations"] >= 2
    assert res["mixed_rr"]["iterations"] <= 1.5 * res["fp64"]["iterations"] + 25, res


def test_residual_replacement_status_on_iteration_cap():
    op, ref, _ = _pair(4, 2)
    b = _rhs(op, ref, 2)
    s = GpuHCurlPCGSolver({"Precision": "mixed_rr", "Tolerance": 1e-14, "AbsTolerance": 0.0, "MaxIter": 7}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "NOT_CONVERGED" and s.result["iterations"] == 7, s.result
    # the FP32 correction of those 7 iterations is in x: its true residual is the reported one
    r = np.linalg.norm(b - op.Mult(x)) / np.linalg.norm(b)
    assert abs(r - s.result["rel_residual"]) <= 1e-6 * r and r < 1.0


def test_lanczos_bound_matches_oracle():
    op, ref, _ = _pair(4, 2)
    lg = op.LanczosLmax(20)
    lo = ref.lanczos_lmax(20)
    assert abs(lg - lo) / lo < 1e-6


def test_breakdown_and_nonconvergence_statuses():
    op, ref, _ = _pair(4, 2)
    b = _rhs(op, ref, 2)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-14, "MaxIter": 3}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "NOT_CONVERGED" and s.result["iterations"] == 3
    bad = b.copy()
    bad[5] = np.nan
    s2 = GpuHCurlPCGSolver({"Tolerance": 1e-10, "MaxIter": 50}, op)
    x = np.zeros(op.ndof)
    s2.Mult(bad, x)
    assert s2.result["status"] == "BREAKDOWN"


def test_non_affine_hex_rejected():
    n = 2
    v = meshes.box_vertices(n, n, n).copy()
    v[13] += 0.05  # move the centre vertex: trilinear, not affine
    with pytest.raises(Exception) as e:
        HCurlOperator(n, n, n, 1, np.ones(8), None, vertices=v)
    assert "parallelepiped" in str(e.value)


def test_add_mult_device_accumulates():
    import torch

    op, ref, rng = _pair(4, 2)
    x = rng.standard_normal(op.ndof)
    y0 = rng.standard_normal(op.ndof)
    m = op.ess_mask() == 1
    want = y0 + np.where(m, 0.0, ref.apply_masked(np.where(m, 0.0, x)))
    xd = torch.tensor(x, device="cuda")
    yd = torch.tensor(y0, device="cuda")
    op.AddMultDevice(xd, yd)
    torch.cuda.synchronize()
    got = yd.cpu().numpy()
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < TOL64


def _pair_box(nx, ny, nz, p, bits=0x3F, mask=None, shear=False, seed=7):
    rng = np.random.default_rng(seed)
    ne = nx * ny * nz
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    v = meshes.box_vertices(nx, ny, nz)
    if shear:
        v = v @ np.array([[1.0, 0.1, 0.0], [0.05, 1.0, 0.1], [0.0, -0.1, 1.0]]).T
    op = HCurlOperator(nx, ny, nz, p, nu, sigma, dt=0.01, vertices=v, ess_attr_bits=bits, ess_mask=mask)
    ref = oracle.Problem.hex(nx, ny, nz, p, v)
    ref.set_coef(0.01 * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    return op, ref, rng


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("shear", [False, True])
@pytest.mark.parametrize("bits", [0x3F, 0b011001])
def test_apply_parity_full_bricks(p, shear, bits):
    """Grids that are whole multiples of the kernel's brick (fast path) plus a
    ragged one; FP64 and FP32, masked and unmasked."""
    import torch

    for dims in ((32, 8, 4), (33, 9, 5)):
        op, ref, rng = _pair_box(*dims, p, bits=bits, shear=shear)
        x = rng.standard_normal(op.ndof)
        yr = ref.apply_masked(x)
        y = op.Mult(x)
        assert np.linalg.norm(y - yr) / np.linalg.norm(yr) < TOL64
        assert np.linalg.norm(op.ApplyForm(x) - ref.apply(x)) / np.linalg.norm(ref.apply(x)) < TOL64
        xd = torch.tensor(x, dtype=torch.float32, device="cuda")
        yd = torch.empty_like(xd)
        op.MultDevice(xd, yd)
        torch.cuda.synchronize()
        y32r = ref.apply_masked(x.astype(np.float32).astype(np.float64))
        assert np.linalg.norm(yd.double().cpu().numpy() - y32r) / np.linalg.norm(y32r) < TOL32


@pytest.mark.parametrize("p", [1, 2])
def test_apply_parity_explicit_mask(p):
    nx, ny, nz = 32, 8, 4
    from hephaestus_gb300 import meshes as M

    nd = M.hex_ndof(nx, ny, nz, p) if nx == ny == nz else None
    probe = HCurlOperator(nx, ny, nz, p, np.ones(nx * ny * nz), None, ess_attr_bits=0)
    rng = np.random.default_rng(9)
    mask = (rng.random(probe.ndof) < 0.1).astype(np.uint8)
    probe.close()
    op, ref, rng = _pair_box(nx, ny, nz, p, bits=0, mask=mask)
    assert np.array_equal(op.ess_mask(), mask)
    x = rng.standard_normal(op.ndof)
    yr = ref.apply_masked(x)
    assert np.linalg.norm(op.Mult(x) - yr) / np.linalg.norm(yr) < TOL64
    del nd


@pytest.mark.parametrize("p", [1, 2, 3])
def test_curl_matches_oracle(p):
    """B = curl A (CurlAuxSolver) against the oracle's curl at element centres."""
    n = 3
    v = _sheared(n)
    op = HCurlOperator(n, n, n, p, np.ones(n ** 3), None, vertices=v, ess_attr_bits=0)
    ref = oracle.Problem.hex(n, n, n, p, v)
    rng = np.random.default_rng(11)
    A = rng.standard_normal(op.ndof)
    B = op.Curl(A)
    assert B.shape == (3 * (n * p + 1) * (n * p) ** 2,)
    for e in (0, 7, 13, 26):
        xi = np.array([0.5, 0.3, 0.7])
        _, cref = ref.eval(A, e, xi)
        bref = hexref.rt_eval_ref(B, n, n, n, p, e, xi)
        ex, ey, ez = e % n, (e // n) % n, e // (n * n)
        vid = lambda i, j, k: i + (n + 1) * (j + (n + 1) * k)  # noqa: E731
        v0 = v[vid(ex, ey, ez)]
        J = np.stack([v[vid(ex + 1, ey, ez)] - v0, v[vid(ex, ey + 1, ez)] - v0, v[vid(ex, ey, ez + 1)] - v0], axis=1)
        bphys = J @ bref / np.linalg.det(J)
        assert np.allclose(bphys, cref, rtol=1e-11, atol=1e-11 * np.abs(cref).max())


def test_curl_of_gradient_is_zero_rt():
    n, p = 4, 2
    op = HCurlOperator(n, n, n, p, np.ones(n ** 3), None, vertices=_sheared(n), ess_attr_bits=0)
    phi = np.random.default_rng(12).standard_normal((n * p + 1,) * 3)
    B = op.Curl(hexref.discrete_gradient(n, n, n, p, phi))
    assert np.abs(B).max() < 1e-12 * np.abs(phi).max() * 10


@pytest.mark.parametrize("p,q", [(1, 3), (2, 4), (3, 5)])
def test_load_coil_matches_oracle(p, q):
    n = 6
    op = HCurlOperator(n, n, n, p, np.ones(n ** 3), np.ones(n ** 3), ess_attr_bits=0)
    ref = oracle.Problem.hex(n, n, n, p)
    b = op.LoadCoil(I0=1.5, xc=0.45, yc=0.55, q=q)
    br = ref.load_coil(I0=1.5, xc=0.45, yc=0.55, q=q)
    assert np.linalg.norm(b - br) / np.linalg.norm(br) < 1e-13
