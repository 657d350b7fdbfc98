"""GPU parity at the benchmark configurations, against the FP64 oracle.

* Config 1 exactly: unit cube 16^3 hexes, Nedelec p = 1, nu = 1, dt = 0.01,
  sigma = 1 in [0.25, 0.75]^3 and 1e-6 elsewhere, A x n = 0, loop-coil load,
  FP64 Jacobi PCG to a relative residual of 1e-12 -- against the oracle's
  Jacobi PCG of the same system (test_aform_source.cpp:100-115 solves with
  the reference's PCG; problem_builder_base.hpp:144-150 its defaults) and a
  refined sparse direct solve.  FP64 reproduces this system's solution only
  to ~2e-9 (true-residual floor ~1e-10), so its checks use that spread.
* Config 2's coefficient draws (nu = 10^U(0,3), sigma = 10^U(-2,6) per
  element) on a 10^3 slice at p = 2: FP64 and mixed solves with the
  auxiliary-space preconditioner against the oracle's sparse direct solve;
  and on a 32^3 slice: the oracle's independently assembled operator
  certifies the true residual of the mixed solution, and mixed agrees with
  the FP64-refined FP64 solution within 1e-10.  "mixed" is FP32 PCG inside
  FP64 iterative refinement, "mixed_rr" one FP32 PCG with FP64 residual
  replacement.
* Tets (config 3's mesh family and fields): Kuhn 8^3, p = 2, 16 seeded coil
  right-hand sides solved together (block PCG, mixed precision, tet
  auxiliary-space AMG), column by column against the oracle's direct solve.

Accuracy criterion: ||x - x_ref|| / ||x_ref|| <= 1e-10 per solution.
"""
import numpy as np
import pytest

import oracle
from hephaestus_gb300 import GpuHCurlPCGSolver, HCurlOperator, meshes
from tests import oracle_ref as R

pytestmark = pytest.mark.gpu

XERR = 1e-10


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _config1():
    n, p, dt = 16, 1, 0.01
    ne = n ** 3
    nu = np.ones(ne)
    c = (np.indices((n, n, n))[::-1].reshape(3, -1).T + 0.5) / n  # element centroids, x fastest
    sigma = np.where(np.all((c >= 0.25) & (c <= 0.75), axis=1), 1.0, 1e-6)
    op = HCurlOperator(n, n, n, p, nu, sigma, dt=dt, ess_attr_bits=0x3F)
    ref = oracle.Problem.hex(n, n, n, p)
    ref.set_coef(dt * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    b = op.LoadCoil(q=p + 2)
    b[op.ess_mask() != 0] = 0.0
    return op, ref, b


def _config2_slice(n, seed=0):
    p, dt = 2, 0.01
    rng = np.random.default_rng(seed)
    ne = n ** 3
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    op = HCurlOperator(n, n, n, p, nu, sigma, dt=dt, ess_attr_bits=0x3F)
    ref = oracle.Problem.hex(n, n, n, p)
    ref.set_coef(dt * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    b = op.LoadCoil(q=p + 2)
    b[op.ess_mask() != 0] = 0.0
    return op, ref, b


def _direct_refined(J, b, steps=2):
    """Sparse direct solve with iterative refinement in FP64."""
    import scipy.sparse.linalg as sla

    lu = sla.splu(J)
    x = lu.solve(b)
    for _ in range(steps):
        x = x + lu.solve(b - J @ x)
    return x


def test_config1_fp64_pcg_matches_oracle_pcg():
    """Config 1 is conditioned so that FP64 itself reproduces x only to ~2e-9:
    the true residual of any FP64 solution bottoms out near 1e-10
    (eps_64 ||J|| ||x|| / ||b||), and PCG's recursive residual drifts below
    its true one (the oracle's PCG reports 1e-12 at a true 1.8e-9).  The GPU's
    FP64 Jacobi PCG must behave as the oracle's: same iterations, same
    solution within that spread, same true residual."""
    op, ref, b = _config1()
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 20000,
                           "Preconditioner": "jacobi"}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    res = s.result
    assert res["status"] == "OK", res
    xo, st, it_o, _ = ref.pcg(b, precond=1, rtol=1e-12, maxit=20000)
    assert st == 0
    # same algorithm and start, different summation orders (the GPU's face
    # atomics also change order from run to run): over ~3,000 iterations on
    # this conditioning, with the recursive residual below the true one at
    # the end, the counts drift apart by up to ~7 % (2,813 against 3,013 seen)
    assert abs(res["iterations"] - it_o) <= 0.10 * it_o, (res["iterations"], it_o)
    J = R.eliminated(ref)
    rr = lambda v: np.linalg.norm(b - J @ v) / np.linalg.norm(b)  # noqa: E731
    assert rr(x) <= 3.0 * rr(xo) + 1e-12, (rr(x), rr(xo))
    xt = _direct_refined(J, b, steps=3)
    assert _rel(x, xt) <= 1e-8 and _rel(xo, xt) <= 1e-8, (_rel(x, xt), _rel(xo, xt))
    # B = curl A (the configuration's second output)
    assert _rel(op.Curl(x), op.Curl(xt)) <= 1e-8


def _inner(precision):
    """Inner setting: refinement tolerance, or the residual reduction between
    replacements of the residual-replacement solve."""
    return 0.1 if precision == "mixed_rr" else 3e-4


@pytest.mark.parametrize("precision", ["mixed", "mixed_rr"])
def test_config1_mixed_meets_the_fp64_floor(precision):
    """Mixed precision on config 1 (the FP32 iteration stalls on the air
    region, the FP64 polish finishes) reaches the FP64 true-residual floor,
    certified by the oracle's operator, and the FP64 solution within FP64's
    own spread."""
    op, ref, b = _config1()
    s = GpuHCurlPCGSolver({"Tolerance": 3e-10, "AbsTolerance": 0.0, "MaxIter": 40000, "Precision": precision,
                           "Preconditioner": "aux"}, op)
    xm = np.zeros(op.ndof)
    s.Mult(b, xm)
    assert s.result["status"] == "OK", s.result
    J = R.eliminated(ref)
    assert np.linalg.norm(b - J @ xm) / np.linalg.norm(b) <= 3e-10
    xt = _direct_refined(J, b, steps=3)
    assert _rel(xm, xt) <= 1e-8, _rel(xm, xt)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_rr"])
def test_config2_slice10_matches_oracle_direct(precision):
    op, ref, b = _config2_slice(10)
    xd = _direct_refined(R.eliminated(ref), b)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 20000, "Precision": precision,
                           "Preconditioner": "aux", "InnerTolerance": _inner(precision)}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "OK", s.result
    assert _rel(x, xd) <= XERR, (_rel(x, xd), s.result)


@pytest.mark.parametrize("precision", ["mixed", "mixed_rr"])
def test_config2_slice32_mixed_certified_by_oracle_operator(precision):
    """32^3 slice: the mixed solve's true residual, computed with the oracle's
    independently assembled operator, meets its tolerance, and the solution
    is within 1e-10 of the FP64 solution refined in FP64 (true residuals)."""
    import torch

    op, ref, b = _config2_slice(32)
    bd = torch.tensor(b, device="cuda")

    def fp64(rhs, tol):
        x = torch.zeros_like(rhs)
        s = GpuHCurlPCGSolver({"Tolerance": tol, "AbsTolerance": 0.0, "MaxIter": 20000, "Preconditioner": "aux"}, op)
        s.MultDevice(rhs, x)
        return x

    xt = fp64(bd, 1e-12)
    for _ in range(3):
        r = torch.empty_like(bd)
        op.MultDevice(xt, r)
        xt += fp64(bd - r, 1e-8)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-11, "AbsTolerance": 0.0, "MaxIter": 20000, "Precision": precision,
                           "Preconditioner": "aux", "InnerTolerance": _inner(precision)}, op)
    x = torch.zeros_like(bd)
    s.MultDevice(bd, x)
    assert s.result["status"] == "OK", s.result
    xm = x.cpu().numpy()
    r = b - ref.apply_masked(xm)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-11
    assert _rel(xm, xt.cpu().numpy()) <= XERR


def _tets(n, nrhs, seed=0):
    v, t, bt, ba = meshes.kuhn_mesh(n, jitter=0.15, seed=seed)
    rng = np.random.default_rng(seed)
    ne = len(t)
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    op = HCurlOperator.from_tets(v, t, 2, nu, sigma, dt=0.01, btris=bt, battr=ba, ess_attr_bits=0x3F)
    ref = oracle.Problem.tet(v, t, 2)
    ref.set_coef(0.01 * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    crng = np.random.default_rng(1)
    cols = []
    for _ in range(nrhs):
        I0 = crng.uniform(0.5, 2.0)
        xc, yc = 0.5 + crng.uniform(-0.1, 0.1, size=2)
        cols.append(ref.load_coil(I0=I0, xc=xc, yc=yc, q=4))
    B = np.stack(cols, axis=1)
    B[op.ess_mask() != 0, :] = 0.0
    return op, ref, np.ascontiguousarray(B)


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_rr"])
def test_tets8_16rhs_block_solve_matches_oracle_direct(precision):
    import torch

    op, ref, B = _tets(8, 16)
    Xd = _direct_refined(R.eliminated(ref), B)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "AbsTolerance": 0.0, "MaxIter": 40000, "Precision": precision,
                           "Preconditioner": "aux", "InnerTolerance": 0.1}, op)
    X = torch.zeros(op.ndof, 16, dtype=torch.float64, device="cuda")
    res = s.MultMultiDevice(torch.tensor(B, device="cuda"), X)
    assert all(r["status"] == "OK" for r in res), res
    Xh = X.cpu().numpy()
    errs = [_rel(Xh[:, k], Xd[:, k]) for k in range(16)]
    assert max(errs) <= XERR, errs
