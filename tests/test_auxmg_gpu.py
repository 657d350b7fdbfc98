"""GPU tests of the auxiliary-space (gradient) preconditioner HC_PRECOND_AUX:
solutions equal the direct solve of the eliminated system (the preconditioner
changes the iteration, not the answer), and the iteration counts drop where
Jacobi stalls (the gradient near-null space of the curl-curl form)."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle
from oracle import complex_ref as CR
from hephaestus_gb300 import GpuComplexCOCGSolver, GpuHCurlPCGSolver, HCurlOperator, meshes

pytestmark = pytest.mark.gpu


def _sheared(n):
    v = meshes.box_vertices(n, n, n)
    A = np.array([[1.0, 0.2, 0.1], [0.0, 0.9, -0.15], [0.05, 0.0, 1.1]])
    return v @ A.T


def _real_pair(n, p, seed=0, dt=0.01, shear=False, bits=0x3F, mask=None):
    rng = np.random.default_rng(seed)
    ne = n ** 3
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    verts = _sheared(n) if shear else None
    op = HCurlOperator(n, n, n, p, nu, sigma, dt=dt, vertices=verts, ess_attr_bits=bits, ess_mask=mask)
    ref = oracle.Problem.hex(n, n, n, p, verts)
    ref.set_coef(dt * nu, sigma)
    ref.assemble()
    K = ref.csr()
    ess = op.ess_mask()
    free = sp.diags((ess == 0).astype(float))
    J = (free @ K @ free + sp.diags((ess != 0).astype(float))).tocsc()
    return op, J, rng


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_aux_pcg_matches_direct_solve(p, precision):
    op, J, rng = _real_pair(4, p, seed=p)
    b = rng.standard_normal(op.ndof)
    x_ref = spla.spsolve(J, b)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "MaxIter": 20000, "Precision": precision,
                           "Preconditioner": "aux"}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "OK", s.result
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-9, s.result


@pytest.mark.parametrize("p", [1, 2])
def test_aux_pcg_on_sheared_grid_and_partial_boundary(p):
    op, J, rng = _real_pair(4, p, seed=10 + p, shear=True, bits=0x13)
    b = rng.standard_normal(op.ndof)
    x_ref = spla.spsolve(J, b)
    s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "MaxIter": 20000, "Preconditioner": "aux"}, op)
    x = np.zeros(op.ndof)
    s.Mult(b, x)
    assert s.result["status"] == "OK", s.result
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-9


def test_aux_pcg_with_explicit_mask_and_no_boundary():
    n, p = 4, 2
    probe = HCurlOperator(n, n, n, p, np.ones(n ** 3), None, ess_attr_bits=0x3F)
    mask = probe.ess_mask().copy()
    mask[: len(mask) // 3] = 0   # essential on part of the boundary only
    for m, bits in ((mask, 0), (None, 0)):
        op, J, rng = _real_pair(n, p, seed=21, mask=m, bits=bits)
        b = rng.standard_normal(op.ndof)
        x_ref = spla.spsolve(J, b)
        s = GpuHCurlPCGSolver({"Tolerance": 1e-12, "MaxIter": 20000, "Preconditioner": "aux"}, op)
        x = np.zeros(op.ndof)
        s.Mult(b, x)
        assert s.result["status"] == "OK", s.result
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-9


def test_aux_cuts_iterations_where_jacobi_stalls():
    n, p = 8, 2
    rng = np.random.default_rng(3)
    ne = n ** 3
    op = HCurlOperator(n, n, n, p, meshes.loguniform(ne, 1.0, 1e3, rng), meshes.loguniform(ne, 1e-2, 1e6, rng),
                       dt=0.01, ess_attr_bits=0x3F)
    b = np.where(op.ess_mask() != 0, 0.0, op.LoadCoil())
    its = {}
    for pre in ("jacobi", "aux"):
        s = GpuHCurlPCGSolver({"Tolerance": 1e-10, "MaxIter": 4000, "Preconditioner": pre}, op)
        x = np.zeros(op.ndof)
        s.Mult(b, x)
        its[pre] = (s.result["status"], s.result["iterations"])
    assert its["aux"][0] == "OK", its
    assert its["jacobi"][0] != "OK" or its["jacobi"][1] > 5 * its["aux"][1], its


@pytest.mark.parametrize("p", [1, 2, 3])
@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_rr"])
def test_aux_mult_pcg_matches_direct_solve(p, precision):
    """HC_PRECOND_AUX_MULT (Chebyshev-Jacobi smoothing around the gradient
    correction, a symmetric multiplicative cycle) against the oracle's sparse
    direct solve; also with a sheared grid and part of the boundary free.
    (rtol 1e-10: at p = 3 the FP64 true residual of these systems floors
    near 8e-12, and the mixed forms judge convergence on it.)"""
    for kw in ({}, {"shear": True, "bits": 0x13}):
        op, J, rng = _real_pair(4, p, seed=50 + p, **kw)
        b = rng.standard_normal(op.ndof)
        x_ref = spla.spsolve(J, b)
        s = GpuHCurlPCGSolver({"Tolerance": 1e-10, "MaxIter": 20000, "Precision": precision,
                               "Preconditioner": "aux_mult"}, op)
        x = np.zeros(op.ndof)
        s.Mult(b, x)
        assert s.result["status"] == "OK", s.result
        assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-9, s.result


def test_aux_mult_cuts_aux_iterations():
    """On the benchmark's coefficient draws (8^3, p = 2) the multiplicative
    cycle needs well under half of the additive form's iterations."""
    n, p = 8, 2
    rng = np.random.default_rng(3)
    ne = n ** 3
    op = HCurlOperator(n, n, n, p, meshes.loguniform(ne, 1.0, 1e3, rng), meshes.loguniform(ne, 1e-2, 1e6, rng),
                       dt=0.01, ess_attr_bits=0x3F)
    b = np.where(op.ess_mask() != 0, 0.0, op.LoadCoil())
    its, xs = {}, {}
    for pre in ("aux", "aux_mult"):
        s = GpuHCurlPCGSolver({"Tolerance": 1e-10, "AbsTolerance": 0.0, "MaxIter": 4000, "Preconditioner": pre}, op)
        xs[pre] = np.zeros(op.ndof)
        s.Mult(b, xs[pre])
        its[pre] = (s.result["status"], s.result["iterations"])
    assert its["aux"][0] == "OK" and its["aux_mult"][0] == "OK", its
    assert its["aux_mult"][1] < 0.5 * its["aux"][1], its
    assert np.linalg.norm(xs["aux_mult"] - xs["aux"]) / np.linalg.norm(xs["aux"]) < 1e-8


def test_aux_mult_rejected_where_not_built():
    v, t, bt, ba = meshes.kuhn_mesh(2)
    op = HCurlOperator.from_tets(v, t, 1, np.ones(len(t)), np.ones(len(t)), btris=bt, battr=ba, ess_attr_bits=0x3F)
    s = GpuHCurlPCGSolver({"Preconditioner": "aux_mult"}, op)
    with pytest.raises(Exception):
        s.Mult(np.ones(op.ndof), np.zeros(op.ndof))


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_rr"])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_aux_cocg_matches_direct(precision, p):
    import torch

    n, omega = 4, 10.0
    rng = np.random.default_rng(40 + p)
    ne = n ** 3
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    op = HCurlOperator(n, n, n, p, nu, sigma, dt=1.0, ess_attr_bits=0x3F)
    ref = oracle.Problem.hex(n, n, n, p)
    Cn, M = CR.forms(ref, nu, sigma)
    J = CR.eliminated(Cn, M, omega, op.ess_mask())
    b = rng.standard_normal(op.ndof) + 1j * rng.standard_normal(op.ndof)
    x_lu = CR.direct_solve(J, b)
    s = GpuComplexCOCGSolver({"Tolerance": 1e-12, "MaxIter": 30000, "Precision": precision,
                              "Preconditioner": "aux"}, op, omega)
    x = np.zeros(op.ndof, dtype=np.complex128)
    s.Mult(b, x)
    assert s.result["status"] == "OK", s.result
    assert np.linalg.norm(x - x_lu) / np.linalg.norm(x_lu) < 1e-9, s.result
    # graph-driven form with the same preconditioner
    s = GpuComplexCOCGSolver({"Tolerance": 1e-12, "MaxIter": 30000, "Precision": precision,
                              "Preconditioner": "aux"}, op, omega)
    br = torch.tensor(b.real, device="cuda")
    bi = torch.tensor(b.imag, device="cuda")
    xr, xi = torch.zeros_like(br), torch.zeros_like(bi)
    s.MultGraph(br, bi, xr, xi)
    r = s.Finish()
    assert r["status"] == "OK", r
    xg = xr.cpu().numpy() + 1j * xi.cpu().numpy()
    assert np.linalg.norm(xg - x_lu) / np.linalg.norm(x_lu) < 1e-9, r


def test_aux_cocg_converges_at_low_frequency_where_jacobi_stalls():
    n, p, omega = 12, 2, 10.0
    rng = np.random.default_rng(4)
    ne = n ** 3
    op = HCurlOperator(n, n, n, p, meshes.loguniform(ne, 1.0, 1e3, rng), meshes.loguniform(ne, 1e-2, 1e6, rng),
                       dt=1.0, ess_attr_bits=0x3F)
    b = np.where(op.ess_mask() != 0, 0.0, op.LoadCoil()).astype(np.complex128)
    res = {}
    for pre in ("jacobi", "aux"):
        s = GpuComplexCOCGSolver({"Tolerance": 1e-10, "MaxIter": 3000, "Preconditioner": pre}, op, omega)
        x = np.zeros(op.ndof, dtype=np.complex128)
        s.Mult(b, x)
        res[pre] = (s.result["status"], s.result["iterations"])
    assert res["aux"][0] == "OK", res
    assert res["jacobi"][0] != "OK" or res["jacobi"][1] > 3 * res["aux"][1], res


@pytest.mark.parametrize("n, p", [(40, 2), (24, 1), (17, 3)])
def test_cooperative_vcycle_equals_per_step_kernels(n, p, monkeypatch):
    """The Q1 V-cycle's launch forms -- one cooperative launch with grid
    barriers (HC_AUX_VCYCLE=coop: all levels, =hybrid: the levels below the
    finest), the coarse levels in one thread-block cluster (=cluster; with
    n = 17, p = 3 the whole cycle) -- run the same steps with the same per-node
    arithmetic as the per-step kernels (HC_AUX_VCYCLE=kernels, the default):
    on one handle, z = B r through
    hc_precond_apply_device is bit-identical (no atomics on this path), on
    hierarchies of 3-4 levels and odd grid sizes; and B is D^-1 plus a
    positive semi-definite correction (r.(z - D^-1 r) >= 0 up to the
    V-cycle's FP32 rounding)."""
    import torch

    rng = np.random.default_rng(8 + p)
    ne = n ** 3
    op = HCurlOperator(n, n, n, p, meshes.loguniform(ne, 1.0, 1e3, rng), meshes.loguniform(ne, 1e-2, 1e6, rng),
                       dt=0.01, ess_attr_bits=0x3F)
    r = torch.tensor(np.random.default_rng(3).standard_normal(op.ndof), device="cuda")
    r2 = torch.tensor(np.random.default_rng(4).standard_normal(op.ndof), device="cuda")
    zs = {}
    for mode in ("coop", "kernels", "hybrid", "cluster", "coop"):
        monkeypatch.setenv("HC_AUX_VCYCLE", mode)
        z, z2 = torch.empty_like(r), torch.empty_like(r)
        op.PrecondApplyDevice(r, z, "aux")
        op.PrecondApplyDevice(r2, z2, "aux")
        torch.cuda.synchronize()
        zs.setdefault(mode, []).append((z.cpu().numpy(), z2.cpu().numpy()))
    zj = torch.empty_like(r)
    op.PrecondApplyDevice(r, zj, "jacobi")
    for k in (0, 1):
        b = zs["kernels"][0][k]
        for mode in ("coop", "hybrid", "cluster"):
            a = zs[mode][0][k]
            d = np.abs(a - b)
            assert np.array_equal(a, b), (mode, k, int(np.count_nonzero(d)), float(d.max() / np.abs(b).max()))
        assert np.array_equal(zs["coop"][0][k], zs["coop"][1][k])  # replays are reproducible
    rh, z = r.cpu().numpy(), zs["coop"][0][0]
    assert rh @ (z - zj.cpu().numpy()) >= -1e-6 * abs(rh @ z)
