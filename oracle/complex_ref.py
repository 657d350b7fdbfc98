"""CPU restatement of the frequency-domain (eddy-current) solve -- test
infrastructure only: tests/ and bench.py's CPU-baseline leg use it as the
checker, the product package never imports it.

Reference: ComplexMaxwellOperator::Solve
(src/formulations/ComplexMaxwell/complex_maxwell_formulation.cpp:171-222)
assembles a ParSesquilinearForm with CurlCurlIntegrator(1/mu) and
VectorFEMassIntegrator(-omega^2 eps) in the real part and
VectorFEMassIntegrator(omega sigma) in the imaginary part, eliminates the
essential dofs with FormLinearSystem and solves the 2N x 2N real form of the
system with SuperLU (complex_maxwell_formulation.cpp:28-31, 209-218).  With
eps = 0 the complex operator is

    A = C_nu + i omega M_sigma,

and after elimination  J = P A P + (I - P).  `direct_solve` is that solve
(scipy's spsolve is SuperLU); `cocg` restates the conjugate orthogonal CG
iteration (van der Vorst & Melissen, IEEE Trans. Magn. 26(2), 1990) with the
complex Jacobi preconditioner that the GPU path runs.
"""
import numpy as np


def forms(problem, nu, sigma):
    """(C_nu, M_sigma) as scipy CSR matrices from an oracle.Problem (hex or tet)."""
    problem.set_coef(np.asarray(nu, dtype=np.float64), None)
    problem.assemble()
    Cn = problem.csr()
    problem.set_coef(np.zeros(len(nu)), np.asarray(sigma, dtype=np.float64))
    problem.assemble()
    M = problem.csr()
    return Cn, M


def eliminated(Cn, M, omega, ess):
    """J = P (C + i omega M) P + (I - P) as a complex CSR matrix."""
    import scipy.sparse as sp

    free = sp.diags((np.asarray(ess) == 0).astype(np.float64))
    A = (Cn + 1j * omega * M).tocsr()
    return (free @ A @ free + sp.diags((np.asarray(ess) != 0).astype(np.complex128))).tocsr()


def direct_solve(J, b):
    """SuperLU solve of J x = b (the reference's direct solver)."""
    import scipy.sparse.linalg as spla

    return spla.spsolve(J.tocsc(), np.asarray(b, dtype=np.complex128))


def cocg(J, b, x0=None, rtol=1e-12, maxit=10000):
    """COCG with the complex Jacobi preconditioner D^-1, D = diag(J).

    Unconjugated bilinear products u^T v throughout; stops when
    ||b - J x||_2 <= rtol ||b||_2 (recursive residual).  Returns (x, iterations).
    """
    b = np.asarray(b, dtype=np.complex128)
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.complex128)
    dinv = 1.0 / J.diagonal()
    r = b - J @ x
    z = dinv * r
    p = z.copy()
    rho = r @ z
    tol = rtol * np.linalg.norm(b)
    it = 0
    while np.linalg.norm(r) > tol and it < maxit:
        q = J @ p
        alpha = rho / (p @ q)
        x += alpha * p
        r -= alpha * q
        z = dinv * r
        rho_new = r @ z
        p = z + (rho_new / rho) * p
        rho = rho_new
        it += 1
    return x, it
