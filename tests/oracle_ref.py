"""Test helpers built on the FP64 oracle: the eliminated operator as a scipy
matrix, direct solves, and backward-Euler steps of the A-formulation.

Backward Euler follows TimeDomainEquationSystemProblemOperator::ImplicitSolve
(src/problem_builders/time_domain_equation_system_problem_operator.cpp:31-51)
with the one-step Newton solve of problem_builder_base.cpp:313-323: per step
b = P (f - C_nu A) (WeakCurlCurlKernel, src/kernels/weak_curl_curl_kernel.cpp:27-31),
J dA = b, A += dt dA (BackwardEulerSolver, time_domain_problem_builder.cpp:59-64).
"""
import numpy as np


def eliminated(ref):
    """J = P K P + (I - P) of an assembled oracle problem with its mask set."""
    import scipy.sparse as sp

    K = ref.csr()
    free = (ref._m == 0).astype(np.float64)
    P = sp.diags(free)
    return (P @ K @ P + sp.diags(1.0 - free)).tocsc()


def direct_solve(J, b):
    import scipy.sparse.linalg as sla

    return sla.spsolve(J, b)


def be_steps(ref, f, dt, nsteps, J=None):
    """nsteps backward-Euler steps from A = 0 with source load f (oracle,
    FP64, sparse direct solves).  ref's alpha must be dt * nu."""
    J = eliminated(ref) if J is None else J
    ess = ref._m != 0
    A = np.zeros(ref.ndof)
    for _ in range(nsteps):
        b = f - ref.apply_curlcurl(A) / dt
        b[ess] = 0.0
        dA = direct_solve(J, b)
        A = A + dt * dA
    return A
