"""CPU check of the design of the tet auxiliary-space preconditioner on the
oracle's matrices: the discrete gradient assembled from the shared coefficient
tables (hephaestus_gb300/csrc/hc_tet_grad.h) is exact (C_nu G = 0), and on an
order-2 mesh with log-uniform coefficient jumps the correction
B = D^-1 + G (G^T J G)^-1 G^T over the P2 nodal space (vertex hats and edge
bubbles) cuts Jacobi's PCG iterations several-fold, while the P1 (vertex-only)
correction does not help: the slow modes are gradients of the edge bubbles."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from hephaestus_gb300 import meshes

sp = pytest.importorskip("scipy.sparse")
spl = pytest.importorskip("scipy.sparse.linalg")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


@pytest.fixture(scope="module")
def local_tables():
    exe = os.path.join(tempfile.mkdtemp(), "tet_grad_check")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "hephaestus_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "tet_grad_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    txt = subprocess.run([exe, "2"], capture_output=True, text=True, check=True).stdout
    return np.array([[float(w) for w in line.split()] for line in txt.strip().splitlines()])  # 20 x (4 + 6)


def _problem(n, seed=3):
    v, t, bt, ba = meshes.kuhn_mesh(n, jitter=0.15, seed=seed)
    rng = np.random.default_rng(seed)
    ne = len(t)
    nu, sigma = meshes.loguniform(ne, 1.0, 1e3, rng), meshes.loguniform(ne, 1e-2, 1e6, rng)
    ref = oracle.Problem.tet(v, t, 2)
    ref.set_coef(0.01 * nu, sigma)
    ref.assemble()
    m = ref.tet_ess_mask(bt, ba, 0x3F)
    ref.set_ess(m)
    return v, t, ref, m.astype(bool), nu


def _global_gradient(v, t, ref, T):
    """N x (vertices + edges) gradient matrix from the 20 x 10 local table:
    columns 0..nv-1 vertex hats, nv + g the bubble of global edge g."""
    ed = ref.elem_dofs()
    sv = np.sort(t, axis=1)
    nv = len(v)
    G = {}
    for e in range(len(t)):
        gedge = [ed[e, 2 * k] // 2 for k in range(6)]
        for I in range(20):
            for a in range(4):
                if T[I, a] != 0:
                    G[(ed[e, I], sv[e, a])] = T[I, a]
            for k in range(6):
                if T[I, 4 + k] != 0:
                    G[(ed[e, I], nv + gedge[k])] = T[I, 4 + k]
    nE = max(c for (_, c) in G) - nv + 1
    rows = np.array([r for (r, _) in G])
    cols = np.array([c for (_, c) in G])
    return sp.csr_matrix((np.array(list(G.values())), (rows, cols)), shape=(ref.ndof, nv + nE)), nv


def _pcg(K, b, prec, maxit=20000):
    x = np.zeros_like(b)
    r = b.copy()
    z = prec(r)
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    for it in range(maxit):
        q = K @ p
        al = rz / (p @ q)
        x += al * p
        r -= al * q
        if np.linalg.norm(r) <= 1e-12 * nb:
            return it + 1
        z = prec(r)
        rzn = r @ z
        p = z + rzn / rz * p
        rz = rzn
    return maxit


def test_assembled_gradient_is_curl_free(local_tables):
    v, t, ref, ess, nu = _problem(3)
    G, nv = _global_gradient(v, t, ref, local_tables)
    ref.set_coef(np.ones(len(t)), None)
    ref.assemble()
    C = ref.csr()
    u = np.random.default_rng(1).standard_normal(G.shape[1])
    g = G @ u
    assert np.linalg.norm(C @ g) <= 1e-10 * np.linalg.norm(C.diagonal()) * np.linalg.norm(g)


def test_p2_gradient_correction_is_what_order_2_needs(local_tables):
    v, t, ref, ess, nu = _problem(5)
    K0 = ref.csr().tocsr()
    P = sp.diags((~ess).astype(float))
    K = (P @ K0 @ P + sp.diags(ess.astype(float))).tocsr()  # eliminated operator J
    d = K.diagonal()
    b = ref.load_coil(I0=1.0, q=4)
    b[ess] = 0.0
    G, nv = _global_gradient(v, t, ref, local_tables)
    fixed = np.asarray(abs(G[ess]).sum(axis=0)).ravel() > 0
    Gf = P @ G[:, np.where(~fixed)[0]]
    n1 = int((~fixed[:nv]).sum())  # free vertex columns come first
    lu2 = spl.splu((Gf.T @ K @ Gf).tocsc())
    G1 = Gf[:, :n1]
    lu1 = spl.splu((G1.T @ K @ G1).tocsc())
    jac = _pcg(K, b, lambda r: r / d)
    aux_p2 = _pcg(K, b, lambda r: r / d + Gf @ lu2.solve(Gf.T @ r))
    aux_p1 = _pcg(K, b, lambda r: r / d + G1 @ lu1.solve(G1.T @ r))
    assert aux_p2 < 0.35 * jac, (aux_p2, jac)
    assert aux_p1 > 0.8 * jac, (aux_p1, jac)


def test_multiplicative_cycle_on_tets(local_tables):
    """The symmetric multiplicative cycle (Chebyshev-Jacobi(2) smoothing around
    the exact P2 gradient correction) cuts the additive form's iterations about
    threefold on tets too.  It is not built for the 16-column block solve: each
    iteration would add four block applies (0.49 ms each on tets48) and four
    Chebyshev steps over 273 MB blocks, about 2.6x the iteration's cost."""
    v, t, ref, ess, nu = _problem(5)
    K0 = ref.csr().tocsr()
    P = sp.diags((~ess).astype(float))
    K = (P @ K0 @ P + sp.diags(ess.astype(float))).tocsr()
    dinv = 1.0 / K.diagonal()
    b = ref.load_coil(I0=1.0, q=4)
    b[ess] = 0.0
    G, nv = _global_gradient(v, t, ref, local_tables)
    fixed = np.asarray(abs(G[ess]).sum(axis=0)).ravel() > 0
    Gf = P @ G[:, np.where(~fixed)[0]]
    lu = spl.splu((Gf.T @ K @ Gf).tocsc())
    lmax = 1.1 * abs(spl.eigs(sp.diags(dinv) @ K, k=1, which="LM", return_eigenvectors=False)[0])

    def cheb(r, x, deg=2, ratio=30.0):
        lo = lmax / ratio
        th, de = 0.5 * (lmax + lo), 0.5 * (lmax - lo)
        rho = de / th
        d = dinv * (r - K @ x) / th
        x = x + d
        for _ in range(1, deg):
            rho2 = 1.0 / (2.0 * th / de - rho)
            d = rho2 * rho * d + 2.0 * rho2 / de * (dinv * (r - K @ x))
            x = x + d
            rho = rho2
        return x

    def mult(r):
        z = cheb(r, np.zeros_like(r))
        z = z + Gf @ lu.solve(Gf.T @ (r - K @ z))
        return cheb(r, z)

    additive = _pcg(K, b, lambda r: dinv * r + Gf @ lu.solve(Gf.T @ r))
    multiplicative = _pcg(K, b, mult)
    assert multiplicative * 2.5 < additive, (additive, multiplicative)
