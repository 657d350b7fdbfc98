"""Test helpers: 1-D bases and the discrete gradient of the structured hex space.

Independent numpy restatement (numpy.polynomial) of the closed (Gauss-Lobatto)
and open (Gauss-Legendre) nodal bases, used to build exact-sequence tests.
"""
import numpy as np
from numpy.polynomial import legendre as npl


def gll_nodes(n):
    N = n - 1
    inner = np.real(npl.Legendre.basis(N).deriv().roots()) if N >= 2 else np.array([])
    return np.concatenate([[0.0], 0.5 * (np.sort(inner) + 1.0), [1.0]])


def gl_nodes(n):
    x, _ = npl.leggauss(n)
    return 0.5 * (x + 1.0)


def lagrange_deriv_matrix(nodes, at):
    """D[a, j] = phi_j'(at[a]) for the Lagrange basis on nodes."""
    m = len(nodes)
    D = np.zeros((len(at), m))
    for j in range(m):
        others = np.delete(nodes, j)
        c = np.poly(others) / np.prod(nodes[j] - others)
        dc = np.polyder(c)
        D[:, j] = np.polyval(dc, at)
    return D


def discrete_gradient(nx, ny, nz, p, phi):
    """Nedelec dofs (our layout) of grad phi, phi a Q_p field on GLL nodes.

    phi has shape (nz*p+1, ny*p+1, nx*p+1) [k, j, i].  Reference-coordinate
    derivatives: in each element the open-direction dof a is
    sum_m D[a, m] phi(e*p + m).
    """
    D = lagrange_deriv_matrix(gll_nodes(p + 1), gl_nodes(p))  # p x (p+1)
    out = []
    for c, n in enumerate((nx, ny, nz)):
        axis = 2 - c  # array axis of direction c
        ph = np.moveaxis(phi, axis, -1)  # (..., n*p+1)
        sh = ph.shape[:-1]
        g = np.zeros(sh + (n * p,))
        for e in range(n):
            seg = ph[..., e * p:e * p + p + 1]  # (..., p+1)
            g[..., e * p:(e + 1) * p] = seg @ D.T
        out.append(np.moveaxis(g, -1, axis).ravel())
    return np.concatenate(out)
