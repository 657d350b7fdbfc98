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


def lagrange_values(nodes, at):
    """V[a, j] = phi_j(at[a]) for the Lagrange basis on nodes."""
    m = len(nodes)
    V = np.ones((len(at), m))
    for j in range(m):
        for k in range(m):
            if k != j:
                V[:, j] *= (np.asarray(at) - nodes[k]) / (nodes[j] - nodes[k])
    return V


def rt_eval_ref(B, nx, ny, nz, p, e, xi):
    """Reference-frame value of the Raviart-Thomas field with dofs B (our
    layout) in element e at reference point xi."""
    ex, ey, ez = e % nx, (e // nx) % ny, e // (nx * ny)
    gc, go = gll_nodes(p + 1), gl_nodes(p)
    vals = [(lagrange_values(gc, [xi[d]])[0], lagrange_values(go, [xi[d]])[0]) for d in range(3)]
    mx, my, mz = nx * p, ny * p, nz * p
    dims = [(mx + 1, my, mz), (mx, my + 1, mz), (mx, my, mz + 1)]
    offs = [0, dims[0][0] * dims[0][1] * dims[0][2]]
    offs.append(offs[1] + dims[1][0] * dims[1][1] * dims[1][2])
    out = np.zeros(3)
    for c in range(3):
        d0, d1, d2 = dims[c]
        arr = B[offs[c]:offs[c] + d0 * d1 * d2].reshape(d2, d1, d0)
        bx = vals[0][0] if c == 0 else vals[0][1]
        by = vals[1][0] if c == 1 else vals[1][1]
        bz = vals[2][0] if c == 2 else vals[2][1]
        sub = arr[ez * p:ez * p + len(bz), ey * p:ey * p + len(by), ex * p:ex * p + len(bx)]
        out[c] = np.einsum("kji,k,j,i->", sub, bz, by, bx)
    return out
