"""Mesh and coefficient generators for the synthetic workloads (host side, numpy).

These build the same inputs for the device path and for the CPU oracle:
structured hex grids on a box, Kuhn (6 tets per cube) subdivisions with seeded
vertex jitter, uniform red refinement of tet meshes, and seeded per-element
coefficient fields.  An MFEM-ASCII (v1.0) tet mesh reader is included for the
reference's data/beam-tet.mesh, which the reference's A-form MMS test reads
(test/integration/test_aform_source.cpp:80).
"""
from __future__ import annotations

import numpy as np


# ----------------------------------------------------------------------------
# structured hexes
# ----------------------------------------------------------------------------
def box_vertices(nx, ny, nz, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """(nx+1)(ny+1)(nz+1) x 3 vertex array, x fastest."""
    xs = np.linspace(lo[0], hi[0], nx + 1)
    ys = np.linspace(lo[1], hi[1], ny + 1)
    zs = np.linspace(lo[2], hi[2], nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def hex_centroids(nx, ny, nz, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    h = [(hi[d] - lo[d]) / n for d, n in enumerate((nx, ny, nz))]
    xs = lo[0] + (np.arange(nx) + 0.5) * h[0]
    ys = lo[1] + (np.arange(ny) + 0.5) * h[1]
    zs = lo[2] + (np.arange(nz) + 0.5) * h[2]
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def hex_ndof(nx, ny, nz, p):
    a, b, c = nx * p, ny * p, nz * p
    return a * (b + 1) * (c + 1) + (a + 1) * b * (c + 1) + (a + 1) * (b + 1) * c


# ----------------------------------------------------------------------------
# coefficient fields
# ----------------------------------------------------------------------------
def coil_sigma(centroids, inside=1.0, outside=1e-6, lo=0.25, hi=0.75):
    """sigma = inside for centroids in [lo,hi]^3, else outside."""
    c = np.asarray(centroids)
    m = np.all((c >= lo) & (c <= hi), axis=1)
    return np.where(m, inside, outside)


def loguniform(n, lo, hi, rng):
    return 10.0 ** rng.uniform(np.log10(lo), np.log10(hi), size=n)


# ----------------------------------------------------------------------------
# tets
# ----------------------------------------------------------------------------
# Kuhn / Freudenthal split of the unit cube along the (0,0,0)-(1,1,1) diagonal.
_KUHN = [
    (0, 1, 3, 7),
    (0, 1, 5, 7),
    (0, 2, 3, 7),
    (0, 2, 6, 7),
    (0, 4, 5, 7),
    (0, 4, 6, 7),
]


def kuhn_mesh(n, jitter=0.0, seed=0):
    """Kuhn subdivision of the unit cube into 6 n^3 tets.

    Interior vertices are moved by U(-jitter*h, jitter*h) per coordinate.
    Returns (verts, tets, btris, battr) with boundary attributes 1..6 =
    x-, x+, y-, y+, z-, z+.
    """
    h = 1.0 / n
    verts = box_vertices(n, n, n)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter * h, jitter * h, size=verts.shape)
        ijk = np.stack(np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij"), -1)
        ijk = ijk[..., ::-1].reshape(-1, 3)  # (z,y,x) meshgrid -> x fastest ordering
        interior = np.all((ijk > 0) & (ijk < n), axis=1)
        verts = verts + d * interior[:, None]
    V = lambda i, j, k: i + (n + 1) * (j + (n + 1) * k)  # noqa: E731
    I, J, K = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    I, J, K = I.transpose(2, 1, 0).ravel(), J.transpose(2, 1, 0).ravel(), K.transpose(2, 1, 0).ravel()
    corner = np.stack([V(I + (c & 1), J + ((c >> 1) & 1), K + ((c >> 2) & 1)) for c in range(8)], axis=1)
    tets = np.concatenate([corner[:, list(t)] for t in _KUHN], axis=1).reshape(-1, 4)
    btris, battr = boundary_faces(tets, verts)
    return verts, tets.astype(np.int64), btris, battr


def boundary_faces(tets, verts, box_lo=0.0, box_hi=1.0, tol=1e-9):
    """Faces with one adjacent tet; attribute by the box face they lie on (else 7)."""
    f = np.concatenate([tets[:, [0, 1, 2]], tets[:, [0, 1, 3]], tets[:, [0, 2, 3]], tets[:, [1, 2, 3]]])
    fs = np.sort(f, axis=1)
    _, idx, cnt = np.unique(fs, axis=0, return_index=True, return_counts=True)
    b = f[idx[cnt == 1]]
    c = verts[b].mean(axis=1)
    attr = np.full(len(b), 7, dtype=np.int32)
    for d in range(3):
        attr[np.abs(c[:, d] - box_lo) < tol] = 2 * d + 1
        attr[np.abs(c[:, d] - box_hi) < tol] = 2 * d + 2
    return b.astype(np.int64), attr


def refine_tets(verts, tets, btris, battr):
    """Uniform red refinement: each tet -> 8, each boundary triangle -> 4.

    The inner octahedron is split along its shortest diagonal (Bey's
    quality-preserving choice), which keeps the refined family shape-regular.
    """
    tets = np.asarray(tets)
    nv = len(verts)
    pairs = np.concatenate([tets[:, [a, b]] for a, b in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3))])
    pairs = np.sort(pairs, axis=1)
    uniq, inv = np.unique(pairs, axis=0, return_inverse=True)
    inv = inv.ravel()
    mid = 0.5 * (verts[uniq[:, 0]] + verts[uniq[:, 1]])
    nverts = np.concatenate([verts, mid])
    ne = len(tets)
    m = (nv + inv).reshape(6, ne).T  # m01 m02 m03 m12 m13 m23
    v0, v1, v2, v3 = tets.T
    m01, m02, m03, m12, m13, m23 = m.T
    corners = [(v0, m01, m02, m03), (v1, m01, m12, m13), (v2, m02, m12, m23), (v3, m03, m13, m23)]
    oct_a = [(m01, m02, m03, m13), (m01, m02, m12, m13), (m02, m03, m13, m23), (m02, m12, m13, m23)]
    oct_b = [(m01, m23, m02, m03), (m01, m23, m03, m13), (m01, m23, m13, m12), (m01, m23, m12, m02)]
    oct_c = [(m03, m12, m01, m02), (m03, m12, m02, m23), (m03, m12, m23, m13), (m03, m12, m13, m01)]
    L = lambda a, b: np.linalg.norm(nverts[a] - nverts[b], axis=1)  # noqa: E731
    k = np.argmin(np.stack([L(m02, m13), L(m01, m23), L(m03, m12)], axis=1), axis=1)
    inner = []
    for ca, cb, cc in zip(oct_a, oct_b, oct_c):
        inner.append(tuple(np.where(k == 0, a, np.where(k == 1, b, c)) for a, b, c in zip(ca, cb, cc)))
    children = corners + inner
    ntets = np.stack([np.stack(c, axis=1) for c in children], axis=1).reshape(-1, 4)
    # boundary triangles
    key = {tuple(p): i for i, p in enumerate(uniq.tolist())}

    def midv(a, b):
        return nv + key[(min(a, b), max(a, b))]

    nb, na = [], []
    for (a, b, c), at in zip(np.asarray(btris).tolist(), np.asarray(battr).tolist()):
        ab, ac, bc = midv(a, b), midv(a, c), midv(b, c)
        nb += [(a, ab, ac), (b, ab, bc), (c, ac, bc), (ab, ac, bc)]
        na += [at] * 4
    return nverts, ntets.astype(np.int64), np.array(nb, dtype=np.int64), np.array(na, dtype=np.int32)


def tet_quality_ok(verts, tets):
    """True if every tet has nonzero volume (jitter did not invert)."""
    v = verts[tets]
    d = np.einsum("ij,ij->i", v[:, 1] - v[:, 0], np.cross(v[:, 2] - v[:, 0], v[:, 3] - v[:, 0]))
    return bool(np.all(np.abs(d) > 0)), d


def read_mfem_tet_mesh(path):
    """Minimal MFEM mesh v1.0 reader for tetrahedral meshes."""
    with open(path) as f:
        toks = [ln.strip() for ln in f if ln.strip() and not ln.lstrip().startswith("#")]
    i = 0
    verts = tets = btris = battr = eattr = None
    while i < len(toks):
        t = toks[i]
        if t == "elements":
            n = int(toks[i + 1])
            rows = [list(map(int, toks[i + 2 + k].split())) for k in range(n)]
            eattr = np.array([r[0] for r in rows], dtype=np.int32)
            assert all(r[1] == 4 for r in rows), "only tetrahedra supported"
            tets = np.array([r[2:6] for r in rows], dtype=np.int64)
            i += 2 + n
        elif t == "boundary":
            n = int(toks[i + 1])
            rows = [list(map(int, toks[i + 2 + k].split())) for k in range(n)]
            battr = np.array([r[0] for r in rows], dtype=np.int32)
            btris = np.array([r[2:5] for r in rows], dtype=np.int64)
            i += 2 + n
        elif t == "vertices":
            n = int(toks[i + 1])
            dim = int(toks[i + 2])
            verts = np.array([list(map(float, toks[i + 3 + k].split()))[:dim] for k in range(n)])
            i += 3 + n
        else:
            i += 1
    return verts, tets, btris, battr, eattr
