"""CPU test of the host structure of the tet auxiliary-space preconditioner
(hephaestus_gb300/csrc/hc_tetaux_host.h): free vertices and edge bubbles,
(PG)^T, the P1 nodal operator (PG)^T J (PG), the P2 nodal diagonal and the
per-dof gradient slots the device kernels read, against numpy built from the
oracle's element matrices and the shared gradient tables."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from hephaestus_gb300 import meshes

sp = pytest.importorskip("scipy.sparse")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "hephaestus_gb300", "csrc")


def _exe(name, tmp):
    exe = os.path.join(tmp, name)
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", CSRC, os.path.join(ROOT, "tests", name + ".cpp"),
                        "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.fixture(scope="module")
def tools():
    tmp = tempfile.mkdtemp()
    grad = _exe("tet_grad_check", tmp)
    tables = {}
    for p in (1, 2):
        txt = subprocess.run([grad, str(p)], capture_output=True, text=True, check=True).stdout
        tables[p] = np.array([[float(w) for w in ln.split()] for ln in txt.strip().splitlines()])
    return _exe("tetaux_host_check", tmp), tables


def _run(exe, p, sv, ed, ess, Ae, nE):
    d = tempfile.mkdtemp()
    fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    with open(fin, "wb") as f:
        np.array([p, len(sv), len(ess), nE], dtype=np.int64).tofile(f)
        sv.astype(np.int32).tofile(f)
        ed.astype(np.int32).tofile(f)
        ess.astype(np.uint8).tofile(f)
        Ae.astype(np.float64).tofile(f)
    r = subprocess.run([exe, fin, fout], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    buf = open(fout, "rb").read()
    ok, nfree, nfe, nn = np.frombuffer(buf, dtype=np.int32, count=4)
    nface0 = int(np.frombuffer(buf, dtype=np.int64, count=1, offset=16)[0])
    pos = 24
    N = len(ess)

    def take(dt, k):
        nonlocal pos
        a = np.frombuffer(buf, dtype=dt, count=k, offset=pos)
        pos += a.nbytes
        return a

    def csr(ncols):
        n, nnz = take(np.int32, 2)
        rp, ci, va = take(np.int32, n + 1), take(np.int32, nnz), take(np.float64, nnz)
        return sp.csr_matrix((va, ci, rp), shape=(n, ncols))

    gnode = take(np.int32, 3 * N).reshape(N, 3)
    gedge = take(np.int32, 3 * N).reshape(N, 3) if p == 2 else None
    Gt = csr(N)
    A = csr(int(nfree))
    dl = take(np.float32, int(nn)) if p == 2 else None
    return dict(nfree=int(nfree), nfe=int(nfe), nn=int(nn), nface0=nface0, gnode=gnode, gedge=gedge, Gt=Gt, A=A, dl=dl)


@pytest.mark.parametrize("p,bits", [(1, 0x3F), (2, 0x3F), (2, 0)])
def test_aux_structure_matches_numpy(tools, p, bits):
    exe, tables = tools
    T = tables[p]
    L = T.shape[0]
    v, t, bt, ba = meshes.kuhn_mesh(3, jitter=0.15, seed=2)
    rng = np.random.default_rng(2)
    ne = len(t)
    nu, sigma = meshes.loguniform(ne, 1.0, 1e3, rng), meshes.loguniform(ne, 1e-2, 1e6, rng)
    ref = oracle.Problem.tet(v, t, p)
    ref.set_coef(0.01 * nu, sigma)
    ref.assemble()
    ess = ref.tet_ess_mask(bt, ba, bits).astype(bool)
    ref.set_ess(ess.astype(np.uint8))
    ed = ref.elem_dofs()
    sv = np.sort(t, axis=1)
    N = ref.ndof
    nE = N if p == 1 else int(ed[:, 0:12:2].max()) // 2 + 1
    nv = len(v)
    # element nodal matrices as the device kernel forms them (rows of essential dofs zeroed)
    nout = 10 if p == 1 else 16
    Ae = np.zeros((ne, nout))
    iu = np.triu_indices(4)
    for e in range(ne):
        K = ref.element_matrix(e)
        m = (~ess[ed[e]]).astype(float)[:, None]
        Gv = T[:, :4] * m
        Av = Gv.T @ K @ Gv
        Ae[e, :10] = (0.5 * (Av + Av.T))[iu]
        if p == 2:
            Gb = T[:, 4:] * m
            Ae[e, 10:] = np.einsum("ik,ij,jk->k", Gb, K, Gb)
    out = _run(exe, p, sv, ed, ess, Ae, nE)
    # reference: global gradient, free vertices / edges, masked
    rows, cols, vals = [], [], []
    for e in range(ne):
        for I in range(L):
            for a in range(4):
                if T[I, a]:
                    rows.append(ed[e, I]); cols.append(sv[e, a]); vals.append(T[I, a])
            if p == 2:
                for k in range(6):
                    if T[I, 4 + k]:
                        rows.append(ed[e, I]); cols.append(nv + ed[e, 2 * k] // 2); vals.append(T[I, 4 + k])
    G = sp.coo_matrix((vals, (rows, cols)), shape=(N, nv + (nE if p == 2 else 0))).tocsr()
    G.sum_duplicates()
    G.data[:] = np.sign(G.data) * np.abs(G.data)  # duplicates were identical entries
    Gdup = sp.coo_matrix((np.ones(len(vals)), (rows, cols)), shape=G.shape).tocsr()
    G = sp.csr_matrix((G.data / Gdup.data, G.indices, G.indptr), shape=G.shape)  # undo summing of repeats
    fixed = np.zeros(nv, bool)
    for e in range(ne):
        for I in range(L):
            if ess[ed[e, I]]:
                fixed[sv[e, np.nonzero(T[I, :4])[0]]] = True
    if not fixed.any():
        fixed[sv.min()] = True
    free_v = np.nonzero(~fixed)[0]
    cols = list(free_v)
    if p == 2:
        free_e = np.nonzero(~(ess[0:2 * nE:2] | ess[1:2 * nE:2]))[0]
        cols += list(nv + free_e)
    P = sp.diags((~ess).astype(float))
    Gf = (P @ G[:, cols]).tocsr()
    assert out["nfree"] == len(free_v) and out["nn"] == len(cols)
    assert np.abs((out["Gt"] - Gf.T).toarray()).max() == 0.0
    K0 = ref.csr()
    J = P @ K0 @ P + sp.diags(ess.astype(float))
    G1 = Gf[:, :len(free_v)]
    Aref = (G1.T @ J @ G1).toarray()
    assert np.abs(out["A"].toarray() - Aref).max() <= 1e-12 * np.abs(Aref).max()
    if p == 2:
        dref = (Gf.T @ J @ Gf).diagonal()
        assert np.allclose(out["dl"], 1.0 / dref, rtol=1e-6)
    # the per-dof slots with the device kernel's coefficient rule reproduce (PG)
    nface0, nfree = out["nface0"], out["nfree"]
    R = np.zeros((N, out["nn"]))
    for d in range(N):
        face = d >= nface0
        s1 = face and ((d - nface0) & 1)
        cv = (-1.0, (-1.0 if s1 else 2.0) if face else 1.0, (2.0 if s1 else -1.0) if face else 0.0)
        for k in range(3):
            if out["gnode"][d, k] >= 0:
                R[d, out["gnode"][d, k]] += cv[k]
        if p == 2:
            cb = ((-2.0 if s1 else 1.0) if face else (1.0 if d % 2 == 0 else -1.0), 1.0 if s1 else -2.0, 1.0)
            for k in range(3):
                if out["gedge"][d, k] >= 0:
                    R[d, nfree + out["gedge"][d, k]] += cb[k]
    assert np.abs(R - Gf.toarray()).max() == 0.0
