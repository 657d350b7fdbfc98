"""CPU tests of the host set-up of the tet auxiliary-space AMG
(hephaestus_gb300/csrc/hc_amg_host.h): aggregation, smoothed prolongator,
Galerkin product, transpose and the dense scaled coarse inverse against
scipy/numpy on a 3-D coefficient-jump Laplacian."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

sp = pytest.importorskip("scipy.sparse")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def driver():
    exe = os.path.join(tempfile.mkdtemp(), "amg_host_check")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "hephaestus_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "amg_host_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _laplacian(m, seed):
    """7-point Laplacian on an m^3 grid with log-uniform cell coefficients in
    [1e-2, 1e6] (harmonic averages on the faces) plus a small mass term."""
    rng = np.random.default_rng(seed)
    c = 10.0 ** rng.uniform(-2, 6, size=(m, m, m))
    n = m ** 3
    idx = np.arange(n).reshape(m, m, m)
    rows, cols, vals = [], [], []
    diag = 1e-3 * c.ravel().copy()
    for ax in range(3):
        a = [slice(None)] * 3
        b = [slice(None)] * 3
        a[ax] = slice(0, m - 1)
        b[ax] = slice(1, m)
        w = 2.0 / (1.0 / c[tuple(a)] + 1.0 / c[tuple(b)])
        i, j = idx[tuple(a)].ravel(), idx[tuple(b)].ravel()
        rows += [i, j]
        cols += [j, i]
        vals += [-w.ravel(), -w.ravel()]
        np.add.at(diag, i, w.ravel())
        np.add.at(diag, j, w.ravel())
    rows.append(np.arange(n))
    cols.append(np.arange(n))
    vals.append(diag)
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, n))
    A.sort_indices()
    return A


def _run(driver, A):
    d = tempfile.mkdtemp()
    fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    with open(fin, "wb") as f:
        np.array([A.shape[0], A.nnz], dtype=np.int32).tofile(f)
        A.indptr.astype(np.int32).tofile(f)
        A.indices.astype(np.int32).tofile(f)
        A.data.astype(np.float64).tofile(f)
    r = subprocess.run([driver, fin, fout], capture_output=True, text=True)
    assert r.returncode == 0, (r.returncode, r.stderr)
    buf = open(fout, "rb").read()
    pos = 0

    def take(dt, k):
        nonlocal pos
        a = np.frombuffer(buf, dtype=dt, count=k, offset=pos)
        pos += a.nbytes
        return a

    def csr(ncols):
        n, nnz = take(np.int32, 2)
        rp, ci, va = take(np.int32, n + 1), take(np.int32, nnz), take(np.float64, nnz)
        return sp.csr_matrix((va, ci, rp), shape=(n, ncols))

    lmax = take(np.float64, 1)[0]
    na = int(take(np.int32, 1)[0])
    agg = take(np.int32, A.shape[0])
    P = csr(na)
    Ac = csr(na)
    ok = int(take(np.int32, 1)[0])
    inv = take(np.float32, na * na).reshape(na, na) if ok else None
    sc = take(np.float32, na) if ok else None
    return lmax, na, agg, P, Ac, ok, inv, sc


@pytest.mark.parametrize("m,seed", [(9, 0), (12, 1)])
def test_amg_level_matches_scipy(driver, m, seed):
    A = _laplacian(m, seed)
    n = A.shape[0]
    lmax, na, agg, P, Ac, ok, inv, sc = _run(driver, A)
    # aggregation: every node in exactly one aggregate, ids 0..na-1 all used, real coarsening
    assert agg.min() == 0 and agg.max() == na - 1 and len(np.unique(agg)) == na
    assert na < 0.6 * n
    # lambda_max of D^-1 A from the power iteration: a lower bound within a few percent
    d = A.diagonal()
    S = sp.diags(1.0 / np.sqrt(d))
    true = np.linalg.eigvalsh((S @ A @ S).toarray()).max()
    assert 0.9 * true <= lmax <= true * (1 + 1e-12)
    # smoothed prolongator (I - omega D^-1 A) P_tent
    cnt = np.bincount(agg, minlength=na)
    Pt = sp.csr_matrix((1.0 / np.sqrt(cnt[agg]), (np.arange(n), agg)), shape=(n, na))
    omega = 4.0 / (3.0 * lmax)
    Pref = Pt - omega * sp.diags(1.0 / d) @ A @ Pt
    assert abs(P - Pref).max() <= 1e-12 * abs(Pref).max()
    # Galerkin product R A P with R = P^T, rows sorted
    Acref = P.T @ A @ P
    assert abs(Ac - Acref).max() <= 1e-10 * abs(Acref).max()
    assert all(np.all(np.diff(Ac.indices[Ac.indptr[i]:Ac.indptr[i + 1]]) > 0) for i in range(na))
    # dense inverse of the diagonally scaled coarse operator (FP32 result)
    assert ok == 1
    dc = Ac.diagonal()
    assert np.allclose(sc, 1.0 / np.sqrt(dc), rtol=1e-6)
    M = (sp.diags(sc.astype(np.float64)) @ Ac @ sp.diags(sc.astype(np.float64))).toarray()
    err = np.abs(inv.astype(np.float64) @ M - np.eye(na)).max()
    assert err < 1e-4, err  # FP32 rounding of the inverse times cond(M) ~ 2e2
    assert np.array_equal(inv, inv.T)
