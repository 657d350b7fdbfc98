"""CPU tests of the host tet topology (hephaestus_gb300/csrc/hc_tet_topo.h,
the code hc_create runs for tet meshes): element dof lists and essential
flags equal the oracle's numbering on Kuhn meshes (small, and large enough for
the threaded sorts) and on the refined beam mesh; invalid meshes are reported."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from hephaestus_gb300 import meshes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def driver():
    exe = os.path.join(tempfile.mkdtemp(), "tet_topo_check")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "hephaestus_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "tet_topo_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _topo(driver, nv, tets, p, bt, ba, bits):
    d = tempfile.mkdtemp()
    fin, fout = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
    tets = np.ascontiguousarray(tets, dtype=np.int64)
    bt = np.ascontiguousarray(bt, dtype=np.int64).reshape(-1, 3)
    ba = np.ascontiguousarray(ba, dtype=np.int32)
    with open(fin, "wb") as f:
        np.array([len(tets), nv, p, bits, len(bt)], dtype=np.int64).tofile(f)
        tets.tofile(f)
        bt.tofile(f)
        ba.tofile(f)
    r = subprocess.run([driver, fin, fout], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    buf = open(fout, "rb").read()
    st, ln = np.frombuffer(buf, dtype=np.int32, count=2)
    msg = buf[8:8 + ln].decode()
    pos = 8 + ln
    ndof, ne_, nf_ = np.frombuffer(buf, dtype=np.int64, count=3, offset=pos)
    pos += 24
    if st != 0:
        return int(st), msg, None, None
    L = 6 if p == 1 else 20
    ed = np.frombuffer(buf, dtype=np.int32, count=len(tets) * L, offset=pos).reshape(-1, L)
    pos += ed.nbytes
    ess = np.frombuffer(buf, dtype=np.uint8, count=int(ndof), offset=pos)
    return 0, msg, ed, ess


@pytest.mark.parametrize("n,p", [(3, 1), (3, 2), (20, 1), (20, 2)])
def test_kuhn_topology_matches_oracle(driver, n, p):
    v, t, bt, ba = meshes.kuhn_mesh(n, jitter=0.1, seed=n)
    st, msg, ed, ess = _topo(driver, len(v), t, p, bt, ba, 0x2D)
    assert st == 0, msg
    ref = oracle.Problem.tet(v, t, p)
    assert np.array_equal(ed, ref.elem_dofs())
    assert np.array_equal(ess, ref.tet_ess_mask(bt, ba, 0x2D))


def test_beam_topology_matches_oracle(driver):
    d = np.load(os.path.join(GOLD, "beam_tet.npz"))
    v, t, bt, ba = meshes.refine_tets(d["verts"], d["tets"], d["btris"], d["battr"])
    st, msg, ed, ess = _topo(driver, len(v), t, 2, bt, ba, 0b111)
    assert st == 0, msg
    ref = oracle.Problem.tet(v, t, 2)
    assert np.array_equal(ed, ref.elem_dofs())
    assert np.array_equal(ess, ref.tet_ess_mask(bt, ba, 0b111))


def test_invalid_meshes_are_reported(driver):
    t = np.array([[0, 1, 2, 3], [0, 1, 1, 3], [0, 1, 2, 9]])
    st, msg, _, _ = _topo(driver, 4, t, 1, np.zeros((0, 3)), np.zeros(0), 0)
    assert st == 1 and "degenerate" in msg  # the first failing element in order
    st, msg, _, _ = _topo(driver, 4, t[[0, 2]], 1, np.zeros((0, 3)), np.zeros(0), 0)
    assert st == 1 and "range" in msg
    st, msg, _, _ = _topo(driver, 5, np.array([[0, 1, 2, 3]]), 2, np.array([[0, 1, 4]]), np.array([1]), 1)
    assert st == 1 and "boundary triangle" in msg
