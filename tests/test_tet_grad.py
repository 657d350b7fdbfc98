"""CPU check of the discrete-gradient tables the tet auxiliary-space kernels
use (hephaestus_gb300/csrc/hc_tet_grad.h): the Nedelec field with those
coefficients, evaluated with the oracle's basis on a jittered tet, equals the
gradient of the vertex hat functions and of the quadratic edge bubbles."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


@pytest.fixture(scope="module")
def tables():
    exe = os.path.join(tempfile.mkdtemp(), "tet_grad_check")
    r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "hephaestus_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "tet_grad_check.cpp"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = {}
    for p in (1, 2):
        txt = subprocess.run([exe, str(p)], capture_output=True, text=True, check=True).stdout
        out[p] = np.array([[float(w) for w in line.split()] for line in txt.strip().splitlines()])
    return out


@pytest.mark.parametrize("p", [1, 2])
def test_gradient_tables_reproduce_gradients(tables, p):
    rng = np.random.default_rng(7)
    v = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
    v += 0.2 * rng.uniform(-1, 1, size=v.shape)
    ref = oracle.Problem.tet(v, np.array([[0, 1, 2, 3]]), p)
    G = tables[p]
    assert G.shape == ((6, 4) if p == 1 else (20, 10))
    J = (v[1:] - v[0]).T
    gl = np.zeros((4, 3))
    gl[1:] = np.linalg.inv(J)
    gl[0] = -gl[1:].sum(axis=0)
    for xi in ([0.2, 0.3, 0.1], [0.05, 0.6, 0.25], [0.25, 0.25, 0.25]):
        lam = np.array([1.0 - sum(xi), *xi])
        for col in range(G.shape[1]):
            val, curl = ref.eval(G[:, col], 0, np.array(xi))
            if col < 4:
                exact = gl[col]
            else:
                a, b = EDGES[col - 4]
                exact = lam[a] * gl[b] + lam[b] * gl[a]
            assert np.abs(val - exact).max() < 1e-12, (p, col, xi)
            assert np.abs(curl).max() < 1e-11
