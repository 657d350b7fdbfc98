"""GPU tests of the launch configurations of the tiled hex kernels: both
brick shapes (16x4x2 and 8x8x2 elements per CTA) and every CTA count per SM
give the oracle's operator on grids that fill neither shape evenly, real and
complex; the autotuner picks one of them and stores it for later handles of
the same problem (HC_TUNE_FILE)."""
import os
import subprocess
import sys

import numpy as np
import pytest

import oracle
from oracle import complex_ref as CR
from hephaestus_gb300 import HCurlOperator, meshes

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CONFIGS = [(0, 0), (1, 0), (1, 1), (1, 3), (0, 2)]


def _grid(p, shear, nx=11, ny=9, nz=5, seed=0, dt=0.01):
    rng = np.random.default_rng(seed)
    ne = nx * ny * nz
    nu = meshes.loguniform(ne, 1.0, 1e3, rng)
    sigma = meshes.loguniform(ne, 1e-2, 1e6, rng)
    verts = None
    if shear:
        A = np.array([[1.0, 0.2, 0.1], [0.0, 0.9, -0.15], [0.05, 0.0, 1.1]])
        verts = meshes.box_vertices(nx, ny, nz) @ A.T
    op = HCurlOperator(nx, ny, nz, p, nu, sigma, dt=dt, vertices=verts, ess_attr_bits=0x15)
    ref = oracle.Problem.hex(nx, ny, nz, p, verts)
    return op, ref, nu, sigma, rng


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("shear", [False, True])
def test_brick_shapes_match_oracle(p, shear):
    import torch

    op, ref, nu, sigma, rng = _grid(p, shear)
    ref.set_coef(0.01 * nu, sigma)
    ref.assemble()
    ref.set_ess(op.ess_mask())
    x = rng.standard_normal(op.ndof)
    want = ref.apply_masked(x)
    want32 = ref.apply_masked(x.astype(np.float32).astype(np.float64))
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    yd = torch.empty_like(xd)
    for shape, per in CONFIGS:
        op.SetLaunch(shape, per)
        assert op.GetLaunch() == {"shape": shape, "per_sm": per}
        y = op.Mult(x)
        assert np.linalg.norm(y - want) / np.linalg.norm(want) < 1e-12, (shape, per)
        op.MultDevice(xd, yd)
        torch.cuda.synchronize()
        y32 = yd.double().cpu().numpy()
        assert np.linalg.norm(y32 - want32) / np.linalg.norm(want32) < 2e-6, (shape, per)


@pytest.mark.parametrize("p", [1, 2])
def test_brick_shapes_complex_apply(p):
    op, ref, nu, sigma, rng = _grid(p, False, nx=13, ny=6, nz=3, seed=4, dt=1.0)
    Cn, M = CR.forms(ref, nu, sigma)
    omega = 50.0
    J = CR.eliminated(Cn, M, omega, op.ess_mask())
    x = rng.standard_normal(op.ndof) + 1j * rng.standard_normal(op.ndof)
    want = J @ x
    for shape, per in CONFIGS:
        op.SetLaunch(shape, per)
        y = op.MultComplex(omega, x)
        assert np.linalg.norm(y - want) / np.linalg.norm(want) < 1e-12, (shape, per)


def test_set_launch_rejects_bad_values():
    op, _, _, _, _ = _grid(2, False, nx=4, ny=4, nz=4)
    from hephaestus_gb300 import _native as N

    for shape, per in ((2, 0), (-1, 0), (0, -1), (0, 65)):
        with pytest.raises(N.HcError):
            op.SetLaunch(shape, per)


_CHILD = r"""
import json, sys
sys.path.insert(0, %r)
import numpy as np
from hephaestus_gb300 import HCurlOperator
op = HCurlOperator(20, 12, 6, 2, np.ones(1440), np.ones(1440), dt=0.01)
out = {"before": op.GetLaunch()}
if sys.argv[1] == "tune":
    out["tune"] = op.Autotune("real")
    out["tune_complex"] = op.Autotune("complex")
print(json.dumps(out))
"""


def test_autotune_chooses_and_persists(tmp_path):
    import json

    env = dict(os.environ, HC_TUNE_FILE=str(tmp_path / "tune.txt"))
    code = _CHILD % ROOT
    r1 = subprocess.run([sys.executable, "-c", code, "tune"], env=env, capture_output=True, text=True, timeout=600)
    assert r1.returncode == 0, r1.stderr
    a = json.loads(r1.stdout.strip().splitlines()[-1])
    assert a["before"] == {"shape": 0, "per_sm": 0}
    for t in (a["tune"], a["tune_complex"]):
        assert t["shape"] in (0, 1) and 0 <= t["per_sm"] <= 4
        assert 0 < t["us"] <= t["us_default"] * 1.0001
    lines = open(tmp_path / "tune.txt").read().split("\n")
    assert len([ln for ln in lines if ln.strip()]) == 2
    # a new process starts with the last stored choice for this problem
    r2 = subprocess.run([sys.executable, "-c", code, "none"], env=env, capture_output=True, text=True, timeout=600)
    assert r2.returncode == 0, r2.stderr
    b = json.loads(r2.stdout.strip().splitlines()[-1])
    last = a["tune_complex"]
    assert b["before"] == {"shape": last["shape"], "per_sm": last["per_sm"]}
