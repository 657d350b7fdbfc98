"""hc_curl_static (B = curl A staged in static device memory, no allocation in
the call) against hc_curl, through the C ABI.  Collected last on purpose: it
must pass both alone in a fresh process and after every other GPU test."""
import ctypes as C

import numpy as np
import pytest

from hephaestus_gb300 import HCurlOperator
from hephaestus_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


@pytest.mark.parametrize("nx,ny,nz,p", [(16, 16, 16, 1), (10, 7, 5, 2), (6, 5, 4, 3)])
def test_curl_static_matches_curl_twice(nx, ny, nz, p):
    rng = np.random.default_rng(100 + p)
    op = HCurlOperator(nx, ny, nz, p, rng.uniform(0.5, 2.0, nx * ny * nz), None, ess_attr_bits=0)
    L = N.lib()
    nrt = L.hc_num_rt_dofs(op.h)
    assert 0 < nrt <= (1 << 20)
    for call in range(2):
        A = rng.standard_normal(op.ndof)
        ref = np.empty(nrt)
        N.check(L.hc_curl(op.h, _p(A), _p(ref)), op.h)
        B = np.full(nrt, np.nan)
        N.check(L.hc_curl_static(op.h, _p(A), _p(B)), op.h)
        scale = np.abs(ref).max()
        assert np.all(np.isfinite(B)), call
        # same kernel and inputs: equal up to rounding (tolerance 1e-13 of the largest entry)
        assert np.abs(B - ref).max() <= 1e-13 * scale, call


def test_curl_static_rejects_grids_beyond_the_scratch():
    n, p = 48, 2   # 3 * 97 * 96 * 96 = 2,681,856 RT dofs > 2^20
    op = HCurlOperator(n, n, n, p, np.ones(n ** 3), None, ess_attr_bits=0)
    L = N.lib()
    assert L.hc_num_rt_dofs(op.h) > (1 << 20)
    A = np.ones(op.ndof)
    B = np.zeros(L.hc_num_rt_dofs(op.h))
    st = L.hc_curl_static(op.h, _p(A), _p(B))
    assert st == N.HC_EINVAL
    assert "static scratch" in N.last_error(op.h)
    # a smaller handle still works after the rejection
    small = HCurlOperator(4, 4, 4, 1, np.ones(64), None, ess_attr_bits=0)
    A = np.random.default_rng(7).standard_normal(small.ndof)
    nrt = L.hc_num_rt_dofs(small.h)
    ref, B = np.empty(nrt), np.empty(nrt)
    N.check(L.hc_curl(small.h, _p(A), _p(ref)), small.h)
    N.check(L.hc_curl_static(small.h, _p(A), _p(B)), small.h)
    assert np.abs(B - ref).max() <= 1e-13 * np.abs(ref).max()
