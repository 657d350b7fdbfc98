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


def _cudart():
    """The CUDA runtime as a shared library (the device's default memory pool
    is one per device, shared by every runtime instance in the process)."""
    import os

    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return C.CDLL(os.path.join(cuda_home, "lib64", "libcudart.so"))


def test_curl_static_allocates_nothing_in_the_call():
    """After the first call (which looks the static area up), a call leaves
    the default pool's used-memory high-water mark and the device's free
    memory unchanged: the library's per-handle work memory is stream-ordered
    from that pool, so a per-call allocation would raise the high-water mark
    even if it were freed again inside the call."""
    import torch

    cr = _cudart()
    USED_CURRENT, USED_HIGH = 7, 8  # cudaMemPoolAttrUsedMemCurrent / UsedMemHigh (driver_types.h)
    nx = ny = nz = 12
    op = HCurlOperator(nx, ny, nz, 2, np.ones(nx * ny * nz), None, ess_attr_bits=0)
    L = N.lib()
    nrt = L.hc_num_rt_dofs(op.h)
    A = np.random.default_rng(3).standard_normal(op.ndof)
    B = np.empty(nrt)
    N.check(L.hc_curl_static(op.h, _p(A), _p(B)), op.h)  # set-up call
    torch.cuda.synchronize()
    dev = C.c_int(0)
    assert cr.cudaGetDevice(C.byref(dev)) == 0
    pool = C.c_void_p()
    assert cr.cudaDeviceGetDefaultMemPool(C.byref(pool), dev) == 0

    def attr(a):
        v = C.c_uint64(0)
        assert cr.cudaMemPoolGetAttribute(pool, a, C.byref(v)) == 0
        return v.value

    zero = C.c_uint64(0)
    assert cr.cudaMemPoolSetAttribute(pool, USED_HIGH, C.byref(zero)) == 0  # reset the mark to the current use
    used0, high0 = attr(USED_CURRENT), attr(USED_HIGH)
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        N.check(L.hc_curl_static(op.h, _p(A), _p(B)), op.h)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert attr(USED_CURRENT) == used0
    assert attr(USED_HIGH) == high0
    assert free1 == free0


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
