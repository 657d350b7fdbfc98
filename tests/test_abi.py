"""CPU tests of the C ABI boundary: the library loads, exports exactly what
include/hcurl_op.h declares, and rejects bad input before touching a GPU."""
import ctypes as C

import numpy as np
import pytest

from hephaestus_gb300 import _native as N


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = N.declared_symbols()
    assert len(names) >= 18
    for n in names:
        assert hasattr(L, n), n


def _desc(**kw):
    d = N.ProblemDesc()
    d.elem_type = N.HC_HEX
    d.order = 2
    d.nx = d.ny = d.nz = 2
    d.dt = 1.0
    for k, v in kw.items():
        setattr(d, k, v)
    return d


@pytest.mark.parametrize("field,value,needle", [
    ("order", 0, "order"),
    ("order", 4, "order"),
    ("nx", 0, "nx"),
    ("dt", 0.0, "dt"),
    ("elem_type", 7, "elem_type"),
])
def test_create_rejects_bad_descriptor(field, value, needle):
    nu = np.ones(8)
    d = _desc(nu=nu.ctypes.data_as(C.c_void_p))
    setattr(d, field, value)
    h = C.c_void_p()
    st = N.lib().hc_create(C.byref(d), C.byref(h))
    assert st == N.HC_EINVAL
    assert needle in N.last_error(None)
    assert not h.value


def test_create_rejects_missing_or_bad_coefficients():
    h = C.c_void_p()
    d = _desc()
    assert N.lib().hc_create(C.byref(d), C.byref(h)) == N.HC_EINVAL
    assert "nu" in N.last_error(None)
    nu = np.ones(8)
    nu[3] = np.nan
    d = _desc(nu=nu.ctypes.data_as(C.c_void_p))
    assert N.lib().hc_create(C.byref(d), C.byref(h)) == N.HC_EINVAL
    sig = -np.ones(8)
    nu = np.ones(8)
    d = _desc(nu=nu.ctypes.data_as(C.c_void_p), sigma=sig.ctypes.data_as(C.c_void_p))
    assert N.lib().hc_create(C.byref(d), C.byref(h)) == N.HC_EINVAL
    assert "sigma" in N.last_error(None)


def test_null_arguments_return_einval():
    L = N.lib()
    assert L.hc_create(None, None) == N.HC_EINVAL
    assert L.hc_mult(None, None, None) == N.HC_EINVAL
    assert L.hc_solve(None, None, None, None, None) == N.HC_EINVAL
    assert L.hc_diag(None, None) == N.HC_EINVAL
    assert L.hc_num_dofs(None) == -1
    assert L.hc_last_error(None, None, 0) == N.HC_EINVAL
    L.hc_destroy(None)  # no-op
    # sources, fields and time stepping
    assert L.hc_quad_points_device(None, 2, None) == N.HC_EINVAL
    assert L.hc_load_field_device(None, N.HC_FIELD_ELEM, 2, None, None) == N.HC_EINVAL
    assert L.hc_curl_load_device(None, None, None) == N.HC_EINVAL
    assert L.hc_magnetic_field_device(None, None, None, 1e-12, None) == N.HC_EINVAL
    assert L.hc_tet_curl_points_device(None, None, 1, None, None) == N.HC_EINVAL
    assert L.hc_be_rhs_device(None, None, None, None) == N.HC_EINVAL
    assert L.hc_be_update_device(None, None, None) == N.HC_EINVAL
    assert L.hc_be_steps_device(None, None, 1, None, None, None, None, None) == N.HC_EINVAL
    assert L.hc_precond_apply_device(None, N.HC_PRECOND_AUX, None, None) == N.HC_EINVAL


def test_mfem_shim_compiles_against_stub():
    """include/hcurl_mfem.hpp (the reference-side binding) type-checks and
    links against the library."""
    import os
    import subprocess
    import tempfile

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = os.path.join(tempfile.mkdtemp(), "shim.so")
    cmd = ["g++", "-std=c++17", "-shared", "-fPIC", "-I", os.path.join(root, "include"),
           "-I", os.path.join(root, "tests", "mfem_stub"), os.path.join(root, "tests", "mfem_shim_check.cpp"),
           "-o", out, "-L", os.path.dirname(N.LIB_PATH), "-lhcurl_gb300"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_header_is_plain_c():
    """The ABI header compiles as C (no C++ or torch types)."""
    import os
    import subprocess

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-x", "c", os.path.join(root, "include", "hcurl_op.h")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_tet_descriptor_validation():
    L = N.lib()
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], dtype=np.float64)
    t = np.array([[0, 1, 2, 3]], dtype=np.int64)
    nu = np.ones(1)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    for order, tets, msg in ((3, t, "order"), (1, np.array([[0, 1, 1, 3]], dtype=np.int64), "degenerate"),
                             (1, np.array([[0, 1, 2, 7]], dtype=np.int64), "range")):
        d = N.ProblemDesc()
        d.elem_type, d.order, d.dt = N.HC_TET, order, 1.0
        d.n_vert, d.n_elem = 4, 1
        d.vertices, d.elem_verts, d.nu = P(v), P(tets), P(nu)
        h = C.c_void_p()
        assert L.hc_create(C.byref(d), C.byref(h)) == N.HC_EINVAL
        assert msg in N.last_error(None)


def test_block_solve_and_gradient_entries_reject_null_arguments():
    """The multi-RHS solve, the discrete gradient and the AMG level query
    reject missing handles or arrays before any device work."""
    L = N.lib()
    p = N.SolveParams()
    info = (N.SolveInfo * 16)()
    assert L.hc_solve_multi_device(None, C.byref(p), 16, None, None, info) == N.HC_EINVAL
    assert L.hc_tet_gradient_device(None, None, None) == N.HC_EINVAL
    sizes = np.zeros(8, dtype=np.int64)
    assert L.hc_aux_levels(None, sizes.ctypes.data_as(C.c_void_p), 8) == 0
    assert L.hc_load_coil_device(None, None, 4, None) == N.HC_EINVAL


def test_solver_option_names_map_to_the_abi():
    """GpuHCurlPCGSolver reads the reference's option names plus the build's
    precision/preconditioner options into hc_solve_params."""
    from hephaestus_gb300 import GpuHCurlPCGSolver

    s = GpuHCurlPCGSolver({"Tolerance": 1e-10, "AbsTolerance": 0.0, "MaxIter": 123, "Precision": "mixed",
                           "Preconditioner": "aux", "InnerTolerance": 0.1, "MaxOuter": 7})
    assert s.p.rtol == 1e-10 and s.p.atol == 0.0 and s.p.maxit == 123
    assert s.p.precision == N.HC_MIXED and s.p.precond == N.HC_PRECOND_AUX
    assert s.p.inner_rtol == 0.1 and s.p.max_outer == 7


def test_block_solve_wrapper_checks_shapes_before_the_device():
    """Shape errors are reported by the Python wrapper before any device call."""
    torch = pytest.importorskip("torch")
    from hephaestus_gb300 import GpuHCurlPCGSolver

    class FakeOp:
        ndof = 10
        h = None

    s = GpuHCurlPCGSolver({}, FakeOp())
    with pytest.raises(ValueError, match="same shape"):
        s.MultMultiDevice(torch.zeros(10, 4, dtype=torch.float64), torch.zeros(10, 2, dtype=torch.float64))
    with pytest.raises(ValueError, match="rows"):
        s.MultMultiDevice(torch.zeros(9, 4, dtype=torch.float64), torch.zeros(9, 4, dtype=torch.float64))
    with pytest.raises(ValueError, match="right-hand sides"):
        s.MultMultiDevice(torch.zeros(10, 3, dtype=torch.float64), torch.zeros(10, 3, dtype=torch.float64))


def test_host_block_solve_rejects_bad_arguments():
    L = N.lib()
    p = N.SolveParams()
    info = (N.SolveInfo * 16)()
    assert L.hc_solve_multi(None, C.byref(p), 16, None, None, info) == N.HC_EINVAL
