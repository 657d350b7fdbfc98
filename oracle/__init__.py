"""ctypes binding of the FP64 CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; the product package never does.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int, C.c_double
        P = C.POINTER
        sig = {
            "orc_hex_new": (vp, [i32, i32, i32, i32, vp]),
            "orc_tet_new": (vp, [i64, vp, i64, vp, i32]),
            "orc_free": (None, [vp]),
            "orc_ndof": (i64, [vp]),
            "orc_nelem": (i64, [vp]),
            "orc_ldof": (i32, [vp]),
            "orc_elem_dofs": (None, [vp, vp]),
            "orc_tet_nedges": (i64, [vp]),
            "orc_tet_nfaces": (i64, [vp]),
            "orc_set_coef": (None, [vp, vp, vp]),
            "orc_set_coef_mms": (None, [vp, dbl, dbl, dbl]),
            "orc_set_quad": (None, [vp, i32, i32]),
            "orc_assemble": (i32, [vp, i32]),
            "orc_nnz": (i64, [vp]),
            "orc_csr": (None, [vp, vp, vp, vp]),
            "orc_element_matrix": (None, [vp, i64, vp]),
            "orc_hex_ess_mask": (None, [vp, i32, vp]),
            "orc_tet_ess_mask": (None, [vp, i64, vp, vp, i32, vp]),
            "orc_set_ess": (None, [vp, vp]),
            "orc_apply": (None, [vp, vp, vp, i32]),
            "orc_apply_masked": (None, [vp, vp, vp, i32]),
            "orc_diag_masked": (None, [vp, vp]),
            "orc_apply_curlcurl": (None, [vp, vp, vp]),
            "orc_build_eliminated": (i64, [vp]),
            "orc_spmv_eliminated": (None, [vp, vp, vp, i32]),
            "orc_pcg": (i32, [vp, vp, vp, i32, i32, dbl, dbl, dbl, dbl, i32, i32, P(i32), P(dbl)]),
            "orc_lanczos_lmax": (dbl, [vp, i32, i32]),
            "orc_cheb_apply": (None, [vp, i32, dbl, dbl, vp, vp, i32]),
            "orc_load_coil": (None, [vp, dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, vp]),
            "orc_load_mms": (None, [vp, dbl, dbl, i32, vp]),
            "orc_load_elem_field": (None, [vp, vp, i32, vp]),
            "orc_load_affine": (None, [vp, vp, vp, i32, vp]),
            "orc_curl_load": (None, [vp, vp, vp, i32, vp]),
            "orc_l2err_mms": (dbl, [vp, vp, dbl, i32]),
            "orc_eval": (None, [vp, vp, i64, vp, vp, vp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


NT = max(1, os.cpu_count() or 1)


class Problem:
    """One discretised problem (hex or tet) held by the oracle."""

    def __init__(self, handle):
        if not handle:
            raise ValueError("oracle rejected the problem description")
        self.h = handle
        L = lib()
        self.ndof = L.orc_ndof(handle)
        self.ne = L.orc_nelem(handle)
        self.ldof = L.orc_ldof(handle)

    @classmethod
    def hex(cls, nx, ny, nz, p, verts=None):
        v = None if verts is None else np.ascontiguousarray(verts, dtype=np.float64)
        return cls(lib().orc_hex_new(nx, ny, nz, p, _p(v)))

    @classmethod
    def tet(cls, verts, tets, p):
        v = np.ascontiguousarray(verts, dtype=np.float64)
        t = np.ascontiguousarray(tets, dtype=np.int64)
        return cls(lib().orc_tet_new(v.shape[0], _p(v), t.shape[0], _p(t), p))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_free(self.h)
            self.h = None

    def elem_dofs(self):
        out = np.empty((self.ne, self.ldof), dtype=np.int64)
        lib().orc_elem_dofs(self.h, _p(out))
        return out

    def set_coef(self, alpha, beta=None):
        self._a = np.ascontiguousarray(alpha, dtype=np.float64)
        self._b = None if beta is None else np.ascontiguousarray(beta, dtype=np.float64)
        lib().orc_set_coef(self.h, _p(self._a), _p(self._b))

    def set_coef_mms(self, dt, var_scale, sigma):
        lib().orc_set_coef_mms(self.h, dt, var_scale, sigma)

    def set_quad(self, q_curl, q_mass):
        lib().orc_set_quad(self.h, q_curl, q_mass)

    def assemble(self):
        lib().orc_assemble(self.h, NT)

    def csr(self):
        import scipy.sparse as sp

        nnz = lib().orc_nnz(self.h)
        rp = np.empty(self.ndof + 1, dtype=np.int64)
        ci = np.empty(nnz, dtype=np.int64)
        va = np.empty(nnz, dtype=np.float64)
        lib().orc_csr(self.h, _p(rp), _p(ci), _p(va))
        return sp.csr_matrix((va, ci, rp), shape=(self.ndof, self.ndof))

    def element_matrix(self, e):
        out = np.empty((self.ldof, self.ldof))
        lib().orc_element_matrix(self.h, e, _p(out))
        return out

    def hex_ess_mask(self, attr_bits=0x3F):
        m = np.zeros(self.ndof, dtype=np.uint8)
        lib().orc_hex_ess_mask(self.h, attr_bits, _p(m))
        return m

    def tet_ess_mask(self, tris, attrs, attr_bits=~0):
        t = np.ascontiguousarray(tris, dtype=np.int64)
        a = np.ascontiguousarray(attrs, dtype=np.int32)
        m = np.zeros(self.ndof, dtype=np.uint8)
        lib().orc_tet_ess_mask(self.h, t.shape[0], _p(t), _p(a), attr_bits & 0x7FFFFFFF, _p(m))
        return m

    def set_ess(self, mask):
        self._m = np.ascontiguousarray(mask, dtype=np.uint8)
        lib().orc_set_ess(self.h, _p(self._m))

    def apply(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib().orc_apply(self.h, _p(x), _p(y), NT)
        return y

    def apply_masked(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib().orc_apply_masked(self.h, _p(x), _p(y), NT)
        return y

    def apply_curlcurl(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib().orc_apply_curlcurl(self.h, _p(x), _p(y))
        return y

    def diag_masked(self):
        d = np.empty(self.ndof)
        lib().orc_diag_masked(self.h, _p(d))
        return d

    def lanczos_lmax(self, steps=20):
        return lib().orc_lanczos_lmax(self.h, steps, NT)

    def cheb_apply(self, r, degree, lmax, ratio):
        r = np.ascontiguousarray(r, dtype=np.float64)
        z = np.empty_like(r)
        lib().orc_cheb_apply(self.h, degree, lmax, ratio, _p(r), _p(z), NT)
        return z

    def pcg(self, b, x0=None, precond=1, cheb_degree=2, cheb_lmax=0.0, cheb_ratio=30.0,
            rtol=1e-12, atol=0.0, maxit=10000, nthreads=None):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=np.float64)
        it = C.c_int(0)
        rr = C.c_double(0)
        st = lib().orc_pcg(self.h, _p(b), _p(x), precond, cheb_degree, cheb_lmax, cheb_ratio,
                           rtol, atol, maxit, nthreads or NT, C.byref(it), C.byref(rr))
        return x, st, it.value, rr.value

    def load_coil(self, I0=1.0, xc=0.5, yc=0.5, r0=0.2, r1=0.35, z0=0.3, z1=0.7, q=None):
        b = np.empty(self.ndof)
        lib().orc_load_coil(self.h, I0, xc, yc, r0, r1, z0, z1, q or 4, _p(b))
        return b

    def load_elem_field(self, J, q=4):
        J = np.ascontiguousarray(J, dtype=np.float64)
        b = np.empty(self.ndof)
        lib().orc_load_elem_field(self.h, _p(J), q, _p(b))
        return b

    def load_affine(self, a, B, q=4):
        a = np.ascontiguousarray(a, dtype=np.float64)
        B = np.ascontiguousarray(B, dtype=np.float64)
        b = np.empty(self.ndof)
        lib().orc_load_affine(self.h, _p(a), _p(B), q, _p(b))
        return b

    def curl_load(self, nu, A, q=6):
        nu = np.ascontiguousarray(nu, dtype=np.float64)
        A = np.ascontiguousarray(A, dtype=np.float64)
        b = np.empty(self.ndof)
        lib().orc_curl_load(self.h, _p(nu), _p(A), q, _p(b))
        return b

    def load_mms(self, t, var_scale=0.5, q=6):
        b = np.empty(self.ndof)
        lib().orc_load_mms(self.h, t, var_scale, q, _p(b))
        return b

    def l2err_mms(self, A, t, q=6):
        A = np.ascontiguousarray(A, dtype=np.float64)
        return lib().orc_l2err_mms(self.h, _p(A), t, q)

    def eval(self, A, e, xi):
        A = np.ascontiguousarray(A, dtype=np.float64)
        xi = np.ascontiguousarray(xi, dtype=np.float64)
        v = np.empty(3)
        c = np.empty(3)
        lib().orc_eval(self.h, _p(A), e, _p(xi), _p(v), _p(c))
        return v, c
