"""ctypes binding of the CUDA library's C ABI (include/hcurl_op.h).

The library is built in-tree (hephaestus_gb300/_lib/libhcurl_gb300.so).  There
is no CPU fallback: if the library is missing or cannot be loaded, every call
raises NativeUnavailable.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libhcurl_gb300.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "hcurl_op.h")

HC_OK, HC_EINVAL, HC_ENOMEM, HC_ECUDA, HC_NOT_CONVERGED, HC_BREAKDOWN, HC_TIMEOUT, HC_ENOTSUP = range(8)
STATUS_NAMES = ["OK", "EINVAL", "ENOMEM", "ECUDA", "NOT_CONVERGED", "BREAKDOWN", "TIMEOUT", "ENOTSUP"]
HC_HEX, HC_TET = 0, 1
HC_FP64, HC_FP32, HC_MIXED, HC_BF16, HC_MIXED_RR = 0, 1, 2, 3, 4
HC_PRECOND_NONE, HC_PRECOND_JACOBI, HC_PRECOND_CHEBYSHEV, HC_PRECOND_AUX, HC_PRECOND_AUX_MULT = 0, 1, 2, 3, 4
HC_FIELD_ELEM, HC_FIELD_QUAD = 0, 1


class NativeUnavailable(RuntimeError):
    pass


class HcError(RuntimeError):
    def __init__(self, status, msg):
        self.status = status
        super().__init__("%s: %s" % (STATUS_NAMES[status] if 0 <= status < 8 else status, msg))


class ProblemDesc(C.Structure):
    _fields_ = [
        ("elem_type", C.c_int32),
        ("order", C.c_int32),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("nz", C.c_int32),
        ("n_vert", C.c_int64),
        ("n_elem", C.c_int64),
        ("elem_verts", C.c_void_p),
        ("vertices", C.c_void_p),
        ("nu", C.c_void_p),
        ("sigma", C.c_void_p),
        ("dt", C.c_double),
        ("ess_mask", C.c_void_p),
        ("ess_attr_bits", C.c_int32),
        ("n_bdr", C.c_int64),
        ("bdr_tris", C.c_void_p),
        ("bdr_attr", C.c_void_p),
    ]


class SolveParams(C.Structure):
    _fields_ = [
        ("precision", C.c_int32),
        ("precond", C.c_int32),
        ("cheb_degree", C.c_int32),
        ("cheb_ratio", C.c_double),
        ("cheb_lmax", C.c_double),
        ("rtol", C.c_double),
        ("atol", C.c_double),
        ("maxit", C.c_int32),
        ("inner_rtol", C.c_double),
        ("max_outer", C.c_int32),
    ]


class SolveInfo(C.Structure):
    _fields_ = [
        ("status", C.c_int32),
        ("iterations", C.c_int32),
        ("outer_iterations", C.c_int32),
        ("applies", C.c_int32),
        ("rel_residual", C.c_double),
        ("lmax", C.c_double),
    ]


class Coil(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("I0", "xc", "yc", "r0", "r1", "z0", "z1")]


_lib = None

_SIGS = {
    "hc_create": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(C.c_void_p)]),
    "hc_destroy": (None, [C.c_void_p]),
    "hc_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hc_last_error": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "hc_num_dofs": (C.c_int64, [C.c_void_p]),
    "hc_num_elems": (C.c_int64, [C.c_void_p]),
    "hc_hex_dof_index": (C.c_int64, [C.c_void_p, C.c_int, C.c_int64, C.c_int64, C.c_int64]),
    "hc_get_ess_mask": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hc_mult": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_apply_form": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_add_weak_curlcurl": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    "hc_add_weak_curlcurl_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double]),
    "hc_diag": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hc_mult_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_mult_device_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_apply_form_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_add_mult_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_add_mult_device_f32": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_solve": (C.c_int, [C.c_void_p, C.POINTER(SolveParams), C.c_void_p, C.c_void_p, C.POINTER(SolveInfo)]),
    "hc_solve_device": (C.c_int, [C.c_void_p, C.POINTER(SolveParams), C.c_void_p, C.c_void_p,
                                  C.POINTER(SolveInfo)]),
    "hc_lanczos_lmax": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "hc_precond_apply_device": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "hc_set_launch": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "hc_get_launch": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "hc_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                              C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "hc_mult_multi_device": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "hc_elem_type": (C.c_int32, [C.c_void_p]),
    "hc_tet_element_matrix": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p]),
    "hc_num_rt_dofs": (C.c_int64, [C.c_void_p]),
    "hc_hex_rt_dof_index": (C.c_int64, [C.c_void_p, C.c_int, C.c_int64, C.c_int64, C.c_int64]),
    "hc_curl": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_curl_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_curl_static": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_mult_complex": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]),
    "hc_mult_complex_device": (C.c_int, [C.c_void_p, C.c_double] + [C.c_void_p] * 4),
    "hc_mult_complex_device_f32": (C.c_int, [C.c_void_p, C.c_double] + [C.c_void_p] * 4),
    "hc_solve_complex": (C.c_int, [C.c_void_p, C.POINTER(SolveParams), C.c_double, C.c_void_p, C.c_void_p,
                                   C.POINTER(SolveInfo)]),
    "hc_solve_complex_device": (C.c_int, [C.c_void_p, C.POINTER(SolveParams), C.c_double] + [C.c_void_p] * 4
                                + [C.POINTER(SolveInfo)]),
    "hc_solve_complex_graph": (C.c_int, [C.c_void_p, C.POINTER(SolveParams), C.c_double] + [C.c_void_p] * 4),
    "hc_graph_solve_info": (C.c_int, [C.c_void_p, C.POINTER(SolveInfo)]),
    "hc_solve_complex_batch": (C.c_int, [C.c_int32, C.c_void_p, C.POINTER(SolveParams), C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(SolveInfo)]),
    "hc_aux_levels": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32]),
    "hc_tet_gradient_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_solve_multi_device": (C.c_int, [C.c_void_p, C.POINTER(SolveParams), C.c_int32, C.c_void_p, C.c_void_p,
                                        C.POINTER(SolveInfo)]),
    "hc_solve_multi": (C.c_int, [C.c_void_p, C.POINTER(SolveParams), C.c_int32, C.c_void_p, C.c_void_p,
                                 C.POINTER(SolveInfo)]),
    "hc_load_coil": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "hc_hex_elem_dofs": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_void_p]),
    "hc_tet_elem_dofs": (C.c_int, [C.c_int32, C.c_int64, C.c_int64, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    "hc_dofmap_create": (C.c_int, [C.c_int64, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p,
                                   C.POINTER(C.c_void_p)]),
    "hc_dofmap_to_lib": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_dofmap_from_lib": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_dofmap_ess_mask": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]),
    "hc_dofmap_size": (C.c_int64, [C.c_void_p]),
    "hc_dofmap_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "hc_dofmap_destroy": (None, [C.c_void_p]),
    "hc_quad_points_device": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "hc_load_field_device": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    "hc_curl_load_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_magnetic_field_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.POINTER(SolveInfo)]),
    "hc_tet_curl_points_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "hc_be_rhs_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_be_update_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hc_be_steps_device": (C.c_int, [C.c_void_p, C.POINTER(SolveParams), C.c_int32, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.POINTER(SolveInfo)]),
    "hc_load_coil_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
}


def lib():
    """Load the native library (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise NativeUnavailable(
                "CUDA library %s is missing: run `python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        try:
            L = C.CDLL(LIB_PATH)
        except OSError as e:  # pragma: no cover
            raise NativeUnavailable("cannot load %s: %s" % (LIB_PATH, e))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def last_error(h=None):
    buf = C.create_string_buffer(512)
    lib().hc_last_error(h, buf, 512)
    return buf.value.decode(errors="replace")


def check(status, h=None):
    if status != HC_OK:
        raise HcError(status, last_error(h))
    return status


def declared_symbols(header=HEADER):
    """Function names declared by include/hcurl_op.h."""
    import re

    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(hc_[a-z0-9_]+)\s*\(", txt)))
