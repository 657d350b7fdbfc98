"""Host-side mirror of the reference's operator/solver interface for this path.

Reference shape (C++, MFEM-based):
  - kernels add integrators to a ParBilinearForm:
      CurlCurlKernel::Apply     -> CurlCurlIntegrator(dt*alpha)
                                   (src/kernels/curl_curl_kernel.cpp:21-24)
      VectorFEMassKernel::Apply -> VectorFEMassIntegrator(beta)
                                   (src/kernels/vector_fe_mass_kernel.cpp:21-24)
      WeakCurlCurlKernel::Apply -> lf += -C_alpha u_n
                                   (src/kernels/weak_curl_curl_kernel.cpp:14-31)
  - EquationSystem (an mfem::Operator) exposes Mult / GetGradient of the
    eliminated system (src/equation_systems/equation_system.cpp:133-210);
  - solvers are configured from InputParameters "Tolerance", "AbsTolerance",
    "MaxIter", "PrintLevel" (src/solvers/hephaestus_solvers.hpp:34-86).

Here the same roles sit on the C ABI: HCurlForm collects the kernels'
coefficients like a ParBilinearForm, HCurlOperator is the assembled
(matrix-free, device-resident) Jacobian with Mult/GetGradient/
FormLinearSystem, and GpuHCurlPCGSolver takes the reference's solver option
names.  Errors raise, mirroring MFEM_ABORT at this layer.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def _ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(C.c_void_p)
    return C.c_void_p(int(a.data_ptr()))  # torch tensor


def _dev_ptr(t, dtype_name):
    import torch

    if not isinstance(t, torch.Tensor) or not t.is_cuda or not t.is_contiguous():
        raise TypeError("expected a contiguous CUDA tensor")
    if str(t.dtype) != "torch." + dtype_name:
        raise TypeError("expected dtype %s, got %s" % (dtype_name, t.dtype))
    return C.c_void_p(t.data_ptr())


# ----------------------------------------------------------------------------
# kernels (coefficient registration, like hephaestus::Kernel<ParBilinearForm>)
# ----------------------------------------------------------------------------
class CurlCurlKernel:
    """Adds (coef curl u, curl u') to a form; coef is per element."""

    def __init__(self, coef):
        self.coef = np.ascontiguousarray(coef, dtype=np.float64)

    def Apply(self, form):
        form.curl_coefs.append(self.coef)


class VectorFEMassKernel:
    """Adds (coef u, u') to a form; coef is per element."""

    def __init__(self, coef):
        self.coef = np.ascontiguousarray(coef, dtype=np.float64)

    def Apply(self, form):
        form.mass_coefs.append(self.coef)


class HCurlForm:
    """Structured-hex Nedelec bilinear form, filled by kernels, assembled on the device.

    Geometry: nx*ny*nz parallelepiped hexes with vertices (x fastest) or the
    unit cube.  The assembled operator is K = sum curl terms + sum mass terms.
    """

    def __init__(self, nx, ny, nz, order, vertices=None):
        self.nx, self.ny, self.nz, self.order = nx, ny, nz, order
        self.vertices = None if vertices is None else np.ascontiguousarray(vertices, dtype=np.float64)
        self.curl_coefs = []
        self.mass_coefs = []

    def Assemble(self, ess_attr_bits=0, ess_mask=None):
        if not self.curl_coefs:
            raise ValueError("a curl-curl kernel is required")
        nu = np.sum(self.curl_coefs, axis=0)
        sigma = np.sum(self.mass_coefs, axis=0) if self.mass_coefs else None
        return HCurlOperator(self.nx, self.ny, self.nz, self.order, nu, sigma, dt=1.0,
                             vertices=self.vertices, ess_attr_bits=ess_attr_bits, ess_mask=ess_mask)


class HCurlOperator:
    """Device-resident eliminated operator J = P K P + (I - P),  K = dt C_nu + M_sigma.

    Mult(x, y) is EquationSystem::Mult; GetGradient() returns self (the
    operator is linear); FormLinearSystem applies MFEM's elimination to a
    right-hand side.
    """

    @classmethod
    def from_tets(cls, verts, tets, order, nu, sigma=None, dt=1.0, btris=None, battr=None, ess_attr_bits=~0,
                  ess_mask=None, stream=None):
        """Tetrahedral mesh (vertices n x 3, tets m x 4), Nedelec order 1 or 2.
        Essential dofs: boundary triangles with attributes selected by
        ess_attr_bits, or an explicit per-dof mask."""
        self = cls.__new__(cls)
        keep = dict(verts=np.ascontiguousarray(verts, dtype=np.float64),
                    tets=np.ascontiguousarray(tets, dtype=np.int64),
                    nu=np.ascontiguousarray(nu, dtype=np.float64),
                    sigma=None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64),
                    btris=None if btris is None else np.ascontiguousarray(btris, dtype=np.int64),
                    battr=None if battr is None else np.ascontiguousarray(battr, dtype=np.int32),
                    mask=None if ess_mask is None else np.ascontiguousarray(ess_mask, dtype=np.uint8))
        d = N.ProblemDesc()
        d.elem_type = N.HC_TET
        d.order = order
        d.n_vert = keep["verts"].shape[0]
        d.n_elem = keep["tets"].shape[0]
        d.vertices = _ptr(keep["verts"])
        d.elem_verts = _ptr(keep["tets"])
        d.nu = _ptr(keep["nu"])
        d.sigma = _ptr(keep["sigma"])
        d.dt = dt
        d.ess_mask = _ptr(keep["mask"])
        d.ess_attr_bits = ess_attr_bits & 0x7FFFFFFF
        if keep["btris"] is not None:
            d.n_bdr = keep["btris"].shape[0]
            d.bdr_tris = _ptr(keep["btris"])
            d.bdr_attr = _ptr(keep["battr"])
        self._finish(d, keep, dt, order, stream)
        self.nx = self.ny = self.nz = None
        return self

    def _finish(self, d, keep, dt, order, stream):
        L = N.lib()
        h = C.c_void_p()
        st = L.hc_create(C.byref(d), C.byref(h))
        if st != N.HC_OK:
            raise N.HcError(st, N.last_error(None))
        self._keep = keep
        self._nu = keep["nu"]
        self.h = h
        self.order, self.dt = order, dt
        self.ndof = L.hc_num_dofs(h)
        self.ne = L.hc_num_elems(h)
        self.height = self.width = self.ndof
        if stream is not None:
            self.set_stream(stream)

    def __init__(self, nx, ny, nz, order, nu, sigma=None, dt=1.0, vertices=None, ess_attr_bits=0x3F,
                 ess_mask=None, stream=None):
        L = N.lib()
        ne = nx * ny * nz
        self._nu = np.ascontiguousarray(nu, dtype=np.float64)
        self._sigma = None if sigma is None else np.ascontiguousarray(sigma, dtype=np.float64)
        if self._nu.shape != (ne,) or (self._sigma is not None and self._sigma.shape != (ne,)):
            raise ValueError("nu/sigma must have one value per element (%d)" % ne)
        self._verts = None if vertices is None else np.ascontiguousarray(vertices, dtype=np.float64)
        self._mask = None if ess_mask is None else np.ascontiguousarray(ess_mask, dtype=np.uint8)
        d = N.ProblemDesc()
        d.elem_type = N.HC_HEX
        d.order = order
        d.nx, d.ny, d.nz = nx, ny, nz
        d.vertices = _ptr(self._verts)
        d.nu = _ptr(self._nu)
        d.sigma = _ptr(self._sigma)
        d.dt = dt
        d.ess_mask = _ptr(self._mask)
        d.ess_attr_bits = ess_attr_bits
        h = C.c_void_p()
        st = L.hc_create(C.byref(d), C.byref(h))
        if st != N.HC_OK:
            raise N.HcError(st, N.last_error(None))
        self.h = h
        self.nx, self.ny, self.nz, self.order, self.dt = nx, ny, nz, order, dt
        self.ndof = L.hc_num_dofs(h)
        self.ne = L.hc_num_elems(h)
        self.height = self.width = self.ndof
        if stream is not None:
            self.set_stream(stream)

    # -- lifecycle --
    def close(self):
        if getattr(self, "h", None):
            N.lib().hc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        """stream: a torch.cuda.Stream or a raw cudaStream_t integer."""
        s = getattr(stream, "cuda_stream", stream)
        N.check(N.lib().hc_set_stream(self.h, C.c_void_p(int(s) if s else 0)), self.h)

    # -- layout --
    def dof_index(self, c, i, j, k):
        return N.lib().hc_hex_dof_index(self.h, c, i, j, k)

    def ess_mask(self):
        m = np.zeros(self.ndof, dtype=np.uint8)
        N.check(N.lib().hc_get_ess_mask(self.h, _ptr(m)), self.h)
        return m

    # -- host-vector actions (mfem::Vector host data) --
    def _h(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != (self.ndof,):
            raise ValueError("vector length %s != %d" % (x.shape, self.ndof))
        return x

    def Mult(self, x, y=None):
        x = self._h(x)
        y = np.empty_like(x) if y is None else y
        N.check(N.lib().hc_mult(self.h, _ptr(x), _ptr(y)), self.h)
        return y

    def GetGradient(self, x=None):
        return self

    def ApplyForm(self, x):
        """K x without elimination."""
        x = self._h(x)
        y = np.empty_like(x)
        N.check(N.lib().hc_apply_form(self.h, _ptr(x), _ptr(y)), self.h)
        return y

    def AddWeakCurlCurl(self, u, lf, scale=-1.0):
        """lf += scale * C_nu u   (WeakCurlCurlKernel::Apply with scale -1)."""
        u = self._h(u)
        if not (isinstance(lf, np.ndarray) and lf.dtype == np.float64 and lf.flags.c_contiguous):
            raise TypeError("lf must be a contiguous float64 array (updated in place)")
        N.check(N.lib().hc_add_weak_curlcurl(self.h, _ptr(u), _ptr(lf), scale), self.h)
        return lf

    def AddWeakCurlCurlDevice(self, u, lf, scale=-1.0):
        """lf += scale * C_nu u on float64 device tensors (WeakCurlCurlKernel::Apply)."""
        N.check(N.lib().hc_add_weak_curlcurl_device(self.h, _dev_ptr(u, "float64"), _dev_ptr(lf, "float64"),
                                                    float(scale)), self.h)
        return lf

    def Diagonal(self):
        d = np.empty(self.ndof)
        N.check(N.lib().hc_diag(self.h, _ptr(d)), self.h)
        return d

    def FormLinearSystem(self, x_bc, b):
        """MFEM FormLinearSystem for J: B = P (b - K (I-P) x_bc) + (I-P) x_bc, X = x_bc."""
        m = self.ess_mask().astype(bool)
        xb = np.where(m, self._h(x_bc), 0.0)
        B = np.array(self._h(b), copy=True)
        if np.any(xb):
            B -= self.ApplyForm(xb)
        B[m] = xb[m]
        return np.array(x_bc, dtype=np.float64, copy=True), B

    # -- device actions (torch CUDA tensors) --
    def MultDevice(self, x, y):
        if str(x.dtype) == "torch.float32":
            N.check(N.lib().hc_mult_device_f32(self.h, _dev_ptr(x, "float32"), _dev_ptr(y, "float32")), self.h)
        else:
            N.check(N.lib().hc_mult_device(self.h, _dev_ptr(x, "float64"), _dev_ptr(y, "float64")), self.h)
        return y

    def AddMultDevice(self, x, y):
        """y += P K P x on device tensors (float32 or float64)."""
        if str(x.dtype) == "torch.float32":
            N.check(N.lib().hc_add_mult_device_f32(self.h, _dev_ptr(x, "float32"), _dev_ptr(y, "float32")), self.h)
        else:
            N.check(N.lib().hc_add_mult_device(self.h, _dev_ptr(x, "float64"), _dev_ptr(y, "float64")), self.h)
        return y

    def ElementMatrix(self, e):
        """FP64 element matrix of tet e (local dof order of the basis)."""
        L = 6 if self.order == 1 else 20
        out = np.empty((L, L))
        N.check(N.lib().hc_tet_element_matrix(self.h, e, _ptr(out)), self.h)
        return out

    def MultMultiDevice(self, X, Y, bf16_matrices=False):
        """Y = J X for a (ndof, nrhs) row-major CUDA tensor (float32 or float64);
        bf16_matrices (float32 tensors, tets): element matrices read as BF16."""
        prec = N.HC_FP32 if str(X.dtype) == "torch.float32" else N.HC_FP64
        if bf16_matrices:
            prec = N.HC_BF16
        name = "float64" if prec == N.HC_FP64 else "float32"
        nrhs = 1 if X.dim() == 1 else X.shape[1]
        if int(X.shape[0]) != self.ndof or tuple(Y.shape) != tuple(X.shape):
            raise ValueError("X and Y must both be (ndof, nrhs) with ndof = %d" % self.ndof)
        N.check(N.lib().hc_mult_multi_device(self.h, prec, nrhs, _dev_ptr(X, name), _dev_ptr(Y, name)), self.h)
        return Y

    def AuxLevels(self):
        """Sizes of the tet auxiliary-space AMG levels (free vertices first) and
        the number of free edge bubbles, once an 'aux' solve has set it up."""
        sizes = np.zeros(16, dtype=np.int64)
        n = N.lib().hc_aux_levels(self.h, _ptr(sizes), 15)
        return {"levels": [int(x) for x in sizes[:n]], "edge_bubbles": int(sizes[n]) if n else 0}

    def GradientDevice(self, u, y):
        """y = G u: discrete gradient of P1 vertex values u (float64 CUDA tensor
        of n_vert entries) into this Nedelec space (tet meshes)."""
        N.check(N.lib().hc_tet_gradient_device(self.h, _dev_ptr(u, "float64"), _dev_ptr(y, "float64")), self.h)
        return y

    def ApplyFormDevice(self, x, y):
        N.check(N.lib().hc_apply_form_device(self.h, _dev_ptr(x, "float64"), _dev_ptr(y, "float64")), self.h)
        return y

    # -- around the solve --
    def Curl(self, A):
        """B = curl A as Raviart-Thomas dofs (CurlAuxSolver)."""
        A = self._h(A)
        B = np.empty(N.lib().hc_num_rt_dofs(self.h))
        N.check(N.lib().hc_curl(self.h, _ptr(A), _ptr(B)), self.h)
        return B

    def rt_dof_index(self, c, i, j, k):
        return N.lib().hc_hex_rt_dof_index(self.h, c, i, j, k)

    def LoadCoil(self, I0=1.0, xc=0.5, yc=0.5, r0=0.2, r1=0.35, z0=0.3, z1=0.7, q=None):
        """b_i = (J, w_i) of the loop coil (DivFreeSource's right-hand side)."""
        coil = N.Coil(I0, xc, yc, r0, r1, z0, z1)
        b = np.empty(self.ndof)
        N.check(N.lib().hc_load_coil(self.h, C.byref(coil), int(q or self.order + 2), _ptr(b)), self.h)
        return b

    def LoadCoilDevice(self, b, I0=1.0, xc=0.5, yc=0.5, r0=0.2, r1=0.35, z0=0.3, z1=0.7, q=None):
        coil = N.Coil(I0, xc, yc, r0, r1, z0, z1)
        N.check(N.lib().hc_load_coil_device(self.h, C.byref(coil), int(q or self.order + 2),
                                            _dev_ptr(b, "float64")), self.h)
        return b

    # -- sources and fields (DivFreeSource load, CurlAuxSolver, ScaledCurlVectorGridFunctionAux) --
    def QuadPointsDevice(self, q):
        """Physical points of the q^3 rule the load entry points use, a
        (ne, q^3, 3) float64 CUDA tensor (hex: kx + q (ky + q kz); tet:
        collapsed rule, ic + q (ib + q ia))."""
        import torch

        xyz = torch.empty(self.ne, q ** 3, 3, dtype=torch.float64, device="cuda")
        N.check(N.lib().hc_quad_points_device(self.h, int(q), _dev_ptr(xyz, "float64")), self.h)
        return xyz

    def LoadFieldDevice(self, J, b, q=None):
        """b = (J, w_i) for a caller-supplied source: J of shape (ne, 3) (one
        vector per element) or (ne, q^3, 3) (values at QuadPointsDevice(q))."""
        per_point = J.dim() == 3
        if per_point:
            q = round(int(J.shape[1]) ** (1.0 / 3.0))
            if q ** 3 != int(J.shape[1]):
                raise ValueError("J must be (ne, q^3, 3)")
        else:
            q = int(q or self.order + 1)
        if int(J.shape[0]) != self.ne or int(J.shape[-1]) != 3:
            raise ValueError("J must have ne = %d rows of 3-vectors" % self.ne)
        mode = N.HC_FIELD_QUAD if per_point else N.HC_FIELD_ELEM
        N.check(N.lib().hc_load_field_device(self.h, mode, int(q), _dev_ptr(J, "float64"), _dev_ptr(b, "float64")),
                self.h)
        return b

    def CurlLoadDevice(self, A, b):
        """b_i = (nu curl A, w_i) with the operator's per-element nu."""
        N.check(N.lib().hc_curl_load_device(self.h, _dev_ptr(A, "float64"), _dev_ptr(b, "float64")), self.h)
        return b

    def MagneticFieldDevice(self, A, H, rtol=1e-12):
        """H = nu curl A projected into this Nedelec space (M H = (nu curl A, w),
        Jacobi PCG); H holds the initial guess.  Returns the solve report."""
        info = N.SolveInfo()
        st = N.lib().hc_magnetic_field_device(self.h, _dev_ptr(A, "float64"), _dev_ptr(H, "float64"), float(rtol),
                                              C.byref(info))
        N.check(st, self.h)
        return {"status": N.STATUS_NAMES[info.status], "iterations": info.iterations,
                "rel_residual": info.rel_residual}

    def TetCurlPointsDevice(self, A, xi):
        """curl A at reference points xi (npts x 3, simplex of the sorted
        element vertices) of every tet: (ne, npts, 3) float64 CUDA tensor."""
        import torch

        xi = np.ascontiguousarray(xi, dtype=np.float64).reshape(-1, 3)
        B = torch.empty(self.ne, xi.shape[0], 3, dtype=torch.float64, device="cuda")
        N.check(N.lib().hc_tet_curl_points_device(self.h, _dev_ptr(A, "float64"), int(xi.shape[0]), _ptr(xi),
                                                  _dev_ptr(B, "float64")), self.h)
        return B

    # -- backward-Euler steps on device state --
    def BeRhsDevice(self, f, A, b):
        """b = P (f - C_nu A) (one step's right-hand side)."""
        N.check(N.lib().hc_be_rhs_device(self.h, _dev_ptr(f, "float64"), _dev_ptr(A, "float64"),
                                         _dev_ptr(b, "float64")), self.h)
        return b

    def BeUpdateDevice(self, A, dA):
        """A += dt dA."""
        N.check(N.lib().hc_be_update_device(self.h, _dev_ptr(A, "float64"), _dev_ptr(dA, "float64")), self.h)
        return A

    # -- frequency domain: C_nu + i omega M_sigma (ComplexMaxwellOperator, eps = 0) --
    def MultComplex(self, omega, x):
        """y = J x for the eliminated complex operator, complex host vectors."""
        x = np.asarray(x, dtype=np.complex128)
        xb = np.ascontiguousarray(np.concatenate([x.real, x.imag]))
        yb = np.empty_like(xb)
        N.check(N.lib().hc_mult_complex(self.h, float(omega), _ptr(xb), _ptr(yb)), self.h)
        n = self.ndof
        return yb[:n] + 1j * yb[n:]

    def MultComplexDevice(self, omega, xr, xi, yr, yi):
        """Planar device tensors (all float64 or all float32)."""
        import torch

        if xr.dtype == torch.float64:
            f, t = N.lib().hc_mult_complex_device, "float64"
        else:
            f, t = N.lib().hc_mult_complex_device_f32, "float32"
        N.check(f(self.h, float(omega), _dev_ptr(xr, t), _dev_ptr(xi, t), _dev_ptr(yr, t), _dev_ptr(yi, t)),
                self.h)
        return yr, yi

    def PrecondApplyDevice(self, r, z, precond="aux"):
        """z = B r (device FP64 tensors): precond 'jacobi' (D^-1) or 'aux' (D^-1 + G V G^T)."""
        N.check(N.lib().hc_precond_apply_device(self.h, _PRECOND[precond], _dev_ptr(r, "float64"),
                                                _dev_ptr(z, "float64")), self.h)
        return z

    def SetLaunch(self, shape=0, per_sm=0):
        """Brick shape (0: 16x4x2, 1: 8x8x2 elements) and CTAs per SM (0: the
        launcher's choice) of the tiled hex kernels (hc_set_launch)."""
        N.check(N.lib().hc_set_launch(self.h, int(shape), int(per_sm)), self.h)

    def GetLaunch(self):
        sh, per = C.c_int32(0), C.c_int32(0)
        N.check(N.lib().hc_get_launch(self.h, C.byref(sh), C.byref(per)), self.h)
        return {"shape": sh.value, "per_sm": per.value}

    def Autotune(self, kind="real"):
        """Time the FP32 apply (kind 'real' or 'complex') over brick shapes and
        CTAs per SM, keep the fastest (hc_autotune); returns the choice with
        the mean launch times of it and of the default configuration."""
        sh, per = C.c_int32(0), C.c_int32(0)
        best, dflt = C.c_double(0), C.c_double(0)
        N.check(N.lib().hc_autotune(self.h, {"real": 0, "complex": 1}[kind], C.byref(sh), C.byref(per),
                                    C.byref(best), C.byref(dflt)), self.h)
        return {"shape": sh.value, "per_sm": per.value, "us": best.value, "us_default": dflt.value}

    def LanczosLmax(self, steps=20):
        v = C.c_double(0)
        N.check(N.lib().hc_lanczos_lmax(self.h, steps, C.byref(v)), self.h)
        return v.value


_PRECOND = {"none": N.HC_PRECOND_NONE, "jacobi": N.HC_PRECOND_JACOBI, "chebyshev": N.HC_PRECOND_CHEBYSHEV,
            "aux": N.HC_PRECOND_AUX, "aux_mult": N.HC_PRECOND_AUX_MULT}
_PREC = {"fp64": N.HC_FP64, "mixed": N.HC_MIXED, "mixed_rr": N.HC_MIXED_RR}


class GpuHCurlPCGSolver:
    """PCG on the device, configured with the reference's option names.

    Options (defaults as DefaultJacobiPCGSolver, hephaestus_solvers.hpp:34-57):
      Tolerance (1e-9), AbsTolerance (1e-16), MaxIter (1000), PrintLevel (ignored),
    plus: Precision ('fp64' | 'mixed' | 'mixed_rr': one FP32 PCG with FP64
    residual replacement), Preconditioner ('jacobi' |
    'chebyshev' | 'aux' | 'none'; 'aux' = Jacobi + the auxiliary-space
    gradient correction, the gradient part of AMS), ChebyshevDegree (2), ChebyshevRatio (30),
    ChebyshevLmax (0 = estimate), InnerTolerance (1e-4; for 'mixed_rr' the
    residual reduction between replacements, 0.1), MaxOuter (50).
    """

    def __init__(self, params=None, op=None):
        params = dict(params or {})
        self.p = N.SolveParams()
        self.p.precision = _PREC[params.get("Precision", "fp64")]
        self.p.precond = _PRECOND[params.get("Preconditioner", "jacobi")]
        self.p.cheb_degree = int(params.get("ChebyshevDegree", 2))
        self.p.cheb_ratio = float(params.get("ChebyshevRatio", 30.0))
        self.p.cheb_lmax = float(params.get("ChebyshevLmax", 0.0))
        self.p.rtol = float(params.get("Tolerance", 1e-9))
        self.p.atol = float(params.get("AbsTolerance", 1e-16))
        self.p.maxit = int(params.get("MaxIter", 1000))
        rr = self.p.precision == N.HC_MIXED_RR
        self.p.inner_rtol = float(params.get("InnerTolerance", 0.1 if rr else 1e-4))
        self.p.max_outer = int(params.get("MaxOuter", 50))
        self.op = op
        self.info = N.SolveInfo()
        self.raise_on_nonconvergence = bool(params.get("RaiseOnNonConvergence", False))

    def SetOperator(self, op):
        self.op = op

    def Mult(self, b, x):
        """Solve J x = b (host float64 arrays; x is the initial guess, updated in place)."""
        op = self.op
        b = op._h(b)
        if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous):
            raise TypeError("x must be a contiguous float64 array (updated in place)")
        st = N.lib().hc_solve(op.h, C.byref(self.p), _ptr(b), _ptr(x), C.byref(self.info))
        self._check(st)
        return x

    def MultDevice(self, b, x):
        """Solve with device float64 tensors (x updated in place)."""
        op = self.op
        st = N.lib().hc_solve_device(op.h, C.byref(self.p), _dev_ptr(b, "float64"), _dev_ptr(x, "float64"),
                                     C.byref(self.info))
        self._check(st)
        return x

    def MultMultiDevice(self, B, X):
        """Solve J X = B for the columns of (ndof, nrhs) row-major float64 CUDA
        tensors together (hc_solve_multi_device: block PCG, one batched
        apply per iteration; tet meshes).  X holds the initial guesses and is
        updated in place; returns the list of per-column result dicts."""
        op = self.op
        nrhs = 1 if B.dim() == 1 else int(B.shape[1])
        if tuple(X.shape) != tuple(B.shape):
            raise ValueError("B and X must have the same shape")
        if int(B.shape[0]) != op.ndof:
            raise ValueError("B has %d rows, the operator %d dofs" % (int(B.shape[0]), op.ndof))
        if nrhs not in (1, 2, 4, 8, 16, 32):
            raise ValueError("the number of right-hand sides must be 1, 2, 4, 8, 16 or 32")
        infos = (N.SolveInfo * nrhs)()
        st = N.lib().hc_solve_multi_device(op.h, C.byref(self.p), nrhs, _dev_ptr(B, "float64"),
                                           _dev_ptr(X, "float64"), infos)
        self._check(st)
        out = []
        for i in infos:
            self.info = i
            out.append(self.result)
        return out

    def StepsDevice(self, f, A, dA, b, nsteps):
        """nsteps backward-Euler steps on device state (hc_be_steps_device):
        per step b = P (f - C_nu A), dA = 0, solve J dA = b with these
        options, A += dt dA.  A is updated in place; returns the per-step
        result dicts of the steps taken (the last one is the first non-OK)."""
        op = self.op
        infos = (N.SolveInfo * int(nsteps))()
        st = N.lib().hc_be_steps_device(op.h, C.byref(self.p), int(nsteps), _dev_ptr(f, "float64"),
                                        _dev_ptr(A, "float64"), _dev_ptr(dA, "float64"), _dev_ptr(b, "float64"),
                                        infos)
        self._check(st)
        out = []
        for i in infos:
            if i.status < 0:
                break
            self.info = i
            out.append(self.result)
        return out

    def MultMulti(self, B, X):
        """Host form of MultMultiDevice: B, X are (ndof, nrhs) C-contiguous float64
        numpy arrays ([dof][rhs]); X holds the initial guesses and is updated
        in place.  Returns the per-column result dicts."""
        op = self.op
        if not (isinstance(X, np.ndarray) and X.dtype == np.float64 and X.flags.c_contiguous):
            raise TypeError("X must be a C-contiguous float64 array (updated in place)")
        B = np.ascontiguousarray(B, dtype=np.float64)
        if B.shape != X.shape:
            raise ValueError("B and X must have the same shape")
        nrhs = 1 if B.ndim == 1 else int(B.shape[1])
        if int(B.shape[0]) != op.ndof:
            raise ValueError("B has %d rows, the operator %d dofs" % (int(B.shape[0]), op.ndof))
        if nrhs not in (1, 2, 4, 8, 16, 32):
            raise ValueError("the number of right-hand sides must be 1, 2, 4, 8, 16 or 32")
        infos = (N.SolveInfo * nrhs)()
        st = N.lib().hc_solve_multi(op.h, C.byref(self.p), nrhs, _ptr(B), _ptr(X), infos)
        self._check(st)
        out = []
        for i in infos:
            self.info = i
            out.append(self.result)
        return out

    def _check(self, st):
        if st in (N.HC_OK,):
            return
        if st in (N.HC_NOT_CONVERGED, N.HC_BREAKDOWN) and not self.raise_on_nonconvergence:
            return
        raise N.HcError(st, N.last_error(self.op.h))

    @property
    def result(self):
        i = self.info
        return {"status": N.STATUS_NAMES[i.status], "iterations": i.iterations,
                "outer_iterations": i.outer_iterations, "applies": i.applies,
                "rel_residual": i.rel_residual, "lmax": i.lmax}


class GpuComplexCOCGSolver(GpuHCurlPCGSolver):
    """COCG on J = P (C_nu + i omega M_sigma) P + (I - P) with the complex
    Jacobi preconditioner: the solve of ComplexMaxwellOperator::Solve
    (src/formulations/ComplexMaxwell/complex_maxwell_formulation.cpp:171-222)
    with an iterative solver in place of SuperLU.  Options as
    GpuHCurlPCGSolver (Precision 'fp64' | 'mixed'); Preconditioner 'jacobi'
    (default) or 'aux' (Jacobi + G V G^T / (i omega))."""

    def __init__(self, params=None, op=None, omega=0.0):
        params = dict(params or {})
        params.setdefault("Preconditioner", "jacobi")
        super().__init__(params, op)
        self.omega = float(omega)

    def Mult(self, b, x):
        """Solve J x = b; b, x complex host arrays (x: initial guess, updated in place)."""
        op = self.op
        if not (isinstance(x, np.ndarray) and x.dtype == np.complex128):
            raise TypeError("x must be a complex128 array (updated in place)")
        b = np.asarray(b, dtype=np.complex128)
        bb = np.ascontiguousarray(np.concatenate([b.real, b.imag]))
        xb = np.ascontiguousarray(np.concatenate([x.real, x.imag]))
        st = N.lib().hc_solve_complex(op.h, C.byref(self.p), self.omega, _ptr(bb), _ptr(xb), C.byref(self.info))
        self._check(st)
        n = op.ndof
        x[:] = xb[:n] + 1j * xb[n:]
        return x

    def MultGraph(self, br, bi, xr, xi):
        """Enqueue the graph-driven solve (planar float64 device tensors); the
        result is read by Finish().  The graph is reused while the tensors stay
        the same."""
        op = self.op
        st = N.lib().hc_solve_complex_graph(op.h, C.byref(self.p), self.omega, _dev_ptr(br, "float64"),
                                            _dev_ptr(bi, "float64"), _dev_ptr(xr, "float64"),
                                            _dev_ptr(xi, "float64"))
        if st != N.HC_OK:
            raise N.HcError(st, N.last_error(op.h))
        return xr, xi

    def Finish(self):
        """Wait for the graph-driven solve of MultGraph and record its report."""
        self._check(N.lib().hc_graph_solve_info(self.op.h, C.byref(self.info)))
        return self.result

    def MultDevice(self, br, bi, xr, xi):
        """Planar float64 device tensors (xr, xi updated in place)."""
        op = self.op
        st = N.lib().hc_solve_complex_device(op.h, C.byref(self.p), self.omega, _dev_ptr(br, "float64"),
                                             _dev_ptr(bi, "float64"), _dev_ptr(xr, "float64"),
                                             _dev_ptr(xi, "float64"), C.byref(self.info))
        self._check(st)
        return xr, xi


def solve_complex_batch(solvers, rhs, sols):
    """Run several GpuComplexCOCGSolver solves at once (hc_solve_complex_batch).

    solvers: list of GpuComplexCOCGSolver (same parameters; each operator
    should have its own stream); rhs / sols: lists of (re, im) float64 device
    tensors.  Returns the list of result dicts.
    """
    n = len(solvers)
    if n == 0:
        return []
    hs = (C.c_void_p * n)(*[s.op.h.value for s in solvers])
    om = (C.c_double * n)(*[s.omega for s in solvers])
    br = (C.c_void_p * n)(*[_dev_ptr(b[0], "float64").value for b in rhs])
    bi = (C.c_void_p * n)(*[_dev_ptr(b[1], "float64").value for b in rhs])
    xr = (C.c_void_p * n)(*[_dev_ptr(x[0], "float64").value for x in sols])
    xi = (C.c_void_p * n)(*[_dev_ptr(x[1], "float64").value for x in sols])
    infos = (N.SolveInfo * n)()
    st = N.lib().hc_solve_complex_batch(n, hs, C.byref(solvers[0].p), om, br, bi, xr, xi, infos)
    if st not in (N.HC_OK, N.HC_NOT_CONVERGED, N.HC_BREAKDOWN):
        raise N.HcError(st, N.last_error(solvers[0].op.h))
    out = []
    for s, i in zip(solvers, infos):
        s.info = i
        out.append(s.result)
    return out
