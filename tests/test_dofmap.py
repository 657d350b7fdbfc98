"""CPU tests of the dof correspondence the MFEM shim uses (hc_dofmap_*, host
code): the library's element dof lists against the oracle's numbering, and
maps built from synthetic caller numberings (a random signed permutation of
the library's dofs, encoded as MFEM encodes orientation: -1 - d for minus)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from hephaestus_gb300 import _native as N
from hephaestus_gb300 import meshes


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _err():
    buf = C.create_string_buffer(512)
    N.lib().hc_dofmap_last_error(buf, 512)
    return buf.value.decode()


def hex_elem_dofs(p, nx, ny, nz):
    L = 3 * p * (p + 1) ** 2
    out = np.empty((nx * ny * nz, L), dtype=np.int64)
    assert N.lib().hc_hex_elem_dofs(p, nx, ny, nz, _p(out)) == N.HC_OK
    return out


def tet_elem_dofs(p, verts, tets):
    L = 6 if p == 1 else 20
    t = np.ascontiguousarray(tets, dtype=np.int64)
    out = np.empty((len(t), L), dtype=np.int64)
    nd = C.c_int64(0)
    assert N.lib().hc_tet_elem_dofs(p, len(verts), len(t), _p(t), _p(out), C.byref(nd)) == N.HC_OK
    return out, nd.value


class DofMap:
    def __init__(self, n, lib, caller):
        self.h = C.c_void_p()
        lib = np.ascontiguousarray(lib, dtype=np.int64)
        caller = np.ascontiguousarray(caller, dtype=np.int32)
        self.status = N.lib().hc_dofmap_create(n, lib.shape[0], lib.shape[1], _p(lib), _p(caller), C.byref(self.h))
        self.n = n

    def to_lib(self, x):
        y = np.empty(self.n)
        assert N.lib().hc_dofmap_to_lib(self.h, _p(np.ascontiguousarray(x)), _p(y)) == N.HC_OK
        return y

    def from_lib(self, x):
        y = np.empty(self.n)
        assert N.lib().hc_dofmap_from_lib(self.h, _p(np.ascontiguousarray(x)), _p(y)) == N.HC_OK
        return y

    def __del__(self):
        if getattr(self, "h", None):
            N.lib().hc_dofmap_destroy(self.h)


def synthetic_caller(lib, n, seed):
    """A caller numbering: caller dof perm[l] holds library dof l with sign s[l]."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n)
    s = rng.choice([-1, 1], size=n)
    enc = np.where(s[lib] > 0, perm[lib], -1 - perm[lib])
    return enc.astype(np.int32), perm, s


@pytest.mark.parametrize("p", [1, 2, 3])
def test_hex_element_dofs_match_the_oracle_numbering(p):
    nx, ny, nz = 4, 3, 5
    assert np.array_equal(hex_elem_dofs(p, nx, ny, nz), oracle.Problem.hex(nx, ny, nz, p).elem_dofs())


@pytest.mark.parametrize("p", [1, 2])
def test_tet_element_dofs_match_the_oracle_numbering(p):
    v, t, _, _ = meshes.kuhn_mesh(3, jitter=0.15, seed=2)
    d, n = tet_elem_dofs(p, v, t)
    ref = oracle.Problem.tet(v, t, p)
    assert n == ref.ndof
    assert np.array_equal(d, ref.elem_dofs())


@pytest.mark.parametrize("kind", ["hex", "tet"])
def test_map_round_trips_and_applies_the_signed_permutation(kind):
    if kind == "hex":
        lib = hex_elem_dofs(2, 3, 4, 2)
        n = int(lib.max()) + 1
    else:
        v, t, _, _ = meshes.kuhn_mesh(3, jitter=0.1, seed=1)
        lib, n = tet_elem_dofs(1, v, t)
    enc, perm, s = synthetic_caller(lib, n, 7)
    m = DofMap(n, lib, enc)
    assert m.status == N.HC_OK, _err()
    assert N.lib().hc_dofmap_size(m.h) == n
    xc = np.random.default_rng(3).standard_normal(n)
    xl = m.to_lib(xc)
    assert np.array_equal(xl, s * xc[perm])  # library dof l = s[l] * caller dof perm[l]
    assert np.array_equal(m.from_lib(xl), xc)
    # the map is orthogonal: <P x, P y> = <x, y>
    yc = np.random.default_rng(4).standard_normal(n)
    assert abs(m.to_lib(xc) @ m.to_lib(yc) - xc @ yc) < 1e-12 * np.linalg.norm(xc) * np.linalg.norm(yc)


def test_map_rejects_inconsistent_element_lists():
    lib = hex_elem_dofs(1, 3, 3, 3)
    n = int(lib.max()) + 1
    enc, perm, s = synthetic_caller(lib, n, 9)
    # a shared dof with the opposite sign in one element only
    bad = enc.copy()
    e, l = 13, 0  # an interior element: its local dof 0 is shared with a neighbour
    bad[e, l] = -1 - bad[e, l]
    m = DofMap(n, lib, bad)
    assert m.status == N.HC_EINVAL
    assert "reached as caller dof" in _err()
    # two library dofs on one caller dof
    bad = enc.copy()
    d0 = lib[0, 0]
    bad[lib == d0] = np.int32(perm[lib[0, 1]] if s[lib[0, 1]] > 0 else -1 - perm[lib[0, 1]])
    m = DofMap(n, lib, bad)
    assert m.status == N.HC_EINVAL
    # out of range
    bad = enc.copy()
    bad[0, 0] = n + 5
    assert DofMap(n, lib, bad).status == N.HC_EINVAL


def test_essential_tdof_list_maps_to_the_library_mask():
    lib = hex_elem_dofs(2, 3, 3, 3)
    n = int(lib.max()) + 1
    enc, perm, s = synthetic_caller(lib, n, 11)
    m = DofMap(n, lib, enc)
    want = oracle.Problem.hex(3, 3, 3, 2).hex_ess_mask(0x3F)  # library numbering
    ess_caller = np.sort(perm[np.nonzero(want)[0]]).astype(np.int32)  # what GetEssentialTrueDofs would list
    mask = np.zeros(n, dtype=np.uint8)
    assert N.lib().hc_dofmap_ess_mask(m.h, len(ess_caller), _p(ess_caller), _p(mask)) == N.HC_OK
    assert np.array_equal(mask, want)
    bad = np.array([n], dtype=np.int32)
    assert N.lib().hc_dofmap_ess_mask(m.h, 1, _p(bad), _p(mask)) == N.HC_EINVAL


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["hex2", "tet1"])
def test_operator_and_solve_in_caller_numbering_match_the_oracle(kind):
    """The drop-in path in a caller's numbering: the essential set comes from
    the caller's ess_tdof_list through the map, y_caller = map^T J map x_caller
    equals the oracle's operator in that numbering, and a solve through the
    map returns the oracle's solution in that numbering."""
    from hephaestus_gb300 import GpuHCurlPCGSolver, HCurlOperator

    rng = np.random.default_rng(21)
    if kind == "hex2":
        n, p = 4, 2
        lib = hex_elem_dofs(p, n, n, n)
        nd = int(lib.max()) + 1
        ne = n ** 3
        ref = oracle.Problem.hex(n, n, n, p)
        lib_mask = ref.hex_ess_mask(0x3F)
    else:
        v, t, bt, ba = meshes.kuhn_mesh(4, jitter=0.15, seed=3)
        p = 1
        lib, nd = tet_elem_dofs(p, v, t)
        ne = len(t)
        ref = oracle.Problem.tet(v, t, p)
        lib_mask = ref.tet_ess_mask(bt, ba, 0x3F)
    enc, perm, s = synthetic_caller(lib, nd, 5)
    m = DofMap(nd, lib, enc)
    assert m.status == N.HC_OK, _err()
    ess_caller = np.sort(perm[np.nonzero(lib_mask)[0]]).astype(np.int32)
    mask = np.zeros(nd, dtype=np.uint8)
    assert N.lib().hc_dofmap_ess_mask(m.h, len(ess_caller), _p(ess_caller), _p(mask)) == N.HC_OK
    nu = meshes.loguniform(ne, 1.0, 10.0, rng)
    sigma = meshes.loguniform(ne, 0.1, 10.0, rng)
    if kind == "hex2":
        op = HCurlOperator(n, n, n, p, nu, sigma, dt=0.05, ess_mask=mask)
    else:
        op = HCurlOperator.from_tets(v, t, p, nu, sigma, dt=0.05, ess_mask=mask)
    ref.set_coef(0.05 * nu, sigma)
    ref.assemble()
    ref.set_ess(mask)
    xc = rng.standard_normal(nd)
    yc = m.from_lib(op.Mult(m.to_lib(xc)))
    want = m.from_lib(ref.apply_masked(m.to_lib(xc)))
    assert np.linalg.norm(yc - want) / np.linalg.norm(want) < 1e-12
    bc = m.from_lib(np.where(mask != 0, 0.0, ref.load_coil(q=4)))
    xl = np.zeros(nd)
    sol = GpuHCurlPCGSolver({"Tolerance": 1e-13, "AbsTolerance": 0.0, "MaxIter": 20000}, op)
    sol.Mult(m.to_lib(bc), xl)
    assert sol.result["status"] == "OK", sol.result
    xo, st, _, _ = ref.pcg(m.to_lib(bc), precond=1, rtol=1e-13, maxit=100000)
    assert np.linalg.norm(m.from_lib(xl) - m.from_lib(xo)) / np.linalg.norm(xo) < 1e-9
